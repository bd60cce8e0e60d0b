// libcm_fe: surface-pressure follower load, device code shared by the
// boundary-face kernel (fe_surface.cu) and the batched kernel (fe_batch.cu).
//
// FiniteElasticity_SurfacePressureResidualEvaluate (finite_elasticity_routines.f90:
// 3215-3361) and ..JacobianEvaluate (:3049-3208): on every boundary face whose
// nodal pressure values (component = the face's normal xi direction) are not
// all zero,
//   r(c, f)  += sum_g w_g p_g orientation n_c N_f
//   K(mh,ms; nh,ns) += sum_g sum_i (n_mh g^i_nh - g^i_mh n_nh) w_g p_g orientation dN_ns/dxi_i N_ms
// for the lower displacement blocks mh > nh, mirrored to the upper blocks
// like the element matrix (:1149-1153).  n = g_1 x g_2 is the unnormalised
// face normal and g^i the surface dual basis of COORDINATE_METRICS_CALCULATE
// (coordinate_routines.f90:908-915).  One warp handles one boundary element.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "fe_internal.h"

namespace {


constexpr double SURF_ZERO_TOL = 5.0 * 2.220446049250313e-16;  // ZERO_TOLERANCE (constants.f90:68)

// Local faces in the reference's order (basis_routines.f90:2162-2224): -xi1,
// -xi2, -xi3, +xi1, +xi2, +xi3; face node f = f1 + n1 f2 runs along the first
// in-face direction (normal xi1 -> xi2, xi3; xi2 -> xi1, xi3; xi3 -> xi1, xi2).
__device__ __forceinline__ int face_node(int lf, int n1, int f) {
  const int ni = lf % 3, side = lf / 3;
  const int xa = ni == 0 ? 1 : 0, xb = ni == 2 ? 1 : 2;
  int pos[3];
  pos[ni] = side ? n1 - 1 : 0;
  pos[xa] = f % n1;
  pos[xb] = f / n1;
  return pos[0] + n1 * (pos[1] + n1 * pos[2]);
}

__device__ __forceinline__ double lag(int n1, int k, int d, double t) {
  if (n1 == 2) return d == 0 ? (k == 0 ? 1.0 - t : t) : (k == 0 ? -1.0 : 1.0);
  if (d == 0) return k == 0 ? 1.0 - 3.0 * t + 2.0 * t * t : (k == 1 ? 4.0 * t * (1.0 - t) : t * (t + t - 1.0));
  return k == 0 ? 4.0 * t - 3.0 : (k == 1 ? 4.0 - 8.0 * t : 4.0 * t - 1.0);
}

struct SurfWarpSmem {
  double z[9][3];
  double p[9];
  double gq[9][10];  // per face Gauss point: w p orientation, n(3), g^1(3), g^2(3)
  int node[9];       // element-local node of each face node
};

// All loaded faces of boundary element e, by one warp (S is the warp's
// shared scratch).  mode: 0 = CSR (FP64 values, or FP32 uu values when
// P.vals_uu), 1 = element outputs (P.elem_out, elements first_elem ..
// first_elem + count - 1), 2 = the element's staging records (SO->uu,
// SO->r), which only this warp touches, so it adds without atomics.
template <int N1>
__device__ __forceinline__ void surface_element(const cmfe::KParams& P, int e, const uint8_t* bmask, int mode,
                                                int want_jac, SurfWarpSmem& S, int lane,
                                                const cmfe::StageOut* SO = nullptr) {
  constexpr int NPE = N1 * N1 * N1, NF = N1 * N1;
  const int nr = P.nr, nrow = 3 * NPE + (P.pmode ? 8 : 1);
  const uint8_t mask = bmask[e];
  for (int lf = 0; lf < 6; ++lf) {
    if (!(mask >> lf & 1)) continue;
    const int ni = lf % 3, side = lf / 3;
    __syncwarp();
    bool nz = false;
    if (lane < NF) {
      const int a = face_node(lf, N1, lane);
      const int node = P.elem_u[(size_t)e * NPE + a];
      S.node[lane] = a;
      const double pv = P.surf_p[(size_t)ni * P.nu + node];
      S.p[lane] = pv;
      nz = fabs(pv) > SURF_ZERO_TOL;
#pragma unroll
      for (int c = 0; c < 3; ++c) S.z[lane][c] = P.x[(size_t)c * P.nu + node];
    }
    if (!__any_sync(0xffffffffu, nz)) continue;
    __syncwarp();
    // per face Gauss point geometry (3x3 Gauss-Legendre on [0,1]^2, point i + 3j)
    if (lane < 9) {
      const double x3[3] = {(-sqrt(0.6) + 1.0) / 2.0, 0.5, (sqrt(0.6) + 1.0) / 2.0};
      const double w3[3] = {2.5 / 9.0, 4.0 / 9.0, 2.5 / 9.0};
      const int gi = lane % 3, gj = lane / 3;
      double p = 0.0, g[3][2] = {{0, 0}, {0, 0}, {0, 0}};
      for (int f = 0; f < NF; ++f) {
        const int f1 = f % N1, f2 = f / N1;
        const double l1 = lag(N1, f1, 0, x3[gi]), l2 = lag(N1, f2, 0, x3[gj]);
        const double d1 = lag(N1, f1, 1, x3[gi]), d2 = lag(N1, f2, 1, x3[gj]);
        const double N = l1 * l2, dN0 = d1 * l2, dN1 = l1 * d2;
        p = fma(N, S.p[f], p);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          g[c][0] = fma(dN0, S.z[f][c], g[c][0]);
          g[c][1] = fma(dN1, S.z[f][c], g[c][1]);
        }
      }
      double GL[2][2];
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) GL[a][b] = g[0][a] * g[0][b] + g[1][a] * g[1][b] + g[2][a] * g[2][b];
      const double rdet = 1.0 / (GL[0][0] * GL[1][1] - GL[1][0] * GL[0][1]);
      const int orient = ((side ? 1 : -1) * (ni == 1 ? -1 : 1)) > 0 ? 1 : -1;
      double* q = S.gq[lane];
      q[0] = w3[gi] * w3[gj] * (p * orient);
      q[1] = g[1][0] * g[2][1] - g[2][0] * g[1][1];
      q[2] = g[2][0] * g[0][1] - g[0][0] * g[2][1];
      q[3] = g[0][0] * g[1][1] - g[1][0] * g[0][1];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        q[4 + c] = (GL[1][1] * g[c][0] - GL[0][1] * g[c][1]) * rdet;
        q[7 + c] = (GL[0][0] * g[c][1] - GL[1][0] * g[c][0]) * rdet;
      }
    }
    __syncwarp();
    const uint16_t* tab = P.tables + (size_t)P.elem_table[e] * nr * nr;
    const int* en = P.elem_u + (size_t)e * NPE;
    // residual rows
    if (P.r != nullptr || (mode == 1 && !want_jac) || mode == 2) {
      if (lane < 3 * NF) {
        const int c = lane / NF, f = lane % NF;
        const double x3[3] = {(-sqrt(0.6) + 1.0) / 2.0, 0.5, (sqrt(0.6) + 1.0) / 2.0};
        double acc = 0.0;
        for (int ng = 0; ng < 9; ++ng) {
          const double N = lag(N1, f % N1, 0, x3[ng % 3]) * lag(N1, f / N1, 0, x3[ng / 3]);
          acc = fma(S.gq[ng][0] * S.gq[ng][1 + c], N, acc);
        }
        const int a = S.node[f];
        if (mode == 2) {
          SO->r[(size_t)e * cmfe::rec_stride_r(NPE, nrow - 3 * NPE) + c * NPE + a] += acc;
        } else if (mode == 1) {
          P.elem_out[(size_t)(e - P.first_elem) * nrow + c * NPE + a] += acc;
        } else {
          atomicAdd(&P.r[(size_t)c * P.nu + en[a]], acc);
        }
      }
    }
    if (!want_jac) continue;
    // lower off-diagonal displacement blocks and their mirrors
    for (int k = lane; k < 3 * NF * NF; k += 32) {
      const int oh = k / (NF * NF), ms = (k / NF) % NF, ns = k % NF;
      const int nh = oh == 2 ? 1 : 0, mh = oh == 0 ? 1 : 2;
      const double x3[3] = {(-sqrt(0.6) + 1.0) / 2.0, 0.5, (sqrt(0.6) + 1.0) / 2.0};
      double acc = 0.0;
      for (int ng = 0; ng < 9; ++ng) {
        const double* q = S.gq[ng];
        const double gi = x3[ng % 3], gj = x3[ng / 3];
        const double w0 = (q[1 + mh] * q[4 + nh] - q[4 + mh] * q[1 + nh]) * q[0];
        const double w1 = (q[1 + mh] * q[7 + nh] - q[7 + mh] * q[1 + nh]) * q[0];
        const int s1 = ns % N1, s2 = ns / N1, m1 = ms % N1, m2 = ms / N1;
        const double dn0 = lag(N1, s1, 1, gi) * lag(N1, s2, 0, gj);
        const double dn1 = lag(N1, s1, 0, gi) * lag(N1, s2, 1, gj);
        const double nm = lag(N1, m1, 0, gi) * lag(N1, m2, 0, gj);
        acc += (w0 * dn0) * nm + (w1 * dn1) * nm;
      }
      const int a = S.node[ms], b = S.node[ns];
      if (mode == 2) {
        // the lower block entry and its mirror: distinct entries for distinct
        // (oh, ms, ns), so the lanes never touch the same word
        float* st = SO->uu + (size_t)e * cmfe::rec_stride_uu(NPE);
        const int R = mh * NPE + a, Cc = nh * NPE + b;
        st[(size_t)R * (3 * NPE) + Cc] += (float)acc;
        st[(size_t)Cc * (3 * NPE) + R] += (float)acc;
        continue;
      }
      if (mode == 1) {
        double* out = P.elem_out + (size_t)(e - P.first_elem) * nrow * nrow;
        const int R = mh * NPE + a, Cc = nh * NPE + b;
        out[(size_t)Cc * nrow + R] += acc;
        out[(size_t)R * nrow + Cc] += acc;
        continue;
      }
      const int na = en[a], nb2 = en[b];
      const uint16_t tab_ab = tab[a * nr + b], tab_ba = tab[b * nr + a];
      if (P.vals_uu) {
        const size_t p1 = (size_t)P.uu_row_ptr[(size_t)mh * P.nu + na] + (size_t)nh * P.wu[na] + (tab_ab & 0x7fff);
        const size_t p2 = (size_t)P.uu_row_ptr[(size_t)nh * P.nu + nb2] + (size_t)mh * P.wu[nb2] + (tab_ba & 0x7fff);
        atomicAdd(&P.vals_uu[p1], (float)acc);
        atomicAdd(&P.vals_uu[p2], (float)acc);
      } else {
        const size_t p1 = (size_t)P.row_ptr[(size_t)mh * P.nu + na] + (size_t)nh * P.wu[na] + (tab_ab & 0x7fff);
        const size_t p2 = (size_t)P.row_ptr[(size_t)nh * P.nu + nb2] + (size_t)mh * P.wu[nb2] + (tab_ba & 0x7fff);
        atomicAdd(&P.vals[p1], acc);
        atomicAdd(&P.vals[p2], acc);
      }
    }
  }
}

}  // namespace
