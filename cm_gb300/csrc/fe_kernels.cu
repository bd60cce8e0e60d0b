// libcm_fe: GB300 (sm_103a) finite-elasticity element assembly and the C ABI
// declared in include/cm_fe.h.
//
// One CTA assembles one element at a time (persistent over the elements of
// one colour).  Per element:
//   P0  gather the deformed coordinates z and pressures of the element;
//   P1  interpolate dz/dxi at the 27 Gauss points (243 independent sums);
//   P2  per Gauss point: metrics, F, Cauchy stress and spatial tangent
//       (FINITE_ELASTICITY_GAUSS_STRESS_TENSOR / _ELASTICITY_TENSOR);
//   P3  dN/dz at every Gauss point (DPHIDZ);
//   P4  residual rows, accumulated over Gauss points in the reference order;
//   P5  lower-triangle Jacobian entries held in registers, accumulated over
//       Gauss points in the reference order (per Gauss point the 3-vectors
//       JGW*(c + sigma)*dN/dz of every column are formed once in shared
//       memory, then each entry adds one 3-term dot product);
//   P6  scatter into the CSR values and the residual (each entry and its
//       mirror; first contributor in colour order stores, later ones add).
// Elements of one colour share no node, so P6 needs no atomics and the
// result does not depend on scheduling.
//
// The mixed-precision variant keeps P1-P4 and the pressure coupling in FP64
// and runs the tangent (elasticity tensor, uu block) in FP32.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <type_traits>

#include "fe_internal.h"
#include "fe_math.cuh"

using cmfe::HostSetup;
using cmfe::KParams;
using cmfe::NG;

namespace {

thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                           \
  do {                                                                                           \
    cudaError_t err__ = (expr);                                                                  \
    if (err__ != cudaSuccess)                                                                    \
      return set_error(FE_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(err__));      \
  } while (0)

enum Mode { M_RES = 0, M_JAC = 1, M_MIX = 2, M_ERES = 3, M_EJAC = 4 };



template <int N1, int PM>
struct Cfg {
  static constexpr int NPE = N1 * N1 * N1;
  static constexpr int NPP = PM ? 8 : 1;
  static constexpr int NR = NPE + NPP;
  static constexpr int NU3 = 3 * NPE;
  static constexpr int NROW = NU3 + NPP;
  static constexpr int NUU = NU3 * (NU3 + 1) / 2;
  static constexpr int NPU = NPP * NU3;
  static constexpr int THREADS = 128;
  static constexpr int EUU = (NUU + THREADS - 1) / THREADS;
  static constexpr int EPU = (NPU + THREADS - 1) / THREADS;
  static constexpr int GPS = 60;  // per-Gauss-point record, doubles
  // shared-memory layout (doubles)
  static constexpr int O_GBF = 0;
  static constexpr int O_GBFP = O_GBF + NG * 4 * NPE;
  static constexpr int O_W = O_GBFP + NG * 8;
  static constexpr int O_Z = O_W + NG;
  static constexpr int O_P = O_Z + 3 * NPE;
  static constexpr int O_DZ = O_P + 8;
  static constexpr int O_PG = O_DZ + NG * 9;
  static constexpr int O_GP = O_PG + NG;
  static constexpr int O_DPHI = O_GP + NG * GPS;
  static constexpr int O_T = O_DPHI + NG * NPE * 3;
  static constexpr int O_END = O_T + 6 * NPE * 3;
  static constexpr size_t SMEM = O_END * sizeof(double) + (NR + 4) * sizeof(int);
};

// Block index of the (row comp m, col comp n) tempvec block: 0..2 diagonal,
// 3,4,5 for (n,m) = (0,1), (0,2), (1,2).
__device__ __forceinline__ int blk_of(int m, int n) { return m == n ? n : (n == 0 ? (m == 1 ? 3 : 4) : 5); }

// ---------------------------------------------------------- the kernel ----
template <int N1, int PM, int MODE>
__global__ void __launch_bounds__(128) fe_element_kernel(KParams P) {
  using C = Cfg<N1, PM>;
  constexpr int NPE = C::NPE, NPP = C::NPP, NR = C::NR, NU3 = C::NU3, NROW = C::NROW;
  constexpr bool JAC = (MODE == M_JAC || MODE == M_MIX || MODE == M_EJAC);
  constexpr bool MIX = (MODE == M_MIX);
  using TT = typename std::conditional<MIX, float, double>::type;  // tangent precision
  extern __shared__ __align__(16) double smem[];
  double* s_gbf = smem + C::O_GBF;
  double* s_gbfp = smem + C::O_GBFP;
  double* s_w = smem + C::O_W;
  double* s_z = smem + C::O_Z;
  double* s_p = smem + C::O_P;
  double* s_dz = smem + C::O_DZ;
  double* s_pg = smem + C::O_PG;
  double* s_gp = smem + C::O_GP;
  double* s_dphi = smem + C::O_DPHI;
  TT* s_T = reinterpret_cast<TT*>(smem + C::O_T);
  int* s_node = reinterpret_cast<int*>(smem + C::O_END);  // [NR] row nodes, then table id
  const int tid = threadIdx.x;
  const bool want_res = (MODE == M_RES || MODE == M_ERES || P.r != nullptr) && MODE != M_EJAC;

  for (int i = tid; i < NG * 4 * NPE; i += C::THREADS) s_gbf[i] = P.gbf_u[i];
  for (int i = tid; i < NG * 8; i += C::THREADS) s_gbfp[i] = P.gbf_p[i];
  for (int i = tid; i < NG; i += C::THREADS) s_w[i] = P.gw[i];

  // Per-thread Jacobian entry descriptors: uu lower triangle in row-major
  // order (row R, col Cc <= R over the 3*NPE displacement dofs), then the
  // pressure-row x displacement-column block.
  int e_uu[C::EUU];
  int e_pu[C::EPU];
  if (JAC) {
#pragma unroll
    for (int j = 0; j < C::EUU; ++j) {
      const int k = tid + j * C::THREADS;
      if (k < C::NUU) {
        int R = (int)((sqrtf(8.0f * (float)k + 1.0f) - 1.0f) * 0.5f);
        while (R * (R + 1) / 2 > k) --R;
        while ((R + 1) * (R + 2) / 2 <= k) ++R;
        const int Cc = k - R * (R + 1) / 2;
        e_uu[j] = (R << 8) | Cc;
      } else {
        e_uu[j] = -1;
      }
    }
#pragma unroll
    for (int j = 0; j < C::EPU; ++j) {
      const int k = tid + j * C::THREADS;
      e_pu[j] = (k < C::NPU) ? (((k / NU3) << 8) | (k % NU3)) : -1;
    }
  }

  for (int it = blockIdx.x; it < P.count; it += gridDim.x) {
    const int e = P.elems ? P.elems[it] : P.first_elem + it;
    __syncthreads();  // previous element done with shared memory
    // P0: gather
    if (tid < NPE) s_node[tid] = P.elem_u[(size_t)e * NPE + tid];
    if (tid >= NPE && tid < NR) s_node[tid] = PM ? P.elem_p[(size_t)e * 8 + (tid - NPE)] : e;
    if (tid == NR) s_node[NR] = P.elem_table[e];
    __syncthreads();
    for (int i = tid; i < 3 * NPE; i += C::THREADS) {
      const int c = i / NPE, a = i % NPE;
      s_z[c * NPE + a] = P.x[(size_t)c * P.nu + s_node[a]];
    }
    if (tid < NPP) s_p[tid] = P.x[(size_t)3 * P.nu + s_node[NPE + tid]];
    __syncthreads();
    // P1: dz/dxi at every Gauss point; pressure at every Gauss point
    for (int i = tid; i < NG * 9; i += C::THREADS) {
      const int g = i / 9, c = (i / 3) % 3, k = i % 3;
      const double* gb = &s_gbf[(g * 4 + k + 1) * NPE];
      const double* zc = &s_z[c * NPE];
      double acc = 0.0;
#pragma unroll 9
      for (int a = 0; a < NPE; ++a) acc = acc + gb[a] * zc[a];
      s_dz[i] = acc;
    }
    if (tid < NG) {
      double pg;
      if (PM) {
        pg = 0.0;
#pragma unroll
        for (int q = 0; q < 8; ++q) pg = pg + s_gbfp[tid * 8 + q] * s_p[q];
      } else {
        pg = s_p[0];
      }
      s_pg[tid] = pg;
    }
    __syncthreads();
    // P2: per Gauss point kinematics and constitutive law
    if (tid < NG) {
      const int g = tid;
      double dz[3][3], dxi[3][3], det_dz, gl[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int k = 0; k < 3; ++k) dz[c][k] = s_dz[g * 9 + c * 3 + k];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) gl[i][j] = dz[0][i] * dz[0][j] + dz[1][i] * dz[1][j] + dz[2][i] * dz[2][j];
      const double det_gl = gl[0][0] * gl[1][1] * gl[2][2] + gl[0][1] * gl[1][2] * gl[2][0] +
                            gl[0][2] * gl[1][0] * gl[2][1] - gl[0][0] * gl[2][1] * gl[1][2] -
                            gl[1][0] * gl[0][1] * gl[2][2] - gl[2][0] * gl[1][1] * gl[0][2];
      const double jz = sqrt(fabs(det_gl));
      d_inv3(dz, dxi, det_dz);
      const double* geo = &P.geo[((size_t)e * NG + g) * 10];
      double dn[3][3], F[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) dn[i][j] = geo[i * 3 + j];
      const double jx = geo[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) F[i][j] = dz[i][0] * dn[0][j] + dz[i][1] * dn[1][j] + dz[i][2] * dn[2][j];
      const double jznu = jz / jx;
      double* rec = &s_gp[g * C::GPS];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) rec[i * 3 + j] = dxi[i][j];
      rec[9] = jz * s_w[g];
      rec[10] = jx * s_w[g];
      rec[11] = jznu;
      const double* cm = P.mat + (P.matpe ? (size_t)e * P.nmat : 0);
      double cc[4] = {cm[0], cm[1], P.nmat > 2 ? cm[2] : 0.0, P.nmat > 3 ? cm[3] : 0.0};
      const double pg = s_pg[g];
      bool ok = (det_dz > 0.0) && (jznu > 0.0);
      if (want_res) {
        double S[6];
        d_gauss_stress(P.law, cc, F, jznu, pg, S);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          rec[12 + i] = S[i];
          ok = ok && isfinite(S[i]);
        }
      }
      if (JAC) {
        TT Ct[6][6], St[6], Ft[3][3], ct[4];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) Ft[i][j] = (TT)F[i][j];
#pragma unroll
        for (int i = 0; i < 4; ++i) ct[i] = (TT)cc[i];
        d_gauss_elasticity<TT>(P.law, ct, Ft, (TT)jznu, (TT)pg, Ct, St);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          rec[18 + i] = (double)St[i];
          ok = ok && isfinite((double)St[i]);
        }
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
          for (int j = 0; j < 6; ++j) rec[24 + i * 6 + j] = (double)Ct[i][j];
      }
      if (!ok) atomicOr(P.status, 1u);
    }
    __syncthreads();
    // P3: DPHIDZ[g][a][mh] = sum_ni dN_a/dxi_ni * dxi_ni/dz_mh
    for (int i = tid; i < NG * NPE * 3; i += C::THREADS) {
      const int g = i / (NPE * 3), a = (i / 3) % NPE, mh = i % 3;
      const double* rec = &s_gp[g * C::GPS];
      double s = 0.0;
#pragma unroll
      for (int ni = 0; ni < 3; ++ni) s = s + s_gbf[(g * 4 + ni + 1) * NPE + a] * rec[ni * 3 + mh];
      s_dphi[i] = s;
    }
    __syncthreads();
    const uint16_t* tab = P.tables + (size_t)s_node[NR] * NR * NR;
    // P4: residual
    if (want_res && tid < NROW) {
      double acc = 0.0;
      if (tid < NU3) {
        const int m = tid / NPE, a = tid % NPE;
        for (int g = 0; g < NG; ++g) {
          const double* rec = &s_gp[g * C::GPS];
          const double* dp = &s_dphi[(g * NPE + a) * 3];
          const double jgw = rec[9];
          const double d = dp[0] * (jgw * rec[12 + t2v(0, m)]) + dp[1] * (jgw * rec[12 + t2v(1, m)]) +
                           dp[2] * (jgw * rec[12 + t2v(2, m)]);
          acc = acc + d;
        }
      } else {
        const int q = tid - NU3;
        for (int g = 0; g < NG; ++g) {
          const double* rec = &s_gp[g * C::GPS];
          const double t1 = rec[10] * (rec[11] - 1.0);
          acc = PM ? acc + t1 * s_gbfp[g * 8 + q] : acc + t1;
        }
      }
      if (MODE == M_ERES) {
        P.elem_out[(size_t)(it)*NROW + tid] = acc;
      } else {
        const int ln = tid < NU3 ? tid % NPE : NPE + (tid - NU3);
        const size_t R = tid < NU3 ? (size_t)(tid / NPE) * P.nu + s_node[ln] : (size_t)3 * P.nu + s_node[ln];
        const bool first = tab[ln * NR + ln] & 0x8000;
        if (first)
          P.r[R] = acc;
        else
          atomicAdd(&P.r[R], acc);
      }
    }
    if (!JAC) continue;
    // P5: Jacobian entries
    TT acc_uu[C::EUU];
    double acc_pu[C::EPU];
#pragma unroll
    for (int j = 0; j < C::EUU; ++j) acc_uu[j] = TT(0);
#pragma unroll
    for (int j = 0; j < C::EPU; ++j) acc_pu[j] = 0.0;
    for (int g = 0; g < NG; ++g) {
      const double* rec = &s_gp[g * C::GPS];
      const double* dpg = &s_dphi[g * NPE * 3];
      // a) tempvecs TEMPVEC = JGW_SUB_MAT * DPHIDZ(:,ns,nh) for the six blocks
      for (int i = tid; i < 6 * NPE; i += C::THREADS) {
        const int blk = i / NPE, b = i % NPE;
        const int nh = blk < 3 ? blk : (blk == 5 ? 1 : 0);
        const int mh = blk < 3 ? blk : (blk == 3 ? 1 : 2);
        const TT jgw = (TT)rec[9];
        TT sub[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const TT cv = (TT)rec[24 + t2v(r, mh) * 6 + t2v(c, nh)];
            sub[r][c] = blk < 3 ? jgw * (cv + (TT)rec[18 + t2v(r, c)]) : jgw * cv;
          }
        const TT d0 = (TT)dpg[b * 3 + 0], d1 = (TT)dpg[b * 3 + 1], d2 = (TT)dpg[b * 3 + 2];
#pragma unroll
        for (int r = 0; r < 3; ++r) s_T[i * 3 + r] = sub[r][0] * d0 + sub[r][1] * d1 + sub[r][2] * d2;
      }
      __syncthreads();
      // b) K(row, col) += DOT_PRODUCT(DPHIDZ(:,ms,mh), TEMPVEC)
#pragma unroll
      for (int j = 0; j < C::EUU; ++j) {
        const int d = e_uu[j];
        if (d >= 0) {
          const int R = d >> 8, Cc = d & 0xff;
          const int m = R / NPE, a = R % NPE, n = Cc / NPE, b = Cc % NPE;
          const TT* tv = &s_T[(blk_of(m, n) * NPE + b) * 3];
          const TT d0 = (TT)dpg[a * 3 + 0], d1 = (TT)dpg[a * 3 + 1], d2 = (TT)dpg[a * 3 + 2];
          acc_uu[j] = acc_uu[j] + (d0 * tv[0] + d1 * tv[1] + d2 * tv[2]);
        }
      }
#pragma unroll
      for (int j = 0; j < C::EPU; ++j) {
        const int d = e_pu[j];
        if (d >= 0) {
          const int q = d >> 8, Cc = d & 0xff;
          const int n = Cc / NPE, b = Cc % NPE;
          const double jd = rec[9] * dpg[b * 3 + n];
          acc_pu[j] = PM ? acc_pu[j] + jd * s_gbfp[g * 8 + q] : acc_pu[j] + jd;
        }
      }
      __syncthreads();
    }
    // P6: scatter the entries and their mirrors
    if (MODE == M_EJAC) {
      double* out = P.elem_out + (size_t)it * NROW * NROW;
#pragma unroll
      for (int j = 0; j < C::EUU; ++j) {
        const int d = e_uu[j];
        if (d >= 0) {
          const int R = d >> 8, Cc = d & 0xff;
          out[(size_t)Cc * NROW + R] = (double)acc_uu[j];
          out[(size_t)R * NROW + Cc] = (double)acc_uu[j];
        }
      }
#pragma unroll
      for (int j = 0; j < C::EPU; ++j) {
        const int d = e_pu[j];
        if (d >= 0) {
          const int R = NU3 + (d >> 8), Cc = d & 0xff;
          out[(size_t)Cc * NROW + R] = acc_pu[j];
          out[(size_t)R * NROW + Cc] = acc_pu[j];
        }
      }
      for (int i = tid; i < NPP * NPP; i += C::THREADS) out[(size_t)(NU3 + i / NPP) * NROW + NU3 + i % NPP] = 0.0;
      continue;
    }
    const int nu = P.nu;
#pragma unroll
    for (int j = 0; j < C::EUU; ++j) {
      const int d = e_uu[j];
      if (d >= 0) {
        const int R = d >> 8, Cc = d & 0xff;
        const int m = R / NPE, a = R % NPE, n = Cc / NPE, b = Cc % NPE;
        const int na = s_node[a], nb = s_node[b];
        const uint16_t tab_ab = tab[a * NR + b], tab_ba = tab[b * NR + a];
        const TT v = acc_uu[j];
        if (MIX) {
          const size_t p1 = (size_t)P.uu_row_ptr[(size_t)m * nu + na] + (size_t)n * P.wu[na] + (tab_ab & 0x7fff);
          if (tab_ab & 0x8000)
            P.vals_uu[p1] = (float)v;
          else
            atomicAdd(&P.vals_uu[p1], (float)v);
          if (R != Cc) {
            const size_t p2 = (size_t)P.uu_row_ptr[(size_t)n * nu + nb] + (size_t)m * P.wu[nb] + (tab_ba & 0x7fff);
            if (tab_ba & 0x8000)
              P.vals_uu[p2] = (float)v;
            else
              atomicAdd(&P.vals_uu[p2], (float)v);
          }
        } else {
          const size_t p1 = (size_t)P.row_ptr[(size_t)m * nu + na] + (size_t)n * P.wu[na] + (tab_ab & 0x7fff);
          if (tab_ab & 0x8000)
            P.vals[p1] = (double)v;
          else
            atomicAdd(&P.vals[p1], (double)v);
          if (R != Cc) {
            const size_t p2 = (size_t)P.row_ptr[(size_t)n * nu + nb] + (size_t)m * P.wu[nb] + (tab_ba & 0x7fff);
            if (tab_ba & 0x8000)
              P.vals[p2] = (double)v;
            else
              atomicAdd(&P.vals[p2], (double)v);
          }
        }
      }
    }
    const int32_t* rp = MIX ? P.cp_row_ptr : P.row_ptr;
#pragma unroll
    for (int j = 0; j < C::EPU; ++j) {
      const int d = e_pu[j];
      if (d >= 0) {
        const int q = d >> 8, Cc = d & 0xff;
        const int n = Cc / NPE, b = Cc % NPE;
        const int lq = NPE + q;
        const int pq = s_node[lq], nb = s_node[b];
        const uint16_t t_qb = tab[lq * NR + b], t_bq = tab[b * NR + lq];
        const double v = acc_pu[j];
        const size_t p1 = (size_t)rp[(size_t)3 * nu + pq] + (size_t)n * P.wp[pq] + (t_qb & 0x7fff);
        if ((t_qb & 0x8000))
          P.vals[p1] = v;
        else
          atomicAdd(&P.vals[p1], v);
        // mirror: displacement row (n, b), pressure column q
        const size_t p2 = MIX ? (size_t)rp[(size_t)n * nu + nb] + (t_bq & 0x7fff)
                              : (size_t)rp[(size_t)n * nu + nb] + 3 * (size_t)P.wu[nb] + (t_bq & 0x7fff);
        if ((t_bq & 0x8000))
          P.vals[p2] = v;
        else
          atomicAdd(&P.vals[p2], v);
      }
    }
    // structurally zero pressure-pressure entries: stored by their first contributor
    for (int i = tid; i < NPP * NPP; i += C::THREADS) {
      const int lq = NPE + i / NPP, lq2 = NPE + i % NPP;
      const uint16_t t = tab[lq * NR + lq2];
      if (t & 0x8000) {
        const int pq = s_node[lq];
        const size_t pos = MIX ? (size_t)rp[(size_t)3 * nu + pq] + 3 * (size_t)P.wp[pq] + (t & 0x7fff)
                               : (size_t)rp[(size_t)3 * nu + pq] + 3 * (size_t)P.wp[pq] + (t & 0x7fff);
        P.vals[pos] = 0.0;
      }
    }
  }
}

// ------------------------------------------------------------ handle ----
template <class T>
int dev_upload(T** dst, const std::vector<T>& src) {
  *dst = nullptr;
  if (src.empty()) return FE_NO_ERROR;
  CUDA_TRY(cudaMalloc(dst, src.size() * sizeof(T)));
  CUDA_TRY(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return FE_NO_ERROR;
}

}  // namespace

// Device arrays that depend only on the mesh (connectivity, pattern, rank
// tables, geometry cache, quadrature, colouring, incidence lists): owned
// together and shared by the handles fe_clone makes from one set-up.
struct SharedDeviceSetup {
  std::vector<void*> ptrs;
  ~SharedDeviceSetup() {
    for (void* p : ptrs)
      if (p) cudaFree(p);
  }
};

struct fe_equations_set {
  HostSetup hs;
  std::shared_ptr<SharedDeviceSetup> shared;
  int device = 0;
  int num_sms = 0;
  int32_t *d_elem_u = nullptr, *d_elem_p = nullptr, *d_row_ptr = nullptr, *d_uu_row_ptr = nullptr,
          *d_cp_row_ptr = nullptr, *d_wu = nullptr, *d_wp = nullptr, *d_elem_table = nullptr,
          *d_colour_elems = nullptr;
  uint16_t* d_tables = nullptr;
  double *d_geo = nullptr, *d_mat = nullptr, *d_gbf_u = nullptr, *d_gbf_p = nullptr, *d_gw = nullptr;
  float* d_geo_dd = nullptr;
  double* d_surfp = nullptr;
  int32_t* d_bnd_elems = nullptr;
  uint8_t* d_bnd_mask = nullptr;
  bool has_surfp = false;
  int high_precision = FE_HIGH_PRECISION_FP64;
  int assembly_order = FE_ASSEMBLY_STAGED;
  // staged assembly: incidence lists (uploaded at creation) and the
  // per-element records (allocated on the first staged evaluation)
  int32_t *d_u_inc_ptr = nullptr, *d_u_inc = nullptr, *d_p_inc_ptr = nullptr, *d_p_inc = nullptr;
  float* d_st_uu = nullptr;
  double *d_st_cp = nullptr, *d_st_r = nullptr;
  int* d_fuse = nullptr;  // fused staged assembly: [0, kFuseChunks) group counters, then per-row-node counts
  int host_output = FE_HOST_OUTPUT_STREAMED;
  int stream_chunks = 0;  // launches of a streamed assembly; 0: equal runs of whole waves
  // streamed host outputs: the copy stream and one event per chunk (+ the last copy)
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> chunk_events;
  unsigned* d_status = nullptr;
  int32_t* d_col = nullptr;  // CSR columns on the device, uploaded on first use (Newton driver)
  // staging for calls given host memory
  double *s_x = nullptr, *s_r = nullptr, *s_vals = nullptr, *s_cp = nullptr, *s_elem = nullptr;
  float* s_uu = nullptr;
  size_t s_elem_bytes = 0;
  int64_t launches = 0;
  std::mutex mu;
};

struct fe_batch_s {
  std::vector<fe_handle> members;
  int device = 0;
  int num_sms = 0;
  int ncol = 0;                       // colours: the most of any member
  std::vector<int32_t> slot_member;   // member of each constant-table slot (slots ordered by element type)
  cmfe::BatchMember* h_table = nullptr;   // pinned host copy of the member table
  cmfe::BatchMember* d_table = nullptr;   // device copy, source of the constant table for direct launches
  cmfe::BatchMember* d_table_graph = nullptr;  // snapshot taken at capture, source for graph replays
  bool table_dirty = true;
  int32_t* d_offsets = nullptr;       // [slot][2][ncol + 1]: colour element offsets, boundary element offsets
  std::vector<const void*> surf_sig;  // per member: d_surfp when loaded, else NULL
  unsigned* d_sync = nullptr;         // [0] barrier count, [1] barrier generation, [2] status
  int variant = 1, ctas_per_sm = 2, block_groups = 1;
  unsigned barrier_polls = 0, barrier_extra = 0;  // grid-barrier limits (fe_batch_set_barrier_limits)
  unsigned type_mask = 0;             // element types present (bit 4: surface loads)
  double tuned_ms = -1.0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int64_t graph_kernels = 0;  // kernels in the captured graph
  int64_t launches = 0;
  std::mutex mu;
};

namespace {

template <int N1, int PM, int MODE>
int launch_t(fe_handle h, KParams& kp, cudaStream_t st) {
  using C = Cfg<N1, PM>;
  static std::atomic<bool> attr_done[64];
  auto kern = fe_element_kernel<N1, PM, MODE>;
  const int dev = h->device;
  if (!attr_done[dev & 63]) {
    CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM));
    attr_done[dev & 63] = true;
  }
  int per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::THREADS, C::SMEM));
  if (per_sm < 1) per_sm = 1;
  const int grid = std::max(1, std::min(kp.count, per_sm * h->num_sms));
  kern<<<grid, C::THREADS, C::SMEM, st>>>(kp);
  CUDA_TRY(cudaGetLastError());
  h->launches++;
  return FE_NO_ERROR;
}

template <int MODE>
int launch(fe_handle h, KParams& kp, cudaStream_t st) {
  const auto& s = h->hs;
  if (kp.count <= 0) return FE_NO_ERROR;
  if (s.n1 == 2 && s.pmode == 0) return launch_t<2, 0, MODE>(h, kp, st);
  if (s.n1 == 2 && s.pmode == 1) return launch_t<2, 1, MODE>(h, kp, st);
  if (s.n1 == 3 && s.pmode == 0) return launch_t<3, 0, MODE>(h, kp, st);
  return launch_t<3, 1, MODE>(h, kp, st);
}

KParams base_params(fe_handle h) {
  KParams k;
  std::memset(&k, 0, sizeof(k));
  const auto& s = h->hs;
  k.nu = s.nu;
  k.law = s.law;
  k.nmat = s.nmat;
  k.matpe = s.mat_per_element;
  k.elem_u = h->d_elem_u;
  k.elem_p = h->d_elem_p;
  k.geo = h->d_geo;
  k.geo_dd = h->d_geo_dd;
  k.nr = s.nr;
  k.pmode = s.pmode;
  k.surf_p = h->d_surfp;
  k.mat = h->d_mat;
  k.gbf_u = h->d_gbf_u;
  k.gbf_p = h->d_gbf_p;
  k.gw = h->d_gw;
  k.row_ptr = h->d_row_ptr;
  k.uu_row_ptr = h->d_uu_row_ptr;
  k.cp_row_ptr = h->d_cp_row_ptr;
  k.wu = h->d_wu;
  k.wp = h->d_wp;
  k.tables = h->d_tables;
  k.elem_table = h->d_elem_table;
  k.status = h->d_status;
  return k;
}

// Surface-pressure contributions of the boundary elements of colour c, after
// that colour's volume kernel (no-op without surface pressure).
int surface_after(fe_handle h, const KParams& kp, int c, int want_jac, cudaStream_t st) {
  const auto& s = h->hs;
  if (!h->has_surfp) return FE_NO_ERROR;
  const int nb = s.bnd_ptr[c + 1] - s.bnd_ptr[c];
  if (nb == 0) return FE_NO_ERROR;
  const int e = cmfe::launch_surface(s, kp, h->d_bnd_elems + s.bnd_ptr[c], h->d_bnd_mask, nb, 0, want_jac,
                                     h->num_sms, st);
  if (e != 0) return set_error(FE_ERR_CUDA, std::string("surface kernel launch: ") + cudaGetErrorString((cudaError_t)e));
  h->launches++;
  return FE_NO_ERROR;
}

int ensure(void** buf, size_t bytes);

// Group counters at the head of d_fuse: the most launches one fused assembly
// is split into.
constexpr int kFuseChunks = 64;
// The most chunks a streamed assembly is split into, and the most the
// default plan uses.
constexpr int kStreamChunks = 16;
constexpr int kStreamAuto = 12;

// The fused staged assembly (element records and row gathers in one kernel)
// in launches over consecutive ranges of element groups, launch c taking
// groups [bounds[c], bounds[c + 1]); when `done` is given, done[c] is
// recorded on the stream after launch c.  The per-node counts run on across
// the launches: a node's rows are gathered by the launch that assembles the
// last element around it.
int mixed_fused(fe_handle h, const KParams& kp, const cmfe::StageOut& so, bool double_float, cudaStream_t st,
                const std::vector<int64_t>& bounds, cudaEvent_t* done, int64_t* count) {
  const auto& s = h->hs;
  int rc;
  const int chunks = (int)bounds.size() - 1;
  if (chunks < 1 || chunks > kFuseChunks) return set_error(FE_ERR_INVALID_ARGUMENT, "fused launches: 1..64");
  const size_t counters = kFuseChunks + (size_t)s.nu + (size_t)s.npn;
  if ((rc = ensure((void**)&h->d_fuse, sizeof(int) * counters))) return rc;
  CUDA_TRY(cudaMemsetAsync(h->d_fuse, 0, sizeof(int) * counters, st));
  const int nb = s.bnd_ptr.empty() ? 0 : s.bnd_ptr[s.ncolours];
  cmfe::FusedArgs fa;
  std::memset(&fa, 0, sizeof(fa));
  fa.u_inc_ptr = h->d_u_inc_ptr;
  fa.u_inc = h->d_u_inc;
  fa.p_inc_ptr = h->d_p_inc_ptr;
  fa.p_inc = h->d_p_inc;
  fa.node_done = h->d_fuse + kFuseChunks;
  fa.bmask = h->has_surfp && nb > 0 ? h->d_bnd_mask : nullptr;
  for (int c = 0; c < chunks; ++c) {
    fa.work = h->d_fuse + c;
    fa.g0 = (int)bounds[c];
    fa.g1 = (int)bounds[c + 1];
    const int e = cmfe::launch_mixed_fused(s, kp, so, fa, h->num_sms, st, double_float);
    if (e != 0)
      return set_error(FE_ERR_CUDA, std::string("fused kernel launch: ") + cudaGetErrorString((cudaError_t)e));
    if (done) CUDA_TRY(cudaEventRecord(done[c], st));
  }
  h->launches += chunks;
  if (count) *count += chunks;
  return FE_NO_ERROR;
}

int64_t fused_groups(const HostSetup& s) {
  const int eg = cmfe::fused_group_size(s);
  return (s.ne + eg - 1) / eg;
}

int ensure_records(fe_handle h) {
  const auto& s = h->hs;
  int rc;
  if ((rc = ensure((void**)&h->d_st_uu, sizeof(float) * cmfe::rec_stride_uu(s.npe) * (size_t)s.ne)) ||
      (rc = ensure((void**)&h->d_st_cp, sizeof(double) * cmfe::rec_stride_cp(s.npe, s.npp) * (size_t)s.ne)) ||
      (rc = ensure((void**)&h->d_st_r, sizeof(double) * cmfe::rec_stride_r(s.npe, s.npp) * (size_t)s.ne)))
    return rc;
  return FE_NO_ERROR;
}

KParams staged_params(fe_handle h, const double* dx, float* du, double* dc, double* dr) {
  KParams kp = base_params(h);
  kp.x = dx;
  kp.vals_uu = du;
  kp.vals = dc;
  kp.r = dr;
  kp.elems = nullptr;
  kp.first_elem = 0;
  kp.count = h->hs.ne;
  return kp;
}

// The staged mixed assembly into device buffers: one launch over all
// elements into the per-element records, the surface-pressure faces added to
// the records of their elements, then the row gather (or all three in the
// fused kernel where its gather scratch fits).  Adds the number of kernels
// launched to *count when count is set.
int mixed_staged(fe_handle h, const double* dx, float* du, double* dc, double* dr, bool double_float,
                 cudaStream_t st, int64_t* count) {
  const auto& s = h->hs;
  int rc;
  if ((rc = ensure_records(h))) return rc;
  const KParams kp = staged_params(h, dx, du, dc, dr);
  const cmfe::StageOut so{h->d_st_uu, h->d_st_cp, h->d_st_r};
  if (cmfe::fused_fits(s)) return mixed_fused(h, kp, so, double_float, st, {0, fused_groups(s)}, nullptr, count);
  const int nb = s.bnd_ptr.empty() ? 0 : s.bnd_ptr[s.ncolours];
  int e = cmfe::launch_mixed_staged(s, kp, so, h->num_sms, st, double_float);
  if (e != 0) return set_error(FE_ERR_CUDA, std::string("staged kernel launch: ") + cudaGetErrorString((cudaError_t)e));
  int64_t n = 1;
  if (h->has_surfp && nb > 0) {
    e = cmfe::launch_surface(s, kp, h->d_bnd_elems, h->d_bnd_mask, nb, 2, 1, h->num_sms, st, so);
    if (e != 0) return set_error(FE_ERR_CUDA, std::string("surface kernel launch: ") + cudaGetErrorString((cudaError_t)e));
    ++n;
  }
  e = cmfe::launch_gather(s, kp, so, h->d_u_inc_ptr, h->d_u_inc, h->d_p_inc_ptr, h->d_p_inc, h->num_sms, st);
  if (e != 0) return set_error(FE_ERR_CUDA, std::string("gather kernel launch: ") + cudaGetErrorString((cudaError_t)e));
  ++n;
  h->launches += n;
  if (count) *count += n;
  return FE_NO_ERROR;
}

// Streamed host outputs: the fused assembly in chunks of element groups into
// the device buffers du / dc / dr; after each chunk, the rows it completed --
// the leading u nodes and pressure row nodes whose elements are all assembled,
// in each of the row blocks -- are copied to the host outputs hu / hc / hr
// (NULL: that output is device memory, written directly) on a copy stream,
// while the next chunks assemble.  The caller's stream waits for the last copy.
int mixed_streamed(fe_handle h, const double* dx, float* du, double* dc, double* dr, float* hu, double* hc,
                   double* hr, bool double_float, cudaStream_t st) {
  const auto& s = h->hs;
  int rc;
  if ((rc = ensure_records(h))) return rc;
  const int64_t groups = fused_groups(s);
  const int wave = cmfe::fused_wave(s, h->num_sms, double_float);
  if (wave <= 0)
    return set_error(FE_ERR_CUDA, std::string("fused kernel occupancy: ") + cudaGetErrorString((cudaError_t)-wave));
  // By default the launch boundaries fall on whole waves of the resident
  // blocks, so that no launch but the last ends with part of the GPU idle:
  // equal runs of waves, at most kStreamAuto launches (each launch adds seven
  // copies to the copy stream; smaller first launches do not start the copies
  // sooner, since a node's rows complete only with the next layer of
  // elements).  An explicit count splits the groups evenly.
  std::vector<int64_t> bounds{0};
  const int64_t waves = (groups + wave - 1) / wave;
  if (h->stream_chunks > 0) {
    for (int c = 1; c <= h->stream_chunks; ++c) {
      const int64_t g = groups * c / h->stream_chunks;
      if (g > bounds.back()) bounds.push_back(g);
    }
  } else {
    const int64_t run = std::max<int64_t>(1, (waves + kStreamAuto - 1) / kStreamAuto);
    for (int64_t g = std::min<int64_t>(run * wave, groups); bounds.back() < groups;
         g = std::min<int64_t>(g + run * wave, groups))
      bounds.push_back(g);
  }
  const int chunks = (int)bounds.size() - 1;
  if (!h->copy_stream) CUDA_TRY(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  while ((int)h->chunk_events.size() < kStreamChunks + 1) {
    cudaEvent_t ev;
    CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    h->chunk_events.push_back(ev);
  }
  const KParams kp = staged_params(h, dx, du, dc, dr);
  const cmfe::StageOut so{h->d_st_uu, h->d_st_cp, h->d_st_r};
  cudaEvent_t* ev = h->chunk_events.data();
  if ((rc = mixed_fused(h, kp, so, double_float, st, bounds, ev, nullptr))) return rc;
  cudaStream_t cs = h->copy_stream;
  const int nu = s.nu, npn = s.npn, EG = cmfe::fused_group_size(s);
  auto copy_rows = [&](int64_t r0, int64_t r1) -> int {
    if (r1 <= r0) return FE_NO_ERROR;
    if (hu && r0 < 3 * (int64_t)nu) {
      const int64_t a = s.uu_row_ptr[r0], b = s.uu_row_ptr[r1];
      if (b > a) CUDA_TRY(cudaMemcpyAsync(hu + a, du + a, sizeof(float) * (b - a), cudaMemcpyDeviceToHost, cs));
    }
    if (hc) {
      const int64_t a = s.cp_row_ptr[r0], b = s.cp_row_ptr[r1];
      if (b > a) CUDA_TRY(cudaMemcpyAsync(hc + a, dc + a, sizeof(double) * (b - a), cudaMemcpyDeviceToHost, cs));
    }
    return FE_NO_ERROR;
  };
  int a0 = 0, q0 = 0;
  for (int c = 0; c < chunks; ++c) {
    const int64_t end = std::min<int64_t>(bounds[c + 1] * EG, s.ne);  // elements assembled
    int a1 = nu, q1 = npn;
    if (c + 1 < chunks) {
      a1 = (int)(std::upper_bound(s.u_last_prefix.begin(), s.u_last_prefix.end(), (int32_t)(end - 1)) -
                 s.u_last_prefix.begin());
      q1 = (int)(std::upper_bound(s.p_last_prefix.begin(), s.p_last_prefix.end(), (int32_t)(end - 1)) -
                 s.p_last_prefix.begin());
    }
    if (a1 == a0 && q1 == q0) continue;
    CUDA_TRY(cudaStreamWaitEvent(cs, ev[c], 0));
    for (int m = 0; m < 3; ++m)
      if ((rc = copy_rows((int64_t)m * nu + a0, (int64_t)m * nu + a1))) return rc;
    if ((rc = copy_rows(3 * (int64_t)nu + q0, 3 * (int64_t)nu + q1))) return rc;
    a0 = a1;
    q0 = q1;
  }
  // the residual (one value per row: small) in one copy after the last launch
  if (hr) {
    CUDA_TRY(cudaStreamWaitEvent(cs, ev[chunks - 1], 0));
    CUDA_TRY(cudaMemcpyAsync(hr, dr, sizeof(double) * (size_t)s.ndofs, cudaMemcpyDeviceToHost, cs));
  }
  CUDA_TRY(cudaEventRecord(ev[kStreamChunks], cs));
  CUDA_TRY(cudaStreamWaitEvent(st, ev[kStreamChunks], 0));
  return FE_NO_ERROR;
}

// Colour-by-colour launches over all elements.
template <int MODE>
int run_colours(fe_handle h, KParams kp, cudaStream_t st) {
  const auto& s = h->hs;
  for (int c = 0; c < s.ncolours; ++c) {
    kp.elems = h->d_colour_elems + s.colour_ptr[c];
    kp.count = s.colour_ptr[c + 1] - s.colour_ptr[c];
    int rc = launch<MODE>(h, kp, st);
    if (rc) return rc;
    if ((rc = surface_after(h, kp, c, MODE == M_JAC, st))) return rc;
  }
  return FE_NO_ERROR;
}

// The mixed assembly of one equations set into device buffers: one launch
// per colour, each followed by that colour's surface-pressure faces.  Adds
// the number of kernels launched to *count when count is set.
int mixed_colours(fe_handle h, const double* dx, float* du, double* dc, double* dr, bool double_float,
                  cudaStream_t st, int64_t* count);

// The mixed assembly in the handle's assembly order.
int mixed_assemble(fe_handle h, const double* dx, float* du, double* dc, double* dr, bool double_float,
                   cudaStream_t st, int64_t* count) {
  if (h->assembly_order == FE_ASSEMBLY_STAGED && h->hs.gather_bytes > 0)
    return mixed_staged(h, dx, du, dc, dr, double_float, st, count);
  return mixed_colours(h, dx, du, dc, dr, double_float, st, count);
}

int mixed_colours(fe_handle h, const double* dx, float* du, double* dc, double* dr, bool double_float,
                  cudaStream_t st, int64_t* count) {
  KParams kp = base_params(h);
  kp.x = dx;
  kp.vals_uu = du;
  kp.vals = dc;
  kp.r = dr;
  for (int c = 0; c < h->hs.ncolours; ++c) {
    kp.elems = h->d_colour_elems + h->hs.colour_ptr[c];
    kp.count = h->hs.colour_ptr[c + 1] - h->hs.colour_ptr[c];
    const int e = cmfe::launch_mixed(h->hs, kp, h->num_sms, st, double_float);
    if (e != 0) return set_error(FE_ERR_CUDA, std::string("mixed kernel launch: ") + cudaGetErrorString((cudaError_t)e));
    if (kp.count > 0) {
      h->launches++;
      if (count) ++*count;
    }
    const int64_t before = h->launches;
    int rc = surface_after(h, kp, c, 1, st);
    if (rc) return rc;
    if (count) *count += h->launches - before;
  }
  return FE_NO_ERROR;
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Page-locked host memory that the device can address (cudaHostAlloc,
// cudaHostRegister, or torch's pinned tensors): *dptr receives the address
// kernels use for it (under unified addressing, the host address itself).
bool mapped_host_ptr(const void* p, void** dptr) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
  *dptr = a.devicePointer;
  return true;
}

int ensure(void** buf, size_t bytes) {
  if (*buf) return FE_NO_ERROR;
  cudaError_t e = cudaMalloc(buf, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *buf = nullptr;
    return set_error(FE_ERR_OUT_OF_MEMORY, std::string("device staging allocation failed: ") + cudaGetErrorString(e));
  }
  return FE_NO_ERROR;
}

int check_handle(fe_handle h) {
  if (!h) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL handle");
  int cur = 0;
  CUDA_TRY(cudaGetDevice(&cur));
  if (cur != h->device) return set_error(FE_ERR_INVALID_ARGUMENT, "handle belongs to another CUDA device");
  return FE_NO_ERROR;
}

// Stages x to the device if it is host memory.
int stage_in(fe_handle h, const double* x, const double** dx, cudaStream_t st, bool* host) {
  *host = !is_device_ptr(x);
  if (!*host) {
    *dx = x;
    return FE_NO_ERROR;
  }
  int rc = ensure((void**)&h->s_x, sizeof(double) * h->hs.ndofs);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(h->s_x, x, sizeof(double) * h->hs.ndofs, cudaMemcpyHostToDevice, st));
  *dx = h->s_x;
  return FE_NO_ERROR;
}

int finish_status(fe_handle h, cudaStream_t st) {
  unsigned v = 0;
  CUDA_TRY(cudaMemcpyAsync(&v, h->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned), st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (v) return set_error(FE_ERR_NUMERICAL, "a Gauss point had det F <= 0 or a non-finite stress");
  return FE_NO_ERROR;
}

}  // namespace

namespace {

int member_type(const HostSetup& s) { return (s.n1 == 3 ? 2 : 0) + (s.pmode ? 1 : 0); }

// The batched kernel reads the member table from the batch module's constant
// memory: launches of all batches on a device are serialised through one
// event per device, so that no launch overwrites the table while another
// batch's kernel still reads it.
std::mutex g_batch_mu;
cudaEvent_t g_batch_event[64] = {};

int batch_serialise_begin(int device, cudaStream_t st) {
  if (device < 0 || device >= 64) return set_error(FE_ERR_NOT_SUPPORTED, "device ordinal out of range");
  if (!g_batch_event[device]) CUDA_TRY(cudaEventCreateWithFlags(&g_batch_event[device], cudaEventDisableTiming));
  CUDA_TRY(cudaStreamWaitEvent(st, g_batch_event[device], 0));
  return FE_NO_ERROR;
}

int batch_serialise_end(int device, cudaStream_t st) {
  CUDA_TRY(cudaEventRecord(g_batch_event[device], st));
  return FE_NO_ERROR;
}

// Sets the per-call output pointers of every slot (uploaded with the table).
int batch_set_pointers(fe_batch b, const double* const* x, float* const* uu, double* const* cp, double* const* r,
                       cudaStream_t st) {
  (void)st;
  const size_t n = b->members.size();
  for (size_t m = 0; m < n; ++m) {
    if (!x[m] || !uu[m] || !cp[m]) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL member pointer");
    if (!is_device_ptr(x[m]) || !is_device_ptr(uu[m]) || !is_device_ptr(cp[m]) || (r && r[m] && !is_device_ptr(r[m])))
      return set_error(FE_ERR_INVALID_ARGUMENT, "batched evaluation takes device pointers only");
  }
  for (size_t s = 0; s < n; ++s) {
    const int m = b->slot_member[s];
    KParams& k = b->h_table[s].kp;
    double* rr = r ? r[m] : nullptr;
    if (k.x != x[m] || k.r != rr || k.vals != cp[m] || k.vals_uu != uu[m]) {
      k.x = x[m];
      k.r = rr;
      k.vals = cp[m];
      k.vals_uu = uu[m];
      b->table_dirty = true;
    }
  }
  return FE_NO_ERROR;
}

// Surface-pressure state of the members (pressure pointer per slot).
int refresh_surface(fe_batch b) {
  const size_t n = b->members.size();
  std::vector<const void*> sig(n);
  for (size_t m = 0; m < n; ++m) sig[m] = b->members[m]->has_surfp ? (const void*)b->members[m]->d_surfp : nullptr;
  if (sig == b->surf_sig) return FE_NO_ERROR;
  bool any = false;
  for (size_t s = 0; s < n; ++s) {
    const int m = b->slot_member[s];
    b->h_table[s].kp.surf_p = static_cast<const double*>(sig[m]);
    b->h_table[s].has_surface = sig[m] != nullptr;
    any = any || sig[m] != nullptr;
  }
  b->type_mask = any ? (b->type_mask | 16u) : (b->type_mask & 15u);
  b->surf_sig = sig;
  b->table_dirty = true;
  return FE_NO_ERROR;
}

// Uploads the host member table to its device copy when it changed.
int sync_table(fe_batch b, cudaStream_t st) {
  if (!b->table_dirty) return FE_NO_ERROR;
  const size_t bytes = b->members.size() * sizeof(cmfe::BatchMember);
  // the pinned table is rewritten by a later call: wait for this copy
  CUDA_TRY(cudaMemcpyAsync(b->d_table, b->h_table, bytes, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  b->table_dirty = false;
  return FE_NO_ERROR;
}

// One batched launch on st; table is the device copy of the member table the
// launch copies into constant memory.
int batch_launch_from(fe_batch b, const cmfe::BatchMember* table, cudaStream_t st) {
  if (b->variant == cmfe::batch_variants()) {
    // one launch per member and colour: the single-set kernels, in member order
    for (size_t s = 0; s < b->members.size(); ++s) {
      const KParams& k = b->h_table[s].kp;
      fe_handle h = b->members[b->slot_member[s]];
      std::lock_guard<std::mutex> lk(h->mu);
      const int rc = mixed_assemble(h, k.x, k.vals_uu, k.vals, k.r, false, st, &b->launches);
      if (rc) return rc;
    }
    return FE_NO_ERROR;
  }
  CUDA_TRY(cudaMemsetAsync(b->d_sync, 0, 2 * sizeof(unsigned), st));
  cmfe::BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.offsets = b->d_offsets;
  a.nmembers = (int)b->members.size();
  a.ncolours = b->ncol;
  a.block_groups = b->block_groups;
  a.bar_count = b->d_sync;
  a.bar_gen = b->d_sync + 1;
  a.status = b->d_sync + 2;
  a.barrier_polls = b->barrier_polls;
  a.barrier_extra = b->barrier_extra;
  const int e = cmfe::launch_mixed_batch(b->variant, b->type_mask, table, (int)b->members.size(), a, b->ctas_per_sm,
                                         b->num_sms, st);
  if (e != 0) return set_error(FE_ERR_CUDA, std::string("batched kernel launch: ") + cudaGetErrorString((cudaError_t)e));
  b->launches++;
  return FE_NO_ERROR;
}

int batch_launch(fe_batch b, cudaStream_t st) {
  int rc = refresh_surface(b);
  if (rc || (rc = sync_table(b, st))) return rc;
  std::lock_guard<std::mutex> lk(g_batch_mu);
  if ((rc = batch_serialise_begin(b->device, st))) return rc;
  rc = batch_launch_from(b, b->d_table, st);
  const int rc2 = batch_serialise_end(b->device, st);
  return rc ? rc : rc2;
}

int check_batch(fe_batch b) {
  if (!b) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL batch");
  int cur = 0;
  CUDA_TRY(cudaGetDevice(&cur));
  if (cur != b->device) return set_error(FE_ERR_INVALID_ARGUMENT, "batch belongs to another CUDA device");
  return FE_NO_ERROR;
}

}  // namespace

// Staging array of fe_residual_evaluate_noalloc: x in the first half, r in
// the second.  Part of the module's device image, so using it allocates nothing.
static __device__ __align__(256) double g_noalloc_scratch[2 * (size_t)FE_NOALLOC_MAX_DOFS];

namespace {

std::mutex g_noalloc_mu;           // one scratch array per device: calls are serialised
double* g_noalloc_addr[64] = {};   // its device address, per device ordinal

int noalloc_scratch(int device, double** out) {
  if (device < 0 || device >= 64) return set_error(FE_ERR_NOT_SUPPORTED, "device ordinal out of range");
  if (!g_noalloc_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_error(FE_ERR_CUDA, std::string("scratch address lookup: ") + cudaGetErrorString(e));
    g_noalloc_addr[device] = static_cast<double*>(p);
  }
  *out = g_noalloc_addr[device];
  return FE_NO_ERROR;
}

}  // namespace

namespace cmfe {
int record_error(int code, const std::string& msg) { return set_error(code, msg); }

int device_pattern(fe_handle h, const int32_t** row_ptr, const int32_t** col, int64_t* ndofs, int64_t* nnz,
                   int64_t* nu3) {
  if (!h) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL handle");
  std::lock_guard<std::mutex> lk(h->mu);
  if (!h->d_col) {
    CUDA_TRY(cudaMalloc(&h->d_col, sizeof(int32_t) * h->hs.col.size()));
    CUDA_TRY(cudaMemcpy(h->d_col, h->hs.col.data(), sizeof(int32_t) * h->hs.col.size(), cudaMemcpyHostToDevice));
  }
  *row_ptr = h->d_row_ptr;
  *col = h->d_col;
  *ndofs = h->hs.ndofs;
  *nnz = h->hs.nnz;
  *nu3 = 3 * (int64_t)h->hs.nu;
  return FE_NO_ERROR;
}
}  // namespace cmfe

namespace {
// The mesh-only device arrays of a handle (shared with its clones).
std::vector<void*> shared_arrays(fe_handle h) {
  return {h->d_bnd_elems, h->d_bnd_mask, h->d_geo_dd, h->d_elem_u, h->d_elem_p, h->d_row_ptr, h->d_uu_row_ptr,
          h->d_cp_row_ptr, h->d_wu, h->d_wp, h->d_elem_table, h->d_colour_elems, h->d_tables, h->d_geo,
          h->d_gbf_u, h->d_gbf_p, h->d_gw, h->d_u_inc_ptr, h->d_u_inc, h->d_p_inc_ptr, h->d_p_inc};
}
}  // namespace

extern "C" {

int fe_last_error(char* buf, int32_t size) {
  if (!buf || size <= 0) return FE_ERR_INVALID_ARGUMENT;
  std::snprintf(buf, (size_t)size, "%s", g_last_error.c_str());
  return FE_NO_ERROR;
}

int fe_create(const fe_mesh_desc* desc, fe_handle* out) {
  if (!out) return set_error(FE_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  fe_handle h = new (std::nothrow) fe_equations_set();
  if (!h) return set_error(FE_ERR_OUT_OF_MEMORY, "host allocation failed");
  std::string msg;
  int rc = cmfe::build_setup(desc, h->hs, msg);
  if (rc) {
    delete h;
    return set_error(rc, msg);
  }
  auto fail = [&](int code) {
    fe_destroy(h);
    return code;
  };
  if (cudaGetDevice(&h->device) != cudaSuccess) return fail(set_error(FE_ERR_CUDA, "no CUDA device"));
  if (cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess)
    return fail(set_error(FE_ERR_CUDA, "cannot query the device"));
  const auto& s = h->hs;
  if ((rc = dev_upload(&h->d_elem_u, s.elem_u)) || (rc = dev_upload(&h->d_elem_p, s.elem_p)) ||
      (rc = dev_upload(&h->d_row_ptr, s.row_ptr)) || (rc = dev_upload(&h->d_uu_row_ptr, s.uu_row_ptr)) ||
      (rc = dev_upload(&h->d_cp_row_ptr, s.cp_row_ptr)) || (rc = dev_upload(&h->d_wu, s.wu)) ||
      (rc = dev_upload(&h->d_wp, s.wp)) || (rc = dev_upload(&h->d_elem_table, s.elem_table)) ||
      (rc = dev_upload(&h->d_colour_elems, s.colour_elems)) || (rc = dev_upload(&h->d_tables, s.tables)) ||
      (rc = dev_upload(&h->d_geo, s.geo)) || (rc = dev_upload(&h->d_mat, s.mat)) ||
      (rc = dev_upload(&h->d_gbf_u, s.gbf_u)) || (rc = dev_upload(&h->d_gbf_p, s.gbf_p)) ||
      (rc = dev_upload(&h->d_gw, s.gw)))
    return fail(rc);
  {
    std::vector<float> gdd(s.geo.size() * 2);
    for (size_t i = 0; i < s.geo.size(); ++i) {
      const float hi = (float)s.geo[i];
      gdd[2 * i] = hi;
      gdd[2 * i + 1] = (float)(s.geo[i] - (double)hi);
    }
    if ((rc = dev_upload(&h->d_geo_dd, gdd))) return fail(rc);
  }
  if ((rc = dev_upload(&h->d_bnd_elems, s.bnd_elems)) || (rc = dev_upload(&h->d_bnd_mask, s.bnd_mask))) return fail(rc);
  if ((rc = dev_upload(&h->d_u_inc_ptr, s.u_inc_ptr)) || (rc = dev_upload(&h->d_u_inc, s.u_inc)) ||
      (rc = dev_upload(&h->d_p_inc_ptr, s.p_inc_ptr)) || (rc = dev_upload(&h->d_p_inc, s.p_inc)))
    return fail(rc);
  {
    auto owner = std::make_shared<SharedDeviceSetup>();
    owner->ptrs = shared_arrays(h);
    h->shared = owner;
  }
  if (cudaMalloc(&h->d_status, sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(h->d_status, 0, sizeof(unsigned)) != cudaSuccess)
    return fail(set_error(FE_ERR_CUDA, "status allocation failed"));
  {
    // Resolving the address of the allocation-free entry point's array loads
    // the module that holds it, which commits its 16 MiB on this device now,
    // at handle creation, rather than inside a later allocation-free call.
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    double* scratch = nullptr;
    if ((rc = noalloc_scratch(h->device, &scratch))) return fail(rc);
  }
  *out = h;
  return FE_NO_ERROR;
}

int fe_destroy(fe_handle h) {
  if (!h) return FE_NO_ERROR;
  if (!h->shared) {  // a handle whose creation failed part-way owns what it uploaded
    for (void* p : shared_arrays(h))
      if (p) cudaFree(p);
  }
  // per-handle state: materials, surface load, status word, staging and records
  void* own[] = {h->d_surfp, h->d_mat, h->d_status, h->s_x, h->s_r, h->s_vals, h->s_cp, h->s_uu, h->s_elem,
                 h->d_col, h->d_st_uu, h->d_st_cp, h->d_st_r, h->d_fuse};
  for (void* p : own)
    if (p) cudaFree(p);
  for (cudaEvent_t ev : h->chunk_events)
    if (ev) cudaEventDestroy(ev);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  delete h;  // releases this handle's share of the mesh arrays
  return FE_NO_ERROR;
}

int fe_clone(fe_handle src, fe_handle* out) {
  if (!out) return set_error(FE_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  int rc = check_handle(src);
  if (rc) return rc;
  fe_handle h = new (std::nothrow) fe_equations_set();
  if (!h) return set_error(FE_ERR_OUT_OF_MEMORY, "host allocation failed");
  {
    std::lock_guard<std::mutex> lk(src->mu);
    h->hs = src->hs;  // vectors copied; the CSR column array is shared
    h->shared = src->shared;
    h->device = src->device;
    h->num_sms = src->num_sms;
    h->d_elem_u = src->d_elem_u;
    h->d_elem_p = src->d_elem_p;
    h->d_row_ptr = src->d_row_ptr;
    h->d_uu_row_ptr = src->d_uu_row_ptr;
    h->d_cp_row_ptr = src->d_cp_row_ptr;
    h->d_wu = src->d_wu;
    h->d_wp = src->d_wp;
    h->d_elem_table = src->d_elem_table;
    h->d_colour_elems = src->d_colour_elems;
    h->d_tables = src->d_tables;
    h->d_geo = src->d_geo;
    h->d_geo_dd = src->d_geo_dd;
    h->d_gbf_u = src->d_gbf_u;
    h->d_gbf_p = src->d_gbf_p;
    h->d_gw = src->d_gw;
    h->d_bnd_elems = src->d_bnd_elems;
    h->d_bnd_mask = src->d_bnd_mask;
    h->d_u_inc_ptr = src->d_u_inc_ptr;
    h->d_u_inc = src->d_u_inc;
    h->d_p_inc_ptr = src->d_p_inc_ptr;
    h->d_p_inc = src->d_p_inc;
    h->high_precision = src->high_precision;
    h->assembly_order = src->assembly_order;
    h->host_output = src->host_output;
    h->stream_chunks = src->stream_chunks;
  }
  auto fail = [&](int code) {
    fe_destroy(h);
    return code;
  };
  const size_t mat_bytes = sizeof(double) * h->hs.mat.size();
  if (cudaMalloc(&h->d_mat, mat_bytes) != cudaSuccess ||
      cudaMemcpy(h->d_mat, src->d_mat, mat_bytes, cudaMemcpyDeviceToDevice) != cudaSuccess ||
      cudaMalloc(&h->d_status, sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(h->d_status, 0, sizeof(unsigned)) != cudaSuccess)
    return fail(set_error(FE_ERR_CUDA, "clone: device allocation failed"));
  if (src->has_surfp) {
    const size_t bytes = sizeof(double) * 3 * (size_t)h->hs.nu;
    if (cudaMalloc(&h->d_surfp, bytes) != cudaSuccess ||
        cudaMemcpy(h->d_surfp, src->d_surfp, bytes, cudaMemcpyDeviceToDevice) != cudaSuccess)
      return fail(set_error(FE_ERR_CUDA, "clone: device allocation failed"));
    h->has_surfp = true;
  }
  *out = h;
  return FE_NO_ERROR;
}

int fe_structure_calculate(const fe_mesh_desc* desc, int32_t base, int64_t* num_dofs, int64_t* nnz,
                           int32_t* row_ptr, int32_t* col) {
  if (base != 0 && base != 1) return set_error(FE_ERR_INVALID_ARGUMENT, "base must be 0 or 1");
  HostSetup s;
  std::string msg;
  int rc = cmfe::build_setup(desc, s, msg);
  if (rc) return set_error(rc, msg);
  if (num_dofs) *num_dofs = s.ndofs;
  if (nnz) *nnz = s.nnz;
  if (row_ptr)
    for (int64_t i = 0; i <= s.ndofs; ++i) row_ptr[i] = s.row_ptr[i] + base;
  if (col)
    for (int64_t i = 0; i < s.nnz; ++i) col[i] = s.col[i] + base;
  return FE_NO_ERROR;
}

int fe_sizes(fe_handle h, int64_t* num_dofs, int64_t* nnz) {
  if (!h) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL handle");
  if (num_dofs) *num_dofs = h->hs.ndofs;
  if (nnz) *nnz = h->hs.nnz;
  return FE_NO_ERROR;
}

int fe_element_size(fe_handle h, int32_t* n) {
  if (!h || !n) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = h->hs.nrow;
  return FE_NO_ERROR;
}

int fe_csr_pattern(fe_handle h, int32_t base, int32_t* row_ptr, int32_t* col) {
  if (!h) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL handle");
  if (base != 0 && base != 1) return set_error(FE_ERR_INVALID_ARGUMENT, "base must be 0 or 1");
  const auto& s = h->hs;
  if (row_ptr)
    for (int64_t i = 0; i <= s.ndofs; ++i) row_ptr[i] = s.row_ptr[i] + base;
  if (col)
    for (int64_t i = 0; i < s.nnz; ++i) col[i] = s.col[i] + base;
  return FE_NO_ERROR;
}

int fe_mixed_layout(fe_handle h, int64_t* nnz_uu, int64_t* nnz_coupling, int32_t* uu_row_ptr, int32_t* cp_row_ptr) {
  if (!h) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL handle");
  const auto& s = h->hs;
  if (nnz_uu) *nnz_uu = s.nnz_uu;
  if (nnz_coupling) *nnz_coupling = s.nnz_cp;
  if (uu_row_ptr) std::memcpy(uu_row_ptr, s.uu_row_ptr.data(), s.uu_row_ptr.size() * sizeof(int32_t));
  if (cp_row_ptr) std::memcpy(cp_row_ptr, s.cp_row_ptr.data(), s.cp_row_ptr.size() * sizeof(int32_t));
  return FE_NO_ERROR;
}

int fe_residual_evaluate(fe_handle h, const double* x, double* r, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!x || !r) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL x or r");
  std::lock_guard<std::mutex> lk(h->mu);
  cudaStream_t st = (cudaStream_t)stream;
  bool hx;
  const double* dx;
  if ((rc = stage_in(h, x, &dx, st, &hx))) return rc;
  const bool hr = !is_device_ptr(r);
  double* dr = r;
  if (hr) {
    if ((rc = ensure((void**)&h->s_r, sizeof(double) * h->hs.ndofs))) return rc;
    dr = h->s_r;
  }
  KParams kp = base_params(h);
  kp.x = dx;
  kp.r = dr;
  kp.res_only = 1;
  for (int c = 0; c < h->hs.ncolours; ++c) {
    kp.elems = h->d_colour_elems + h->hs.colour_ptr[c];
    kp.count = h->hs.colour_ptr[c + 1] - h->hs.colour_ptr[c];
    const int e = cmfe::launch_mixed(h->hs, kp, h->num_sms, st, h->high_precision == FE_HIGH_PRECISION_DOUBLE_FLOAT);
    if (e != 0) return set_error(FE_ERR_CUDA, std::string("residual kernel launch: ") + cudaGetErrorString((cudaError_t)e));
    h->launches++;
    if ((rc = surface_after(h, kp, c, 0, st))) return rc;
  }
  if (hr) {
    CUDA_TRY(cudaMemcpyAsync(r, dr, sizeof(double) * h->hs.ndofs, cudaMemcpyDeviceToHost, st));
    return finish_status(h, st);
  }
  return FE_NO_ERROR;
}

int fe_residual_evaluate_noalloc(fe_handle h, const double* x, double* r, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!x || !r) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL x or r");
  if (h->hs.ndofs > FE_NOALLOC_MAX_DOFS)
    return set_error(FE_ERR_INVALID_ARGUMENT, "fe_residual_evaluate_noalloc: " + std::to_string(h->hs.ndofs) +
                                                  " dofs exceed the static scratch limit FE_NOALLOC_MAX_DOFS = " +
                                                  std::to_string((long long)FE_NOALLOC_MAX_DOFS));
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  std::lock_guard<std::mutex> lk(h->mu);
  cudaStream_t st = (cudaStream_t)stream;
  double* base = nullptr;
  if ((rc = noalloc_scratch(h->device, &base))) return rc;
  double* dx = base;
  double* dr = base + FE_NOALLOC_MAX_DOFS;
  const size_t bytes = sizeof(double) * (size_t)h->hs.ndofs;
  // Declared after the locks, so destroyed before them: every return below,
  // the error returns included, first waits for the work this call queued on
  // the shared array, and the next call cannot overwrite it in flight.
  struct DrainOnReturn {
    cudaStream_t st;
    ~DrainOnReturn() {
      if (cudaStreamSynchronize(st) != cudaSuccess) cudaGetLastError();
    }
  } drain{st};
  CUDA_TRY(cudaMemcpyAsync(dx, x, bytes, cudaMemcpyDefault, st));
  KParams kp = base_params(h);
  kp.x = dx;
  kp.r = dr;
  kp.res_only = 1;
  for (int c = 0; c < h->hs.ncolours; ++c) {
    kp.elems = h->d_colour_elems + h->hs.colour_ptr[c];
    kp.count = h->hs.colour_ptr[c + 1] - h->hs.colour_ptr[c];
    const int e = cmfe::launch_mixed(h->hs, kp, h->num_sms, st, h->high_precision == FE_HIGH_PRECISION_DOUBLE_FLOAT);
    if (e != 0) return set_error(FE_ERR_CUDA, std::string("residual kernel launch: ") + cudaGetErrorString((cudaError_t)e));
    h->launches++;
    if ((rc = surface_after(h, kp, c, 0, st))) return rc;
  }
  CUDA_TRY(cudaMemcpyAsync(r, dr, bytes, cudaMemcpyDefault, st));
  return finish_status(h, st);
}

int fe_jacobian_evaluate(fe_handle h, const double* x, double* values, double* r, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!x || !values) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL x or values");
  std::lock_guard<std::mutex> lk(h->mu);
  cudaStream_t st = (cudaStream_t)stream;
  bool hx;
  const double* dx;
  if ((rc = stage_in(h, x, &dx, st, &hx))) return rc;
  const bool hv = !is_device_ptr(values);
  const bool hr = r && !is_device_ptr(r);
  double* dv = values;
  double* dr = r;
  if (hv) {
    if ((rc = ensure((void**)&h->s_vals, sizeof(double) * h->hs.nnz))) return rc;
    dv = h->s_vals;
  }
  if (hr) {
    if ((rc = ensure((void**)&h->s_r, sizeof(double) * h->hs.ndofs))) return rc;
    dr = h->s_r;
  }
  KParams kp = base_params(h);
  kp.x = dx;
  kp.vals = dv;
  kp.r = dr;
  if ((rc = run_colours<M_JAC>(h, kp, st))) return rc;
  if (hv) CUDA_TRY(cudaMemcpyAsync(values, dv, sizeof(double) * h->hs.nnz, cudaMemcpyDeviceToHost, st));
  if (hr) CUDA_TRY(cudaMemcpyAsync(r, dr, sizeof(double) * h->hs.ndofs, cudaMemcpyDeviceToHost, st));
  if (hv || hr) return finish_status(h, st);
  return FE_NO_ERROR;
}

int fe_jacobian_evaluate_mixed(fe_handle h, const double* x, float* values_uu, double* values_coupling, double* r,
                               void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!x || !values_uu || !values_coupling) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(h->mu);
  cudaStream_t st = (cudaStream_t)stream;
  bool hx;
  const double* dx;
  if ((rc = stage_in(h, x, &dx, st, &hx))) return rc;
  bool hu = !is_device_ptr(values_uu), hc = !is_device_ptr(values_coupling);
  bool hr = r && !is_device_ptr(r);
  float* du = values_uu;
  double* dc = values_coupling;
  double* dr = r;
  bool mapped_out = false;  // some output is host memory written in place: wait before returning
  const bool staged = h->assembly_order == FE_ASSEMBLY_STAGED && h->hs.gather_bytes > 0;
  if (staged && (hu || hc || hr) && h->host_output == FE_HOST_OUTPUT_STREAMED && cmfe::fused_fits(h->hs)) {
    // the rows each chunk of elements completes go to the host while the
    // next chunks assemble
    if (hu && (rc = ensure((void**)&h->s_uu, sizeof(float) * h->hs.nnz_uu))) return rc;
    if (hc && (rc = ensure((void**)&h->s_cp, sizeof(double) * h->hs.nnz_cp))) return rc;
    if (hr && (rc = ensure((void**)&h->s_r, sizeof(double) * h->hs.ndofs))) return rc;
    if ((rc = mixed_streamed(h, dx, hu ? h->s_uu : values_uu, hc ? h->s_cp : values_coupling, hr ? h->s_r : r,
                             hu ? values_uu : nullptr, hc ? values_coupling : nullptr, hr ? r : nullptr,
                             h->high_precision == FE_HIGH_PRECISION_DOUBLE_FLOAT, st))) {
      // launches or copies may be queued already: none may write the
      // caller's host buffers after the call has returned
      if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
      cudaStreamSynchronize(st);
      return rc;
    }
    return finish_status(h, st);
  }
  if (staged && h->host_output == FE_HOST_OUTPUT_IN_PLACE) {
    // the row gather writes each output row once, contiguously: page-locked
    // host outputs are written in place over the host link, with no device
    // copy of the result and no separate device-to-host copy
    void* p;
    if (hu && mapped_host_ptr(values_uu, &p)) du = static_cast<float*>(p), hu = false, mapped_out = true;
    if (hc && mapped_host_ptr(values_coupling, &p)) dc = static_cast<double*>(p), hc = false, mapped_out = true;
    if (hr && mapped_host_ptr(r, &p)) dr = static_cast<double*>(p), hr = false, mapped_out = true;
  }
  if (hu) {
    if ((rc = ensure((void**)&h->s_uu, sizeof(float) * h->hs.nnz_uu))) return rc;
    du = h->s_uu;
  }
  if (hc) {
    if ((rc = ensure((void**)&h->s_cp, sizeof(double) * h->hs.nnz_cp))) return rc;
    dc = h->s_cp;
  }
  if (hr) {
    if ((rc = ensure((void**)&h->s_r, sizeof(double) * h->hs.ndofs))) return rc;
    dr = h->s_r;
  }
  if ((rc = mixed_assemble(h, dx, du, dc, dr, h->high_precision == FE_HIGH_PRECISION_DOUBLE_FLOAT, st, nullptr)))
    return rc;
  if (hu) CUDA_TRY(cudaMemcpyAsync(values_uu, du, sizeof(float) * h->hs.nnz_uu, cudaMemcpyDeviceToHost, st));
  if (hc) CUDA_TRY(cudaMemcpyAsync(values_coupling, dc, sizeof(double) * h->hs.nnz_cp, cudaMemcpyDeviceToHost, st));
  if (hr) CUDA_TRY(cudaMemcpyAsync(r, dr, sizeof(double) * h->hs.ndofs, cudaMemcpyDeviceToHost, st));
  if (hu || hc || hr || mapped_out) return finish_status(h, st);
  return FE_NO_ERROR;
}

static int element_eval(fe_handle h, const double* x, int32_t first, int32_t count, double* out, void* stream,
                        bool jac) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!x || !out || first < 0 || count < 0 || (int64_t)first + count > h->hs.ne)
    return set_error(FE_ERR_INVALID_ARGUMENT, "invalid element range or NULL pointer");
  if (count == 0) return FE_NO_ERROR;
  std::lock_guard<std::mutex> lk(h->mu);
  cudaStream_t st = (cudaStream_t)stream;
  bool hx;
  const double* dx;
  if ((rc = stage_in(h, x, &dx, st, &hx))) return rc;
  const size_t n = (size_t)h->hs.nrow;
  const size_t bytes = sizeof(double) * (size_t)count * (jac ? n * n : n);
  const bool ho = !is_device_ptr(out);
  double* dout = out;
  if (ho) {
    if (h->s_elem_bytes < bytes) {
      if (h->s_elem) cudaFree(h->s_elem);
      h->s_elem = nullptr;
      h->s_elem_bytes = 0;
      if ((rc = ensure((void**)&h->s_elem, bytes))) return rc;
      h->s_elem_bytes = bytes;
    }
    dout = h->s_elem;
  }
  KParams kp = base_params(h);
  kp.x = dx;
  kp.elem_out = dout;
  kp.first_elem = first;
  kp.count = count;
  kp.elems = nullptr;
  if ((rc = jac ? launch<M_EJAC>(h, kp, st) : launch<M_ERES>(h, kp, st))) return rc;
  if (h->has_surfp && !h->hs.bnd_elems.empty()) {
    const int e = cmfe::launch_surface(h->hs, kp, h->d_bnd_elems, h->d_bnd_mask, (int)h->hs.bnd_elems.size(), 1,
                                       jac ? 1 : 0, h->num_sms, st);
    if (e != 0) return set_error(FE_ERR_CUDA, std::string("surface kernel launch: ") + cudaGetErrorString((cudaError_t)e));
    h->launches++;
  }
  if (ho) {
    CUDA_TRY(cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, st));
    return finish_status(h, st);
  }
  return FE_NO_ERROR;
}

int fe_element_residuals(fe_handle h, const double* x, int32_t first, int32_t count, double* out, void* stream) {
  return element_eval(h, x, first, count, out, stream, false);
}

int fe_element_jacobians(fe_handle h, const double* x, int32_t first, int32_t count, double* out, void* stream) {
  return element_eval(h, x, first, count, out, stream, true);
}

int fe_set_surface_pressure(fe_handle h, const double* values) {
  int rc = check_handle(h);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(h->mu);
  if (!values) {
    h->has_surfp = false;
    return FE_NO_ERROR;
  }
  const size_t bytes = sizeof(double) * 3 * (size_t)h->hs.nu;
  if ((rc = ensure((void**)&h->d_surfp, bytes))) return rc;
  CUDA_TRY(cudaMemcpy(h->d_surfp, values, bytes, cudaMemcpyDefault));
  h->has_surfp = true;
  return FE_NO_ERROR;
}

int fe_set_materials(fe_handle h, const double* materials) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!materials) return set_error(FE_ERR_INVALID_ARGUMENT, "materials is NULL");
  std::lock_guard<std::mutex> lk(h->mu);
  CUDA_TRY(cudaMemcpy(h->d_mat, materials, sizeof(double) * h->hs.mat.size(), cudaMemcpyDefault));
  return FE_NO_ERROR;
}

int fe_set_high_precision(fe_handle h, int32_t mode) {
  if (!h) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL handle");
  if (mode != FE_HIGH_PRECISION_FP64 && mode != FE_HIGH_PRECISION_DOUBLE_FLOAT)
    return set_error(FE_ERR_INVALID_ARGUMENT, "unknown high-precision mode");
  h->high_precision = mode;
  return FE_NO_ERROR;
}

int fe_set_assembly_order(fe_handle h, int32_t order) {
  if (!h) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL handle");
  if (order != FE_ASSEMBLY_STAGED && order != FE_ASSEMBLY_COLOURED)
    return set_error(FE_ERR_INVALID_ARGUMENT, "unknown assembly order");
  std::lock_guard<std::mutex> lk(h->mu);
  h->assembly_order = order;
  return FE_NO_ERROR;
}

int fe_set_host_output(fe_handle h, int32_t mode, int32_t chunks) {
  if (!h) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL handle");
  if (mode != FE_HOST_OUTPUT_STREAMED && mode != FE_HOST_OUTPUT_IN_PLACE && mode != FE_HOST_OUTPUT_AFTER)
    return set_error(FE_ERR_INVALID_ARGUMENT, "unknown host output mode");
  if (chunks < 0 || chunks > kStreamChunks) return set_error(FE_ERR_INVALID_ARGUMENT, "chunks must be 0..16");
  std::lock_guard<std::mutex> lk(h->mu);
  h->host_output = mode;
  h->stream_chunks = chunks;
  return FE_NO_ERROR;
}

int fe_check(fe_handle h, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(h->mu);
  return finish_status(h, (cudaStream_t)stream);
}

int fe_launch_count(fe_handle h, int64_t* count) {
  if (!h || !count) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  *count = h->launches;
  return FE_NO_ERROR;
}

int fe_batch_create(const fe_handle* handles, int32_t count, fe_batch* out) {
  if (!out) return set_error(FE_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!handles || count <= 0) return set_error(FE_ERR_INVALID_ARGUMENT, "empty batch");
  int cur = 0;
  CUDA_TRY(cudaGetDevice(&cur));
  auto b = new (std::nothrow) fe_batch_s;
  if (!b) return set_error(FE_ERR_OUT_OF_MEMORY, "batch allocation failed");
  b->device = cur;
  int rc = FE_NO_ERROR;
  for (int32_t i = 0; i < count && !rc; ++i) {
    if (!handles[i]) rc = set_error(FE_ERR_INVALID_ARGUMENT, "NULL member handle");
    else if (handles[i]->device != cur) rc = set_error(FE_ERR_INVALID_ARGUMENT, "member on another CUDA device");
    else {
      b->members.push_back(handles[i]);
      b->ncol = std::max(b->ncol, handles[i]->hs.ncolours);
    }
  }
  if (!rc && count > cmfe::BATCH_MAX_MEMBERS)
    rc = set_error(FE_ERR_NOT_SUPPORTED, "a batch holds at most " + std::to_string(cmfe::BATCH_MAX_MEMBERS) + " members");
  if (!rc) {
    b->num_sms = b->members[0]->num_sms;
    // slots ordered by element type, members in their given order within a type
    for (int t = 0; t < 4; ++t)
      for (int32_t m = 0; m < count; ++m)
        if (member_type(b->members[m]->hs) == t) b->slot_member.push_back(m);
    auto fail = [&](cudaError_t e) {
      return e == cudaSuccess ? FE_NO_ERROR : set_error(FE_ERR_CUDA, std::string("batch set-up: ") + cudaGetErrorString(e));
    };
    const size_t tbytes = (size_t)count * sizeof(cmfe::BatchMember);
    rc = fail(cudaMallocHost(&b->h_table, tbytes));
    if (!rc) rc = fail(cudaMalloc(&b->d_table, tbytes));
    if (!rc) rc = fail(cudaMalloc(&b->d_table_graph, tbytes));
    std::vector<int32_t> offsets((size_t)count * 2 * (b->ncol + 1));
    for (int32_t s = 0; s < count && !rc; ++s) {
      fe_handle h = b->members[b->slot_member[s]];
      const HostSetup& hs = h->hs;
      b->type_mask |= 1u << member_type(hs);
      cmfe::BatchMember& e = b->h_table[s];
      std::memset(&e, 0, sizeof(e));
      e.kp = base_params(h);
      e.kp.elems = h->d_colour_elems;
      e.kp.count = hs.ne;
      e.kp.surf_p = nullptr;
      e.belems = h->d_bnd_elems;
      e.bmask = h->d_bnd_mask;
      e.type = member_type(hs);
      e.has_surface = 0;
      int32_t* o = &offsets[(size_t)s * 2 * (b->ncol + 1)];
      for (int c = 0; c <= b->ncol; ++c) {
        o[c] = hs.colour_ptr[std::min(c, hs.ncolours)];
        o[b->ncol + 1 + c] = hs.bnd_ptr[std::min(c, hs.ncolours)];
      }
    }
    b->surf_sig.assign((size_t)count, nullptr);
    if (!rc) rc = fail(cudaMalloc(&b->d_offsets, offsets.size() * sizeof(int32_t)));
    if (!rc) rc = fail(cudaMemcpy(b->d_offsets, offsets.data(), offsets.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    if (!rc) rc = fail(cudaMalloc(&b->d_sync, 4 * sizeof(unsigned)));
    if (!rc) rc = fail(cudaMemset(b->d_sync, 0, 4 * sizeof(unsigned)));
  }
  if (rc) {
    fe_batch_destroy(b);
    return rc;
  }
  *out = b;
  return FE_NO_ERROR;
}

int fe_batch_destroy(fe_batch b) {
  if (!b) return FE_NO_ERROR;
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  void* ptrs[] = {b->d_table, b->d_table_graph, b->d_offsets, b->d_sync};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (b->h_table) cudaFreeHost(b->h_table);
  delete b;
  return FE_NO_ERROR;
}

int fe_batch_jacobian_evaluate_mixed(fe_batch b, const double* const* x, float* const* values_uu,
                                     double* const* values_coupling, double* const* r, void* stream) {
  int rc = check_batch(b);
  if (rc) return rc;
  if (!x || !values_uu || !values_coupling) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL pointer array");
  std::lock_guard<std::mutex> lk(b->mu);
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = batch_set_pointers(b, x, values_uu, values_coupling, r, st))) return rc;
  return batch_launch(b, st);
}

int fe_batch_check(fe_batch b, void* stream) {
  int rc = check_batch(b);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned v = 0;
  CUDA_TRY(cudaMemcpyAsync(&v, b->d_sync + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemsetAsync(b->d_sync + 2, 0, sizeof(unsigned), st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (v & 2u) return set_error(FE_ERR_CUDA, "batched launch: a grid barrier gave up waiting");
  for (fe_handle h : b->members)
    if ((rc = finish_status(h, st))) return rc;
  return FE_NO_ERROR;
}

int fe_batch_set_barrier_limits(fe_batch b, uint32_t polls, uint32_t extra_arrivals) {
  int rc = check_batch(b);
  if (rc) return rc;
  if (extra_arrivals > 1) return set_error(FE_ERR_INVALID_ARGUMENT, "extra_arrivals must be 0 or 1");
  if (extra_arrivals && (polls == 0 || polls > 4096))
    return set_error(FE_ERR_INVALID_ARGUMENT, "an unreachable barrier needs a poll limit in 1..4096");
  std::lock_guard<std::mutex> lk(b->mu);
  b->barrier_polls = polls;
  b->barrier_extra = extra_arrivals;
  return FE_NO_ERROR;
}

int fe_batch_set_config(fe_batch b, int32_t variant, int32_t ctas_per_sm, int32_t block_groups) {
  int rc = check_batch(b);
  if (rc) return rc;
  if (variant < 0 || variant > cmfe::batch_variants() || ctas_per_sm < 1 || ctas_per_sm > 4 || block_groups < 1)
    return set_error(FE_ERR_INVALID_ARGUMENT, "invalid batch configuration");
  std::lock_guard<std::mutex> lk(b->mu);
  b->variant = variant;
  b->ctas_per_sm = ctas_per_sm;
  b->block_groups = block_groups;
  return FE_NO_ERROR;
}

int fe_batch_get_config(fe_batch b, int32_t* variant, int32_t* ctas_per_sm, int32_t* block_groups, double* tuned_ms) {
  int rc = check_batch(b);
  if (rc) return rc;
  if (variant) *variant = b->variant;
  if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
  if (block_groups) *block_groups = b->block_groups;
  if (tuned_ms) *tuned_ms = b->tuned_ms;
  return FE_NO_ERROR;
}

int fe_batch_autotune(fe_batch b, const double* const* x, float* const* values_uu, double* const* values_coupling,
                      double* const* r, int32_t repeats, void* stream) {
  int rc = check_batch(b);
  if (rc) return rc;
  if (!x || !values_uu || !values_coupling || repeats < 1) return set_error(FE_ERR_INVALID_ARGUMENT, "bad arguments");
  std::lock_guard<std::mutex> lk(b->mu);
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = batch_set_pointers(b, x, values_uu, values_coupling, r, st))) return rc;
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  int smem_per_sm = 0, smem_reserved = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, b->device));
  CUDA_TRY(cudaDeviceGetAttribute(&smem_reserved, cudaDevAttrReservedSharedMemoryPerBlock, b->device));
  const int keep_v = b->variant, keep_c = b->ctas_per_sm, keep_b = b->block_groups;
  double best = 1e300;
  int bv = keep_v, bc = keep_c, bb = keep_b;
  const int blocks[] = {1, 2, 4};
  for (int v = 0; v <= cmfe::batch_variants() && !rc; ++v)
    for (int cps = 1; cps <= 3 && !rc; ++cps) {
      // the last variant (one launch per member and colour) has no launch shape
      const bool per_member = v == cmfe::batch_variants();
      if (per_member && cps > 1) break;
      // skip a CTA count the shared memory cannot hold (the launch would use fewer)
      if (!per_member && cps * (cmfe::batch_smem(v, b->type_mask) + smem_reserved) > smem_per_sm) continue;
      for (int bg : blocks) {
        if (per_member && bg > 1) break;
        b->variant = v;
        b->ctas_per_sm = cps;
        b->block_groups = bg;
        if ((rc = batch_launch(b, st))) break;  // warm-up (and table upload)
        cudaEventRecord(e0, st);
        for (int i = 0; i < repeats && !rc; ++i) rc = batch_launch(b, st);
        cudaEventRecord(e1, st);
        if (rc) break;
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double per = ms / repeats;
        if (per < best) {
          best = per;
          bv = v;
          bc = cps;
          bb = bg;
        }
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) {
    b->variant = keep_v;
    b->ctas_per_sm = keep_c;
    b->block_groups = keep_b;
    return rc;
  }
  b->variant = bv;
  b->ctas_per_sm = bc;
  b->block_groups = bb;
  b->tuned_ms = best;
  return FE_NO_ERROR;
}

int fe_batch_capture(fe_batch b, const double* const* x, float* const* values_uu, double* const* values_coupling,
                     double* const* r, void* stream) {
  int rc = check_batch(b);
  if (rc) return rc;
  if (!x || !values_uu || !values_coupling) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL pointer array");
  std::lock_guard<std::mutex> lk(b->mu);
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = batch_set_pointers(b, x, values_uu, values_coupling, r, st))) return rc;
  if ((rc = refresh_surface(b)) || (rc = sync_table(b, st))) return rc;
  {
    // the graph reads its own snapshot of the table, written after every
    // launch already queued on the device (an earlier replay may read it)
    std::lock_guard<std::mutex> g(g_batch_mu);
    if ((rc = batch_serialise_begin(b->device, st))) return rc;
    CUDA_TRY(cudaMemcpyAsync(b->d_table_graph, b->d_table, b->members.size() * sizeof(cmfe::BatchMember),
                             cudaMemcpyDeviceToDevice, st));
    if ((rc = batch_serialise_end(b->device, st))) return rc;
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  cudaStream_t cs;
  CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->graph_exec = nullptr;
  b->graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const int64_t l0 = b->launches;
    rc = batch_launch_from(b, b->d_table_graph, cs);
    b->graph_kernels = b->launches - l0;  // counted when the graph runs, not at capture
    b->launches = l0;
    e = cudaStreamEndCapture(cs, &b->graph);
    if (!rc && e == cudaSuccess) e = cudaGraphInstantiate(&b->graph_exec, b->graph, 0);
  }
  cudaStreamDestroy(cs);
  if (rc) return rc;
  if (e != cudaSuccess) return set_error(FE_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
  return FE_NO_ERROR;
}

int fe_batch_replay(fe_batch b, void* stream) {
  int rc = check_batch(b);
  if (rc) return rc;
  if (!b->graph_exec) return set_error(FE_ERR_INVALID_ARGUMENT, "no captured graph: call fe_batch_capture first");
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> g(g_batch_mu);
  if ((rc = batch_serialise_begin(b->device, st))) return rc;
  CUDA_TRY(cudaGraphLaunch(b->graph_exec, st));
  b->launches += b->graph_kernels;
  return batch_serialise_end(b->device, st);
}

int fe_batch_launch_count(fe_batch b, int64_t* count) {
  if (!b || !count) return set_error(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  *count = b->launches;
  return FE_NO_ERROR;
}

}  // extern "C"
