// libcm_fe: mixed-precision element assembly, device code shared by the
// per-equations-set kernel (fe_mixed.cu) and the batched kernel (fe_batch.cu).
//
// Same arithmetic content as the reference's element residual and Jacobian
// (FiniteElasticity_FiniteElement{Residual,Jacobian}Evaluate,
// finite_elasticity_routines.f90:1260-1639 and :842-1175), reorganised for
// the GB300:
//
//  * FP64 only where the residual and the pressure coupling need it.  Per
//    Gauss point the kinematics use the adjugate of dz/dxi (J_z dxi/dz =
//    adj(dz/dxi), so no 3x3 division), the Cauchy stress is formed as
//    F_bar S_bar F_bar^T / J (the push-forward of :1221-1253 written as a
//    matrix product), and the residual is contracted against the fixed table
//    of reference-element gradients: r(m,a) = sum_g sum_k dN_a/dxi_k (g) *
//    P_g(k,m) with P_g = J_z w_g dxi/dz sigma.  The pressure-coupling block
//    K(p_q, u_nb) = sum_g psi_q(g) J_z w_g dN_b/dz_n is contracted with the
//    tensor-product (sum-factorised) form of the trilinear pressure basis.
//  * The displacement block is FP32 with the contraction on tensor cores.
//    Per Gauss point the spatial tangent is pulled back to xi space:
//    D^{mn}(k,l) = sum_ij dxi_k/dz_i SUB^{mn}(i,j) dxi_l/dz_j with the
//    reference's SUB^{mn} = J_z w (c(T2V(:,m),T2V(:,n)) + delta_mn sigma)
//    (:1003-1034), so K^{mn}(a,b) = sum_{(g,k)} Phi(g,k;a) W^{mn}(g,k;b) with
//    W = D Phi and Phi the constant gradient table.  That product runs as
//    mma.sync m16n8k16 BF16 with FP32 accumulation; with SPLIT = 3 both
//    operands are split into a BF16 high part and a BF16 residual and three
//    products are accumulated, which keeps about 16 significant bits.
//  * Elements of one colour share no node; a CTA processes EG elements at a
//    time for the per-Gauss-point work (so 100+ threads do the FP64
//    kinematics at once) and then contracts them one by one.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "fe_dd.cuh"
#include "fe_internal.h"
#include "fe_math.cuh"

using cmfe::HostSetup;
using cmfe::KParams;
using cmfe::NG;

namespace {

constexpr int align16(int x) { return (x + 15) & ~15; }

// Default elements per group: 3 for triquadratic elements with nodal pressure
// (about 72 KB of shared memory, so three 256-thread CTAs fit on an SM, which
// measured 17 % faster than two CTAs of 4 elements despite the register
// spills the 80-register budget causes), 4 for element-based pressure, 8 for
// trilinear elements.
template <int N1, int PM, int EG_ = (N1 == 3 ? (PM ? 3 : 4) : 8)>
struct MixCfg {
  static constexpr int MINB = (N1 == 3 && PM) ? 3 : 2;  // CTAs per SM the launch bounds ask for
  static constexpr int NPE = N1 * N1 * N1;
  static constexpr int NPP = PM ? 8 : 1;
  static constexpr int NR = NPE + NPP;
  static constexpr int NU3 = 3 * NPE;
  static constexpr int NROW = NU3 + NPP;
  static constexpr int THREADS = 256;
  static constexpr int EG = EG_;                // elements per group
  static constexpr int MT = (NPE + 15) / 16;    // m16 tiles over a
  static constexpr int NT = (NPE + 7) / 8;      // n8 tiles over b
  static constexpr int KT = 6;                  // k16 tiles over (g,k): 81 -> 96
  static constexpr int KPW = 52;                // padded row length in 32-bit words (104 bf16)
  static constexpr int AROWS = MT * 16;
  static constexpr int BROWS = NT * 8;
  static constexpr int REC64 = 20;  // P(9), A(9), t1, pad
  static constexpr int REC32 = 60;  // D^{mn}(k,l) for 6 blocks, padded so Gauss points 2 apart hit banks 24 apart
  static constexpr int PHS = 4 * NPE;  // per-Gauss-point stride of the FP32 gradient table: [b][d0, d1, d2, 0]
  static constexpr int KAP = 84;    // contraction length: kappa = 28 k + g, g < 27 (g = 27 is padding)
  static constexpr int O_PSI64 = 0;
  static constexpr int O_L = align16(O_PSI64 + NG * 8 * 8);
  static constexpr int O_W = align16(O_L + 6 * 8);
  static constexpr int O_1D = align16(O_W + NG * 8);
  static constexpr int O_LM = align16(O_1D + 6 * N1 * 8);  // L x (1-D value | derivative) products
  // constant tables first, then the per-group scratch from O_Z on (the fused
  // kernel reuses the scratch between groups for its row gathers)
  static constexpr int O_PHI32 = align16(O_LM + 12 * N1 * 8);
  static constexpr int O_A = align16(O_PHI32 + NG * PHS * 4);
  static constexpr int O_Z = align16(O_A + 2 * AROWS * KPW * 4);
  static constexpr int O_P = align16(O_Z + EG * 3 * NPE * 8);
  static constexpr int O_DZ = align16(O_P + EG * 8 * 8);
  static constexpr int O_PG = align16(O_DZ + EG * NG * 9 * 8);
  static constexpr int O_R64 = align16(O_PG + EG * NG * 8);
  static constexpr int O_R32 = align16(O_R64 + EG * NG * REC64 * 8);
  static constexpr int O_F32 = align16(O_R32 + EG * NG * REC32 * 4);
  static constexpr int O_NODE = align16(O_F32 + EG * NG * 24 * 4);
  static constexpr int SMEM = align16(O_NODE + EG * (NR + 1) * 4);
  static constexpr int O_SCRATCH = O_Z;
  // fused kernel: the list of row nodes a group completed, just below O_NODE
  static constexpr int O_READY = O_NODE - align16(EG * NR * 4);
};

__device__ __forceinline__ uint32_t pack_bf16(float lo_elem, float hi_elem) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo_elem, hi_elem);  // .x -> low 16 bits
  return *reinterpret_cast<uint32_t*>(&v);
}

// Splits (v0, v1) into BF16 high parts and BF16 residuals.
__device__ __forceinline__ void split_bf16(float v0, float v1, uint32_t& hi, uint32_t& lo) {
  __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
  const float r0 = v0 - __bfloat162float(h.x);
  const float r1 = v1 - __bfloat162float(h.y);
  __nv_bfloat162 l = __floats2bfloat162_rn(r0, r1);
  hi = *reinterpret_cast<uint32_t*>(&h);
  lo = *reinterpret_cast<uint32_t*>(&l);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Four 8x8 b16 matrices from shared memory (ldmatrix, not transposed): lane L
// gives the address of row L % 8 of matrix L / 8 (16-byte aligned); register i
// receives the thread's element pair of matrix i (row lane / 4, pair lane % 4).
__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const void* row_addr) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(row_addr);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

// Block (m, n) of the lower-triangle displacement blocks: 0..2 diagonal,
// 3 = (1,0), 4 = (2,0), 5 = (2,1).
__device__ __forceinline__ void blk_mn(int blk, int& m, int& n) {
  m = blk < 3 ? blk : (blk == 3 ? 1 : 2);
  n = blk < 3 ? blk : (blk == 5 ? 1 : 0);
}

// Cauchy stress of the MR or Guccione law in the high-precision type H from
// F (material frame) and J = Jznu: sigma = dev(F_bar S_bar F_bar^T / J) + p I.
template <class H>
__device__ void mix_stress(int law, const H* c, const H F[3][3], H J, H p, H sig[3][3]) {
  const H s = hrcbrt(J);
  const H zero = hval<H>(0.0), one = hval<H>(1.0), two = hval<H>(2.0), half = hval<H>(0.5);
  if (law == FE_LAW_MOONEY_RIVLIN) {
    // S_bar = al I + be C_bar, so F_bar S_bar F_bar^T = al B_bar + be B_bar^2 with
    // B_bar = F_bar F_bar^T (and tr C_bar = tr B_bar): fewer FP64 operations
    // than forming C_bar and both products
    const H s2 = s * s;
    H Bb[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = i; j < 3; ++j) {
        Bb[i][j] = s2 * (F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2]);
        Bb[j][i] = Bb[i][j];
      }
    const H I1 = Bb[0][0] + Bb[1][1] + Bb[2][2];
    const H al = two * (c[0] + I1 * c[1]);
    const H be = -(two * c[1]);
    const H rJ = one / J;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = i; j < 3; ++j) {
        const H b2 = Bb[i][0] * Bb[0][j] + Bb[i][1] * Bb[1][j] + Bb[i][2] * Bb[2][j];
        sig[i][j] = (al * Bb[i][j] + be * b2) * rJ;
        sig[j][i] = sig[i][j];
      }
    const H tr3 = (sig[0][0] + sig[1][1] + sig[2][2]) * hval<H>(1.0 / 3.0);
#pragma unroll
    for (int i = 0; i < 3; ++i) sig[i][i] = sig[i][i] - tr3 + p;
    return;
  }
  H Fb[3][3], Cb[3][3], S[3][3], T[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Fb[i][j] = F[i][j] * s;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      Cb[i][j] = Fb[0][i] * Fb[0][j] + Fb[1][i] * Fb[1][j] + Fb[2][i] * Fb[2][j];
      Cb[j][i] = Cb[i][j];
    }
  if (law == FE_LAW_MOONEY_RIVLIN) {
    const H I1 = Cb[0][0] + Cb[1][1] + Cb[2][2];
    const H al = two * (c[0] + I1 * c[1]);
    const H be = -(two * c[1]);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S[i][j] = i == j ? be * Cb[i][j] + al : be * Cb[i][j];
  } else {
    const H B[6] = {two * c[1], two * c[2], two * c[2], c[3], c[3], c[2]};
    const H E[6] = {half * (Cb[0][0] - one), half * (Cb[1][1] - one), half * (Cb[2][2] - one), Cb[1][0], Cb[2][0],
                    Cb[2][1]};
    H DQ[6], dot = zero;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      DQ[i] = B[i] * E[i];
      dot = dot + E[i] * DQ[i];
    }
    const H t1 = half * c[0] * hexp(half * dot);
    S[0][0] = t1 * DQ[0];
    S[1][1] = t1 * DQ[1];
    S[2][2] = t1 * DQ[2];
    S[0][1] = S[1][0] = t1 * DQ[3];
    S[0][2] = S[2][0] = t1 * DQ[4];
    S[1][2] = S[2][1] = t1 * DQ[5];
  }
  // sigma_bar = F_bar S F_bar^T / J
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) T[i][j] = Fb[i][0] * S[0][j] + Fb[i][1] * S[1][j] + Fb[i][2] * S[2][j];
  const H rJ = one / J;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      sig[i][j] = (T[i][0] * Fb[j][0] + T[i][1] * Fb[j][1] + T[i][2] * Fb[j][2]) * rJ;
      sig[j][i] = sig[i][j];
    }
  const H tr3 = (sig[0][0] + sig[1][1] + sig[2][2]) * hval<H>(1.0 / 3.0);
#pragma unroll
  for (int i = 0; i < 3; ++i) sig[i][i] = sig[i][i] - tr3 + p;
}

// Geometric Gauss-point data (dXi/dNu row-major, J_x) in H.
__device__ __forceinline__ void load_geo(const KParams& P, int e, int g, double dn[9], double& jx) {
  const double* geo = &P.geo[((size_t)e * NG + g) * 10];
#pragma unroll
  for (int i = 0; i < 9; ++i) dn[i] = geo[i];
  jx = geo[9];
}
__device__ __forceinline__ void load_geo(const KParams& P, int e, int g, dd dn[9], dd& jx) {
  const float2* geo = reinterpret_cast<const float2*>(P.geo_dd) + ((size_t)e * NG + g) * 10;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const float2 v = geo[i];
    dn[i] = {v.x, v.y};
  }
  const float2 v = geo[9];
  jx = {v.x, v.y};
}

// The 3-point Gauss-Legendre abscissae on [0, 1].
__device__ __forceinline__ double gauss_1d(int gi) {
  return gi == 0 ? (-sqrt(0.6) + 1.0) / 2.0 : (gi == 1 ? 0.5 : (sqrt(0.6) + 1.0) / 2.0);
}

// 1-D Lagrange basis function a of degree N1 - 1 on [0, 1] and its derivative at t.
template <int N1>
__device__ __forceinline__ void lagrange_1d(int a, double t, double& bv, double& dv) {
  if (N1 == 2) {
    bv = a == 0 ? 1.0 - t : t;
    dv = a == 0 ? -1.0 : 1.0;
  } else {
    bv = a == 0 ? 1.0 - 3.0 * t + 2.0 * t * t : (a == 1 ? 4.0 * t * (1.0 - t) : t * (t + t - 1.0));
    dv = a == 0 ? 4.0 * t - 3.0 : (a == 1 ? 4.0 - 8.0 * t : 4.0 * t - 1.0);
  }
}

// Constant tables (basis values and derivatives at the Gauss points, the
// split BF16 gradient table of the tensor-core stage) into shared memory.
template <int N1, int PM, int EG_, class H>
__device__ __forceinline__ void mix_tables(const KParams& P, unsigned char* sm) {
  using C = MixCfg<N1, PM, EG_>;
  constexpr int NPE = C::NPE, KPW = C::KPW;
  H* s_psi = reinterpret_cast<H*>(sm + C::O_PSI64);  // [g][q]
  H* s_L = reinterpret_cast<H*>(sm + C::O_L);        // [q][gi]
  H* s_w = reinterpret_cast<H*>(sm + C::O_W);        // [g]
  H* s_B1 = reinterpret_cast<H*>(sm + C::O_1D);      // [gi][a] 1-D values
  H* s_D1 = s_B1 + 3 * N1;                                // [gi][a] 1-D derivatives
  H* s_LM = reinterpret_cast<H*>(sm + C::O_LM);      // [B|D][q][gi][a]: L(q, gi) x 1-D value | derivative
  float* s_phi32 = reinterpret_cast<float*>(sm + C::O_PHI32);  // [g][b][l], l padded to 4
  uint32_t* s_A = reinterpret_cast<uint32_t*>(sm + C::O_A);    // [hi/lo][a][KPW]
  const int tid = threadIdx.x;
  // ---- constant tables
  for (int i = tid; i < NG * 8; i += C::THREADS) s_psi[i] = hval<H>(P.gbf_p[i]);
  for (int i = tid; i < NG; i += C::THREADS) s_w[i] = hval<H>(P.gw[i]);
  if (tid < 6) {
    const int q = tid / 3, gi = tid % 3;
    const double t = gauss_1d(gi);
    s_L[tid] = hval<H>(q == 0 ? 1.0 - t : t);
  }
  if (tid < 3 * N1) {  // 1-D Lagrange values and derivatives at the Gauss points
    const int gi = tid / N1, a = tid % N1;
    double bv, dv;
    lagrange_1d<N1>(a, gauss_1d(gi), bv, dv);
    s_B1[tid] = hval<H>(bv);
    s_D1[tid] = hval<H>(dv);
  }
  if (tid < 12 * N1) {  // their products with the linear pressure basis (nodal-pressure coupling)
    const int a = tid % N1, gi = (tid / N1) % 3, q = (tid / (3 * N1)) % 2, d = tid / (6 * N1);
    const double t = gauss_1d(gi);
    double bv, dv;
    lagrange_1d<N1>(a, t, bv, dv);
    s_LM[tid] = hval<H>((q == 0 ? 1.0 - t : t) * (d ? dv : bv));
  }
  for (int i = tid; i < NG * 3 * NPE; i += C::THREADS) {
    const int g = i / (3 * NPE), l = (i / NPE) % 3, b = i % NPE;
    s_phi32[g * C::PHS + 4 * b + l] = (float)P.gbf_u[(g * 4 + l + 1) * NPE + b];
    if (l == 0) s_phi32[g * C::PHS + 4 * b + 3] = 0.0f;
  }
  for (int i = tid; i < C::AROWS * KPW; i += C::THREADS) {
    const int a = i / KPW, wd = i % KPW;
    float v[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int kap = 2 * wd + h;
      const int kk = kap / 28, gg = kap % 28;
      v[h] = (a < NPE && kap < C::KAP && gg < NG) ? (float)P.gbf_u[(gg * 4 + kk + 1) * NPE + a] : 0.0f;
    }
    uint32_t hi, lo;
    split_bf16(v[0], v[1], hi, lo);
    s_A[i] = hi;
    s_A[C::AROWS * KPW + i] = lo;
  }
}

// Element number of entry i of an element list (NULL: P.first_elem + i).
__device__ __forceinline__ int elem_at(const KParams& P, const int32_t* elems, int i) {
  return elems ? elems[i] : P.first_elem + i;
}

// One group of up to EG elements, elems[grp*EG ...] of the count elements
// of the current colour.  p4_first swaps the order of the independent FP64
// (P3) and tensor-core (P4) stages.  OUT = 0 adds the element's entries into
// the CSR values and the residual (first contributor in colour order stores,
// later ones add); OUT = 1 stores them into the element's staging records
// (*SO), which the row gather sums afterwards.
template <int N1, int PM, int EG_, int SPLIT, class H, int OUT = 0>
__device__ __forceinline__ void mix_group(const KParams& P, const int32_t* elems, int count, int grp, bool p4_first,
                                          unsigned char* sm, const cmfe::StageOut* SO = nullptr) {
  using C = MixCfg<N1, PM, EG_>;
  constexpr int NPE = C::NPE, NPP = C::NPP, NR = C::NR, NU3 = C::NU3, NROW = C::NROW, EG = C::EG;
  constexpr int KPW = C::KPW;
  H* s_psi = reinterpret_cast<H*>(sm + C::O_PSI64);  // [g][q]
  H* s_L = reinterpret_cast<H*>(sm + C::O_L);        // [q][gi]
  H* s_w = reinterpret_cast<H*>(sm + C::O_W);        // [g]
  H* s_B1 = reinterpret_cast<H*>(sm + C::O_1D);      // [gi][a] 1-D values
  H* s_D1 = s_B1 + 3 * N1;                                // [gi][a] 1-D derivatives
  H* s_LM = reinterpret_cast<H*>(sm + C::O_LM);      // [B|D][q][gi][a]: L(q, gi) x 1-D value | derivative
  H* s_z = reinterpret_cast<H*>(sm + C::O_Z);        // [el][c][a]
  H* s_p = reinterpret_cast<H*>(sm + C::O_P);        // [el][q]
  H* s_dz = reinterpret_cast<H*>(sm + C::O_DZ);      // [el][g][c*3+k]
  H* s_pg = reinterpret_cast<H*>(sm + C::O_PG);      // [el][g]
  H* s_r64 = reinterpret_cast<H*>(sm + C::O_R64);    // [el][g][REC64]
  float* s_phi32 = reinterpret_cast<float*>(sm + C::O_PHI32);  // [g][b][l], l padded to 4
  float* s_r32 = reinterpret_cast<float*>(sm + C::O_R32);      // [el][g][REC32]
  uint32_t* s_A = reinterpret_cast<uint32_t*>(sm + C::O_A);    // [hi/lo][a][KPW]
  float* s_f32 = reinterpret_cast<float*>(sm + C::O_F32);      // scratch of P3 and P4 (EG x 2592 B)
  int* s_node = reinterpret_cast<int*>(sm + C::O_NODE);        // [el][NR+1]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nu = P.nu;
  const int nvalid = min(EG, count - grp * EG);
  __syncthreads();
  // ---- P0: element nodes and table ids
  for (int i = tid; i < EG * (NR + 1); i += C::THREADS) {
    const int el = i / (NR + 1), r = i % (NR + 1);
    int v = 0;
    if (el < nvalid) {
      const int e = elem_at(P, elems, grp * EG + el);
      if (r < NPE)
        v = P.elem_u[(size_t)e * NPE + r];
      else if (r < NR)
        v = PM ? P.elem_p[(size_t)e * 8 + (r - NPE)] : e;
      else
        v = P.elem_table[e];
    }
    s_node[i] = v;
  }
  __syncthreads();
  for (int i = tid; i < EG * 3 * NPE; i += C::THREADS) {
    const int el = i / (3 * NPE), c = (i / NPE) % 3, a = i % NPE;
    s_z[i] = hval<H>(el < nvalid ? P.x[(size_t)c * nu + s_node[el * (NR + 1) + a]] : 0.0);
  }
  for (int i = tid; i < EG * NPP; i += C::THREADS) {
    const int el = i / NPP, q = i % NPP;
    s_p[el * 8 + q] = hval<H>(el < nvalid ? P.x[(size_t)3 * nu + s_node[el * (NR + 1) + NPE + q]] : 0.0);
  }
  __syncthreads();
  // ---- P1: dz/dxi at the Gauss points by sum factorisation over the
  // tensor-product basis (FP64): xi1, then xi2, then xi3 contractions with
  // the 1-D value (B) and derivative (D) tables.
  {
    constexpr int N2 = N1 * N1;
    H* S1 = reinterpret_cast<H*>(sm + C::O_R32);  // [el][c][B|D][g1][a2a3]
    H* S2 = S1 + EG * 3 * 2 * 3 * N2;                  // [el][c][BB|BD|DB][g1][g2][a3]
    for (int i = tid; i < EG * 3 * 2 * 3 * N2; i += C::THREADS) {
      const int j = i % N2, g1 = (i / N2) % 3, typ = (i / (3 * N2)) % 2, ec = i / (6 * N2);
      const H* M = typ ? s_D1 : s_B1;
      const H* zr = &s_z[ec * NPE + N1 * j];
      H acc = hval<H>(0.0);
#pragma unroll
      for (int a1 = 0; a1 < N1; ++a1) acc = hfma(M[g1 * N1 + a1], zr[a1], acc);
      S1[i] = acc;
    }
    __syncthreads();
    for (int i = tid; i < EG * 3 * 3 * 9 * N1; i += C::THREADS) {
      const int a3 = i % N1, g2 = (i / N1) % 3, g1 = (i / (3 * N1)) % 3, typ2 = (i / (9 * N1)) % 3,
                ec = i / (27 * N1);
      const int src = typ2 == 2 ? 1 : 0;                     // DB reads the D stage-1 output
      const H* M = typ2 == 1 ? s_D1 : s_B1;             // BD applies D along xi2
      const H* sr = &S1[((ec * 2 + src) * 3 + g1) * N2 + N1 * a3];
      H acc = hval<H>(0.0);
#pragma unroll
      for (int a2 = 0; a2 < N1; ++a2) acc = hfma(M[g2 * N1 + a2], sr[a2], acc);
      S2[i] = acc;
    }
    __syncthreads();
    for (int i = tid; i < EG * 3 * 3 * NG; i += C::THREADS) {
      const int g = i % NG, k = (i / NG) % 3, ec = i / (3 * NG);
      const int g1 = g % 3, g2 = (g / 3) % 3, g3 = g / 9;
      const int typ2 = k == 0 ? 2 : (k == 1 ? 1 : 0);        // d/dxi1: DB, d/dxi2: BD, d/dxi3: BB
      const H* M = k == 2 ? s_D1 : s_B1;
      const H* sr = &S2[(((ec * 3 + typ2) * 3 + g1) * 3 + g2) * N1];
      H acc = hval<H>(0.0);
#pragma unroll
      for (int a3 = 0; a3 < N1; ++a3) acc = hfma(M[g3 * N1 + a3], sr[a3], acc);
      const int el = ec / 3, c = ec % 3;
      s_dz[(el * NG + g) * 9 + c * 3 + k] = acc;
    }
  }
  for (int i = tid; i < EG * NG; i += C::THREADS) {
    const int el = i / NG, g = i % NG;
    H pg;
    if (PM) {
      pg = hval<H>(0.0);
#pragma unroll
      for (int q = 0; q < 8; ++q) pg = hfma(s_psi[g * 8 + q], s_p[el * 8 + q], pg);
    } else {
      pg = s_p[el * 8];
    }
    s_pg[i] = pg;
  }
  __syncthreads();
  // ---- P2 (H: kinematics, stress and the residual / coupling records per
  // Gauss point) and P2b (FP32: the spatial tangent pulled back to xi space)
  // run at the same time on the two halves of the CTA, so that the FP64 and
  // the FP32 pipes overlap; P2b forms the FP32 kinematics it needs itself from
  // the same gradients.
  constexpr int HALF = C::THREADS / 2;
  if (tid < HALF) {
    for (int t = tid; t < EG * NG; t += HALF) {
      const int el = t / NG, g = t % NG;
      if (el >= nvalid) continue;
      const int e = elem_at(P, elems, grp * EG + el);
      H M[3][3], adj[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int k = 0; k < 3; ++k) M[c][k] = s_dz[t * 9 + c * 3 + k];
      adj[0][0] = M[1][1] * M[2][2] - M[1][2] * M[2][1];
      adj[0][1] = M[0][2] * M[2][1] - M[0][1] * M[2][2];
      adj[0][2] = M[0][1] * M[1][2] - M[0][2] * M[1][1];
      adj[1][0] = M[1][2] * M[2][0] - M[1][0] * M[2][2];
      adj[1][1] = M[0][0] * M[2][2] - M[0][2] * M[2][0];
      adj[1][2] = M[0][2] * M[1][0] - M[0][0] * M[1][2];
      adj[2][0] = M[1][0] * M[2][1] - M[1][1] * M[2][0];
      adj[2][1] = M[0][1] * M[2][0] - M[0][0] * M[2][1];
      adj[2][2] = M[0][0] * M[1][1] - M[0][1] * M[1][0];
      const H det = M[0][0] * adj[0][0] + M[0][1] * adj[1][0] + M[0][2] * adj[2][0];
      H dn[9], jx;
      load_geo(P, e, g, dn, jx);
      H F[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) F[i][j] = M[i][0] * dn[j] + M[i][1] * dn[3 + j] + M[i][2] * dn[6 + j];
      const H jz = habs(det);
      const H jznu = jz / jx;
      const H w = s_w[g];
      const bool dpos = hpos(det);
      const H sw = dpos ? w : -w;  // J_z w dxi/dz = sign(det) w adj
      const double* cm = P.mat + (P.matpe ? (size_t)e * P.nmat : 0);
      const H cc[4] = {hval<H>(cm[0]), hval<H>(cm[1]), hval<H>(P.nmat > 2 ? cm[2] : 0.0),
                       hval<H>(P.nmat > 3 ? cm[3] : 0.0)};
      const H pgv = s_pg[t];
      H* rec = &s_r64[t * C::REC64];
      bool ok = dpos;
      if (P.r != nullptr) {
        H sig[3][3];
        mix_stress<H>(P.law, cc, F, jznu, pgv, sig);
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            const H v = sw * (adj[k][0] * sig[0][m] + adj[k][1] * sig[1][m] + adj[k][2] * sig[2][m]);
            rec[k * 3 + m] = v;
            ok = ok && hfinite(v);
          }
        rec[18] = jx * w * (jznu - hval<H>(1.0));
      }
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int n = 0; n < 3; ++n) rec[9 + k * 3 + n] = sw * adj[k][n];
      if (!ok) atomicOr(P.status, 1u);
    }
  } else {
    for (int t = tid - HALF; t < (P.res_only ? 0 : EG * NG); t += HALF) {
      const int el = t / NG, g = t % NG;
      if (el >= nvalid) continue;
      const int e = elem_at(P, elems, grp * EG + el);
      float Mf[3][3], Ff[3][3], cf[4], Cf[6][6], Sf[6], inv[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int k = 0; k < 3; ++k) Mf[c][k] = hf(s_dz[t * 9 + c * 3 + k]);
      H dnh[9], jxh;
      load_geo(P, e, g, dnh, jxh);
      float dn[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) dn[i] = hf(dnh[i]);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Ff[i][j] = Mf[i][0] * dn[j] + Mf[i][1] * dn[3 + j] + Mf[i][2] * dn[6 + j];
      float adj[3][3];
      adj[0][0] = Mf[1][1] * Mf[2][2] - Mf[1][2] * Mf[2][1];
      adj[0][1] = Mf[0][2] * Mf[2][1] - Mf[0][1] * Mf[2][2];
      adj[0][2] = Mf[0][1] * Mf[1][2] - Mf[0][2] * Mf[1][1];
      adj[1][0] = Mf[1][2] * Mf[2][0] - Mf[1][0] * Mf[2][2];
      adj[1][1] = Mf[0][0] * Mf[2][2] - Mf[0][2] * Mf[2][0];
      adj[1][2] = Mf[0][2] * Mf[1][0] - Mf[0][0] * Mf[1][2];
      adj[2][0] = Mf[1][0] * Mf[2][1] - Mf[1][1] * Mf[2][0];
      adj[2][1] = Mf[0][1] * Mf[2][0] - Mf[0][0] * Mf[2][1];
      adj[2][2] = Mf[0][0] * Mf[1][1] - Mf[0][1] * Mf[1][0];
      const float det = Mf[0][0] * adj[0][0] + Mf[0][1] * adj[1][0] + Mf[0][2] * adj[2][0];
      const float rdet = 1.0f / det;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) inv[i][j] = adj[i][j] * rdet;
      const float jz = fabsf(det);
      const float jznuf = jz / hf(jxh);
      const float jgwf = jz * hf(s_w[g]);
      const float pgf = hf(s_pg[t]);
      const double* cm = P.mat + (P.matpe ? (size_t)e * P.nmat : 0);
#pragma unroll
      for (int i = 0; i < 4; ++i) cf[i] = i < P.nmat ? (float)cm[i] : 0.0f;
      d_gauss_elasticity<float>(P.law, cf, Ff, jznuf, pgf, Cf, Sf);
      float* r32 = &s_r32[t * C::REC32];
#pragma unroll
      for (int blk = 0; blk < 6; ++blk) {
        int m, n;
        blk_mn(blk, m, n);
        float sub[3][3], tmp[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            sub[i][j] = jgwf * (Cf[t2v(i, m)][t2v(j, n)] + (m == n ? Sf[t2v(i, j)] : 0.0f));
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int j = 0; j < 3; ++j) tmp[k][j] = inv[k][0] * sub[0][j] + inv[k][1] * sub[1][j] + inv[k][2] * sub[2][j];
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int l = 0; l < 3; ++l)
            r32[blk * 9 + k * 3 + l] = tmp[k][0] * inv[l][0] + tmp[k][1] * inv[l][1] + tmp[k][2] * inv[l][2];
      }
      if (!(isfinite(Cf[0][0]) && isfinite(Cf[3][3]))) atomicOr(P.status, 1u);
    }
  }
  __syncthreads();
  // P3 (FP64 pipe) and P4 (tensor cores, scatter) are independent; the
  // second wave of CTAs runs them in the opposite order so that the two
  // CTAs sharing an SM work on different pipes.
  for (int ph = 0; ph < 2; ++ph) {
    if ((ph == 0) != p4_first) {
      // ---- P3: residual rows and pressure-coupling columns (high precision H)
      __syncthreads();
      // Sum factorisation over the tensor-product basis:
      //   RK[el][mk][a] = sum_g M_k(g; a) V_g(k, m),  V_g(k, m) = rec_g[roff + 3 k + m],
      // with M_k the product of the 1-D derivative table along xi_k and the
      // 1-D value table along the other two directions; one xi direction
      // contracted per stage.  roff = 0: V = P, the residual rows are
      // sum_k RK; roff = 9: V = A = J_z w dxi/dz, the element-based pressure
      // coupling column of (n, b) is sum_k RK[el][3 n + k][b].
      constexpr int N2 = N1 * N1;
      auto sumfact = [&](int roff) {
        H* U1 = s_dz;                         // [el][mk][a1][g2 + 3 g3]
        H* U2 = reinterpret_cast<H*>(s_f32);  // [el][mk][a1 + N1 a2][g3]
        H* RK = s_dz;                         // [el][mk][a]
        for (int i = tid; i < EG * 9 * N1 * 9; i += C::THREADS) {
          const int j = i % 9, a1 = (i / 9) % N1, mk = (i / (9 * N1)) % 9, el = i / (81 * N1);
          const int m = mk / 3, k = mk % 3;
          const H* M = k == 0 ? s_D1 : s_B1;
          const H* rec = &s_r64[(el * NG + 3 * j) * C::REC64 + roff + k * 3 + m];
          H acc = hval<H>(0.0);
#pragma unroll
          for (int g1 = 0; g1 < 3; ++g1) acc = hfma(M[g1 * N1 + a1], rec[g1 * C::REC64], acc);
          U1[i] = acc;
        }
        __syncthreads();
        for (int i = tid; i < EG * 9 * N2 * 3; i += C::THREADS) {
          const int g3 = i % 3, a1 = (i / 3) % N1, a2 = (i / (3 * N1)) % N1, mk = (i / (3 * N2)) % 9,
                    el = i / (27 * N2);
          const H* M = mk % 3 == 1 ? s_D1 : s_B1;
          const H* u = &U1[((el * 9 + mk) * N1 + a1) * 9 + 3 * g3];
          H acc = hval<H>(0.0);
#pragma unroll
          for (int g2 = 0; g2 < 3; ++g2) acc = hfma(M[g2 * N1 + a2], u[g2], acc);
          U2[i] = acc;
        }
        __syncthreads();
        for (int i = tid; i < EG * 9 * NPE; i += C::THREADS) {
          const int a = i % NPE, mk = (i / NPE) % 9, el = i / (9 * NPE);
          const int a12 = a % N2, a3 = a / N2;
          const H* M = mk % 3 == 2 ? s_D1 : s_B1;
          const H* u = &U2[((el * 9 + mk) * N2 + a12) * 3];
          H acc = hval<H>(0.0);
#pragma unroll
          for (int g3 = 0; g3 < 3; ++g3) acc = hfma(M[g3 * N1 + a3], u[g3], acc);
          RK[i] = acc;
        }
        __syncthreads();
      };
      if (P.r != nullptr) {
        sumfact(0);
        for (int it = tid; it < EG * NROW; it += C::THREADS) {
          const int el = it / NROW, row = it % NROW;
          if (el >= nvalid) continue;
          const H* rec = &s_r64[el * NG * C::REC64];
          const int* nd = &s_node[el * (NR + 1)];
          const uint16_t* tab = P.tables + (size_t)nd[NR] * NR * NR;
          H acc = hval<H>(0.0);
          int ln;
          size_t R;
          if (row < NU3) {
            const int m = row / NPE, a = row % NPE;
            const H* rk = &s_dz[(el * 9 + m * 3) * NPE + a];
            acc = rk[0] + rk[NPE] + rk[2 * NPE];
            ln = a;
            R = (size_t)m * nu + nd[a];
          } else {
            const int q = row - NU3;
            for (int g = 0; g < NG; ++g) acc = PM ? hfma(s_psi[g * 8 + q], rec[g * C::REC64 + 18], acc)
                                                  : acc + rec[g * C::REC64 + 18];
            ln = NPE + q;
            R = (size_t)3 * nu + nd[ln];
          }
          const double accd = hd(acc);
          if constexpr (OUT == 1) {
            SO->r[(size_t)elem_at(P, elems, grp * EG + el) * cmfe::rec_stride_r(NPE, NPP) + row] = accd;
          } else {
            const bool first = tab[ln * NR + ln] & 0x8000;
            if (first)
              P.r[R] = accd;
            else
              atomicAdd(&P.r[R], accd);
          }
        }
      }
      if (!PM && !P.res_only) {
        __syncthreads();  // the residual rows have read RK
        sumfact(9);
        for (int it = tid; it < EG * NU3; it += C::THREADS) {
          const int el = it / NU3, col = it % NU3;
          if (el >= nvalid) continue;
          const int n = col / NPE, b = col % NPE;
          const int* nd = &s_node[el * (NR + 1)];
          const uint16_t* tab = P.tables + (size_t)nd[NR] * NR * NR;
          const H* rk = &s_dz[(el * 9 + n * 3) * NPE + b];
          const double kv = hd(rk[0] + rk[NPE] + rk[2 * NPE]);
          if constexpr (OUT == 1) {
            SO->cp[(size_t)elem_at(P, elems, grp * EG + el) * cmfe::rec_stride_cp(NPE, NPP) + col] = kv;
            continue;
          }
          const int nb = nd[b], pq = nd[NPE];
          const uint16_t tqb = tab[NPE * NR + b], tbq = tab[b * NR + NPE];
          const size_t p1 = (size_t)P.cp_row_ptr[(size_t)3 * nu + pq] + (size_t)n * P.wp[pq] + (tqb & 0x7fff);
          if (tqb & 0x8000)
            P.vals[p1] = kv;
          else
            atomicAdd(&P.vals[p1], kv);
          const size_t p2 = (size_t)P.cp_row_ptr[(size_t)n * nu + nb] + (tbq & 0x7fff);
          if (tbq & 0x8000)
            P.vals[p2] = kv;
          else
            atomicAdd(&P.vals[p2], kv);
        }
      }
      // Pressure-coupling block for nodal (trilinear) pressure,
      //   K(q, n, b) = sum_k sum_g psi_q(g) A_g(k, n) dN_b/dxi_k(g),  A_g = J_z w dxi/dz,
      // psi_q = L(q1) L(q2) L(q3), dN_b/dxi_k = M1k(b1) M2k(b2) M3k(b3) (M = 1-D
      // derivative along xi_k, 1-D value otherwise), by sum factorisation with
      // the products LB = L x value, LD = L x derivative of the 1-D tables.
      // Stage 1 contracts g1 for every (n, k) into T1_n[el][k][q1][b1][g2 + 3 g3]
      // (n = 0, 1 in the s_f32 scratch region, n = 2 in the gradient region,
      // both free by now); then one thread per (n, el, q1, b1, q2, b2)
      // contracts g2 -- the k = 0 and k = 1 terms, which share the value table
      // along xi3, summed into w, the k = 2 term into u -- and g3.
      if (PM && !P.res_only) {
        constexpr int NT1 = 3 * 2 * N1 * 9;  // T1 entries per element and n
        H* T1f = reinterpret_cast<H*>(s_f32);
        const H* LB = s_LM;
        const H* LD = s_LM + 6 * N1;
        __syncthreads();  // the residual rows have read the gradient region
        for (int i = tid; i < 3 * EG * NT1; i += C::THREADS) {
          const int n = i / (EG * NT1), r = i % (EG * NT1);
          const int j = r % 9, b1 = (r / 9) % N1, q1 = (r / (9 * N1)) % 2, k = (r / (18 * N1)) % 3,
                    el = r / NT1;
          const H* lm = (k == 0 ? LD : LB) + q1 * 3 * N1 + b1;
          const H* a = &s_r64[(el * NG + 3 * j) * C::REC64 + 9 + 3 * k + n];
          H* T1 = n < 2 ? T1f + n * EG * NT1 : s_dz;
          T1[r] = hfma(lm[0], a[0], hfma(lm[N1], a[C::REC64], lm[2 * N1] * a[2 * C::REC64]));
        }
        __syncthreads();
        for (int tt = tid; tt < 3 * EG * 4 * N2; tt += C::THREADS) {
          const int n = tt / (EG * 4 * N2), t = tt % (EG * 4 * N2);
          const int b2 = t % N1, q2 = (t / N1) % 2, b1 = (t / (2 * N1)) % N1, q1 = (t / (2 * N2)) % 2,
                    el = t / (4 * N2);
          if (el >= nvalid) continue;
          const H* T1 = n < 2 ? T1f + n * EG * NT1 : s_dz;
          const H* t0 = &T1[el * NT1 + (q1 * N1 + b1) * 9];  // k stride 18 N1
          const H* lb2 = LB + q2 * 3 * N1 + b2;
          const H* ld2 = LD + q2 * 3 * N1 + b2;
          H w[3], u[3];
#pragma unroll
          for (int g3 = 0; g3 < 3; ++g3) {
            H wa = hval<H>(0.0), ua = hval<H>(0.0);
#pragma unroll
            for (int g2 = 0; g2 < 3; ++g2) {
              const int jj = g2 + 3 * g3;
              wa = hfma(lb2[g2 * N1], t0[jj], wa);
              wa = hfma(ld2[g2 * N1], t0[18 * N1 + jj], wa);
              ua = hfma(lb2[g2 * N1], t0[36 * N1 + jj], ua);
            }
            w[g3] = wa;
            u[g3] = ua;
          }
          const int* nd = &s_node[el * (NR + 1)];
          const uint16_t* tab = P.tables + (size_t)nd[NR] * NR * NR;
#pragma unroll
          for (int q3 = 0; q3 < 2; ++q3)
#pragma unroll
            for (int b3 = 0; b3 < N1; ++b3) {
              H acc = hval<H>(0.0);
#pragma unroll
              for (int g3 = 0; g3 < 3; ++g3)
                acc = hfma(LD[(q3 * 3 + g3) * N1 + b3], u[g3], hfma(LB[(q3 * 3 + g3) * N1 + b3], w[g3], acc));
              const int q = q1 + 2 * q2 + 4 * q3, b = b1 + N1 * b2 + N2 * b3;
              const double kv = hd(acc);
              if constexpr (OUT == 1) {
                SO->cp[(size_t)elem_at(P, elems, grp * EG + el) * cmfe::rec_stride_cp(NPE, NPP) + q * NU3 + n * NPE + b] = kv;
                continue;
              }
              const int lq = NPE + q, pq = nd[lq], nb = nd[b];
              const uint16_t tqb = tab[lq * NR + b], tbq = tab[b * NR + lq];
              const size_t p1 = (size_t)P.cp_row_ptr[(size_t)3 * nu + pq] + (size_t)n * P.wp[pq] + (tqb & 0x7fff);
              if (tqb & 0x8000)
                P.vals[p1] = kv;
              else
                atomicAdd(&P.vals[p1], kv);
              const size_t p2 = (size_t)P.cp_row_ptr[(size_t)n * nu + nb] + (tbq & 0x7fff);
              if (tbq & 0x8000)
                P.vals[p2] = kv;
              else
                atomicAdd(&P.vals[p2], kv);
            }
        }
      }
      // structurally zero pressure-pressure entries, stored by their first contributor
      for (int i = tid; i < (P.res_only || OUT == 1 ? 0 : EG * NPP * NPP); i += C::THREADS) {
        const int el = i / (NPP * NPP), q = (i / NPP) % NPP, q2 = i % NPP;
        if (el >= nvalid) continue;
        const int* nd = &s_node[el * (NR + 1)];
        const uint16_t t = P.tables[(size_t)nd[NR] * NR * NR + (NPE + q) * NR + NPE + q2];
        if (t & 0x8000) {
          const int pq = nd[NPE + q];
          P.vals[(size_t)P.cp_row_ptr[(size_t)3 * nu + pq] + 3 * (size_t)P.wp[pq] + (t & 0x7fff)] = 0.0;
        }
      }
    } else {
      // ---- P4: displacement blocks on tensor cores (FP32 accumulate).
      // The six lower blocks of one element are stacked along M:
      //   D'[(blk,b)][a] = sum_kappa W^{blk}[kappa][b] Phi[kappa][a] = K^{blk}(a,b),
      // kappa = 28k + g (derivative-major, one padding slot per derivative).  Each warp owns (element, m-tile) tasks; it forms its
      // A fragments (W values) in registers from the per-Gauss-point D^{blk}
      // records and the gradient table, and takes B = Phi from shared memory.
      if (!P.res_only) {
        // Rows of the stacked blocks: block blk occupies rows [blk * BS, blk * BS + NPE).
        // For triquadratic elements BS = 32, so that a 16-row tile never spans
        // two blocks and the two rows a thread holds share the D^{blk} loads.
        constexpr int BS = NPE > 16 ? 32 : NPE;
        constexpr int MROWS = 6 * BS;
        constexpr int MT2 = (MROWS + 15) / 16;
        const int gq = lane >> 2, tq = lane & 3;
        const uint32_t* Bhi = s_A;
        const uint32_t* Blo = s_A + C::AROWS * KPW;
        // Scatter addresses staged in shared memory (regions P3 does not read
        // while this stage runs): base[el][3m+n][a] = start of the n-block of
        // row (m, node a), and the element's rank table over its u nodes.
        int* s_base = reinterpret_cast<int*>(s_dz);
        uint16_t* s_tab = reinterpret_cast<uint16_t*>(s_f32);
        __syncthreads();
        if constexpr (OUT == 0) {
          for (int i = tid; i < EG * 9 * NPE; i += C::THREADS) {
            const int a = i % NPE, mn = (i / NPE) % 9, el = i / (9 * NPE);
            const int na = s_node[el * (NR + 1) + a];
            s_base[i] = el < nvalid ? P.uu_row_ptr[(size_t)(mn / 3) * nu + na] + (mn % 3) * P.wu[na] : 0;
          }
          for (int i = tid; i < EG * NPE * NPE; i += C::THREADS) {
            const int ab = i % (NPE * NPE), el = i / (NPE * NPE);
            const int a = ab / NPE, b = ab % NPE;
            s_tab[i] = el < nvalid ? P.tables[(size_t)s_node[el * (NR + 1) + NR] * NR * NR + a * NR + b] : 0;
          }
          __syncthreads();
        }
        for (int task = warp; task < nvalid * MT2; task += C::THREADS / 32) {
          const int el = task / MT2, mt = task % MT2;
          const int* bs = &s_base[el * 9 * NPE];
          const uint16_t* tb = &s_tab[el * NPE * NPE];
          const float* r32 = &s_r32[el * NG * C::REC32];
          float acc[C::NT][4];
#pragma unroll
          for (int nt = 0; nt < C::NT; ++nt)
#pragma unroll
            for (int h = 0; h < 4; ++h) acc[nt][h] = 0.f;
          const int R0 = 16 * mt + gq, R1 = R0 + 8;
          const int blk0 = R0 / BS, b0 = R0 % BS, blk1 = R1 / BS, b1 = R1 % BS;
          const bool v0 = R0 < MROWS && b0 < NPE, v1 = R1 < MROWS && b1 < NPE;
#pragma unroll 1
          for (int kt = 0; kt < C::KT; ++kt) {
            float wv[2][4];  // [row r0/r1][kappa 2t, 2t+1, 2t+8, 2t+9]
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int kap = 16 * kt + 2 * tq + (j & 1) + (j >= 2 ? 8 : 0);
              const int k = kap / 28, g = kap % 28;
              const bool kv = kap < C::KAP && g < NG;
              float w0 = 0.f, w1 = 0.f;
              if constexpr (BS % 16 == 0) {  // both rows in block blk0
                if (kv && (v0 || v1)) {
                  const float* dt = &r32[g * C::REC32 + blk0 * 9 + k * 3];
                  const float d0 = dt[0], d1 = dt[1], d2 = dt[2];
                  if (v0) {
                    const float4 ph = *reinterpret_cast<const float4*>(&s_phi32[g * C::PHS + 4 * b0]);
                    w0 = d0 * ph.x + d1 * ph.y + d2 * ph.z;
                  }
                  if (v1) {
                    const float4 ph = *reinterpret_cast<const float4*>(&s_phi32[g * C::PHS + 4 * b1]);
                    w1 = d0 * ph.x + d1 * ph.y + d2 * ph.z;
                  }
                }
              } else {
                if (kv && v0) {
                  const float* dt = &r32[g * C::REC32 + blk0 * 9 + k * 3];
                  const float4 ph = *reinterpret_cast<const float4*>(&s_phi32[g * C::PHS + 4 * b0]);
                  w0 = dt[0] * ph.x + dt[1] * ph.y + dt[2] * ph.z;
                }
                if (kv && v1) {
                  const float* dt = &r32[g * C::REC32 + blk1 * 9 + k * 3];
                  const float4 ph = *reinterpret_cast<const float4*>(&s_phi32[g * C::PHS + 4 * b1]);
                  w1 = dt[0] * ph.x + dt[1] * ph.y + dt[2] * ph.z;
                }
              }
              wv[0][j] = w0;
              wv[1][j] = w1;
            }
            uint32_t ah[4], al[4];
            split_bf16(wv[0][0], wv[0][1], ah[0], al[0]);  // row r0, cols 2t..2t+1
            split_bf16(wv[1][0], wv[1][1], ah[1], al[1]);  // row r1, cols 2t..2t+1
            split_bf16(wv[0][2], wv[0][3], ah[2], al[2]);  // row r0, cols 2t+8..
            split_bf16(wv[1][2], wv[1][3], ah[3], al[3]);  // row r1, cols 2t+8..
#pragma unroll
            for (int nt = 0; nt < C::NT; ++nt) {
              // B fragments of this n-tile: high and low parts, kappa halves
              // 16 kt .. 16 kt + 7 and 16 kt + 8 .. 16 kt + 15, in one ldmatrix
              const int mi = lane >> 3;
              uint32_t bf[4];
              ldmatrix_x4(bf, (mi < 2 ? Bhi : Blo) + (8 * nt + (lane & 7)) * KPW + 8 * kt + 4 * (mi & 1));
              mma_bf16(acc[nt], ah[0], ah[1], ah[2], ah[3], bf[0], bf[1]);
              if (SPLIT == 3) {
                mma_bf16(acc[nt], ah[0], ah[1], ah[2], ah[3], bf[2], bf[3]);
                mma_bf16(acc[nt], al[0], al[1], al[2], al[3], bf[0], bf[1]);
              }
            }
          }
          // scatter K^{blk}(a, b) and its mirror
#pragma unroll
          for (int nt = 0; nt < C::NT; ++nt)
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              const bool vr = h < 2 ? v0 : v1;
              const int blk = h < 2 ? blk0 : blk1, b = h < 2 ? b0 : b1;
              const int a = 8 * nt + 2 * tq + (h & 1);
              if (!vr || a >= NPE) continue;
              int m, n;
              blk_mn(blk, m, n);
              if (m == n && a < b) continue;
              const float v = acc[nt][h];
              if constexpr (OUT == 1) {
                float* st = SO->uu + (size_t)elem_at(P, elems, grp * EG + el) * cmfe::rec_stride_uu(NPE);
                st[(size_t)(m * NPE + a) * NU3 + n * NPE + b] = v;
                if (!(m == n && a == b)) st[(size_t)(n * NPE + b) * NU3 + m * NPE + a] = v;
                continue;
              }
              const uint16_t tab_ab = tb[a * NPE + b];
              const int p1 = bs[(m * 3 + n) * NPE + a] + (tab_ab & 0x7fff);
              if (tab_ab & 0x8000)
                P.vals_uu[p1] = v;
              else
                atomicAdd(&P.vals_uu[p1], v);
              if (!(m == n && a == b)) {
                const uint16_t tab_ba = tb[b * NPE + a];
                const int p2 = bs[(n * 3 + m) * NPE + b] + (tab_ba & 0x7fff);
                if (tab_ba & 0x8000)
                  P.vals_uu[p2] = v;
                else
                  atomicAdd(&P.vals_uu[p2], v);
              }
            }
        }
        __syncthreads();  // P3 may run next and reuse the staging regions
      }
    }
  }
}

}  // namespace
