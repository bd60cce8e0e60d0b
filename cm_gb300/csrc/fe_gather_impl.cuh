// libcm_fe: the row gather of the staged assembly, device code shared by the
// separate gather kernel (fe_gather.cu) and the fused assembly kernel
// (fe_mixed.cu), which gathers a node's rows as soon as the last element
// around the node has stored its records.
//
// One warp forms the rows of one row node from the per-element records
// (StageOut) of the elements around it, adding them in increasing element
// number -- a fixed order, so the result is deterministic -- into a
// shared-memory copy of the rows, and then writes each row once,
// contiguously.  This is the addition of EQUATIONS_MATRICES_JACOBIAN_ELEMENT_ADD
// / MATRIX_VALUES_ADD_DP2 (equations_matrices_routines.f90:3174-3225,
// matrix_vector.f90:2756-2880) and of the residual vector add
// (distributed_matrix_vector.f90:8853-8927), organised by rows instead of by
// elements: every matrix sector is written once, in full, and never read.
//
// The incidences of a row node are read 32 at a time, lane i loading
// incidence i and its element's rank-table row, and handed to the warp by
// shuffles: the loads of one incidence (its ranks and record values) then
// depend on no other load.
//
// Row layout (the mixed split of the handle): a displacement row (m, a)
// holds [u_x | u_y | u_z] blocks of wu[a] columns in the FP32 array at
// uu_row_ptr[m nu + a] and its pressure columns in the FP64 array at
// cp_row_ptr[m nu + a]; a pressure row q holds [u_x | u_y | u_z] blocks of
// wp[q] columns and then its pressure-pressure columns (structural zeros) at
// cp_row_ptr[3 nu + q].  The column of a neighbour inside a block is its rank
// in the row node's neighbour list, read from the element's rank table.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "fe_internal.h"

namespace {

// Record loads: through L2 only (CG = true) when other CTAs of the same
// launch wrote the records, which this SM's L1 does not see.
template <bool CG, class T>
__device__ __forceinline__ T rec_load(const T* p) {
  if constexpr (CG)
    return __ldcg(p);
  else
    return *p;
}

// The three displacement rows of u node a, by one warp; `mine` is the warp's
// shared scratch (36 wu bytes rounded up to 16, then 24 wc bytes).
template <int NPE, int NPP, bool CG>
__device__ __forceinline__ void gather_unode(const cmfe::KParams& P, const cmfe::StageOut& S, const int32_t* u_inc_ptr,
                                             const int32_t* u_inc, int a, unsigned char* mine, int lane) {
  constexpr int NR = NPE + NPP, NU3 = 3 * NPE;
  const int nu = P.nu;
  const int wu = P.wu[a];
  const int ru = 3 * wu;  // uu row length
  const int wc = P.cp_row_ptr[(size_t)a + 1] - P.cp_row_ptr[(size_t)a];  // pressure columns, the same for m = 0..2
  float* acc_u = reinterpret_cast<float*>(mine);                            // [3][ru]
  double* acc_c = reinterpret_cast<double*>(mine + ((12 * ru + 15) & ~15));  // [3][wc]
  for (int i = lane; i < 3 * ru; i += 32) acc_u[i] = 0.f;
  for (int i = lane; i < 3 * wc; i += 32) acc_c[i] = 0.0;
  double racc = 0.0;
  __syncwarp();
  const int k0 = u_inc_ptr[a], k1 = u_inc_ptr[a + 1];
  for (int kb = k0; kb < k1; kb += 32) {
    // up to 32 incidences at once: lane i holds incidence kb + i and its rank-table row
    const int cnt = min(32, k1 - kb);
    int pk = 0, trow = 0;
    if (lane < cnt) {
      pk = u_inc[kb + lane];
      trow = P.elem_table[pk >> 5] * NR + (pk & 31);
    }
    for (int j = 0; j < cnt; ++j) {
      const int packed = __shfl_sync(0xffffffffu, pk, j);
      const int e = packed >> 5, la = packed & 31;
      const uint16_t* tab = P.tables + (size_t)__shfl_sync(0xffffffffu, trow, j) * NR;
      if (lane < NPE) {
        const int rk = tab[lane] & 0x7fff;
        const float* src = S.uu + (size_t)e * cmfe::rec_stride_uu(NPE) + (size_t)la * NU3 + lane;
        float v[9];
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
          for (int n = 0; n < 3; ++n) v[m * 3 + n] = rec_load<CG>(src + (size_t)m * NPE * NU3 + n * NPE);
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
          for (int n = 0; n < 3; ++n) acc_u[m * ru + n * wu + rk] += v[m * 3 + n];
      }
      if (lane < NPP) {
        const int rq = tab[NPE + lane] & 0x7fff;
        const double* src = S.cp + (size_t)e * cmfe::rec_stride_cp(NPE, NPP) + lane * NU3 + la;
#pragma unroll
        for (int m = 0; m < 3; ++m) acc_c[m * wc + rq] += rec_load<CG>(src + m * NPE);
      }
      if (lane < 3 && P.r) racc += rec_load<CG>(S.r + (size_t)e * cmfe::rec_stride_r(NPE, NPP) + lane * NPE + la);
      __syncwarp();
    }
  }
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    float* du = P.vals_uu + P.uu_row_ptr[(size_t)m * nu + a];
    for (int i = lane; i < ru; i += 32) du[i] = acc_u[m * ru + i];
    double* dc = P.vals + P.cp_row_ptr[(size_t)m * nu + a];
    for (int i = lane; i < wc; i += 32) dc[i] = acc_c[m * wc + i];
  }
  if (lane < 3 && P.r) P.r[(size_t)lane * nu + a] = racc;
  __syncwarp();
}

// The row of pressure row node q, by one warp (scratch: 8 bytes per column).
template <int NPE, int NPP, bool CG>
__device__ __forceinline__ void gather_pnode(const cmfe::KParams& P, const cmfe::StageOut& S, const int32_t* p_inc_ptr,
                                             const int32_t* p_inc, int q, unsigned char* mine, int lane) {
  constexpr int NR = NPE + NPP, NU3 = 3 * NPE;
  const size_t row = (size_t)3 * P.nu + q;
  const int wp = P.wp[q];
  const int len = P.cp_row_ptr[row + 1] - P.cp_row_ptr[row];
  double* acc = reinterpret_cast<double*>(mine);  // [len]
  for (int i = lane; i < len; i += 32) acc[i] = 0.0;  // pressure-pressure entries stay zero
  double racc = 0.0;
  __syncwarp();
  const int k0 = p_inc_ptr[q], k1 = p_inc_ptr[q + 1];
  for (int kb = k0; kb < k1; kb += 32) {
    const int cnt = min(32, k1 - kb);
    int pk = 0, trow = 0;
    if (lane < cnt) {
      pk = p_inc[kb + lane];
      trow = P.elem_table[pk >> 3] * NR + NPE + (pk & 7);
    }
    for (int j = 0; j < cnt; ++j) {
      const int packed = __shfl_sync(0xffffffffu, pk, j);
      const int tr = __shfl_sync(0xffffffffu, trow, j);
      const int e = packed >> 3, lq = packed & 7;
      if (lane < NPE) {
        const int rk = P.tables[(size_t)tr * NR + lane] & 0x7fff;
        const double* src = S.cp + (size_t)e * cmfe::rec_stride_cp(NPE, NPP) + lq * NU3 + lane;
        double v[3];
#pragma unroll
        for (int n = 0; n < 3; ++n) v[n] = rec_load<CG>(src + n * NPE);
#pragma unroll
        for (int n = 0; n < 3; ++n) acc[n * wp + rk] += v[n];
      }
      if (lane == 0 && P.r) racc += rec_load<CG>(S.r + (size_t)e * cmfe::rec_stride_r(NPE, NPP) + NU3 + lq);
      __syncwarp();
    }
  }
  double* dc = P.vals + P.cp_row_ptr[row];
  for (int i = lane; i < len; i += 32) dc[i] = acc[i];
  if (lane == 0 && P.r) P.r[row] = racc;
  __syncwarp();
}

}  // namespace
