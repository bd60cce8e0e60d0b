// libcm_fe: row gather of the staged assembly (sm_103a).
//
// The staged mixed kernel stores every element's displacement block (FP32,
// full 3 NPE x 3 NPE, mirrored), its pressure-coupling rows (FP64) and its
// residual (FP64) into per-element records.  This kernel forms the CSR rows
// from them: one warp per row node, which adds the contributions of the
// elements around the node in increasing element number -- a fixed order, so
// the result is deterministic -- into a shared-memory copy of the node's rows
// and then writes each row once, contiguously.  This is the addition of
// EQUATIONS_MATRICES_JACOBIAN_ELEMENT_ADD / MATRIX_VALUES_ADD_DP2
// (equations_matrices_routines.f90:3174-3225, matrix_vector.f90:2756-2880)
// and of the residual vector add (distributed_matrix_vector.f90:8853-8927),
// organised by rows instead of by elements: every matrix sector is written
// once, in full, and never read, where adding element by element into a
// matrix larger than L2 reads and writes each sector once per element
// colour.
//
// Row layout (the mixed split of the handle): a displacement row (m, a)
// holds [u_x | u_y | u_z] blocks of wu[a] columns in the FP32 array at
// uu_row_ptr[m nu + a] and its pressure columns in the FP64 array at
// cp_row_ptr[m nu + a]; a pressure row q holds [u_x | u_y | u_z] blocks of
// wp[q] columns and then its pressure-pressure columns (structural zeros) at
// cp_row_ptr[3 nu + q].  The column of a neighbour inside a block is its rank
// in the row node's neighbour list, read from the element's rank table.
#include <cuda_runtime.h>

#include <cstdint>

#include "fe_internal.h"

using cmfe::HostSetup;
using cmfe::KParams;

namespace {

constexpr int GW = 8;  // warps per CTA

struct GatherArgs {
  KParams P;
  cmfe::StageOut S;
  const int32_t* u_inc_ptr;
  const int32_t* u_inc;
  const int32_t* p_inc_ptr;
  const int32_t* p_inc;
  int npn;            // pressure row nodes
  int warp_bytes;     // shared memory per warp
};

template <int NPE, int NPP>
__global__ void __launch_bounds__(32 * GW) fe_gather_kernel(GatherArgs A) {
  constexpr int NR = NPE + NPP, NU3 = 3 * NPE, NROW = NU3 + NPP;
  extern __shared__ __align__(16) unsigned char gsm[];
  const KParams& P = A.P;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* mine = gsm + (size_t)warp * A.warp_bytes;
  const int nu = P.nu;
  const int total = nu + A.npn;
  for (int w = blockIdx.x * GW + warp; w < total; w += gridDim.x * GW) {
    if (w < nu) {
      // ---- the three displacement rows of u node a
      const int a = w;
      const int wu = P.wu[a];
      const int ru = 3 * wu;                 // uu row length
      int wc[3];
#pragma unroll
      for (int m = 0; m < 3; ++m) wc[m] = P.cp_row_ptr[(size_t)m * nu + a + 1] - P.cp_row_ptr[(size_t)m * nu + a];
      float* acc_u = reinterpret_cast<float*>(mine);                            // [3][ru]
      double* acc_c = reinterpret_cast<double*>(mine + ((12 * ru + 15) & ~15));  // [3][wc]
      for (int i = lane; i < 3 * ru; i += 32) acc_u[i] = 0.f;
      for (int i = lane; i < 3 * wc[0]; i += 32) acc_c[i] = 0.0;
      double racc = 0.0;
      __syncwarp();
      const int k1 = A.u_inc_ptr[a + 1];
      for (int k = A.u_inc_ptr[a]; k < k1; ++k) {
        const int packed = A.u_inc[k];
        const int e = packed >> 5, la = packed & 31;
        const uint16_t* tab = P.tables + ((size_t)P.elem_table[e] * NR + la) * NR;
        if (lane < NPE) {
          const int rk = tab[lane] & 0x7fff;
          const float* src = A.S.uu + (size_t)e * NU3 * NU3 + (size_t)la * NU3 + lane;
          float v[9];
#pragma unroll
          for (int m = 0; m < 3; ++m)
#pragma unroll
            for (int n = 0; n < 3; ++n) v[m * 3 + n] = src[(size_t)m * NPE * NU3 + n * NPE];
#pragma unroll
          for (int m = 0; m < 3; ++m)
#pragma unroll
            for (int n = 0; n < 3; ++n) acc_u[m * ru + n * wu + rk] += v[m * 3 + n];
        }
        if (lane < NPP) {
          const int rq = tab[NPE + lane] & 0x7fff;
          const double* src = A.S.cp + ((size_t)e * NPP + lane) * NU3 + la;
#pragma unroll
          for (int m = 0; m < 3; ++m) acc_c[m * wc[0] + rq] += src[m * NPE];
        }
        if (lane < 3 && P.r) racc += A.S.r[(size_t)e * NROW + lane * NPE + la];
        __syncwarp();
      }
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        float* du = P.vals_uu + P.uu_row_ptr[(size_t)m * nu + a];
        for (int i = lane; i < ru; i += 32) du[i] = acc_u[m * ru + i];
        double* dc = P.vals + P.cp_row_ptr[(size_t)m * nu + a];
        for (int i = lane; i < wc[m]; i += 32) dc[i] = acc_c[m * wc[0] + i];
      }
      if (lane < 3 && P.r) P.r[(size_t)lane * nu + a] = racc;
      __syncwarp();
    } else {
      // ---- the row of pressure row node q
      const int q = w - nu;
      const size_t row = (size_t)3 * nu + q;
      const int wp = P.wp[q];
      const int len = P.cp_row_ptr[row + 1] - P.cp_row_ptr[row];
      double* acc = reinterpret_cast<double*>(mine);  // [len]
      for (int i = lane; i < len; i += 32) acc[i] = 0.0;  // pressure-pressure entries stay zero
      double racc = 0.0;
      __syncwarp();
      const int k1 = A.p_inc_ptr[q + 1];
      for (int k = A.p_inc_ptr[q]; k < k1; ++k) {
        const int packed = A.p_inc[k];
        const int e = packed >> 3, lq = packed & 7;
        if (lane < NPE) {
          const uint16_t* tab = P.tables + ((size_t)P.elem_table[e] * NR + NPE + lq) * NR;
          const int rk = tab[lane] & 0x7fff;
          const double* src = A.S.cp + ((size_t)e * NPP + lq) * NU3 + lane;
          double v[3];
#pragma unroll
          for (int n = 0; n < 3; ++n) v[n] = src[n * NPE];
#pragma unroll
          for (int n = 0; n < 3; ++n) acc[n * wp + rk] += v[n];
        }
        if (lane == 0 && P.r) racc += A.S.r[(size_t)e * NROW + NU3 + lq];
        __syncwarp();
      }
      double* dc = P.vals + P.cp_row_ptr[row];
      for (int i = lane; i < len; i += 32) dc[i] = acc[i];
      if (lane == 0 && P.r) P.r[row] = racc;
      __syncwarp();
    }
  }
}

template <int NPE, int NPP>
int launch_t(const GatherArgs& a, int num_sms, cudaStream_t st) {
  auto kern = fe_gather_kernel<NPE, NPP>;
  const int smem = GW * a.warp_bytes;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return (int)e;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * GW, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  const long long warps = (long long)a.P.nu + a.npn;
  long long grid = (warps + GW - 1) / GW;
  if (grid > (long long)per_sm * num_sms) grid = (long long)per_sm * num_sms;
  kern<<<(int)grid, 32 * GW, smem, st>>>(a);
  return (int)cudaGetLastError();
}

}  // namespace

namespace cmfe {

int launch_gather(const HostSetup& s, const KParams& kp, const StageOut& so, const int32_t* u_inc_ptr,
                  const int32_t* u_inc, const int32_t* p_inc_ptr, const int32_t* p_inc, int num_sms, void* stream) {
  GatherArgs a;
  a.P = kp;
  a.S = so;
  a.u_inc_ptr = u_inc_ptr;
  a.u_inc = u_inc;
  a.p_inc_ptr = p_inc_ptr;
  a.p_inc = p_inc;
  a.npn = s.npn;
  if ((int64_t)s.gather_bytes * GW > 227 * 1024) return (int)cudaErrorInvalidConfiguration;
  a.warp_bytes = s.gather_bytes;
  cudaStream_t st = (cudaStream_t)stream;
  if (s.n1 == 2) return s.pmode ? launch_t<8, 8>(a, num_sms, st) : launch_t<8, 1>(a, num_sms, st);
  return s.pmode ? launch_t<27, 8>(a, num_sms, st) : launch_t<27, 1>(a, num_sms, st);
}

}  // namespace cmfe
