// libcm_fe: row gather of the staged assembly as its own kernel (sm_103a).
//
// The staged mixed kernel stores every element's displacement block (FP32,
// full 3 NPE x 3 NPE, mirrored), its pressure-coupling rows (FP64) and its
// residual (FP64) into per-element records; this kernel then forms every CSR
// row from them, one warp per row node (device code in fe_gather_impl.cuh).
// Every matrix sector is written once, in full, and never read, where adding
// element by element into a matrix larger than L2 reads and writes each
// sector once per element colour.  The fused assembly kernel (fe_mixed.cu)
// does the same gathers inside its own launch; this kernel serves meshes
// whose node neighbourhoods are too large for the fused kernel's scratch.
#include <cuda_runtime.h>

#include <cstdint>

#include "fe_gather_impl.cuh"
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
  extern __shared__ __align__(16) unsigned char gsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* mine = gsm + (size_t)warp * A.warp_bytes;
  const int nu = A.P.nu;
  const int total = nu + A.npn;
  for (int w = blockIdx.x * GW + warp; w < total; w += gridDim.x * GW) {
    if (w < nu)
      gather_unode<NPE, NPP, false>(A.P, A.S, A.u_inc_ptr, A.u_inc, w, mine, lane);
    else
      gather_pnode<NPE, NPP, false>(A.P, A.S, A.p_inc_ptr, A.p_inc, w - nu, mine, lane);
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
