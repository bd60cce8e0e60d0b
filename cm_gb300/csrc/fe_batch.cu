// libcm_fe: batched mixed-precision assembly of many equations sets in one
// persistent launch (sm_103a).
//
// The members of a batch are independent meshes (any mix of trilinear and
// triquadratic elements, element-based or nodal pressure).  One cooperative
// launch walks the element colours in order; for colour c it processes the
// colour-c element groups of every member (work items sorted by element type,
// so a CTA reloads its constant tables rarely), then all CTAs meet at a grid
// barrier before colour c + 1.  Within a member the colour order is the one
// of the single-set path, so every CSR slot receives its contributions in the
// same order: repeated launches are bit-identical, and the result agrees with
// one fe_jacobian_evaluate_mixed call per member to the rounding of the
// separately compiled device code.
//
// Members with a surface-pressure load get, after the volume work of each
// colour and a grid barrier, that colour's boundary elements (one warp each)
// and a second barrier, the order of the single-set path.
//
// The grid barrier spins with a bounded number of polls: if it ever gives up
// (which only a non-co-resident grid could cause, and the cooperative launch
// rules that out), it sets bit 1 of the batch status word and the host call
// reports an error instead of hanging.
#include "fe_mixed_impl.cuh"
#include "fe_surface_impl.cuh"

#include <cooperative_groups.h>

namespace {

constexpr int BT_THREADS = 256;
constexpr unsigned BARRIER_POLLS = 1u << 24;  // x ~256 ns sleep: a few seconds at most

using cmfe::BatchArgs;
using cmfe::BatchPtrs;

__device__ void grid_barrier(const BatchArgs& A) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = A.bar_gen;
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(A.bar_count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(A.bar_count, 0u);
      __threadfence();
      atomicAdd(A.bar_gen, 1u);
    } else {
      unsigned polls = 0;
      while (*gen == g) {
        if (++polls > BARRIER_POLLS) {
          atomicOr(A.status, 2u);
          break;
        }
        __nanosleep(256);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

template <int EGQ, int EGL>
struct BatchCfg {
  static constexpr int s(int a, int b) { return a > b ? a : b; }
  static constexpr int WORK = s(s(s(MixCfg<2, 0, EGL>::SMEM, MixCfg<2, 1, EGL>::SMEM),
                                  s(MixCfg<3, 0, EGQ>::SMEM, MixCfg<3, 1, EGQ>::SMEM)),
                                (int)(BT_THREADS / 32 * sizeof(SurfWarpSmem)));
  static constexpr int O_WORK = align16((int)sizeof(KParams));
  static constexpr int SMEM = O_WORK + WORK;
};

template <int EGQ, int EGL, class H>
__device__ __forceinline__ void load_tables(int type, const KParams& P, unsigned char* w) {
  switch (type) {
    case 0: mix_tables<2, 0, EGL, H>(P, w); break;
    case 1: mix_tables<2, 1, EGL, H>(P, w); break;
    case 2: mix_tables<3, 0, EGQ, H>(P, w); break;
    default: mix_tables<3, 1, EGQ, H>(P, w); break;
  }
}

template <int EGQ, int EGL, class H>
__device__ __forceinline__ void run_group(int type, const KParams& P, int grp, bool p4_first, unsigned char* w) {
  switch (type) {
    case 0: mix_group<2, 0, EGL, 3, H>(P, grp, p4_first, w); break;
    case 1: mix_group<2, 1, EGL, 3, H>(P, grp, p4_first, w); break;
    case 2: mix_group<3, 0, EGQ, 3, H>(P, grp, p4_first, w); break;
    default: mix_group<3, 1, EGQ, 3, H>(P, grp, p4_first, w); break;
  }
}

template <int EGQ, int EGL, int MINB, class H>
__global__ void __launch_bounds__(BT_THREADS, MINB) fe_mixed_batch_kernel(BatchArgs A) {
  using B = BatchCfg<EGQ, EGL>;
  extern __shared__ __align__(16) unsigned char sm[];
  KParams* kp = reinterpret_cast<KParams*>(sm);
  unsigned char* work = sm + B::O_WORK;
  int cur_kp = -1, cur_type = -1;
  const bool p4_first = (blockIdx.x / A.wave) & 1;
  for (int c = 0; c < A.ncolours; ++c) {
    for (int w = A.item_ptr[c] + blockIdx.x; w < A.item_ptr[c + 1]; w += gridDim.x) {
      const int4 it = reinterpret_cast<const int4*>(A.items)[w];
      if (it.x != cur_kp) {
        __syncthreads();  // every thread is done with the previous parameters
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&A.kps[it.x]);
        uint32_t* dst = reinterpret_cast<uint32_t*>(kp);
        for (int i = threadIdx.x; i < (int)(sizeof(KParams) / 4); i += blockDim.x) dst[i] = src[i];
        __syncthreads();
        if (threadIdx.x == 0) {
          const BatchPtrs p = A.ptrs[it.x / A.ncol_kp];
          kp->x = p.x;
          kp->r = p.r;
          kp->vals = p.vals;
          kp->vals_uu = p.vals_uu;
        }
        __syncthreads();
        cur_kp = it.x;
      }
      if (it.w != cur_type) {
        __syncthreads();
        load_tables<EGQ, EGL, H>(it.w, *kp, work);
        cur_type = it.w;  // mix_group starts with a barrier, after which the tables are visible
      }
      for (int g = it.y; g < it.y + it.z; ++g) run_group<EGQ, EGL, H>(it.w, *kp, g, p4_first, work);
    }
    grid_barrier(A);
    if (A.sitem_ptr[c + 1] > A.sitem_ptr[c]) {  // surface loads of this colour (grid-uniform test)
      SurfWarpSmem* ws = reinterpret_cast<SurfWarpSmem*>(work);
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      for (int w = A.sitem_ptr[c] + blockIdx.x; w < A.sitem_ptr[c + 1]; w += gridDim.x) {
        const int4 it = reinterpret_cast<const int4*>(A.sitems)[w];
        __syncthreads();
        if (it.x != cur_kp) {
          const uint32_t* src = reinterpret_cast<const uint32_t*>(&A.kps[it.x]);
          uint32_t* dst = reinterpret_cast<uint32_t*>(kp);
          for (int i = threadIdx.x; i < (int)(sizeof(KParams) / 4); i += blockDim.x) dst[i] = src[i];
          __syncthreads();
          if (threadIdx.x == 0) {
            const BatchPtrs p = A.ptrs[it.x / A.ncol_kp];
            kp->x = p.x;
            kp->r = p.r;
            kp->vals = p.vals;
            kp->vals_uu = p.vals_uu;
          }
          __syncthreads();
          cur_kp = it.x;
        }
        const cmfe::BatchSurf sf = A.surf[it.x / A.ncol_kp];
        if (warp < it.z) {
          const int e = sf.belems[it.y + warp];
          if (it.w == 3)
            surface_element<3>(*kp, e, sf.bmask, 0, 1, ws[warp], lane);
          else
            surface_element<2>(*kp, e, sf.bmask, 0, 1, ws[warp], lane);
        }
      }
      cur_type = -1;  // the constant tables were overwritten
      grid_barrier(A);
    }
  }
}

// Launch variants the autotuner chooses from: elements per group for
// triquadratic / trilinear members, and the CTAs per SM the register budget
// is compiled for (3 = 80 registers, some spills; 2 = 128).
struct Variant {
  int egq, egl, minb;
};
constexpr Variant VARIANTS[] = {{4, 8, 2}, {4, 4, 2}, {2, 4, 2}, {2, 2, 2}, {3, 2, 3}};
constexpr int NVARIANTS = 5;

template <int EGQ, int EGL, int MINB = 2>
int launch_variant(const BatchArgs& a, int ctas_per_sm, int num_sms, cudaStream_t st, int* grid_out) {
  using B = BatchCfg<EGQ, EGL>;
  auto kern = fe_mixed_batch_kernel<EGQ, EGL, MINB, double>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, B::SMEM);
    if (e != cudaSuccess) return (int)e;
    attr = true;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BT_THREADS, B::SMEM);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  const int use = ctas_per_sm < per_sm ? ctas_per_sm : per_sm;
  const int grid = use * num_sms;
  BatchArgs args = a;
  args.wave = num_sms;
  void* params[] = {&args};
  e = cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(BT_THREADS), params, B::SMEM, st);
  if (grid_out) *grid_out = grid;
  return (int)e;
}

}  // namespace

namespace cmfe {

int batch_variants() { return NVARIANTS; }

int batch_variant_eg(int v, int* egq, int* egl) {
  if (v < 0 || v >= NVARIANTS) return -1;
  *egq = VARIANTS[v].egq;
  *egl = VARIANTS[v].egl;
  return 0;
}

int batch_smem(int v) {
  switch (v) {
    case 0: return BatchCfg<4, 8>::SMEM;
    case 1: return BatchCfg<4, 4>::SMEM;
    case 2: return BatchCfg<2, 4>::SMEM;
    case 3: return BatchCfg<2, 2>::SMEM;
    default: return BatchCfg<3, 2>::SMEM;
  }
}

int launch_mixed_batch(int variant, const BatchArgs& a, int ctas_per_sm, int num_sms, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  switch (variant) {
    case 0: return launch_variant<4, 8>(a, ctas_per_sm, num_sms, st, nullptr);
    case 1: return launch_variant<4, 4>(a, ctas_per_sm, num_sms, st, nullptr);
    case 2: return launch_variant<2, 4>(a, ctas_per_sm, num_sms, st, nullptr);
    case 3: return launch_variant<2, 2>(a, ctas_per_sm, num_sms, st, nullptr);
    default: return launch_variant<3, 2, 3>(a, ctas_per_sm, num_sms, st, nullptr);
  }
}

}  // namespace cmfe
