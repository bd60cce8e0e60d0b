// libcm_fe: device code of the batched mixed-precision assembly (the
// persistent kernel, its grid barrier and the member constant table),
// included by the translation units that instantiate it: fe_batch.cu (kernels
// for batches of mixed element types) and fe_batch_typed.cu (one element
// type).  Each translation unit is its own module with its own constant
// table, written by the launch helper of that unit before its kernel runs.
#pragma once
#include "fe_mixed_impl.cuh"
#include "fe_surface_impl.cuh"

#include <cooperative_groups.h>

#include <atomic>

namespace {

constexpr int BT_THREADS = 256;
constexpr int BT_WARPS = BT_THREADS / 32;
constexpr unsigned BARRIER_POLLS = 1u << 21;  // x at most 2 us sleep: a few seconds at most

using cmfe::BatchArgs;
using cmfe::BatchMember;

__constant__ BatchMember c_members[cmfe::BATCH_MAX_MEMBERS];

__device__ void grid_barrier(const BatchArgs& A) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = A.bar_gen;
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(A.bar_count, 1u);
    const unsigned limit = A.barrier_polls ? A.barrier_polls : BARRIER_POLLS;
    if (arrived == gridDim.x - 1 + A.barrier_extra) {
      atomicExch(A.bar_count, 0u);
      __threadfence();
      atomicAdd(A.bar_gen, 1u);
    } else {
      // exponential back-off: a waiting CTA polls the barrier word rarely,
      // so that it takes few issue slots and little L2 bandwidth from the
      // CTAs still working on the colour
      unsigned polls = 0, ns = 64;
      while (*gen == g) {
        if (++polls > limit) {
          atomicOr(A.status, 2u);
          break;
        }
        __nanosleep(ns);
        ns = ns < 2048 ? 2 * ns : 2048;
      }
    }
    __threadfence();
  }
  __syncthreads();
}

template <int EGQ, int EGL>
struct BatchCfg {
  static constexpr int s(int a, int b) { return a > b ? a : b; }
  static constexpr int SMEM = s(s(s(MixCfg<2, 0, EGL>::SMEM, MixCfg<2, 1, EGL>::SMEM),
                                  s(MixCfg<3, 0, EGQ>::SMEM, MixCfg<3, 1, EGQ>::SMEM)),
                                (int)(BT_WARPS * sizeof(SurfWarpSmem)));
  // The dynamic shared memory a launch needs: the work area of the element
  // types present (mask bit t = type t, bit 4 = surface loads), so that a
  // batch of one type gets the occupancy of that type alone.
  static int smem_for(unsigned mask) {
    const int sz[5] = {MixCfg<2, 0, EGL>::SMEM, MixCfg<2, 1, EGL>::SMEM, MixCfg<3, 0, EGQ>::SMEM,
                       MixCfg<3, 1, EGQ>::SMEM, (int)(BT_WARPS * sizeof(SurfWarpSmem))};
    int w = 0;
    for (int t = 0; t < 5; ++t)
      if (mask & (1u << t)) w = s(w, sz[t]);
    return w;
  }
};

template <int EGQ, int EGL, int TM, class H>
__device__ __forceinline__ void load_tables(int type, const KParams& P, unsigned char* w) {
  switch (type) {
    case 0: if constexpr (TM & 1) mix_tables<2, 0, EGL, H>(P, w); break;
    case 1: if constexpr (TM & 2) mix_tables<2, 1, EGL, H>(P, w); break;
    case 2: if constexpr (TM & 4) mix_tables<3, 0, EGQ, H>(P, w); break;
    default: if constexpr (TM & 8) mix_tables<3, 1, EGQ, H>(P, w); break;
  }
}

// This CTA's work units of one member in the current colour: units u = j,
// j + gridDim.x, ... of nunits, unit u = element groups [u * bg, u * bg + bg).
template <int N1, int PM, int EG, class H>
__device__ __forceinline__ void member_units(const KParams& P, const int32_t* elems, int count, int j, int nunits,
                                             int bg, bool p4_first, unsigned char* w) {
  const int ng = (count + EG - 1) / EG;
  for (int u = j; u < nunits; u += gridDim.x) {
    const int g1 = min(ng, (u + 1) * bg);
    for (int g = u * bg; g < g1; ++g) mix_group<N1, PM, EG, 3, H>(P, elems, count, g, p4_first, w);
  }
}

template <int EGQ, int EGL, int MINB, int TM, class H>
__global__ void __launch_bounds__(BT_THREADS, MINB) fe_mixed_batch_kernel(BatchArgs A) {
  extern __shared__ __align__(16) unsigned char sm[];
  int cur_type = -1;
  const bool p4_first = (blockIdx.x / A.wave) & 1;
  const int stride = A.ncolours + 1;
  const int grid = gridDim.x;
  for (int c = 0; c < A.ncolours; ++c) {
    // ---- volume: colour-c element groups of every member
    int base = 0;  // work units of this colour in the slots before s
    for (int s = 0; s < A.nmembers; ++s) {
      const int t = c_members[s].type;
      const int eg = t >= 2 ? EGQ : EGL;
      const int32_t* off = A.offsets + (size_t)s * 2 * stride;
      const int e0 = __ldg(off + c), count = __ldg(off + c + 1) - e0;
      const int nunits = ((count + eg - 1) / eg + A.block_groups - 1) / A.block_groups;
      int j = (int)blockIdx.x - base % grid;  // first unit of this CTA: base + j = blockIdx.x (mod grid)
      if (j < 0) j += grid;
      if (j < nunits) {
        const KParams& P = c_members[s].kp;
        if (t != cur_type) {
          __syncthreads();  // every thread is done with the previous tables
          load_tables<EGQ, EGL, TM, H>(t, P, sm);
          cur_type = t;  // mix_group starts with a barrier, after which the tables are visible
        }
        const int32_t* elems = P.elems + e0;
        switch (t) {
          case 0:
            if constexpr (TM & 1) member_units<2, 0, EGL, H>(P, elems, count, j, nunits, A.block_groups, p4_first, sm);
            break;
          case 1:
            if constexpr (TM & 2) member_units<2, 1, EGL, H>(P, elems, count, j, nunits, A.block_groups, p4_first, sm);
            break;
          case 2:
            if constexpr (TM & 4) member_units<3, 0, EGQ, H>(P, elems, count, j, nunits, A.block_groups, p4_first, sm);
            break;
          default:
            if constexpr (TM & 8) member_units<3, 1, EGQ, H>(P, elems, count, j, nunits, A.block_groups, p4_first, sm);
            break;
        }
      }
      base += nunits;
    }
    grid_barrier(A);
    // ---- surface loads of colour c: one warp per boundary element, units of
    // BT_WARPS elements dealt to the CTAs like the volume units
    bool any = false;
    int sbase = 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    SurfWarpSmem* ws = reinterpret_cast<SurfWarpSmem*>(sm);
    for (int s = 0; s < A.nmembers; ++s) {
      if (!c_members[s].has_surface) continue;
      const int32_t* off = A.offsets + (size_t)s * 2 * stride + stride;
      const int b0 = __ldg(off + c), nb = __ldg(off + c + 1) - b0;
      if (nb == 0) continue;
      if (!any) {
        __syncthreads();  // the work area held the volume tables
        any = true;
        cur_type = -1;
      }
      const int nunits = (nb + BT_WARPS - 1) / BT_WARPS;
      int j = (int)blockIdx.x - sbase % grid;
      if (j < 0) j += grid;
      const KParams& P = c_members[s].kp;
      const int32_t* belems = c_members[s].belems + b0;
      const uint8_t* bmask = c_members[s].bmask;
      for (int u = j; u < nunits; u += grid) {
        const int i = u * BT_WARPS + warp;
        if (i < nb) {
          if (c_members[s].type >= 2) {
            if constexpr ((TM & 12) != 0) surface_element<3>(P, belems[i], bmask, 0, 1, ws[warp], lane);
          } else {
            if constexpr ((TM & 3) != 0) surface_element<2>(P, belems[i], bmask, 0, 1, ws[warp], lane);
          }
        }
      }
      sbase += nunits;
    }
    if (any) grid_barrier(A);  // grid-uniform: every CTA walks the same slots
  }
}

// Copies the member table into this module's constant table and launches
// fe_mixed_batch_kernel<EGQ, EGL, MINB, TM> cooperatively with the shared
// memory of the element types in mask; returns a cudaError_t.
template <int EGQ, int EGL, int MINB, int TM>
int launch_kernel(const BatchMember* members, int n, const BatchArgs& a, unsigned mask, int ctas_per_sm,
                  int num_sms, cudaStream_t st) {
  using B = BatchCfg<EGQ, EGL>;
  auto kern = fe_mixed_batch_kernel<EGQ, EGL, MINB, TM, double>;
  // the attribute belongs to the device that is current: set once per device
  static std::atomic<bool> attr[64];
  int dev = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 != cudaSuccess) return (int)e0;
  if (dev < 0 || dev >= 64 || !attr[dev].load()) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, B::SMEM);
    if (e != cudaSuccess) return (int)e;
    if (dev >= 0 && dev < 64) attr[dev].store(true);
  }
  const int smem = B::smem_for(mask);
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BT_THREADS, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  const int use = ctas_per_sm < per_sm ? ctas_per_sm : per_sm;
  const int grid = use * num_sms;
  e = cudaMemcpyToSymbolAsync(c_members, members, (size_t)n * sizeof(BatchMember), 0, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return (int)e;
  BatchArgs args = a;
  args.wave = num_sms;
  void* params[] = {&args};
  return (int)cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(BT_THREADS), params, smem, st);
}

}  // namespace
