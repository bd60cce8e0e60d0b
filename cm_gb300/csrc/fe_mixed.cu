// libcm_fe: mixed-precision element assembly (sm_103a), one launch per
// element colour of one equations set.  The device code is in
// fe_mixed_impl.cuh.
#include "fe_mixed_impl.cuh"
#include "fe_gather_impl.cuh"
#include "fe_surface_impl.cuh"

#include <atomic>


namespace {

template <int N1, int PM, int SPLIT, class H>
__global__ void __launch_bounds__(256, MixCfg<N1, PM>::MINB) fe_mixed_kernel(KParams P) {
  using C = MixCfg<N1, PM>;
  extern __shared__ __align__(16) unsigned char sm[];
  mix_tables<N1, PM, C::EG, H>(P, sm);
  const int ngroups = (P.count + C::EG - 1) / C::EG;
  const bool p4_first = (blockIdx.x / P.wave) & 1;
  for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) mix_group<N1, PM, C::EG, SPLIT, H>(P, P.elems, P.count, grp, p4_first, sm);
}

// The same element code over all elements in element order, each element's
// entries stored into its staging records instead of the CSR arrays (no
// colour order is needed: elements write disjoint records).
template <int N1, int PM, int SPLIT, class H>
__global__ void __launch_bounds__(256, MixCfg<N1, PM>::MINB) fe_mixed_staged_kernel(KParams P, cmfe::StageOut so) {
  using C = MixCfg<N1, PM>;
  extern __shared__ __align__(16) unsigned char sm[];
  mix_tables<N1, PM, C::EG, H>(P, sm);
  const int ngroups = (P.count + C::EG - 1) / C::EG;
  const bool p4_first = (blockIdx.x / P.wave) & 1;
  for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x)
    mix_group<N1, PM, C::EG, SPLIT, H, 1>(P, nullptr, P.count, grp, p4_first, sm, &so);
}

// Staged assembly in one launch: CTAs take element groups in element order
// from a global counter, store each group's records (and the surface-pressure
// faces of its boundary elements), then count, for every row node of the
// group, how many of the elements around the node are done.  The CTA whose
// count completes a node gathers that node's rows right away, while the
// records of the elements around it are still in L2 -- no CTA ever waits for
// another.  Publication follows the release/acquire pattern: every thread
// fences its record stores before the counting, and a completing count is
// followed by a fence before the records are read (through L2, not L1).
template <int N1, int PM, int SPLIT, class H>
__global__ void __launch_bounds__(256, MixCfg<N1, PM>::MINB)
    fe_mixed_fused_kernel(KParams P, cmfe::StageOut so, cmfe::FusedArgs F) {
  using C = MixCfg<N1, PM>;
  constexpr int NPE = C::NPE, NPP = C::NPP, NR = C::NR, EG = C::EG;
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ int s_grp, s_nready;
  mix_tables<N1, PM, EG, H>(P, sm);
  const int ngroups = min((P.count + EG - 1) / EG, F.g1);
  const bool p4_first = (blockIdx.x / P.wave) & 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int* s_node = reinterpret_cast<const int*>(sm + C::O_NODE);
  int* ready = reinterpret_cast<int*>(sm + C::O_READY);
  unsigned char* scratch = sm + C::O_SCRATCH;
  for (;;) {
    if (tid == 0) s_grp = F.g0 + atomicAdd(F.work, 1);
    __syncthreads();
    const int grp = s_grp;
    if (grp >= ngroups) break;
    mix_group<N1, PM, EG, SPLIT, H, 1>(P, nullptr, P.count, grp, p4_first, sm, &so);
    const int nvalid = min(EG, P.count - grp * EG);
    __syncthreads();  // the group's records are complete within the CTA; the scratch is free
    if (F.bmask) {
      SurfWarpSmem* ws = reinterpret_cast<SurfWarpSmem*>(scratch);
      for (int el = warp; el < nvalid; el += C::THREADS / 32) {
        const int e = grp * EG + el;
        if (F.bmask[e]) surface_element<N1>(P, e, F.bmask, 2, 1, ws[warp], lane, &so);
      }
    }
    __threadfence();  // release: this thread's record stores before the counts below
    if (tid == 0) s_nready = 0;
    __syncthreads();
    for (int i = tid; i < nvalid * NR; i += C::THREADS) {
      __threadfence();  // cumulative release, after the barrier, for the stores of the whole CTA
      const int el = i / NR, r = i % NR;
      const int node = s_node[el * (NR + 1) + r];
      const bool un = r < NPE;
      const int id = un ? node : P.nu + node;
      const int target = un ? F.u_inc_ptr[node + 1] - F.u_inc_ptr[node] : F.p_inc_ptr[node + 1] - F.p_inc_ptr[node];
      if (atomicAdd(F.node_done + id, 1) + 1 == target) {
        __threadfence();  // acquire: the records of every element around the node
        ready[atomicAdd(&s_nready, 1)] = id;
      }
    }
    __syncthreads();
    const int nready = s_nready;
    if (warp < F.gwarps) {
      unsigned char* mine = scratch + (size_t)warp * F.gbytes;
      for (int j = warp; j < nready; j += F.gwarps) {
        const int id = ready[j];
        if (id < P.nu)
          gather_unode<NPE, NPP, true>(P, so, F.u_inc_ptr, F.u_inc, id, mine, lane);
        else
          gather_pnode<NPE, NPP, true>(P, so, F.p_inc_ptr, F.p_inc, id - P.nu, mine, lane);
      }
    }
    __syncthreads();  // the next group reuses the scratch and the ready list
  }
}

// Resident blocks per SM of the fused kernel (its shared-memory attribute set
// once per device first); 0 on error, with the error in *err.
template <int N1, int PM, int SPLIT, class H>
int fused_per_sm(cudaError_t* err) {
  using C = MixCfg<N1, PM>;
  static std::atomic<bool> attr[64];
  auto kern = fe_mixed_fused_kernel<N1, PM, SPLIT, H>;
  int dev = 0;
  *err = cudaGetDevice(&dev);
  if (*err != cudaSuccess) return 0;
  if (dev < 0 || dev >= 64 || !attr[dev].load()) {
    *err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (*err != cudaSuccess) return 0;
    if (dev >= 0 && dev < 64) attr[dev].store(true);
  }
  int per_sm = 0;
  *err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::THREADS, C::SMEM);
  if (*err != cudaSuccess) return 0;
  return per_sm < 1 ? 1 : per_sm;
}

template <int N1, int PM, int SPLIT, class H>
int launch_fused_t(const KParams& kp, const cmfe::StageOut& so, cmfe::FusedArgs fa, int gather_bytes, int num_sms,
                   cudaStream_t st) {
  using C = MixCfg<N1, PM>;
  auto kern = fe_mixed_fused_kernel<N1, PM, SPLIT, H>;
  const int avail = C::O_READY - C::O_SCRATCH;
  fa.gbytes = gather_bytes;
  fa.gwarps = gather_bytes > 0 ? avail / gather_bytes : 0;
  if (fa.gwarps > C::THREADS / 32) fa.gwarps = C::THREADS / 32;
  if (fa.gwarps < 1) return (int)cudaErrorInvalidConfiguration;
  cudaError_t e;
  const int per_sm = fused_per_sm<N1, PM, SPLIT, H>(&e);
  if (!per_sm) return (int)e;
  const int all = (kp.count + C::EG - 1) / C::EG;
  if (fa.g1 > all) fa.g1 = all;
  if (fa.g0 < 0 || fa.g0 >= fa.g1) return (int)cudaSuccess;  // no groups in this launch
  const int groups = fa.g1 - fa.g0;
  int grid = per_sm * num_sms;
  grid = grid < groups ? grid : groups;
  grid = grid < 1 ? 1 : grid;
  KParams k = kp;
  k.wave = num_sms > 0 ? num_sms : 1;
  kern<<<grid, C::THREADS, C::SMEM, st>>>(k, so, fa);
  return (int)cudaGetLastError();
}

template <class H>
int launch_fused_h(const HostSetup& s, const KParams& kp, const cmfe::StageOut& so, const cmfe::FusedArgs& fa,
                   int num_sms, cudaStream_t st) {
  if (s.n1 == 2 && s.pmode == 0) return launch_fused_t<2, 0, 3, H>(kp, so, fa, s.gather_bytes, num_sms, st);
  if (s.n1 == 2 && s.pmode == 1) return launch_fused_t<2, 1, 3, H>(kp, so, fa, s.gather_bytes, num_sms, st);
  if (s.n1 == 3 && s.pmode == 0) return launch_fused_t<3, 0, 3, H>(kp, so, fa, s.gather_bytes, num_sms, st);
  return launch_fused_t<3, 1, 3, H>(kp, so, fa, s.gather_bytes, num_sms, st);
}

template <int N1, int PM, int SPLIT, class H, bool STAGED = false>
int launch_t(const KParams& kp, int num_sms, cudaStream_t st, const cmfe::StageOut& so = cmfe::StageOut{}) {
  using C = MixCfg<N1, PM>;
  // the attribute belongs to the device that is current: set once per device
  static std::atomic<bool> attr[64];
  const void* kern = STAGED ? (const void*)fe_mixed_staged_kernel<N1, PM, SPLIT, H>
                            : (const void*)fe_mixed_kernel<N1, PM, SPLIT, H>;
  int dev = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 != cudaSuccess) return (int)e0;
  if (dev < 0 || dev >= 64 || !attr[dev].load()) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (e != cudaSuccess) return (int)e;
    if (dev >= 0 && dev < 64) attr[dev].store(true);
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::THREADS, C::SMEM);
  if (e != cudaSuccess) return (int)e;
  per_sm = per_sm < 1 ? 1 : per_sm;
  const int groups = (kp.count + C::EG - 1) / C::EG;
  int grid = per_sm * num_sms;
  grid = grid < groups ? grid : groups;
  grid = grid < 1 ? 1 : grid;
  KParams k = kp;
  k.wave = num_sms > 0 ? num_sms : 1;
  if constexpr (STAGED)
    fe_mixed_staged_kernel<N1, PM, SPLIT, H><<<grid, C::THREADS, C::SMEM, st>>>(k, so);
  else
    fe_mixed_kernel<N1, PM, SPLIT, H><<<grid, C::THREADS, C::SMEM, st>>>(k);
  return (int)cudaGetLastError();
}

template <class H, bool STAGED = false>
int launch_h(const HostSetup& s, const KParams& kp, int num_sms, cudaStream_t st,
             const cmfe::StageOut& so = cmfe::StageOut{}) {
  if (s.n1 == 2 && s.pmode == 0) return launch_t<2, 0, 3, H, STAGED>(kp, num_sms, st, so);
  if (s.n1 == 2 && s.pmode == 1) return launch_t<2, 1, 3, H, STAGED>(kp, num_sms, st, so);
  if (s.n1 == 3 && s.pmode == 0) return launch_t<3, 0, 3, H, STAGED>(kp, num_sms, st, so);
  return launch_t<3, 1, 3, H, STAGED>(kp, num_sms, st, so);
}

}  // namespace

namespace cmfe {

int launch_mixed(const HostSetup& s, const KParams& kp, int num_sms, void* stream, bool double_float) {
  cudaStream_t st = (cudaStream_t)stream;
  if (kp.count <= 0) return 0;
  return double_float ? launch_h<dd>(s, kp, num_sms, st) : launch_h<double>(s, kp, num_sms, st);
}

int fused_wave(const HostSetup& s, int num_sms, bool double_float) {
  cudaError_t e;
  int per_sm;
  if (double_float)
    per_sm = s.n1 == 2 ? (s.pmode ? fused_per_sm<2, 1, 3, dd>(&e) : fused_per_sm<2, 0, 3, dd>(&e))
                       : (s.pmode ? fused_per_sm<3, 1, 3, dd>(&e) : fused_per_sm<3, 0, 3, dd>(&e));
  else
    per_sm = s.n1 == 2 ? (s.pmode ? fused_per_sm<2, 1, 3, double>(&e) : fused_per_sm<2, 0, 3, double>(&e))
                       : (s.pmode ? fused_per_sm<3, 1, 3, double>(&e) : fused_per_sm<3, 0, 3, double>(&e));
  if (!per_sm) return -(int)e;
  return per_sm * (num_sms > 0 ? num_sms : 1);
}

int fused_group_size(const HostSetup& s) {
  if (s.n1 == 2) return s.pmode ? MixCfg<2, 1>::EG : MixCfg<2, 0>::EG;
  return s.pmode ? MixCfg<3, 1>::EG : MixCfg<3, 0>::EG;
}

int fused_fits(const HostSetup& s) {
  int avail;
  if (s.n1 == 2)
    avail = s.pmode ? MixCfg<2, 1>::O_READY - MixCfg<2, 1>::O_SCRATCH : MixCfg<2, 0>::O_READY - MixCfg<2, 0>::O_SCRATCH;
  else
    avail = s.pmode ? MixCfg<3, 1>::O_READY - MixCfg<3, 1>::O_SCRATCH : MixCfg<3, 0>::O_READY - MixCfg<3, 0>::O_SCRATCH;
  return s.gather_bytes > 0 && avail / s.gather_bytes >= 1 && (int)sizeof(SurfWarpSmem) * 8 <= avail;
}

int launch_mixed_fused(const HostSetup& s, const KParams& kp, const StageOut& so, const FusedArgs& fa, int num_sms,
                       void* stream, bool double_float) {
  cudaStream_t st = (cudaStream_t)stream;
  if (kp.count <= 0) return 0;
  return double_float ? launch_fused_h<dd>(s, kp, so, fa, num_sms, st)
                      : launch_fused_h<double>(s, kp, so, fa, num_sms, st);
}

int launch_mixed_staged(const HostSetup& s, const KParams& kp, const StageOut& so, int num_sms, void* stream,
                        bool double_float) {
  cudaStream_t st = (cudaStream_t)stream;
  if (kp.count <= 0) return 0;
  return double_float ? launch_h<dd, true>(s, kp, num_sms, st, so) : launch_h<double, true>(s, kp, num_sms, st, so);
}

}  // namespace cmfe
