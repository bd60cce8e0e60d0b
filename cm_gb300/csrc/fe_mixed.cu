// libcm_fe: mixed-precision element assembly (sm_103a), one launch per
// element colour of one equations set.  The device code is in
// fe_mixed_impl.cuh.
#include "fe_mixed_impl.cuh"

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

int launch_mixed_staged(const HostSetup& s, const KParams& kp, const StageOut& so, int num_sms, void* stream,
                        bool double_float) {
  cudaStream_t st = (cudaStream_t)stream;
  if (kp.count <= 0) return 0;
  return double_float ? launch_h<dd, true>(s, kp, num_sms, st, so) : launch_h<double, true>(s, kp, num_sms, st, so);
}

}  // namespace cmfe
