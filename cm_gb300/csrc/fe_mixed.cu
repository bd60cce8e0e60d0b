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

template <int N1, int PM, int SPLIT, class H>
int launch_t(const KParams& kp, int num_sms, cudaStream_t st) {
  using C = MixCfg<N1, PM>;
  // the attribute belongs to the device that is current: set once per device
  static std::atomic<bool> attr[64];
  auto kern = fe_mixed_kernel<N1, PM, SPLIT, H>;
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
  kern<<<grid, C::THREADS, C::SMEM, st>>>(k);
  return (int)cudaGetLastError();
}

template <class H>
int launch_h(const HostSetup& s, const KParams& kp, int num_sms, cudaStream_t st) {
  if (s.n1 == 2 && s.pmode == 0) return launch_t<2, 0, 3, H>(kp, num_sms, st);
  if (s.n1 == 2 && s.pmode == 1) return launch_t<2, 1, 3, H>(kp, num_sms, st);
  if (s.n1 == 3 && s.pmode == 0) return launch_t<3, 0, 3, H>(kp, num_sms, st);
  return launch_t<3, 1, 3, H>(kp, num_sms, st);
}

}  // namespace

namespace cmfe {

int launch_mixed(const HostSetup& s, const KParams& kp, int num_sms, void* stream, bool double_float) {
  cudaStream_t st = (cudaStream_t)stream;
  if (kp.count <= 0) return 0;
  return double_float ? launch_h<dd>(s, kp, num_sms, st) : launch_h<double>(s, kp, num_sms, st);
}

}  // namespace cmfe
