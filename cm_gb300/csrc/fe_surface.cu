// libcm_fe: surface-pressure follower load on boundary faces (sm_103a).
// One warp per boundary element of one element colour; the kernel runs after
// the volume kernel of the same colour, so every CSR slot it touches already
// holds a value and it only adds (red.global.add).  Device code in
// fe_surface_impl.cuh.
#include "fe_surface_impl.cuh"

using cmfe::KParams;

namespace {

constexpr int WARPS = 4;

template <int N1>
__global__ void __launch_bounds__(32 * WARPS) fe_surface_kernel(KParams P, const int32_t* belems,
                                                                const uint8_t* bmask, int nb, int mode,
                                                                int want_jac, cmfe::StageOut so) {
  __shared__ SurfWarpSmem ws[WARPS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x * WARPS + warp; it < nb; it += gridDim.x * WARPS) {
    const int e = belems[it];
    if (mode == 1 && (e < P.first_elem || e >= P.first_elem + P.count)) continue;
    surface_element<N1>(P, e, bmask, mode, want_jac, ws[warp], lane, &so);
  }
}

}  // namespace

namespace cmfe {

int launch_surface(const HostSetup& s, const KParams& kp, const int32_t* belems, const uint8_t* bmask, int nb,
                   int mode, int want_jac, int num_sms, void* stream, const StageOut& so) {
  if (nb <= 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  int grid = (nb + WARPS - 1) / WARPS;
  grid = grid < 4 * num_sms ? grid : 4 * num_sms;
  if (s.n1 == 2)
    fe_surface_kernel<2><<<grid, 32 * WARPS, 0, st>>>(kp, belems, bmask, nb, mode, want_jac, so);
  else
    fe_surface_kernel<3><<<grid, 32 * WARPS, 0, st>>>(kp, belems, bmask, nb, mode, want_jac, so);
  return (int)cudaGetLastError();
}

}  // namespace cmfe
