// libcm_fe: batched mixed-precision assembly, kernels for batches whose
// members all have one element type (sm_103a).  The kernel body holds that
// type's element code only, so it is smaller and register-allocated for that
// type alone; the launch variants keep the elements per group and CTAs per
// SM of the mixed-type kernels (fe_batch.cu), the other type's group size
// being irrelevant.
#include "fe_batch_impl.cuh"

namespace {

// Triquadratic types (2, 3): elements per group and CTAs per SM of variant v.
template <int TM>
int launch_quadratic(int v, const BatchMember* members, int n, const BatchArgs& a, unsigned mask, int cps, int sms,
                     cudaStream_t st) {
  switch (v) {
    case 0:
    case 1: return launch_kernel<4, 2, 2, TM>(members, n, a, mask, cps, sms, st);
    case 2:
    case 3: return launch_kernel<2, 2, 2, TM>(members, n, a, mask, cps, sms, st);
    default: return launch_kernel<3, 2, 3, TM>(members, n, a, mask, cps, sms, st);
  }
}

// Trilinear types (0, 1).
template <int TM>
int launch_linear(int v, const BatchMember* members, int n, const BatchArgs& a, unsigned mask, int cps, int sms,
                  cudaStream_t st) {
  switch (v) {
    case 0: return launch_kernel<2, 8, 2, TM>(members, n, a, mask, cps, sms, st);
    case 1:
    case 2: return launch_kernel<2, 4, 2, TM>(members, n, a, mask, cps, sms, st);
    case 3: return launch_kernel<2, 2, 2, TM>(members, n, a, mask, cps, sms, st);
    default: return launch_kernel<2, 2, 3, TM>(members, n, a, mask, cps, sms, st);
  }
}

}  // namespace

namespace cmfe {

int launch_batch_typed(int variant, int type, unsigned mask, const BatchMember* members, int n, const BatchArgs& a,
                       int ctas_per_sm, int num_sms, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  switch (type) {
    case 0: return launch_linear<1>(variant, members, n, a, mask, ctas_per_sm, num_sms, st);
    case 1: return launch_linear<2>(variant, members, n, a, mask, ctas_per_sm, num_sms, st);
    case 2: return launch_quadratic<4>(variant, members, n, a, mask, ctas_per_sm, num_sms, st);
    default: return launch_quadratic<8>(variant, members, n, a, mask, ctas_per_sm, num_sms, st);
  }
}

}  // namespace cmfe
