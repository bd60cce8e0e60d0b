// libcm_fe: batched mixed-precision assembly of many equations sets in one
// persistent launch (sm_103a).
//
// The members of a batch are independent meshes (any mix of trilinear and
// triquadratic elements, element-based or nodal pressure).  One cooperative
// launch walks the element colours in order; for colour c every CTA walks the
// member slots (ordered by element type, so a CTA reloads its constant tables
// rarely) and takes every gridDim.x-th work unit (block_groups element
// groups) of the colour-c elements of all members, then all CTAs meet at a
// grid barrier before colour c + 1.  Within a member the colour order is the
// one of the single-set path, so every CSR slot receives its contributions in
// the same order: repeated launches are bit-identical, and the result agrees
// with one fe_jacobian_evaluate_mixed call per member to the rounding of the
// separately compiled device code.
//
// The member parameters are read from a constant-memory table indexed by the
// slot, a loop counter the compiler knows to be warp-uniform: pointers,
// sizes and the material law stay uniform operands as in the single-set
// kernel, where they are launch parameters.  The table belongs to the module,
// so the host serialises batched launches of all batches on a device.
//
// Members with a surface-pressure load get, after the volume work of each
// colour and a grid barrier, that colour's boundary elements (one warp each)
// and a second barrier, the order of the single-set path.
//
// The grid barrier spins with a bounded number of polls: if it ever gives up
// (which only a non-co-resident grid could cause, and the cooperative launch
// rules that out), it sets bit 1 of the batch status word and the host call
// reports an error instead of hanging.
#include "fe_batch_impl.cuh"

namespace {

// Launch variants the autotuner chooses from: elements per group for
// triquadratic / trilinear members, and the CTAs per SM the register budget
// is compiled for (3 = 80 registers, some spills; 2 = 128).
struct Variant {
  int egq, egl, minb;
};
constexpr Variant VARIANTS[] = {{4, 8, 2}, {4, 4, 2}, {2, 4, 2}, {2, 2, 2}, {3, 2, 3}};
constexpr int NVARIANTS = 5;

template <int EGQ, int EGL, int MINB = 2>
int launch_variant(const BatchMember* members, int n, const BatchArgs& a, unsigned mask, int ctas_per_sm,
                   int num_sms, cudaStream_t st) {
  return launch_kernel<EGQ, EGL, MINB, 15>(members, n, a, mask, ctas_per_sm, num_sms, st);
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

int batch_smem(int v, unsigned mask) {
  switch (v) {
    case 0: return BatchCfg<4, 8>::smem_for(mask);
    case 1: return BatchCfg<4, 4>::smem_for(mask);
    case 2: return BatchCfg<2, 4>::smem_for(mask);
    case 3: return BatchCfg<2, 2>::smem_for(mask);
    default: return BatchCfg<3, 2>::smem_for(mask);
  }
}

int launch_mixed_batch(int variant, unsigned mask, const BatchMember* members, int n, const BatchArgs& a,
                       int ctas_per_sm, int num_sms, void* stream) {
  if (n < 1 || n > BATCH_MAX_MEMBERS) return (int)cudaErrorInvalidValue;
  // one element type: the kernel compiled for that type alone (a smaller
  // body, register-allocated for that type only)
  for (int t = 0; t < 4; ++t)
    if ((mask & 15u) == (1u << t)) return launch_batch_typed(variant, t, mask, members, n, a, ctas_per_sm, num_sms, stream);
  cudaStream_t st = (cudaStream_t)stream;
  switch (variant) {
    case 0: return launch_variant<4, 8>(members, n, a, mask, ctas_per_sm, num_sms, st);
    case 1: return launch_variant<4, 4>(members, n, a, mask, ctas_per_sm, num_sms, st);
    case 2: return launch_variant<2, 4>(members, n, a, mask, ctas_per_sm, num_sms, st);
    case 3: return launch_variant<2, 2>(members, n, a, mask, ctas_per_sm, num_sms, st);
    default: return launch_variant<3, 2, 3>(members, n, a, mask, ctas_per_sm, num_sms, st);
  }
}

}  // namespace cmfe
