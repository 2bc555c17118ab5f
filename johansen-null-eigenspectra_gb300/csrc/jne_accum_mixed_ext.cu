// jne_accum_mixed_ext.cu -- the mixed-precision accumulation kernels on
// explicit increments (jne_eigs_from_increments: the TF32 split, whose range
// suits unbounded inputs), 4 blocks per SM; device code in jne_accum_mixed.cuh.
#include "jne_accum_mixed.cuh"

cudaError_t jne_launch_accum_mixed_ext(const jne_accum_args& a, const jne_finalize_args* fin, int sms,
                                       cudaStream_t st) {
  return launch_mixed<4, true>(a, fin, sms, st);
}
