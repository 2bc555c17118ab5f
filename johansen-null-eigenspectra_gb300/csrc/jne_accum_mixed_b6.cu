// jne_accum_mixed_b6.cu -- the mixed-precision accumulation kernels budgeted
// for 6 blocks per SM (80 registers a thread): a speed variant the autotuner
// may pick per (dim, class of steps); the arithmetic is that of the 4-block
// kernels (jne_accum_mixed.cuh).
#include "jne_accum_mixed.cuh"

cudaError_t jne_launch_accum_mixed_b6(const jne_accum_args& a, const jne_finalize_args* fin, int sms, cudaStream_t st) {
  return launch_mixed<6, false>(a, fin, sms, st);
}
