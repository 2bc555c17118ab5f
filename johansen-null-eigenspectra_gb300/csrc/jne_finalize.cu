// jne_finalize.cu -- the finalize kernels: one thread per run turns the run's
// moment record into its eigenvalues (jne_finalize_run.cuh; replaces
// johansen_statistics.rs:24-47).  Used by the FP64 path and by multi-model
// requests (one accumulation, one finalize per model); the mixed kernels
// finalize their own runs.
#include "jne_finalize_run.cuh"

namespace {

constexpr int kFinThreads = 64;
using jne_fin::finalize_run;

__global__ void __launch_bounds__(kFinThreads) k_finalize(const jne_finalize_args f) {
  const int run = blockIdx.x * kFinThreads + threadIdx.x;
  if (run < f.n_runs) finalize_run(f, run);
}

}  // namespace

cudaError_t jne_launch_finalize(const jne_finalize_args& f, int sms, cudaStream_t st) {
  (void)sms;
  if (f.n_runs <= 0) return cudaSuccess;
  const int grid = (f.n_runs + kFinThreads - 1) / kFinThreads;
  k_finalize<<<grid, kFinThreads, 0, st>>>(f);
  return cudaGetLastError();
}
