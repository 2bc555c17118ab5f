// jne_export.cu -- writes out the increments (and raw Philox words) the
// accumulation kernels draw, so the per-run result of the in-kernel random
// path can be checked against an independent CPU evaluation of the same path.
// Uses the very device functions the accumulation kernels call.
#include "jne_kernels.h"

namespace {

__global__ void k_export(int dim, int steps, int n_runs, uint32_t seed_first, uint32_t key0, uint32_t key1,
                         double scale, double* __restrict__ out, uint32_t* __restrict__ words) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n_runs * steps) return;
  const int run = (int)(idx / steps), i = (int)(idx % steps);
  const int nq = (dim + 3) >> 2;
  const uint32_t seed = seed_first + (uint32_t)run;
  const jne_round_keys rk = jne_make_round_keys(key0, key1);
  for (int j = 0; j < nq; j++) {
    if (words) {
      uint32_t w[4];
      jne_philox4x32_10((uint32_t)(i + 1), (uint32_t)j, seed, 0u, rk, w);
      uint32_t* dst = words + ((size_t)idx * nq + j) * 4;
      dst[0] = w[0]; dst[1] = w[1]; dst[2] = w[2]; dst[3] = w[3];
    }
    if (out) {
      float z[4];
      jne_normal_quad((uint32_t)(i + 1), (uint32_t)j, seed, rk, z);
      for (int e = 0; e < 4; e++) {
        const int f = 4 * j + e;
        if (f < dim) out[(size_t)idx * dim + f] = (double)z[e] * scale;
      }
    }
  }
}

}  // namespace

cudaError_t jne_launch_export(int dim, int steps, int n_runs, uint32_t seed_first, uint32_t key0, uint32_t key1,
                              double scale, double* out, uint32_t* words, cudaStream_t st) {
  const long long n = (long long)n_runs * steps;
  if (n <= 0) return cudaSuccess;
  const int threads = 256;
  const long long blocks = (n + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  k_export<<<(unsigned)blocks, threads, 0, st>>>(dim, steps, n_runs, seed_first, key0, key1, scale, out, words);
  return cudaGetLastError();
}
