// jne_kernels.h -- host-side launch wrappers of the device kernels.
#pragma once
#include <cuda_runtime.h>
#include "jne_common.cuh"

// Deterministic time sums Y[p] = sum_{i=0}^{T-1} ((i+1)/T)^p, p = 0..4.
struct jne_time_sums {
  double Y[5];
};

// The mixed kernels can pack two runs into one warp ("unit") for dims up to
// this: a request of n runs is then ceil(n / 2) units, else n.
#define JNE_PACK_MAX_DIM 4
__host__ __device__ __forceinline__ long long jne_units(int dim, long long n_runs, bool pack = true) {
  return pack && dim <= JNE_PACK_MAX_DIM ? (n_runs + 1) / 2 : n_runs;
}

// Argument block of the finalize kernel.
struct jne_finalize_args {
  int model, dim, steps, n_runs;
  double zscale;            // B = zscale * W, dB = zscale * z
  jne_time_sums ts;
  const double* mom;        // moment records (SoA)
  long long mom_ld;
  double* out;              // n_runs x k eigenvalues, descending
  unsigned int* status;
};

// One request of a ragged batch, as the device sees it: the accumulation and
// finalize argument blocks and the request's first index in the flattened run
// space of the batch.
struct jne_ragged_req {
  jne_accum_args acc;
  jne_finalize_args fin;
  long long first;
};

// batch_done (may be null): ceil(total / 32) zeroed counts; the launch then
// also finalizes every item
cudaError_t jne_launch_accum_mixed_ragged(const jne_ragged_req* reqs, int n_req, long long total,
                                         unsigned long long* counter, unsigned int* batch_done, int sms,
                                         cudaStream_t st);
cudaError_t jne_launch_accum_f64(const jne_accum_args& a, const int4* ent, int nent, int sms, cudaStream_t st);
int jne_build_f64_entries(int model, int d, int4* out, int cap);
// fin (may be null) finalizes the same request's runs inside the launch.
// a.blocks_per_sm (4, or 6 for the kernels budgeted to 80 registers) and
// a.pack (< 0: one run per warp at every dim) select the kernel variant.
cudaError_t jne_launch_accum_mixed(const jne_accum_args& a, const jne_finalize_args* fin, int sms, cudaStream_t st);
// the 6-blocks-per-SM variants and the explicit-increment ones (their own translation units)
cudaError_t jne_launch_accum_mixed_b6(const jne_accum_args& a, const jne_finalize_args* fin, int sms, cudaStream_t st);
cudaError_t jne_launch_accum_mixed_ext(const jne_accum_args& a, const jne_finalize_args* fin, int sms,
                                       cudaStream_t st);
cudaError_t jne_launch_finalize(const jne_finalize_args& f, int sms, cudaStream_t st);
// The .dat records of n results of consecutive seeds (jne_pack.cu): out is
// 16-byte aligned and holds jne_records_bytes(seed_first, n, k) bytes.
cudaError_t jne_launch_pack_records(const double* eigs, unsigned char* out, uint32_t seed_first, long long n, int k,
                                    int sms, cudaStream_t st);
cudaError_t jne_launch_export(int dim, int steps, int n_runs, uint32_t seed_first, uint32_t key0, uint32_t key1,
                              double scale, double* out, uint32_t* words, cudaStream_t st);
