// jne_accum_mixed.cu -- the mixed-precision accumulation kernels budgeted for 4
// blocks per SM (128 registers a thread), the ragged batch kernel and the
// launch dispatch.  The device code is in jne_accum_mixed.cuh; the
// 6-blocks-per-SM variants are compiled in jne_accum_mixed_b6.cu and the
// explicit-increment ones in jne_accum_mixed_ext.cu (translation units built
// in parallel).
#include "jne_accum_mixed.cuh"

namespace {

// A ragged batch of requests (any dims, step counts and sizes) in one
// persistent launch: each warp takes the next unit of the flattened batch from
// a global counter, so long and short requests share the GPU without tails.
// reqs[r].first counts units.
__device__ __forceinline__ int request_of(const jne_ragged_req* __restrict__ reqs, int n_req, long long item) {
  int lo = 0, hi = n_req - 1;  // request r with reqs[r].first <= item < reqs[r + 1].first
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (reqs[mid].first <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// batch_done (ceil(total / 32) zeroed counts): every item is also finalized
// in the launch, batches of 32 consecutive items spanning requests as needed.
__global__ void __launch_bounds__(kMixWarps * JNE_WARP, 4)
    k_accum_mixed_ragged(const jne_ragged_req* __restrict__ reqs, int n_req, long long total,
                         unsigned long long* __restrict__ counter, unsigned int* __restrict__ batch_done) {
  __shared__ WarpSmem sm_all[kMixWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  for (;;) {
    unsigned long long item = 0;
    if (lane == 0) item = atomicAdd(counter, 1ull);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= (unsigned long long)total) break;
    const int lo = request_of(reqs, n_req, (long long)item);
    const jne_accum_args& a = reqs[lo].acc;
    const int unit = (int)(item - (unsigned long long)reqs[lo].first);
    const jne_round_keys rk = jne_make_round_keys(a.key0, a.key1);
    switch (a.dim) {
      case 1: accum_unit<1, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 2: accum_unit<2, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 3: accum_unit<3, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 4: accum_unit<4, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 5: accum_unit<5, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 6: accum_unit<6, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 7: accum_unit<7, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 8: accum_unit<8, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 9: accum_unit<9, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 10: accum_unit<10, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      case 11: accum_unit<11, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
      default: accum_unit<12, false, false, true>(a, unit, sm_all[wib], rk, lane); break;
    }
    if (batch_done) {
      const long long first = batch_complete(batch_done, (long long)item, total, lane);
      if (first >= 0 && first + lane < total) {
        const int r = request_of(reqs, n_req, first + lane);
        finalize_unit(reqs[r].fin, first + lane - reqs[r].first, true);
      }
      __syncwarp();
    }
  }
}

}  // namespace

cudaError_t jne_launch_accum_mixed_ragged(const jne_ragged_req* reqs, int n_req, long long total,
                                         unsigned long long* counter, unsigned int* batch_done, int sms,
                                         cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  const int threads = kMixWarps * JNE_WARP;
  k_accum_mixed_ragged<<<resident_grid(k_accum_mixed_ragged, threads, 0, sms, total, kMixWarps), threads, 0, st>>>(
      reqs, n_req, total, counter, batch_done);
  return cudaGetLastError();
}

cudaError_t jne_launch_accum_mixed(const jne_accum_args& a, const jne_finalize_args* fin, int sms, cudaStream_t st) {
  if (a.blocks_per_sm != 0 && a.blocks_per_sm != 4 && a.blocks_per_sm != 6) return cudaErrorInvalidValue;
  if (a.ext) return jne_launch_accum_mixed_ext(a, fin, sms, st);
  if (a.blocks_per_sm == 6) return jne_launch_accum_mixed_b6(a, fin, sms, st);
  return launch_mixed<4, false>(a, fin, sms, st);
}
