// jne_quantile.cu -- device quantile analyzer.
//
// Replaces calculate_percentiles (simulation_analyzers.rs:42-65): the Sum or
// Max aggregate of every run's eigenvalues (:26-39), then the percentiles with
// the interpolation rule of get_percentile_value (:4-18).  The reference sorts
// all aggregates; only the two order statistics around each rank p (n - 1) are
// needed, so they are found by a most-significant-digit radix select on
// order-preserving 64-bit keys: 8 passes of 8 bits over the n keys, each pass
// one histogram per wanted rank (restricted to the keys that share the rank's
// prefix found so far).  The selected keys are exact aggregate values, and the
// interpolation runs on the host with the reference's arithmetic, so the
// result is bit-identical to a full sort.
#include <cfloat>
#include <cstring>
#include "jne_context.h"

using namespace jne_detail;

namespace {

constexpr int kQThreads = 256;
constexpr int kGroup = 16;  // ranks per select group (16 x 256 histogram bins in shared memory)

// Order-preserving map of doubles to unsigned keys: negative values flip all
// bits, non-negative values set the sign bit.
__device__ __forceinline__ unsigned long long key_of(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

double value_of(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  double v;
  std::memcpy(&v, &b, sizeof v);
  return v;
}

// Sum (in index order, as the reference's iterator sum) or max (folded from
// f64::MIN) of each run's k eigenvalues; counts NaN aggregates.
__global__ void k_aggregate(const double* __restrict__ eigs, long long n, int k, int stat,
                            unsigned long long* __restrict__ keys, unsigned int* __restrict__ n_nan) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const double* e = eigs + r * k;
    double a = stat == 0 ? 0.0 : -DBL_MAX;
    for (int j = 0; j < k; j++) a = stat == 0 ? __dadd_rn(a, e[j]) : fmax(a, e[j]);
    if (a != a) atomicAdd(n_nan, 1u);
    keys[r] = key_of(a);
  }
}

// One radix pass for a group of ranks: hist[g][bin] counts the keys whose bits
// above `shift + 8` equal prefix[g], by their 8 bits at `shift`.  Lanes that
// hit the same bin are combined before the shared-memory atomic.
__global__ void __launch_bounds__(kQThreads) k_hist(const unsigned long long* __restrict__ keys, long long n, int shift,
                                                    int nr, const unsigned long long* __restrict__ prefix,
                                                    unsigned int* __restrict__ hist) {
  __shared__ unsigned int sh[kGroup * 256];
  __shared__ unsigned long long pf[kGroup];
  for (int i = threadIdx.x; i < kGroup * 256; i += blockDim.x) sh[i] = 0;
  if (threadIdx.x < nr) pf[threadIdx.x] = prefix[threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long first = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  // warp-uniform trip count: every lane runs the same number of iterations
  const long long base0 = first - lane;
  for (long long base = base0; base < n; base += stride) {
    const long long i = base + lane;
    const bool valid = i < n;
    const unsigned long long key = valid ? keys[i] : 0ull;
    const unsigned long long hi = shift >= 56 ? 0ull : (key >> (shift + 8));
    const unsigned int bin = (unsigned int)(key >> shift) & 255u;
    for (int g = 0; g < nr; g++) {
      const bool m = valid && hi == pf[g];
      if (!__any_sync(0xffffffffu, m)) continue;
      const unsigned int peers = __match_any_sync(0xffffffffu, m ? bin : 0x100u + lane);
      if (m && lane == __ffs(peers) - 1) atomicAdd(&sh[g * 256 + bin], (unsigned int)__popc(peers));
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nr * 256; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// Picks, for every rank of the group, the bin that holds it: prefix gains the
// bin's 8 bits and rank becomes the rank within the bin.
__global__ void k_pick(int nr, unsigned long long* __restrict__ prefix, unsigned long long* __restrict__ rank,
                       const unsigned int* __restrict__ hist) {
  const int g = threadIdx.x;
  if (g >= nr) return;
  unsigned long long r = rank[g], below = 0;
  int bin = 0;
  for (; bin < 255; bin++) {
    const unsigned long long c = hist[g * 256 + bin];
    if (r < below + c) break;
    below += c;
  }
  prefix[g] = (prefix[g] << 8) | (unsigned long long)bin;
  rank[g] = r - below;
}

}  // namespace

extern "C" int jne_percentiles_device(jne_context* c, const double* eigs_device, int64_t n, int k, int stat,
                                      const double* ps, int np, double* out, void* stream) {
  if (!c) return JNE_ERR_ARG;
  if ((n > 0 && !eigs_device) || (np > 0 && (!ps || !out)) || k < 1 || n < 0 || np < 0 || (stat != 0 && stat != 1))
    return fail(c, JNE_ERR_ARG, "bad percentile arguments");
  for (int i = 0; i < np; i++)
    if (!(ps[i] >= 0.0 && ps[i] <= 1.0)) return fail(c, JNE_ERR_ARG, "percentiles must lie in [0, 1]");
  if (np == 0) return JNE_OK;
  if (n == 0) {
    for (int i = 0; i < np; i++) out[i] = NAN;
    return JNE_OK;
  }
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, JNE_ERR_CUDA, "cudaSetDevice failed");
  int rc = drain(c);
  if (rc) return rc;
  if ((rc = join_in(c, (cudaStream_t)stream))) return rc;
  // the distinct ranks floor / ceil of p (n - 1)
  std::vector<unsigned long long> ranks;
  for (int i = 0; i < np; i++) {
    const double rank = ps[i] * (double)(n - 1);
    ranks.push_back((unsigned long long)std::floor(rank));
    ranks.push_back((unsigned long long)std::ceil(rank));
  }
  std::sort(ranks.begin(), ranks.end());
  ranks.erase(std::unique(ranks.begin(), ranks.end()), ranks.end());
  const int nr = (int)ranks.size();
  // scratch: keys | NaN count | per rank: prefix, rank | histograms
  const size_t words = (size_t)n + 1 + 2 * (size_t)nr + ((size_t)nr * 256 + 1) / 2;
  if ((rc = ensure(c, &c->d_qscratch, &c->qscratch_cap, words, "percentile scratch"))) return rc;
  unsigned long long* keys = c->d_qscratch;
  unsigned int* n_nan = reinterpret_cast<unsigned int*>(keys + n);
  unsigned long long* prefix = keys + n + 1;
  unsigned long long* rank = prefix + nr;
  unsigned int* hist = reinterpret_cast<unsigned int*>(rank + nr);
  cudaStream_t st = c->stream;
  cudaError_t e = cudaMemsetAsync(n_nan, 0, sizeof(unsigned int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(prefix, 0, sizeof(unsigned long long) * nr, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(rank, ranks.data(), sizeof(unsigned long long) * nr, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(c, e, "percentile setup");
  const long long want = (n + kQThreads - 1) / kQThreads;
  const int grid = (int)std::min<long long>(want, (long long)c->sms * 8);
  k_aggregate<<<grid, kQThreads, 0, st>>>(eigs_device, n, k, stat, keys, n_nan);
  for (int g0 = 0; g0 < nr && e == cudaSuccess; g0 += kGroup) {
    const int ng = std::min(kGroup, nr - g0);
    for (int pass = 0; pass < 8 && e == cudaSuccess; pass++) {
      e = cudaMemsetAsync(hist, 0, sizeof(unsigned int) * 256 * ng, st);
      if (e != cudaSuccess) break;
      k_hist<<<grid, kQThreads, 0, st>>>(keys, n, 56 - 8 * pass, ng, prefix + g0, hist);
      k_pick<<<1, kGroup, 0, st>>>(ng, prefix + g0, rank + g0, hist);
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "percentile launch");
  std::vector<unsigned long long> sel(nr);
  unsigned int nans = 0;
  e = cudaMemcpyAsync(sel.data(), prefix, sizeof(unsigned long long) * nr, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&nans, n_nan, sizeof nans, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "percentile select");
  if (nans) return fail(c, JNE_ERR_NUMERIC, std::to_string(nans) + " runs have a NaN aggregate (unordered)");
  auto at = [&](unsigned long long r) {
    const size_t i = (size_t)(std::lower_bound(ranks.begin(), ranks.end(), r) - ranks.begin());
    return value_of(sel[i]);
  };
  for (int i = 0; i < np; i++) {  // get_percentile_value, simulation_analyzers.rs:4-18
    const double rank = ps[i] * (double)(n - 1);
    const unsigned long long lo = (unsigned long long)std::floor(rank), hi = (unsigned long long)std::ceil(rank);
    if (lo == hi) {
      out[i] = at(lo);
    } else {
      const double wgt = rank - (double)lo;
      out[i] = at(lo) * (1.0 - wgt) + at(hi) * wgt;
    }
  }
  return JNE_OK;
}
