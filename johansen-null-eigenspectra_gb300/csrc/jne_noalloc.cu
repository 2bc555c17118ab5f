// jne_noalloc.cu -- jne_eigs_seeded_noalloc: the seeded batch for callers that
// cannot allocate device memory.
//
// Some hosts of this path cannot call cudaMalloc: an allocator-owning framework
// that forbids foreign allocations, a real-time loop with no allocation after
// start-up, or an embedding that only hands out device pointers for its own
// inputs and outputs.  This entry point takes its scratch (the FP64 moment
// records, the chunk time table, the FP64 entry table, the work and batch
// counters and the status word) from one file-scope __device__ array of fixed
// size that every GPU loading this library holds until the process exits.  It
// calls no cudaMalloc, cudaFree or allocating library routine.
//
// It runs exactly the kernels and tables of the context entry point
// (jne_eigs_seeded): the chunk table and the FP64 entry table come from the
// same host functions, and a mixed request is the same fused accumulate +
// finalize launch, so the two give the same bits.
#include <cstring>
#include <mutex>
#include <string>

#include "jne_context.h"

namespace {

// ---- the scratch array and its layout ----
constexpr size_t kAlign = 256;
constexpr size_t round_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
constexpr int kRecordMax = JNE_MAX_DIM * (JNE_MAX_DIM + 1) / 2 + 6 * JNE_MAX_DIM + JNE_MAX_DIM * JNE_MAX_DIM;
constexpr size_t kEntCap = 512;
constexpr size_t kMomBytes = round_up(sizeof(double) * (size_t)JNE_NOALLOC_MAX_RUNS * kRecordMax);
constexpr size_t kChunkBytes = round_up(sizeof(jne_chunk_time) * (size_t)JNE_NOALLOC_MAX_CHUNKS);
constexpr size_t kEntBytes = round_up(sizeof(int4) * kEntCap);
// status word (offset 0) and the mixed kernel's work counter (offset 8)
constexpr size_t kWordsBytes = kAlign;
// completion counts of the fused finalize, one per 32 runs
constexpr size_t kBatchBytes = round_up(sizeof(unsigned int) * ((JNE_NOALLOC_MAX_RUNS + 31) / 32));
constexpr size_t kScratchBytes = kMomBytes + kChunkBytes + kEntBytes + kWordsBytes + kBatchBytes;
static_assert(kScratchBytes == JNE_NOALLOC_SCRATCH_BYTES, "scratch size stated in jne.h");

static __device__ __align__(256) unsigned char jne_noalloc_scratch[kScratchBytes];

// In host code jne_noalloc_scratch names a host-side stand-in, not device
// memory: its device address comes from cudaGetSymbolAddress, once per device.
std::mutex g_mu;
void* g_scratch[64] = {};
int g_sms[64] = {};
// host staging of the tables (copied to the device under g_mu; a copy from
// pageable memory has read its source when the call returns)
jne_chunk_time g_hchunk[JNE_NOALLOC_MAX_CHUNKS];
int4 g_hent[kEntCap];

thread_local std::string g_err;
int fail(int code, const std::string& m) {
  g_err = m;
  return code;
}

}  // namespace

extern "C" int jne_eigs_seeded_noalloc(int device, int model, int dim, int steps, uint64_t base_seed,
                                       uint32_t seed_first, int n_runs, int precision, double* out_device,
                                       void* stream) {
  using namespace jne_detail;
  if (!valid_model_dim(model, dim) || steps < 1 || n_runs < 0)
    return fail(JNE_ERR_ARG, "model must be 0..4, dim 1.." + std::to_string(JNE_MAX_DIM) + ", steps >= 1");
  if (precision != JNE_PREC_FP64 && precision != JNE_PREC_MIXED) return fail(JNE_ERR_ARG, "unknown precision");
  if (n_runs > JNE_NOALLOC_MAX_RUNS)
    return fail(JNE_ERR_BUDGET, "n_runs " + std::to_string(n_runs) + " exceeds the no-allocation limit of " +
                                    std::to_string(JNE_NOALLOC_MAX_RUNS) + " runs per call");
  const bool mixed = kernel_precision(precision, steps) == JNE_PREC_MIXED;
  const int chunk = adaptive_chunk(steps);  // the context's default rule
  const int nch = (steps + chunk - 1) / chunk;
  if (mixed && nch > JNE_NOALLOC_MAX_CHUNKS)
    return fail(JNE_ERR_BUDGET, "steps " + std::to_string(steps) + " exceed the no-allocation limit of " +
                                    std::to_string(JNE_NOALLOC_MAX_CHUNKS * 512) + " steps for mixed precision");
  if ((uint64_t)seed_first + (uint64_t)n_runs > 0x100000000ull) return fail(JNE_ERR_ARG, "seed range exceeds u32");
  if (n_runs == 0) return JNE_OK;
  if (!out_device) return fail(JNE_ERR_ARG, "null output buffer");
  if (device < 0 || device >= 64) return fail(JNE_ERR_ARG, "device index out of range");

  int prev = 0;
  cudaError_t e = cudaGetDevice(&prev);
  if (e == cudaSuccess && prev != device) e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(JNE_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  cudaStream_t st = (cudaStream_t)stream;
  std::unique_lock<std::mutex> lk(g_mu);
  if (!g_scratch[device]) {  // once per device, with that device current
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, jne_noalloc_scratch);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_sms[device], cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
      lk.unlock();
      if (prev != device) cudaSetDevice(prev);
      return fail(JNE_ERR_CUDA, std::string("scratch set-up: ") + cudaGetErrorString(e));
    }
    g_scratch[device] = p;
  }
  unsigned char* base = static_cast<unsigned char*>(g_scratch[device]);
  const int sms = g_sms[device];
  double* mom = reinterpret_cast<double*>(base);
  jne_chunk_time* ctab = reinterpret_cast<jne_chunk_time*>(base + kMomBytes);
  int4* ent = reinterpret_cast<int4*>(base + kMomBytes + kChunkBytes);
  unsigned char* words = base + kMomBytes + kChunkBytes + kEntBytes;
  unsigned int* status = reinterpret_cast<unsigned int*>(words);
  unsigned long long* next_run = reinterpret_cast<unsigned long long*>(words + 8);
  unsigned int* batch_done = reinterpret_cast<unsigned int*>(words + kWordsBytes);

  uint32_t k0, k1;
  stream_key(base_seed, dim, &k0, &k1);
  jne_accum_args a{};
  a.model = model;
  a.dim = dim;
  a.steps = steps;
  a.n_runs = n_runs;
  a.seed_first = seed_first;
  a.key0 = k0;
  a.key1 = k1;
  a.chunk = chunk;
  a.ext_inv_scale = std::sqrt((double)steps);
  a.mom = mom;
  a.mom_ld = n_runs;
  a.status = status;
  jne_finalize_args f{};
  f.model = model;
  f.dim = dim;
  f.steps = steps;
  f.n_runs = n_runs;
  f.zscale = 1.0 / std::sqrt((double)steps);
  f.ts = time_sums(steps);
  f.mom = mom;
  f.mom_ld = n_runs;
  f.out = out_device;
  f.status = status;
  // every call clears what must start at zero: the status word and the counters
  e = cudaMemsetAsync(words, 0, kWordsBytes + kBatchBytes, st);
  if (e == cudaSuccess) {
    if (mixed) {
      fill_chunk_table(steps, chunk, g_hchunk);
      e = cudaMemcpyAsync(ctab, g_hchunk, sizeof(jne_chunk_time) * nch, cudaMemcpyHostToDevice, st);
      a.chunk_tab = ctab;
      a.next_run = next_run;
      a.batch_done = batch_done;
      if (e == cudaSuccess) e = jne_launch_accum_mixed(a, &f, sms, st);  // accumulation + fused finalize
    } else {
      const int nent = jne_build_f64_entries(model, dim, g_hent, (int)kEntCap);
      e = cudaMemcpyAsync(ent, g_hent, sizeof(int4) * nent, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = jne_launch_accum_f64(a, ent, nent, sms, st);
      if (e == cudaSuccess) e = jne_launch_finalize(f, sms, st);
    }
  }
  lk.unlock();
  unsigned int stv = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&stv, status, sizeof(stv), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (prev != device) cudaSetDevice(prev);
  if (e != cudaSuccess) return fail(JNE_ERR_CUDA, std::string("no-allocation batch: ") + cudaGetErrorString(e));
  if (stv & JNE_DEV_BAD_ARGS) return fail(JNE_ERR_ARG, "a kernel rejected its arguments");
  if (stv & JNE_DEV_NOT_SPD) return fail(JNE_ERR_NUMERIC, "S11 not positive definite for some run (NaN written)");
  return JNE_OK;
}

extern "C" const char* jne_noalloc_last_error(void) { return g_err.c_str(); }
