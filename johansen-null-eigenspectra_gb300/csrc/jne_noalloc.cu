// jne_noalloc.cu -- jne_eigs_seeded_noalloc: the seeded batch for callers that
// cannot allocate device memory.
//
// Some hosts of this path cannot call cudaMalloc: an allocator-owning framework
// that forbids foreign allocations, a CUDA-graph-captured region, a real-time
// loop with no allocation after start-up, or an embedding that only hands out
// device pointers for its own inputs and outputs.  This entry point takes its
// scratch (the FP64 moment records, the chunk time table, the FP64 entry table
// and the status word) from one file-scope __device__ array of fixed size that
// every GPU loading this library holds until the process exits.  It calls no
// cudaMalloc, cudaFree or allocating library routine.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/jne.h"
#include "jne_kernels.h"

namespace {

// ---- the scratch array and its layout ----
constexpr size_t kAlign = 256;
constexpr size_t round_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
constexpr int kRecordMax = JNE_MAX_DIM * (JNE_MAX_DIM + 1) / 2 + 6 * JNE_MAX_DIM + JNE_MAX_DIM * JNE_MAX_DIM;
constexpr size_t kMomBytes = round_up(sizeof(double) * (size_t)JNE_NOALLOC_MAX_RUNS * kRecordMax);
constexpr size_t kChunkBytes = round_up(sizeof(jne_chunk_time) * (size_t)JNE_NOALLOC_MAX_CHUNKS);
constexpr size_t kEntCap = 512;
constexpr size_t kEntBytes = round_up(sizeof(int4) * kEntCap);
constexpr size_t kStatusBytes = kAlign;
constexpr size_t kScratchBytes = kMomBytes + kChunkBytes + kEntBytes + kStatusBytes;
static_assert(kScratchBytes == JNE_NOALLOC_SCRATCH_BYTES, "scratch size stated in jne.h");

static __device__ __align__(256) unsigned char jne_noalloc_scratch[kScratchBytes];

// In host code jne_noalloc_scratch names a host-side stand-in, not device
// memory: its device address comes from cudaGetSymbolAddress, once per device.
std::mutex g_mu;
void* g_scratch[64] = {};
int g_sms[64] = {};

thread_local std::string g_err;
int fail(int code, const std::string& m) {
  g_err = m;
  return code;
}

// Same policy as the context entry points: mixed requests on short paths run
// the FP64 kernel, and the mixed chunk length is the largest power of two
// <= steps/16 in [32, 512].
int noalloc_chunk(int steps) {
  int L = 32;
  while (L < 512 && 2 * L * 16 <= steps) L *= 2;
  return L;
}

// Per-chunk time means of the mixed kernel, computed on the device.
__global__ void k_fill_chunk_table(jne_chunk_time* tab, int steps, int chunk, int nch) {
  const int ch = blockIdx.x * blockDim.x + threadIdx.x;
  if (ch >= nch) return;
  const double T = steps;
  const double c0 = (double)ch * chunk;
  const double lc = fmin((double)chunk, T - c0);
  const double s1 = lc * (2.0 * c0 + lc + 1.0) / 2.0;  // sum of (i+1) over the chunk's columns
  // sum of (i+1)^2 = sum_{j=c0+1}^{c0+lc} j^2, written without the large-number cancellation
  const double s2 = lc * (c0 * c0 + c0 * (lc + 1.0)) + lc * (lc + 1.0) * (2.0 * lc + 1.0) / 6.0;
  const double yb = s1 / (T * lc), y2b = s2 / (T * T * lc);
  const float ybh = (float)yb, y2h = (float)y2b;
  tab[ch] = {ybh, (float)(yb - (double)ybh), y2h, (float)(y2b - (double)y2h), (float)lc, 1.0f / (float)lc, 0.f, 0.f};
}

// FP64 moment entries of a (model, dim) pair, built on the device (the same
// list the context path builds on the host).
__global__ void k_fill_entries(int4* out, int model, int d, int* count) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int W = 0, Z = d, ONE = 2 * d, Y = 2 * d + 1, YY = 2 * d + 2;
  const int nb = (model == 2 || model == 4) ? d - 1 : d;
  const bool need_w1 = model >= 1, need_y = model >= 2, need_yy = model == 4;
  int n = 0;
  for (int p = 0; p < nb; p++)
    for (int q = p; q < nb; q++) out[n++] = make_int4(W + p, W + q, jne_slot_MWW(p, q, d), 0);
  for (int p = 0; p < nb; p++) {
    if (need_w1) out[n++] = make_int4(W + p, ONE, jne_slot_MW1(p, d), 0);
    if (need_y) out[n++] = make_int4(W + p, Y, jne_slot_MWy(p, d), 0);
    if (need_yy) out[n++] = make_int4(W + p, YY, jne_slot_MWyy(p, d), 0);
  }
  for (int a = 0; a < d; a++)
    for (int b = 0; b < nb; b++) out[n++] = make_int4(Z + a, W + b, jne_slot_NzW(a, b, d), 0);
  for (int a = 0; a < d; a++) {
    if (need_y) out[n++] = make_int4(Z + a, Y, jne_slot_Nzy(a, d), 0);
    if (need_yy) out[n++] = make_int4(Z + a, YY, jne_slot_Nzyy(a, d), 0);
  }
  *count = n;
}

int host_entry_count(int model, int d) {
  const int nb = (model == 2 || model == 4) ? d - 1 : d;
  const int per_walk = (model >= 1) + (model >= 2) + (model == 4);
  const int per_inc = (model >= 2) + (model == 4);
  return nb * (nb + 1) / 2 + nb * per_walk + d * nb + d * per_inc;
}

}  // namespace

extern "C" int jne_eigs_seeded_noalloc(int device, int model, int dim, int steps, uint64_t base_seed,
                                       uint32_t seed_first, int n_runs, int precision, double* out_device,
                                       void* stream) {
  if (model < 0 || model > 4 || dim < 1 || dim > JNE_MAX_DIM || steps < 1 || n_runs < 0)
    return fail(JNE_ERR_ARG, "model must be 0..4, dim 1.." + std::to_string(JNE_MAX_DIM) + ", steps >= 1");
  if (precision != JNE_PREC_FP64 && precision != JNE_PREC_MIXED) return fail(JNE_ERR_ARG, "unknown precision");
  if (n_runs > JNE_NOALLOC_MAX_RUNS)
    return fail(JNE_ERR_BUDGET, "n_runs " + std::to_string(n_runs) + " exceeds the no-allocation limit of " +
                                    std::to_string(JNE_NOALLOC_MAX_RUNS) + " runs per call");
  const bool mixed = precision == JNE_PREC_MIXED && steps >= JNE_MIXED_MIN_STEPS;
  const int chunk = noalloc_chunk(steps);
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
  unsigned char* base = nullptr;
  int sms = 0;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch[device]) {  // once per device, with that device current
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, jne_noalloc_scratch);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_sms[device], cudaDevAttrMultiProcessorCount, device);
      if (e != cudaSuccess) {
        if (prev != device) cudaSetDevice(prev);
        return fail(JNE_ERR_CUDA, std::string("scratch set-up: ") + cudaGetErrorString(e));
      }
      g_scratch[device] = p;
    }
    base = static_cast<unsigned char*>(g_scratch[device]);
    sms = g_sms[device];
  }
  double* mom = reinterpret_cast<double*>(base);
  jne_chunk_time* ctab = reinterpret_cast<jne_chunk_time*>(base + kMomBytes);
  int4* ent = reinterpret_cast<int4*>(base + kMomBytes + kChunkBytes);
  unsigned int* status = reinterpret_cast<unsigned int*>(base + kMomBytes + kChunkBytes + kEntBytes);
  int* ent_count = reinterpret_cast<int*>(status + 1);
  cudaStream_t st = (cudaStream_t)stream;

  uint32_t k0 = (uint32_t)base_seed, k1 = (uint32_t)(base_seed >> 32) ^ (0x4A4E0000u | (uint32_t)(dim & 0xFF));
  jne_accum_args a{};
  a.model = model;
  a.dim = dim;
  a.steps = steps;
  a.n_runs = n_runs;
  a.seed_first = seed_first;
  a.key0 = k0;
  a.key1 = k1;
  a.chunk = chunk;
  a.chunk_tab = ctab;
  a.mom = mom;
  a.mom_ld = n_runs;
  a.status = status;
  e = cudaMemsetAsync(status, 0, sizeof(unsigned int), st);
  if (e == cudaSuccess) {
    if (mixed) {
      k_fill_chunk_table<<<(nch + 127) / 128, 128, 0, st>>>(ctab, steps, chunk, nch);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = jne_launch_accum_mixed(a, nullptr, sms, st);
    } else {
      k_fill_entries<<<1, 1, 0, st>>>(ent, model, dim, ent_count);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = jne_launch_accum_f64(a, ent, host_entry_count(model, dim), sms, st);
    }
  }
  if (e == cudaSuccess) {
    jne_finalize_args f{};
    f.model = model;
    f.dim = dim;
    f.steps = steps;
    f.n_runs = n_runs;
    f.zscale = 1.0 / std::sqrt((double)steps);
    const long double T = steps;  // Y_p = sum_{i=1}^{T} (i/T)^p
    f.ts.Y[0] = (double)T;
    f.ts.Y[1] = (double)((T + 1.0L) / 2.0L);
    f.ts.Y[2] = (double)((T + 1.0L) * (2.0L * T + 1.0L) / (6.0L * T));
    f.ts.Y[3] = (double)((T + 1.0L) * (T + 1.0L) / (4.0L * T));
    f.ts.Y[4] = (double)((T + 1.0L) * (2.0L * T + 1.0L) * (3.0L * T * T + 3.0L * T - 1.0L) / (30.0L * T * T * T));
    f.mom = mom;
    f.mom_ld = n_runs;
    f.out = out_device;
    f.status = status;
    e = jne_launch_finalize(f, sms, st);
  }
  unsigned int stv = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&stv, status, sizeof(stv), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (prev != device) cudaSetDevice(prev);
  if (e != cudaSuccess) return fail(JNE_ERR_CUDA, std::string("no-allocation batch: ") + cudaGetErrorString(e));
  if (stv & JNE_DEV_NOT_SPD) return fail(JNE_ERR_NUMERIC, "S11 not positive definite for some run (NaN written)");
  return JNE_OK;
}

extern "C" const char* jne_noalloc_last_error(void) { return g_err.c_str(); }
