// jne_api.cu -- the C ABI (include/jne.h): contexts, device buffers under a
// memory budget, request validation, kernel sequencing and host copies.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/jne.h"
#include "jne_kernels.h"

struct jne_context {
  int device = 0;
  int sms = 0;
  unsigned long long budget = 0;
  unsigned long long in_use = 0;
  int chunk = 0;  // 0: chunk length chosen from the step count
  jne_chunk_time* d_ctab = nullptr;
  size_t ctab_cap = 0;
  std::vector<jne_chunk_time> h_ctab;
  int ctab_steps = -1, ctab_chunk = -1;  // table currently on the device
  int ent_model = -2, ent_dim = -1, ent_n = 0;
  cudaStream_t stream = nullptr;
  double* d_mom = nullptr;
  size_t mom_cap = 0;  // doubles
  double* d_out = nullptr;
  size_t out_cap = 0;
  double* d_ext = nullptr;
  size_t ext_cap = 0;
  uint32_t* d_words = nullptr;
  size_t words_cap = 0;
  int4* d_ent = nullptr;
  size_t ent_cap = 0;
  unsigned int* d_status = nullptr;
  std::string err;
  // asynchronous device path: two record buffers, finalize on a second stream
  cudaStream_t fin_stream = nullptr;
  cudaEvent_t ev_acc[2] = {nullptr, nullptr}, ev_fin[2] = {nullptr, nullptr};
  bool fin_pending[2] = {false, false};
  double* d_momb[2] = {nullptr, nullptr};
  size_t momb_cap[2] = {0, 0};
  unsigned long long batch_seq = 0;
  // per-kernel event timing (jne_profile)
  bool profiling = false;
  struct Timed {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<Timed> timed;
  std::vector<cudaEvent_t> event_pool;
  double prof_ms[JNE_KERNEL_KINDS] = {0, 0, 0, 0};
  long long prof_n[JNE_KERNEL_KINDS] = {0, 0, 0, 0};
};

namespace {

const char* kNoCtx = "null context";

int fail(jne_context* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(jne_context* c, cudaError_t e, const char* what) {
  return fail(c, JNE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Grows a device buffer (contents are not preserved) within the budget.
template <typename T>
int ensure(jne_context* c, T** p, size_t* cap, size_t n, const char* what) {
  if (n <= *cap) return JNE_OK;
  const unsigned long long old_bytes = (unsigned long long)(*cap) * sizeof(T);
  const unsigned long long new_bytes = (unsigned long long)n * sizeof(T);
  if (c->in_use - old_bytes + new_bytes > c->budget)
    return fail(c, JNE_ERR_BUDGET, std::string(what) + ": " + std::to_string(new_bytes) +
                                       " bytes exceed the device-memory budget of " + std::to_string(c->budget));
  if (*p) cudaFree(*p);
  *p = nullptr;
  c->in_use -= old_bytes;
  *cap = 0;
  cudaError_t e = cudaMalloc((void**)p, new_bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  c->in_use += new_bytes;
  *cap = n;
  return JNE_OK;
}

cudaEvent_t take_event(jne_context* c) {
  if (!c->event_pool.empty()) {
    cudaEvent_t e = c->event_pool.back();
    c->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// Folds finished event pairs into the per-kind totals (waits for them).
void prof_flush(jne_context* c) {
  for (auto& t : c->timed) {
    float ms = 0.f;
    if (cudaEventSynchronize(t.b) == cudaSuccess && cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) {
      c->prof_ms[t.kind] += ms;
      c->prof_n[t.kind] += 1;
    }
    c->event_pool.push_back(t.a);
    c->event_pool.push_back(t.b);
  }
  c->timed.clear();
}

// Brackets one kernel launch with events on its stream when profiling is on.
struct ProfScope {
  jne_context* c;
  int kind;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  ProfScope(jne_context* c_, int kind_, cudaStream_t st_) : c(c_), kind(kind_), st(st_) {
    if (c->profiling && (a = take_event(c))) cudaEventRecord(a, st);
  }
  ~ProfScope() {
    if (!a) return;
    cudaEvent_t b = take_event(c);
    if (!b) {
      c->event_pool.push_back(a);
      return;
    }
    cudaEventRecord(b, st);
    c->timed.push_back({kind, a, b});
    if (c->timed.size() > 4096) prof_flush(c);
  }
};

// Steps per FP32 chunk of the mixed kernel: about T/32, a power of two in
// [32, 256].  Short paths get short chunks, so that the FP64 chunk means carry
// most of every moment and the FP32 centred parts stay a small share.
int adaptive_chunk(int steps) {
  int L = 32;
  while (L < 256 && 2 * L * 32 <= steps) L *= 2;
  return L;
}

bool valid_model_dim(int model, int dim) { return model >= 0 && model <= 4 && dim >= 1 && dim <= JNE_MAX_DIM; }

jne_time_sums time_sums(int steps) {
  // Y_p = sum_{i=1}^{T} (i/T)^p by Faulhaber's formulas, in long double
  const long double T = steps;
  jne_time_sums s;
  s.Y[0] = (double)T;
  s.Y[1] = (double)((T + 1.0L) / 2.0L);
  s.Y[2] = (double)((T + 1.0L) * (2.0L * T + 1.0L) / (6.0L * T));
  s.Y[3] = (double)((T + 1.0L) * (T + 1.0L) / (4.0L * T));
  s.Y[4] = (double)((T + 1.0L) * (2.0L * T + 1.0L) * (3.0L * T * T + 3.0L * T - 1.0L) / (30.0L * T * T * T));
  return s;
}

void stream_key(uint64_t base_seed, int dim, uint32_t* k0, uint32_t* k1) {
  *k0 = (uint32_t)base_seed;
  *k1 = (uint32_t)(base_seed >> 32) ^ (0x4A4E0000u | (uint32_t)(dim & 0xFF));
}

int check_status(jne_context* c) {
  unsigned int st = 0;
  cudaError_t e = cudaMemcpyAsync(&st, c->d_status, sizeof(st), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "status read");
  if (st & JNE_DEV_BAD_ARGS) return fail(c, JNE_ERR_ARG, "a kernel rejected its arguments");
  if (st & JNE_DEV_NOT_SPD) return fail(c, JNE_ERR_NUMERIC, "S11 not positive definite for some run (NaN written)");
  return JNE_OK;
}

// Runs per device batch: moment records + outputs of a batch stay well inside the budget.
int64_t batch_runs(const jne_context* c, int dim, int k_total) {
  const size_t per_run = sizeof(double) * ((size_t)jne_record_slots(dim) + (size_t)k_total);
  const unsigned long long avail = c->budget > c->in_use ? c->budget / 2 : 0;
  int64_t n = (int64_t)(avail / per_run);
  if (n > (1 << 22)) n = 1 << 22;
  return n;
}

// The kernel a request runs on.  Mixed-precision requests on paths shorter
// than JNE_MIXED_MIN_STEPS use the FP64 kernel: with so few chunks the FP32
// part is most of every moment (errors up to ~1e-4 at T = 16, dim 12), and
// such paths are cheap in FP64 anyway.
int kernel_precision(int precision, int steps) {
  return (precision == JNE_PREC_MIXED && steps >= JNE_MIXED_MIN_STEPS) ? JNE_PREC_MIXED : JNE_PREC_FP64;
}

// Moments of runs [seed_first, seed_first + n) into c->d_mom (leading dim n).
int accumulate(jne_context* c, int model, int dim, int steps, uint32_t key0, uint32_t key1, uint32_t seed_first,
               int n, int precision, const double* d_ext, double* mom, cudaStream_t st) {
  precision = kernel_precision(precision, steps);
  jne_accum_args a{};
  a.model = model;
  a.dim = dim;
  a.steps = steps;
  a.n_runs = n;
  a.seed_first = seed_first;
  a.key0 = key0;
  a.key1 = key1;
  a.chunk = c->chunk ? c->chunk : adaptive_chunk(steps);
  a.ext = d_ext;
  a.ext_inv_scale = std::sqrt((double)steps);
  a.mom = mom;
  a.mom_ld = n;
  a.status = c->d_status;
  cudaError_t e;
  if (precision == JNE_PREC_FP64) {
    if (c->ent_model != model || c->ent_dim != dim) {
      int4 host_ent[512];
      c->ent_n = jne_build_f64_entries(model, dim, host_ent, 512);
      int rc = ensure(c, &c->d_ent, &c->ent_cap, 512, "entry table");
      if (rc) return rc;
      e = cudaMemcpyAsync(c->d_ent, host_ent, sizeof(int4) * c->ent_n, cudaMemcpyHostToDevice, st);
      if (e != cudaSuccess) return cuda_fail(c, e, "entry table upload");
      c->ent_model = model;
      c->ent_dim = dim;
    }
    const int nent = c->ent_n;
    ProfScope ps(c, JNE_KERNEL_ACCUM_FP64, st);
    e = jne_launch_accum_f64(a, c->d_ent, nent, c->sms, st);
  } else {
    // per-chunk time means, exact (integer sums) then rounded once
    const int nch = (steps + a.chunk - 1) / a.chunk;
    if (c->ctab_steps != steps || c->ctab_chunk != a.chunk) {
    int rc = ensure(c, &c->d_ctab, &c->ctab_cap, (size_t)nch, "chunk table");
    if (rc) return rc;
    c->h_ctab.resize(nch);
    const long double T = steps;
    for (int ch = 0; ch < nch; ch++) {
      const long long c0 = (long long)ch * a.chunk, lc = std::min<long long>(a.chunk, steps - c0);
      // columns i = c0 .. c0+lc-1 carry y = (i+1)/T
      const long double s1 = (long double)lc * (2.0L * c0 + lc + 1.0L) / 2.0L;
      auto sq = [](long double n) { return n * (n + 1.0L) * (2.0L * n + 1.0L) / 6.0L; };
      const long double s2 = sq((long double)(c0 + lc)) - sq((long double)c0);
      c->h_ctab[ch] = {(double)(s1 / (T * lc)), (double)(s2 / (T * T * lc)), (double)lc, 1.0 / (double)lc};
    }
    e = cudaMemcpyAsync(c->d_ctab, c->h_ctab.data(), sizeof(jne_chunk_time) * nch, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "chunk table upload");
    c->ctab_steps = steps;
    c->ctab_chunk = a.chunk;
    }
    a.chunk_tab = c->d_ctab;
    ProfScope ps(c, JNE_KERNEL_ACCUM_MIXED, st);
    e = jne_launch_accum_mixed(a, c->sms, st);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "accumulation launch");
  return JNE_OK;
}

int finalize(jne_context* c, int model, int dim, int steps, int n, double zscale, const double* mom, double* d_out,
             cudaStream_t st) {
  jne_finalize_args f{};
  f.model = model;
  f.dim = dim;
  f.steps = steps;
  f.n_runs = n;
  f.zscale = zscale;
  f.ts = time_sums(steps);
  f.mom = mom;
  f.mom_ld = n;
  f.out = d_out;
  f.status = c->d_status;
  ProfScope ps(c, JNE_KERNEL_FINALIZE, st);
  cudaError_t e = jne_launch_finalize(f, c->sms, st);
  if (e != cudaSuccess) return cuda_fail(c, e, "finalize launch");
  return JNE_OK;
}

int check_common(jne_context* c, int model, int dim, int steps, int64_t n_runs, int precision) {
  if (!c) return JNE_ERR_ARG;
  if (!valid_model_dim(model, dim))
    return fail(c, JNE_ERR_ARG, "model must be 0..4 and dim 1.." + std::to_string(JNE_MAX_DIM));
  if (steps < 1) return fail(c, JNE_ERR_ARG, "steps must be >= 1");
  if (n_runs < 0) return fail(c, JNE_ERR_ARG, "n_runs must be >= 0");
  if (precision != JNE_PREC_FP64 && precision != JNE_PREC_MIXED) return fail(c, JNE_ERR_ARG, "unknown precision");
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, JNE_ERR_CUDA, "cudaSetDevice failed");
  return JNE_OK;
}

// Waits for the asynchronous device path, so a synchronous call owns the status word.
int drain(jne_context* c) {
  cudaError_t e = cudaStreamSynchronize(c->fin_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "drain");
}

int clear_status(jne_context* c, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(c->d_status, 0, sizeof(unsigned int), st);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "status reset");
}

}  // namespace

extern "C" {

int jne_version(void) { return 100; }

int jne_eigen_count(int model, int dim) {
  if (model < 0 || model > 4 || dim < 1) return -1;
  return (model == 1 || model == 3) ? dim + 1 : dim;
}

int jne_open(int device, unsigned long long mem_budget_bytes, jne_context** out) {
  if (!out) return JNE_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return JNE_ERR_CUDA;
  if (device < 0 || device >= ndev) return JNE_ERR_ARG;
  jne_context* c = new jne_context();
  c->device = device;
  c->budget = mem_budget_bytes ? mem_budget_bytes : (40ull << 30);
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->fin_stream, cudaStreamNonBlocking);
  for (int i = 0; i < 2 && e == cudaSuccess; i++) {
    e = cudaEventCreateWithFlags(&c->ev_acc[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fin[i], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_status, sizeof(unsigned int));
  if (e != cudaSuccess) {
    jne_close(c);
    return JNE_ERR_CUDA;
  }
  c->in_use = sizeof(unsigned int);
  *out = c;
  return JNE_OK;
}

void jne_close(jne_context* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->fin_stream) cudaStreamSynchronize(c->fin_stream);
  if (c->stream) cudaStreamSynchronize(c->stream);
  prof_flush(c);
  for (cudaEvent_t e : c->event_pool) cudaEventDestroy(e);
  cudaFree(c->d_mom);
  cudaFree(c->d_out);
  cudaFree(c->d_ext);
  cudaFree(c->d_words);
  cudaFree(c->d_ent);
  cudaFree(c->d_ctab);
  cudaFree(c->d_status);
  for (int i = 0; i < 2; i++) {
    cudaFree(c->d_momb[i]);
    if (c->ev_acc[i]) cudaEventDestroy(c->ev_acc[i]);
    if (c->ev_fin[i]) cudaEventDestroy(c->ev_fin[i]);
  }
  if (c->fin_stream) cudaStreamDestroy(c->fin_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* jne_last_error(const jne_context* c) { return c ? c->err.c_str() : kNoCtx; }

int jne_set_chunk(jne_context* c, int chunk) {
  if (!c) return JNE_ERR_ARG;
  if (chunk != 0 && (chunk < 32 || chunk % 32 != 0 || chunk > (1 << 20)))
    return fail(c, JNE_ERR_ARG, "chunk must be 0 (adaptive) or a multiple of 32");
  c->chunk = chunk;
  return JNE_OK;
}

int jne_profile(jne_context* c, int enable) {
  if (!c) return JNE_ERR_ARG;
  c->profiling = enable != 0;
  return JNE_OK;
}

int jne_profile_read(jne_context* c, double* ms, long long* launches, int reset) {
  if (!c) return JNE_ERR_ARG;
  prof_flush(c);
  for (int k = 0; k < JNE_KERNEL_KINDS; k++) {
    if (ms) ms[k] = c->prof_ms[k];
    if (launches) launches[k] = c->prof_n[k];
    if (reset) {
      c->prof_ms[k] = 0.0;
      c->prof_n[k] = 0;
    }
  }
  return JNE_OK;
}

int jne_eigs_from_increments(jne_context* c, int model, int dim, int steps, const double* dB, int n_runs,
                             int precision, double* out) {
  int rc = check_common(c, model, dim, steps, n_runs, precision);
  if (rc) return rc;
  if (n_runs == 0) return JNE_OK;
  if (!dB || !out) return fail(c, JNE_ERR_ARG, "null buffer");
  const int k = jne_eigen_count(model, dim);
  const size_t n_ext = (size_t)n_runs * steps * dim;
  if ((rc = ensure(c, &c->d_ext, &c->ext_cap, n_ext, "increment buffer"))) return rc;
  if ((rc = ensure(c, &c->d_mom, &c->mom_cap, (size_t)n_runs * jne_record_slots(dim), "moment buffer"))) return rc;
  if ((rc = ensure(c, &c->d_out, &c->out_cap, (size_t)n_runs * k, "output buffer"))) return rc;
  cudaStream_t st = c->stream;
  if ((rc = drain(c))) return rc;
  if ((rc = clear_status(c, st))) return rc;
  cudaError_t e = cudaMemcpyAsync(c->d_ext, dB, sizeof(double) * n_ext, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(c, e, "increment upload");
  if ((rc = accumulate(c, model, dim, steps, 0, 0, 0, n_runs, precision, c->d_ext, c->d_mom, st))) return rc;
  // FP64 walks the increments as given; the mixed kernel walks dB * sqrt(T)
  const double zscale = kernel_precision(precision, steps) == JNE_PREC_FP64 ? 1.0 : 1.0 / std::sqrt((double)steps);
  if ((rc = finalize(c, model, dim, steps, n_runs, zscale, c->d_mom, c->d_out, st))) return rc;
  e = cudaMemcpyAsync(out, c->d_out, sizeof(double) * n_runs * k, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(c, e, "result download");
  return check_status(c);
}

int jne_eigs_seeded_models(jne_context* c, const int* models, int n_models, int dim, int steps, uint64_t base_seed,
                           uint32_t seed_first, int64_t n_runs, int precision, double* const* outs) {
  if (!c) return JNE_ERR_ARG;
  if (!models || !outs || n_models < 1 || n_models > 5) return fail(c, JNE_ERR_ARG, "1..5 models required");
  for (int m = 0; m < n_models; m++) {
    int rc = check_common(c, models[m], dim, steps, n_runs, precision);
    if (rc) return rc;
    if (!outs[m] && n_runs) return fail(c, JNE_ERR_ARG, "null output buffer");
  }
  if ((uint64_t)seed_first + (uint64_t)n_runs > 0x100000000ull) return fail(c, JNE_ERR_ARG, "seed range exceeds u32");
  int k_total = 0;
  for (int m = 0; m < n_models; m++) k_total += jne_eigen_count(models[m], dim);
  uint32_t k0, k1;
  stream_key(base_seed, dim, &k0, &k1);
  // a single FP64 pass needs every moment any requested model uses
  const int acc_model = (n_models == 1) ? models[0] : -1;
  const double zscale = 1.0 / std::sqrt((double)steps);
  cudaStream_t st = c->stream;
  int rc = drain(c);
  if (rc) return rc;
  if ((rc = clear_status(c, st))) return rc;
  const int64_t per = batch_runs(c, dim, k_total);
  if (per < 1) return fail(c, JNE_ERR_BUDGET, "budget too small for one run");
  for (int64_t done = 0; done < n_runs; done += per) {
    const int n = (int)std::min<int64_t>(per, n_runs - done);
    if ((rc = ensure(c, &c->d_mom, &c->mom_cap, (size_t)n * jne_record_slots(dim), "moment buffer"))) return rc;
    if ((rc = ensure(c, &c->d_out, &c->out_cap, (size_t)n * k_total, "output buffer"))) return rc;
    if ((rc = accumulate(c, acc_model, dim, steps, k0, k1, seed_first + (uint32_t)done, n, precision, nullptr,
                         c->d_mom, st)))
      return rc;
    size_t off = 0;
    for (int m = 0; m < n_models; m++) {
      const int k = jne_eigen_count(models[m], dim);
      if ((rc = finalize(c, models[m], dim, steps, n, zscale, c->d_mom, c->d_out + off, st))) return rc;
      cudaError_t e = cudaMemcpyAsync(outs[m] + (size_t)done * k, c->d_out + off, sizeof(double) * n * k,
                                      cudaMemcpyDeviceToHost, st);
      if (e != cudaSuccess) return cuda_fail(c, e, "result download");
      off += (size_t)n * k;
    }
  }
  return check_status(c);
}

int jne_eigs_seeded(jne_context* c, int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first,
                    int64_t n_runs, int precision, double* out) {
  double* outs[1] = {out};
  return jne_eigs_seeded_models(c, &model, 1, dim, steps, base_seed, seed_first, n_runs, precision, outs);
}

int jne_eigs_seeded_device(jne_context* c, int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first,
                           int64_t n_runs, int precision, double* out_device, void* stream) {
  int rc = check_common(c, model, dim, steps, n_runs, precision);
  if (rc) return rc;
  if (n_runs == 0) return JNE_OK;
  if (!out_device) return fail(c, JNE_ERR_ARG, "null output buffer");
  if ((uint64_t)seed_first + (uint64_t)n_runs > 0x100000000ull) return fail(c, JNE_ERR_ARG, "seed range exceeds u32");
  const int k = jne_eigen_count(model, dim);
  uint32_t k0, k1;
  stream_key(base_seed, dim, &k0, &k1);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const int64_t per = batch_runs(c, dim, 0) / 2;  // two record buffers in flight
  if (per < 1) return fail(c, JNE_ERR_BUDGET, "budget too small for one run");
  const double zscale = 1.0 / std::sqrt((double)steps);
  cudaError_t e = cudaSuccess;
  int last = -1;
  // Batch b accumulates into record buffer b % 2 on `st` while the finalize of
  // batch b - 1 runs on the context's second stream; events order the reuse.
  for (int64_t done = 0; done < n_runs; done += per) {
    const int n = (int)std::min<int64_t>(per, n_runs - done);
    const int b = (int)(c->batch_seq++ & 1);
    if ((rc = ensure(c, &c->d_momb[b], &c->momb_cap[b], (size_t)n * jne_record_slots(dim), "moment buffer")))
      return rc;
    if (c->fin_pending[b] && (e = cudaStreamWaitEvent(st, c->ev_fin[b], 0)) != cudaSuccess)
      return cuda_fail(c, e, "stream wait");
    if ((rc = accumulate(c, model, dim, steps, k0, k1, seed_first + (uint32_t)done, n, precision, nullptr,
                         c->d_momb[b], st)))
      return rc;
    if ((e = cudaEventRecord(c->ev_acc[b], st)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(c->fin_stream, c->ev_acc[b], 0)) != cudaSuccess)
      return cuda_fail(c, e, "stream order");
    if ((rc = finalize(c, model, dim, steps, n, zscale, c->d_momb[b], out_device + (size_t)done * k,
                       c->fin_stream)))
      return rc;
    if ((e = cudaEventRecord(c->ev_fin[b], c->fin_stream)) != cudaSuccess) return cuda_fail(c, e, "event record");
    c->fin_pending[b] = true;
    last = b;
  }
  // later work on `st` sees the finished results
  if (last >= 0 && (e = cudaStreamWaitEvent(st, c->ev_fin[last], 0)) != cudaSuccess)
    return cuda_fail(c, e, "stream wait");
  return JNE_OK;
}

int jne_sync(jne_context* c) {
  if (!c) return JNE_ERR_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, JNE_ERR_CUDA, "cudaSetDevice failed");
  cudaError_t e = cudaStreamSynchronize(c->fin_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  unsigned int stv = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&stv, c->d_status, sizeof(stv), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(unsigned int));
  if (e != cudaSuccess) return cuda_fail(c, e, "sync");
  if (stv & JNE_DEV_NOT_SPD) return fail(c, JNE_ERR_NUMERIC, "S11 not positive definite for some run (NaN written)");
  return JNE_OK;
}

int jne_export_increments(jne_context* c, int dim, int steps, uint64_t base_seed, uint32_t seed_first, int n_runs,
                          double* dB_out, uint32_t* words_out) {
  int rc = check_common(c, 0, dim, steps, n_runs, JNE_PREC_FP64);
  if (rc) return rc;
  if (n_runs == 0 || (!dB_out && !words_out)) return JNE_OK;
  uint32_t k0, k1;
  stream_key(base_seed, dim, &k0, &k1);
  const size_t n_val = (size_t)n_runs * steps * dim;
  const size_t n_words = (size_t)n_runs * steps * ((dim + 3) / 4) * 4;
  if (dB_out && (rc = ensure(c, &c->d_ext, &c->ext_cap, n_val, "export buffer"))) return rc;
  if (words_out && (rc = ensure(c, &c->d_words, &c->words_cap, n_words, "word buffer"))) return rc;
  cudaStream_t st = c->stream;
  cudaError_t e;
  {
    ProfScope ps(c, JNE_KERNEL_EXPORT, st);
    e = jne_launch_export(dim, steps, n_runs, seed_first, k0, k1, 1.0 / std::sqrt((double)steps),
                          dB_out ? c->d_ext : nullptr, words_out ? c->d_words : nullptr, st);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "export launch");
  if (dB_out) {
    e = cudaMemcpyAsync(dB_out, c->d_ext, sizeof(double) * n_val, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "export download");
  }
  if (words_out) {
    e = cudaMemcpyAsync(words_out, c->d_words, sizeof(uint32_t) * n_words, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "export download");
  }
  e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "export");
}

}  // extern "C"
