// jne_context.h -- the context behind the C ABI and the host helpers shared by
// the translation units that implement it (internal to libjne_gb300.so).
#pragma once
#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/jne.h"
#include "jne_kernels.h"

// The mixed kernel's launch shape for one (dim, class of steps): chunk length,
// blocks per SM of the kernel variant (4 or 6) and whether dims <= 4 pack two
// runs per warp.  Only the chunk changes the arithmetic.
struct jne_shape {
  int chunk = 0, blocks_per_sm = 4, pack = 1;
};

struct jne_context {
  int device = 0;
  int sms = 0;
  unsigned long long budget = 0;
  unsigned long long in_use = 0;
  int chunk = 0;  // 0: chunk length chosen from the step count; JNE_CHUNK_TUNED: tuned table
  std::map<std::pair<int, int>, jne_shape> tuned;  // (dim, floor(log2 steps)) -> shape
  jne_shape force;  // while tuning: blocks per SM and packing of every single-request launch
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
  unsigned int* d_req_status = nullptr;  // per-request status words (jne_run_batch_status)
  size_t req_status_cap = 0;
  unsigned long long* d_next_run = nullptr;  // work counter of single-request mixed launches
  unsigned int* d_batch = nullptr;           // per-32-run completion counts of fused finalizes
  size_t batch_cap = 0;
  unsigned long long* d_qscratch = nullptr;  // percentile analyzer: keys, ranks, histograms
  size_t qscratch_cap = 0;
  std::string err;
  // asynchronous device path: two record buffers, finalize on a second stream
  cudaStream_t fin_stream = nullptr;
  cudaEvent_t ev_acc[2] = {nullptr, nullptr}, ev_fin[2] = {nullptr, nullptr};
  bool fin_pending[2] = {false, false};
  double* d_momb[2] = {nullptr, nullptr};
  size_t momb_cap[2] = {0, 0};
  unsigned long long batch_seq = 0;
  cudaEvent_t ev_in = nullptr;    // joins a caller's stream into the context's streams
  cudaEvent_t ev_join = nullptr;  // the finalize stream's work of a batch -> the caller's stream
  // ragged batches: per record buffer, the device request table, chunk tables,
  // work counter, and pinned host staging for the tables
  jne_ragged_req* d_reqs[2] = {nullptr, nullptr};
  size_t reqs_cap[2] = {0, 0};
  jne_chunk_time* d_rtab[2] = {nullptr, nullptr};
  size_t rtab_cap[2] = {0, 0};
  unsigned long long* d_counter[2] = {nullptr, nullptr};
  size_t counter_cap[2] = {0, 0};
  unsigned int* d_bdone[2] = {nullptr, nullptr};
  size_t bdone_cap[2] = {0, 0};
  jne_ragged_req* h_reqs[2] = {nullptr, nullptr};
  size_t h_reqs_cap[2] = {0, 0};
  jne_chunk_time* h_rtab[2] = {nullptr, nullptr};
  size_t h_rtab_cap[2] = {0, 0};
  // streaming sink: per round slot, device results and status words, pinned host copies
  double* d_sink[2] = {nullptr, nullptr};
  size_t d_sink_cap[2] = {0, 0};
  unsigned int* d_sink_st[2] = {nullptr, nullptr};
  size_t d_sink_st_cap[2] = {0, 0};
  double* h_sink[2] = {nullptr, nullptr};
  size_t h_sink_cap[2] = {0, 0};
  unsigned int* h_sink_st[2] = {nullptr, nullptr};
  size_t h_sink_st_cap[2] = {0, 0};
  // ... and, for sinks that take packed records, the records on the device and their pinned host copy
  unsigned char* d_pack[2] = {nullptr, nullptr};
  size_t d_pack_cap[2] = {0, 0};
  unsigned char* h_pack[2] = {nullptr, nullptr};
  size_t h_pack_cap[2] = {0, 0};
  cudaEvent_t ev_sink[2] = {nullptr, nullptr};
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

namespace jne_detail {


constexpr const char* kNoCtx = "null context";

inline int fail(jne_context* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

inline int cuda_fail(jne_context* c, cudaError_t e, const char* what) {
  return fail(c, JNE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Grows a device buffer (contents are not preserved) within the budget.
template <typename T>
inline int ensure(jne_context* c, T** p, size_t* cap, size_t n, const char* what) {
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

inline cudaEvent_t take_event(jne_context* c) {
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
inline void prof_flush(jne_context* c) {
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

// Steps per FP32 chunk of the mixed kernel: the largest power of two <= T/16,
// clamped to [32, 512].  Short paths get short chunks, so that the exact chunk
// means carry most of every moment and the FP32 centred parts stay a small
// share (max-eig errors vs FP64 at dim 12 stay near 5e-7 to 7e-7).
inline int adaptive_chunk(int steps) {
  int L = 32;
  while (L < 512 && 2 * L * 16 <= steps) L *= 2;
  return L;
}

inline int steps_bucket(int steps) {
  int b = 0;
  while ((2ll << b) <= steps) b++;
  return b;  // 2^b <= steps < 2^(b+1)
}

// The mixed kernel's chunk length for a request of (dim, steps).
inline int chunk_for(const jne_context* c, int dim, int steps) {
  if (c->chunk > 0) return c->chunk;
  if (c->chunk == JNE_CHUNK_TUNED) {
    const auto it = c->tuned.find({dim, steps_bucket(steps)});
    if (it != c->tuned.end()) return it->second.chunk;
  }
  return adaptive_chunk(steps);
}

// The single-request kernel variant for (dim, steps): the tuned one in
// JNE_CHUNK_TUNED mode, else 4 blocks per SM with packed small dims (or the
// tuner's candidate while it times one).
inline jne_shape shape_for(const jne_context* c, int dim, int steps) {
  jne_shape s = c->force;
  if (c->chunk == JNE_CHUNK_TUNED) {
    const auto it = c->tuned.find({dim, steps_bucket(steps)});
    if (it != c->tuned.end()) s = it->second;
  }
  s.chunk = chunk_for(c, dim, steps);
  return s;
}

inline bool valid_model_dim(int model, int dim) { return model >= 0 && model <= 4 && dim >= 1 && dim <= JNE_MAX_DIM; }

inline jne_time_sums time_sums(int steps) {
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

inline void stream_key(uint64_t base_seed, int dim, uint32_t* k0, uint32_t* k1) {
  *k0 = (uint32_t)base_seed;
  *k1 = (uint32_t)(base_seed >> 32) ^ (0x4A4E0000u | (uint32_t)(dim & 0xFF));
}

inline int check_status(jne_context* c) {
  unsigned int st = 0;
  cudaError_t e = cudaMemcpyAsync(&st, c->d_status, sizeof(st), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "status read");
  if (st & JNE_DEV_BAD_ARGS) return fail(c, JNE_ERR_ARG, "a kernel rejected its arguments");
  if (st & JNE_DEV_NOT_SPD) return fail(c, JNE_ERR_NUMERIC, "S11 not positive definite for some run (NaN written)");
  return JNE_OK;
}

// Runs per device batch: moment records + outputs of a batch stay well inside the budget.
inline int64_t batch_runs(const jne_context* c, int dim, int k_total) {
  const size_t per_run = sizeof(double) * ((size_t)jne_record_slots(dim) + (size_t)k_total);
  const unsigned long long avail = c->budget > c->in_use ? c->budget / 2 : 0;
  int64_t n = (int64_t)(avail / per_run);
  if (n > (1 << 22)) n = 1 << 22;
  return n;
}

// Per-chunk time constants of the mixed kernel for a (steps, chunk) pair: the
// means of y and y^2 over each chunk's columns, exact (integer sums in long
// double) and rounded once.
inline void fill_chunk_table(int steps, int chunk, jne_chunk_time* dst) {
  const int nch = (steps + chunk - 1) / chunk;
  const long double T = steps;
  auto sq = [](long double n) { return n * (n + 1.0L) * (2.0L * n + 1.0L) / 6.0L; };
  for (int ch = 0; ch < nch; ch++) {
    const long long c0 = (long long)ch * chunk, lc = std::min<long long>(chunk, steps - c0);
    // columns i = c0 .. c0+lc-1 carry y = (i+1)/T
    const long double s1 = (long double)lc * (2.0L * c0 + lc + 1.0L) / 2.0L;
    const long double s2 = sq((long double)(c0 + lc)) - sq((long double)c0);
    const long double yb = s1 / (T * lc), y2b = s2 / (T * T * lc);
    const float ybh = (float)yb, y2h = (float)y2b;
    dst[ch] = {ybh, (float)(yb - ybh), y2h, (float)(y2b - y2h), (float)lc, 1.0f / (float)lc, 0.f, 0.f};
  }
}

// The kernel a request runs on.  Mixed-precision requests on paths shorter
// than JNE_MIXED_MIN_STEPS use the FP64 kernel: with so few chunks the FP32
// part is most of every moment (errors up to ~1e-4 at T = 16, dim 12), and
// such paths are cheap in FP64 anyway.
inline int kernel_precision(int precision, int steps) {
  return (precision == JNE_PREC_MIXED && steps >= JNE_MIXED_MIN_STEPS) ? JNE_PREC_MIXED : JNE_PREC_FP64;
}

inline int finalize(jne_context* c, const jne_finalize_args& f, cudaStream_t st);

// The finalize argument block of n runs of one request (records in mom);
// device status bits go to `status` (null: the context's status word).
inline jne_finalize_args finalize_args(jne_context* c, int model, int dim, int steps, int n, const double* mom,
                                       double* d_out, unsigned int* status = nullptr) {
  jne_finalize_args f{};
  f.model = model;
  f.dim = dim;
  f.steps = steps;
  f.n_runs = n;
  f.zscale = 1.0 / std::sqrt((double)steps);
  f.ts = time_sums(steps);
  f.mom = mom;
  f.mom_ld = n;
  f.out = d_out;
  f.status = status ? status : c->d_status;
  return f;
}

// Moments of runs [seed_first, seed_first + n) into mom (leading dim n).  With
// `fin`, the runs' eigenvalues are also produced on st: inside the mixed
// kernel (each warp finalizes its runs), or by a finalize launch after the
// FP64 kernel.  The accumulation's status bits go to `status` (null: the
// context's status word).
inline int accumulate(jne_context* c, int model, int dim, int steps, uint32_t key0, uint32_t key1, uint32_t seed_first,
                      int n, int precision, const double* d_ext, double* mom, cudaStream_t st,
                      const jne_finalize_args* fin = nullptr, unsigned int* status = nullptr) {
  precision = kernel_precision(precision, steps);
  jne_accum_args a{};
  a.model = model;
  a.dim = dim;
  a.steps = steps;
  a.n_runs = n;
  a.seed_first = seed_first;
  a.key0 = key0;
  a.key1 = key1;
  a.chunk = chunk_for(c, dim, steps);
  a.ext = d_ext;
  a.ext_inv_scale = std::sqrt((double)steps);
  a.mom = mom;
  a.mom_ld = n;
  a.status = status ? status : c->d_status;
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
    {
      ProfScope ps(c, JNE_KERNEL_ACCUM_FP64, st);
      e = jne_launch_accum_f64(a, c->d_ent, nent, c->sms, st);
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "accumulation launch");
    return fin ? finalize(c, *fin, st) : JNE_OK;
  } else {
    // per-chunk time means, exact (integer sums) then rounded once
    const int nch = (steps + a.chunk - 1) / a.chunk;
    if (c->ctab_steps != steps || c->ctab_chunk != a.chunk) {
    int rc = ensure(c, &c->d_ctab, &c->ctab_cap, (size_t)nch, "chunk table");
    if (rc) return rc;
    c->h_ctab.resize(nch);
    fill_chunk_table(steps, a.chunk, c->h_ctab.data());
    e = cudaMemcpyAsync(c->d_ctab, c->h_ctab.data(), sizeof(jne_chunk_time) * nch, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "chunk table upload");
    c->ctab_steps = steps;
    c->ctab_chunk = a.chunk;
    }
    a.chunk_tab = c->d_ctab;
    const jne_shape shape = shape_for(c, dim, steps);
    a.blocks_per_sm = d_ext ? 4 : shape.blocks_per_sm;
    a.pack = d_ext || shape.pack ? 0 : -1;
    // warps take runs from a counter, so blocks that start late (behind a
    // concurrent finalize) take fewer runs instead of leaving a tail
    e = cudaMemsetAsync(c->d_next_run, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return cuda_fail(c, e, "work counter reset");
    a.next_run = c->d_next_run;
    if (fin) {
      const size_t nb = ((size_t)n + 31) / 32;
      int rc = ensure(c, &c->d_batch, &c->batch_cap, nb, "batch counts");
      if (rc) return rc;
      e = cudaMemsetAsync(c->d_batch, 0, sizeof(unsigned int) * nb, st);
      if (e != cudaSuccess) return cuda_fail(c, e, "batch count reset");
      a.batch_done = c->d_batch;
    }
    ProfScope ps(c, JNE_KERNEL_ACCUM_MIXED, st);
    e = jne_launch_accum_mixed(a, fin, c->sms, st);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "accumulation launch");
  return JNE_OK;
}

inline int finalize(jne_context* c, const jne_finalize_args& f, cudaStream_t st) {
  ProfScope ps(c, JNE_KERNEL_FINALIZE, st);
  cudaError_t e = jne_launch_finalize(f, c->sms, st);
  if (e != cudaSuccess) return cuda_fail(c, e, "finalize launch");
  return JNE_OK;
}

inline int finalize(jne_context* c, int model, int dim, int steps, int n, const double* mom, double* d_out,
                    cudaStream_t st) {
  return finalize(c, finalize_args(c, model, dim, steps, n, mom, d_out), st);
}

inline int check_common(jne_context* c, int model, int dim, int steps, int64_t n_runs, int precision) {
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
inline int drain(jne_context* c) {
  cudaError_t e = cudaStreamSynchronize(c->fin_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "drain");
}

inline int clear_status(jne_context* c, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(c->d_status, 0, sizeof(unsigned int), st);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "status reset");
}

// The caller's stream `user` -> the context's accumulation stream (so work the
// caller enqueued earlier comes first).
inline int join_in(jne_context* c, cudaStream_t user) {
  if (user == c->stream) return JNE_OK;
  cudaError_t e = cudaEventRecord(c->ev_in, user);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_in, 0);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "stream join");
}

// The last finalize (record buffer `last`, -1 for none) -> the caller's stream,
// so later work on `user` sees the results.
inline int join_out(jne_context* c, cudaStream_t user, int last) {
  if (last < 0) return JNE_OK;
  cudaError_t e = cudaStreamWaitEvent(user, c->ev_fin[last], 0);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "stream join");
}

// Asynchronous seeded batch of one request.  Batch b uses record buffer b % 2.
// Mixed precision: the accumulation kernel finalizes its own runs, on
// c->stream.  FP64: the finalize of a batch runs on c->fin_stream beside the
// next batch's accumulation.  Events order the buffer reuse; *last receives
// the record buffer of the final batch (its ev_fin marks the results).  Device
// status bits go to `status` (null: the context's status word).
inline int enqueue_seeded(jne_context* c, int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first,
                          int64_t n_runs, int precision, double* out_device, int* last,
                          unsigned int* status = nullptr) {
  const int k = jne_eigen_count(model, dim);
  uint32_t k0, k1;
  stream_key(base_seed, dim, &k0, &k1);
  const int64_t per = batch_runs(c, dim, 0) / 2;  // two record buffers in flight
  if (per < 1) return fail(c, JNE_ERR_BUDGET, "budget too small for one run");
  const bool fused = kernel_precision(precision, steps) == JNE_PREC_MIXED;
  cudaStream_t st = c->stream;
  cudaError_t e = cudaSuccess;
  int rc;
  for (int64_t done = 0; done < n_runs; done += per) {
    const int n = (int)std::min<int64_t>(per, n_runs - done);
    const int b = (int)(c->batch_seq++ & 1);
    if (c->fin_pending[b] && (e = cudaStreamWaitEvent(st, c->ev_fin[b], 0)) != cudaSuccess)
      return cuda_fail(c, e, "stream wait");
    if ((rc = ensure(c, &c->d_momb[b], &c->momb_cap[b], (size_t)n * jne_record_slots(dim), "moment buffer")))
      return rc;
    const jne_finalize_args fa =
        finalize_args(c, model, dim, steps, n, c->d_momb[b], out_device + (size_t)done * k, status);
    if (fused) {
      if ((rc = accumulate(c, model, dim, steps, k0, k1, seed_first + (uint32_t)done, n, precision, nullptr,
                           c->d_momb[b], st, &fa, status)))
        return rc;
      if ((e = cudaEventRecord(c->ev_fin[b], st)) != cudaSuccess) return cuda_fail(c, e, "event record");
    } else {
      if ((rc = accumulate(c, model, dim, steps, k0, k1, seed_first + (uint32_t)done, n, precision, nullptr,
                           c->d_momb[b], st, nullptr, status)))
        return rc;
      if ((e = cudaEventRecord(c->ev_acc[b], st)) != cudaSuccess ||
          (e = cudaStreamWaitEvent(c->fin_stream, c->ev_acc[b], 0)) != cudaSuccess)
        return cuda_fail(c, e, "stream order");
      if ((rc = finalize(c, fa, c->fin_stream))) return rc;
      if ((e = cudaEventRecord(c->ev_fin[b], c->fin_stream)) != cudaSuccess) return cuda_fail(c, e, "event record");
    }
    c->fin_pending[b] = true;
    *last = b;
  }
  return JNE_OK;
}

// A ragged batch (jne_batch.cu): request i's device status bits go to
// req_status[i] when req_status is given, else to the context's status word.
int run_batch(jne_context* c, const jne_request* reqs, int n_req, double* const* outs, cudaStream_t user,
              unsigned int* const* req_status);

// Converts a word of JNE_DEV_* bits into a status code.
inline int status_code(unsigned int bits) {
  if (bits & JNE_DEV_BAD_ARGS) return JNE_ERR_ARG;
  if (bits & JNE_DEV_NOT_SPD) return JNE_ERR_NUMERIC;
  return JNE_OK;
}

}  // namespace jne_detail
