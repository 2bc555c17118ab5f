// jne_batch.cu -- ragged batches of requests in one persistent launch, and
// plans: a ragged batch captured once into a CUDA graph and replayed.
//
// A batch mixes (model, dim, steps, seeds, size) freely.  Mixed-precision
// requests with steps >= JNE_MIXED_MIN_STEPS go through k_accum_mixed_ragged
// (one launch; warps pull runs of the flattened batch from a global counter and
// finalize every completed batch of 32 runs); the others run through the
// per-request path.  The batch
// loop of the reference CLI (src/main.rs:85-136: every model of every dim) is
// one such batch.
#include <cstring>
#include <vector>

#include "jne_context.h"

using namespace jne_detail;

namespace {

// A contiguous run range of one request, as placed in a ragged launch.
struct Piece {
  int req;
  int64_t offset, n;
};

bool ragged_ok(const jne_request& r) { return kernel_precision(r.precision, r.steps) == JNE_PREC_MIXED; }

int check_request(jne_context* c, const jne_request& r, double* out) {
  int rc = check_common(c, r.model, r.dim, r.steps, r.n_runs, r.precision);
  if (rc) return rc;
  if (r.n_runs > 0 && !out) return fail(c, JNE_ERR_ARG, "null output buffer");
  if ((uint64_t)r.seed_first + (uint64_t)r.n_runs > 0x100000000ull) return fail(c, JNE_ERR_ARG, "seed range exceeds u32");
  return JNE_OK;
}

// Host side of one ragged launch: device descriptors (request table and chunk
// tables) for `pieces`, record slots laid out back to back from `mom`.  Each
// piece reports its device status to its request's word (req_status[req]), or
// to the context's word when req_status is null.
void describe(jne_context* c, const jne_request* reqs, double* const* outs, const std::vector<Piece>& pieces,
              double* mom, const jne_chunk_time* d_tab, jne_ragged_req* hr, jne_chunk_time* ht, long long* total,
              size_t* n_tab, unsigned int* const* req_status = nullptr) {
  long long first = 0;
  size_t moff = 0, toff = 0;
  for (size_t i = 0; i < pieces.size(); i++) {
    const Piece& p = pieces[i];
    const jne_request& r = reqs[p.req];
    jne_ragged_req& d = hr[i];
    std::memset(&d, 0, sizeof d);
    const int chunk = chunk_for(c, r.dim, r.steps);
    const int nch = (r.steps + chunk - 1) / chunk;
    uint32_t k0, k1;
    stream_key(r.base_seed, r.dim, &k0, &k1);
    d.acc.model = r.model;
    d.acc.dim = r.dim;
    d.acc.steps = r.steps;
    d.acc.n_runs = (int)p.n;
    d.acc.seed_first = r.seed_first + (uint32_t)p.offset;
    d.acc.key0 = k0;
    d.acc.key1 = k1;
    d.acc.chunk = chunk;
    d.acc.chunk_tab = d_tab + toff;
    d.acc.mom = mom + moff;
    d.acc.mom_ld = p.n;
    unsigned int* status = req_status ? req_status[p.req] : c->d_status;
    d.acc.status = status;
    d.fin.model = r.model;
    d.fin.dim = r.dim;
    d.fin.steps = r.steps;
    d.fin.n_runs = (int)p.n;
    d.fin.zscale = 1.0 / std::sqrt((double)r.steps);
    d.fin.ts = time_sums(r.steps);
    d.fin.mom = mom + moff;
    d.fin.mom_ld = p.n;
    d.fin.out = outs[p.req] + (size_t)p.offset * jne_eigen_count(r.model, r.dim);
    d.fin.status = status;
    d.first = first;
    fill_chunk_table(r.steps, chunk, ht + toff);
    first += jne_units(r.dim, p.n);  // the kernel's items are units (packed pairs for small dims)
    moff += (size_t)p.n * jne_record_slots(r.dim);
    toff += (size_t)nch;
  }
  *total = first;
  *n_tab = toff;
}

// Splits the ragged-capable requests into launches whose records fit `cap`
// doubles (a request larger than that is cut into run ranges).
std::vector<std::vector<Piece>> plan_launches(const jne_request* reqs, const std::vector<int>& idx, size_t cap) {
  std::vector<std::vector<Piece>> out(1);
  size_t used = 0;
  for (int i : idx) {
    const size_t rec = (size_t)jne_record_slots(reqs[i].dim);
    int64_t off = 0;
    while (off < reqs[i].n_runs) {
      size_t room = cap > used ? (cap - used) / rec : 0;
      if (room == 0) {
        out.emplace_back();
        used = 0;
        room = cap / rec;
      }
      const int64_t n = std::min<int64_t>(reqs[i].n_runs - off, (int64_t)std::min<size_t>(room, 1u << 30));
      out.back().push_back({i, off, n});
      used += (size_t)n * rec;
      off += n;
    }
  }
  if (out.back().empty()) out.pop_back();
  return out;
}

// Items of a ragged launch: units, i.e. runs, or pairs of runs for packed dims.
long long total_units(const jne_request* reqs, const std::vector<Piece>& pieces) {
  long long n = 0;
  for (const Piece& p : pieces) n += jne_units(reqs[p.req].dim, p.n);
  return n;
}

size_t chunks_of(jne_context* c, const jne_request* reqs, const std::vector<Piece>& pieces) {
  size_t n = 0;
  for (const Piece& p : pieces) {
    const int chunk = chunk_for(c, reqs[p.req].dim, reqs[p.req].steps);
    n += (size_t)((reqs[p.req].steps + chunk - 1) / chunk);
  }
  return n;
}

template <typename T>
int ensure_pinned(jne_context* c, T** p, size_t* cap, size_t n) {
  if (n <= *cap) return JNE_OK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMallocHost((void**)p, n * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(c, e, "pinned staging");
  *cap = n;
  return JNE_OK;
}

}  // namespace

struct jne_plan {
  jne_context* ctx = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double* d_mom = nullptr;
  jne_ragged_req* d_reqs = nullptr;
  jne_chunk_time* d_tab = nullptr;
  unsigned long long* d_counter = nullptr;
  unsigned int* d_bdone = nullptr;
  unsigned long long bytes = 0;
  cudaEvent_t done = nullptr;
};

int jne_detail::run_batch(jne_context* c, const jne_request* reqs, int n_req, double* const* outs, cudaStream_t user,
                          unsigned int* const* req_status) {
  if (!c) return JNE_ERR_ARG;
  if (n_req < 0 || (n_req > 0 && (!reqs || !outs))) return fail(c, JNE_ERR_ARG, "null request list");
  int rc;
  for (int i = 0; i < n_req; i++)
    if ((rc = check_request(c, reqs[i], outs[i]))) return rc;
  if ((rc = join_in(c, user))) return rc;
  int last = -1;
  bool seeded = false;  // some request finalizes on the context's second stream
  std::vector<int> ragged;
  for (int i = 0; i < n_req; i++) {
    if (reqs[i].n_runs == 0) continue;
    if (ragged_ok(reqs[i])) {
      ragged.push_back(i);
    } else if (seeded = true, (rc = enqueue_seeded(c, reqs[i].model, reqs[i].dim, reqs[i].steps, reqs[i].base_seed,
                                    reqs[i].seed_first, reqs[i].n_runs, reqs[i].precision, outs[i], &last,
                                    req_status ? req_status[i] : nullptr))) {
      return rc;
    }
  }
  // records of one launch use at most a quarter of the budget (two in flight)
  const size_t cap = (size_t)(c->budget / 4 / sizeof(double));
  if (!ragged.empty() && cap < (size_t)jne_record_slots(JNE_MAX_DIM))
    return fail(c, JNE_ERR_BUDGET, "budget too small for one run");
  cudaStream_t st = c->stream;
  cudaError_t e;
  for (const std::vector<Piece>& pieces : plan_launches(reqs, ragged, cap)) {
    const int b = (int)(c->batch_seq++ & 1);
    // the previous launch that used slot b must be done before its buffers are rewritten
    if (c->fin_pending[b] && (e = cudaEventSynchronize(c->ev_fin[b])) != cudaSuccess)
      return cuda_fail(c, e, "slot wait");
    size_t slots = 0;
    for (const Piece& p : pieces) slots += (size_t)p.n * jne_record_slots(reqs[p.req].dim);
    const size_t ntab = chunks_of(c, reqs, pieces);
    if ((rc = ensure(c, &c->d_momb[b], &c->momb_cap[b], slots, "moment buffer")) ||
        (rc = ensure(c, &c->d_reqs[b], &c->reqs_cap[b], pieces.size(), "request table")) ||
        (rc = ensure(c, &c->d_rtab[b], &c->rtab_cap[b], ntab, "chunk tables")) ||
        (rc = ensure(c, &c->d_counter[b], &c->counter_cap[b], 1, "work counter")) ||
        (rc = ensure(c, &c->d_bdone[b], &c->bdone_cap[b], ((size_t)total_units(reqs, pieces) + 31) / 32,
                     "batch counts")) ||
        (rc = ensure_pinned(c, &c->h_reqs[b], &c->h_reqs_cap[b], pieces.size())) ||
        (rc = ensure_pinned(c, &c->h_rtab[b], &c->h_rtab_cap[b], ntab)))
      return rc;
    long long total = 0;
    size_t nt = 0;
    describe(c, reqs, outs, pieces, c->d_momb[b], c->d_rtab[b], c->h_reqs[b], c->h_rtab[b], &total, &nt,
             req_status);
    if ((e = cudaMemcpyAsync(c->d_reqs[b], c->h_reqs[b], sizeof(jne_ragged_req) * pieces.size(),
                             cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(c->d_rtab[b], c->h_rtab[b], sizeof(jne_chunk_time) * nt, cudaMemcpyHostToDevice, st)) !=
            cudaSuccess ||
        (e = cudaMemsetAsync(c->d_counter[b], 0, sizeof(unsigned long long), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(c->d_bdone[b], 0, sizeof(unsigned int) * ((total + 31) / 32), st)) != cudaSuccess)
      return cuda_fail(c, e, "batch upload");
    {
      ProfScope ps(c, JNE_KERNEL_ACCUM_MIXED, st);
      e = jne_launch_accum_mixed_ragged(c->d_reqs[b], (int)pieces.size(), total, c->d_counter[b], c->d_bdone[b],
                                        c->sms, st);
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "ragged launch");
    if ((e = cudaEventRecord(c->ev_fin[b], st)) != cudaSuccess) return cuda_fail(c, e, "event record");
    c->fin_pending[b] = true;
    last = b;
  }
  // the caller's stream waits for both streams' work: the ragged launches (the
  // last one's event) and the FP64-path finalizes queued on the second stream
  if (seeded && ((e = cudaEventRecord(c->ev_join, c->fin_stream)) != cudaSuccess ||
                 (e = cudaStreamWaitEvent(user, c->ev_join, 0)) != cudaSuccess))
    return cuda_fail(c, e, "stream join");
  return join_out(c, user, last);
}

extern "C" {

int jne_run_batch(jne_context* c, const jne_request* reqs, int n_req, double* const* outs, void* stream) {
  if (!c) return JNE_ERR_ARG;
  return run_batch(c, reqs, n_req, outs, stream ? (cudaStream_t)stream : c->stream, nullptr);
}

int jne_run_batch_status(jne_context* c, const jne_request* reqs, int n_req, double* const* outs, int* status_out,
                         void* stream) {
  if (!c) return JNE_ERR_ARG;
  if (n_req < 0 || (n_req > 0 && !status_out)) return fail(c, JNE_ERR_ARG, "null status list");
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, JNE_ERR_CUDA, "cudaSetDevice failed");
  if (n_req == 0) return JNE_OK;
  int rc = ensure(c, &c->d_req_status, &c->req_status_cap, (size_t)n_req, "request status words");
  if (rc) return rc;
  cudaStream_t user = stream ? (cudaStream_t)stream : c->stream;
  cudaError_t e = cudaMemsetAsync(c->d_req_status, 0, sizeof(unsigned int) * n_req, user);
  if (e != cudaSuccess) return cuda_fail(c, e, "status reset");
  std::vector<unsigned int*> words((size_t)n_req);
  for (int i = 0; i < n_req; i++) words[(size_t)i] = c->d_req_status + i;
  if ((rc = run_batch(c, reqs, n_req, outs, user, words.data()))) return rc;
  std::vector<unsigned int> bits((size_t)n_req);
  e = cudaMemcpyAsync(bits.data(), c->d_req_status, sizeof(unsigned int) * n_req, cudaMemcpyDeviceToHost, user);
  if (e == cudaSuccess) e = cudaStreamSynchronize(user);
  if (e != cudaSuccess) return cuda_fail(c, e, "batch status");
  int worst = JNE_OK;
  for (int i = 0; i < n_req; i++) {
    status_out[i] = status_code(bits[(size_t)i]);
    if (status_out[i] != JNE_OK && worst == JNE_OK) worst = status_out[i];
  }
  if (worst != JNE_OK) return fail(c, worst, "some requests of the batch failed (see their status)");
  return JNE_OK;
}

namespace {

// One round of a streamed batch in flight: its parts (request, first seed,
// runs, offset of its results in the slot's buffers; with packed records, the
// offset and length of their bytes).
struct SinkPart {
  int req;
  uint32_t seed_first;
  int64_t n, off;
  int64_t boff, nbytes;
};
struct SinkRound {
  std::vector<SinkPart> parts;
  bool busy = false;
};

// Hands a finished round's results to the sink, in request order.
int deliver(jne_context* c, const jne_request* reqs, const jne_sink* sink, int s, SinkRound& rd, int* worst) {
  if (!rd.busy) return JNE_OK;
  rd.busy = false;
  cudaError_t e = cudaEventSynchronize(c->ev_sink[s]);
  if (e != cudaSuccess) return cuda_fail(c, e, "sink round");
  for (size_t p = 0; p < rd.parts.size(); p++) {
    const SinkPart& q = rd.parts[p];
    const int st = status_code(c->h_sink_st[s][p]);
    if (st != JNE_OK && *worst == JNE_OK) *worst = st;
    const int k = jne_eigen_count(reqs[q.req].model, reqs[q.req].dim);
    const int rc = sink->write_records
                       ? sink->write_records(sink->user, q.req, q.seed_first, q.n, k, c->h_pack[s] + q.boff,
                                             q.nbytes, st)
                       : sink->write(sink->user, q.req, q.seed_first, q.n, k, c->h_sink[s] + q.off, st);
    if (rc) return fail(c, rc, "the sink stopped the batch");
  }
  return JNE_OK;
}

}  // namespace

int jne_run_batch_sink(jne_context* c, const jne_request* reqs, int n_req, const jne_sink* sink) {
  if (!c) return JNE_ERR_ARG;
  if (!sink || (!sink->write && !sink->write_records) || n_req < 0 || (n_req > 0 && !reqs))
    return fail(c, JNE_ERR_ARG, "null sink or requests");
  const bool packed = sink->write_records != nullptr;  // records packed on the GPU
  int rc;
  for (int i = 0; i < n_req; i++) {
    if ((rc = check_common(c, reqs[i].model, reqs[i].dim, reqs[i].steps, reqs[i].n_runs, reqs[i].precision)))
      return rc;
    if ((uint64_t)reqs[i].seed_first + (uint64_t)reqs[i].n_runs > 0x100000000ull)
      return fail(c, JNE_ERR_ARG, "seed range exceeds u32");
  }
  // runs per round: 2^20, or what two slots of results fit in a sixteenth of the budget
  const int64_t cap = std::max<int64_t>(
      1, std::min<int64_t>(1 << 20, (int64_t)(c->budget / 16 / (2 * sizeof(double) * (JNE_MAX_DIM + 1)))));
  for (int s = 0; s < 2; s++)
    if (!c->ev_sink[s] && cudaEventCreateWithFlags(&c->ev_sink[s], cudaEventDisableTiming) != cudaSuccess)
      return fail(c, JNE_ERR_CUDA, "sink events");
  std::vector<int64_t> next((size_t)n_req, 0);
  SinkRound rounds[2];
  int s = 0, worst = JNE_OK;
  rc = JNE_OK;
  cudaStream_t st = c->stream;
  for (;;) {
    // the round: a slice of every request with runs left, in request order
    std::vector<int> act;
    for (int i = 0; i < n_req; i++)
      if (next[(size_t)i] < reqs[i].n_runs) act.push_back(i);
    if (act.empty()) break;
    if ((rc = deliver(c, reqs, sink, s, rounds[s], &worst))) break;  // the slot's previous round
    const int64_t share = std::max<int64_t>(1, cap / (int64_t)act.size());
    SinkRound& rd = rounds[s];
    rd.parts.clear();
    std::vector<jne_request> sub;
    int64_t doubles = 0, bytes = 0;
    for (int i : act) {
      const int64_t n = std::min<int64_t>(share, reqs[i].n_runs - next[(size_t)i]);
      jne_request r = reqs[i];
      r.seed_first = reqs[i].seed_first + (uint32_t)next[(size_t)i];
      r.n_runs = n;
      sub.push_back(r);
      const int k = jne_eigen_count(r.model, r.dim);
      const int64_t nb = packed ? jne_record_bytes(r.seed_first, n, k) : 0;
      rd.parts.push_back({i, r.seed_first, n, doubles, bytes, nb});
      doubles += n * k;
      bytes += (nb + 15) / 16 * 16;  // every part's records start 16-byte aligned
      next[(size_t)i] += n;
    }
    const size_t np = rd.parts.size();
    if ((rc = ensure(c, &c->d_sink[s], &c->d_sink_cap[s], (size_t)doubles, "sink results")) ||
        (rc = ensure(c, &c->d_sink_st[s], &c->d_sink_st_cap[s], np, "sink status words")) ||
        (rc = ensure_pinned(c, &c->h_sink_st[s], &c->h_sink_st_cap[s], np)))
      break;
    if (packed ? ((rc = ensure(c, &c->d_pack[s], &c->d_pack_cap[s], (size_t)bytes, "sink records")) ||
                  (rc = ensure_pinned(c, &c->h_pack[s], &c->h_pack_cap[s], (size_t)bytes)))
               : (rc = ensure_pinned(c, &c->h_sink[s], &c->h_sink_cap[s], (size_t)doubles)))
      break;
    std::vector<double*> outs(np);
    std::vector<unsigned int*> words(np);
    for (size_t p = 0; p < np; p++) {
      outs[p] = c->d_sink[s] + rd.parts[p].off;
      words[p] = c->d_sink_st[s] + p;
    }
    cudaError_t e = cudaMemsetAsync(c->d_sink_st[s], 0, sizeof(unsigned int) * np, st);
    if (e != cudaSuccess) {
      rc = cuda_fail(c, e, "sink status reset");
      break;
    }
    if ((rc = run_batch(c, sub.data(), (int)np, outs.data(), st, words.data()))) break;
    if (packed) {  // each part's records, packed where its results lie
      for (size_t p = 0; p < np && e == cudaSuccess; p++) {
        const SinkPart& q = rd.parts[p];
        e = jne_launch_pack_records(c->d_sink[s] + q.off, c->d_pack[s] + q.boff, q.seed_first, q.n,
                                    jne_eigen_count(sub[p].model, sub[p].dim), c->sms, st);
      }
      if (e != cudaSuccess) {
        rc = cuda_fail(c, e, "sink record packer");
        break;
      }
    }
    if ((e = packed ? cudaMemcpyAsync(c->h_pack[s], c->d_pack[s], (size_t)bytes, cudaMemcpyDeviceToHost, st)
                    : cudaMemcpyAsync(c->h_sink[s], c->d_sink[s], sizeof(double) * doubles, cudaMemcpyDeviceToHost,
                                      st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(c->h_sink_st[s], c->d_sink_st[s], sizeof(unsigned int) * np, cudaMemcpyDeviceToHost,
                             st)) != cudaSuccess ||
        (e = cudaEventRecord(c->ev_sink[s], st)) != cudaSuccess) {
      rc = cuda_fail(c, e, "sink copy");
      break;
    }
    rd.busy = true;
    s ^= 1;
  }
  if (rc == JNE_OK) {  // the last two rounds, oldest first
    rc = deliver(c, reqs, sink, s, rounds[s], &worst);
    if (rc == JNE_OK) rc = deliver(c, reqs, sink, s ^ 1, rounds[s ^ 1], &worst);
  }
  if (rc) {
    cudaStreamSynchronize(st);  // no round left writing into the slots
    cudaStreamSynchronize(c->fin_stream);
    return rc;
  }
  if (worst != JNE_OK) return fail(c, worst, "some runs of the batch had a non-SPD S11 (NaN rows delivered)");
  return JNE_OK;
}

int jne_plan_create(jne_context* c, const jne_request* reqs, int n_req, double* const* outs, jne_plan** out) {
  if (!c) return JNE_ERR_ARG;
  if (!out || n_req < 1 || !reqs || !outs) return fail(c, JNE_ERR_ARG, "plans take a non-empty request list");
  *out = nullptr;
  int rc;
  std::vector<int> idx;
  for (int i = 0; i < n_req; i++) {
    if ((rc = check_request(c, reqs[i], outs[i]))) return rc;
    if (!ragged_ok(reqs[i]))
      return fail(c, JNE_ERR_ARG, "plans take mixed-precision requests with steps >= " +
                                      std::to_string(JNE_MIXED_MIN_STEPS));
    if (reqs[i].n_runs > 0) idx.push_back(i);
  }
  if (idx.empty()) return fail(c, JNE_ERR_ARG, "plans take at least one run");
  std::vector<Piece> pieces;
  size_t slots = 0;
  for (int i : idx) {
    if (reqs[i].n_runs > (1 << 30)) return fail(c, JNE_ERR_ARG, "request too large for a plan");
    pieces.push_back({i, 0, reqs[i].n_runs});
    slots += (size_t)reqs[i].n_runs * jne_record_slots(reqs[i].dim);
  }
  const size_t ntab = chunks_of(c, reqs, pieces);
  const size_t nbatch = ((size_t)total_units(reqs, pieces) + 31) / 32;
  const unsigned long long bytes = slots * sizeof(double) + pieces.size() * sizeof(jne_ragged_req) +
                                   ntab * sizeof(jne_chunk_time) + sizeof(unsigned long long) +
                                   nbatch * sizeof(unsigned int);
  if (c->in_use + bytes > c->budget)
    return fail(c, JNE_ERR_BUDGET, "plan needs " + std::to_string(bytes) + " bytes beyond the budget");
  if ((rc = drain(c))) return rc;
  jne_plan* p = new jne_plan();
  p->ctx = c;
  p->bytes = bytes;
  std::vector<jne_ragged_req> hr(pieces.size());
  std::vector<jne_chunk_time> ht(ntab);
  cudaError_t e = cudaMalloc((void**)&p->d_mom, slots * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&p->d_reqs, pieces.size() * sizeof(jne_ragged_req));
  if (e == cudaSuccess) e = cudaMalloc((void**)&p->d_tab, ntab * sizeof(jne_chunk_time));
  if (e == cudaSuccess) e = cudaMalloc((void**)&p->d_counter, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc((void**)&p->d_bdone, nbatch * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming);
  long long total = 0;
  size_t nt = 0;
  if (e == cudaSuccess) {
    describe(c, reqs, outs, pieces, p->d_mom, p->d_tab, hr.data(), ht.data(), &total, &nt);
    e = cudaMemcpy(p->d_reqs, hr.data(), sizeof(jne_ragged_req) * hr.size(), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemcpy(p->d_tab, ht.data(), sizeof(jne_chunk_time) * nt, cudaMemcpyHostToDevice);
  // capture: counter resets, then the ragged launch (accumulation + fused finalize)
  cudaStream_t st = c->stream;
  if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t ce = cudaMemsetAsync(p->d_counter, 0, sizeof(unsigned long long), st);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(p->d_bdone, 0, nbatch * sizeof(unsigned int), st);
    if (ce == cudaSuccess)
      ce = jne_launch_accum_mixed_ragged(p->d_reqs, (int)pieces.size(), total, p->d_counter, p->d_bdone, c->sms, st);
    e = cudaStreamEndCapture(st, &p->graph);
    if (e == cudaSuccess) e = ce;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
  if (e != cudaSuccess) {
    jne_plan_destroy(p);
    return cuda_fail(c, e, "plan capture");
  }
  c->in_use += bytes;
  *out = p;
  return JNE_OK;
}

int jne_plan_launch(jne_plan* p, void* stream) {
  if (!p) return JNE_ERR_ARG;
  jne_context* c = p->ctx;
  cudaStream_t user = stream ? (cudaStream_t)stream : c->stream;
  int rc = join_in(c, user);
  if (rc) return rc;
  // an earlier replay of this plan must finish before the counter is reset
  cudaError_t e = cudaStreamWaitEvent(c->stream, p->done, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(p->exec, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(p->done, c->stream);
  if (e == cudaSuccess && user != c->stream) e = cudaStreamWaitEvent(user, p->done, 0);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "plan launch");
}

void jne_plan_destroy(jne_plan* p) {
  if (!p) return;
  jne_context* c = p->ctx;
  cudaSetDevice(c->device);
  if (p->done) cudaEventSynchronize(p->done);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->done) cudaEventDestroy(p->done);
  cudaFree(p->d_mom);
  cudaFree(p->d_reqs);
  cudaFree(p->d_tab);
  cudaFree(p->d_counter);
  cudaFree(p->d_bdone);
  if (p->exec) c->in_use -= p->bytes;
  delete p;
}

}  // extern "C"
