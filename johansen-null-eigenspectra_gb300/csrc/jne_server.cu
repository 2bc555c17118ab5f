// jne_server.cu -- a continuous-batching request loop on one context.
//
// Requests (model, dim, steps, runs, seeds) arrive at any time from any thread.
// A worker thread admits them while their device output buffers fit the
// context's memory budget, and runs the GPU in iterations: each iteration is one
// ragged launch (jne_run_batch) over a slice of every active request, so
// requests that arrive while others are running join at the next iteration
// boundary and share the GPU with them.  Two iterations are in flight.  A
// finished request's eigenvalues are copied to host memory, handed to a writer
// thread that streams them to an EIGENVALS_V6 file (when a data directory is
// given), and reported with submit / start / finish times.  Each run's result
// does not depend on its neighbours, so a request gives the same values alone
// and in any mix.
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "jne_context.h"

using namespace jne_detail;

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  uint64_t id = 0;
  jne_request req{};
  int k = 0;
  double* d_out = nullptr;  // n_runs x k on the device
  size_t bytes = 0;
  int64_t next = 0;         // next run to schedule
  int64_t done = 0;         // runs whose iteration has completed
  double submit_s = 0, start_s = -1, finish_s = 0;
  int status = JNE_OK;
  bool admitted = false;     // its output buffer counts against the budget
  bool writing = false;      // queued for or being written by the writer thread
  std::vector<double> host;  // results, once finished
};

// One ragged launch in flight.  Each part (a slice of one job) reports its
// device status to its own word of d_status, so a failing request marks only
// itself, and a word is read only once its iteration's event has passed.
struct Iteration {
  cudaEvent_t ev = nullptr;
  std::vector<std::pair<Job*, int64_t>> parts;  // job, runs it advanced
  bool busy = false;
  unsigned int* d_status = nullptr;  // one word per part
  size_t status_cap = 0;
  std::vector<unsigned int> h_status;
};

}  // namespace

struct jne_server {
  jne_context* ctx = nullptr;
  std::string data_dir;
  long long iter_work = 0;  // runs x steps per iteration
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv, cv_done;
  std::deque<Job*> pending;
  std::vector<Job*> active;
  std::map<uint64_t, Job*> finished;  // awaiting jne_server_fetch
  std::deque<jne_completion> completions;
  uint64_t next_id = 1;
  bool stopping = false;
  unsigned long long admitted_bytes = 0;
  std::thread worker, writer;
  std::deque<Job*> to_write;
  std::condition_variable cv_write;
  bool writer_stop = false;
  Iteration it[2];
  int it_next = 0;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Device bytes the server may hold for outputs: half the budget less a small
// margin; the records of the two ragged launches in flight take at most a
// quarter each, and the request tables the margin.
unsigned long long output_room(const jne_server* s) {
  const unsigned long long b = s->ctx->budget;
  return b / 2 - b / 64;
}

void finish_job(jne_server* s, Job* j, int status) {
  j->status = status;
  if (status == JNE_OK && j->req.n_runs > 0) {
    j->host.resize((size_t)j->req.n_runs * j->k);
    if (cudaMemcpy(j->host.data(), j->d_out, j->bytes, cudaMemcpyDeviceToHost) != cudaSuccess) j->status = JNE_ERR_CUDA;
  }
  if (j->d_out) cudaFreeAsync(j->d_out, s->ctx->stream);  // stream-ordered: no device-wide sync
  j->d_out = nullptr;
  j->finish_s = s->now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (j->admitted) {
    s->ctx->in_use -= j->bytes;
    s->admitted_bytes -= j->bytes;
    j->admitted = false;
  }
  s->finished[j->id] = j;
  s->completions.push_back({j->id, j->status, j->submit_s, j->start_s < 0 ? j->finish_s : j->start_s, j->finish_s,
                            j->req.n_runs});
  if (!s->data_dir.empty() && j->status == JNE_OK) {
    j->writing = true;
    s->to_write.push_back(j);
    s->cv_write.notify_one();
  }
  s->cv_done.notify_all();
}

// Completes the iteration in slot `i` (waits for its event) and retires jobs;
// each job takes the status of its own part only.
void retire(jne_server* s, int i) {
  Iteration& itr = s->it[i];
  if (!itr.busy) return;
  const size_t np = itr.parts.size();
  itr.h_status.assign(np, 0u);
  cudaError_t e = cudaEventSynchronize(itr.ev);
  if (e == cudaSuccess && np)
    e = cudaMemcpy(itr.h_status.data(), itr.d_status, sizeof(unsigned int) * np, cudaMemcpyDeviceToHost);
  for (size_t k = 0; k < np; k++) {
    auto& p = itr.parts[k];
    Job* j = p.first;
    j->done += p.second;
    const int st = e != cudaSuccess ? JNE_ERR_CUDA : status_code(itr.h_status[k]);
    if (st != JNE_OK && j->status == JNE_OK) j->status = st;
    if (j->done == j->req.n_runs) {
      {
        std::lock_guard<std::mutex> lk(s->mu);
        for (size_t a = 0; a < s->active.size(); a++)
          if (s->active[a] == j) {
            s->active.erase(s->active.begin() + a);
            break;
          }
      }
      finish_job(s, j, j->status);
    }
  }
  itr.parts.clear();
  itr.busy = false;
}

void worker_loop(jne_server* s) {
  jne_context* c = s->ctx;
  cudaSetDevice(c->device);
  for (;;) {
    // admission: FIFO while the outputs fit
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->active.empty() && s->pending.empty() && !s->it[0].busy && !s->it[1].busy) {
        if (s->stopping) return;
        s->cv.wait_for(lk, std::chrono::milliseconds(50));
        continue;
      }
      while (!s->pending.empty()) {
        Job* j = s->pending.front();
        if (j->bytes > output_room(s) || j->req.n_runs == 0) {  // can never fit, or nothing to do
          s->pending.pop_front();
          lk.unlock();
          finish_job(s, j, j->req.n_runs == 0 ? JNE_OK : JNE_ERR_BUDGET);
          lk.lock();
          continue;
        }
        if (s->admitted_bytes + j->bytes > output_room(s)) break;  // wait for running requests to finish
        if (cudaMallocAsync((void**)&j->d_out, j->bytes, c->stream) != cudaSuccess) {
          s->pending.pop_front();
          lk.unlock();
          finish_job(s, j, JNE_ERR_CUDA);
          lk.lock();
          continue;
        }
        s->pending.pop_front();
        s->admitted_bytes += j->bytes;
        c->in_use += j->bytes;
        j->admitted = true;
        j->start_s = -1;
        s->active.push_back(j);
      }
    }
    // one iteration: a slice of every active request that still has runs to schedule
    const int slot = s->it_next;
    retire(s, slot);  // at most two iterations in flight
    std::vector<Job*> act;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (Job* j : s->active)
        if (j->next < j->req.n_runs) act.push_back(j);
    }
    if (act.empty()) {
      retire(s, 1 - slot);
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->pending.empty()) s->cv.wait_for(lk, std::chrono::milliseconds(2));
      continue;
    }
    const long long share = std::max<long long>(1, s->iter_work / (long long)act.size());
    std::vector<jne_request> reqs;
    std::vector<double*> outs;
    Iteration& itr = s->it[slot];
    // the iteration's status words, zeroed on the stream ahead of its launches
    int rc = ensure(c, &itr.d_status, &itr.status_cap, std::max<size_t>(act.size(), 256), "server status words");
    if (rc == JNE_OK && cudaMemsetAsync(itr.d_status, 0, sizeof(unsigned int) * act.size(), c->stream) != cudaSuccess)
      rc = JNE_ERR_CUDA;
    std::vector<unsigned int*> words(act.size());
    for (size_t k = 0; k < act.size(); k++) words[k] = itr.d_status + k;
    for (Job* j : act) {
      const int64_t n = std::max<int64_t>(1, std::min<int64_t>(j->req.n_runs - j->next, share / j->req.steps));
      jne_request r = j->req;
      r.seed_first = j->req.seed_first + (uint32_t)j->next;
      r.n_runs = n;
      reqs.push_back(r);
      outs.push_back(j->d_out + (size_t)j->next * j->k);
      if (j->start_s < 0) j->start_s = s->now();
      j->next += n;
      itr.parts.push_back({j, n});
    }
    // a failed slice still retires (with the error) through the iteration's event
    if (rc == JNE_OK) rc = run_batch(c, reqs.data(), (int)reqs.size(), outs.data(), c->stream, words.data());
    if (rc != JNE_OK)
      for (auto& p : itr.parts) p.first->status = rc;
    cudaEventRecord(itr.ev, c->stream);
    itr.busy = true;
    s->it_next = 1 - slot;
  }
}

void writer_loop(jne_server* s) {
  for (;;) {
    Job* j;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_write.wait(lk, [&] { return s->writer_stop || !s->to_write.empty(); });
      if (s->to_write.empty()) return;
      j = s->to_write.front();
      s->to_write.pop_front();
    }
    char name[512];
    std::snprintf(name, sizeof name, "%s/request%llu_model%d_dim%d_steps%d.dat", s->data_dir.c_str(),
                  (unsigned long long)j->id, j->req.model, j->req.dim, j->req.steps);
    jne_dat_writer* w = nullptr;
    if (jne_dat_open(name, j->req.model, j->req.dim, (uint32_t)j->req.steps, &w, nullptr) == JNE_OK) {
      std::vector<uint32_t> seeds((size_t)j->req.n_runs);
      for (int64_t r = 0; r < j->req.n_runs; r++) seeds[(size_t)r] = j->req.seed_first + (uint32_t)r;
      if (jne_dat_append(w, seeds.data(), j->host.data(), j->req.n_runs, j->k) == JNE_OK)
        jne_dat_finish(w);
      else
        jne_dat_abandon(w);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    j->writing = false;
    s->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

int jne_server_open(jne_context* c, const char* data_dir, long long iter_work, jne_server** out) {
  if (!c || !out) return JNE_ERR_ARG;
  *out = nullptr;
  int rc = drain(c);
  if (rc) return rc;
  jne_server* s = new jne_server();
  s->ctx = c;
  s->data_dir = data_dir ? data_dir : "";
  s->iter_work = iter_work > 0 ? iter_work : 2000000000LL;  // ~2e9 step-runs: ~0.1-0.6 s at dim 12
  s->t0 = Clock::now();
  for (int i = 0; i < 2; i++)
    if (cudaEventCreateWithFlags(&s->it[i].ev, cudaEventDisableTiming) != cudaSuccess) {
      delete s;
      return fail(c, JNE_ERR_CUDA, "server events");
    }
  try {
    s->worker = std::thread(worker_loop, s);
    if (!s->data_dir.empty()) s->writer = std::thread(writer_loop, s);
  } catch (const std::system_error&) {  // no exception leaves the C ABI
    jne_server_close(s);                 // stops whichever thread started
    return fail(c, JNE_ERR_IO, "cannot start the server's threads");
  }
  *out = s;
  return JNE_OK;
}

int jne_server_submit(jne_server* s, const jne_request* r, uint64_t* id) {
  if (!s || !r) return JNE_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return JNE_ERR_ARG;  // closing
  }
  if (jne_eigen_count(r->model, r->dim) < 0 || r->dim > JNE_MAX_DIM || r->steps < 1 || r->n_runs < 0 ||
      (r->precision != JNE_PREC_FP64 && r->precision != JNE_PREC_MIXED) ||
      (uint64_t)r->seed_first + (uint64_t)r->n_runs > 0x100000000ull)
    return JNE_ERR_ARG;
  Job* j = new Job();
  j->req = *r;
  j->k = jne_eigen_count(r->model, r->dim);
  j->bytes = (size_t)r->n_runs * j->k * sizeof(double);
  std::lock_guard<std::mutex> lk(s->mu);
  j->id = s->next_id++;
  j->submit_s = s->now();
  if (id) *id = j->id;
  s->pending.push_back(j);
  s->cv.notify_one();
  return JNE_OK;
}

int jne_server_wait(jne_server* s, jne_completion* out, int max, int timeout_ms, int* n) {
  if (!s || !n || (max > 0 && !out)) return JNE_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->completions.empty() && timeout_ms != 0)
    s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 3600000 : timeout_ms),
                        [&] { return !s->completions.empty(); });
  int k = 0;
  while (k < max && !s->completions.empty()) {
    out[k++] = s->completions.front();
    s->completions.pop_front();
  }
  *n = k;
  return JNE_OK;
}

int jne_server_fetch(jne_server* s, uint64_t id, double* out, int64_t cap) {
  if (!s) return JNE_ERR_ARG;
  Job* j = nullptr;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->finished.find(id);
    // (the worker thread owns the context's error text: these return codes only)
    if (it == s->finished.end()) return JNE_ERR_ARG;  // unknown or unfinished id
    j = it->second;
    if (out && cap < (int64_t)j->host.size()) return JNE_ERR_ARG;
    if (j->writing) return JNE_ERR_TIMEOUT;  // still being written: try again
    s->finished.erase(it);
  }
  const int st = j->status;
  if (out && st == JNE_OK) std::copy(j->host.begin(), j->host.end(), out);
  delete j;
  return st;
}

int jne_server_close(jne_server* s) {
  if (!s) return JNE_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
    s->cv.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->writer_stop = true;
    s->cv_write.notify_all();
  }
  if (s->writer.joinable()) s->writer.join();
  for (auto& kv : s->finished) delete kv.second;
  for (int i = 0; i < 2; i++) {
    cudaEventDestroy(s->it[i].ev);
    if (s->it[i].d_status) {
      cudaFree(s->it[i].d_status);
      s->ctx->in_use -= s->it[i].status_cap * sizeof(unsigned int);
    }
  }
  delete s;
  return JNE_OK;
}

}  // extern "C"
