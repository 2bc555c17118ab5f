// jne_tune.cu -- autotuner of the mixed kernel's launch shape.
//
// Three knobs set a mixed request's speed:
//   * the chunk length L: every chunk ends in a merge into the float-float
//     record (a cost per chunk, so longer is faster), while the FP32 part of
//     every moment grows with L (less accurate) -- the one knob that changes
//     the arithmetic;
//   * blocks per SM of the kernel variant: 4 (128 registers a thread) or 6
//     (80 registers, more warps to hide latency, a few spilled registers);
//   * for dims up to 4, two runs per warp or one.
// Per (dim, class of steps) the tuner measures the error of each chunk against
// the FP64 kernel on the same seeds (all five models), then times every shape
// whose chunk is within the error bound and keeps the fastest.
#include <cmath>
#include <limits>
#include <vector>

#include "jne_context.h"

using namespace jne_detail;

namespace {

// largest over runs and models of the max-eigenvalue and trace differences,
// relative to max(reference value, 1)
double max_error(const std::vector<std::vector<double>>& got, const std::vector<std::vector<double>>& ref,
                 const int* ks, int n_models, int n) {
  double worst = 0.0;
  for (int m = 0; m < n_models; m++) {
    const int k = ks[m];
    for (int r = 0; r < n; r++) {
      const double* a = &got[m][(size_t)r * k];
      const double* b = &ref[m][(size_t)r * k];
      double ta = 0.0, tb = 0.0;
      for (int j = 0; j < k; j++) {
        ta += a[j];
        tb += b[j];
      }
      const double e1 = std::fabs(a[0] - b[0]) / std::fmax(std::fabs(b[0]), 1.0);
      const double e2 = std::fabs(ta - tb) / std::fmax(std::fabs(tb), 1.0);
      if (!(e1 <= worst)) worst = e1;  // NaN propagates as the worst error
      if (!(e2 <= worst)) worst = e2;
    }
  }
  return worst;
}

// Restores the context's chunk mode and forced shape when the tuner returns.
struct ModeGuard {
  jne_context* c;
  int chunk;
  jne_shape force;
  explicit ModeGuard(jne_context* c_) : c(c_), chunk(c_->chunk), force(c_->force) {}
  ~ModeGuard() {
    c->chunk = chunk;
    c->force = force;
  }
};

// Device milliseconds of one seeded mixed launch of n runs (model 0) in the
// context's current mode: a warm-up launch, then the faster of two timed ones.
int time_launch(jne_context* c, int dim, int steps, int64_t n, double* d_out, cudaEvent_t e0, cudaEvent_t e1,
                double* ms) {
  double best = std::numeric_limits<double>::infinity();
  for (int rep = 0; rep < 3; rep++) {
    cudaError_t e = cudaEventRecord(e0, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "tuner event");
    int rc = jne_eigs_seeded_device(c, 0, dim, steps, JNE_DEFAULT_BASE_SEED, 1, n, JNE_PREC_MIXED, d_out, nullptr);
    if (rc) return rc;
    if ((e = cudaEventRecord(e1, c->stream)) != cudaSuccess || (e = cudaEventSynchronize(e1)) != cudaSuccess)
      return cuda_fail(c, e, "tuner event");
    float t = 0.f;
    if ((e = cudaEventElapsedTime(&t, e0, e1)) != cudaSuccess) return cuda_fail(c, e, "tuner event");
    if (rep > 0 && t < best) best = t;
  }
  *ms = best;
  return jne_sync(c);
}

}  // namespace

extern "C" int jne_autotune(jne_context* c, int dim, int steps, double max_rel_err, int sample_runs,
                            int64_t time_runs, jne_tune_entry* table, int table_cap, int* n_table,
                            jne_tune_entry* chosen) {
  if (!c) return JNE_ERR_ARG;
  if (dim < 1 || dim > JNE_MAX_DIM) return fail(c, JNE_ERR_ARG, "dim must be 1.." + std::to_string(JNE_MAX_DIM));
  if (steps < JNE_MIXED_MIN_STEPS)
    return fail(c, JNE_ERR_ARG, "classes below " + std::to_string(JNE_MIXED_MIN_STEPS) + " steps run in FP64");
  if (sample_runs < 1 || !(max_rel_err > 0.0) || time_runs < 0 || (table_cap > 0 && !table))
    return fail(c, JNE_ERR_ARG, "sample_runs >= 1, max_rel_err > 0 and time_runs >= 0 required");
  if (n_table) *n_table = 0;
  const int b = steps_bucket(steps);
  const int tb = 1 << b;  // the class's shortest paths: the largest errors
  if (time_runs == 0) {   // about 20-60 ms a launch
    const double r = 2e10 / ((double)tb * (dim + 3));
    time_runs = (int64_t)std::fmin(4194304.0, std::fmax(32768.0, r));
  }
  const int models[5] = {0, 1, 2, 3, 4};
  int ks[5];
  std::vector<std::vector<double>> ref(5), got(5);
  double* pref[5];
  double* pgot[5];
  for (int m = 0; m < 5; m++) {
    ks[m] = jne_eigen_count(m, dim);
    ref[m].resize((size_t)sample_runs * ks[m]);
    got[m].resize((size_t)sample_runs * ks[m]);
    pref[m] = ref[m].data();
    pgot[m] = got[m].data();
  }
  ModeGuard guard(c);
  c->force = jne_shape{};
  int rc = jne_eigs_seeded_models(c, models, 5, dim, tb, JNE_DEFAULT_BASE_SEED, 1, sample_runs, JNE_PREC_FP64, pref);
  if (rc) return rc;

  // 1. the error of each chunk length (every shape of a chunk gives the same bits)
  std::vector<std::pair<int, double>> errs;
  for (int L = 32; L <= 1024 && 2 * L <= tb; L *= 2) {
    c->chunk = L;
    if ((rc = jne_eigs_seeded_models(c, models, 5, dim, tb, JNE_DEFAULT_BASE_SEED, 1, sample_runs, JNE_PREC_MIXED,
                                     pgot)))
      return rc;
    const double e = max_error(got, ref, ks, 5, sample_runs);
    errs.push_back({L, e});
    if (!(e <= max_rel_err)) break;  // errors grow with L: longer chunks fail too
  }
  std::vector<int> cands;
  for (auto& le : errs)
    if (le.second <= max_rel_err) cands.push_back(le.first);
  if (cands.empty()) cands.push_back(32);  // the shortest chunk is the fallback

  // 2. the device time of every shape of the admissible chunks
  const int k0 = jne_eigen_count(0, dim);
  if ((rc = ensure(c, &c->d_out, &c->out_cap, (size_t)time_runs * k0, "tuner output"))) return rc;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return cuda_fail(c, ce, "tuner events");
  }
  std::vector<jne_tune_entry> rows;
  jne_tune_entry best{};
  best.ms = std::numeric_limits<double>::infinity();
  for (auto& le : errs) {
    const bool admissible = std::find(cands.begin(), cands.end(), le.first) != cands.end();
    for (int bps : {4, 6})
      for (int pack : {1, 0}) {
        if (pack == 0 && dim > JNE_PACK_MAX_DIM) continue;
        jne_tune_entry t{le.first, bps, pack, le.second, -1.0};
        if (admissible) {
          c->chunk = le.first;
          c->force = jne_shape{le.first, bps, pack};
          if ((rc = time_launch(c, dim, tb, time_runs, c->d_out, e0, e1, &t.ms))) break;
          if (t.ms < best.ms) best = t;
        }
        rows.push_back(t);
      }
    if (rc) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  c->tuned[{dim, b}] = jne_shape{best.chunk, best.blocks_per_sm, best.pack};
  if (chosen) *chosen = best;
  if (table) {
    const int n = (int)std::min<size_t>(rows.size(), (size_t)table_cap);
    for (int i = 0; i < n; i++) table[i] = rows[(size_t)i];
    if (n_table) *n_table = n;
  }
  return JNE_OK;
}

extern "C" int jne_autotune_chunk(jne_context* c, int dim, int steps, double max_rel_err, int sample_runs,
                                  int* chunk_out, double* err_out) {
  jne_tune_entry best{};
  const int rc = jne_autotune(c, dim, steps, max_rel_err, sample_runs, 0, nullptr, 0, nullptr, &best);
  if (rc) return rc;
  if (chunk_out) *chunk_out = best.chunk;
  if (err_out) *err_out = best.max_rel_err;
  return JNE_OK;
}
