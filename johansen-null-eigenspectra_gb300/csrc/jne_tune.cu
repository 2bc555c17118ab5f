// jne_tune.cu -- autotuner of the mixed kernel's chunk length.
//
// The chunk length L is the mixed path's speed / accuracy knob: every chunk
// ends in a merge into the float-float record (cost per chunk, so longer is
// faster), while the FP32 part of every moment grows with L (less accurate).
// The default rule (L ~ steps / 32) is conservative for every class; the tuner
// measures, per (dim, class of steps), how far L can grow before the error
// against the FP64 kernel on the same seeds exceeds a stated bound.
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

}  // namespace

extern "C" int jne_autotune_chunk(jne_context* c, int dim, int steps, double max_rel_err, int sample_runs,
                                  int* chunk_out, double* err_out) {
  if (!c) return JNE_ERR_ARG;
  if (dim < 1 || dim > JNE_MAX_DIM) return fail(c, JNE_ERR_ARG, "dim must be 1.." + std::to_string(JNE_MAX_DIM));
  if (steps < JNE_MIXED_MIN_STEPS)
    return fail(c, JNE_ERR_ARG, "classes below " + std::to_string(JNE_MIXED_MIN_STEPS) + " steps run in FP64");
  if (sample_runs < 1 || !(max_rel_err > 0.0)) return fail(c, JNE_ERR_ARG, "sample_runs >= 1 and max_rel_err > 0");
  const int b = steps_bucket(steps);
  const int tb = 1 << b;  // the class's shortest paths: the largest errors
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
  int rc = jne_eigs_seeded_models(c, models, 5, dim, tb, JNE_DEFAULT_BASE_SEED, 1, sample_runs, JNE_PREC_FP64, pref);
  if (rc) return rc;
  const int mode = c->chunk;
  int best = 0;
  double best_err = std::numeric_limits<double>::infinity();
  for (int L = 32; L <= 1024 && 2 * L <= tb; L *= 2) {
    c->chunk = L;
    rc = jne_eigs_seeded_models(c, models, 5, dim, tb, JNE_DEFAULT_BASE_SEED, 1, sample_runs, JNE_PREC_MIXED, pgot);
    if (rc) break;
    const double e = max_error(got, ref, ks, 5, sample_runs);
    if (L == 32 || e <= max_rel_err) {  // the shortest chunk is the fallback
      best = L;
      best_err = e;
    }
    if (!(e <= max_rel_err)) break;  // errors grow with L: longer chunks fail too
  }
  c->chunk = mode;
  if (rc) return rc;
  c->tuned_chunk[{dim, b}] = best;
  if (chunk_out) *chunk_out = best;
  if (err_out) *err_out = best_err;
  return JNE_OK;
}
