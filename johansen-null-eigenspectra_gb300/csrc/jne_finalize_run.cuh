// jne_finalize_run.cuh -- the per-run FP64 finalize (moment record -> eigenvalues),
// shared by the finalize kernels and by the mixed accumulation kernel, which
// finalizes its own runs in batches of 32 (one run per lane).
//
// Replaces johansen_statistics.rs:24-47 (the F-based Grams, then
// GeneralizedEigen(S10'S10, S11) via LAPACK dggev, |alpha|/beta, descending
// sort).  One thread per run, all in FP64:
//   1. F_j = G[x_j] - alpha_j * 1 - beta_j * y for the model's rows, where
//      G = [B; 1; y; y^2].  This is construct_f_matrix (:102-197) written as a
//      linear map: demeaning (models 2, 3) subtracts the row mean, model 4
//      subtracts the least-squares fit on {1, y}.  S11 = dt F F' and
//      S10 = dB F' then follow from the raw moments alone.
//   2. S11 = L L' (Cholesky), E = S10 L^-T, C = E'E: the pencil's eigenvalues
//      are those of the symmetric PSD matrix C.
//   3. Householder tridiagonalisation + implicit QL (eigenvalues only), then
//      |lambda| and a descending sort -- the reference reports |alpha|/beta.
// The QL path needs ~10x fewer FP64 operations than cyclic Jacobi at k = 13,
// which matters on a GPU whose FP64 rate is ~1/74 of its FP32 rate.
#pragma once
#include <cfloat>
#include <math_constants.h>
#include "jne_kernels.h"

namespace jne_fin {
namespace {  // internal linkage: each translation unit that includes this has its own copy

struct Ctx {
  const double* mom;
  long long ld;
  int run, d;
  double s;
  const double* Y;
  // cached in L2 only: the mixed kernel reads records its own warp wrote moments earlier
  __device__ double rec(int slot) const { return __ldcg(mom + (size_t)slot * ld + run); }
  // M(r, n) = sum_i G_r G_n over the global basis G = [B (d); 1; y; y^2]
  __device__ double M(int r, int n) const {
    if (r > n) { const int t = r; r = n; n = t; }
    if (n < d) return s * s * rec(jne_slot_MWW(r, n, d));
    if (r < d) {
      const int p = n - d;
      return s * rec(p == 0 ? jne_slot_MW1(r, d) : p == 1 ? jne_slot_MWy(r, d) : jne_slot_MWyy(r, d));
    }
    return Y[(r - d) + (n - d)];
  }
  // N(r, c) = sum_i G_r dB_c
  __device__ double N(int r, int c) const {
    if (r < d) return s * s * rec(jne_slot_NzW(c, r, d));
    const int p = r - d;
    return s * rec(p == 0 ? jne_slot_Nz1(c, d) : p == 1 ? jne_slot_Nzy(c, d) : jne_slot_Nzyy(c, d));
  }
};

// Householder reduction of the symmetric n x n matrix A (full storage) to
// tridiagonal form (Golub & Van Loan, Matrix Computations, Algorithm 8.3.1):
// diagonal -> dg[0..n-1], sub-diagonal -> eo[0..n-2].
__device__ __forceinline__ void tridiagonalize(double (*A)[JNE_MAX_K], int n, double* dg, double* eo) {
  for (int k = 0; k + 2 < n; k++) {
    double sigma = 0.0;
    for (int i = k + 2; i < n; i++) sigma += A[i][k] * A[i][k];
    const double x0 = A[k + 1][k];
    if (sigma == 0.0) { eo[k] = x0; continue; }
    const double nrm = sqrt(x0 * x0 + sigma);
    const double alpha = x0 > 0.0 ? -nrm : nrm;  // H x = alpha e1
    double v[JNE_MAX_K];
    v[k + 1] = x0 - alpha;                        // |x0| + nrm: no cancellation
    for (int i = k + 2; i < n; i++) v[i] = A[i][k];
    const double tau = 1.0 / (nrm * (nrm + fabs(x0)));  // 2 / (v'v)
    double p[JNE_MAX_K];
    double pv = 0.0;
    for (int i = k + 1; i < n; i++) {
      double t = 0.0;
      for (int j = k + 1; j < n; j++) t += A[i][j] * v[j];
      p[i] = tau * t;
      pv += p[i] * v[i];
    }
    const double K = 0.5 * tau * pv;
    for (int i = k + 1; i < n; i++) p[i] -= K * v[i];  // w = p - K v
    for (int i = k + 1; i < n; i++)
      for (int j = k + 1; j < n; j++) A[i][j] -= v[i] * p[j] + p[i] * v[j];
    eo[k] = alpha;
  }
  if (n >= 2) eo[n - 2] = A[n - 1][n - 2];
  for (int i = 0; i < n; i++) dg[i] = A[i][i];
}

// Eigenvalues of the symmetric tridiagonal matrix (dg, eo) by the implicit QL
// method with Wilkinson shifts (Bowdler, Martin, Reinsch & Wilkinson, "The QR
// and QL algorithms for symmetric matrices", Numer. Math. 11, 1968).  eo[i]
// couples dg[i] and dg[i+1]; the iteration count per eigenvalue is bounded.
__device__ __forceinline__ bool tridiagonal_ql(double* dg, double* eo, int n) {
  eo[n - 1] = 0.0;
  bool ok = true;
  for (int l = 0; l < n; l++) {
    for (int iter = 0; iter < 64; iter++) {
      int m = l;
      for (; m < n - 1; m++) {
        const double dd = fabs(dg[m]) + fabs(dg[m + 1]);
        if (fabs(eo[m]) <= DBL_EPSILON * dd) break;
      }
      if (m == l) break;
      if (iter == 63) { ok = false; break; }
      double g = (dg[l + 1] - dg[l]) / (2.0 * eo[l]);
      double r = hypot(g, 1.0);
      g = dg[m] - dg[l] + eo[l] / (g + copysign(r, g));
      double s = 1.0, c = 1.0, p = 0.0;
      int i = m - 1;
      bool underflow = false;
      for (; i >= l; i--) {
        const double f = s * eo[i], b = c * eo[i];
        // Givens rotation from one reciprocal square root (the moments keep
        // f and g far from the overflow / underflow range hypot guards)
        const double r2 = fma(f, f, g * g);
        if (r2 == 0.0) {  // recover from underflow
          eo[i + 1] = 0.0;
          dg[i + 1] -= p;
          eo[m] = 0.0;
          underflow = true;
          break;
        }
        const double ir = rsqrt(r2);
        r = r2 * ir;
        eo[i + 1] = r;
        s = f * ir;
        c = g * ir;
        g = dg[i + 1] - p;
        r = (dg[i] - g) * s + 2.0 * c * b;
        p = s * r;
        dg[i + 1] = g + p;
        g = c * r - b;
      }
      if (underflow) continue;
      dg[l] -= p;
      eo[l] = g;
      eo[m] = 0.0;
    }
  }
  return ok;
}

__device__ __noinline__ void finalize_run(const jne_finalize_args& f, int run) {
  const int d = f.dim, model = f.model;
  const int k = (model == 1 || model == 3) ? d + 1 : d;
  const Ctx c{f.mom, f.mom_ld, run, d, f.zscale, f.ts.Y};
  const double T = (double)f.steps, dt = 1.0 / T;
  const double Y0 = f.ts.Y[0], Y1 = f.ts.Y[1], Y2 = f.ts.Y[2];
  const int ONE = d, Yr = d + 1, YY = d + 2;

  // F rows: F_j = G[x_j] - al_j * G[ONE] - be_j * G[Yr]
  int x[JNE_MAX_K];
  double al[JNE_MAX_K], be[JNE_MAX_K], m1[JNE_MAX_K], my[JNE_MAX_K];
  const int nb = (model == 2 || model == 4) ? d - 1 : d;  // walk rows kept
  for (int j = 0; j < k; j++) {
    x[j] = j < nb ? j : (model == 1 ? ONE : model == 4 ? YY : Yr);
    m1[j] = c.M(x[j], ONE);
    my[j] = c.M(x[j], Yr);
    al[j] = 0.0;
    be[j] = 0.0;
  }
  if (model == 2 || model == 3) {
    for (int j = 0; j < nb; j++) al[j] = m1[j] / T;  // row mean
    al[nb] = 0.5;                                    // trend row y - 0.5
  } else if (model == 4) {
    const double det = Y0 * Y2 - Y1 * Y1;
    const double i00 = Y2 / det, i01 = -Y1 / det, i11 = Y0 / det;
    for (int j = 0; j < k; j++) {
      al[j] = m1[j] * i00 + my[j] * i01;
      be[j] = m1[j] * i01 + my[j] * i11;
    }
  }

  double S[JNE_MAX_K][JNE_MAX_K];
  for (int j = 0; j < k; j++)
    for (int l = 0; l <= j; l++) {
      double v = c.M(x[j], x[l]) - al[l] * m1[j] - be[l] * my[j] - al[j] * m1[l] - be[j] * my[l] +
                 al[j] * al[l] * Y0 + (al[j] * be[l] + be[j] * al[l]) * Y1 + be[j] * be[l] * Y2;
      S[j][l] = v * dt;
    }

  // Cholesky S11 = L L' (lower triangle of S); inv[j] = 1 / L[j][j]
  bool ok = true;
  double inv[JNE_MAX_K];
  for (int j = 0; j < k && ok; j++) {
    for (int i = 0; i <= j; i++) {
      double s = S[j][i];
      for (int p = 0; p < i; p++) s -= S[j][p] * S[i][p];
      if (i == j) {
        if (!(s > 0.0)) { ok = false; break; }
        S[j][j] = sqrt(s);
        inv[j] = 1.0 / S[j][j];
      } else {
        S[j][i] = s * inv[i];
      }
    }
  }
  double* out = f.out + (size_t)run * k;
  if (!ok) {
    for (int j = 0; j < k; j++) out[j] = CUDART_NAN;
    if (f.status) atomicOr(f.status, JNE_DEV_NOT_SPD);
    return;
  }
  // C = E'E with E = S10 L^-T, one row of E at a time: row cc solves
  // L e = S10[cc, :]' and adds e e' to C, so E is never stored.  C's strict
  // upper triangle lives in the upper triangle of S (L uses the lower one and
  // inv[] its diagonal), its diagonal in cd[].
  double cd[JNE_MAX_K];
  for (int p = 0; p < k; p++) {
    cd[p] = 0.0;
    for (int q = p + 1; q < k; q++) S[p][q] = 0.0;
  }
  for (int cc = 0; cc < d; cc++) {
    const double n1 = c.N(ONE, cc), ny = c.N(Yr, cc);
    double e[JNE_MAX_K];
    for (int j = 0; j < k; j++) {
      double s = c.N(x[j], cc) - al[j] * n1 - be[j] * ny;
      for (int p = 0; p < j; p++) s -= S[j][p] * e[p];
      e[j] = s * inv[j];
    }
    for (int p = 0; p < k; p++) {
      cd[p] += e[p] * e[p];
      for (int q = 0; q < p; q++) S[q][p] += e[p] * e[q];
    }
  }
  // full symmetric storage for the tridiagonalisation
  for (int p = 0; p < k; p++) {
    S[p][p] = cd[p];
    for (int q = 0; q < p; q++) S[p][q] = S[q][p];
  }
  double dg[JNE_MAX_K], eo[JNE_MAX_K];
  tridiagonalize(S, k, dg, eo);
  if (!tridiagonal_ql(dg, eo, k) && f.status) atomicOr(f.status, JNE_DEV_NOT_SPD);
  for (int j = 0; j < k; j++) dg[j] = fabs(dg[j]);
  for (int j = 1; j < k; j++) {  // insertion sort, descending
    const double v = dg[j];
    int i = j - 1;
    while (i >= 0 && dg[i] < v) { dg[i + 1] = dg[i]; i--; }
    dg[i + 1] = v;
  }
  for (int j = 0; j < k; j++) out[j] = dg[j];
}

}  // namespace
}  // namespace jne_fin
