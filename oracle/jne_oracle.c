/*
 * jne_oracle.c -- CPU oracle for the Johansen null-eigenspectra Monte Carlo path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the pytest suite, the
 * smoke check and the CPU-baseline leg of bench.py load it.  The product
 * library (libjne_gb300.so) never links, loads or calls it.
 *
 * It restates, in plain C and double precision, the reference crate's dense
 * algorithm for one Monte Carlo run:
 *
 *   rng_matrix.rs:57-141        B = cumsum_t([start | sqrt(dt) Z]) with B_0 = 0
 *   matrix_utils.rs:51-63       the RowWise cumsum used for that
 *   johansen_statistics.rs:59-85  bm_prev = B[:,0..T), dbm = B[:,1..T] - B[:,0..T)
 *   johansen_statistics.rs:102-197 F for models 0..4 (dense construction)
 *   matrix_utils.rs:67-85       S10 = sum_t dbm_t F_t',  S11 = dt * sum_t F_t F_t'
 *   johansen_statistics.rs:35-46  eigenvalues of the pencil (S10'S10, S11),
 *                                 |alpha|/beta, sorted descending
 *
 * The reference hands the pencil to LAPACK dggev (QZ).  The oracle solves the
 * same symmetric-definite pencil by Cholesky reduction + cyclic Jacobi; the
 * Python twin (jne_oracle.py) uses scipy's dggev and the test suite checks the
 * two against each other.
 *
 * The random stream is this project's counter-based one (Philox4x32-10,
 * Salmon et al., SC'11, + Box-Muller); the reference's Xoshiro256++/ziggurat
 * stream depends on the host's core count and is not reproduced.  Philox words
 * are bit-exact with the CUDA path; the normals agree to ~1e-6 (the device uses
 * its hardware log/sin/cos approximations).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define JNO_PHILOX_M0 0xD2511F53u
#define JNO_PHILOX_M1 0xCD9E8D57u
#define JNO_PHILOX_W0 0x9E3779B9u
#define JNO_PHILOX_W1 0xBB67AE85u

/* Philox4x32-10: ten rounds of the multiply/xor bijection, key bumped by the
 * Weyl constants between rounds (Salmon et al., SC'11, section 4). */
void jno_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)JNO_PHILOX_M0 * c0;
    uint64_t p1 = (uint64_t)JNO_PHILOX_M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += JNO_PHILOX_W0;
    k1 += JNO_PHILOX_W1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Stream key for a (base seed, dim) pair.  The path of a run depends on
 * (base seed, dim, run seed) only -- not on the model -- as in the reference,
 * where calculate_eigenvalues(dim, steps, seed, model) draws the same Brownian
 * matrix for every model (johansen_statistics.rs:59-78). */
void jno_stream_key(uint64_t base_seed, int dim, uint32_t key[2]) {
  key[0] = (uint32_t)base_seed;
  key[1] = (uint32_t)(base_seed >> 32) ^ (0x4A4E0000u | (uint32_t)(dim & 0xFF));
}

/* Raw Philox words of one run: words[(s-1)*nq*4 + j*4 + w] for step s=1..steps,
 * quad j = 0..ceil(dim/4)-1, word w.  Counter = (s, j, run_seed, 0). */
void jno_philox_words(uint64_t base_seed, int dim, uint32_t run_seed, int steps, uint32_t* words) {
  uint32_t key[2];
  jno_stream_key(base_seed, dim, key);
  int nq = (dim + 3) / 4;
  for (int s = 1; s <= steps; s++)
    for (int j = 0; j < nq; j++) {
      uint32_t ctr[4] = {(uint32_t)s, (uint32_t)j, run_seed, 0u};
      jno_philox4x32_10(ctr, key, words + ((size_t)(s - 1) * nq + j) * 4);
    }
}

/* Angle uniform in (0,1): the top 23 bits m of a word, u = (m + 1/2) 2^-23. */
static inline double jno_u01(uint32_t x) { return ((double)(x >> 9) + 0.5) * (1.0 / 8388608.0); }

/* Radius uniform in [2^-33, 1): the word truncated to its leading 24 bits
 * (x rounded toward zero to a float), u = (that + 1/2) 2^-32 rounded to a
 * float, as the kernels form it in single precision. */
static inline double jno_u01_radius(uint32_t x) {
  int nb = 32;
  while (nb > 0 && !(x >> (nb - 1))) nb--;
  uint32_t t = nb > 24 ? x & ~((1u << (nb - 24)) - 1u) : x;
  return (double)(float)(((double)t + 0.5) * (1.0 / 4294967296.0));
}

/* Box-Muller on two words: z0 = r cos(theta), z1 = r sin(theta) with
 * r = sqrt(-2 ln u(a)), theta = 2 pi u(b) - pi. */
static inline void jno_box_muller(uint32_t a, uint32_t b, double* z0, double* z1) {
  double r = sqrt(-2.0 * log(jno_u01_radius(a)));
  double th = 6.283185307179586 * jno_u01(b) - 3.141592653589793;
  *z0 = r * cos(th);
  *z1 = r * sin(th);
}

/* Standard normals of one run, z[(s-1)*dim + f] (time-major, i.e. the
 * column-major dim x steps matrix of rng_matrix.rs:87-110). */
void jno_normals(uint64_t base_seed, int dim, uint32_t run_seed, int steps, double* z) {
  uint32_t key[2];
  jno_stream_key(base_seed, dim, key);
  int nq = (dim + 3) / 4;
  for (int s = 1; s <= steps; s++) {
    double* zs = z + (size_t)(s - 1) * dim;
    for (int j = 0; j < nq; j++) {
      uint32_t ctr[4] = {(uint32_t)s, (uint32_t)j, run_seed, 0u}, w[4];
      jno_philox4x32_10(ctr, key, w);
      double q[4];
      jno_box_muller(w[0], w[1], &q[0], &q[1]);
      jno_box_muller(w[2], w[3], &q[2], &q[3]);
      for (int e = 0; e < 4 && 4 * j + e < dim; e++) zs[4 * j + e] = q[e];
    }
  }
}

/* dmatrix_cumsum(.., RowWise) of matrix_utils.rs:51-63 on a column-major
 * nrows x ncols matrix: each row is summed left to right. */
void jno_cumsum_rowwise(const double* m, int nrows, int ncols, double* out) {
  for (int r = 0; r < nrows; r++) {
    double acc = 0.0;
    for (int c = 0; c < ncols; c++) {
      acc += m[(size_t)c * nrows + r];
      out[(size_t)c * nrows + r] = acc;
    }
  }
}

/* sum_of_outer_products(a, b) of matrix_utils.rs:67-85: sum over columns i of
 * a[:,i] b[:,i]'.  a is a_rows x n, b is b_rows x n (column-major); out is
 * a_rows x b_rows (column-major). */
void jno_sum_of_outer_products(const double* a, int a_rows, const double* b, int b_rows, int n,
                               double* out) {
  memset(out, 0, sizeof(double) * (size_t)a_rows * b_rows);
  for (int i = 0; i < n; i++) {
    const double* ac = a + (size_t)i * a_rows;
    const double* bc = b + (size_t)i * b_rows;
    for (int q = 0; q < b_rows; q++)
      for (int p = 0; p < a_rows; p++) out[(size_t)q * a_rows + p] += ac[p] * bc[q];
  }
}

/* Number of eigenvalues a run reports (thread_manager.rs:40-44). */
int jno_eigen_count(int model, int dim) { return (model == 1 || model == 3) ? dim + 1 : dim; }

/* construct_f_matrix of johansen_statistics.rs:102-197.  bm is dim x T
 * (column-major, bm[:, i] = B_i), f is k x T (column-major). */
static void jno_construct_f(const double* bm, int dim, int T, int model, double* f) {
  int k = jno_eigen_count(model, dim);
  double Td = (double)T;
  switch (model) {
    case 0: /* F = B_{t-1} (:106) */
      memcpy(f, bm, sizeof(double) * (size_t)dim * T);
      break;
    case 1: /* F = [B_{t-1}; 1] (:108-113) */
      for (int i = 0; i < T; i++) {
        for (int r = 0; r < dim; r++) f[(size_t)i * k + r] = bm[(size_t)i * dim + r];
        f[(size_t)i * k + dim] = 1.0;
      }
      break;
    case 2:   /* F = [demean(first dim-1 rows); (i+1)/T - 0.5] (:115-138) */
    case 3: { /* F = [demean(all rows); (i+1)/T - 0.5] (:140-162) */
      int nb = (model == 2) ? dim - 1 : dim;
      for (int r = 0; r < nb; r++) {
        double mean = 0.0;
        for (int i = 0; i < T; i++) mean += bm[(size_t)i * dim + r];
        mean /= Td;
        for (int i = 0; i < T; i++) f[(size_t)i * k + r] = bm[(size_t)i * dim + r] - mean;
      }
      for (int i = 0; i < T; i++) f[(size_t)i * k + nb] = (double)(i + 1) / Td - 0.5;
      break;
    }
    case 4: { /* F = X - X Z'(ZZ')^-1 Z, X = [first dim-1 rows; y^2], Z = [1; y] (:164-195) */
      int nb = dim - 1;
      double* x = f; /* build X in place, then subtract its projection */
      for (int i = 0; i < T; i++) {
        double y = (double)(i + 1) / Td;
        for (int r = 0; r < nb; r++) x[(size_t)i * k + r] = bm[(size_t)i * dim + r];
        x[(size_t)i * k + nb] = y * y;
      }
      double zz00 = 0, zz01 = 0, zz11 = 0;
      for (int i = 0; i < T; i++) {
        double y = (double)(i + 1) / Td;
        zz00 += 1.0; zz01 += y; zz11 += y * y;
      }
      double det = zz00 * zz11 - zz01 * zz01;
      double i00 = zz11 / det, i01 = -zz01 / det, i11 = zz00 / det;
      for (int r = 0; r < k; r++) {
        double xz0 = 0, xz1 = 0; /* row r of X Z' */
        for (int i = 0; i < T; i++) {
          double y = (double)(i + 1) / Td, v = x[(size_t)i * k + r];
          xz0 += v; xz1 += v * y;
        }
        double c0 = xz0 * i00 + xz1 * i01, c1 = xz0 * i01 + xz1 * i11;
        for (int i = 0; i < T; i++) {
          double y = (double)(i + 1) / Td;
          x[(size_t)i * k + r] -= c0 + c1 * y;
        }
      }
      break;
    }
  }
}

/* Eigenvalues of the symmetric k x k matrix a (row-major, destroyed) by the
 * cyclic Jacobi method (Golub & Van Loan, Matrix Computations, 8.5). */
static void jno_jacobi_eigvals(double* a, int k, double* w) {
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int p = 0; p < k; p++) {
      diag += a[p * k + p] * a[p * k + p];
      for (int q = p + 1; q < k; q++) off += a[p * k + q] * a[p * k + q];
    }
    if (off <= 1e-30 * diag || off == 0.0) break;
    for (int p = 0; p < k - 1; p++)
      for (int q = p + 1; q < k; q++) {
        double apq = a[p * k + q];
        if (apq == 0.0) continue;
        double app = a[p * k + p], aqq = a[q * k + q];
        double tau = (aqq - app) / (2.0 * apq);
        double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for (int r = 0; r < k; r++) { /* columns p, q */
          double arp = a[r * k + p], arq = a[r * k + q];
          a[r * k + p] = c * arp - s * arq;
          a[r * k + q] = s * arp + c * arq;
        }
        for (int r = 0; r < k; r++) { /* rows p, q */
          double apr = a[p * k + r], aqr = a[q * k + r];
          a[p * k + r] = c * apr - s * aqr;
          a[q * k + r] = s * apr + c * aqr;
        }
        a[p * k + q] = a[q * k + p] = 0.0;
      }
  }
  for (int p = 0; p < k; p++) w[p] = a[p * k + p];
}

static int jno_cmp_desc(const void* x, const void* y) {
  double a = *(const double*)x, b = *(const double*)y;
  return (a < b) - (a > b);
}

/* Generalized eigenvalues of the pencil (S10'S10, S11) of
 * johansen_statistics.rs:35-46: S11 = L L' (Cholesky), E = S10 L^-T,
 * eigenvalues of E'E, absolute values, sorted descending.
 * s10 is dim x k (column-major), s11 is k x k.  Returns 0, or -1 if S11 is
 * not numerically positive definite (out is then filled with NaN). */
static int jno_pencil_eigvals(const double* s10, const double* s11, int dim, int k, double* out) {
  double L[16 * 16], E[16 * 16], C[16 * 16];
  for (int j = 0; j < k; j++)
    for (int i = 0; i <= j; i++) {
      double s = s11[(size_t)j * k + i];
      for (int p = 0; p < i; p++) s -= L[j * k + p] * L[i * k + p];
      if (i == j) {
        if (!(s > 0.0)) {
          for (int q = 0; q < k; q++) out[q] = NAN;
          return -1;
        }
        L[j * k + j] = sqrt(s);
      } else {
        L[j * k + i] = s / L[i * k + i];
      }
    }
  /* E = S10 L^-T  <=>  E L' = S10: row a of E solves L e = s10[a,:]' */
  for (int a = 0; a < dim; a++)
    for (int j = 0; j < k; j++) {
      double s = s10[(size_t)j * dim + a];
      for (int p = 0; p < j; p++) s -= L[j * k + p] * E[a * k + p];
      E[a * k + j] = s / L[j * k + j];
    }
  for (int p = 0; p < k; p++)
    for (int q = 0; q < k; q++) {
      double s = 0.0;
      for (int a = 0; a < dim; a++) s += E[a * k + p] * E[a * k + q];
      C[p * k + q] = s;
    }
  jno_jacobi_eigvals(C, k, out);
  for (int q = 0; q < k; q++) out[q] = fabs(out[q]);
  qsort(out, (size_t)k, sizeof(double), jno_cmp_desc);
  return 0;
}

/* Per-thread scratch for one run of the dense algorithm. */
typedef struct {
  int dim, T, k;
  double *bm, *dbm, *f, *z;
} jno_work;

static int jno_work_init(jno_work* w, int dim, int T, int k) {
  w->dim = dim; w->T = T; w->k = k;
  w->bm = (double*)malloc(sizeof(double) * (size_t)dim * (T + 1));
  w->dbm = (double*)malloc(sizeof(double) * (size_t)dim * T);
  w->f = (double*)malloc(sizeof(double) * (size_t)(k > 0 ? k : 1) * T);
  w->z = (double*)malloc(sizeof(double) * (size_t)dim * T);
  return (w->bm && w->dbm && w->f && w->z) ? 0 : -1;
}
static void jno_work_free(jno_work* w) { free(w->bm); free(w->dbm); free(w->f); free(w->z); }

/* calculate_eigenvalues_from_matrices (johansen_statistics.rs:24-47) after
 * brownian_motion_matrix: dB is the dim x T column-major increment matrix
 * (dB[:, i] = B_{i+1} - B_i, i.e. sqrt(dt) * Z). */
static int jno_eigs_dense(jno_work* w, int model, const double* dB, double* out) {
  int dim = w->dim, T = w->T, k = w->k;
  double* B = w->bm; /* dim x (T+1): [start | dB] row-cumsummed, start = 0 */
  for (int r = 0; r < dim; r++) B[r] = 0.0;
  memcpy(B + dim, dB, sizeof(double) * (size_t)dim * T);
  for (int r = 0; r < dim; r++) {
    double acc = 0.0;
    for (int c = 0; c <= T; c++) {
      acc += B[(size_t)c * dim + r];
      B[(size_t)c * dim + r] = acc;
    }
  }
  for (size_t e = 0; e < (size_t)dim * T; e++) w->dbm[e] = B[e + dim] - B[e]; /* :80-82 */
  jno_construct_f(B, dim, T, model, w->f);
  double s10[16 * 16], s11[16 * 16];
  jno_sum_of_outer_products(w->dbm, dim, w->f, k, T, s10);
  jno_sum_of_outer_products(w->f, k, w->f, k, T, s11);
  double dt = 1.0 / (double)T;
  for (int e = 0; e < k * k; e++) s11[e] *= dt;
  return jno_pencil_eigvals(s10, s11, dim, k, out);
}

/* Eigenvalues of n_runs runs from explicit increments.  dB holds n_runs
 * consecutive dim x steps column-major matrices; out holds n_runs x k values.
 * Returns the number of runs whose S11 was not positive definite, or -1 on
 * bad arguments. */
int jno_eigs_from_increments(int model, int dim, int steps, const double* dB, int n_runs, double* out) {
  if (model < 0 || model > 4 || dim < 1 || dim > 15 || steps < 1 || n_runs < 0) return -1;
  int k = jno_eigen_count(model, dim);
  jno_work w;
  if (jno_work_init(&w, dim, steps, k)) { jno_work_free(&w); return -1; }
  int bad = 0;
  for (int r = 0; r < n_runs; r++)
    if (jno_eigs_dense(&w, model, dB + (size_t)r * dim * steps, out + (size_t)r * k)) bad++;
  jno_work_free(&w);
  return bad;
}

/* jno_eigs_from_increments over n_threads POSIX threads (runs split in
 * contiguous blocks); same results, same return convention. */
typedef struct {
  int model, dim, steps, n_runs, ret;
  const double* dB;
  double* out;
} jno_inc_job;

static void* jno_inc_worker(void* arg) {
  jno_inc_job* j = (jno_inc_job*)arg;
  j->ret = jno_eigs_from_increments(j->model, j->dim, j->steps, j->dB, j->n_runs, j->out);
  return NULL;
}

int jno_eigs_from_increments_mt(int model, int dim, int steps, const double* dB, int n_runs, int n_threads,
                                double* out) {
  if (model < 0 || model > 4 || dim < 1 || dim > 15 || steps < 1 || n_runs < 0 || n_threads < 1) return -1;
  if (n_threads > 256) n_threads = 256;
  if (n_threads > n_runs) n_threads = n_runs > 0 ? n_runs : 1;
  int k = jno_eigen_count(model, dim), per = (n_runs + n_threads - 1) / n_threads, bad = 0;
  pthread_t th[256];
  int started[256];
  jno_inc_job jobs[256];
  for (int t = 0; t < n_threads; t++) {
    int r0 = t * per, n = n_runs - r0 < per ? n_runs - r0 : per;
    if (n < 0) n = 0;
    jobs[t] = (jno_inc_job){model, dim, steps, n, 0, dB + (size_t)r0 * dim * steps, out + (size_t)r0 * k};
    started[t] = pthread_create(&th[t], NULL, jno_inc_worker, &jobs[t]) == 0;
    if (!started[t]) jno_inc_worker(&jobs[t]);
  }
  for (int t = 0; t < n_threads; t++) {
    if (started[t]) pthread_join(th[t], NULL);
    if (jobs[t].ret < 0) return -1;
    bad += jobs[t].ret;
  }
  return bad;
}

/* ---- an independent generator, for distribution tests ----
 * xoshiro256++ (Blackman & Vigna, "Scrambled linear pseudorandom number
 * generators", ACM TOMS 47(4), 2021) -- the generator family the reference
 * draws its normals from (rand_xoshiro's Xoshiro256PlusPlus, rng_matrix.rs:23-33)
 * -- with each run's 256-bit state expanded from (base seed, run seed) by
 * SplitMix64 (Steele, Lea & Flood, OOPSLA 2014), as its authors recommend.
 * Normals by Box-Muller in double on 53-bit uniforms u in (0, 1]: radii up to
 * sqrt(-2 ln 2^-53) = 8.6, so the sample is untruncated for any test size,
 * like the reference's StandardNormal.  Shares no code or constant with the
 * counter-based stream of the kernels. */
static inline uint64_t jno_rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t jno_splitmix64(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

typedef struct {
  uint64_t s[4];
} jno_xoshiro;

static void jno_xoshiro_seed(jno_xoshiro* g, uint64_t base_seed, uint32_t run_seed) {
  uint64_t x = base_seed ^ ((uint64_t)run_seed * 0xD1B54A32D192ED03ull);
  for (int i = 0; i < 4; i++) g->s[i] = jno_splitmix64(&x);
}

static inline uint64_t jno_xoshiro_next(jno_xoshiro* g) {
  uint64_t* s = g->s;
  const uint64_t out = jno_rotl64(s[0] + s[3], 23) + s[0];
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = jno_rotl64(s[3], 45);
  return out;
}

/* u in (0, 1]: the top 53 bits m, u = (m + 1) 2^-53 */
static inline double jno_xoshiro_u01(jno_xoshiro* g) {
  return ((double)(jno_xoshiro_next(g) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

/* n standard normals, pairwise Box-Muller */
void jno_xoshiro_normals(uint64_t base_seed, uint32_t run_seed, int n, double* z) {
  jno_xoshiro g;
  jno_xoshiro_seed(&g, base_seed, run_seed);
  for (int i = 0; i < n; i += 2) {
    const double r = sqrt(-2.0 * log(jno_xoshiro_u01(&g)));
    const double th = 6.283185307179586 * jno_xoshiro_u01(&g);
    z[i] = r * cos(th);
    if (i + 1 < n) z[i + 1] = r * sin(th);
  }
}

/* ---- seeded, multi-threaded batch (the CPU baseline) ---- */
typedef struct {
  int model, dim, steps, k, n_runs, nthreads, tid;
  uint64_t base_seed;
  uint32_t seed_first;
  double* out;
  int bad;
  int gen; /* 0: the counter-based stream of the kernels; 1: xoshiro256++ (independent) */
} jno_job;

static void* jno_worker(void* arg) {
  jno_job* j = (jno_job*)arg;
  jno_work w;
  if (jno_work_init(&w, j->dim, j->steps, j->k)) { jno_work_free(&w); j->bad = -1; return NULL; }
  double sdt = sqrt(1.0 / (double)j->steps);
  for (int r = j->tid; r < j->n_runs; r += j->nthreads) {
    if (j->gen)
      jno_xoshiro_normals(j->base_seed, j->seed_first + (uint32_t)r, j->dim * j->steps, w.z);
    else
      jno_normals(j->base_seed, j->dim, j->seed_first + (uint32_t)r, j->steps, w.z);
    for (size_t e = 0; e < (size_t)j->dim * j->steps; e++) w.z[e] *= sdt; /* rng_matrix.rs:138-139 */
    if (jno_eigs_dense(&w, j->model, w.z, j->out + (size_t)r * j->k)) j->bad++;
  }
  jno_work_free(&w);
  return NULL;
}

/* Runs with seeds seed_first .. seed_first+n_runs-1 drawn from generator `gen`
 * (0: the counter-based stream, 1: xoshiro256++), spread over n_threads POSIX
 * threads. */
static int jno_eigs_seeded_gen(int gen, int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first,
                               int n_runs, int n_threads, double* out) {
  if (model < 0 || model > 4 || dim < 1 || dim > 15 || steps < 1 || n_runs < 0 || n_threads < 1) return -1;
  if (n_threads > 256) n_threads = 256;
  pthread_t th[256];
  int started[256];
  jno_job jobs[256];
  int k = jno_eigen_count(model, dim), bad = 0;
  for (int t = 0; t < n_threads; t++) {
    jobs[t] = (jno_job){model, dim, steps, k, n_runs, n_threads, t, base_seed, seed_first, out, 0, gen};
    started[t] = pthread_create(&th[t], NULL, jno_worker, &jobs[t]) == 0;
    if (!started[t]) jno_worker(&jobs[t]);
  }
  for (int t = 0; t < n_threads; t++) {
    if (started[t]) pthread_join(th[t], NULL);
    if (jobs[t].bad < 0) return -1;
    bad += jobs[t].bad;
  }
  return bad;
}

int jno_eigs_seeded(int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first, int n_runs,
                    int n_threads, double* out) {
  return jno_eigs_seeded_gen(0, model, dim, steps, base_seed, seed_first, n_runs, n_threads, out);
}

/* The same runs' statistic from the independent xoshiro256++ stream: a sample of
 * the same distribution that shares no random number with the kernels. */
int jno_eigs_seeded_xoshiro(int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first, int n_runs,
                            int n_threads, double* out) {
  return jno_eigs_seeded_gen(1, model, dim, steps, base_seed, seed_first, n_runs, n_threads, out);
}
