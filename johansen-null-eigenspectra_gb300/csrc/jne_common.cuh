// jne_common.cuh -- shared device definitions: counter-based increments,
// the per-run moment record, and the argument block of the accumulation kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define JNE_MAX_DIM 12
#define JNE_MAX_K 13
#define JNE_WARP 32

// ---------------------------------------------------------------------------
// Counter-based increments (Philox4x32-10, Salmon et al., SC'11).
//
// The standard normal z[f] drawn for step s (1..T) of run `seed` in the
// (base seed, dim) stream comes from Philox block (s, f/4, seed, 0) under
// key (lo32(base), hi32(base) ^ (0x4A4E0000 | dim)), word pair (f%4)/2, via
// Box-Muller.  A run is a pure function of (base seed, dim, seed, s): the model
// is not part of the key, so -- as in the reference, where
// calculate_eigenvalues(dim, steps, seed, model) draws the same Brownian matrix
// for every model (johansen_statistics.rs:59-78) -- all five models see the same
// path for a given seed.
// ---------------------------------------------------------------------------
// Round keys of the Philox4x32-10 key schedule (key bumped by the Weyl
// constants between rounds).  They depend only on the stream key, so a kernel
// computes them once.
struct jne_round_keys {
  uint32_t k0[10], k1[10];
};

__host__ __device__ __forceinline__ jne_round_keys jne_make_round_keys(uint32_t k0, uint32_t k1) {
  jne_round_keys rk;
  for (int r = 0; r < 10; r++) {
    rk.k0[r] = k0 + (uint32_t)r * 0x9E3779B9u;
    rk.k1[r] = k1 + (uint32_t)r * 0xBB67AE85u;
  }
  return rk;
}

// Ten rounds of the multiply/xor bijection; each 32x32->64 product yields both
// halves at once.
__device__ __forceinline__ void jne_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                  const jne_round_keys& rk, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const unsigned long long p0 = (unsigned long long)c0 * 0xD2511F53ull;
    const unsigned long long p1 = (unsigned long long)c2 * 0xCD9E8D57ull;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ rk.k0[r];
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ rk.k1[r];
    c1 = (uint32_t)p1;
    c3 = (uint32_t)p0;
    c0 = n0;
    c2 = n2;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Documented PTX approximations (single hardware instructions, so every kernel
// that draws a value computes it the same way).  The .ftz forms: no input or
// output of the normal transform is subnormal (u >= 2^-33, |theta| >= 3.7e-7,
// radii >= 3.4e-4), so flushing changes no value, and these forms skip the
// subnormal handling the plain forms wrap around the hardware approximation
// (10% more normals per second, bit-identical).
__device__ __forceinline__ float jne_lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float jne_sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float jne_sin_approx(float x) {
  float y;
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float jne_cos_approx(float x) {
  float y;
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// w rounded toward zero to a float (its leading 24 bits, exact)
__device__ __forceinline__ float jne_u32_to_f32_rz(uint32_t w) {
  float y;
  asm("cvt.rz.f32.u32 %0, %1;" : "=f"(y) : "r"(w));
  return y;
}

// Box-Muller pair: r = sqrt(-2 ln u(a)), theta = 2 pi u(b) - pi, z = r (cos, sin).
// Explicit _rn arithmetic keeps any caller from fusing a step into a different
// FMA, so the values are identical in every kernel that draws them.  The two
// pairs of a quad go through the FP32 steps together (the paired
// add/multiply/FMA instructions of this GPU, each half rounded as its scalar
// form): half the issue slots for those steps, the same values.
// The four normals of quad j (features 4j..4j+3) of step s.
__device__ __forceinline__ void jne_normal_quad(uint32_t s, uint32_t j, uint32_t seed, const jne_round_keys& rk,
                                                float z[4]) {
  uint32_t w[4];
  jne_philox4x32_10(s, j, seed, 0u, rk, w);
  // Radius words (w0, w2): u = (rz(w) + 1/2) 2^-32 rounded to a float, in
  // [2^-33, 1 - 2^-24], where rz(w) keeps the leading 24 bits of w.  All 32 bits
  // reach the small u that make the large radii: |z| <= sqrt(66 ln 2) = 6.77, a
  // cap that a pair of draws would exceed with probability 2^-33.
  // Angle words (w1, w3): the top 23 bits m, u = (m + 1/2) 2^-23, built in the
  // mantissa of a float in [1, 2) and shifted down (both steps exact).
  const float2 ur = __ffma2_rn(make_float2(jne_u32_to_f32_rz(w[0]), jne_u32_to_f32_rz(w[2])),
                               make_float2(2.3283064365386963e-10f, 2.3283064365386963e-10f),
                               make_float2(1.1641532182693481e-10f, 1.1641532182693481e-10f));
  const float2 off = make_float2(-0.99999994039535522f, -0.99999994039535522f);
  const float2 ua = __fadd2_rn(make_float2(__uint_as_float(0x3F800000u | (w[1] >> 9)),
                                           __uint_as_float(0x3F800000u | (w[3] >> 9))), off);
  const float2 m = __fmul2_rn(make_float2(-1.3862943611198906f, -1.3862943611198906f),
                              make_float2(jne_lg2_approx(ur.x), jne_lg2_approx(ur.y)));  // -2 ln 2 * log2(u)
  const float r0 = jne_sqrt_approx(m.x), r1 = jne_sqrt_approx(m.y);
  const float2 th = __ffma2_rn(ua, make_float2(6.2831853071795865f, 6.2831853071795865f),
                               make_float2(-3.1415926535897932f, -3.1415926535897932f));
  const float2 z01 = __fmul2_rn(make_float2(r0, r0), make_float2(jne_cos_approx(th.x), jne_sin_approx(th.x)));
  const float2 z23 = __fmul2_rn(make_float2(r1, r1), make_float2(jne_cos_approx(th.y), jne_sin_approx(th.y)));
  z[0] = z01.x;
  z[1] = z01.y;
  z[2] = z23.x;
  z[3] = z23.y;
}

// ---------------------------------------------------------------------------
// Per-run moment record (FP64), in units of the unscaled walk W_i = sum_{s<=i} z_s
// (B = zscale * W, dB = zscale * z).  Column i = 0..T-1 pairs W_i (B_{t-1})
// with the increment z_{i+1} and the time point y_i = (i+1)/T.
//   [0, d(d+1)/2)        MWW[a][b] = sum W_a W_b        (a <= b, row-major upper)
//   +d                   MW1[a]    = sum W_a
//   +d                   MWy[a]    = sum y W_a
//   +d                   MWyy[a]   = sum y^2 W_a
//   +d*d                 NzW[a][b] = sum z_a W_b        (a: increment, b: walk)
//   +d                   Nz1[a]    = sum z_a = W_T
//   +d                   Nzy[a]    = sum y z_a
//   +d                   Nzyy[a]   = sum y^2 z_a
// The record is stored structure-of-arrays: value(slot, run) = mom[slot * ld + run].
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ int jne_tri(int a, int b, int d) {  // a <= b
  return a * d - (a * (a - 1)) / 2 + (b - a);
}
__host__ __device__ __forceinline__ int jne_slot_MWW(int a, int b, int d) {
  return a <= b ? jne_tri(a, b, d) : jne_tri(b, a, d);
}
__host__ __device__ __forceinline__ int jne_slot_MW1(int a, int d) { return d * (d + 1) / 2 + a; }
__host__ __device__ __forceinline__ int jne_slot_MWy(int a, int d) { return d * (d + 1) / 2 + d + a; }
__host__ __device__ __forceinline__ int jne_slot_MWyy(int a, int d) { return d * (d + 1) / 2 + 2 * d + a; }
__host__ __device__ __forceinline__ int jne_slot_NzW(int a, int b, int d) { return d * (d + 1) / 2 + 3 * d + a * d + b; }
__host__ __device__ __forceinline__ int jne_slot_Nz1(int a, int d) { return d * (d + 1) / 2 + 3 * d + d * d + a; }
__host__ __device__ __forceinline__ int jne_slot_Nzy(int a, int d) { return d * (d + 1) / 2 + 4 * d + d * d + a; }
__host__ __device__ __forceinline__ int jne_slot_Nzyy(int a, int d) { return d * (d + 1) / 2 + 5 * d + d * d + a; }
__host__ __device__ __forceinline__ int jne_record_slots(int d) { return d * (d + 1) / 2 + 6 * d + d * d; }

// Per-chunk time constants of the mixed kernel: mean of y and of y^2 over the
// chunk's columns as float-float pairs (hi + lo), its step count and the
// reciprocal.
struct jne_chunk_time {
  float ybar_hi, ybar_lo, y2bar_hi, y2bar_lo;
  float lc, inv_lc, pad0, pad1;
};

// Argument block of one accumulation launch: runs [0, n_runs) of one
// (model, dim, steps) request; run r uses seed seed_first + r.
struct jne_accum_args {
  int model, dim, steps, n_runs;
  uint32_t seed_first, key0, key1;
  int chunk;                 // mixed kernel: steps per FP32 chunk (multiple of 32)
  const jne_chunk_time* chunk_tab;  // mixed kernel, one entry per chunk
  const double* ext;         // explicit increments [run][step][dim] (already scaled), or null
  double ext_inv_scale;      // mixed kernel: z = dB * ext_inv_scale when reading ext
  double* mom;               // moment records, SoA
  long long mom_ld;          // leading dimension (>= n_runs)
  unsigned int* status;      // device status word (bit flags), may be null
  unsigned long long* next_run;  // mixed kernel: zeroed work counter for dynamic run
                                 // assignment, or null for a fixed stride per warp
  unsigned int* batch_done;      // mixed kernel with a fused finalize: zeroed count of
                                 // accumulated runs per 32-run batch (ceil(n_runs / 32))
  int blocks_per_sm;             // mixed kernel variant: 4 (0 = default) or 6
  int pack;                      // mixed kernel, dims <= 4: >= 0 two runs per warp, < 0 one
};

// Status bits a kernel may raise (never a trap).
#define JNE_DEV_BAD_ARGS 0x1u
#define JNE_DEV_NOT_SPD 0x2u
