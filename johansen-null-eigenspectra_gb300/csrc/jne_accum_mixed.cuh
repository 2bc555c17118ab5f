// jne_accum_mixed.cuh -- mixed-precision fused accumulation: one warp per run,
// the Gram contraction on the tensor cores (mma.sync, hi/lo split operands).
//
// Same contract as the plain FP64 kernel (it replaces rng_matrix.rs:57-141,
// johansen_statistics.rs:102-197 and the two sum_of_outer_products calls of
// johansen_statistics.rs:32-33) and writes the same FP64 moment record, always
// the full record, so one pass serves every model.
//
// Time is cut into chunks of `chunk` steps (multiple of 32).  Inside a chunk
// the walk is taken relative to its value Wc at the chunk start (origin
// shift): b_tau = W_{c0+tau} - Wc, kept in FP32 with a float-float carry.  The
// warp accumulates, in FP32 on the tensor cores, the 16 x 32 local Gram
//     sum_tau G_tau [G_tau; z_tau]',   G = [b (d rows); 1; u; u^2; 0...],
// with u = tau / chunk.  Each operand is split x = hi + lo with hi = x rounded
// to an 11-bit significand and every product is hi*hi + hi*lo + lo*hi (three
// MMAs): FP16 words and m16n8k16 for the kernel's own increments, TF32 words
// and m16n8k8 for explicit ones (see mma_split_f16).  At the chunk end the
// local Gram is mapped to the global moments (W = Wc + b, y = yc + h u) by the
// exact shift identities, summed in float-float; the record is written in FP64
// once per run.
//
// Fragment layout (PTX ISA): lane (g = lane/4, q = lane%4) holds rows g and g+8
// of A and column g of B, at k-slots q and q+4 (m16n8k8 .tf32) or 2q, 2q+1,
// 2q+8, 2q+9 (m16n8k16 .f16).  The sum over k does not depend on which time
// step a k-slot carries, so the slots of MMA s carry the lane's own steps --
// 2s, 2s+1 (TF32) or 4s..4s+3 (FP16) of its 8 consecutive steps 8q..8q+7.
// That makes the scan along time cheap, and the A fragment registers double as
// the B fragments of the G x G tiles.
#pragma once
#include <cuda_fp16.h>

#include "jne_finalize_run.cuh"

namespace {

constexpr int kMixWarps = 4;
constexpr int kZS = 36;  // z staging row stride (floats): conflict-free float4 reads
constexpr int kCS = 33;  // chunk-Gram staging row stride (floats)

// x rounded to the nearest TF32 value (ties away from zero): the low 13
// mantissa bits are zero, and x - hi is exact in FP32 with |x - hi| <= 2^-12 |x|
// -- half the remainder of truncation, so the remainder keeps one more bit
// when the tensor core truncates it to TF32 in turn.
// (Integer form: add half a TF32 ulp to the magnitude bits, clear the low 13;
// a carry into the exponent is the correct rounding.  Cheaper here than the
// conversion instruction.)
__device__ __forceinline__ uint32_t tf32_hi(float x) { return (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u; }

__device__ __forceinline__ void mma_tf32(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// d = A B (no accumulator input): starts a tile's hi*hi sum without zeroing it first.
__device__ __forceinline__ void mma_tf32_first(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                               uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%10,%10,%10,%10};\n"
      : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1), "f"(0.0f));
}

// x - y on a pair of floats in one instruction (each half rounded as the
// scalar subtraction).
__device__ __forceinline__ float2 sub_pair(float2 x, float2 y) {
  unsigned long long ux, uy, r;
  asm("mov.b64 %0, {%1,%2};" : "=l"(ux) : "f"(x.x), "f"(x.y));
  asm("mov.b64 %0, {%1,%2};" : "=l"(uy) : "f"(y.x), "f"(y.y));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(ux), "l"(uy));
  float2 d;
  asm("mov.b64 {%0,%1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(r));
  return d;
}

// The TF32 split of a pair: hi = each value rounded to TF32, lo = x - hi (exact).
__device__ __forceinline__ void split_pair(float2 x, uint32_t& h0, uint32_t& h1, uint32_t& l0, uint32_t& l1) {
  h0 = tf32_hi(x.x);
  h1 = tf32_hi(x.y);
  const float2 lo = sub_pair(x, make_float2(__uint_as_float(h0), __uint_as_float(h1)));
  l0 = __float_as_uint(lo.x);
  l1 = __float_as_uint(lo.y);
}

// C += A B on the TF32 split, A (a0..a3) and B (b0, b1) given as hi and lo
// words: the hi*hi product goes to `hh` (overwritten when FIRST), the two cross
// products to `x`.  The tensor core's FP32 accumulation truncates, so its
// error is biased and grows with the number of additions into one accumulator:
// keeping the (2^11 times smaller) cross terms apart and emptying `hh` after
// every tile keeps that bias ~10x below a single accumulator per chunk.
template <bool FIRST>
__device__ __forceinline__ void mma_split(float (&hh)[4], float (&x)[4], const uint32_t (&ah)[4],
                                          const uint32_t (&al)[4], uint32_t bh0, uint32_t bh1, uint32_t bl0,
                                          uint32_t bl1) {
  mma_tf32(x, al[0], al[1], al[2], al[3], bh0, bh1);
  mma_tf32(x, ah[0], ah[1], ah[2], ah[3], bl0, bl1);
  if (FIRST)
    mma_tf32_first(hh, ah[0], ah[1], ah[2], ah[3], bh0, bh1);
  else
    mma_tf32(hh, ah[0], ah[1], ah[2], ah[3], bh0, bh1);
}

// The same products on the FP16 split with m16n8k16 MMAs (16 steps per
// instruction, half the MMAs of the TF32 form).  FP16 has TF32's 11-bit
// significand, so hi * hi is exact as before, and the remainder lo is rounded to
// nearest by the conversion instead of truncated by the tensor core.  Its range
// is the limit (largest finite 65504, normals from 6.1e-5): it serves the
// kernel's own increments, which are bounded -- |z| <= 6.77 by the Box-Muller
// uniforms, so the chunk-local walk |b| <= 6.77 L <= 55,500 for chunks of at
// most 8192 steps, and the basis rows lie in [0, 1].  Values below the normal range
// keep an absolute error under 3e-8 through lo.  Explicit increments are
// arbitrary and keep the TF32 split (FP32 range).
__device__ __forceinline__ void mma_f16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                        uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma_f16_first(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                              uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%10,%10,%10,%10};\n"
      : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1), "f"(0.0f));
}

// The FP16 split of two consecutive steps' values of one row (an f16x2 word,
// the first step in the low half): hi = each rounded to FP16, lo = x - hi
// rounded to FP16.  x - hi is exact in FP32; it comes from one mixed-precision
// FMA per value (hi as an FP16 operand, times -1, plus x), so hi is never
// converted back to FP32 (3% less time than the conversion and a paired
// subtraction, the same bits).
__device__ __forceinline__ void split_f16x2(float x0, float x1, uint32_t& h, uint32_t& l) {
  const __half2 hh = __floats2half2_rn(x0, x1);
  h = *reinterpret_cast<const uint32_t*>(&hh);
  float lo0, lo1;
  asm("{.reg .f16 a, b, m;\n"
      " mov.b32 {a, b}, %2;\n"
      " mov.b16 m, 0xBC00;\n"  // -1.0
      " fma.rn.f32.f16 %0, a, m, %3;\n"
      " fma.rn.f32.f16 %1, b, m, %4;\n"
      "}"
      : "=f"(lo0), "=f"(lo1)
      : "r"(h), "f"(x0), "f"(x1));
  const __half2 ll = __floats2half2_rn(lo0, lo1);
  l = *reinterpret_cast<const uint32_t*>(&ll);
}

template <bool FIRST>
__device__ __forceinline__ void mma_split_f16(float (&hh)[4], float (&x)[4], const uint32_t (&ah)[4],
                                              const uint32_t (&al)[4], uint32_t bh0, uint32_t bh1, uint32_t bl0,
                                              uint32_t bl1) {
  mma_f16(x, al[0], al[1], al[2], al[3], bh0, bh1);
  mma_f16(x, ah[0], ah[1], ah[2], ah[3], bl0, bl1);
  if (FIRST)
    mma_f16_first(hh, ah[0], ah[1], ah[2], ah[3], bh0, bh1);
  else
    mma_f16(hh, ah[0], ah[1], ah[2], ah[3], bh0, bh1);
}

// Two-sum carry update: (hi, lo) += t.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float t) {
  const float s = __fadd_rn(hi, t);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(t, bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}

// Float-float arithmetic of the chunk merge (Knuth's two-sum, the FMA two-product;
// explicit round-to-nearest so no step is fused away).  A value is hi + lo with
// |lo| <= ulp(hi) / 2 after renormalisation: about 48 significant bits.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// (hi, lo) += p + t, renormalised
__device__ __forceinline__ void ff_acc(float& hi, float& lo, float p, float t) {
  float s, e;
  two_sum(hi, p, s, e);
  e = __fadd_rn(e, __fadd_rn(lo, t));
  hi = __fadd_rn(s, e);
  lo = __fsub_rn(e, __fsub_rn(hi, s));
}
// (xh + xl)(yh + yl) = p + e to about 2^-46 relative (e not renormalised)
__device__ __forceinline__ void ff_mul(float xh, float xl, float yh, float yl, float& p, float& e) {
  p = __fmul_rn(xh, yh);
  e = __fmaf_rn(xh, yh, -p);
  e = __fmaf_rn(xh, yl, e);
  e = __fmaf_rn(xl, yh, e);
}

// (hi, lo) += p + t on a pair held in shared memory: one 8-byte load and store.
__device__ __forceinline__ void slot_acc(float2& v, float p, float t) {
  float2 r = v;
  ff_acc(r.x, r.y, p, t);
  v = r;
}

// f(t) for t = lane, lane + 32, ... below N.  UNROLL: unrolled, so that the
// lane's independent slot updates overlap instead of running one after the
// other (7% of the time at T = 1000).  The ragged kernel, which holds every
// dim's code, keeps the loop: unrolled, it spills registers.
template <int N, bool UNROLL, typename F>
__device__ __forceinline__ void for_slots(int lane, F&& f) {
  if (UNROLL) {
#pragma unroll
    for (int k = 0; k < (N + 31) / 32; k++) {
      const int t = lane + 32 * k;
      if (t < N) f(t);
    }
  } else {
#pragma unroll 1
    for (int t = lane; t < N; t += 32) f(t);
  }
}

// Dims up to 4 can pack two runs into a warp (PACK): run A owns G rows 0..7,
// run B rows 8..15 (walk rows 0..DIM-1, basis rows DIM..DIM+2, then zero rows),
// so lane g holds local row g of both runs.  The three Gram blocks are then run
// A's G x G, run B's G x G and G x [z of run A | z of run B]: two runs for the
// tensor work of one, and two runs' increments per producer lane.
template <int DIM, bool PACK = true>
struct Packing {
  static constexpr bool kPair = PACK && DIM <= JNE_PACK_MAX_DIM;
  static constexpr int kRuns = kPair ? 2 : 1;
};

// One 32-step tile of one run (or of two, packed).  The staging area holds the
// tile's increments: row f = feature f (unpacked), or row 8 r + f = feature f of
// run r (packed); rows without a feature are zero.  See the file comment for
// the lane <-> (row, step) mapping.
template <int DIM, bool EXT, bool FULL, bool PACK>
__device__ __forceinline__ void tile_body(const float (*zs)[kZS], const float (*bw)[32], int g, int q, int nvalid,
                                          float cA0, float cB0, int selA, int selB, float& chiA, float& cloA,
                                          float& chiB, float& cloB, float (&acc)[3][4], float (&accx)[3][4]) {
  // Unpacked: zA = increments of row g; zB = of row 8 + (g & 3) -- the walk of
  // row g + 8 for g < 4, the B operand of Gram block 1 for g >= 4.  Packed:
  // zA = run A's feature g for g < 4, run B's feature g - 4 for g >= 4 (the B
  // operand of block 2); zB = run B's feature g & 3 (its walk for g < 4).
  constexpr bool PAIR = Packing<DIM, PACK>::kPair;
  float zA[8], zB[8];
  {
    const int ra = PAIR ? (g < 4 ? g : g + 4) : g;
    const float4 p0 = *reinterpret_cast<const float4*>(&zs[ra][8 * q]);
    const float4 p1 = *reinterpret_cast<const float4*>(&zs[ra][8 * q + 4]);
    zA[0] = p0.x; zA[1] = p0.y; zA[2] = p0.z; zA[3] = p0.w; zA[4] = p1.x; zA[5] = p1.y; zA[6] = p1.z; zA[7] = p1.w;
    if (DIM > 8 || PAIR) {
      const float4 r0 = *reinterpret_cast<const float4*>(&zs[8 + (g & 3)][8 * q]);
      const float4 r1 = *reinterpret_cast<const float4*>(&zs[8 + (g & 3)][8 * q + 4]);
      zB[0] = r0.x; zB[1] = r0.y; zB[2] = r0.z; zB[3] = r0.w; zB[4] = r1.x; zB[5] = r1.y; zB[6] = r1.z; zB[7] = r1.w;
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) zB[j] = 0.f;
    }
  }
  // lane-local exclusive prefixes pre[j] = z[0] + ... + z[j-1], the lane totals, and the exclusive scan of
  // the totals over the 4 lanes of the group
  float preA[8], preB[8];
  preA[0] = 0.f; preB[0] = 0.f; preA[1] = zA[0]; preB[1] = zB[0];
#pragma unroll
  for (int j = 2; j < 8; j++) {
    preA[j] = preA[j - 1] + zA[j - 1];
    preB[j] = preB[j - 1] + zB[j - 1];
  }
  float tA = preA[7] + zA[7], tB = preB[7] + zB[7];
  float xA = tA, xB = tB;
  {
    float yA = __shfl_up_sync(0xffffffffu, xA, 1, 4), yB = __shfl_up_sync(0xffffffffu, xB, 1, 4);
    if (q >= 1) { xA += yA; xB += yB; }
    yA = __shfl_up_sync(0xffffffffu, xA, 2, 4);
    yB = __shfl_up_sync(0xffffffffu, xB, 2, 4);
    if (q >= 2) { xA += yA; xB += yB; }
  }
  float eA = __shfl_up_sync(0xffffffffu, xA, 1, 4), eB = __shfl_up_sync(0xffffffffu, xB, 1, 4);
  if (q == 0) { eA = 0.f; eB = 0.f; }
  const float tileA = __shfl_sync(0xffffffffu, xA, 3, 4), tileB = __shfl_sync(0xffffffffu, xB, 3, 4);

  // G rows rA = g and rB = g + 8 at the lane's 8 steps: walk rows c0 = 1 plus a zero basis value, basis rows
  // c0 = 0 plus their value (1, u or u^2) at the step, from the window the producer filled
  float GA[8], GB[8];
  // the walk at the lane's first step: carry (hi + lo) + the group's exclusive prefix, folded into one float
  const float wA = chiA + (cloA + eA), wB = chiB + (cloB + eB);
  constexpr bool A_WALK_ONLY = DIM >= 8 && !PAIR;  // rows 0..7 are all walk rows
  float vA[8], vB[8];
  {
    const float4 b0 = *reinterpret_cast<const float4*>(&bw[selB][8 * q]);
    const float4 b1 = *reinterpret_cast<const float4*>(&bw[selB][8 * q + 4]);
    vB[0] = b0.x; vB[1] = b0.y; vB[2] = b0.z; vB[3] = b0.w; vB[4] = b1.x; vB[5] = b1.y; vB[6] = b1.z; vB[7] = b1.w;
    if (!A_WALK_ONLY) {
      const float4 a0 = *reinterpret_cast<const float4*>(&bw[selA][8 * q]);
      const float4 a1 = *reinterpret_cast<const float4*>(&bw[selA][8 * q + 4]);
      vA[0] = a0.x; vA[1] = a0.y; vA[2] = a0.z; vA[3] = a0.w; vA[4] = a1.x; vA[5] = a1.y; vA[6] = a1.z; vA[7] = a1.w;
    }
  }
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const float bA = j == 0 ? wA : wA + preA[j], bB = j == 0 ? wB : wB + preB[j];
    GA[j] = A_WALK_ONLY ? bA : fmaf(cA0, bA, vA[j]);
    GB[j] = fmaf(cB0, bB, vB[j]);
    if (!FULL) {
      if (8 * q + j >= nvalid) { GA[j] = 0.f; GB[j] = 0.f; }
    }
  }
  ff_add(chiA, cloA, tileA);
  ff_add(chiB, cloB, tileB);

  // Gram blocks (16 G rows x 8 columns each), unpacked:
  //   0: G x walk 0..7;  1 (DIM > 8): G x [walk 8..11 | z 8..11];  2: G x z 0..7.
  // Block 1's column g is walk row 8 + g (held as GB by lane g < 4) or z row
  // 8 + g - 4 (held as zB by lane g >= 4).  Packed: 0: G x run A's rows,
  // 1: G x run B's rows (GB), 2: G x [z of A | z of B] (zA).  Products of the
  // basis rows with themselves are known in closed form and never formed.
  constexpr bool BLOCK1 = DIM > 8 || PAIR;
  float BB[8];
#pragma unroll
  for (int j = 0; j < 8; j++) BB[j] = (PAIR || g < 4) ? GB[j] : zB[j];
  float hh[3][4];
  if (!BLOCK1)
#pragma unroll
    for (int r = 0; r < 4; r++) hh[1][r] = 0.f;
  if (EXT) {
    // TF32 split, m16n8k8: MMA s carries the lane's steps 2s (k-slot q) and 2s + 1 (q + 4)
#pragma unroll
    for (int s = 0; s < 4; s++) {
      const int j0 = 2 * s, j1 = 2 * s + 1;
      // A: rows g, g + 8 at steps j0 (a0, a1) and j1 (a2, a3); block 0's B is rows g of A: (a0, a2)
      uint32_t ah[4], al[4], b1h0, b1h1, b1l0, b1l1, b2h0, b2h1, b2l0, b2l1;
      split_pair(make_float2(GA[j0], GB[j0]), ah[0], ah[1], al[0], al[1]);
      split_pair(make_float2(GA[j1], GB[j1]), ah[2], ah[3], al[2], al[3]);
      if (BLOCK1) split_pair(make_float2(BB[j0], BB[j1]), b1h0, b1h1, b1l0, b1l1);
      split_pair(make_float2(zA[j0], zA[j1]), b2h0, b2h1, b2l0, b2l1);
      if (s == 0) {
        mma_split<true>(hh[0], accx[0], ah, al, ah[0], ah[2], al[0], al[2]);
        if (BLOCK1) mma_split<true>(hh[1], accx[1], ah, al, b1h0, b1h1, b1l0, b1l1);
        mma_split<true>(hh[2], accx[2], ah, al, b2h0, b2h1, b2l0, b2l1);
      } else {
        mma_split<false>(hh[0], accx[0], ah, al, ah[0], ah[2], al[0], al[2]);
        if (BLOCK1) mma_split<false>(hh[1], accx[1], ah, al, b1h0, b1h1, b1l0, b1l1);
        mma_split<false>(hh[2], accx[2], ah, al, b2h0, b2h1, b2l0, b2l1);
      }
    }
  } else {
    // FP16 split, m16n8k16: MMA s carries the lane's steps 4s, 4s + 1 (k-slots 2q, 2q + 1) and
    // 4s + 2, 4s + 3 (2q + 8, 2q + 9)
#pragma unroll
    for (int s = 0; s < 2; s++) {
      const int j = 4 * s;
      // A words: row g at steps j, j+1; row g+8 at j, j+1; row g at j+2, j+3; row g+8 at j+2, j+3.
      // Block 0's B is rows g of A: words 0 and 2.
      uint32_t ah[4], al[4], b1h0, b1h1, b1l0, b1l1, b2h0, b2h1, b2l0, b2l1;
      split_f16x2(GA[j], GA[j + 1], ah[0], al[0]);
      split_f16x2(GB[j], GB[j + 1], ah[1], al[1]);
      split_f16x2(GA[j + 2], GA[j + 3], ah[2], al[2]);
      split_f16x2(GB[j + 2], GB[j + 3], ah[3], al[3]);
      if (BLOCK1) {
        split_f16x2(BB[j], BB[j + 1], b1h0, b1l0);
        split_f16x2(BB[j + 2], BB[j + 3], b1h1, b1l1);
      }
      split_f16x2(zA[j], zA[j + 1], b2h0, b2l0);
      split_f16x2(zA[j + 2], zA[j + 3], b2h1, b2l1);
      if (s == 0) {
        mma_split_f16<true>(hh[0], accx[0], ah, al, ah[0], ah[2], al[0], al[2]);
        if (BLOCK1) mma_split_f16<true>(hh[1], accx[1], ah, al, b1h0, b1h1, b1l0, b1l1);
        mma_split_f16<true>(hh[2], accx[2], ah, al, b2h0, b2h1, b2l0, b2l1);
      } else {
        mma_split_f16<false>(hh[0], accx[0], ah, al, ah[0], ah[2], al[0], al[2]);
        if (BLOCK1) mma_split_f16<false>(hh[1], accx[1], ah, al, b1h0, b1h1, b1l0, b1l1);
        mma_split_f16<false>(hh[2], accx[2], ah, al, b2h0, b2h1, b2l0, b2l1);
      }
    }
  }
  // empty the tile's hi*hi accumulator into the chunk sum (round to nearest)
#pragma unroll
  for (int n = 0; n < 3; n++)
#pragma unroll
    for (int r = 0; r < 4; r += 2) {
      const float2 v = __fadd2_rn(make_float2(acc[n][r], acc[n][r + 1]), make_float2(hh[n][r], hh[n][r + 1]));
      acc[n][r] = v.x;
      acc[n][r + 1] = v.y;
    }
}

// Per-warp shared memory of the accumulation (sized for the largest dim).
constexpr int kRecMax = JNE_MAX_DIM * (JNE_MAX_DIM + 1) / 2 + 6 * JNE_MAX_DIM + JNE_MAX_DIM * JNE_MAX_DIM;
struct alignas(16) WarpSmem {
  float zs[16][kZS];      // increments of the current tile: z[feature][step]
  float bw[4][32];        // basis rows at the current tile's steps: 0, 1, u, u^2
  float cm[16][kCS];      // the chunk's local Gram, staged for the merge
  // float-float values are (hi, lo) pairs
  float2 wc[16];           // walk at the chunk start
  float2 tz[16];           // chunk increment totals
  float2 rec[kRecMax];     // the run's record
  float2 mm[16];           // per feature: chunk mean m of the walk
  float2 lm[16];           // Lc * m
  float sbf[16], tzfs[16], cub[16], cuub[16], cuz[16], cuuz[16];
  unsigned short mww_pr[JNE_MAX_DIM * (JNE_MAX_DIM + 1) / 2];
};

// Lanes that own a walk feature in the merge: lane f < DIM, or (packed) lane
// 8 r + f of run r.
template <int DIM, bool PACK>
__device__ __forceinline__ bool lane_feature_of(int lane) {
  return Packing<DIM, PACK>::kPair ? (lane < 16 && (lane & 7) < DIM) : lane < DIM;
}

// One unit of a request: run `unit`, or (packed dims) runs 2 unit and
// 2 unit + 1 -- the second only if the request has it: accumulate their moment
// records into a.mom[slot * a.mom_ld + run].  Executed by a whole warp.
template <int DIM, bool EXT, bool UNROLL = true, bool PACK = true>
__device__ __forceinline__ void accum_unit(const jne_accum_args& a, int unit, WarpSmem& sm, const jne_round_keys& rk,
                                           int lane) {
  constexpr int d = DIM;
  constexpr bool PAIR = Packing<DIM, PACK>::kPair;
  constexpr int NU = Packing<DIM, PACK>::kRuns;
  constexpr int NQ = (d + 3) / 4;
  constexpr int NMWW = d * (d + 1) / 2, NMW = 3 * d, NNZW = d * d;
  constexpr int NREC = NMWW + NMW + NNZW + 3 * d;  // == jne_record_slots(d)
  static_assert(NU * NREC <= kRecMax, "records of a unit fit the shared record");
  const int g = lane >> 2, q = lane & 3;
  const int run0 = NU * unit;
  const int nrun = min(NU, a.n_runs - run0);
  float (*zs)[kZS] = sm.zs;
  float (*cm)[kCS] = sm.cm;
  float2* wc = sm.wc;
  float2* tz = sm.tz;
  float2* rec = sm.rec;
  float2* mm = sm.mm;
  float2* lm = sm.lm;
  float* sbf = sm.sbf;
  float* tzfs = sm.tzfs;
  float* cub = sm.cub;
  float* cuub = sm.cuub;
  float* cuz = sm.cuz;
  float* cuuz = sm.cuuz;
  unsigned short* mww_pr = sm.mww_pr;

  // staging rows without a feature stay zero; (p, r) of the walk moments
  for (int e = lane; e < 16 * kZS; e += 32) {
    const int row = e / kZS;
    if ((PAIR ? (row & 7) : row) >= d) (&zs[0][0])[e] = 0.f;
  }
  for (int e = lane; e < NMWW; e += 32) {
    int t = e, aa = 0;
    while (t >= d - aa) { t -= d - aa; aa++; }
    mww_pr[e] = (unsigned short)(aa | ((aa + t) << 8));
  }
  // G-row coefficients: value = c[0]*b + c[1] + c[2]*u + c[3]*u^2 (packed: the
  // lane's rows g and g + 8 are local row g of runs A and B)
  // the lane's rows: walk rows take c0 = 1 and the zero basis row (0); the basis rows take c0 = 0 and the
  // window row of their value: 1 (1), u (2), u^2 (3)
  const int rowA = g, rowB = PAIR ? g : g + 8;
  const float cA0 = rowA < d ? 1.f : 0.f, cB0 = rowB < d ? 1.f : 0.f;
  const int selA = rowA == d ? 1 : rowA == d + 1 ? 2 : rowA == d + 2 ? 3 : 0;
  const int selB = rowB == d ? 1 : rowB == d + 1 ? 2 : rowB == d + 2 ? 3 : 0;
  sm.bw[0][lane] = 0.f;
  sm.bw[1][lane] = 1.f;
  const int T = a.steps, L = a.chunk;
  const float invL = 1.0f / (float)L;
  const float invTf = 1.0f / (float)T;
  const uint32_t seed0 = a.seed_first + (uint32_t)run0;
  for (int e = lane; e < NU * NREC; e += 32) {
    rec[e] = make_float2(0.f, 0.f);
  }
  if (lane < 16) {
    wc[lane] = make_float2(0.f, 0.f);
  }
  __syncwarp();

  for (int c0 = 0; c0 < T; c0 += L) {
    const int Lc = min(L, T - c0);
    float acc[3][4], accx[3][4];  // chunk sums: hi*hi (emptied per tile) and cross terms
#pragma unroll
    for (int n = 0; n < 3; n++)
#pragma unroll
      for (int r = 0; r < 4; r++) {
        acc[n][r] = 0.f;
        accx[n][r] = 0.f;
      }
    float chiA = 0.f, cloA = 0.f, chiB = 0.f, cloB = 0.f;

    for (int t0 = c0; t0 < c0 + Lc; t0 += 32) {
      // producer: lane = tile step, all d increments of column t0 + lane of each run
      const int i = t0 + lane;
      const bool valid = i < T;
#pragma unroll
      for (int r = 0; r < NU; r++) {
        const int row0 = 8 * r;
        if (EXT) {
          const bool ok = valid && r < nrun;
          const double* src = a.ext + ((size_t)(run0 + (ok ? r : 0)) * T + (ok ? i : 0)) * d;
#pragma unroll
          for (int f = 0; f < d; f++) zs[row0 + f][lane] = ok ? (float)(src[f] * a.ext_inv_scale) : 0.f;
        } else {
#pragma unroll
          for (int j = 0; j < NQ; j++) {
            float z[4];
            jne_normal_quad((uint32_t)(i + 1), (uint32_t)j, seed0 + (uint32_t)r, rk, z);
#pragma unroll
            for (int e = 0; e < 4; e++)
              if (4 * j + e < d) zs[row0 + 4 * j + e][lane] = z[e];
          }
          if (!valid)
#pragma unroll
            for (int f = 0; f < d; f++) zs[row0 + f][lane] = 0.f;
        }
      }
      {  // the basis rows at this tile's steps: u = (step - chunk start) / L
        const float u = __fmul_rn((float)(i - c0), invL);
        sm.bw[2][lane] = u;
        sm.bw[3][lane] = __fmul_rn(u, u);
      }
      __syncwarp();
      const int nvalid = min(32, T - t0);
      if (nvalid == 32)
        tile_body<DIM, EXT, true, PACK>(zs, sm.bw, g, q, nvalid, cA0, cB0, selA, selB, chiA, cloA, chiB, cloB, acc,
                                        accx);
      else
        tile_body<DIM, EXT, false, PACK>(zs, sm.bw, g, q, nvalid, cA0, cB0, selA, selB, chiA, cloA, chiB, cloB, acc,
                                         accx);
      __syncwarp();
    }

    // ---- chunk end: stage the local Gram (cm[row][col]; row 8 r + local row of
    //      run r when packed; col < 16: walk column, 16 + f: increment f) and the
    //      chunk totals ----
    if (PAIR) {
      cm[g][2 * q] = acc[0][0] + accx[0][0];          // run A: block 0, rows 0..7
      cm[g][2 * q + 1] = acc[0][1] + accx[0][1];
      cm[g + 8][2 * q] = acc[1][2] + accx[1][2];      // run B: block 1, rows 8..15
      cm[g + 8][2 * q + 1] = acc[1][3] + accx[1][3];
      const int zr = q < 2 ? g : g + 8, zc = 16 + 2 * (q & 1);  // block 2: [z of A | z of B]
      cm[zr][zc] = (q < 2 ? acc[2][0] + accx[2][0] : acc[2][2] + accx[2][2]);
      cm[zr][zc + 1] = (q < 2 ? acc[2][1] + accx[2][1] : acc[2][3] + accx[2][3]);
    } else {
#pragma unroll
      for (int n = 0; n < 3; n++) {
        if (n == 1 && DIM <= 8) continue;
        const int col = n == 0 ? 2 * q : n == 2 ? 16 + 2 * q : (q < 2 ? 8 + 2 * q : 20 + 2 * q);
        cm[g][col] = acc[n][0] + accx[n][0];
        cm[g][col + 1] = acc[n][1] + accx[n][1];
        cm[g + 8][col] = acc[n][2] + accx[n][2];
        cm[g + 8][col + 1] = acc[n][3] + accx[n][3];
      }
    }
    if (q == 0) {
      float th, tl;
      if (g < d) {
        two_sum(chiA, cloA, th, tl);
        tz[g] = make_float2(th, tl);
      }
      if (PAIR ? g < d : g + 8 < d) {
        two_sum(chiB, cloB, th, tl);
        tz[g + 8] = make_float2(th, tl);
      }
    }
    __syncwarp();
    // ---- merge into the runs' records: W = m + beta (m = chunk mean of W, sum beta = 0),
    //      y = ybar + h (u - ubar).  Every moment splits into a "mean" part, a product of
    //      chunk means (float-float), and a centred local part (FP32, small); both are
    //      summed across chunks in float-float.  No FP64 instruction: on this GPU one warp's
    //      FP64 instruction holds the FP64 pipe for ~75 cycles, and the merge would be
    //      bound by it on short chunks.  Per-feature values of run r live at index
    //      8 r + f. ----
    const jne_chunk_time ct = a.chunk_tab[c0 / L];
    const float Lcf = (float)Lc, invLcf = 1.0f / Lcf;
    const float P1f = 0.5f * Lcf * (Lcf - 1.0f) * invL;
    const float P2f = (Lcf - 1.0f) * Lcf * (2.0f * Lcf - 1.0f) * invL * invL * (1.0f / 6.0f);
    const float ub = P1f * invLcf;                 // mean of u over the chunk
    const float sig2 = P2f - P1f * ub;             // sum of (u - ubar)^2
    const float qbar = sig2 * invLcf;              // mean of (u - ubar)^2
    const float hf = (float)L * invTf, ybf = ct.ybar_hi;
    const int lf = PAIR ? (lane & 7) : lane, lr0 = PAIR ? (lane & 8) : 0;  // lane's feature and its run's row 0
    const bool lane_feature = lane_feature_of<DIM, PACK>(lane);
    if (lane_feature) {
      const int f = lf, x = lane;
      const float Sb = cm[lr0 + d][f], Sub = cm[lr0 + d + 1][f], Suub = cm[lr0 + d + 2][f];
      const float Suz = cm[lr0 + d + 1][16 + f], Suuz = cm[lr0 + d + 2][16 + f];
      // m = wc + Sb / Lc: the quotient with its exact remainder
      const float qh = __fmul_rn(Sb, ct.inv_lc);
      const float ql = __fmul_rn(__fmaf_rn(-qh, ct.lc, Sb), ct.inv_lc);
      const float2 w0 = wc[x];
      float mh = w0.x, ml = w0.y;
      ff_acc(mh, ml, qh, ql);
      mm[x] = make_float2(mh, ml);
      float ph, pe;
      ff_mul(mh, ml, ct.lc, 0.f, ph, pe);
      float lh, ll = 0.f;
      two_sum(ph, pe, lh, ll);
      lm[x] = make_float2(lh, ll);
      const float tzf = tz[x].x;
      sbf[x] = Sb;
      tzfs[x] = tzf;
      cub[x] = Sub - ub * Sb;                                              // sum (u-ubar) beta
      cuub[x] = Suub - 2.0f * ub * Sub + ub * ub * Sb - Sb * invLcf * sig2;  // sum (u-ubar)^2 beta
      cuz[x] = Suz - ub * tzf;                                             // sum (u-ubar) z
      cuuz[x] = Suuz - 2.0f * ub * Suz + ub * ub * tzf - qbar * tzf;       // sum ((u-ubar)^2 - qbar) z
    }
    __syncwarp();
    // record slots, in order: MWW | MW1 MWy MWyy | NzW | Nz1 (from wc at the end) | Nzy Nzyy.
    // One loop per slot kind, so the lanes of an iteration take one path.
    const float c1y = hf, c2y = 2.0f * ybf * hf, c2yy = hf * hf;  // y and y^2 coefficients
    for_slots<NU * NMWW, UNROLL>(lane, [&](int t) {
      const int r = NU == 1 ? 0 : t / NMWW, e = t - r * NMWW, o = 8 * r;
      const int p = o + (mww_pr[e] & 0xff), c = mww_pr[e] >> 8;
      const float2 x = lm[p], y = mm[o + c];
      float ph, pe;
      ff_mul(x.x, x.y, y.x, y.y, ph, pe);
      slot_acc(rec[r * NREC + e], ph, __fadd_rn(pe, cm[p][c] - sbf[p] * sbf[o + c] * invLcf));
    });
    for_slots<NU * NMW, UNROLL>(lane, [&](int t) {
      const int r = NU == 1 ? 0 : t / NMW, tt = t - r * NMW, pp = tt / d, x = 8 * r + tt - pp * d;
      const int e = r * NREC + NMWW + tt;
      const float wh = pp == 0 ? 1.f : pp == 1 ? ct.ybar_hi : ct.y2bar_hi;
      const float wl = pp == 0 ? 0.f : pp == 1 ? ct.ybar_lo : ct.y2bar_lo;
      const float a1 = pp == 0 ? 0.f : pp == 1 ? c1y : c2y, a2 = pp == 2 ? c2yy : 0.f;
      float ph, pe;
      const float2 v = lm[x];
      ff_mul(wh, wl, v.x, v.y, ph, pe);
      slot_acc(rec[e], ph, __fadd_rn(pe, a1 * cub[x] + a2 * cuub[x]));
    });
    for_slots<NU * NNZW, UNROLL>(lane, [&](int t) {
      const int r = NU == 1 ? 0 : t / NNZW, tt = t - r * NNZW, za = tt / d, wb = tt - za * d, o = 8 * r;
      const int e = r * NREC + NMWW + NMW + tt;
      float ph, pe;
      const float2 x = tz[o + za], y = mm[o + wb];
      ff_mul(x.x, x.y, y.x, y.y, ph, pe);
      slot_acc(rec[e], ph, __fadd_rn(pe, cm[o + wb][16 + za] - tzfs[o + za] * sbf[o + wb] * invLcf));
    });
    for_slots<NU * 2 * d, UNROLL>(lane, [&](int t) {
      const int r = NU == 1 ? 0 : t / (2 * d), tt = t - r * 2 * d, pp = tt / d, x = 8 * r + tt - pp * d;
      const int e = r * NREC + NMWW + NMW + NNZW + d + tt;
      const float wh = pp == 0 ? ct.ybar_hi : ct.y2bar_hi, wl = pp == 0 ? ct.ybar_lo : ct.y2bar_lo;
      const float a1 = pp == 0 ? c1y : c2y, a2 = pp == 0 ? 0.f : c2yy;
      float ph, pe;
      const float2 v = tz[x];
      ff_mul(wh, wl, v.x, v.y, ph, pe);
      slot_acc(rec[e], ph, __fadd_rn(pe, a1 * cuz[x] + a2 * cuuz[x]));
    });
    __syncwarp();
    if (lane_feature) {
      float2 w = wc[lane];
      const float2 v = tz[lane];
      ff_acc(w.x, w.y, v.x, v.y);
      wc[lane] = w;
    }
    __syncwarp();
  }

  // ---- write the records (slot order of jne_common.cuh) in FP64 ----
  if (lane_feature_of<DIM, PACK>(lane)) {
    const int r = PAIR ? lane >> 3 : 0, f = PAIR ? (lane & 7) : lane;
    rec[r * NREC + jne_slot_Nz1(f, d)] = wc[lane];
  }
  __syncwarp();
  const size_t ld = (size_t)a.mom_ld;
  for (int t = lane; t < NU * NREC; t += 32) {
    const int r = t / NREC, e = t - r * NREC;
    if (r < nrun) a.mom[(size_t)e * ld + run0 + r] = (double)rec[t].x + (double)rec[t].y;
  }
  __syncwarp();
}

// Fused finalize.  Units (runs, or packed pairs of runs) are counted per batch
// of 32 consecutive items; the warp that accumulates the last unit of a batch
// finalizes the whole batch, one unit per lane, in FP64 -- a pipe the accumulation leaves idle, so the
// finalize runs in the shadow of the other warps' accumulation instead of in a
// second kernel after it.  Every batch is full except the very last, and a
// lane's record reads are contiguous with its neighbours'.  Ordering: the
// writers fence their record slots before the count, the finalizing warp
// fences after it and reads the records from L2.  Returns the first item of
// the batch to finalize, or -1.
__device__ __forceinline__ long long batch_complete(unsigned int* batch_done, long long item, long long total,
                                                    int lane) {
  __threadfence();
  __syncwarp();
  unsigned int seen = 0;
  if (lane == 0) seen = atomicAdd(&batch_done[item >> 5], 1u);
  seen = __shfl_sync(0xffffffffu, seen, 0);
  const long long first = item & ~31ll;
  const long long cnt = total - first < 32 ? total - first : 32;
  if ((long long)seen != cnt - 1) return -1;
  __threadfence();
  return first;
}

// The finalize of one unit's runs (one, or a packed pair).
__device__ __forceinline__ void finalize_unit(const jne_finalize_args& fin, long long unit, bool pack) {
  const int nu = pack && fin.dim <= JNE_PACK_MAX_DIM ? 2 : 1;
  for (int r = 0; r < nu; r++) {
    const long long run = nu * unit + r;
    if (run < fin.n_runs) jne_fin::finalize_run(fin, (int)run);
  }
}

// One request: every warp strides over its units.  The round keys arrive as a
// kernel parameter (computed on the host): the Philox rounds read them from
// the parameter bank instead of holding 20 registers.  With fin.out set, the
// kernel also finalizes its runs (fin describes the same request).
// MINB: blocks per SM the registers are budgeted for (4: 128 registers a
// thread, 6: 80); PACK: two runs per warp for dims up to 4.  Both are speed
// knobs only: a run's arithmetic is the same in every variant.
template <int DIM, bool EXT, int MINB, bool PACK>
__global__ void __launch_bounds__(kMixWarps * JNE_WARP, MINB)
    k_accum_mixed(const __grid_constant__ jne_accum_args a, const __grid_constant__ jne_round_keys rk,
                  const __grid_constant__ jne_finalize_args fin) {
  __shared__ WarpSmem sm_all[kMixWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nwarps = gridDim.x * kMixWarps;
  const bool fused = fin.out != nullptr && a.batch_done != nullptr;
  const long long units = jne_units(DIM, a.n_runs, PACK);
  auto finalize_batch = [&](long long unit) {
    const long long first = batch_complete(a.batch_done, unit, units, lane);
    if (first >= 0 && first + lane < units) finalize_unit(fin, first + lane, PACK);
    __syncwarp();
  };
  if (a.next_run == nullptr) {
    for (long long unit = blockIdx.x * kMixWarps + wib; unit < units; unit += nwarps) {
      accum_unit<DIM, EXT, true, PACK>(a, (int)unit, sm_all[wib], rk, lane);
      if (fused) finalize_batch(unit);
    }
  } else {
    // first unit by warp index, then the next free one from the counter
    for (long long unit = blockIdx.x * kMixWarps + wib; unit < units;) {
      accum_unit<DIM, EXT, true, PACK>(a, (int)unit, sm_all[wib], rk, lane);
      if (fused) finalize_batch(unit);
      unsigned long long item = 0;
      if (lane == 0) item = atomicAdd(a.next_run, 1ull);
      unit = nwarps + (long long)__shfl_sync(0xffffffffu, item, 0);
    }
  }
}

// Persistent grid: exactly the resident blocks, or fewer when the batch is small.
template <typename K>
int resident_grid(K kernel, int threads, size_t shm, int sms, long long n_runs, int warps_per_block) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, shm) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const long long needed = (n_runs + warps_per_block - 1) / warps_per_block;
  const long long full = (long long)per_sm * sms;
  return (int)(needed < full ? needed : full);
}

// Launch of one request on the kernel set compiled for MINB blocks per SM and
// EXT (explicit increments, packed dims always packed).  Packed dims run packed
// unless a.pack < 0.
template <int DIM, int MINB, bool EXT>
cudaError_t launch_dim(const jne_accum_args& a, const jne_finalize_args& fin, int sms, cudaStream_t st) {
  const int threads = kMixWarps * JNE_WARP;
  const jne_round_keys rk = jne_make_round_keys(a.key0, a.key1);
  const bool pack = a.pack >= 0;
  if (EXT) {
    auto k = k_accum_mixed<DIM, true, MINB, true>;
    k<<<resident_grid(k, threads, 0, sms, jne_units(DIM, a.n_runs, true), kMixWarps), threads, 0, st>>>(a, rk, fin);
  } else if (pack || DIM > JNE_PACK_MAX_DIM) {
    auto k = k_accum_mixed<DIM, false, MINB, true>;
    k<<<resident_grid(k, threads, 0, sms, jne_units(DIM, a.n_runs, true), kMixWarps), threads, 0, st>>>(a, rk, fin);
  } else {
    auto k = k_accum_mixed<DIM, false, MINB, false>;
    k<<<resident_grid(k, threads, 0, sms, jne_units(DIM, a.n_runs, false), kMixWarps), threads, 0, st>>>(a, rk, fin);
  }
  return cudaGetLastError();
}

template <int MINB, bool EXT>
cudaError_t launch_mixed(const jne_accum_args& a, const jne_finalize_args* fin, int sms, cudaStream_t st) {
  if (a.n_runs <= 0) return cudaSuccess;
  if (a.chunk <= 0 || a.chunk % 32 != 0) return cudaErrorInvalidValue;
  jne_finalize_args f{};  // out == nullptr: accumulation only
  if (fin) f = *fin;
  switch (a.dim) {
    case 1: return launch_dim<1, MINB, EXT>(a, f, sms, st);
    case 2: return launch_dim<2, MINB, EXT>(a, f, sms, st);
    case 3: return launch_dim<3, MINB, EXT>(a, f, sms, st);
    case 4: return launch_dim<4, MINB, EXT>(a, f, sms, st);
    case 5: return launch_dim<5, MINB, EXT>(a, f, sms, st);
    case 6: return launch_dim<6, MINB, EXT>(a, f, sms, st);
    case 7: return launch_dim<7, MINB, EXT>(a, f, sms, st);
    case 8: return launch_dim<8, MINB, EXT>(a, f, sms, st);
    case 9: return launch_dim<9, MINB, EXT>(a, f, sms, st);
    case 10: return launch_dim<10, MINB, EXT>(a, f, sms, st);
    case 11: return launch_dim<11, MINB, EXT>(a, f, sms, st);
    case 12: return launch_dim<12, MINB, EXT>(a, f, sms, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace
