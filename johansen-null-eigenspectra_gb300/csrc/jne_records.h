// jne_records.h -- sizes and byte offsets of .dat records of consecutive
// seeds, in closed form (host and device).
//
// A record is  ULEB128 u32 seed | u8 count | count x f64 (LE)  (writer.rs:242-249,
// uleb128.rs:68-87), so its size depends only on the ULEB128 length of its seed,
// which is constant between the thresholds 2^7, 2^14, 2^21 and 2^28.  For the
// seeds a, a+1, ..., a+n-1 the records therefore fall into at most five bands
// of equal-sized records, and both directions -- the bytes before record r,
// and the record that holds byte x -- take a few comparisons and one division.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define JNE_HD __host__ __device__ __forceinline__
#else
#define JNE_HD inline
#endif

// bytes of the ULEB128 encoding of a u32
JNE_HD int jne_uleb_len(uint32_t s) {
  return 1 + (s >= (1u << 7)) + (s >= (1u << 14)) + (s >= (1u << 21)) + (s >= (1u << 28));
}

// bytes of the records of seeds a .. a + r - 1, k values each (a + r <= 2^32)
JNE_HD long long jne_records_bytes(uint32_t a, long long r, int k) {
  long long b = r * (2 + 8 * (long long)k);
  const unsigned long long end = (unsigned long long)a + (unsigned long long)r;
  for (int i = 1; i <= 4; i++) {  // one more byte for every seed at or above 2^(7i)
    const unsigned long long t = 1ull << (7 * i);
    const unsigned long long lo = a > t ? a : t;
    if (end > lo) b += (long long)(end - lo);
  }
  return b;
}

// The bands of n records of seeds a..: band i holds records [r0[i], r0[i+1]),
// starting at byte b0[i], each len[i] + 1 + 8k bytes.
struct jne_record_bands {
  long long r0[6], b0[6];
  int len[5];
  int n;
};

inline jne_record_bands jne_make_bands(uint32_t a, long long n, int k) {
  jne_record_bands b{};
  long long cut[6];
  int nc = 0;
  cut[nc++] = 0;
  for (int i = 1; i <= 4; i++) {
    const unsigned long long t = 1ull << (7 * i);
    const long long r = t <= a ? 0 : (t - a < (unsigned long long)n ? (long long)(t - a) : n);
    if (r > cut[nc - 1] && r < n) cut[nc++] = r;
  }
  cut[nc++] = n;
  b.n = nc - 1;
  for (int i = 0; i < nc; i++) {
    b.r0[i] = cut[i];
    b.b0[i] = jne_records_bytes(a, cut[i], k);
  }
  for (int i = 0; i < b.n; i++) b.len[i] = jne_uleb_len(a + (uint32_t)cut[i]);
  return b;
}

// The record holding byte x (0 <= x < bytes of all the records), and its first
// byte in *start.
// (Fixed indexes only, so a kernel reads the bands from its parameters instead
// of a local copy.)
JNE_HD long long jne_record_at(const jne_record_bands& b, int k, long long x, long long* start) {
  long long r0 = b.r0[0], b0 = b.b0[0];
  int len = b.len[0];
  for (int j = 1; j < 5; j++)
    if (j < b.n && x >= b.b0[j]) {  // band starts increase: the last one at or below x holds it
      r0 = b.r0[j];
      b0 = b.b0[j];
      len = b.len[j];
    }
  const long long size = len + 1 + 8 * (long long)k;
  const unsigned long long d = (unsigned long long)(x - b0);
  // 32-bit division where the offset allows (every stream below 4 GiB): a few
  // instructions instead of the 64-bit routine
  const long long q = d < 0x100000000ull ? (long long)((uint32_t)d / (uint32_t)size)
                                         : (long long)(d / (unsigned long long)size);
  *start = b0 + q * size;
  return r0 + q;
}

// Bytes [16 c, 16 c + 16) of the n records of seeds a.. whose values are eigs
// (n x k, run-major), one byte at a time (the form for k < 2; jne_pack_chunk
// below has the arguments and results).
// The record holding the first byte comes in closed form.  The values the 16
// bytes can show are at most three consecutive f64 of eigs (the values of
// consecutive records are consecutive, and 16 bytes cannot hold bytes of
// four), so they are loaded first, together.  Every byte is then formed
// without a branch -- header byte, count or value byte chosen by selects, the
// step to the next record too -- so the lanes of a warp, each at its own place
// in a record, never take different paths.  Bytes past the stream's end are
// formed from stale state and discarded.
JNE_HD int jne_pack_chunk_bytes(const double* eigs, uint32_t a, long long n, int k, long long total,
                          const jne_record_bands& bands, long long c, unsigned long long* lo_out,
                          unsigned long long* hi_out) {
  const long long x0 = c << 4;
  long long start;
  const long long r = jne_record_at(bands, k, x0, &start);
  uint32_t seed = a + (uint32_t)r;
  int len = jne_uleb_len(seed);
  int pos = (int)(x0 - start);
  const int size_v = 1 + 8 * k;  // a record's bytes after its seed
  const int nb = total - x0 < 16 ? (int)(total - x0) : 16;
  // the first value the bytes can touch: the one under byte x0, or the first of its record
  const long long i0 = r * k + (pos > len ? (pos - len - 1) >> 3 : 0);
  const long long nv = n * k;
  unsigned long long v0 = 0, v1 = 0, v2 = 0;
#ifdef __CUDA_ARCH__
  if (i0 < nv) v0 = (unsigned long long)__double_as_longlong(__ldg(eigs + i0));
  if (i0 + 1 < nv) v1 = (unsigned long long)__double_as_longlong(__ldg(eigs + i0 + 1));
  if (i0 + 2 < nv) v2 = (unsigned long long)__double_as_longlong(__ldg(eigs + i0 + 2));
#else
  if (i0 < nv) __builtin_memcpy(&v0, eigs + i0, 8);
  if (i0 + 1 < nv) __builtin_memcpy(&v1, eigs + i0 + 1, 8);
  if (i0 + 2 < nv) __builtin_memcpy(&v2, eigs + i0 + 2, 8);
#endif
  int rel = (int)(r * k - i0);  // the current record's first value, relative to i0 (<= 0)
  unsigned long long lo = 0, hi = 0;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int i = 0; i < 16; i++) {
    const bool next = pos == len + size_v;  // past the record's end: the next record
    seed += next ? 1u : 0u;
    rel += next ? k : 0;
    len = next ? jne_uleb_len(seed) : len;
    pos = next ? 0 : pos;
    const int q = pos - len - 1;                 // value byte (when >= 0)
    const int t = rel + (q >> 3);                // its value, relative to i0 (0, 1 or 2 when q >= 0)
    const unsigned long long bits = t == 0 ? v0 : (t == 1 ? v1 : v2);
    const uint32_t vb = (uint32_t)(bits >> (8 * (q & 7))) & 0xFFu;  // little-endian bytes of the f64
    const uint32_t ub = ((seed >> (pos < 5 ? 7 * pos : 0)) & 0x7Fu) | (pos + 1 < len ? 0x80u : 0u);
    const uint32_t b = pos < len ? ub : (pos == len ? (uint32_t)k : vb);
    if (i < 8)
      lo |= (unsigned long long)b << (8 * i);
    else
      hi |= (unsigned long long)b << (8 * (i - 8));
    pos++;
  }
  *lo_out = lo;
  *hi_out = hi;
  return nb;
}

// 128-bit values as (lo, hi) 64-bit halves, shifted and masked by whole bytes
// (little-endian: byte 0 is the low byte of lo).  Selects only, no branches,
// so lanes with different counts stay on one path.
struct jne_u128 {
  unsigned long long lo, hi;
};
JNE_HD jne_u128 jne_shl_bytes(jne_u128 x, int b) {  // b >= 0; 0 for b >= 16
  const int s = 8 * (b & 7);
  unsigned long long lo = b >= 8 ? 0ull : x.lo, hi = b >= 8 ? x.lo : x.hi;
  hi = (hi << s) | (s ? lo >> (64 - s) : 0ull);
  lo <<= s;
  return {b >= 16 ? 0ull : lo, b >= 16 ? 0ull : hi};
}
JNE_HD jne_u128 jne_shr_bytes(jne_u128 x, int b) {  // b >= 0; 0 for b >= 16
  const int s = 8 * (b & 7);
  unsigned long long lo = b >= 8 ? x.hi : x.lo, hi = b >= 8 ? 0ull : x.hi;
  lo = (lo >> s) | (s ? hi << (64 - s) : 0ull);
  hi >>= s;
  return {b >= 16 ? 0ull : lo, b >= 16 ? 0ull : hi};
}
JNE_HD jne_u128 jne_low_bytes(jne_u128 x, int b) {  // bytes 0 .. b-1 of x, 0 <= b <= 16
  const unsigned long long mlo = b >= 8 ? ~0ull : (b == 0 ? 0ull : (1ull << (8 * b)) - 1);
  const unsigned long long mhi = b >= 16 ? ~0ull : (b <= 8 ? 0ull : (1ull << (8 * (b - 8))) - 1);
  return {x.lo & mlo, x.hi & mhi};
}

// A record's header -- ULEB128 seed (len bytes) and the count byte k -- as the
// low len + 1 bytes of a word.
JNE_HD unsigned long long jne_record_header(uint32_t seed, int len, int k) {
  unsigned long long h = 0;
  for (int i = 0; i < 5; i++) {
    const unsigned long long b = ((seed >> (7 * i)) & 0x7Fu) | (i + 1 < len ? 0x80u : 0u);
    h |= (i < len ? b : 0ull) << (8 * i);
  }
  return h | ((unsigned long long)(uint32_t)k << (8 * len));
}

JNE_HD unsigned long long jne_load_bits(const double* p) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(__ldg(p));
#else
  unsigned long long u;
  __builtin_memcpy(&u, p, 8);
  return u;
#endif
}

// Bytes [16 c, 16 c + 16) of the n records of seeds a.. whose values are eigs
// (n x k, run-major) -- the work of one thread of the device packer, also
// callable on the host.  Returns how many of the 16 bytes exist (16 except at
// the end of the stream, total = all the records' bytes); they are packed
// little-endian into *lo (bytes 0-7) and *hi (8-15).
// For k >= 2 a record takes more than 16 bytes, so the 16 bytes hold at most
// one record header, with consecutive bytes of the value stream around it (the
// values of consecutive records are consecutive in eigs).  Every case is then
// one formula: the first `na` bytes of the value stream from byte q, the header
// bytes (all of record r + 1's, or the rest of record r's when the 16 bytes
// start inside it: then na = 0), and the value stream again from byte q + na.
// The value-stream bytes come from three loaded values (a funnel shift); the
// per-lane parameters are chosen by selects, so the warp never diverges.
// Bytes past the stream's end are formed from values read as zero and discarded.
JNE_HD int jne_pack_chunk(const double* eigs, uint32_t a, long long n, int k, long long total,
                          const jne_record_bands& bands, long long c, unsigned long long* lo_out,
                          unsigned long long* hi_out) {
  if (k < 2) return jne_pack_chunk_bytes(eigs, a, n, k, total, bands, c, lo_out, hi_out);
  const long long x0 = c << 4;
  long long start;
  const long long r = jne_record_at(bands, k, x0, &start);
  const uint32_t seed = a + (uint32_t)r;
  const int len = jne_uleb_len(seed), hlen = len + 1;
  const int pos = (int)(x0 - start);
  const int nb = total - x0 < 16 ? (int)(total - x0) : 16;
  const long long nv = n * k;
  const bool in_hdr = pos < hlen;
  // value-stream byte of the first value byte; bytes before record r + 1's header
  const long long q = 8 * (r * k) + (in_hdr ? 0 : pos - hlen);
  const int to_next = hlen + 8 * k - pos;
  const int na = in_hdr ? 0 : (to_next < 16 ? to_next : 16);
  // the header in the 16 bytes: the rest of record r's, or record r + 1's (past the last record: discarded)
  const uint32_t hseed = in_hdr ? seed : seed + 1u;
  const int hl = in_hdr ? len : jne_uleb_len(hseed);
  const unsigned long long hbits = jne_record_header(hseed, hl, k) >> (in_hdr ? 8 * pos : 0);
  const int hb = in_hdr ? hlen - pos : hl + 1;
  const long long j0 = q >> 3;  // a value of record r
  const int sh = (int)(q & 7);
  const unsigned long long v0 = jne_load_bits(eigs + j0);
  const unsigned long long v1 = j0 + 1 < nv ? jne_load_bits(eigs + j0 + 1) : 0ull;
  const unsigned long long v2 = j0 + 2 < nv ? jne_load_bits(eigs + j0 + 2) : 0ull;
  const jne_u128 v = {(v0 >> (8 * sh)) | (sh ? v1 << (64 - 8 * sh) : 0ull),
                      (v1 >> (8 * sh)) | (sh ? v2 << (64 - 8 * sh) : 0ull)};
  const jne_u128 before = jne_low_bytes(v, na);
  const jne_u128 hdr = jne_shl_bytes(jne_u128{hbits, 0}, na);
  const jne_u128 after = jne_shl_bytes(jne_shr_bytes(v, na), na + hb);
  *lo_out = before.lo | hdr.lo | after.lo;
  *hi_out = before.hi | hdr.hi | after.hi;
  return nb;
}
