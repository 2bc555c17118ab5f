// Host check of jne_records.h, the closed-form record arithmetic and the per-thread body of the device
// record packer (jne_pack_chunk): for seed ranges across every ULEB128 length boundary and up to 2^32 - 1,
// record counts k from 0 to 255, and random ranges, the sizes, the record lookup of every byte and the packed
// bytes must equal a plain record-by-record encoder.  Built with sanitizers where available, so a read past
// the values or an out-of-range shift fails the run.  Prints "<cases> cases, <failures> failures".
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../../johansen-null-eigenspectra_gb300/csrc/jne_records.h"

static void encode(uint32_t a, long long n, int k, const double* e, std::vector<unsigned char>& out) {
  for (long long r = 0; r < n; r++) {
    uint32_t v = a + (uint32_t)r;
    do {
      unsigned char b = v & 0x7F;
      v >>= 7;
      if (v) b |= 0x80;
      out.push_back(b);
    } while (v);
    out.push_back((unsigned char)k);
    for (int j = 0; j < k; j++) {
      unsigned char b[8];
      std::memcpy(b, &e[r * k + j], 8);
      out.insert(out.end(), b, b + 8);
    }
  }
}

static long long cases = 0, fails = 0;

static void check(std::mt19937_64& rng, uint32_t a, long long n, int k, bool every_byte) {
  std::vector<double> e((size_t)(n * k));  // exactly the values: a read past them is caught
  for (auto& x : e) {
    const uint64_t u = rng();
    std::memcpy(&x, &u, 8);
  }
  std::vector<unsigned char> ref;
  encode(a, n, k, e.data(), ref);
  cases++;
  const long long total = jne_records_bytes(a, n, k);
  if (total != (long long)ref.size()) {
    std::printf("size a=%u n=%lld k=%d: %lld vs %zu\n", a, n, k, total, ref.size());
    fails++;
    return;
  }
  const jne_record_bands b = jne_make_bands(a, n, k);
  if (every_byte && n > 0) {
    long long pos = 0;
    for (long long r = 0; r < n; r++) {
      const long long sz = jne_uleb_len(a + (uint32_t)r) + 1 + 8LL * k;
      for (long long x = pos; x < pos + sz; x += (sz > 64 ? 7 : 1)) {
        long long st;
        if (jne_record_at(b, k, x, &st) != r || st != pos) {
          std::printf("lookup a=%u n=%lld k=%d x=%lld\n", a, n, k, x);
          fails++;
          return;
        }
      }
      pos += sz;
    }
  }
  std::vector<unsigned char> got((size_t)total);
  for (long long c = 0; c < (total + 15) >> 4; c++) {
    unsigned long long lo, hi;
    const int nb = jne_pack_chunk(n * k ? e.data() : nullptr, a, n, k, total, b, c, &lo, &hi);
    if (nb != (total - 16 * c < 16 ? (int)(total - 16 * c) : 16)) {
      std::printf("count a=%u n=%lld k=%d c=%lld\n", a, n, k, c);
      fails++;
      return;
    }
    for (int i = 0; i < nb; i++) got[(size_t)(16 * c + i)] = (unsigned char)(i < 8 ? lo >> (8 * i) : hi >> (8 * (i - 8)));
  }
  if (got != ref) {
    std::printf("bytes a=%u n=%lld k=%d\n", a, n, k);
    fails++;
  }
}

int main() {
  std::mt19937_64 rng(7);
  const uint32_t as[] = {0, 1, 100, 126, 127, 128, 129, 16380, 16383, 16384, (1u << 21) - 3, 1u << 21,
                         (1u << 28) - 2, 1u << 28, 0xFFFFFFFFu - 300, 0xFFFFFFFFu, 120, 16000, 2097000};
  const long long ns[] = {0, 1, 2, 3, 5, 17, 100, 1000, 40000};
  const int ks[] = {0, 1, 2, 12, 13, 255};
  for (uint32_t a : as)
    for (long long n : ns) {
      if ((unsigned long long)a + n > 0x100000000ull) continue;
      for (int k : ks)
        if (n * (long long)k <= 4000000) check(rng, a, n, k, n * (8LL * k + 6) < 400000);
    }
  const uint32_t edges[] = {0, 1u << 7, 1u << 14, 1u << 21, 1u << 28, 0xFFFFFFFFu};
  std::uniform_int_distribution<int> kd(0, 40), nd(0, 3000), pick(0, 5);
  for (int t = 0; t < 2000; t++) {
    long long n = nd(rng);
    const int k = kd(rng);
    uint64_t a = pick(rng) == 0 ? rng() % 0x100000000ull : (uint64_t)edges[pick(rng)] - (rng() % 2000);
    if (a > 0xFFFFFFFFull) a = 0;
    if (a + n > 0x100000000ull) n = (long long)(0x100000000ull - a);
    check(rng, (uint32_t)a, n, k, false);
  }
  std::printf("%lld cases, %lld failures\n", cases, fails);
  return fails != 0;
}
