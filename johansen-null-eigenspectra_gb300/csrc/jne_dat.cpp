// jne_dat.cpp -- EIGENVALS_V6 storage, the simulation driver with resume, and
// the percentile analyzer: the host side around the GPU path.
//
// Format (DATA_FORMAT.md, writer.rs:56-62, 242-249, 262-290):
//   header  "EIGENVALS_V6" | u8 model | u8 dim | u32 steps (LE)           18 bytes
//   record  ULEB128 u32 seed | u8 count | count x f64 (LE)
//   trailer "EOF_MARK" | u64 record count (LE) | u8 eigenvalues per record  17 bytes
#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/jne.h"
#include "jne_records.h"

namespace {

thread_local std::string g_err;

int dat_fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

const char kMagic[12] = {'E', 'I', 'G', 'E', 'N', 'V', 'A', 'L', 'S', '_', 'V', '6'};
const char kEof[8] = {'E', 'O', 'F', '_', 'M', 'A', 'R', 'K'};
constexpr size_t kHeader = 18, kTrailer = 17;

// uleb128.rs:68-87
size_t uleb_encode(uint32_t v, unsigned char* out) {
  size_t n = 0;
  do {
    unsigned char b = v & 0x7F;
    v >>= 7;
    if (v) b |= 0x80;
    out[n++] = b;
  } while (v);
  return n;
}

// uleb128.rs:102-137: 0 on success, -1 incomplete, -2 too long, -3 too large
int uleb_decode(const unsigned char* p, size_t avail, uint32_t* v, size_t* used) {
  uint32_t r = 0;
  int shift = 0;
  for (size_t i = 0; i < avail; i++) {
    if (i + 1 > 5) return -2;
    const uint32_t bits = p[i] & 0x7F;
    if (shift == 28 && bits > 0x0F) return -3;
    r |= bits << shift;
    shift += 7;
    if (!(p[i] & 0x80)) {
      *v = r;
      *used = i + 1;
      return 0;
    }
  }
  return -1;
}

void put_u32(unsigned char* p, uint32_t v) {
  for (int i = 0; i < 4; i++) p[i] = (unsigned char)(v >> (8 * i));
}
void put_u64(unsigned char* p, uint64_t v) {
  for (int i = 0; i < 8; i++) p[i] = (unsigned char)(v >> (8 * i));
}
uint32_t get_u32(const unsigned char* p) {
  uint32_t v = 0;
  for (int i = 3; i >= 0; i--) v = (v << 8) | p[i];
  return v;
}
uint64_t get_u64(const unsigned char* p) {
  uint64_t v = 0;
  for (int i = 7; i >= 0; i--) v = (v << 8) | p[i];
  return v;
}
void put_f64(unsigned char* p, double x) {
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
  std::memcpy(p, &x, 8);  // the file's byte order is the host's
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  put_u64(p, u);
#endif
}
double get_f64(const unsigned char* p) {
  const uint64_t u = get_u64(p);
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}

bool file_exists(const char* path) {
  struct stat st;
  return stat(path, &st) == 0;
}

int read_file(const char* path, std::vector<unsigned char>* buf) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return dat_fail(JNE_ERR_IO, std::string(path) + ": " + std::strerror(errno));
  std::fseek(f, 0, SEEK_END);
  const long len = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  buf->resize(len > 0 ? (size_t)len : 0);
  const size_t got = buf->empty() ? 0 : std::fread(buf->data(), 1, buf->size(), f);
  std::fclose(f);
  if (got != buf->size()) return dat_fail(JNE_ERR_IO, std::string(path) + ": short read");
  return JNE_OK;
}

// A file's header fields and record index: the seed of every record and the
// byte offset of its first eigenvalue (the values are decoded separately).
struct Parsed {
  int model = 0, dim = 0, k = 0;
  uint32_t steps = 0;
  std::vector<uint32_t> seeds;
  std::vector<size_t> vals;
};

// reader.rs:23-216.  Fast path when the EOF trailer is present (its record
// count sizes the index up front), scan otherwise.
int parse(const std::vector<unsigned char>& b, Parsed* out) {
  if (b.size() < 12 || std::memcmp(b.data(), kMagic, 12) != 0)
    return dat_fail(JNE_ERR_FORMAT, "File format error: magic header mismatch");
  if (b.size() < kHeader) return dat_fail(JNE_ERR_IO, "failed to fill whole buffer");
  out->model = b[12];
  out->dim = b[13];
  out->steps = get_u32(&b[14]);
  out->k = 0;
  if (b.size() < kHeader + kTrailer) return JNE_OK;  // header only
  const size_t n = b.size();
  size_t pos = kHeader;
  if (std::memcmp(&b[n - kTrailer], kEof, 8) == 0) {
    const uint64_t total = get_u64(&b[n - 9]);
    const int per = b[n - 1];
    // every record takes at least 2 + 8 per bytes: a count beyond that is corrupt
    if (total > (n - kHeader - kTrailer) / (2 + 8 * (size_t)std::max(per, 1)))
      return dat_fail(JNE_ERR_IO, "failed to fill whole buffer");
    out->seeds.reserve((size_t)total);
    out->vals.reserve((size_t)total);
    for (uint64_t r = 0; r < total; r++) {
      uint32_t seed;
      size_t used;
      if (uleb_decode(&b[pos], n - kTrailer - pos, &seed, &used) != 0)
        return dat_fail(JNE_ERR_IO, "failed to fill whole buffer");
      pos += used;
      if (pos >= n) return dat_fail(JNE_ERR_IO, "failed to fill whole buffer");
      const int cnt = b[pos++];
      if (cnt == 0) return dat_fail(JNE_ERR_FORMAT, "Invalid eigenvalue count: cannot be zero");
      if (cnt != per)
        return dat_fail(JNE_ERR_FORMAT, "Eigenvalue count mismatch: expected " + std::to_string(per) + ", actual " +
                                            std::to_string(cnt));
      if (pos + 8 * (size_t)cnt > n) return dat_fail(JNE_ERR_IO, "failed to fill whole buffer");
      out->seeds.push_back(seed);
      out->vals.push_back(pos);
      pos += 8 * (size_t)cnt;
    }
    out->k = per;
    return JNE_OK;
  }
  // scan read (files without a trailer: interrupted runs)
  int k = -1;
  while (pos < n) {
    uint32_t seed;
    size_t used;
    if (uleb_decode(&b[pos], n - pos, &seed, &used) != 0) break;
    if (pos + used >= n) break;
    const int cnt = b[pos + used];
    if (cnt == 0) break;  // zero count: pre-allocated blank space or a trailer
    if (pos + used + 1 + 8 * (size_t)cnt > n) break;  // incomplete record
    if (k >= 0 && cnt != k)
      return dat_fail(JNE_ERR_FORMAT, "Eigenvalue count mismatch: expected " + std::to_string(k) + ", actual " +
                                          std::to_string(cnt));
    k = cnt;
    pos += used + 1;
    out->seeds.push_back(seed);
    out->vals.push_back(pos);
    pos += 8 * (size_t)cnt;
  }
  out->k = k < 0 ? 0 : k;
  return JNE_OK;
}

// The records' eigenvalues (little-endian f64) into eigs (n x k), records
// split across host threads.
void decode_values(const std::vector<unsigned char>& b, const Parsed& p, double* eigs) {
  const size_t n = p.vals.size(), k = (size_t)p.k;
  auto work = [&](size_t lo, size_t hi) {
    for (size_t r = lo; r < hi; r++) {
      const unsigned char* src = &b[p.vals[r]];
      for (size_t j = 0; j < k; j++) eigs[r * k + j] = get_f64(src + 8 * j);
    }
  };
  const size_t hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>(std::min<size_t>(hw, 16), n / 65536 + 1);
  std::vector<std::thread> pool;
  size_t started = 0;  // a part whose thread cannot be started is decoded here (no exception leaves the C ABI)
  for (size_t t = 1; t < nt; t++) {
    try {
      pool.emplace_back(work, n * t / nt, n * (t + 1) / nt);
      started = t;
    } catch (const std::system_error&) {
      break;
    }
  }
  work(0, n / nt);
  for (size_t t = started + 1; t < nt; t++) work(n * t / nt, n * (t + 1) / nt);
  for (auto& th : pool) th.join();
}

int write_header(FILE* f, int model, int dim, uint32_t steps) {
  unsigned char h[kHeader];
  std::memcpy(h, kMagic, 12);
  h[12] = (unsigned char)model;
  h[13] = (unsigned char)dim;
  put_u32(h + 14, steps);
  return std::fwrite(h, 1, kHeader, f) == kHeader ? JNE_OK : dat_fail(JNE_ERR_IO, "header write failed");
}

int mkdirs(const std::string& dir) {
  if (dir.empty()) return JNE_OK;
  std::string cur;
  for (size_t i = 0; i <= dir.size(); i++) {
    if (i == dir.size() || dir[i] == '/') {
      if (!cur.empty() && mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST)
        return dat_fail(JNE_ERR_IO, "Failed to create data directory '" + cur + "': " + std::strerror(errno));
    }
    if (i < dir.size()) cur.push_back(dir[i]);
  }
  return JNE_OK;
}

}  // namespace

struct jne_dat_writer {
  FILE* f = nullptr;
  int64_t count = 0;
  int per_run = -1;
  int model = 0, dim = 0;
  uint32_t steps = 0;
  std::vector<char> buf;
  std::vector<unsigned char> rec;
};

namespace {

// The eigenvalue count of a record: at most 255 (u8), the same for every
// record of a file (the first one written sets it).
int check_count(jne_dat_writer* w, int k) {
  if (k > 255)
    return dat_fail(JNE_ERR_FORMAT, "Too many eigenvalues: " + std::to_string(k) + " exceeds maximum of 255");
  if (k < 0) return dat_fail(JNE_ERR_ARG, "negative eigenvalue count");
  if (w->per_run < 0) w->per_run = k;
  if (k != w->per_run)
    return dat_fail(JNE_ERR_FORMAT, "Eigenvalue count mismatch: expected " + std::to_string(w->per_run) +
                                        ", actual " + std::to_string(k) + " (model " + std::to_string(w->model) +
                                        ", dim " + std::to_string(w->dim) + ", steps " + std::to_string(w->steps) +
                                        ")");
  return JNE_OK;
}

// Writes a block of n whole records straight to the file descriptor (after
// what stdio holds), so a short write is seen here with its exact length, not
// later at close.  On a short write the file and the count stay in step:
// whole(wrote, &bytes) gives the whole records among the bytes written and
// their length, the file is cut back to their end (never a partial record),
// and they are counted.
template <typename Whole>
int write_block(jne_dat_writer* w, const unsigned char* p, size_t size, int64_t n, Whole&& whole) {
  if (std::fflush(w->f) != 0) return dat_fail(JNE_ERR_IO, std::string("write failed: ") + std::strerror(errno));
  const int fd = fileno(w->f);
  const off_t start = lseek(fd, 0, SEEK_CUR);
  size_t wrote = 0;
  int err = 0;
  while (wrote < size) {
    const ssize_t r = ::write(fd, p + wrote, size - wrote);
    if (r < 0 && errno == EINTR) continue;
    if (r <= 0) {
      err = r < 0 ? errno : EIO;
      break;
    }
    wrote += (size_t)r;
  }
  if (wrote != size) {
    size_t bytes = 0;
    const int64_t done = whole(wrote, &bytes);
    if (start >= 0 && ftruncate(fd, start + (off_t)bytes) == 0) lseek(fd, start + (off_t)bytes, SEEK_SET);
    w->count += done;
    return dat_fail(JNE_ERR_IO, "record write failed after " + std::to_string(w->count) + " records: " +
                                    std::strerror(err));
  }
  w->count += n;
  return JNE_OK;
}

}  // namespace

extern "C" {

const char* jne_dat_last_error(void) { return g_err.c_str(); }

int jne_dat_open(const char* path, int model, int dim, uint32_t steps, jne_dat_writer** out, int64_t* existing) {
  if (!path || !out) return dat_fail(JNE_ERR_ARG, "null argument");
  if (model < 0 || model > 255 || dim < 0 || dim > 255) return dat_fail(JNE_ERR_ARG, "model and dim must fit u8");
  *out = nullptr;
  if (existing) *existing = 0;
  jne_dat_writer* w = new jne_dat_writer();
  w->model = model;
  w->dim = dim;
  w->steps = steps;
  w->buf.resize(2u << 20);  // WRITE_BUFFER_CAPACITY, config.rs:9
  bool fresh = !file_exists(path);
  if (!fresh) {
    std::vector<unsigned char> b;
    Parsed p;
    int rc = read_file(path, &b);
    if (rc == JNE_OK) rc = parse(b, &p);
    if (rc == JNE_OK) {
      const char* what = nullptr;
      int have = 0, want = 0;
      if (p.model != model) { what = "Model"; have = p.model; want = model; }
      else if (p.dim != dim) { what = "Dimension"; have = p.dim; want = dim; }
      if (what) {
        delete w;
        return dat_fail(JNE_ERR_FORMAT, std::string(what) + " mismatch: file has " +
                                            (what[0] == 'M' ? "model " : "dim ") + std::to_string(have) +
                                            ", expected " + std::to_string(want));
      }
      if (p.steps != steps) {
        delete w;
        return dat_fail(JNE_ERR_FORMAT, "Steps mismatch: file has steps " + std::to_string(p.steps) +
                                            ", expected " + std::to_string(steps));
      }
      w->count = (int64_t)p.seeds.size();
      if (!p.seeds.empty()) w->per_run = p.k;
    } else if (g_err.find("magic header mismatch") != std::string::npos) {
      std::remove(path);  // incompatible format: recreate (writer.rs:116-150)
      fresh = true;
    }
    if (!fresh) {  // strip a complete trailer so appends continue the record stream (writer.rs:181-203)
      if (b.size() >= kHeader + kTrailer && std::memcmp(&b[b.size() - kTrailer], kEof, 8) == 0) {
        if (truncate(path, (off_t)(b.size() - kTrailer)) != 0) {
          delete w;
          return dat_fail(JNE_ERR_IO, std::string("truncate: ") + std::strerror(errno));
        }
      }
      w->f = std::fopen(path, "ab");
    }
  }
  if (fresh) {
    w->f = std::fopen(path, "wb");
    if (w->f && write_header(w->f, model, dim, steps) != JNE_OK) {
      std::fclose(w->f);
      w->f = nullptr;
    }
  }
  if (!w->f) {
    delete w;
    return dat_fail(JNE_ERR_IO, std::string(path) + ": " + std::strerror(errno));
  }
  std::setvbuf(w->f, w->buf.data(), _IOFBF, w->buf.size());
  if (existing) *existing = w->count;
  *out = w;
  return JNE_OK;
}

int jne_dat_append(jne_dat_writer* w, const uint32_t* seeds, const double* eigs, int64_t n, int k) {
  if (!w || (n > 0 && (!seeds || !eigs)) || n < 0) return dat_fail(JNE_ERR_ARG, "null argument");
  if (n == 0) return k < 0 || k > 255 ? check_count(w, k) : JNE_OK;
  const int crc = check_count(w, k);
  if (crc) return crc;
  // Records are encoded into one block and written with one call per block;
  // large batches are encoded by several threads, each into its own byte
  // range (record sizes differ only in the seed's ULEB128 length).
  const size_t fixed = 1 + 8 * (size_t)k;
  auto rec_size = [&](uint32_t seed) { return fixed + (size_t)jne_uleb_len(seed); };
  auto encode = [&](int64_t r0, int64_t r1, unsigned char* out) {
    for (int64_t r = r0; r < r1; r++) {
      size_t len = uleb_encode(seeds[r], out);
      out[len++] = (unsigned char)k;
      for (int j = 0; j < k; j++) put_f64(out + len + 8 * j, eigs[(size_t)r * k + j]);
      out += len + 8 * (size_t)k;
    }
  };
  const int64_t block = 1 << 20;  // records per block
  for (int64_t b0 = 0; b0 < n; b0 += block) {
    const int64_t b1 = std::min(n, b0 + block);
    const int parts = (b1 - b0) >= (1 << 16) ? (int)std::min<unsigned>(8, std::max(1u, std::thread::hardware_concurrency())) : 1;
    std::vector<size_t> off((size_t)parts + 1, 0);
    auto part_lo = [&](int p) { return b0 + (b1 - b0) * p / parts; };
    for (int p = 0; p < parts; p++) {
      size_t bytes = 0;
      for (int64_t r = part_lo(p); r < part_lo(p + 1); r++) bytes += rec_size(seeds[r]);
      off[(size_t)p + 1] = off[(size_t)p] + bytes;
    }
    w->rec.resize(off[(size_t)parts]);
    // parts run on threads; a part whose thread cannot be started is encoded
    // here instead (no exception leaves the C ABI)
    std::vector<std::thread> th;
    int started = 0;
    for (int p = 1; p < parts; p++) {
      try {
        th.emplace_back([&, p]() { encode(part_lo(p), part_lo(p + 1), w->rec.data() + off[(size_t)p]); });
        started = p;
      } catch (const std::system_error&) {
        break;
      }
    }
    encode(part_lo(0), part_lo(1), w->rec.data());
    for (int p = started + 1; p < parts; p++) encode(part_lo(p), part_lo(p + 1), w->rec.data() + off[(size_t)p]);
    for (std::thread& t : th) t.join();
    const int rc = write_block(w, w->rec.data(), w->rec.size(), b1 - b0, [&](size_t wrote, size_t* bytes) {
      int64_t whole = 0;
      for (int64_t r = b0; r < b1 && *bytes + rec_size(seeds[r]) <= wrote; r++) {
        *bytes += rec_size(seeds[r]);
        whole++;
      }
      return whole;
    });
    if (rc) return rc;
  }
  return JNE_OK;
}

int jne_dat_append_packed(jne_dat_writer* w, uint32_t seed_first, int64_t n, int k, const unsigned char* records) {
  if (!w || n < 0 || (n > 0 && !records)) return dat_fail(JNE_ERR_ARG, "null argument");
  if ((uint64_t)seed_first + (uint64_t)n > 0x100000000ull) return dat_fail(JNE_ERR_ARG, "seed range exceeds u32");
  if (n == 0) return k < 0 || k > 255 ? check_count(w, k) : JNE_OK;  // as jne_dat_append
  const int rc = check_count(w, k);
  if (rc) return rc;
  const jne_record_bands bands = jne_make_bands(seed_first, n, k);
  return write_block(w, records, (size_t)jne_records_bytes(seed_first, n, k), n, [&](size_t wrote, size_t* bytes) {
    long long start = 0;
    const long long r = wrote == 0 ? 0 : jne_record_at(bands, k, (long long)wrote, &start);
    *bytes = (size_t)start;
    return (int64_t)r;
  });
}

int jne_dat_finish(jne_dat_writer* w) {
  if (!w) return dat_fail(JNE_ERR_ARG, "null writer");
  unsigned char t[kTrailer];
  std::memcpy(t, kEof, 8);
  put_u64(t + 8, (uint64_t)w->count);
  t[16] = (unsigned char)(w->per_run < 0 ? 0 : w->per_run);
  int rc = std::fwrite(t, 1, kTrailer, w->f) == kTrailer ? JNE_OK : dat_fail(JNE_ERR_IO, "trailer write failed");
  if (std::fclose(w->f) != 0 && rc == JNE_OK) rc = dat_fail(JNE_ERR_IO, "close failed");
  delete w;
  return rc;
}

void jne_dat_abandon(jne_dat_writer* w) {
  if (!w) return;
  std::fclose(w->f);
  delete w;
}

int jne_dat_read(const char* path, int* model, int* dim, uint32_t* steps, int64_t* n, int* k, uint32_t* seeds,
                 double* eigs, int64_t cap) {
  if (!path) return dat_fail(JNE_ERR_ARG, "null path");
  std::vector<unsigned char> b;
  int rc = read_file(path, &b);
  if (rc) return rc;
  Parsed p;
  const bool want = seeds && eigs;
  if ((rc = parse(b, &p))) return rc;
  if (model) *model = p.model;
  if (dim) *dim = p.dim;
  if (steps) *steps = p.steps;
  if (n) *n = (int64_t)p.seeds.size();
  if (k) *k = p.k;
  if (want) {
    if (cap < (int64_t)p.seeds.size()) return dat_fail(JNE_ERR_ARG, "buffer too small");
    std::copy(p.seeds.begin(), p.seeds.end(), seeds);
    decode_values(b, p, eigs);
  }
  return JNE_OK;
}

}  // extern "C"

namespace {

// The .dat sink: one writer per distinct (model, dim, steps) file, and each
// request's writer.
struct DatSink {
  std::vector<jne_dat_writer*> files;
  std::vector<jne_dat_writer*> of_req;
  std::vector<uint32_t> seeds;
};

int dat_sink_write(void* user, int req, uint32_t seed_first, int64_t n, int k, const double* eigs, int status) {
  DatSink* d = static_cast<DatSink*>(user);
  if (status != JNE_OK) return status;
  d->seeds.resize((size_t)n);
  for (int64_t r = 0; r < n; r++) d->seeds[(size_t)r] = seed_first + (uint32_t)r;
  return jne_dat_append(d->of_req[(size_t)req], d->seeds.data(), eigs, n, k);
}

// the same records, packed on the GPU
int dat_sink_write_records(void* user, int req, uint32_t seed_first, int64_t n, int k, const unsigned char* records,
                           int64_t, int status) {
  DatSink* d = static_cast<DatSink*>(user);
  if (status != JNE_OK) return status;
  return jne_dat_append_packed(d->of_req[(size_t)req], seed_first, n, k, records);
}

}  // namespace

extern "C" {

int jne_dat_sink_open(const char* data_dir, const jne_request* reqs, int n_req, jne_sink* out) {
  if (!out || n_req < 0 || (n_req > 0 && !reqs)) return dat_fail(JNE_ERR_ARG, "null argument");
  out->write = nullptr;
  out->user = nullptr;
  out->write_records = nullptr;
  const std::string dir = data_dir && *data_dir ? data_dir : "data";
  int rc = mkdirs(dir);
  if (rc) return rc;
  DatSink* d = new DatSink();
  std::vector<std::string> names;
  for (int i = 0; i < n_req && rc == JNE_OK; i++) {
    char buf[4096];
    if (jne_eigen_count(reqs[i].model, reqs[i].dim) < 0 || reqs[i].dim > JNE_MAX_DIM || reqs[i].steps < 1) {
      rc = dat_fail(JNE_ERR_ARG, "bad request");
      break;
    }
    if ((rc = jne_simulation_filename(dir.c_str(), reqs[i].model, reqs[i].dim, reqs[i].steps, buf, sizeof buf)))
      break;
    const auto it = std::find(names.begin(), names.end(), std::string(buf));
    if (it != names.end()) {
      d->of_req.push_back(d->files[(size_t)(it - names.begin())]);
      continue;
    }
    jne_dat_writer* w = nullptr;
    if ((rc = jne_dat_open(buf, reqs[i].model, reqs[i].dim, (uint32_t)reqs[i].steps, &w, nullptr))) break;
    names.push_back(buf);
    d->files.push_back(w);
    d->of_req.push_back(w);
  }
  if (rc) {
    for (jne_dat_writer* w : d->files) jne_dat_abandon(w);
    delete d;
    return rc;
  }
  out->write = dat_sink_write;
  out->write_records = dat_sink_write_records;
  out->user = d;
  return JNE_OK;
}

int jne_dat_sink_close(jne_sink* sink, int finish) {
  if (!sink || !sink->user) return dat_fail(JNE_ERR_ARG, "null sink");
  DatSink* d = static_cast<DatSink*>(sink->user);
  int rc = JNE_OK;
  for (jne_dat_writer* w : d->files) {
    if (finish) {
      const int r = jne_dat_finish(w);
      if (r && rc == JNE_OK) rc = r;
    } else {
      jne_dat_abandon(w);
    }
  }
  delete d;
  sink->user = nullptr;
  sink->write = nullptr;
  sink->write_records = nullptr;
  return rc;
}

int jne_simulation_filename(const char* data_dir, int model, int dim, int steps, char* buf, size_t cap) {
  if (!buf || cap == 0) return dat_fail(JNE_ERR_ARG, "null buffer");
  const std::string dir = data_dir && *data_dir ? data_dir : "data";
  const std::string name = dir + "/eigenvalues_model" + std::to_string(model) + "_dim" + std::to_string(dim) +
                           "_steps" + std::to_string(steps) + ".dat";
  if (name.size() + 1 > cap) return dat_fail(JNE_ERR_ARG, "buffer too small");
  std::memcpy(buf, name.c_str(), name.size() + 1);
  return JNE_OK;
}

}  // extern "C"

namespace {

// The seeds 1..=num_runs still missing from a model's file (progress.rs:11-61);
// a file with other parameters is removed (it will be recreated).
int remaining_seeds(const std::string& dir, int model, int dim, int steps, int64_t num_runs, int quiet,
                    std::string* path, std::vector<uint32_t>* remaining) {
  char buf[4096];
  int rc = jne_simulation_filename(dir.c_str(), model, dim, steps, buf, sizeof buf);
  if (rc) return rc;
  *path = buf;
  std::vector<uint32_t> done;  // seeds already in the file, sorted
  if (file_exists(buf)) {
    std::vector<unsigned char> b;
    Parsed p;
    if (read_file(buf, &b) == JNE_OK && parse(b, &p) == JNE_OK) {
      if (p.model != model || p.dim != dim || p.steps != (uint32_t)steps) {
        if (!quiet) std::printf("WARNING: Existing file has incompatible parameters; recreating %s\n", buf);
        std::remove(buf);
      } else {
        done = std::move(p.seeds);
        std::sort(done.begin(), done.end());
      }
    }
  }
  // seeds 1..num_runs not in the file, by one merge walk over the sorted seeds
  remaining->clear();
  const int64_t in_range = std::lower_bound(done.begin(), done.end(), (uint64_t)num_runs + 1 > 0xFFFFFFFFull
                                                                          ? 0xFFFFFFFFu
                                                                          : (uint32_t)(num_runs + 1)) -
                           std::lower_bound(done.begin(), done.end(), 1u);
  remaining->reserve((size_t)std::max<int64_t>(0, num_runs - in_range));
  size_t d = 0;
  for (int64_t s = 1; s <= num_runs; s++) {
    while (d < done.size() && done[d] < (uint32_t)s) d++;
    if (d < done.size() && done[d] == (uint32_t)s) continue;
    remaining->push_back((uint32_t)s);
  }
  if (!quiet) {
    if (remaining->empty())
      std::printf("SUCCESS: calculation for this model already completed, skipping\n");
    else
      std::printf("Remaining %zu calculations to complete (model %d, dim %d, steps %d)\n", remaining->size(), model,
                  dim, steps);
  }
  return JNE_OK;
}

// Runs `remaining` for every model of `models` (all models share the list):
// one pass over the paths per contiguous seed range (jne_eigs_seeded_models),
// the records appended to each model's file in seed order.
int run_models(jne_context* ctx, const std::vector<int>& models, const std::vector<std::string>& paths, int dim,
               int steps, const std::vector<uint32_t>& remaining, int precision, uint64_t base_seed) {
  const size_t nm = models.size();
  std::vector<jne_dat_writer*> w(nm, nullptr);
  // Batches are written by a second thread while the next one computes (two
  // buffers): the files then cost no GPU time.  The writer owns w[] while it
  // runs; every exit path joins it first.
  std::thread writer;
  int wrc = 0;
  std::string werr;
  auto join = [&]() {
    if (writer.joinable()) writer.join();
    if (wrc) g_err = werr;  // the writer's message (errors are per thread)
    return wrc;
  };
  auto abandon = [&]() {
    join();
    for (jne_dat_writer* x : w)
      if (x) jne_dat_abandon(x);  // keep what was written; a rerun resumes
  };
  int rc;
  for (size_t m = 0; m < nm; m++)
    if ((rc = jne_dat_open(paths[m].c_str(), models[m], dim, (uint32_t)steps, &w[m], nullptr))) {
      abandon();
      return rc;
    }
  const int64_t batch = 1 << 18;
  std::vector<std::vector<double>> eig[2] = {std::vector<std::vector<double>>(nm),
                                             std::vector<std::vector<double>>(nm)};
  std::vector<double*> outs(nm);
  int cur = 0;
  for (size_t i = 0; i < remaining.size();) {
    // largest contiguous seed range starting at remaining[i], capped at `batch`
    size_t j = i + 1;
    while (j < remaining.size() && remaining[j] == remaining[j - 1] + 1 && (int64_t)(j - i) < batch) j++;
    const int64_t n = (int64_t)(j - i);
    for (size_t m = 0; m < nm; m++) {
      eig[cur][m].resize((size_t)n * jne_eigen_count(models[m], dim));
      outs[m] = eig[cur][m].data();
    }
    rc = jne_eigs_seeded_models(ctx, models.data(), (int)nm, dim, steps, base_seed, remaining[i], n, precision,
                                outs.data());
    if (rc) {
      const std::string msg = jne_last_error(ctx);
      abandon();
      g_err = msg;
      return rc;
    }
    if ((rc = join())) {
      abandon();
      return rc;
    }
    auto write_batch = [&, buf = cur, i0 = i, n]() {
      for (size_t m = 0; m < nm && !wrc; m++)
        if ((wrc = jne_dat_append(w[m], &remaining[i0], eig[buf][m].data(), n, jne_eigen_count(models[m], dim))))
          werr = g_err;
    };
    try {
      writer = std::thread(write_batch);
    } catch (const std::system_error&) {  // the thread cannot be started: write this batch here
      write_batch();
    }
    cur ^= 1;
    i = j;
  }
  if ((rc = join())) {
    abandon();
    return rc;
  }
  for (size_t m = 0; m < nm; m++) {
    jne_dat_writer* x = w[m];
    w[m] = nullptr;
    if ((rc = jne_dat_finish(x))) {
      abandon();
      return rc;
    }
  }
  return JNE_OK;
}

}  // namespace

extern "C" {

int jne_simulation_run(jne_context* ctx, const char* data_dir, int model, int dim, int steps, int64_t num_runs,
                       int precision, uint64_t base_seed, int quiet) {
  return jne_simulation_run_models(ctx, data_dir, &model, 1, dim, steps, num_runs, precision, base_seed, quiet);
}

int jne_simulation_run_models(jne_context* ctx, const char* data_dir, const int* models, int n_models, int dim,
                              int steps, int64_t num_runs, int precision, uint64_t base_seed, int quiet) {
  if (!ctx) return dat_fail(JNE_ERR_ARG, "null context");
  if (!models || n_models < 1 || n_models > 5) return dat_fail(JNE_ERR_ARG, "1..5 models required");
  for (int m = 0; m < n_models; m++) {
    if (jne_eigen_count(models[m], dim) < 0 || dim > JNE_MAX_DIM)
      return dat_fail(JNE_ERR_ARG, "bad simulation parameters");
    for (int q = 0; q < m; q++)
      if (models[q] == models[m]) return dat_fail(JNE_ERR_ARG, "a model is listed twice");
  }
  if (steps < 1 || num_runs < 0 || num_runs > 0xFFFFFFFFll) return dat_fail(JNE_ERR_ARG, "bad simulation parameters");
  const std::string dir = data_dir && *data_dir ? data_dir : "data";
  int rc = mkdirs(dir);
  if (rc) return rc;
  // models that still miss seeds, grouped by their missing-seed list: models
  // with the same list (every fresh run) share one pass over the paths
  std::vector<std::vector<uint32_t>> rem(n_models);
  std::vector<std::string> path(n_models);
  for (int m = 0; m < n_models; m++)
    if ((rc = remaining_seeds(dir, models[m], dim, steps, num_runs, quiet, &path[m], &rem[m]))) return rc;
  std::vector<bool> taken(n_models, false);
  for (int m = 0; m < n_models; m++) {
    if (taken[m] || rem[m].empty()) continue;
    std::vector<int> group;
    std::vector<std::string> gpath;
    for (int q = m; q < n_models; q++)
      if (!taken[q] && rem[q] == rem[m]) {
        taken[q] = true;
        group.push_back(models[q]);
        gpath.push_back(path[q]);
      }
    if ((rc = run_models(ctx, group, gpath, dim, steps, rem[m], precision, base_seed))) return rc;
  }
  return JNE_OK;
}

int jne_percentiles(const double* eigs, int64_t n, int k, int stat, const double* ps, int np, double* out) {
  if ((n > 0 && !eigs) || (np > 0 && (!ps || !out)) || k < 1 || n < 0 || np < 0 || (stat != 0 && stat != 1))
    return dat_fail(JNE_ERR_ARG, "bad percentile arguments");
  for (int i = 0; i < np; i++)
    if (!(ps[i] >= 0.0 && ps[i] <= 1.0)) return dat_fail(JNE_ERR_ARG, "percentiles must lie in [0, 1]");
  std::vector<double> v((size_t)n);
  int64_t nans = 0;
  for (int64_t r = 0; r < n; r++) {  // Sum / Max aggregators, simulation_analyzers.rs:26-39
    const double* e = eigs + (size_t)r * k;
    double a = stat == 0 ? 0.0 : -1.7976931348623157e308;
    for (int j = 0; j < k; j++) a = stat == 0 ? a + e[j] : std::fmax(a, e[j]);
    nans += a != a;
    v[(size_t)r] = a;
  }
  // the reference's sort (partial_cmp().unwrap(), simulation_analyzers.rs:60) panics on NaN
  if (nans) return dat_fail(JNE_ERR_NUMERIC, std::to_string(nans) + " runs have a NaN aggregate (unordered)");
  std::sort(v.begin(), v.end());
  for (int i = 0; i < np; i++) {  // simulation_analyzers.rs:4-18
    if (n == 0) {
      out[i] = NAN;
      continue;
    }
    const double rank = ps[i] * (double)(n - 1);
    const int64_t lo = (int64_t)std::floor(rank), hi = (int64_t)std::ceil(rank);
    if (lo == hi) {
      out[i] = v[(size_t)lo];
    } else {
      const double wgt = rank - (double)lo;
      out[i] = v[(size_t)lo] * (1.0 - wgt) + v[(size_t)hi] * wgt;
    }
  }
  return JNE_OK;
}

}  // extern "C"
