// jne_pack.cu -- the device-side record packer of the .dat sink: eigenvalues
// in device memory -> the byte stream of their .dat records (ULEB128 seed,
// u8 count, count x f64 LE; writer.rs:242-249, uleb128.rs:68-87), so the host
// only copies and writes bytes.
//
// Byte work, bound by memory traffic: one thread per 16 output bytes
// (jne_pack_chunk, jne_records.h), written with one 16-byte store (coalesced
// across the warp).
#include "jne_context.h"
#include "jne_records.h"

namespace {

__global__ void __launch_bounds__(256) k_pack_records(const double* __restrict__ eigs, uint4* __restrict__ out,
                                                      uint32_t a, long long n, int k, long long total,
                                                      const jne_record_bands bands) {
  const long long chunks = (total + 15) >> 4;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < chunks; c += stride) {
    unsigned long long lo, hi;
    const int nb = jne_pack_chunk(eigs, a, n, k, total, bands, c, &lo, &hi);
    if (nb == 16) {
      out[c] = make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
    } else {  // the stream's ragged end: byte stores, never past `total`
      unsigned char* o = reinterpret_cast<unsigned char*>(out) + (c << 4);
      for (int i = 0; i < nb; i++) o[i] = (unsigned char)(i < 8 ? lo >> (8 * i) : hi >> (8 * (i - 8)));
    }
  }
}

}  // namespace

cudaError_t jne_launch_pack_records(const double* eigs, unsigned char* out, uint32_t seed_first, long long n, int k,
                                    int sms, cudaStream_t st) {
  const long long total = jne_records_bytes(seed_first, n, k);
  const long long chunks = (total + 15) >> 4;
  if (chunks == 0) return cudaSuccess;
  const long long want = (chunks + 255) / 256;
  const int blocks = (int)(want < 8LL * sms ? want : 8LL * sms);
  k_pack_records<<<blocks, 256, 0, st>>>(eigs, reinterpret_cast<uint4*>(out), seed_first, n, k, total,
                                         jne_make_bands(seed_first, n, k));
  return cudaGetLastError();
}

extern "C" int64_t jne_record_bytes(uint32_t seed_first, int64_t n, int k) {
  if (n < 0 || k < 0 || k > 255 || (uint64_t)seed_first + (uint64_t)n > 0x100000000ull) return -1;
  return jne_records_bytes(seed_first, n, k);
}

extern "C" int jne_pack_records_device(jne_context* c, uint32_t seed_first, int64_t n, int k,
                                       const double* eigs_device, unsigned char* out_device, int64_t cap,
                                       void* stream) {
  using namespace jne_detail;
  if (!c) return JNE_ERR_ARG;
  const int64_t bytes = jne_record_bytes(seed_first, n, k);
  if (bytes < 0) return fail(c, JNE_ERR_ARG, "n >= 0, k in 0..255 and seeds within u32 required");
  if (bytes == 0) return JNE_OK;
  if (!out_device || (n > 0 && k > 0 && !eigs_device)) return fail(c, JNE_ERR_ARG, "null buffer");
  if (reinterpret_cast<uintptr_t>(out_device) % 16 != 0)
    return fail(c, JNE_ERR_ARG, "the record buffer must be 16-byte aligned");
  if (cap < bytes)
    return fail(c, JNE_ERR_ARG, "the records need " + std::to_string(bytes) + " bytes, the buffer holds " +
                                    std::to_string(cap));
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, JNE_ERR_CUDA, "cudaSetDevice failed");
  const cudaError_t e = jne_launch_pack_records(eigs_device, out_device, seed_first, n, k, c->sms,
                                                stream ? (cudaStream_t)stream : c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "record packer");
  return JNE_OK;
}
