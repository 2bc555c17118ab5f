// jne_probe.cu -- pipe-rate probes: the denominators of the kernels' rooflines,
// measured on the running GPU with the same device code the kernels use.
//   rates[0]  normals/s  drawn by jne_normal_quad (Philox4x32-10 + Box-Muller)
//   rates[1]  FP64 flop/s of independent DFMA chains
//   rates[2]  flop/s of mma.sync.m16n8k8 TF32 (the mixed kernel's form for explicit increments)
//   rates[3]  FP32 flop/s of independent FFMA chains
//   rates[4]  flop/s of mma.sync.m16n8k16 FP16 with FP32 accumulation (the form for its own increments)
#include "jne_context.h"

using namespace jne_detail;

namespace {

constexpr int kProbeThreads = 256;

__global__ void k_probe_normals(float* out, int iters, jne_round_keys rk) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.f;
  for (int i = 0; i < iters; i++) {
    float z[4];
    jne_normal_quad((uint32_t)i + 1u, 0u, tid, rk, z);
    acc += (z[0] + z[1]) + (z[2] + z[3]);
  }
  out[tid] = acc;
}

__global__ void k_probe_dfma(double* out, int iters) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  double a[8];
  const double x = 1.0 + tid * 1e-9, y = 0.999999;
  for (int j = 0; j < 8; j++) a[j] = j * 0.1;
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = fma(a[j], y, x);
  double s = 0;
  for (int j = 0; j < 8; j++) s += a[j];
  out[tid] = s;
}

__global__ void k_probe_ffma(float* out, int iters) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  float a[16];
  const float x = 1.0f + tid * 1e-9f, y = 0.999999f;
  for (int j = 0; j < 16; j++) a[j] = j * 0.1f;
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int j = 0; j < 16; j++) a[j] = fmaf(a[j], y, x);
  float s = 0;
  for (int j = 0; j < 16; j++) s += a[j];
  out[tid] = s;
}

__global__ void k_probe_mma(float* out, int iters) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t a0 = 0x3f800000u ^ (tid & 0x1000u), b0 = 0x3f800000u;
  float c[8][4];
  for (int j = 0; j < 8; j++)
    for (int q = 0; q < 4; q++) c[j][q] = 0.f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++)
      asm volatile(
          "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
          "{%0,%1,%2,%3};\n"
          : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
          : "r"(a0), "r"(a0), "r"(a0), "r"(a0), "r"(b0), "r"(b0));
  }
  float s = 0;
  for (int j = 0; j < 8; j++)
    for (int q = 0; q < 4; q++) s += c[j][q];
  out[tid] = s;
}

__global__ void k_probe_mma_f16(float* out, int iters) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t a0 = 0x3c003c00u ^ (tid & 0x100u), b0 = 0x3c003c00u;  // f16x2 words near 1.0
  float c[8][4];
  for (int j = 0; j < 8; j++)
    for (int q = 0; q < 4; q++) c[j][q] = 0.f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
          "{%0,%1,%2,%3};\n"
          : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
          : "r"(a0), "r"(a0), "r"(a0), "r"(a0), "r"(b0), "r"(b0));
  }
  float s = 0;
  for (int j = 0; j < 8; j++)
    for (int q = 0; q < 4; q++) s += c[j][q];
  out[tid] = s;
}

}  // namespace

extern "C" int jne_probe_rates(jne_context* c, double* rates) {
  if (!c || !rates) return JNE_ERR_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, JNE_ERR_CUDA, "cudaSetDevice failed");
  int rc = drain(c);
  if (rc) return rc;
  const int blocks = c->sms * 8;
  const size_t n = (size_t)blocks * kProbeThreads;
  double* buf = nullptr;
  if ((rc = ensure(c, &c->d_out, &c->out_cap, n, "probe buffer"))) return rc;
  buf = c->d_out;
  cudaStream_t st = c->stream;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const jne_round_keys rk = jne_make_round_keys(0x12345u, 0x6789u);
  auto timed = [&](auto launch, double ops) -> double {
    launch(2);  // warm-up
    cudaEventRecord(a, st);
    launch(0);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms > 0.f ? ops / (ms * 1e-3) : 0.0;
  };
  const int it_n = 4000, it_d = 1000, it_m = 16000, it_f = 40000;
  rates[0] = timed([&](int w) { k_probe_normals<<<blocks, kProbeThreads, 0, st>>>((float*)buf, w ? w : it_n, rk); },
                   4.0 * it_n * n);
  rates[1] = timed([&](int w) { k_probe_dfma<<<blocks, kProbeThreads, 0, st>>>(buf, w ? w : it_d); },
                   16.0 * it_d * n);
  rates[2] = timed([&](int w) { k_probe_mma<<<blocks, kProbeThreads, 0, st>>>((float*)buf, w ? w : it_m); },
                   8.0 * 16 * 8 * 8 * 2 * it_m * n / 32.0);
  rates[3] = timed([&](int w) { k_probe_ffma<<<blocks, kProbeThreads, 0, st>>>((float*)buf, w ? w : it_f); },
                   32.0 * it_f * n);
  rates[4] = timed([&](int w) { k_probe_mma_f16<<<blocks, kProbeThreads, 0, st>>>((float*)buf, w ? w : it_m); },
                   8.0 * 16 * 8 * 16 * 2 * it_m * n / 32.0);
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "probe");
}
