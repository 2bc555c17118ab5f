// jne_api.cu -- the C ABI (include/jne.h): contexts, device buffers under a
// memory budget, request validation, kernel sequencing and host copies.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "jne_context.h"

using namespace jne_detail;



extern "C" {

int jne_version(void) { return 100; }

int jne_eigen_count(int model, int dim) {
  if (model < 0 || model > 4 || dim < 1) return -1;
  return (model == 1 || model == 3) ? dim + 1 : dim;
}

int jne_open(int device, unsigned long long mem_budget_bytes, jne_context** out) {
  if (!out) return JNE_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return JNE_ERR_CUDA;
  if (device < 0 || device >= ndev) return JNE_ERR_ARG;
  jne_context* c = new jne_context();
  c->device = device;
  c->budget = mem_budget_bytes ? mem_budget_bytes : (40ull << 30);
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->fin_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  for (int i = 0; i < 2 && e == cudaSuccess; i++) {
    e = cudaEventCreateWithFlags(&c->ev_acc[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fin[i], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_status, sizeof(unsigned int));
  // the asynchronous paths only clear the status in jne_sync: start from zero
  if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_next_run, sizeof(unsigned long long));
  if (e != cudaSuccess) {
    jne_close(c);
    return JNE_ERR_CUDA;
  }
  c->in_use = sizeof(unsigned int) + sizeof(unsigned long long);
  *out = c;
  return JNE_OK;
}

void jne_close(jne_context* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->fin_stream) cudaStreamSynchronize(c->fin_stream);
  if (c->stream) cudaStreamSynchronize(c->stream);
  prof_flush(c);
  for (cudaEvent_t e : c->event_pool) cudaEventDestroy(e);
  cudaFree(c->d_mom);
  cudaFree(c->d_out);
  cudaFree(c->d_ext);
  cudaFree(c->d_words);
  cudaFree(c->d_ent);
  cudaFree(c->d_ctab);
  cudaFree(c->d_status);
  cudaFree(c->d_req_status);
  cudaFree(c->d_next_run);
  cudaFree(c->d_batch);
  cudaFree(c->d_qscratch);
  if (c->ev_in) cudaEventDestroy(c->ev_in);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  for (int i = 0; i < 2; i++) {
    cudaFree(c->d_sink[i]);
    cudaFree(c->d_sink_st[i]);
    cudaFreeHost(c->h_sink[i]);
    cudaFreeHost(c->h_sink_st[i]);
    cudaFree(c->d_pack[i]);
    cudaFreeHost(c->h_pack[i]);
    if (c->ev_sink[i]) cudaEventDestroy(c->ev_sink[i]);
    cudaFree(c->d_reqs[i]);
    cudaFree(c->d_rtab[i]);
    cudaFree(c->d_counter[i]);
    cudaFree(c->d_bdone[i]);
    cudaFreeHost(c->h_reqs[i]);
    cudaFreeHost(c->h_rtab[i]);
    cudaFree(c->d_momb[i]);
    if (c->ev_acc[i]) cudaEventDestroy(c->ev_acc[i]);
    if (c->ev_fin[i]) cudaEventDestroy(c->ev_fin[i]);
  }
  if (c->fin_stream) cudaStreamDestroy(c->fin_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* jne_last_error(const jne_context* c) { return c ? c->err.c_str() : kNoCtx; }

int jne_set_chunk(jne_context* c, int chunk) {
  if (!c) return JNE_ERR_ARG;
  // at most 8192 steps: the FP16 operands of the mixed kernel then hold any chunk-local walk
  if (chunk != 0 && chunk != JNE_CHUNK_TUNED && (chunk < 32 || chunk % 32 != 0 || chunk > 8192))
    return fail(c, JNE_ERR_ARG, "chunk must be 0 (adaptive), JNE_CHUNK_TUNED or a multiple of 32 up to 8192");
  c->chunk = chunk;
  return JNE_OK;
}

int jne_set_launch_shape(jne_context* c, int blocks_per_sm, int pack) {
  if (!c) return JNE_ERR_ARG;
  if ((blocks_per_sm != 0 && blocks_per_sm != 4 && blocks_per_sm != 6) || pack < 0 || pack > 1)
    return fail(c, JNE_ERR_ARG, "blocks_per_sm must be 0, 4 or 6 and pack 0 or 1");
  c->force.blocks_per_sm = blocks_per_sm ? blocks_per_sm : 4;
  c->force.pack = pack;
  return JNE_OK;
}

int jne_profile(jne_context* c, int enable) {
  if (!c) return JNE_ERR_ARG;
  c->profiling = enable != 0;
  return JNE_OK;
}

int jne_profile_read(jne_context* c, double* ms, long long* launches, int reset) {
  if (!c) return JNE_ERR_ARG;
  prof_flush(c);
  for (int k = 0; k < JNE_KERNEL_KINDS; k++) {
    if (ms) ms[k] = c->prof_ms[k];
    if (launches) launches[k] = c->prof_n[k];
    if (reset) {
      c->prof_ms[k] = 0.0;
      c->prof_n[k] = 0;
    }
  }
  return JNE_OK;
}

int jne_eigs_from_increments(jne_context* c, int model, int dim, int steps, const double* dB, int n_runs,
                             int precision, double* out) {
  int rc = check_common(c, model, dim, steps, n_runs, precision);
  if (rc) return rc;
  if (n_runs == 0) return JNE_OK;
  if (!dB || !out) return fail(c, JNE_ERR_ARG, "null buffer");
  const int k = jne_eigen_count(model, dim);
  const size_t n_ext = (size_t)n_runs * steps * dim;
  if ((rc = ensure(c, &c->d_ext, &c->ext_cap, n_ext, "increment buffer"))) return rc;
  if ((rc = ensure(c, &c->d_mom, &c->mom_cap, (size_t)n_runs * jne_record_slots(dim), "moment buffer"))) return rc;
  if ((rc = ensure(c, &c->d_out, &c->out_cap, (size_t)n_runs * k, "output buffer"))) return rc;
  cudaStream_t st = c->stream;
  if ((rc = drain(c))) return rc;
  if ((rc = clear_status(c, st))) return rc;
  cudaError_t e = cudaMemcpyAsync(c->d_ext, dB, sizeof(double) * n_ext, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(c, e, "increment upload");
  jne_finalize_args fa = finalize_args(c, model, dim, steps, n_runs, c->d_mom, c->d_out);
  // FP64 walks the increments as given; the mixed kernel walks dB * sqrt(T)
  if (kernel_precision(precision, steps) == JNE_PREC_FP64) fa.zscale = 1.0;
  if ((rc = accumulate(c, model, dim, steps, 0, 0, 0, n_runs, precision, c->d_ext, c->d_mom, st, &fa))) return rc;
  e = cudaMemcpyAsync(out, c->d_out, sizeof(double) * n_runs * k, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(c, e, "result download");
  return check_status(c);
}

int jne_eigs_seeded_models(jne_context* c, const int* models, int n_models, int dim, int steps, uint64_t base_seed,
                           uint32_t seed_first, int64_t n_runs, int precision, double* const* outs) {
  if (!c) return JNE_ERR_ARG;
  if (!models || !outs || n_models < 1 || n_models > 5) return fail(c, JNE_ERR_ARG, "1..5 models required");
  for (int m = 0; m < n_models; m++) {
    int rc = check_common(c, models[m], dim, steps, n_runs, precision);
    if (rc) return rc;
    if (!outs[m] && n_runs) return fail(c, JNE_ERR_ARG, "null output buffer");
  }
  if ((uint64_t)seed_first + (uint64_t)n_runs > 0x100000000ull) return fail(c, JNE_ERR_ARG, "seed range exceeds u32");
  int k_total = 0;
  for (int m = 0; m < n_models; m++) k_total += jne_eigen_count(models[m], dim);
  uint32_t k0, k1;
  stream_key(base_seed, dim, &k0, &k1);
  // a single FP64 pass needs every moment any requested model uses
  const int acc_model = (n_models == 1) ? models[0] : -1;
  cudaStream_t st = c->stream;
  int rc = drain(c);
  if (rc) return rc;
  if ((rc = clear_status(c, st))) return rc;
  const int64_t per = batch_runs(c, dim, k_total);
  if (per < 1) return fail(c, JNE_ERR_BUDGET, "budget too small for one run");
  for (int64_t done = 0; done < n_runs; done += per) {
    const int n = (int)std::min<int64_t>(per, n_runs - done);
    if ((rc = ensure(c, &c->d_mom, &c->mom_cap, (size_t)n * jne_record_slots(dim), "moment buffer"))) return rc;
    if ((rc = ensure(c, &c->d_out, &c->out_cap, (size_t)n * k_total, "output buffer"))) return rc;
    // one model: the accumulation finalizes its runs itself; several: one finalize kernel per model
    // (finalizing five models per batch inside the accumulation stalls its warps longer than the
    // separate kernels take: 0.14 s against 0.08 s for 5 x 200k runs)
    const jne_finalize_args f0 = finalize_args(c, models[0], dim, steps, n, c->d_mom, c->d_out);
    if ((rc = accumulate(c, acc_model, dim, steps, k0, k1, seed_first + (uint32_t)done, n, precision, nullptr,
                         c->d_mom, st, n_models == 1 ? &f0 : nullptr)))
      return rc;
    size_t off = 0;
    for (int m = 0; m < n_models; m++) {
      const int k = jne_eigen_count(models[m], dim);
      if (n_models > 1 && (rc = finalize(c, models[m], dim, steps, n, c->d_mom, c->d_out + off, st))) return rc;
      cudaError_t e = cudaMemcpyAsync(outs[m] + (size_t)done * k, c->d_out + off, sizeof(double) * n * k,
                                      cudaMemcpyDeviceToHost, st);
      if (e != cudaSuccess) return cuda_fail(c, e, "result download");
      off += (size_t)n * k;
    }
  }
  return check_status(c);
}

int jne_eigs_seeded(jne_context* c, int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first,
                    int64_t n_runs, int precision, double* out) {
  double* outs[1] = {out};
  return jne_eigs_seeded_models(c, &model, 1, dim, steps, base_seed, seed_first, n_runs, precision, outs);
}

int jne_eigs_seeded_device(jne_context* c, int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first,
                           int64_t n_runs, int precision, double* out_device, void* stream) {
  int rc = check_common(c, model, dim, steps, n_runs, precision);
  if (rc) return rc;
  if (n_runs == 0) return JNE_OK;
  if (!out_device) return fail(c, JNE_ERR_ARG, "null output buffer");
  if ((uint64_t)seed_first + (uint64_t)n_runs > 0x100000000ull) return fail(c, JNE_ERR_ARG, "seed range exceeds u32");
  cudaStream_t user = stream ? (cudaStream_t)stream : c->stream;
  if ((rc = join_in(c, user))) return rc;
  int last = -1;
  if ((rc = enqueue_seeded(c, model, dim, steps, base_seed, seed_first, n_runs, precision, out_device, &last)))
    return rc;
  return join_out(c, user, last);
}

int jne_sync(jne_context* c) {
  if (!c) return JNE_ERR_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, JNE_ERR_CUDA, "cudaSetDevice failed");
  cudaError_t e = cudaStreamSynchronize(c->fin_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  unsigned int stv = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&stv, c->d_status, sizeof(stv), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(unsigned int));
  if (e != cudaSuccess) return cuda_fail(c, e, "sync");
  if (stv & JNE_DEV_NOT_SPD) return fail(c, JNE_ERR_NUMERIC, "S11 not positive definite for some run (NaN written)");
  return JNE_OK;
}

int jne_export_increments(jne_context* c, int dim, int steps, uint64_t base_seed, uint32_t seed_first, int n_runs,
                          double* dB_out, uint32_t* words_out) {
  int rc = check_common(c, 0, dim, steps, n_runs, JNE_PREC_FP64);
  if (rc) return rc;
  if (n_runs == 0 || (!dB_out && !words_out)) return JNE_OK;
  uint32_t k0, k1;
  stream_key(base_seed, dim, &k0, &k1);
  const size_t n_val = (size_t)n_runs * steps * dim;
  const size_t n_words = (size_t)n_runs * steps * ((dim + 3) / 4) * 4;
  if (dB_out && (rc = ensure(c, &c->d_ext, &c->ext_cap, n_val, "export buffer"))) return rc;
  if (words_out && (rc = ensure(c, &c->d_words, &c->words_cap, n_words, "word buffer"))) return rc;
  cudaStream_t st = c->stream;
  cudaError_t e;
  {
    ProfScope ps(c, JNE_KERNEL_EXPORT, st);
    e = jne_launch_export(dim, steps, n_runs, seed_first, k0, k1, 1.0 / std::sqrt((double)steps),
                          dB_out ? c->d_ext : nullptr, words_out ? c->d_words : nullptr, st);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "export launch");
  if (dB_out) {
    e = cudaMemcpyAsync(dB_out, c->d_ext, sizeof(double) * n_val, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "export download");
  }
  if (words_out) {
    e = cudaMemcpyAsync(words_out, c->d_words, sizeof(uint32_t) * n_words, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "export download");
  }
  e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? JNE_OK : cuda_fail(c, e, "export");
}

}  // extern "C"
