/*
 * jne.h -- C ABI of the GB300 engine for the Johansen null-eigenspectra
 * Monte Carlo path (Kuan-Lun/johansen-null-eigenspectra).
 *
 * Plain C types only.  Every function returns a status code (JNE_OK = 0) and
 * writes results into caller-owned buffers.  A context is used from one host
 * thread at a time.  Eigenvalues are reported as the reference reports them:
 * |alpha|/beta of the pencil (S10'S10, S11), sorted descending, k per run with
 * k = dim + 1 for models 1 and 3 and k = dim otherwise.
 *
 * Reference interfaces replaced (paths within the reference crate):
 *   jne_eigen_count            src/data_storage/thread_manager.rs:40-44
 *   jne_eigs_from_increments   src/johansen_statistics.rs:24-85 (from the
 *                              increment matrix rather than a seed)
 *   jne_eigs_seeded(_device)   the per-seed calculate_eigenvalues calls of
 *                              src/data_storage/parallel_compute.rs:14-41
 *                              (johansen_statistics.rs:59-85 for seeds
 *                              seed_first .. seed_first + n_runs - 1)
 *   jne_eigs_seeded_models     the same, for several models of one
 *                              (dim, steps) pair in one pass (the CLI loop over
 *                              models, src/main.rs:109-114)
 *   jne_export_increments      src/rng_matrix.rs:57-141 (the path itself)
 *   jne_dat_*                  src/data_storage/{writer,reader,uleb128}.rs
 *   jne_record_bytes,          the record encoding of writer.rs:206-259 and
 *   jne_pack_records_device    uleb128.rs:68-87, on the GPU
 *   jne_simulation_*           src/data_storage/simulation.rs:25-122 and
 *                              parallel_compute.rs:150-232
 *   jne_percentiles(_device)   src/simulation_analyzers.rs:4-81
 */
#ifndef JNE_H
#define JNE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define JNE_OK 0
#define JNE_ERR_ARG 1     /* bad argument (model, dim, steps, sizes, null pointers) */
#define JNE_ERR_BUDGET 2  /* request does not fit the context's device-memory budget */
#define JNE_ERR_CUDA 3    /* CUDA runtime error (no device, launch failure, ...) */
#define JNE_ERR_TIMEOUT 4 /* a bounded device wait ran out */
#define JNE_ERR_NUMERIC 5 /* S11 not positive definite for some run (NaN written) */
#define JNE_ERR_IO 6      /* file system error */
#define JNE_ERR_FORMAT 7  /* not an EIGENVALS_V6 file, or inconsistent records */

/* arithmetic of the Gram contraction */
#define JNE_PREC_FP64 0  /* plain FP64 fused kernel */
#define JNE_PREC_MIXED 1 /* split FP16/TF32 tensor-core Grams, FP32 chunks, float-float merge, FP64 solve */
/* JNE_PREC_MIXED requests with fewer steps than this run the FP64 kernel: on
 * such short paths the FP32 chunk part is most of every moment. */
#define JNE_MIXED_MIN_STEPS 256

#define JNE_MAX_DIM 12
#define JNE_DEFAULT_BASE_SEED 0x4A4F48ull

typedef struct jne_context jne_context;

/* library version (major * 10000 + minor * 100 + patch) */
int jne_version(void);

/* number of eigenvalues per run, or -1 for a bad (model, dim) */
int jne_eigen_count(int model, int dim);

/* Opens a context on CUDA device `device`; device allocations of the context
 * never exceed mem_budget_bytes (0 = 40 GiB). */
int jne_open(int device, unsigned long long mem_budget_bytes, jne_context** out);
void jne_close(jne_context* ctx);

/* message of the last failed call on ctx (never null) */
const char* jne_last_error(const jne_context* ctx);

/* Steps per FP32 chunk of the mixed kernel: a multiple of 32 up to 8192, or 0
 * (the default) for the largest power of two <= steps/16 in [32, 512], or
 * JNE_CHUNK_TUNED for the launch shapes jne_autotune chose (chunk, kernel
 * variant, packing; the default rule for classes it has not tuned). */
#define JNE_CHUNK_TUNED (-1)
int jne_set_chunk(jne_context* ctx, int chunk);

/* The mixed single-request kernel's variant outside JNE_CHUNK_TUNED mode:
 * blocks_per_sm 4 (the default, 128 registers a thread) or 6 (80), and for
 * dims up to 4 pack = 1 (the default, two runs per warp) or 0 (one).  0 for
 * either keeps its default.  Speed only: every variant gives the same bits.
 * No counterpart in the reference. */
int jne_set_launch_shape(jne_context* ctx, int blocks_per_sm, int pack);

/* One candidate launch shape of the mixed kernel, as jne_autotune measured it. */
typedef struct jne_tune_entry {
  int chunk;          /* steps per FP32 chunk */
  int blocks_per_sm;  /* kernel variant: 4 (128 registers a thread) or 6 (80) */
  int pack;           /* dims <= 4: 1 = two runs per warp, 0 = one */
  double max_rel_err; /* worst max-eig / trace error vs FP64 on the sample (five models), relative to max(value, 1) */
  double ms;          /* device time of one launch of time_runs runs (model 0); < 0: not timed (over the bound) */
} jne_tune_entry;

/* Autotuner of the mixed kernel (no counterpart in the reference, whose only
 * knob is its thread count, src/cli.rs:311-329).  For the class of
 * (dim, steps) -- steps in [2^b, 2^(b+1)), tuned at 2^b where errors are
 * largest -- it runs seeds 1..sample_runs of all five models with the FP64
 * kernel and with each chunk 32, 64, ... (at most 1024 and half the steps) up
 * to the first over max_rel_err; then it times, with CUDA events, one launch of
 * time_runs runs (0: sized for about 20-60 ms) for every shape of every chunk
 * within the bound: blocks per SM 4 or 6, and one or two runs per warp for dims
 * up to 4.  The fastest shape is stored in ctx for JNE_CHUNK_TUNED and written
 * to *chosen; the measured candidates go to table (up to table_cap, *n_table of
 * them).  Only the chunk changes results: shapes of one chunk give the same
 * bits.  Classes below JNE_MIXED_MIN_STEPS run the FP64 kernel and are not
 * tuned (JNE_ERR_ARG).  table, n_table and chosen may be null. */
int jne_autotune(jne_context* ctx, int dim, int steps, double max_rel_err, int sample_runs, int64_t time_runs,
                 jne_tune_entry* table, int table_cap, int* n_table, jne_tune_entry* chosen);

/* jne_autotune with time_runs sized automatically and no table: the chosen
 * (fastest admissible) chunk and its error.  chunk_out / err_out may be null. */
int jne_autotune_chunk(jne_context* ctx, int dim, int steps, double max_rel_err, int sample_runs, int* chunk_out,
                       double* err_out);

/* Eigenvalues of n_runs runs from explicit increments.  dB holds n_runs
 * consecutive dim x steps column-major matrices (dB[:, i] = B_{i+1} - B_i,
 * B_0 = 0), host memory; out receives n_runs x k values (host). */
int jne_eigs_from_increments(jne_context* ctx, int model, int dim, int steps, const double* dB, int n_runs,
                             int precision, double* out);

/* Eigenvalues of runs with seeds seed_first .. seed_first + n_runs - 1 drawn
 * from the counter-based stream (base_seed, dim); out is host memory. */
int jne_eigs_seeded(jne_context* ctx, int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first,
                    int64_t n_runs, int precision, double* out);

/* As jne_eigs_seeded, with out in device memory, enqueued asynchronously:
 * work later enqueued on `stream` (a cudaStream_t; null = the context's
 * stream) sees the results, and the call returns without waiting.  Consecutive
 * calls overlap (the finalize of one batch runs beside the accumulation of the
 * next).  Device-side errors (a non-SPD S11) are reported by jne_sync. */
int jne_eigs_seeded_device(jne_context* ctx, int model, int dim, int steps, uint64_t base_seed,
                           uint32_t seed_first, int64_t n_runs, int precision, double* out_device, void* stream);

/* Waits for all work of ctx and returns (then clears) the device status of the
 * asynchronous calls since the last jne_sync. */
int jne_sync(jne_context* ctx);

/* Several models of one (dim, steps) pair from one pass over the paths (the
 * path of a seed does not depend on the model).  models[m] lists n_models
 * model ids; outs[m] receives n_runs x k(models[m], dim) values (host). */
int jne_eigs_seeded_models(jne_context* ctx, const int* models, int n_models, int dim, int steps,
                           uint64_t base_seed, uint32_t seed_first, int64_t n_runs, int precision,
                           double* const* outs);

/* No counterpart in the reference crate.  The seeded batch for callers that
 * cannot allocate device memory -- a host framework that owns the GPU's
 * allocator and forbids foreign allocations, a real-time loop that allows no
 * allocation after start-up.  It needs no context: its scratch (the moment
 * records, the chunk and entry tables, the counters and the status word) is one
 * file-scope __device__ array of JNE_NOALLOC_SCRATCH_BYTES (4.7 MiB) that every
 * GPU loading this library holds until the process exits, and it calls no
 * cudaMalloc, cudaFree or allocating library routine.  It runs the kernels and
 * tables of jne_eigs_seeded, so the results are the same bits.  Results go to
 * out_device (n_runs x k doubles) on `stream` (a cudaStream_t; null = the
 * legacy default stream); the call waits for them (it reads the status word
 * back and synchronizes the stream).  At most JNE_NOALLOC_MAX_RUNS runs per call
 * (and, for mixed precision, at most JNE_NOALLOC_MAX_CHUNKS chunks: 2,097,152
 * steps), else JNE_ERR_BUDGET.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture.  All calls share the one array, which
 * keeps the last call's contents (each call clears the words that must start at
 * zero), so calls whose GPU work overlaps (other threads or streams) race and
 * must be serialised by the caller.  The message of a failed call comes from
 * jne_noalloc_last_error (per thread). */
#define JNE_NOALLOC_MAX_RUNS 2048
#define JNE_NOALLOC_MAX_CHUNKS 4096
#define JNE_NOALLOC_SCRATCH_BYTES 4956672
int jne_eigs_seeded_noalloc(int device, int model, int dim, int steps, uint64_t base_seed, uint32_t seed_first,
                            int n_runs, int precision, double* out_device, void* stream);
const char* jne_noalloc_last_error(void);

/* One request of a batch. */
typedef struct jne_request {
  int model, dim, steps, precision;
  uint64_t base_seed;
  uint32_t seed_first;
  int64_t n_runs;
} jne_request;

/* A ragged batch: requests of any (model, dim, steps, seeds, size) in one
 * persistent launch (the loop of the reference CLI over models and dims,
 * src/main.rs:85-136, is one batch).  outs_device[i] receives request i's
 * n_runs x k values.  Asynchronous, like jne_eigs_seeded_device. */
int jne_run_batch(jne_context* ctx, const jne_request* reqs, int n_req, double* const* outs_device, void* stream);

/* As jne_run_batch, then waits for the batch and reports each request's own
 * status in status_out[i] (host, n_req ints): JNE_OK, or JNE_ERR_NUMERIC when
 * some run of request i had a non-SPD S11 (its rows are NaN).  A failing
 * request does not fail the others it shares a launch with: every request of
 * the reference CLI's loop is its own simulation, which fails alone
 * (src/data_storage/parallel_compute.rs:129-147, src/main.rs:85-136).  Returns
 * JNE_OK when every request succeeded, the first failing request's code when
 * some did, or the error that stopped the batch. */
int jne_run_batch_status(jne_context* ctx, const jne_request* reqs, int n_req, double* const* outs_device,
                         int* status_out, void* stream);

/* ---- streaming sink: the batch with its results delivered to host code ----
 * The reference computes each run and sends (seed, eigenvalues) over a channel
 * to a writer thread that appends it to the simulation's file
 * (src/data_storage/parallel_compute.rs:14-41, thread_manager.rs:25-92,
 * writer.rs:206-259).  Here a batch is computed in rounds of ragged launches
 * and each round's results reach `write` on the calling thread while the GPU
 * computes the next round. */
typedef struct jne_sink {
  /* n consecutive results of request `req` (its index in the batch): seeds
   * seed_first .. seed_first + n - 1, k eigenvalues each (descending,
   * run-major, host memory valid during the call).  A request's results arrive
   * in seed order.  status: JNE_OK, or JNE_ERR_NUMERIC when some of these rows
   * are NaN (S11 not positive definite).  A non-zero return stops the batch, and
   * jne_run_batch_sink returns it. */
  int (*write)(void* user, int req, uint32_t seed_first, int64_t n, int k, const double* eigs, int status);
  void* user;
  /* Optional (null: unused).  When set, the batch packs each slice of results
   * into .dat records on the GPU (jne_pack_records_device) and hands over their
   * bytes instead of the eigenvalues: n_bytes = jne_record_bytes(seed_first, n,
   * k) bytes in host memory, valid during the call, that jne_dat_append_packed
   * appends as they are.  `write` is then not called and may be null.  The
   * record stream replaces writer.rs:206-259's per-record encoding. */
  int (*write_records)(void* user, int req, uint32_t seed_first, int64_t n, int k, const unsigned char* records,
                       int64_t n_bytes, int status);
} jne_sink;

/* The batch of jne_run_batch, streamed to `sink`.  Synchronous: returns when
 * every result has been delivered (JNE_OK, or JNE_ERR_NUMERIC when some rows
 * were NaN), when the sink stops it (its code), or on an error.  Rounds hold up
 * to 2^20 runs (fewer under a small budget).  The sink needs write or
 * write_records; with write_records the records are packed on the GPU. */
int jne_run_batch_sink(jne_context* ctx, const jne_request* reqs, int n_req, const jne_sink* sink);

/* A sink that appends each request's records to its simulation file
 * <data_dir>/eigenvalues_model{m}_dim{d}_steps{T}.dat (data_dir null or empty:
 * "data", created on demand; requests with the same (model, dim, steps) share
 * the file; an existing file is appended to as jne_dat_open does).  Results
 * with a non-OK status stop the batch with that status (the reference's writer
 * never sees such a run: its sort panics first).  It sets both callbacks, so
 * jne_run_batch_sink packs the records on the GPU (clear write_records to have
 * them encoded on the host instead: the same bytes).  jne_dat_sink_close writes
 * the EOF trailers (finish != 0) or leaves the files as an interrupted run does. */
int jne_dat_sink_open(const char* data_dir, const jne_request* reqs, int n_req, jne_sink* out);
int jne_dat_sink_close(jne_sink* sink, int finish);

/* Plans: a ragged batch prepared once (device tables and records inside the
 * context's budget) and captured into a CUDA graph; each jne_plan_launch
 * replays it asynchronously on `stream`.  Requests must be mixed precision with
 * steps >= JNE_MIXED_MIN_STEPS.  jne_plan_destroy waits for the last replay. */
typedef struct jne_plan jne_plan;
int jne_plan_create(jne_context* ctx, const jne_request* reqs, int n_req, double* const* outs_device,
                    jne_plan** out);
int jne_plan_launch(jne_plan* plan, void* stream);
void jne_plan_destroy(jne_plan* plan);

/* ---- continuous-batching request loop (serving) ----
 * A worker thread owns the context while the server is open (do not call other
 * jne_* functions on that context meanwhile).  Requests are admitted FIFO while
 * their device output buffers fit half the context's budget; every iteration is
 * one ragged launch over a slice of each active request (about iter_work
 * runs x steps in total, 0 = 2e9), so new requests join running ones at the
 * next iteration.  Finished results wait in host memory for jne_server_fetch;
 * with a data directory they are also streamed, by a writer thread, to
 * <data_dir>/request<id>_model<m>_dim<d>_steps<T>.dat (EIGENVALS_V6). */
typedef struct jne_server jne_server;
typedef struct jne_completion {
  uint64_t id;
  int status;                           /* JNE_OK or the request's error */
  double submit_s, start_s, finish_s;  /* seconds since jne_server_open */
  int64_t n_runs;
} jne_completion;
int jne_server_open(jne_context* ctx, const char* data_dir, long long iter_work, jne_server** out);
int jne_server_submit(jne_server* server, const jne_request* req, uint64_t* id);
/* Up to max completions into out (*n of them), waiting up to timeout_ms (-1: no limit) for the first. */
int jne_server_wait(jne_server* server, jne_completion* out, int max, int timeout_ms, int* n);
/* Copies a finished request's n_runs x k eigenvalues (host) and forgets the
 * request; returns its status, JNE_ERR_ARG for an unknown or unfinished id or a
 * short buffer, JNE_ERR_TIMEOUT while its file is still being written. */
int jne_server_fetch(jne_server* server, uint64_t id, double* out, int64_t cap);
/* Finishes every submitted request, then stops the worker and writer threads. */
int jne_server_close(jne_server* server);

/* Per-kernel timing: when enabled, every kernel launch of ctx is bracketed by
 * CUDA events on its launching stream.  jne_profile_read returns the summed
 * device milliseconds and launch counts per kernel kind (index JNE_KERNEL_*),
 * and resets them when `reset` is non-zero. */
#define JNE_KERNEL_ACCUM_FP64 0
#define JNE_KERNEL_ACCUM_MIXED 1
#define JNE_KERNEL_FINALIZE 2
#define JNE_KERNEL_EXPORT 3
#define JNE_KERNEL_KINDS 4
int jne_profile(jne_context* ctx, int enable);
int jne_profile_read(jne_context* ctx, double* ms, long long* launches, int reset);

/* Measures, on ctx's device, the rates that bound the accumulation kernels:
 * rates[0] normals/s drawn by the kernels' own Philox4x32-10 + Box-Muller code,
 * rates[1] FP64 FMA flop/s, rates[2] TF32 mma.sync (m16n8k8) flop/s, rates[3]
 * FP32 FMA flop/s, rates[4] FP16 mma.sync (m16n8k16, FP32 accumulation) flop/s
 * (JNE_RATE_*).  Each is one ~10-50 ms launch over 8 blocks per SM,
 * timed with CUDA events after a warm-up launch.  Diagnostic: no counterpart in
 * the reference. */
#define JNE_RATE_NORMALS 0
#define JNE_RATE_DFMA 1
#define JNE_RATE_MMA_TF32 2
#define JNE_RATE_FFMA 3
#define JNE_RATE_MMA_F16 4
#define JNE_RATE_KINDS 5
int jne_probe_rates(jne_context* ctx, double* rates);

/* The increments the seeded path draws for these runs, scaled by sqrt(1/steps):
 * dB_out receives n_runs consecutive dim x steps column-major matrices (may be
 * null); words_out receives the raw Philox words, n_runs x steps x
 * ceil(dim/4) x 4 (may be null).  Host memory. */
int jne_export_increments(jne_context* ctx, int dim, int steps, uint64_t base_seed, uint32_t seed_first,
                          int n_runs, double* dB_out, uint32_t* words_out);

/* ---- EIGENVALS_V6 files (src/data_storage/{writer,reader,uleb128}.rs) ---- */
typedef struct jne_dat_writer jne_dat_writer;

/* Opens `path` for appending (writer.rs:28-178).  A new file gets the 18-byte
 * header.  An existing file must carry the same (model, dim, steps), else
 * JNE_ERR_FORMAT ("Model mismatch: file has model X, expected Y", ...); a file
 * with a foreign magic header is recreated; a complete file's EOF trailer is
 * stripped.  *existing (may be null) receives the records already present. */
int jne_dat_open(const char* path, int model, int dim, uint32_t steps, jne_dat_writer** out, int64_t* existing);

/* Appends n records (seeds[r], eigs[r*k .. r*k+k-1]) (writer.rs:206-259): k <= 255
 * and the same for every record of the file, else JNE_ERR_FORMAT. */
int jne_dat_append(jne_dat_writer* w, const uint32_t* seeds, const double* eigs, int64_t n, int k);

/* Bytes of the records of n consecutive seeds seed_first .. seed_first + n - 1
 * with k values each, in the record format above (ULEB128 seed, u8 count, k x
 * f64 LE; uleb128.rs:68-87, writer.rs:242-249); -1 when n < 0, k is outside
 * 0..255 or the seeds leave u32. */
int64_t jne_record_bytes(uint32_t seed_first, int64_t n, int k);

/* The records of n results of consecutive seeds seed_first.. (eigs_device:
 * n x k f64 in device memory, run-major) packed on the GPU into out_device
 * (device memory, 16-byte aligned, cap >= jne_record_bytes bytes).  Enqueued on
 * `stream` (null: the context's stream); asynchronous.  The bytes are those
 * jne_dat_append writes for the same records. */
int jne_pack_records_device(jne_context* ctx, uint32_t seed_first, int64_t n, int k, const double* eigs_device,
                            unsigned char* out_device, int64_t cap, void* stream);

/* Appends n records of consecutive seeds seed_first.. already packed
 * (jne_record_bytes(seed_first, n, k) bytes, host memory), with the checks and
 * the short-write handling of jne_dat_append. */
int jne_dat_append_packed(jne_dat_writer* w, uint32_t seed_first, int64_t n, int k, const unsigned char* records);

/* Writes the EOF trailer (count, eigenvalues per record) and closes (writer.rs:262-302). */
int jne_dat_finish(jne_dat_writer* w);

/* Closes without a trailer, as an interrupted run leaves the file; readers
 * recover such files by scanning (reader.rs:157-216). */
void jne_dat_abandon(jne_dat_writer* w);

/* Reads a file (reader.rs:23-216): header fields, record count *n and
 * eigenvalues per record *k; when seeds and eigs are non-null and cap >= *n,
 * also the records (eigs is n x k).  Any output pointer may be null. */
int jne_dat_read(const char* path, int* model, int* dim, uint32_t* steps, int64_t* n, int* k, uint32_t* seeds,
                 double* eigs, int64_t cap);

/* message of this thread's last failed jne_dat_* / jne_simulation_* / jne_percentiles call */
const char* jne_dat_last_error(void);

/* ---- EigenvalueSimulation (src/data_storage/simulation.rs, parallel_compute.rs:150-232) ---- */

/* "<data_dir>/eigenvalues_model{m}_dim{d}_steps{T}.dat" (simulation.rs:98-122);
 * data_dir null or empty means "data". */
int jne_simulation_filename(const char* data_dir, int model, int dim, int steps, char* buf, size_t cap);

/* Runs or resumes a simulation: the seeds 1..=num_runs missing from the file
 * are computed on the GPU and appended, then the trailer is written.  A file
 * with other (model, dim, steps) is removed and recreated
 * (parallel_compute.rs:155-180).  The directory is created on demand. */
int jne_simulation_run(jne_context* ctx, const char* data_dir, int model, int dim, int steps, int64_t num_runs,
                       int precision, uint64_t base_seed, int quiet);

/* The same for several models of one (dim, steps) -- the reference CLI's loop
 * over models (src/main.rs:109-114).  Models whose files miss the same seeds
 * (every fresh run) share one pass over the paths: one accumulation per seed,
 * one finalize per model; each file gets exactly the records and bytes the
 * per-model driver writes. */
int jne_simulation_run_models(jne_context* ctx, const char* data_dir, const int* models, int n_models, int dim,
                              int steps, int64_t num_runs, int precision, uint64_t base_seed, int quiet);

/* Percentiles (simulation_analyzers.rs:4-81) of the trace (stat 0) or the
 * largest eigenvalue (stat 1) of n records of k eigenvalues: linear
 * interpolation at rank p * (n - 1) of the sorted statistic; NaN when n == 0.
 * Every p must lie in [0, 1] (JNE_ERR_ARG); a NaN statistic gives
 * JNE_ERR_NUMERIC (the reference's sort panics on NaN). */
int jne_percentiles(const double* eigs, int64_t n, int k, int stat, const double* ps, int np, double* out);

/* The same percentiles of eigenvalues in device memory (n x k, run-major), by
 * a radix select on the device instead of a sort; bit-identical to
 * jne_percentiles.  Work the caller enqueued on `stream` (null: the legacy
 * default stream) before the call is waited for; ps / out are host memory and
 * the call returns when `out` is written.  Scratch: 8 bytes per run within the
 * context's budget.  Replaces calculate_percentiles, simulation_analyzers.rs:42-65. */
int jne_percentiles_device(jne_context* ctx, const double* eigs_device, int64_t n, int k, int stat, const double* ps,
                           int np, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* JNE_H */
