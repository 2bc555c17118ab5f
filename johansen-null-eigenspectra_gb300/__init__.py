"""GB300 engine for the Johansen null-eigenspectra Monte Carlo path.

Python host mirror of the reference crate's public API (src/lib.rs:10-11):
``JohansenModel`` and ``EigenvalueSimulation`` keep the reference's names,
argument meaning and error behaviour, and every computation goes through the
C ABI of ``libjne_gb300.so`` (include/jne.h) -- hand-written sm_103a kernels.
There is no CPU fallback: a missing library or device raises.

The directory name contains hyphens, so load this package with
``load_package()`` from ``__graft_entry__`` (or importlib) rather than import.
"""
from __future__ import annotations

import ctypes
import enum
import os
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libjne_gb300.so")

JNE_OK, JNE_ERR_ARG, JNE_ERR_BUDGET, JNE_ERR_CUDA, JNE_ERR_TIMEOUT, JNE_ERR_NUMERIC, JNE_ERR_IO, JNE_ERR_FORMAT = range(8)
PREC_FP64, PREC_MIXED = 0, 1
CHUNK_TUNED = -1
DEFAULT_BASE_SEED = 0x4A4F48
MAX_DIM = 12

# every symbol include/jne.h declares (checked by the CPU test suite)
EXPORTS = (
    "jne_version", "jne_eigen_count", "jne_open", "jne_close", "jne_last_error", "jne_set_chunk",
    "jne_eigs_from_increments", "jne_eigs_seeded", "jne_eigs_seeded_device", "jne_eigs_seeded_models",
    "jne_export_increments", "jne_profile", "jne_profile_read", "jne_probe_rates", "jne_sync", "jne_autotune_chunk",
    "jne_autotune", "jne_set_launch_shape",
    "jne_dat_open", "jne_dat_append", "jne_dat_append_packed", "jne_record_bytes", "jne_pack_records_device",
    "jne_dat_finish", "jne_dat_abandon", "jne_dat_read", "jne_dat_last_error",
    "jne_simulation_filename", "jne_simulation_run", "jne_simulation_run_models", "jne_percentiles",
    "jne_percentiles_device",
    "jne_eigs_seeded_noalloc", "jne_noalloc_last_error",
    "jne_run_batch", "jne_run_batch_status", "jne_run_batch_sink", "jne_dat_sink_open", "jne_dat_sink_close",
    "jne_plan_create", "jne_plan_launch", "jne_plan_destroy",
    "jne_server_open", "jne_server_submit", "jne_server_wait", "jne_server_fetch", "jne_server_close",
)
KERNEL_KINDS = ("accum_fp64", "accum_mixed", "finalize", "export")
RATE_KINDS = ("normals_per_s", "dfma_flops", "mma_tf32_flops", "ffma_flops", "mma_f16_flops")


class Request(ctypes.Structure):
    """jne_request: one request of a batch (model, dim, steps, precision, seeds)."""

    _fields_ = [("model", ctypes.c_int), ("dim", ctypes.c_int), ("steps", ctypes.c_int), ("precision", ctypes.c_int),
                ("base_seed", ctypes.c_uint64), ("seed_first", ctypes.c_uint32), ("n_runs", ctypes.c_int64)]


class TuneEntry(ctypes.Structure):
    """jne_tune_entry: one launch shape the autotuner measured."""

    _fields_ = [("chunk", ctypes.c_int), ("blocks_per_sm", ctypes.c_int), ("pack", ctypes.c_int),
                ("max_rel_err", ctypes.c_double), ("ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


SINK_WRITE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_int64,
                              ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int)


SINK_WRITE_RECORDS = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_int64,
                                      ctypes.c_int, ctypes.POINTER(ctypes.c_ubyte), ctypes.c_int64, ctypes.c_int)


class Sink(ctypes.Structure):
    """jne_sink: a write callback, its user pointer, and the optional callback
    that takes records packed on the GPU instead of eigenvalues."""

    _fields_ = [("write", SINK_WRITE), ("user", ctypes.c_void_p), ("write_records", SINK_WRITE_RECORDS)]


class Completion(ctypes.Structure):
    """jne_completion: a finished request of the server, with its times (seconds since the server opened)."""

    _fields_ = [("id", ctypes.c_uint64), ("status", ctypes.c_int), ("submit_s", ctypes.c_double),
                ("start_s", ctypes.c_double), ("finish_s", ctypes.c_double), ("n_runs", ctypes.c_int64)]


class JneError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[jne status {code}] {msg}")
        self.code = code


class JohansenModel(enum.IntEnum):
    """The five Johansen models (johansen_models.rs:6-26)."""

    NoInterceptNoTrend = 0
    InterceptNoTrendWithInterceptInCoint = 1
    InterceptNoTrendUnrestrictedIntercept = 2
    InterceptTrendUnrestrictedInterceptRestrictedTrend = 3
    InterceptTrendUnrestrictedBoth = 4

    def to_number(self) -> int:
        return int(self)

    @classmethod
    def from_number(cls, n: int) -> Optional["JohansenModel"]:
        return cls(n) if 0 <= n <= 4 else None

    def description(self) -> str:  # johansen_models.rs:54-70
        return _DESCRIPTIONS[int(self)]

    def has_intercept(self) -> bool:
        return self != JohansenModel.NoInterceptNoTrend

    def has_trend(self) -> bool:
        return self in (JohansenModel.InterceptTrendUnrestrictedInterceptRestrictedTrend,
                        JohansenModel.InterceptTrendUnrestrictedBoth)

    def intercept_fully_explained_by_cointegration(self) -> bool:
        return self == JohansenModel.InterceptNoTrendWithInterceptInCoint

    def trend_fully_explained_by_cointegration(self) -> bool:
        return self == JohansenModel.InterceptTrendUnrestrictedInterceptRestrictedTrend

    @classmethod
    def all_models(cls) -> List["JohansenModel"]:
        return [cls(i) for i in range(5)]

    @classmethod
    def default(cls) -> "JohansenModel":  # johansen_models.rs:130-135
        return cls.InterceptNoTrendUnrestrictedIntercept

    def __str__(self) -> str:  # johansen_models.rs:137-141
        return f"Model {int(self)}: {self.description()}"


_DESCRIPTIONS = (
    "No intercept, no trend",
    "Intercept, no trend, intercept in cointegration",
    "Intercept, no trend, intercept not fully explained by cointegration",
    "Intercept, trend, trend in cointegration",
    "Intercept, trend, intercept and trend not fully explained by cointegration",
)


def eigen_count(model: int, dim: int) -> int:
    """thread_manager.rs:40-44."""
    return dim + 1 if int(model) in (1, 3) else dim


# --------------------------------------------------------------------------
# ctypes binding
# --------------------------------------------------------------------------
_lib = None


def lib() -> ctypes.CDLL:
    """Loads libjne_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} is missing: run __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        c_int, c_u32, c_u64, c_i64, c_ull = ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int64, ctypes.c_ulonglong
        dp, vp = ctypes.POINTER(ctypes.c_double), ctypes.c_void_p
        L.jne_version.restype = c_int
        L.jne_eigen_count.argtypes = [c_int, c_int]
        L.jne_open.argtypes = [c_int, c_ull, ctypes.POINTER(vp)]
        L.jne_close.argtypes = [vp]
        L.jne_close.restype = None
        L.jne_last_error.argtypes = [vp]
        L.jne_last_error.restype = ctypes.c_char_p
        L.jne_set_chunk.argtypes = [vp, c_int]
        L.jne_set_launch_shape.argtypes = [vp, c_int, c_int]
        L.jne_eigs_from_increments.argtypes = [vp, c_int, c_int, c_int, dp, c_int, c_int, dp]
        L.jne_eigs_seeded.argtypes = [vp, c_int, c_int, c_int, c_u64, c_u32, c_i64, c_int, dp]
        L.jne_eigs_seeded_device.argtypes = [vp, c_int, c_int, c_int, c_u64, c_u32, c_i64, c_int, vp, vp]
        L.jne_eigs_seeded_models.argtypes = [vp, ctypes.POINTER(c_int), c_int, c_int, c_int, c_u64, c_u32, c_i64,
                                             c_int, ctypes.POINTER(dp)]
        L.jne_export_increments.argtypes = [vp, c_int, c_int, c_u64, c_u32, c_int, dp, ctypes.POINTER(c_u32)]
        L.jne_sync.argtypes = [vp]
        L.jne_run_batch.argtypes = [vp, ctypes.POINTER(Request), c_int, ctypes.POINTER(vp), vp]
        L.jne_run_batch_status.argtypes = [vp, ctypes.POINTER(Request), c_int, ctypes.POINTER(vp),
                                           ctypes.POINTER(c_int), vp]
        L.jne_run_batch_sink.argtypes = [vp, ctypes.POINTER(Request), c_int, ctypes.POINTER(Sink)]
        L.jne_dat_sink_open.argtypes = [ctypes.c_char_p, ctypes.POINTER(Request), c_int, ctypes.POINTER(Sink)]
        L.jne_dat_sink_close.argtypes = [ctypes.POINTER(Sink), c_int]
        L.jne_plan_create.argtypes = [vp, ctypes.POINTER(Request), c_int, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        L.jne_plan_launch.argtypes = [vp, vp]
        L.jne_plan_destroy.argtypes = [vp]
        L.jne_plan_destroy.restype = None
        L.jne_server_open.argtypes = [vp, ctypes.c_char_p, ctypes.c_longlong, ctypes.POINTER(vp)]
        L.jne_server_submit.argtypes = [vp, ctypes.POINTER(Request), ctypes.POINTER(c_u64)]
        L.jne_server_wait.argtypes = [vp, ctypes.POINTER(Completion), c_int, c_int, ctypes.POINTER(c_int)]
        L.jne_server_fetch.argtypes = [vp, c_u64, dp, c_i64]
        L.jne_server_close.argtypes = [vp]
        L.jne_profile.argtypes = [vp, c_int]
        L.jne_profile_read.argtypes = [vp, dp, ctypes.POINTER(ctypes.c_longlong), c_int]
        L.jne_probe_rates.argtypes = [vp, dp]
        L.jne_autotune_chunk.argtypes = [vp, c_int, c_int, ctypes.c_double, c_int, ctypes.POINTER(c_int), dp]
        L.jne_autotune.argtypes = [vp, c_int, c_int, ctypes.c_double, c_int, c_i64, ctypes.POINTER(TuneEntry), c_int,
                                   ctypes.POINTER(c_int), ctypes.POINTER(TuneEntry)]
        L.jne_percentiles_device.argtypes = [vp, vp, c_i64, c_int, c_int, dp, c_int, dp, vp]
        u32p, i64p, ip = ctypes.POINTER(c_u32), ctypes.POINTER(c_i64), ctypes.POINTER(c_int)
        L.jne_dat_open.argtypes = [ctypes.c_char_p, c_int, c_int, c_u32, ctypes.POINTER(vp), i64p]
        L.jne_dat_append.argtypes = [vp, u32p, dp, c_i64, c_int]
        L.jne_dat_append_packed.argtypes = [vp, c_u32, c_i64, c_int, vp]
        L.jne_record_bytes.argtypes = [c_u32, c_i64, c_int]
        L.jne_record_bytes.restype = c_i64
        L.jne_pack_records_device.argtypes = [vp, c_u32, c_i64, c_int, vp, vp, c_i64, vp]
        L.jne_dat_finish.argtypes = [vp]
        L.jne_dat_abandon.argtypes = [vp]
        L.jne_dat_abandon.restype = None
        L.jne_dat_read.argtypes = [ctypes.c_char_p, ip, ip, u32p, i64p, ip, u32p, dp, c_i64]
        L.jne_dat_last_error.restype = ctypes.c_char_p
        L.jne_simulation_filename.argtypes = [ctypes.c_char_p, c_int, c_int, c_int, ctypes.c_char_p, ctypes.c_size_t]
        L.jne_simulation_run.argtypes = [vp, ctypes.c_char_p, c_int, c_int, c_int, c_i64, c_int, c_u64, c_int]
        L.jne_simulation_run_models.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(c_int), c_int, c_int, c_int, c_i64,
                                                c_int, c_u64, c_int]
        L.jne_percentiles.argtypes = [dp, c_i64, c_int, c_int, dp, c_int, dp]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Engine:
    """One C-ABI context on one CUDA device (jne_open / jne_close)."""

    def __init__(self, device: int = 0, mem_budget_bytes: int = 0, chunk: Optional[int] = None):
        self._L = lib()
        h = ctypes.c_void_p()
        rc = self._L.jne_open(device, mem_budget_bytes, ctypes.byref(h))
        if rc != JNE_OK:
            raise JneError(rc, f"jne_open(device={device}) failed: no usable CUDA device")
        self._h = h
        if chunk is not None:
            self._check(self._L.jne_set_chunk(self._h, chunk))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.jne_close(self._h)
            self._h = None

    def __enter__(self) -> "Engine":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        if rc != JNE_OK:
            raise JneError(rc, self._L.jne_last_error(self._h).decode(errors="replace"))

    def set_chunk(self, chunk: int) -> None:
        """Steps per FP32 chunk of the mixed kernel: 0 (default rule), CHUNK_TUNED or a multiple of 32 up to 8192."""
        self._check(self._L.jne_set_chunk(self._h, chunk))

    def set_launch_shape(self, blocks_per_sm: int = 4, pack: int = 1) -> None:
        """The mixed kernel variant outside CHUNK_TUNED mode: 4 or 6 blocks per SM; for dims <= 4 two runs
        per warp (pack=1) or one (pack=0).  Speed only: the same bits."""
        self._check(self._L.jne_set_launch_shape(self._h, blocks_per_sm, pack))

    def autotune(self, dim: int, steps: int, max_rel_err: float = 1e-6, sample_runs: int = 2000,
                 time_runs: int = 0) -> Tuple[dict, List[dict]]:
        """jne_autotune: the fastest launch shape (chunk, blocks per SM, packing) whose chunk keeps the error
        vs the FP64 kernel within max_rel_err on the sample, for steps in [2^b, 2^(b+1)); used after
        set_chunk(CHUNK_TUNED).  Returns (chosen shape, every measured candidate) as dicts."""
        table = (TuneEntry * 64)()
        n, best = ctypes.c_int(), TuneEntry()
        self._check(self._L.jne_autotune(self._h, dim, steps, float(max_rel_err), sample_runs, time_runs, table, 64,
                                         ctypes.byref(n), ctypes.byref(best)))
        return best.as_dict(), [table[i].as_dict() for i in range(n.value)]

    def autotune_chunk(self, dim: int, steps: int, max_rel_err: float = 5e-7, sample_runs: int = 512) -> Tuple[int, float]:
        """The fastest admissible chunk of jne_autotune (its shape is stored too), for steps in
        [2^b, 2^(b+1)); used after set_chunk(CHUNK_TUNED).  Returns (chunk, its error)."""
        ch, err = ctypes.c_int(), np.zeros(1)
        self._check(self._L.jne_autotune_chunk(self._h, dim, steps, float(max_rel_err), sample_runs, ctypes.byref(ch),
                                               _dp(err)))
        return ch.value, float(err[0])

    def profile(self, enable: bool = True) -> None:
        """Bracket every kernel launch with CUDA events on its launching stream."""
        self._check(self._L.jne_profile(self._h, int(enable)))

    def profile_read(self, reset: bool = True) -> Dict[str, Tuple[float, int]]:
        """{kernel kind: (summed device ms, launches)} since the last reset."""
        ms = np.zeros(4)
        n = (ctypes.c_longlong * 4)()
        self._check(self._L.jne_profile_read(self._h, _dp(ms), n, int(reset)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(KERNEL_KINDS)}

    def percentiles_device(self, eigs_ptr: int, n: int, k: int, stat: str, ps: Sequence[float],
                           stream: int = 0) -> List[float]:
        """Percentiles of the trace ('trace') or largest eigenvalue ('maxeig') of n
        runs of k eigenvalues at device address eigs_ptr, selected on the device."""
        p = np.ascontiguousarray(ps, dtype=np.float64)
        out = np.empty(len(p))
        self._check(self._L.jne_percentiles_device(self._h, ctypes.c_void_p(eigs_ptr), int(n), int(k),
                                                    0 if stat == "trace" else 1, _dp(p), len(p), _dp(out),
                                                    ctypes.c_void_p(stream)))
        return out.tolist()

    def pack_records_device(self, seed_first: int, n: int, k: int, eigs_ptr: int, out_ptr: int, cap: int,
                            stream: int = 0) -> int:
        """jne_pack_records_device: the .dat records of n results (n x k doubles at device address eigs_ptr) of
        seeds seed_first.. packed on the GPU into the 16-byte aligned device buffer at out_ptr (cap bytes);
        asynchronous on `stream`.  Returns the byte count."""
        self._check(self._L.jne_pack_records_device(self._h, seed_first, int(n), int(k), ctypes.c_void_p(eigs_ptr),
                                                     ctypes.c_void_p(out_ptr), int(cap), ctypes.c_void_p(stream)))
        return record_bytes(seed_first, n, k)

    def probe_rates(self) -> Dict[str, float]:
        """Measured pipe rates of this GPU: normals/s of the kernels' RNG code, and
        FP64-FMA, TF32-mma, FP32-FMA and FP16-mma flop/s."""
        r = np.zeros(len(RATE_KINDS))
        self._check(self._L.jne_probe_rates(self._h, _dp(r)))
        return {k: float(r[i]) for i, k in enumerate(RATE_KINDS)}

    def eigs_from_increments(self, model: int, dB: np.ndarray, precision: int = PREC_FP64) -> np.ndarray:
        """dB: (n_runs, steps, dim) -- each run's dim x steps increment matrix, column-major."""
        dB = np.ascontiguousarray(dB, dtype=np.float64)
        n, steps, dim = dB.shape
        out = np.empty((n, eigen_count(model, dim)))
        self._check(self._L.jne_eigs_from_increments(self._h, int(model), dim, steps, _dp(dB), n, precision, _dp(out)))
        return out

    def eigs_seeded(self, model: int, dim: int, steps: int, seed_first: int, n_runs: int,
                    precision: int = PREC_FP64, base_seed: int = DEFAULT_BASE_SEED) -> np.ndarray:
        out = np.empty((n_runs, eigen_count(model, dim)))
        self._check(self._L.jne_eigs_seeded(self._h, int(model), dim, steps, base_seed, seed_first, n_runs,
                                            precision, _dp(out)))
        return out

    def eigs_seeded_device(self, model: int, dim: int, steps: int, seed_first: int, n_runs: int, out_ptr: int,
                           precision: int = PREC_FP64, base_seed: int = DEFAULT_BASE_SEED,
                           stream: Optional[int] = None) -> None:
        """Results into the device buffer at out_ptr (n_runs x k doubles); asynchronous:
        work later enqueued on `stream` sees them, and sync() reports device errors."""
        self._check(self._L.jne_eigs_seeded_device(self._h, int(model), dim, steps, base_seed, seed_first, n_runs,
                                                   precision, ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream or 0)))

    def sync(self) -> None:
        """Wait for all asynchronous work and raise on its device status (jne_sync)."""
        self._check(self._L.jne_sync(self._h))

    @staticmethod
    def _requests(reqs) -> "ctypes.Array":
        arr = (Request * len(reqs))()
        for i, r in enumerate(reqs):
            d = dict(precision=PREC_MIXED, base_seed=DEFAULT_BASE_SEED, seed_first=1)
            d.update(r)
            arr[i] = Request(int(d["model"]), d["dim"], d["steps"], d["precision"], d["base_seed"], d["seed_first"],
                             d["n_runs"])
        return arr

    def run_batch(self, reqs: Sequence[dict], out_ptrs: Sequence[int], stream: Optional[int] = None) -> None:
        """jne_run_batch: a ragged batch (dicts with model, dim, steps, n_runs [, precision, seed_first,
        base_seed]) into device buffers out_ptrs[i] (n_runs x k doubles each); asynchronous."""
        arr = self._requests(reqs)
        outs = (ctypes.c_void_p * len(reqs))(*[ctypes.c_void_p(p) for p in out_ptrs])
        self._check(self._L.jne_run_batch(self._h, arr, len(reqs), outs, ctypes.c_void_p(stream or 0)))

    def run_batch_status(self, reqs: Sequence[dict], out_ptrs: Sequence[int],
                         stream: Optional[int] = None) -> List[int]:
        """jne_run_batch_status: the batch, waited for; returns each request's own status (JNE_OK or
        JNE_ERR_NUMERIC), so a singular request fails alone.  Raises only when the batch itself fails."""
        arr = self._requests(reqs)
        outs = (ctypes.c_void_p * len(reqs))(*[ctypes.c_void_p(p) for p in out_ptrs])
        st = (ctypes.c_int * max(1, len(reqs)))()
        rc = self._L.jne_run_batch_status(self._h, arr, len(reqs), outs, st, ctypes.c_void_p(stream or 0))
        codes = [int(st[i]) for i in range(len(reqs))]
        if rc != JNE_OK and not any(c != JNE_OK for c in codes):
            self._check(rc)
        return codes

    def run_batch_sink(self, reqs: Sequence[dict], write) -> None:
        """jne_run_batch_sink: the batch streamed to write(req, seed_first, eigs (n x k array, a copy), status),
        called in seed order per request; a non-zero int return stops the batch (raised as JneError)."""
        arr = self._requests(reqs)

        def cb(user, req, seed_first, n, k, eigs, status):
            try:
                a = np.ctypeslib.as_array(eigs, shape=(n * k,)).reshape(n, k).copy() if n else np.empty((0, k))
                return int(write(req, seed_first, a, status) or 0)
            except Exception:  # no exception may cross the C ABI
                return JNE_ERR_IO

        sink = Sink(SINK_WRITE(cb), None)
        self._check(self._L.jne_run_batch_sink(self._h, arr, len(reqs), ctypes.byref(sink)))

    def run_batch_to_dat(self, reqs: Sequence[dict], data_dir: str, finish: bool = True,
                         device_pack: bool = True) -> None:
        """The batch streamed by jne_dat_sink into each request's simulation file under data_dir, with the
        records packed on the GPU (device_pack) or encoded on the host: the same bytes."""
        arr = self._requests(reqs)
        sink = Sink()
        _dat_check(self._L.jne_dat_sink_open(os.fsencode(data_dir), arr, len(reqs), ctypes.byref(sink)))
        if not device_pack:
            sink.write_records = SINK_WRITE_RECORDS()
        rc = self._L.jne_run_batch_sink(self._h, arr, len(reqs), ctypes.byref(sink))
        rc2 = self._L.jne_dat_sink_close(ctypes.byref(sink), int(finish and rc == JNE_OK))
        self._check(rc)
        _dat_check(rc2)

    def plan(self, reqs: Sequence[dict], out_ptrs: Sequence[int]) -> "Plan":
        """jne_plan_create: the batch captured into a CUDA graph, replayed by Plan.launch()."""
        arr = self._requests(reqs)
        outs = (ctypes.c_void_p * len(reqs))(*[ctypes.c_void_p(p) for p in out_ptrs])
        h = ctypes.c_void_p()
        self._check(self._L.jne_plan_create(self._h, arr, len(reqs), outs, ctypes.byref(h)))
        return Plan(self, h)

    def eigs_seeded_models(self, models: Sequence[int], dim: int, steps: int, seed_first: int, n_runs: int,
                           precision: int = PREC_FP64, base_seed: int = DEFAULT_BASE_SEED) -> Dict[int, np.ndarray]:
        outs = {int(m): np.empty((n_runs, eigen_count(m, dim))) for m in models}
        arr = (ctypes.c_int * len(models))(*[int(m) for m in models])
        ptrs = (ctypes.POINTER(ctypes.c_double) * len(models))(*[_dp(outs[int(m)]) for m in models])
        self._check(self._L.jne_eigs_seeded_models(self._h, arr, len(models), dim, steps, base_seed, seed_first,
                                                   n_runs, precision, ptrs))
        return outs

    def export_increments(self, dim: int, steps: int, seed_first: int, n_runs: int,
                          base_seed: int = DEFAULT_BASE_SEED, words: bool = False) -> Tuple[np.ndarray, Optional[np.ndarray]]:
        dB = np.empty((n_runs, steps, dim))
        w = np.empty((n_runs, steps, (dim + 3) // 4, 4), dtype=np.uint32) if words else None
        wp = w.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)) if words else None
        self._check(self._L.jne_export_increments(self._h, dim, steps, base_seed, seed_first, n_runs, _dp(dB), wp))
        return dB, w


class Plan:
    """A captured ragged batch (jne_plan); launch() replays it asynchronously."""

    def __init__(self, engine: Engine, handle: ctypes.c_void_p):
        self._eng, self._h = engine, handle

    def launch(self, stream: Optional[int] = None) -> None:
        self._eng._check(self._eng._L.jne_plan_launch(self._h, ctypes.c_void_p(stream or 0)))

    def destroy(self) -> None:
        if self._h:
            self._eng._L.jne_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop on an engine (jne_server_*).  While it is
    open, its worker thread owns the engine's context."""

    def __init__(self, engine: Engine, data_dir: Optional[str] = None, iter_work: int = 0):
        self._eng, self._L = engine, engine._L
        h = ctypes.c_void_p()
        engine._check(self._L.jne_server_open(engine._h, os.fsencode(data_dir) if data_dir else None, iter_work,
                                              ctypes.byref(h)))
        self._h = h
        self._k: Dict[int, int] = {}

    def submit(self, model: int, dim: int, steps: int, n_runs: int, seed_first: int = 1,
               base_seed: int = DEFAULT_BASE_SEED, precision: int = PREC_MIXED) -> int:
        r = Request(int(model), dim, steps, precision, base_seed, seed_first, n_runs)
        rid = ctypes.c_uint64()
        rc = self._L.jne_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid))
        if rc != JNE_OK:
            raise JneError(rc, "request rejected")
        self._k[rid.value] = (n_runs, eigen_count(model, dim))
        return rid.value

    def wait(self, max_n: int = 256, timeout_ms: int = -1) -> List[Completion]:
        buf = (Completion * max_n)()
        n = ctypes.c_int()
        self._eng._check(self._L.jne_server_wait(self._h, buf, max_n, timeout_ms, ctypes.byref(n)))
        return [buf[i] for i in range(n.value)]

    def fetch(self, rid: int) -> np.ndarray:
        n, k = self._k.pop(rid)
        out = np.empty((n, k))
        rc = self._L.jne_server_fetch(self._h, rid, _dp(out), out.size)
        if rc != JNE_OK:
            if rc in (JNE_ERR_ARG, JNE_ERR_TIMEOUT):  # not finished / still being written: fetch again
                self._k[rid] = (n, k)
            raise JneError(rc, f"request {rid} not fetched")
        return out

    def close(self) -> None:
        if self._h:
            self._L.jne_server_close(self._h)
            self._h = None

    def __enter__(self) -> "Server":
        return self

    def __exit__(self, *exc) -> None:
        self.close()


# --------------------------------------------------------------------------
# EIGENVALS_V6 files, percentiles and the EigenvalueSimulation mirror
# --------------------------------------------------------------------------
class DatError(JneError):
    """A failed jne_dat_* / jne_simulation_* / jne_percentiles call (std::io::Error in the reference)."""


def _dat_check(rc: int) -> None:
    if rc != JNE_OK:
        raise DatError(rc, lib().jne_dat_last_error().decode(errors="replace"))


class Records:
    """(seed, eigenvalues) records backed by two arrays: a sequence of tuples like
    the reference's Vec<(u32, Vec<f64>)>, with .seeds (uint32) and .eigs (n x k)."""

    def __init__(self, seeds: np.ndarray, eigs: np.ndarray):
        self.seeds, self.eigs = seeds, eigs

    def __len__(self) -> int:
        return len(self.seeds)

    def __getitem__(self, i):
        return int(self.seeds[i]), self.eigs[i]

    def __iter__(self):
        return ((int(s), e) for s, e in zip(self.seeds, self.eigs))

    def sorted_by_seed(self) -> "Records":
        o = np.argsort(self.seeds, kind="stable")
        return Records(self.seeds[o], self.eigs[o])


class DatWriter:
    """Append-only writer (writer.rs:16-303)."""

    def __init__(self, path: str, model: int, dim: int, steps: int):
        L = lib()
        h, existing = ctypes.c_void_p(), ctypes.c_int64()
        _dat_check(L.jne_dat_open(os.fsencode(path), int(model), dim, steps, ctypes.byref(h), ctypes.byref(existing)))
        self._h, self.existing = h, existing.value

    def append(self, seeds: Sequence[int], eigs: np.ndarray) -> None:
        s = np.ascontiguousarray(seeds, dtype=np.uint32)
        e = np.ascontiguousarray(eigs, dtype=np.float64).reshape(len(s), -1)
        _dat_check(lib().jne_dat_append(self._h, s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), _dp(e),
                                        len(s), e.shape[1]))

    def append_packed(self, seed_first: int, n: int, k: int, records: bytes) -> None:
        """jne_dat_append_packed: n records of seeds seed_first.. already packed (record_bytes(...) bytes)."""
        if len(records) != record_bytes(seed_first, n, k):
            raise ValueError("records must hold record_bytes(seed_first, n, k) bytes")
        buf = ctypes.create_string_buffer(bytes(records), len(records))
        _dat_check(lib().jne_dat_append_packed(self._h, seed_first, int(n), int(k), buf))

    def append_eigenvalues(self, seed: int, eigenvalues: Sequence[float]) -> None:
        self.append([seed], np.asarray(eigenvalues, dtype=np.float64).reshape(1, -1))

    def finish(self) -> None:
        h, self._h = self._h, None
        _dat_check(lib().jne_dat_finish(h))

    def abandon(self) -> None:
        """Close without the EOF trailer (as an interrupted run leaves the file)."""
        h, self._h = self._h, None
        lib().jne_dat_abandon(h)


def record_bytes(seed_first: int, n: int, k: int) -> int:
    """jne_record_bytes: bytes of the .dat records of n consecutive seeds with k values each (-1: bad arguments)."""
    return int(lib().jne_record_bytes(seed_first, int(n), int(k)))


def read_dat(path: str) -> Tuple[Records, int, int, int]:
    """read_append_file (reader.rs:23-73): (records, model, dim, steps)."""
    L = lib()
    model, dim, k = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    steps, n = ctypes.c_uint32(), ctypes.c_int64()
    p = os.fsencode(path)
    _dat_check(L.jne_dat_read(p, ctypes.byref(model), ctypes.byref(dim), ctypes.byref(steps), ctypes.byref(n),
                              ctypes.byref(k), None, None, 0))
    seeds = np.empty(n.value, dtype=np.uint32)
    eigs = np.empty((n.value, k.value))
    if n.value:
        _dat_check(L.jne_dat_read(p, None, None, None, ctypes.byref(n), ctypes.byref(k),
                                  seeds.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), _dp(eigs), n.value))
    return Records(seeds, eigs), model.value, dim.value, steps.value


def percentiles(eigs: np.ndarray, stat: str, ps: Sequence[float]) -> List[float]:
    """simulation_analyzers.rs:4-81 for stat 'trace' (Sum) or 'maxeig' (Max)."""
    e = np.ascontiguousarray(eigs, dtype=np.float64)
    e = e.reshape(len(e), -1) if e.size else np.zeros((0, 1))
    p = np.ascontiguousarray(ps, dtype=np.float64)
    out = np.empty(len(p))
    _dat_check(lib().jne_percentiles(_dp(e), len(e), e.shape[1], 0 if stat == "trace" else 1, _dp(p), len(p),
                                     _dp(out)))
    return out.tolist()


def run_simulations(models: Sequence[int], dim: int, steps: int, num_runs: int, data_dir: str = "data",
                    precision: int = PREC_MIXED, base_seed: int = DEFAULT_BASE_SEED, quiet: bool = True,
                    engine: Optional["Engine"] = None) -> None:
    """run_simulation for several models of one (dim, steps) at once: the same files as one
    EigenvalueSimulation per model, from one pass over the paths when their missing seeds agree."""
    eng = engine or default_engine()
    arr = (ctypes.c_int * len(models))(*[int(m) for m in models])
    rc = lib().jne_simulation_run_models(eng._h, os.fsencode(data_dir), arr, len(models), dim, steps, num_runs,
                                         precision, base_seed, int(quiet))
    if rc != JNE_OK:
        raise DatError(rc, lib().jne_dat_last_error().decode(errors="replace"))


_engine: Optional[Engine] = None


def default_engine() -> Engine:
    global _engine
    if _engine is None:
        _engine = Engine(0)
    return _engine


class EigenvalueSimulation:
    """Mirror of the reference's EigenvalueSimulation (src/data_storage/simulation.rs:11-122).

    Runs go to the GPU (precision JNE_PREC_MIXED by default, JNE_PREC_FP64 on
    request); records are written to data_dir/eigenvalues_model{m}_dim{d}_steps{T}.dat
    in the reference's EIGENVALS_V6 format, with the same resume semantics."""

    def __init__(self, model, dim: int, steps: int, num_runs: int, data_dir: str = "data",
                 precision: int = PREC_MIXED, base_seed: int = DEFAULT_BASE_SEED, engine: Optional[Engine] = None):
        self.model = JohansenModel(int(model))
        self.dim, self.steps, self.num_runs = dim, steps, num_runs
        self.data_dir, self.precision, self.base_seed = data_dir, precision, base_seed
        self._engine = engine

    @classmethod
    def new(cls, model, dim: int, steps: int, num_runs: int, **kw) -> "EigenvalueSimulation":
        return cls(model, dim, steps, num_runs, **kw)

    def _run(self, quiet: bool) -> None:
        eng = self._engine or default_engine()
        rc = lib().jne_simulation_run(eng._h, os.fsencode(self.data_dir), int(self.model), self.dim, self.steps,
                                      self.num_runs, self.precision, self.base_seed, int(quiet))
        if rc != JNE_OK:
            # reference: run_model_simulation panics on writer or compute errors
            raise DatError(rc, lib().jne_dat_last_error().decode(errors="replace"))

    def run_simulation(self) -> None:
        self._run(False)

    def run_simulation_quiet(self) -> None:
        self._run(True)

    def get_filename(self, model=None) -> str:
        m = self.model if model is None else JohansenModel(int(model))
        os.makedirs(self.data_dir, exist_ok=True)
        buf = ctypes.create_string_buffer(4096)
        _dat_check(lib().jne_simulation_filename(os.fsencode(self.data_dir), int(m), self.dim, self.steps, buf, 4096))
        return buf.value.decode()

    def read_all_data(self) -> Records:
        return read_dat(self.get_filename(self.model))[0]

    def read_data(self) -> Records:
        """Records with seed <= num_runs; an error when their count is not num_runs (simulation.rs:61-87)."""
        allr = self.read_all_data()
        keep = allr.seeds <= np.uint32(min(self.num_runs, 0xFFFFFFFF))
        got = Records(allr.seeds[keep], allr.eigs[keep])
        if len(got) != self.num_runs:
            m = len(got)
            raise DatError(JNE_ERR_FORMAT,
                           f"Data count mismatch: expected {self.num_runs} records, found {m} records. "
                           "This indicates incomplete simulation data.\nSolutions:\n"
                           f"1. Use `read_all_data()` to read available data ({m} records)\n"
                           "2. Run `run_simulation()` to complete the simulation\n"
                           f"3. Create a new EigenvalueSimulation with num_runs={m} to match existing data")
        return got

    def calculate_trace_percentiles(self, ps: Sequence[float]) -> List[float]:
        data = self.read_data()
        return [] if len(data) == 0 else percentiles(data.eigs, "trace", ps)

    def calculate_maxeig_percentiles(self, ps: Sequence[float]) -> List[float]:
        data = self.read_data()
        return [] if len(data) == 0 else percentiles(data.eigs, "maxeig", ps)
