"""CPU oracle (Python twin) for the Johansen null-eigenspectra Monte Carlo path.

TEST INFRASTRUCTURE ONLY: the checker for the pytest suite, the smoke check and
the CPU-baseline leg of bench.py.  The product library never imports it.

Two halves:

* A numpy/scipy restatement of the reference crate's dense algorithm for one run
  (``eigs_dense``), with the generalized eigenproblem handed to LAPACK
  ``dggev`` through ``scipy.linalg.eigvals`` -- the same routine the reference
  binds through nalgebra-lapack (johansen_statistics.rs:35-44).
* ctypes bindings to the C restatement ``jne_oracle.c`` (Cholesky + Jacobi),
  which is fast enough to serve as the threaded CPU baseline.

Plus restatements of the reference's storage format (ULEB128, the EIGENVALS_V6
``.dat`` layout) and its percentile rule, used to check the product's host code.
"""
from __future__ import annotations

import ctypes
import os
import struct
from typing import Iterable, List, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libjne_oracle.so")
DEFAULT_BASE_SEED = 0x4A4F48

PHILOX_M0, PHILOX_M1 = 0xD2511F53, 0xCD9E8D57
PHILOX_W0, PHILOX_W1 = 0x9E3779B9, 0xBB67AE85


# --------------------------------------------------------------------------
# Counter-based stream (bit-exact integer restatement, vectorised)
# --------------------------------------------------------------------------
def philox4x32_10(ctr: np.ndarray, key: Sequence[int]) -> np.ndarray:
    """Philox4x32-10 (Salmon et al., SC'11) on an (n, 4) uint32 counter array."""
    c = np.asarray(ctr, dtype=np.uint64).reshape(-1, 4).copy()
    k0, k1 = np.uint64(key[0]), np.uint64(key[1])
    m0, m1, mask = np.uint64(PHILOX_M0), np.uint64(PHILOX_M1), np.uint64(0xFFFFFFFF)
    for _ in range(10):
        p0 = m0 * c[:, 0]
        p1 = m1 * c[:, 2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & mask
        hi1, lo1 = p1 >> np.uint64(32), p1 & mask
        n0 = hi1 ^ c[:, 1] ^ k0
        n2 = hi0 ^ c[:, 3] ^ k1
        c = np.stack([n0, lo1, n2, lo0], axis=1)
        k0 = (k0 + np.uint64(PHILOX_W0)) & mask
        k1 = (k1 + np.uint64(PHILOX_W1)) & mask
    return c.astype(np.uint32)


def stream_key(base_seed: int, dim: int) -> Tuple[int, int]:
    """Key of the (base seed, dim) stream; the model is deliberately not part of it."""
    return (base_seed & 0xFFFFFFFF, ((base_seed >> 32) & 0xFFFFFFFF) ^ (0x4A4E0000 | (dim & 0xFF)))


def philox_words(base_seed: int, dim: int, run_seed: int, steps: int) -> np.ndarray:
    """Raw words of one run, shape (steps, ceil(dim/4), 4); counter = (s, j, seed, 0)."""
    nq = (dim + 3) // 4
    s = np.repeat(np.arange(1, steps + 1, dtype=np.uint64), nq)
    j = np.tile(np.arange(nq, dtype=np.uint64), steps)
    ctr = np.stack([s, j, np.full_like(s, run_seed), np.zeros_like(s)], axis=1)
    return philox4x32_10(ctr, stream_key(base_seed, dim)).reshape(steps, nq, 4)


def normals(base_seed: int, dim: int, run_seed: int, steps: int) -> np.ndarray:
    """Standard normals of one run, shape (steps, dim) (Box-Muller in float64)."""
    words = philox_words(base_seed, dim, run_seed, steps)
    w = words.astype(np.float64)
    u = (np.floor(w / 512.0) + 0.5) / 8388608.0  # angle words: top 23 bits + half an ulp
    # radius words: leading 24 bits (rounded toward zero to a float), + 1/2, times 2^-32, rounded to a float
    nb = np.where(words > 0, np.floor(np.log2(np.maximum(w, 1.0))).astype(np.int64) + 1, 0)
    drop = np.maximum(nb - 24, 0).astype(np.uint64)
    t = ((words.astype(np.uint64) >> drop) << drop).astype(np.float64)
    ur = ((t + 0.5) / 4294967296.0).astype(np.float32).astype(np.float64)
    r01 = np.sqrt(-2.0 * np.log(ur[..., 0]))
    r23 = np.sqrt(-2.0 * np.log(ur[..., 2]))
    t01 = 2.0 * np.pi * u[..., 1] - np.pi
    t23 = 2.0 * np.pi * u[..., 3] - np.pi
    z = np.stack([r01 * np.cos(t01), r01 * np.sin(t01), r23 * np.cos(t23), r23 * np.sin(t23)], axis=2)
    return z.reshape(steps, -1)[:, :dim]


# --------------------------------------------------------------------------
# Dense restatement of the reference algorithm
# --------------------------------------------------------------------------
def eigen_count(model: int, dim: int) -> int:
    """thread_manager.rs:40-44: dim+1 eigenvalues for models 1 and 3, dim otherwise."""
    return dim + 1 if model in (1, 3) else dim


def cumsum_rowwise(m: np.ndarray) -> np.ndarray:
    """dmatrix_cumsum(.., RowWise), matrix_utils.rs:51-63 (left-to-right per row)."""
    return np.cumsum(np.asarray(m, dtype=np.float64), axis=1)


def sum_of_outer_products(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """matrix_utils.rs:67-85: sum over columns i of a[:, i] b[:, i]'."""
    out = np.zeros((a.shape[0], b.shape[0]))
    for i in range(a.shape[1]):
        out += np.outer(a[:, i], b[:, i])
    return out


def brownian_from_increments(dB: np.ndarray) -> np.ndarray:
    """rng_matrix.rs:87-140 with start = 0: B = RowWise cumsum of [0 | dB], shape dim x (T+1)."""
    dim = dB.shape[0]
    return cumsum_rowwise(np.concatenate([np.zeros((dim, 1)), dB], axis=1))


def construct_f(bm_prev: np.ndarray, model: int) -> np.ndarray:
    """construct_f_matrix, johansen_statistics.rs:102-197."""
    rows, cols = bm_prev.shape
    t = float(cols)
    if model == 0:
        return bm_prev.copy()
    if model == 1:
        return np.vstack([bm_prev, np.ones((1, cols))])
    y = np.arange(1, cols + 1, dtype=np.float64) / t
    if model in (2, 3):
        nb = rows - 1 if model == 2 else rows
        x = bm_prev[:nb] - bm_prev[:nb].mean(axis=1, keepdims=True)
        return np.vstack([x, (y - 0.5)[None, :]])
    if model == 4:
        x = np.vstack([bm_prev[: rows - 1], (y ** 2)[None, :]])
        z = np.vstack([np.ones(cols), y])
        zzt_inv = np.linalg.inv(z @ z.T)
        return x - ((x @ z.T) @ zzt_inv) @ z
    raise ValueError(f"model {model} out of range 0..4")


def eigs_from_matrices(bm_prev: np.ndarray, dbm: np.ndarray, dt: float, model: int) -> np.ndarray:
    """calculate_eigenvalues_from_matrices, johansen_statistics.rs:24-47 (dggev via scipy)."""
    import scipy.linalg

    f = construct_f(bm_prev, model)
    s10 = dbm @ f.T
    s11 = (f @ f.T) * dt
    alpha, beta = scipy.linalg.eigvals(s10.T @ s10, s11, homogeneous_eigvals=True)
    lam = np.abs(alpha) / np.real(beta)
    return np.sort(lam)[::-1].copy()


def eigs_dense(model: int, dB: np.ndarray) -> np.ndarray:
    """calculate_eigenvalues, johansen_statistics.rs:59-85, from a dim x T increment matrix."""
    dB = np.asarray(dB, dtype=np.float64)
    steps = dB.shape[1]
    bm = brownian_from_increments(dB)
    bm_prev = bm[:, :steps]
    dbm = bm[:, 1:] - bm_prev
    return eigs_from_matrices(bm_prev, dbm, 1.0 / steps, model)


def pencil_matrices(model: int, dB: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """(S10, S11) of one run, as the reference forms them before the eigen call."""
    dB = np.asarray(dB, dtype=np.float64)
    steps = dB.shape[1]
    bm = brownian_from_increments(dB)
    f = construct_f(bm[:, :steps], model)
    dbm = bm[:, 1:] - bm[:, :steps]
    return dbm @ f.T, (f @ f.T) / steps


# --------------------------------------------------------------------------
# Storage format (EIGENVALS_V6) and analysis rules
# --------------------------------------------------------------------------
MAGIC_HEADER = b"EIGENVALS_V6"
EOF_MARKER = b"EOF_MARK"


def uleb128_encode(value: int) -> bytes:
    """uleb128.rs:68-87."""
    out = bytearray()
    while True:
        byte = value & 0x7F
        value >>= 7
        out.append(byte | (0x80 if value else 0))
        if not value:
            return bytes(out)


def uleb128_decode(buf: bytes) -> Tuple[int, int]:
    """uleb128.rs:102-137: (value, bytes used); ValueError on the reference's error cases."""
    result, shift = 0, 0
    for n, byte in enumerate(buf, start=1):
        if n > 5:
            raise ValueError("ULEB128 encoding too long")
        bits = byte & 0x7F
        if shift == 28 and bits > 0x0F:
            raise ValueError("ULEB128 value too large for u32")
        result |= bits << shift
        shift += 7
        if not byte & 0x80:
            return result, n
    raise ValueError("Incomplete ULEB128 encoding")


def dat_bytes(model: int, dim: int, steps: int, records: Iterable[Tuple[int, Sequence[float]]],
              finished: bool = True) -> bytes:
    """A whole EIGENVALS_V6 file (writer.rs:56-62, 242-249, 262-290; DATA_FORMAT.md)."""
    out = bytearray(MAGIC_HEADER + bytes([model, dim]) + struct.pack("<I", steps))
    count, per_run = 0, None
    for seed, eig in records:
        out += uleb128_encode(seed) + bytes([len(eig)]) + struct.pack(f"<{len(eig)}d", *eig)
        count += 1
        per_run = len(eig) if per_run is None else per_run
    if finished:
        out += EOF_MARKER + struct.pack("<Q", count) + bytes([per_run or 0])
    return bytes(out)


def dat_parse(buf: bytes) -> Tuple[List[Tuple[int, List[float]]], int, int, int]:
    """reader.rs:23-216 in one function: fast path when the EOF trailer is present, scan otherwise."""
    if buf[:12] != MAGIC_HEADER:
        raise ValueError("File format error: magic header mismatch")
    model, dim = buf[12], buf[13]
    (steps,) = struct.unpack("<I", buf[14:18])
    recs: List[Tuple[int, List[float]]] = []
    if len(buf) < 35:
        return recs, model, dim, steps
    pos = 18
    if buf[-17:-9] == EOF_MARKER:
        (total,) = struct.unpack("<Q", buf[-9:-1])
        for _ in range(total):
            seed, n = uleb128_decode(buf[pos:pos + 5])
            pos += n
            cnt = buf[pos]
            pos += 1
            recs.append((seed, list(struct.unpack(f"<{cnt}d", buf[pos:pos + 8 * cnt]))))
            pos += 8 * cnt
        return recs, model, dim, steps
    while pos < len(buf):
        try:
            seed, n = uleb128_decode(buf[pos:pos + 5])
        except ValueError:
            break
        if pos + n >= len(buf):
            break
        cnt = buf[pos + n]
        if pos + n + 1 + 8 * cnt > len(buf):
            break
        pos += n + 1
        recs.append((seed, list(struct.unpack(f"<{cnt}d", buf[pos:pos + 8 * cnt]))))
        pos += 8 * cnt
    return recs, model, dim, steps


def percentile_value(sorted_values: Sequence[float], p: float) -> float:
    """simulation_analyzers.rs:4-18: linear interpolation at rank p*(n-1)."""
    n = len(sorted_values)
    if n == 0:
        return float("nan")
    rank = p * (n - 1)
    lo, hi = int(np.floor(rank)), int(np.ceil(rank))
    if lo == hi:
        return float(sorted_values[lo])
    w = rank - lo
    return float(sorted_values[lo] * (1.0 - w) + sorted_values[hi] * w)


# --------------------------------------------------------------------------
# ctypes bindings to the C restatement
# --------------------------------------------------------------------------
_lib = None


def lib() -> ctypes.CDLL:
    """Load oracle/_build/libjne_oracle.so (built by __graft_entry__.build() or oracle/build.sh)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} missing: build it with oracle/build.sh")
        L = ctypes.CDLL(LIB_PATH)
        dp, u32p = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint32)
        L.jno_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.jno_philox_words.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_uint32, ctypes.c_int, u32p]
        L.jno_normals.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_uint32, ctypes.c_int, dp]
        L.jno_cumsum_rowwise.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp]
        L.jno_sum_of_outer_products.argtypes = [dp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, dp]
        L.jno_eigen_count.argtypes = [ctypes.c_int, ctypes.c_int]
        L.jno_eigs_from_increments.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, dp]
        L.jno_eigs_seeded.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                      ctypes.c_uint32, ctypes.c_int, ctypes.c_int, dp]
        L.jno_eigs_seeded_xoshiro.argtypes = L.jno_eigs_seeded.argtypes
        L.jno_eigs_from_increments_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int,
                                                  ctypes.c_int, dp]
        L.jno_xoshiro_normals.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, dp]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def c_philox(ctr: Sequence[int], key: Sequence[int]) -> List[int]:
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().jno_philox4x32_10(c, k, o)
    return list(o)


def c_philox_words(base_seed: int, dim: int, run_seed: int, steps: int) -> np.ndarray:
    nq = (dim + 3) // 4
    out = np.zeros((steps, nq, 4), dtype=np.uint32)
    lib().jno_philox_words(base_seed, dim, run_seed, steps, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return out


def c_normals(base_seed: int, dim: int, run_seed: int, steps: int) -> np.ndarray:
    out = np.zeros((steps, dim))
    lib().jno_normals(base_seed, dim, run_seed, steps, _dp(out))
    return out


def c_cumsum_rowwise(m: np.ndarray) -> np.ndarray:
    m = np.asfortranarray(m, dtype=np.float64)
    out = np.zeros_like(m, order="F")
    lib().jno_cumsum_rowwise(_dp(m), m.shape[0], m.shape[1], _dp(out))
    return out


def c_sum_of_outer_products(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a = np.asfortranarray(a, dtype=np.float64)
    b = np.asfortranarray(b, dtype=np.float64)
    out = np.zeros((a.shape[0], b.shape[0]), order="F")
    lib().jno_sum_of_outer_products(_dp(a), a.shape[0], _dp(b), b.shape[0], a.shape[1], _dp(out))
    return out


def c_eigs_from_increments(model: int, dB: np.ndarray, n_threads: int = 1) -> np.ndarray:
    """dB: (n_runs, steps, dim) array (each run's dim x T column-major matrix); returns (n_runs, k).
    n_threads > 1 splits the runs over POSIX threads (same results)."""
    dB = np.ascontiguousarray(dB, dtype=np.float64)
    n, steps, dim = dB.shape
    k = eigen_count(model, dim)
    out = np.zeros((n, k))
    if n_threads > 1:
        rc = lib().jno_eigs_from_increments_mt(model, dim, steps, _dp(dB), n, n_threads, _dp(out))
    else:
        rc = lib().jno_eigs_from_increments(model, dim, steps, _dp(dB), n, _dp(out))
    if rc < 0:
        raise ValueError("bad arguments")
    return out


def c_xoshiro_normals(base_seed: int, run_seed: int, n: int) -> np.ndarray:
    """n standard normals of the independent xoshiro256++ / Box-Muller stream (53-bit uniforms)."""
    out = np.zeros(n)
    lib().jno_xoshiro_normals(base_seed, run_seed, n, _dp(out))
    return out


def c_eigs_seeded_xoshiro(model: int, dim: int, steps: int, seed_first: int, n_runs: int,
                          n_threads: int = 1, base_seed: int = DEFAULT_BASE_SEED) -> np.ndarray:
    """Runs of the dense algorithm on increments from the independent xoshiro256++ stream: a sample of
    the same null distribution that shares no random number with the kernels (distribution tests)."""
    k = eigen_count(model, dim)
    out = np.zeros((n_runs, k))
    rc = lib().jno_eigs_seeded_xoshiro(model, dim, steps, base_seed, seed_first, n_runs, n_threads, _dp(out))
    if rc < 0:
        raise ValueError("bad arguments")
    return out


def c_eigs_seeded(model: int, dim: int, steps: int, seed_first: int, n_runs: int,
                  n_threads: int = 1, base_seed: int = DEFAULT_BASE_SEED) -> np.ndarray:
    k = eigen_count(model, dim)
    out = np.zeros((n_runs, k))
    rc = lib().jno_eigs_seeded(model, dim, steps, base_seed, seed_first, n_runs, n_threads, _dp(out))
    if rc < 0:
        raise ValueError("bad arguments")
    return out
