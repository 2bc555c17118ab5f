"""jne_eigs_seeded_noalloc: the seeded batch for callers that cannot allocate
device memory (a host framework that owns the GPU's allocator, a region being
captured into a CUDA graph, a real-time loop).  It is called through the C ABI
and checked against the context entry point, jne_eigs_seeded, on two calls in a
row that reuse the same static scratch.  This file is collected last, so a run
that stops at the first failure has already run every other test."""
import ctypes

import pytest

from conftest import normwise_err

pytestmark = pytest.mark.gpu


def _entry(jne):
    L = jne.lib()
    f = L.jne_eigs_seeded_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32,
                  ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    L.jne_noalloc_last_error.restype = ctypes.c_char_p
    return f, L


def test_no_alloc_matches_context_entry_point(jne, engine):
    import torch

    f, L = _entry(jne)
    # (model, dim, steps, seed_first, n_runs, precision); the second call fills the scratch to its limit
    calls = [(4, 12, 1000, 1, 700, jne.PREC_MIXED), (1, 5, 300, 50, 2048, jne.PREC_FP64)]
    for model, dim, steps, s0, n, prec in calls:
        k = jne.eigen_count(model, dim)
        out = torch.full((n, k), float("nan"), dtype=torch.float64, device="cuda")
        rc = f(0, model, dim, steps, jne.DEFAULT_BASE_SEED, s0, n, prec, out.data_ptr(), None)
        assert rc == jne.JNE_OK, L.jne_noalloc_last_error()
        ref = engine.eigs_seeded(model, dim, steps, s0, n, precision=prec)
        got = out.cpu().numpy()
        # the parity tests' tolerances: FP64 1e-9 normwise; mixed 2e-6 relative to max(lambda_max, 1)
        if prec == jne.PREC_FP64:
            assert normwise_err(got, ref) < 1e-9
        else:
            assert normwise_err(got, ref, 1.0) < 2e-6


def test_no_alloc_rejects_sizes_beyond_its_scratch(jne):
    import torch

    f, L = _entry(jne)
    out = torch.empty((2049, 2), dtype=torch.float64, device="cuda")
    rc = f(0, 0, 2, 100, jne.DEFAULT_BASE_SEED, 1, 2049, jne.PREC_FP64, out.data_ptr(), None)
    assert rc == jne.JNE_ERR_BUDGET
    assert b"2048" in L.jne_noalloc_last_error()
    rc = f(0, 0, 2, 300_000_000, jne.DEFAULT_BASE_SEED, 1, 4, jne.PREC_MIXED, out.data_ptr(), None)
    assert rc == jne.JNE_ERR_BUDGET
    assert b"steps" in L.jne_noalloc_last_error()
