"""jne_eigs_seeded_noalloc: the seeded batch for callers that cannot allocate
device memory (a host framework that owns the GPU's allocator, a real-time loop
that allows no allocation after start-up).  It is called through the C ABI and
checked against the context entry point, jne_eigs_seeded, on calls in a row
that reuse the same static scratch: it runs the same kernels and tables, so the
results must be the same bits.  This file is collected last, so a run that
stops at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

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
    # (model, dim, steps, seed_first, n_runs, precision): mixed, FP64 filling the scratch to its limit,
    # then mixed again at the headline shape (packed small dims in between)
    calls = [(4, 12, 1000, 1, 700, jne.PREC_MIXED), (1, 5, 300, 50, 2048, jne.PREC_FP64),
             (2, 3, 2000, 9, 333, jne.PREC_MIXED), (0, 12, 10_000, 1, 256, jne.PREC_MIXED)]
    for model, dim, steps, s0, n, prec in calls:
        k = jne.eigen_count(model, dim)
        out = torch.full((n, k), float("nan"), dtype=torch.float64, device="cuda")
        rc = f(0, model, dim, steps, jne.DEFAULT_BASE_SEED, s0, n, prec, out.data_ptr(), None)
        assert rc == jne.JNE_OK, L.jne_noalloc_last_error()
        ref = engine.eigs_seeded(model, dim, steps, s0, n, precision=prec)
        assert np.array_equal(out.cpu().numpy(), ref), (model, dim, steps, prec)


def test_no_alloc_reports_a_singular_run(jne):
    import torch

    f, L = _entry(jne)
    out = torch.empty((4, 1), dtype=torch.float64, device="cuda")
    # steps = 1: S11 = 0, not positive definite (NaN written)
    rc = f(0, 0, 1, 1, jne.DEFAULT_BASE_SEED, 1, 4, jne.PREC_FP64, out.data_ptr(), None)
    assert rc == jne.JNE_ERR_NUMERIC
    assert torch.isnan(out).all()
    # the status word is cleared by the next call
    out2 = torch.empty((4, 2), dtype=torch.float64, device="cuda")
    rc = f(0, 0, 2, 300, jne.DEFAULT_BASE_SEED, 1, 4, jne.PREC_FP64, out2.data_ptr(), None)
    assert rc == jne.JNE_OK, L.jne_noalloc_last_error()


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
