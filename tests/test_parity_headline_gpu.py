"""Parity at the benchmarked shape: dim 12, T = 10,000 steps, models 0-4.

The kernels against the CPU oracle (not against each other):

* per run, on the increments the kernels draw (exported through the C ABI and
  walked by the oracle's dense restatement of johansen_statistics.rs:59-85):
  plain FP64 within 1e-9 normwise-relative; mixed precision within 1e-6
  relative on the largest eigenvalue and on the trace, and 1e-6 normwise
  (relative to max(lambda_max, 1));
* on the dggev golden fixture at this shape (explicit increments);
* in distribution: 5,000 GPU runs per model and precision against 5,000 runs of
  the oracle on an independent generator (xoshiro256++ with untruncated
  Box-Muller normals), by a two-sample KS test and the 1/5/10/50/90/95/99 %
  quantiles of the trace and the largest eigenvalue (the percentile rule of
  simulation_analyzers.rs:4-18).  The kernels' normals are bounded at
  |z| <= 6.77 (32-bit radius uniforms); the independent sample is not, so these
  tests also bound the effect of that truncation on the statistic.
"""
import os

import numpy as np
import pytest

from conftest import normwise_err

pytestmark = pytest.mark.gpu

DIM, STEPS = 12, 10_000
TOL_FP64 = 1e-9
TOL_MIXED_STAT = 1e-6  # max-eig and trace, relative
TOL_MIXED_NORMWISE = 1e-6  # every eigenvalue, relative to max(lambda_max, 1): the stated 1e-6 target
PS = (0.01, 0.05, 0.1, 0.5, 0.9, 0.95, 0.99)


def _threads() -> int:
    return max(1, min(32, os.cpu_count() or 1))


def _stat_errors(got: np.ndarray, ref: np.ndarray):
    maxeig = np.abs(got[:, 0] - ref[:, 0]) / np.abs(ref[:, 0])
    trace = np.abs(got.sum(1) - ref.sum(1)) / np.abs(ref.sum(1))
    return float(maxeig.max()), float(trace.max())


@pytest.fixture(scope="module")
def headline_increments(engine):
    """The increments the kernels draw for seeds 1..64 at dim 12, T 10^4."""
    dB, _ = engine.export_increments(DIM, STEPS, 1, 64)
    return dB


@pytest.mark.parametrize("model", range(5))
def test_per_run_vs_oracle(engine, oracle, headline_increments, model):
    dB = headline_increments
    n = dB.shape[0]
    ref = oracle.c_eigs_from_increments(model, dB, n_threads=_threads())
    f64 = engine.eigs_seeded(model, DIM, STEPS, 1, n, precision=0)
    mix = engine.eigs_seeded(model, DIM, STEPS, 1, n, precision=1)
    assert normwise_err(f64, ref) < TOL_FP64, model
    maxeig, trace = _stat_errors(mix, ref)
    assert maxeig <= TOL_MIXED_STAT and trace <= TOL_MIXED_STAT, (model, maxeig, trace)
    assert normwise_err(mix, ref, 1.0) < TOL_MIXED_NORMWISE, model


def test_golden_fixture_at_headline_shape(engine, golden):
    """dggev eigenvalues of fixed increments (regenerated from a frozen stream) through the explicit-
    increment entry point; mixed precision there uses the TF32 split (unbounded inputs)."""
    cases, eigs = golden
    dB = cases[(DIM, STEPS)]
    for model in range(5):
        ref = eigs[(model, DIM, STEPS)]
        f64 = engine.eigs_from_increments(model, dB, precision=0)
        mix = engine.eigs_from_increments(model, dB, precision=1)
        assert normwise_err(f64, ref) < TOL_FP64, model
        maxeig, trace = _stat_errors(mix, ref)
        assert maxeig <= TOL_MIXED_STAT and trace <= TOL_MIXED_STAT, (model, maxeig, trace)


@pytest.fixture(scope="module")
def independent_sample(oracle):
    """5,000 oracle runs per model from the independent stream (seeds 1..5000, another base seed)."""
    return {m: oracle.c_eigs_seeded_xoshiro(m, DIM, STEPS, 1, 5000, n_threads=_threads(), base_seed=0x5EED)
            for m in range(5)}


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_distribution_vs_independent_stream(engine, oracle, independent_sample, precision):
    from scipy.stats import ks_2samp

    n = 5000
    for model in range(5):
        gpu = engine.eigs_seeded(model, DIM, STEPS, 1, n, precision=precision)
        cpu = independent_sample[model]
        assert np.all(np.isfinite(gpu))
        for name, stat in (("trace", lambda e: e.sum(1)), ("maxeig", lambda e: e.max(1))):
            a, b = np.sort(stat(gpu)), np.sort(stat(cpu))
            p = ks_2samp(a, b).pvalue
            assert p > 1e-4, (model, name, p)
            for q in PS:
                qa = oracle.percentile_value(a, q)
                # the GPU quantile's rank in the independent sample: Monte Carlo error of two samples
                rank_b = np.searchsorted(b, qa) / n
                assert abs(rank_b - q) < 5 * np.sqrt(2 * q * (1 - q) / n) + 2.0 / n, (model, name, q, rank_b)
