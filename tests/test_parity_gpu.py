"""Parity of the sm_103a kernels with the CPU oracle, through the C ABI.

Tolerances (per run, max_j |got - ref| / max(max_j |ref|, floor)):
  plain FP64 kernel   1e-9, floor 0 (plain normwise-relative)
  mixed kernel        floor 1 (absolute for runs whose eigenvalues are all below
                      1, see conftest.normwise_err): 2e-6 from T = 1000 on, 4e-6
                      for 256 <= T < 1000 (few chunks: the FP32 centred part is a
                      larger share of every moment); below T = 256 mixed requests
                      run the FP64 kernel (JNE_MIXED_MIN_STEPS).  At dim 12, T 10^4
                      the max-eigenvalue and trace errors against the FP64 kernel
                      on identical seeds must stay <= 1e-6 (relative) every run.
"""
import numpy as np
import pytest

from conftest import normwise_err

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9
TOL_MIXED = 2e-6
FLOOR = {0: 0.0, 1: 1.0}  # per precision


MIXED_MIN_STEPS = 256  # JNE_MIXED_MIN_STEPS: shorter mixed requests run the FP64 kernel


def tol_mixed(steps: int) -> float:
    if steps < MIXED_MIN_STEPS:
        return TOL_FP64
    return 2e-6 if steps >= 1000 else 4e-6


def tol(precision: int, steps: int) -> float:
    return TOL_FP64 if precision == 0 else tol_mixed(steps)


def test_philox_words_bit_exact(engine, oracle):
    for dim in (1, 5, 12):
        _, words = engine.export_increments(dim, 70, 11, 3, words=True)
        for r in range(3):
            ref = oracle.c_philox_words(oracle.DEFAULT_BASE_SEED, dim, 11 + r, 70)
            assert np.array_equal(words[r], ref), dim


def test_normals_match_oracle(engine, oracle):
    dim, steps = 12, 500
    dB, _ = engine.export_increments(dim, steps, 100, 4)
    for r in range(4):
        z = oracle.c_normals(oracle.DEFAULT_BASE_SEED, dim, 100 + r, steps)
        assert np.max(np.abs(dB[r] * np.sqrt(steps) - z)) < 1e-4


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_golden_fixture(engine, golden, precision):
    cases, eigs = golden
    for (model, dim, steps), ref in eigs.items():
        got = engine.eigs_from_increments(model, cases[(dim, steps)], precision=precision)
        assert normwise_err(got, ref, FLOOR[precision]) < tol(precision, steps), (model, dim, steps)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_seeded_path_matches_oracle_on_its_increments(engine, oracle, precision):
    for dim in (1, 2, 5, 9, 12):
        for steps in (37, 1000):
            dB, _ = engine.export_increments(dim, steps, 1, 4)
            for model in range(5):
                if steps <= oracle.eigen_count(model, dim) + 1:
                    continue
                ref = oracle.c_eigs_from_increments(model, dB)
                got = engine.eigs_seeded(model, dim, steps, 1, 4, precision=precision)
                assert normwise_err(got, ref, FLOOR[precision]) < tol(precision, steps), (model, dim, steps)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_all_models_in_one_pass_equal_single_model_calls(engine, precision):
    outs = engine.eigs_seeded_models(range(5), 4, 300, 1, 16, precision=precision)
    for m in range(5):
        single = engine.eigs_seeded(m, 4, 300, 1, 16, precision=precision)
        assert np.array_equal(outs[m], single), m


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_run_result_independent_of_batch_and_repeatable(engine, precision):
    big = engine.eigs_seeded(3, 7, 777, 1, 40, precision=precision)
    small = engine.eigs_seeded(3, 7, 777, 11, 5, precision=precision)
    assert np.array_equal(big[10:15], small)
    assert np.array_equal(big, engine.eigs_seeded(3, 7, 777, 1, 40, precision=precision))


@pytest.mark.parametrize("steps", [2, 3, 31, 32, 33, 63, 255, 256, 257, 300, 513])
def test_ragged_step_counts(engine, oracle, steps):
    for dim in (1, 2, 12):
        dB, _ = engine.export_increments(dim, steps, 5, 3)
        for model in range(5):
            if steps <= oracle.eigen_count(model, dim) + 1:
                continue
            ref = oracle.c_eigs_from_increments(model, dB)
            for precision in (0, 1):
                got = engine.eigs_seeded(model, dim, steps, 5, 3, precision=precision)
                err = normwise_err(got, ref, FLOOR[precision])
                assert err < tol(precision, steps), (model, dim, steps, precision, err)


def test_singular_s11_is_reported(engine, jne):
    # steps = 1: F = B_0 = 0, so S11 = 0 (the reference's dggev returns inf/NaN here)
    with pytest.raises(jne.JneError) as ei:
        engine.eigs_seeded(0, 1, 1, 1, 2)
    assert ei.value.code == jne.JNE_ERR_NUMERIC


def test_short_mixed_requests_run_fp64(engine):
    for steps in (40, 255):
        f = engine.eigs_seeded(2, 5, steps, 1, 6, precision=0)
        assert np.array_equal(engine.eigs_seeded(2, 5, steps, 1, 6, precision=1), f)
    f = engine.eigs_seeded(2, 5, 256, 1, 6, precision=0)
    m = engine.eigs_seeded(2, 5, 256, 1, 6, precision=1)
    assert not np.array_equal(m, f) and normwise_err(m, f, 1.0) < tol_mixed(256)


def test_device_path_matches_host_path(engine):
    import torch

    for prec in (0, 1):
        ref = engine.eigs_seeded(4, 6, 2000, 3, 500, precision=prec)
        out = torch.empty((500, 6), dtype=torch.float64, device="cuda")
        engine.eigs_seeded_device(4, 6, 2000, 3, 500, out.data_ptr(), precision=prec)
        engine.sync()
        assert np.array_equal(out.cpu().numpy(), ref)


def test_device_path_reports_status_at_sync(engine, jne):
    import torch

    out = torch.empty((2, 1), dtype=torch.float64, device="cuda")
    engine.eigs_seeded_device(0, 1, 1, 1, 2, out.data_ptr())  # S11 = 0: not positive definite
    with pytest.raises(jne.JneError) as ei:
        engine.sync()
    assert ei.value.code == jne.JNE_ERR_NUMERIC
    engine.sync()  # cleared


def test_empty_batch(engine):
    assert engine.eigs_seeded(0, 3, 100, 1, 0).shape == (0, 3)


def test_bad_arguments(engine, jne):
    for args in ((0, 13, 100), (5, 2, 100), (0, 2, 0), (-1, 2, 100)):
        with pytest.raises(jne.JneError) as ei:
            engine.eigs_seeded(args[0], args[1], args[2], 1, 1)
        assert ei.value.code == jne.JNE_ERR_ARG
    with pytest.raises(jne.JneError) as ei:
        engine.eigs_seeded(0, 2, 100, 1, 1, precision=7)
    assert ei.value.code == jne.JNE_ERR_ARG
    with pytest.raises(jne.JneError) as ei:  # seed range past u32::MAX
        engine.eigs_seeded(0, 2, 100, 2**32 - 2, 5)
    assert ei.value.code == jne.JNE_ERR_ARG
    with pytest.raises(jne.JneError) as ei:
        engine.set_chunk(100)
    assert ei.value.code == jne.JNE_ERR_ARG
    # chunks longer than 8192 steps could push the chunk-local walk past FP16's range
    with pytest.raises(jne.JneError) as ei:
        engine.set_chunk(8192 + 32)
    assert ei.value.code == jne.JNE_ERR_ARG
    engine.set_chunk(8192)
    engine.set_chunk(0)


def test_budget_is_enforced(jne):
    with jne.Engine(0, mem_budget_bytes=4096) as small:
        with pytest.raises(jne.JneError) as ei:
            small.eigs_seeded(0, 12, 100, 1, 10)
        assert ei.value.code == jne.JNE_ERR_BUDGET
        with pytest.raises(jne.JneError) as ei:
            small.eigs_from_increments(0, np.zeros((4, 100, 12)))
        assert ei.value.code == jne.JNE_ERR_BUDGET


def test_chunk_length_changes_only_rounding(jne):
    with jne.Engine(0, chunk=64) as a, jne.Engine(0, chunk=512) as b:
        x = a.eigs_seeded(4, 6, 3000, 1, 8, precision=1)
        y = b.eigs_seeded(4, 6, 3000, 1, 8, precision=1)
        assert normwise_err(x, y, 1.0) < 2 * TOL_MIXED  # two mixed results


def test_full_size_mixed_error_vs_fp64(engine):
    """dim 12, T 10^4 on identical seeds: mixed max-eig and trace within 1e-6 of FP64."""
    for model in range(5):
        f = engine.eigs_seeded(model, 12, 10_000, 1, 256, precision=0)
        m = engine.eigs_seeded(model, 12, 10_000, 1, 256, precision=1)
        maxeig = np.max(np.abs(m[:, 0] - f[:, 0]) / f[:, 0])
        trace = np.max(np.abs(m.sum(1) - f.sum(1)) / f.sum(1))
        assert maxeig <= 1e-6 and trace <= 1e-6, (model, maxeig, trace)


def test_distribution_matches_cpu_oracle(engine, oracle):
    """Independent samples (different base seeds): two-sample KS and the
    1/5/10/50/90/95/99% quantiles of trace and max-eig (simulation_analyzers.rs rule)."""
    from scipy.stats import ks_2samp

    n, dim, steps = 3000, 2, 1000
    for model in (0, 4):
        for precision in (0, 1):
            gpu = engine.eigs_seeded(model, dim, steps, 1, n, precision=precision)
            cpu = oracle.c_eigs_seeded(model, dim, steps, 1, n, n_threads=8, base_seed=12345)
            for stat in (lambda e: e.sum(1), lambda e: e.max(1)):
                a, b = np.sort(stat(gpu)), np.sort(stat(cpu))
                assert ks_2samp(a, b).pvalue > 1e-3
                for p in (0.01, 0.05, 0.1, 0.5, 0.9, 0.95, 0.99):
                    qa, qb = oracle.percentile_value(a, p), oracle.percentile_value(b, p)
                    # Monte Carlo error of a quantile: ~ sqrt(p(1-p)/n) / density; compare in rank space
                    rank_b = np.searchsorted(b, qa) / n
                    assert abs(rank_b - p) < 5 * np.sqrt(p * (1 - p) / n) + 2.0 / n, (model, p, qa, qb)


def test_probe_rates_are_measured(engine):
    r = engine.probe_rates()
    assert set(r) == {"normals_per_s", "dfma_flops", "mma_tf32_flops", "ffma_flops", "mma_f16_flops"}
    assert 1e10 < r["normals_per_s"] < 1e14
    assert 1e11 < r["dfma_flops"] < r["ffma_flops"]
    assert 1e12 < r["mma_tf32_flops"] < 1e16
    assert 1e12 < r["mma_f16_flops"] < 1e16


def test_longest_chunk_keeps_fp16_operands_finite(jne):
    # chunks of 8192 steps: the chunk-local walk is the largest FP16 operand; results stay finite and close
    # to FP64 (long chunks only cost accuracy, here of order 1e-5)
    with jne.Engine(0, chunk=8192) as eng:
        for dim in (1, 12):
            m = eng.eigs_seeded(0, dim, 16384, 1, 64, precision=1)
            f = eng.eigs_seeded(0, dim, 16384, 1, 64, precision=0)
            assert np.all(np.isfinite(m))
            assert normwise_err(m, f, 1.0) < 1e-3, dim


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_every_dim_and_model_vs_oracle(engine, oracle, precision):
    """dims 1..12 x models 0..4 at T = 3000 (chunk 128: several chunks and a partial last tile), 4 runs each,
    against the oracle on the kernels' own increments; mixed also against its max-eig / trace bound."""
    steps = 3000
    for dim in range(1, 13):
        dB, _ = engine.export_increments(dim, steps, 21, 4)
        for model in range(5):
            ref = oracle.c_eigs_from_increments(model, dB)
            got = engine.eigs_seeded(model, dim, steps, 21, 4, precision=precision)
            assert normwise_err(got, ref, FLOOR[precision]) < tol(precision, steps), (model, dim)
            if precision == 1:
                assert np.max(np.abs(got[:, 0] - ref[:, 0]) / np.maximum(ref[:, 0], 1.0)) <= 1e-6, (model, dim)


def test_long_paths_vs_oracle(engine, oracle):
    """T = 50,000 (98 chunks of 512 steps in mixed precision), dims 4 and 12, all five models, against the
    oracle on the kernels' own increments: FP64 1e-9, mixed 2e-6 normwise and 1e-6 on the largest eigenvalue."""
    steps = 50_000
    for dim in (4, 12):
        dB, _ = engine.export_increments(dim, steps, 7, 3)
        for model in range(5):
            ref = oracle.c_eigs_from_increments(model, dB, n_threads=3)
            f64 = engine.eigs_seeded(model, dim, steps, 7, 3, precision=0)
            mix = engine.eigs_seeded(model, dim, steps, 7, 3, precision=1)
            assert normwise_err(f64, ref) < TOL_FP64, (model, dim)
            assert normwise_err(mix, ref, 1.0) < TOL_MIXED, (model, dim)
            assert np.max(np.abs(mix[:, 0] - ref[:, 0]) / ref[:, 0]) <= 1e-6, (model, dim)


def test_seeds_at_the_top_of_the_u32_range(engine, oracle):
    """The last seeds a request may name (seed_first + n_runs - 1 = 2^32 - 1): Philox words bit-exact with the
    oracle, eigenvalues within the FP64 tolerance on the kernels' own increments."""
    first, n, dim, steps = 2**32 - 5, 5, 6, 400
    dB, words = engine.export_increments(dim, steps, first, n, words=True)
    for r in range(n):
        assert np.array_equal(words[r], oracle.c_philox_words(oracle.DEFAULT_BASE_SEED, dim, first + r, steps))
    for model in (0, 3):
        ref = oracle.c_eigs_from_increments(model, dB)
        assert normwise_err(engine.eigs_seeded(model, dim, steps, first, n, precision=0), ref) < TOL_FP64
        assert normwise_err(engine.eigs_seeded(model, dim, steps, first, n, precision=1), ref, 1.0) < TOL_MIXED


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_distribution_vs_independent_stream_dim6(engine, oracle, precision):
    """A middle shape (dim 6, T 5000, models 0-4): 4,000 GPU runs against 4,000 oracle runs of the independent
    xoshiro256++ stream with untruncated normals -- two-sample KS on the trace and the largest eigenvalue, and
    the 1/5/10/50/90/95/99 % quantiles within five Monte Carlo standard errors in rank space."""
    import os

    from scipy.stats import ks_2samp

    n, dim, steps = 4000, 6, 5000
    threads = max(1, min(32, os.cpu_count() or 1))
    for model in range(5):
        gpu = engine.eigs_seeded(model, dim, steps, 1, n, precision=precision)
        cpu = oracle.c_eigs_seeded_xoshiro(model, dim, steps, 1, n, n_threads=threads, base_seed=0xD16)
        assert np.all(np.isfinite(gpu))
        for name, stat in (("trace", lambda e: e.sum(1)), ("maxeig", lambda e: e.max(1))):
            a, b = np.sort(stat(gpu)), np.sort(stat(cpu))
            assert ks_2samp(a, b).pvalue > 1e-4, (model, name)
            for p in (0.01, 0.05, 0.1, 0.5, 0.9, 0.95, 0.99):
                rank_b = np.searchsorted(b, oracle.percentile_value(a, p)) / n
                assert abs(rank_b - p) < 5 * np.sqrt(2 * p * (1 - p) / n) + 2.0 / n, (model, name, p, rank_b)
