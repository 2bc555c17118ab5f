"""The CPU oracle, pinned against the reference's own known answers and against
LAPACK dggev (the routine the reference binds) -- no GPU needed."""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, normwise_err

KA = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_known_answers.json")))

# Published Philox4x32-10 known-answer vectors (Random123 distribution, kat_vectors).
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_known_answers(oracle, ctr, key, expect):
    assert tuple(oracle.c_philox(ctr, key)) == expect
    assert tuple(int(x) for x in oracle.philox4x32_10(np.array(ctr), key)[0]) == expect


def test_philox_stream_c_matches_numpy(oracle):
    for dim, seed in ((1, 1), (5, 77), (12, 4_000_000_000)):
        assert np.array_equal(oracle.c_philox_words(oracle.DEFAULT_BASE_SEED, dim, seed, 64),
                              oracle.philox_words(oracle.DEFAULT_BASE_SEED, dim, seed, 64))


def test_normals_c_matches_numpy_and_are_normal(oracle):
    z = oracle.c_normals(oracle.DEFAULT_BASE_SEED, 12, 3, 4000)
    assert np.max(np.abs(z - oracle.normals(oracle.DEFAULT_BASE_SEED, 12, 3, 4000))) < 1e-12
    # brownian_motion_test.rs:47-96 style check: empirical CDF at standard-normal quantiles
    from scipy.stats import norm

    zs = np.sort(z.ravel())
    for p in (0.01, 0.05, 0.25, 0.5, 0.75, 0.95, 0.99):
        assert abs(np.searchsorted(zs, norm.ppf(p)) / zs.size - p) < 0.01


def test_stream_depends_on_dim_not_model(oracle):
    a = oracle.philox_words(oracle.DEFAULT_BASE_SEED, 3, 9, 4)
    b = oracle.philox_words(oracle.DEFAULT_BASE_SEED, 4, 9, 4)
    assert not np.array_equal(a, b)


def test_cumsum_rowwise_known_answer(oracle):
    ka = KA["cumsum_rowwise"]
    m = np.array(ka["input_rows"])
    assert np.array_equal(oracle.c_cumsum_rowwise(m), np.array(ka["expected_rows"]))
    assert np.array_equal(oracle.cumsum_rowwise(m), np.array(ka["expected_rows"]))


@pytest.mark.parametrize("case", KA["sum_of_outer_products"], ids=lambda c: c["source"].split(":")[-1])
def test_sum_of_outer_products_known_answers(oracle, case):
    a = np.array(case["a_cols"], dtype=np.float64).T
    b = np.array(case["b_cols"], dtype=np.float64).T
    exp = np.array(case["expected_rows"], dtype=np.float64)
    assert np.max(np.abs(oracle.c_sum_of_outer_products(a, b) - exp)) <= case["tol"]
    assert np.max(np.abs(oracle.sum_of_outer_products(a, b) - exp)) <= case["tol"]


def test_sum_of_outer_products_large(oracle):
    # sum_of_outer_products_test.rs:113-138: a(i,j) = i+j, b(i,j) = i*j+1 (5 x 10)
    i, j = np.meshgrid(np.arange(5), np.arange(10), indexing="ij")
    a, b = (i + j).astype(float), (i * j + 1).astype(float)
    assert np.array_equal(oracle.c_sum_of_outer_products(a, b), a @ b.T)


def test_c_oracle_matches_dggev_twin(oracle):
    """C restatement (Cholesky + Jacobi) vs the numpy/scipy twin (dggev) on random paths."""
    rng = np.random.default_rng(7)
    for model in range(5):
        for dim in (1, 2, 3, 6, 12):
            for steps in (40, 500):
                dB = rng.standard_normal((2, steps, dim)) / np.sqrt(steps)
                c = oracle.c_eigs_from_increments(model, dB)
                p = np.stack([oracle.eigs_dense(model, dB[r].T) for r in range(2)])
                assert normwise_err(c, p) < 1e-10, (model, dim, steps)


def test_oracle_reproduces_golden_fixture(oracle, golden):
    cases, eigs = golden
    for (model, dim, steps), ref in eigs.items():
        dB = cases[(dim, steps)]
        assert normwise_err(oracle.c_eigs_from_increments(model, dB), ref) < 1e-10, (model, dim, steps)


def test_golden_fixture_is_the_dggev_twin(oracle, golden):
    cases, eigs = golden
    for (model, dim, steps), ref in list(eigs.items())[::7]:
        dB = cases[(dim, steps)]
        got = np.stack([oracle.eigs_dense(model, dB[r].T) for r in range(dB.shape[0])])
        assert normwise_err(got, ref) < 1e-12


def test_golden_fixture_covers_the_benchmarked_shape(golden):
    cases, eigs = golden
    assert cases[(12, 10_000)].shape == (4, 10_000, 12)
    assert all((m, 12, 10_000) in eigs for m in range(5))


def test_threaded_increments_entry_agrees(oracle):
    dB = np.random.default_rng(11).standard_normal((9, 257, 5)) / np.sqrt(257)
    for model in (0, 3):
        assert np.array_equal(oracle.c_eigs_from_increments(model, dB),
                              oracle.c_eigs_from_increments(model, dB, n_threads=4))


def test_independent_stream_is_standard_normal_and_untruncated(oracle):
    """xoshiro256++ + Box-Muller on 53-bit uniforms: moments, a KS test, the 4-sigma tail mass
    (6.33e-5), independence across run seeds, and the same draws in the seeded batch."""
    from scipy.stats import kstest, norm

    z = oracle.c_xoshiro_normals(oracle.DEFAULT_BASE_SEED, 5, 2_000_000)
    assert abs(z.mean()) < 5 * np.sqrt(1 / z.size) and abs(z.var() - 1) < 5 * np.sqrt(2 / z.size)
    assert kstest(z, "norm").pvalue > 1e-3
    tail = np.mean(np.abs(z) > 4.0)
    p4 = 2 * norm.sf(4.0)
    assert abs(tail - p4) < 5 * np.sqrt(p4 / z.size)
    other = oracle.c_xoshiro_normals(oracle.DEFAULT_BASE_SEED, 6, 100_000)
    assert abs(np.corrcoef(z[:100_000], other)[0, 1]) < 0.02
    assert not np.array_equal(z[:10], oracle.c_xoshiro_normals(oracle.DEFAULT_BASE_SEED + 1, 5, 10))
    # the seeded batch walks exactly these draws (time-major, scaled by sqrt(dt))
    zz = oracle.c_xoshiro_normals(oracle.DEFAULT_BASE_SEED, 3, 3 * 200).reshape(200, 3) / np.sqrt(200)
    one = oracle.c_eigs_seeded_xoshiro(4, 3, 200, 3, 1)[0]
    assert normwise_err(oracle.eigs_dense(4, zz.T), one) < 1e-10
    many = oracle.c_eigs_seeded_xoshiro(4, 3, 200, 1, 7, n_threads=3)
    assert np.array_equal(many[2], one)


def test_eigen_counts(oracle):
    # basic_api.rs:35 (dim for model 0), thread_manager.rs:40-44 (dim+1 for models 1 and 3)
    assert [oracle.eigen_count(m, 2) for m in range(5)] == [2, 3, 2, 3, 2]


def test_structural_zero_eigenvalue_models_1_3(oracle):
    rng = np.random.default_rng(3)
    dB = rng.standard_normal((1, 300, 4)) / np.sqrt(300)
    for model in (1, 3):
        lam = oracle.c_eigs_from_increments(model, dB)[0]
        assert lam[-1] < 1e-10 * lam[0]


def test_seeded_batch_threads_agree(oracle):
    one = oracle.c_eigs_seeded(2, 3, 300, 1, 12, n_threads=1)
    many = oracle.c_eigs_seeded(2, 3, 300, 1, 12, n_threads=5)
    assert np.array_equal(one, many)
    # and equals the dense path on the same normals
    z = oracle.c_normals(oracle.DEFAULT_BASE_SEED, 3, 5, 300) / np.sqrt(300)
    assert normwise_err(oracle.eigs_dense(2, z.T), one[4]) < 1e-10


# ---- storage format and analysis rules (restated in the oracle) ----
def test_uleb128_known_answers(oracle):
    for v, enc in KA["uleb128_encode"]["cases"]:
        assert list(oracle.uleb128_encode(v)) == enc
        assert oracle.uleb128_decode(bytes(enc)) == (v, len(enc))
    for v, n in KA["uleb128_encoded_size"]["cases"]:
        assert len(oracle.uleb128_encode(v)) == n
    for v in KA["uleb128_roundtrip"]["values"]:
        assert oracle.uleb128_decode(oracle.uleb128_encode(v))[0] == v
    for buf, _ in KA["uleb128_decode_errors"]["cases"]:
        with pytest.raises(ValueError):
            oracle.uleb128_decode(bytes(buf))


def test_dat_format_known_answers(oracle):
    h = KA["dat_header"]
    assert oracle.dat_bytes(h["model"], h["dim"], h["steps"], [], finished=False) == bytes.fromhex(h["hex"])
    for seed, eig, hx in KA["dat_records"]["cases"]:
        body = oracle.dat_bytes(0, 1, 10, [(seed, eig)], finished=False)[18:]
        assert body == bytes.fromhex(hx)
    e = KA["dat_eof"]
    full = oracle.dat_bytes(0, 1, 10, [(s, [0.5]) for s in range(1, 3)])
    assert full[-17:-9] == bytes.fromhex(e["hex"])[:8]
    import struct

    assert bytes.fromhex(e["hex"])[8:16] == struct.pack("<Q", e["count"])
    r = KA["append_writer_roundtrip"]
    buf = oracle.dat_bytes(r["model"], r["dim"], r["steps"], r["records"])
    recs, model, dim, steps = oracle.dat_parse(buf)
    assert (model, dim, steps) == (r["model"], r["dim"], r["steps"])
    assert [(s, e) for s, e in recs] == [tuple(x) for x in r["records"]]
    # no EOF trailer -> scan read (append_writer_test.rs:66-93)
    recs2, *_ = oracle.dat_parse(oracle.dat_bytes(2, 2, 150, r["records"], finished=False))
    assert [(s, e) for s, e in recs2] == [tuple(x) for x in r["records"]]


def test_percentile_rule(oracle):
    pr = KA["percentile_rule"]
    for p, v in pr["cases"]:
        assert abs(oracle.percentile_value(sorted(pr["values"]), p) - v) < 1e-12
    assert np.isnan(oracle.percentile_value([], 0.5))
