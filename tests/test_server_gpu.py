"""The continuous-batching request loop: requests submitted while others run are
admitted at the next iteration, each result equals the request computed alone,
results stream to EIGENVALS_V6 files, and admission respects the budget."""
import os
import time

import numpy as np
import pytest

from conftest import normwise_err

pytestmark = pytest.mark.gpu

MIX = [
    dict(model=4, dim=12, steps=3000, n_runs=2000),
    dict(model=0, dim=2, steps=800, n_runs=5000, seed_first=77),
    dict(model=3, dim=5, steps=1500, n_runs=300, base_seed=5),
    dict(model=1, dim=9, steps=400, n_runs=1200),
    dict(model=2, dim=3, steps=150, n_runs=700),                    # short path: FP64 kernel
    dict(model=4, dim=6, steps=1000, n_runs=250, precision=0),      # FP64 request
    dict(model=0, dim=4, steps=600, n_runs=0),                      # nothing to do
]


def _collect(srv, n, limit_s=120.0):
    done, t0 = {}, time.monotonic()
    while len(done) < n:
        assert time.monotonic() - t0 < limit_s, f"only {len(done)} of {n} requests finished"
        for c in srv.wait(timeout_ms=5_000):
            done[c.id] = c
    return done


def test_results_same_alone_and_in_the_mix(jne):
    with jne.Engine(0) as ref_eng, jne.Engine(0) as eng:
        with jne.Server(eng, iter_work=50_000_000) as srv:
            alone_id = srv.submit(**MIX[0])
            _collect(srv, 1)
            alone = srv.fetch(alone_id)
            ids = []
            for r in MIX:  # staggered: later requests arrive while earlier ones run
                ids.append(srv.submit(**r))
                time.sleep(0.002)
            done = _collect(srv, len(MIX))
            res = {i: srv.fetch(i) for i in ids}
        assert all(done[i].status == jne.JNE_OK for i in ids)
        assert all(done[i].submit_s <= done[i].start_s <= done[i].finish_s for i in ids)
        assert np.array_equal(res[ids[0]], alone)
        for i, r in zip(ids, MIX):
            ref = ref_eng.eigs_seeded(r["model"], r["dim"], r["steps"], r.get("seed_first", 1), r["n_runs"],
                                      precision=r.get("precision", jne.PREC_MIXED),
                                      base_seed=r.get("base_seed", jne.DEFAULT_BASE_SEED))
            assert res[i].shape == ref.shape
            if r["n_runs"]:
                assert normwise_err(res[i], ref, 1.0) < 1e-12, r


def test_results_stream_to_dat_files(jne, tmp_path):
    with jne.Engine(0) as eng:
        with jne.Server(eng, data_dir=str(tmp_path)) as srv:
            rid = srv.submit(model=1, dim=3, steps=500, n_runs=321, seed_first=10)
            _collect(srv, 1)
            for _ in range(200):  # the writer thread may still be writing
                try:
                    res = srv.fetch(rid)
                    break
                except jne.JneError:
                    time.sleep(0.01)
    recs, model, dim, steps = jne.read_dat(os.path.join(str(tmp_path), f"request{rid}_model1_dim3_steps500.dat"))
    assert (model, dim, steps) == (1, 3, 500)
    assert list(recs.seeds) == list(range(10, 331))
    assert np.array_equal(recs.eigs, res)


def test_admission_respects_the_budget(jne):
    with jne.Engine(0, mem_budget_bytes=64 << 20) as eng:
        with jne.Server(eng) as srv:
            big = srv.submit(model=0, dim=12, steps=300, n_runs=1_000_000)  # 96 MB of outputs
            ok = srv.submit(model=0, dim=2, steps=300, n_runs=100)
            done = _collect(srv, 2)
            assert done[big].status == jne.JNE_ERR_BUDGET
            assert done[ok].status == jne.JNE_OK
            assert srv.fetch(ok).shape == (100, 2)


def test_singular_request_fails_alone_in_the_mix(jne):
    """A singular request (steps = 1: S11 = 0) among healthy ones: only it reports JNE_ERR_NUMERIC, and
    the others equal their results alone (each iteration's requests report to their own status words)."""
    healthy = [MIX[0], MIX[1], MIX[5]]
    with jne.Engine(0) as ref_eng, jne.Engine(0) as eng:
        with jne.Server(eng, iter_work=50_000_000) as srv:
            ids = [srv.submit(**healthy[0]), srv.submit(model=0, dim=4, steps=1, n_runs=64),
                   srv.submit(**healthy[1]), srv.submit(**healthy[2])]
            done = _collect(srv, len(ids))
            assert done[ids[1]].status == jne.JNE_ERR_NUMERIC
            with pytest.raises(jne.JneError) as ei:
                srv.fetch(ids[1])
            assert ei.value.code == jne.JNE_ERR_NUMERIC
            for i, r in zip([ids[0], ids[2], ids[3]], healthy):
                assert done[i].status == jne.JNE_OK
                ref = ref_eng.eigs_seeded(r["model"], r["dim"], r["steps"], r.get("seed_first", 1), r["n_runs"],
                                          precision=r.get("precision", jne.PREC_MIXED),
                                          base_seed=r.get("base_seed", jne.DEFAULT_BASE_SEED))
                assert np.array_equal(srv.fetch(i), ref), r
