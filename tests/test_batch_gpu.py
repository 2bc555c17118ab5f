"""Ragged batches (one persistent launch over mixed requests) and plans (a batch
captured into a CUDA graph and replayed): each request's result must equal the
single-request path, and be the same alone and in any mix."""
import numpy as np
import pytest

from conftest import normwise_err

pytestmark = pytest.mark.gpu


def _outs(jne, reqs):
    import torch

    return [torch.full((r["n_runs"], jne.eigen_count(r["model"], r["dim"])), float("nan"), dtype=torch.float64,
                       device="cuda") for r in reqs]


MIX = [
    dict(model=0, dim=12, steps=1000, n_runs=300),
    dict(model=4, dim=3, steps=2500, n_runs=57, seed_first=1000),
    dict(model=1, dim=1, steps=300, n_runs=1000),
    dict(model=3, dim=7, steps=777, n_runs=130, base_seed=99),
    dict(model=2, dim=12, steps=4096, n_runs=64, seed_first=5),
    dict(model=2, dim=5, steps=100, n_runs=40),                    # short path: FP64 kernel
    dict(model=4, dim=9, steps=600, n_runs=33, precision=0),       # FP64 request
    dict(model=0, dim=2, steps=500, n_runs=0),                     # empty
]


def _single(engine, jne, r):
    return engine.eigs_seeded(r["model"], r["dim"], r["steps"], r.get("seed_first", 1), r["n_runs"],
                              precision=r.get("precision", jne.PREC_MIXED),
                              base_seed=r.get("base_seed", jne.DEFAULT_BASE_SEED))


def test_ragged_batch_matches_single_requests(engine, jne):
    outs = _outs(jne, MIX)
    engine.run_batch(MIX, [o.data_ptr() for o in outs])
    engine.sync()
    for r, o in zip(MIX, outs):
        ref = _single(engine, jne, r)
        got = o.cpu().numpy()
        assert got.shape == ref.shape
        if r["n_runs"]:
            assert normwise_err(got, ref, 1.0) < 1e-12, r


def test_result_same_alone_and_in_the_mix(engine, jne):
    alone = _outs(jne, MIX[:1])
    engine.run_batch(MIX[:1], [alone[0].data_ptr()])
    mixed = _outs(jne, MIX)
    engine.run_batch(MIX[::-1], [o.data_ptr() for o in mixed[::-1]])  # other order, other neighbours
    engine.sync()
    assert np.array_equal(alone[0].cpu().numpy(), mixed[0].cpu().numpy())


def test_batches_split_across_launches_under_a_small_budget(jne):
    reqs = [dict(model=m, dim=12, steps=512, n_runs=3000) for m in range(5)]
    with jne.Engine(0, mem_budget_bytes=64 << 20) as small, jne.Engine(0) as big:
        a, b = _outs(jne, reqs), _outs(jne, reqs)
        small.run_batch(reqs, [o.data_ptr() for o in a])  # ~7 MB of records per request: several launches
        big.run_batch(reqs, [o.data_ptr() for o in b])
        small.sync()
        big.sync()
        for x, y in zip(a, b):
            assert np.array_equal(x.cpu().numpy(), y.cpu().numpy())


def test_plan_replays_the_batch(engine, jne):
    reqs = [r for r in MIX[:5]]
    ref = _outs(jne, reqs)
    engine.run_batch(reqs, [o.data_ptr() for o in ref])
    engine.sync()
    outs = _outs(jne, reqs)
    plan = engine.plan(reqs, [o.data_ptr() for o in outs])
    for _ in range(3):
        plan.launch()
        engine.sync()
        for x, y in zip(outs, ref):
            assert np.array_equal(x.cpu().numpy(), y.cpu().numpy())
        for o in outs:
            o.fill_(float("nan"))
    plan.destroy()


def test_plan_rejects_fp64_requests(engine, jne):
    reqs = [dict(model=0, dim=2, steps=1000, n_runs=10, precision=0)]
    with pytest.raises(jne.JneError) as ei:
        engine.plan(reqs, [o.data_ptr() for o in _outs(jne, reqs)])
    assert ei.value.code == jne.JNE_ERR_ARG


def test_ragged_mixed_requests_equal_single_requests_bit_for_bit(engine, jne):
    # the ragged kernel (every dim in one launch) and the single-request kernel
    # compile the merge differently; the arithmetic per value is the same
    reqs = [dict(model=m, dim=d, steps=t, n_runs=n, seed_first=s)
            for m, d, t, n, s in ((0, 12, 1000, 96, 1), (4, 3, 2500, 33, 7), (1, 1, 300, 70, 3),
                                  (3, 7, 777, 40, 11), (2, 12, 4096, 20, 5), (4, 4, 640, 65, 2))]
    outs = _outs(jne, reqs)
    engine.run_batch(reqs, [o.data_ptr() for o in outs])
    engine.sync()
    for r, o in zip(reqs, outs):
        assert np.array_equal(o.cpu().numpy(), _single(engine, jne, r)), r


def test_singular_request_fails_alone(engine, jne):
    """A request whose S11 is singular (steps = 1: F = B_0 = 0) in a batch with healthy ragged and FP64
    requests: it alone reports JNE_ERR_NUMERIC (NaN rows); the others are JNE_OK and equal their
    single-request results bit for bit."""
    reqs = [MIX[0], dict(model=0, dim=3, steps=1, n_runs=5), MIX[1], MIX[6], MIX[2]]
    outs = _outs(jne, reqs)
    codes = engine.run_batch_status(reqs, [o.data_ptr() for o in outs])
    assert codes == [jne.JNE_OK, jne.JNE_ERR_NUMERIC, jne.JNE_OK, jne.JNE_OK, jne.JNE_OK]
    assert bool(outs[1].isnan().all())
    for r, o, c in zip(reqs, outs, codes):
        if c == jne.JNE_OK:
            assert np.array_equal(o.cpu().numpy(), _single(engine, jne, r)), r
    # the context's own status word is untouched: a plain sync reports nothing
    engine.sync()
    assert engine.run_batch_status(reqs[:1], [outs[0].data_ptr()]) == [jne.JNE_OK]


def test_results_visible_on_the_caller_stream_without_sync(engine, jne):
    """FP64-path requests finalize on the context's second stream, ragged ones on its first: work the
    caller enqueues on its own stream after jne_run_batch sees both, with no jne_sync in between."""
    import torch

    reqs = [MIX[6], MIX[5], MIX[0], MIX[3]]
    refs = [_single(engine, jne, r) for r in reqs]
    st = torch.cuda.Stream()
    for _ in range(3):
        outs = _outs(jne, reqs)
        engine.run_batch(reqs, [o.data_ptr() for o in outs], stream=st.cuda_stream)
        with torch.cuda.stream(st):
            copies = [o.clone() for o in outs]  # ordered after the batch on the caller's stream
        st.synchronize()
        for c, ref in zip(copies, refs):
            assert np.array_equal(c.cpu().numpy(), ref)
    engine.sync()


def _collect_sink(eng, jne, reqs):
    got = {i: [] for i in range(len(reqs))}
    seeds = {i: [] for i in range(len(reqs))}
    status = {i: [] for i in range(len(reqs))}

    def write(req, seed_first, eigs, st):
        got[req].append(eigs)
        seeds[req].append((seed_first, eigs.shape[0]))
        status[req].append(st)
        return 0

    return got, seeds, status, write


def test_sink_streams_each_request_in_seed_order(jne):
    """Under a small budget every request spans several rounds: each request's results arrive in seed order,
    contiguous, and equal its single-request results bit for bit (ragged, FP64 and short requests)."""
    reqs = [dict(model=0, dim=2, steps=500, n_runs=50_000), MIX[1], MIX[5], MIX[6], MIX[7],
            dict(model=3, dim=12, steps=1000, n_runs=30_000, seed_first=4)]
    with jne.Engine(0, mem_budget_bytes=64 << 20) as small, jne.Engine(0) as ref_eng:
        got, seeds, status, write = _collect_sink(small, jne, reqs)
        small.run_batch_sink(reqs, write)
        assert len(seeds[0]) > 1 and len(seeds[5]) > 1  # several rounds
        for i, r in enumerate(reqs):
            s0 = r.get("seed_first", 1)
            pos = s0
            for first, n in seeds[i]:
                assert first == pos
                pos += n
            assert pos == s0 + r["n_runs"]
            assert all(st == jne.JNE_OK for st in status[i])
            res = np.concatenate(got[i]) if got[i] else np.empty((0, jne.eigen_count(r["model"], r["dim"])))
            assert np.array_equal(res, _single(ref_eng, jne, r)), r


def test_sink_reports_a_singular_request_and_can_stop_the_batch(engine, jne):
    reqs = [MIX[0], dict(model=0, dim=3, steps=1, n_runs=5), MIX[2]]
    got, seeds, status, write = _collect_sink(engine, jne, reqs)
    with pytest.raises(jne.JneError) as ei:
        engine.run_batch_sink(reqs, write)
    assert ei.value.code == jne.JNE_ERR_NUMERIC  # after every result was delivered
    assert status[1] == [jne.JNE_ERR_NUMERIC] and np.isnan(got[1][0]).all()
    assert status[0] == [jne.JNE_OK] and status[2] == [jne.JNE_OK]
    assert np.array_equal(got[0][0], _single(engine, jne, reqs[0]))
    calls = []

    def stop(req, seed_first, eigs, st):
        calls.append(req)
        return 7  # any non-zero status stops the batch

    with pytest.raises(jne.JneError) as ei:
        engine.run_batch_sink([MIX[0], MIX[2]], stop)
    assert ei.value.code == 7 and calls == [0]
    engine.sync()


def test_dat_sink_writes_the_simulation_files(engine, jne, tmp_path):
    """jne_dat_sink: every request's records appended to its simulation file (the reference's name); two
    requests of the same (model, dim, steps) share a file; the trailer is written at close."""
    reqs = [dict(model=1, dim=3, steps=400, n_runs=700), dict(model=4, dim=9, steps=600, n_runs=90, precision=0),
            dict(model=1, dim=3, steps=400, n_runs=300, seed_first=701)]
    engine.run_batch_to_dat(reqs, str(tmp_path))
    recs, model, dim, steps = jne.read_dat(str(tmp_path / "eigenvalues_model1_dim3_steps400.dat"))
    assert (model, dim, steps) == (1, 3, 400)
    assert list(recs.seeds) == list(range(1, 1001))
    whole = engine.eigs_seeded(1, 3, 400, 1, 1000, precision=jne.PREC_MIXED)
    assert np.array_equal(recs.eigs, whole)
    recs, model, dim, steps = jne.read_dat(str(tmp_path / "eigenvalues_model4_dim9_steps600.dat"))
    assert list(recs.seeds) == list(range(1, 91))
    assert np.array_equal(recs.eigs, engine.eigs_seeded(4, 9, 600, 1, 90, precision=0))
    raw = open(tmp_path / "eigenvalues_model4_dim9_steps600.dat", "rb").read()
    assert raw[-17:-9] == b"EOF_MARK"
