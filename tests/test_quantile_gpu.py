"""The device quantile analyzer (radix select on the GPU) against the host
percentile rule of simulation_analyzers.rs:4-81: bit-identical results on ties,
negative values, tiny and large inputs, and on eigenvalues the engine produced."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PS = [0.01, 0.05, 0.1, 0.5, 0.9, 0.95, 0.99, 0.0, 1.0]


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _both(jne, engine, torch, eigs, stat, ps=PS):
    t = _dev(torch, eigs)
    torch.cuda.synchronize()
    got = engine.percentiles_device(t.data_ptr(), eigs.shape[0], eigs.shape[1], stat, ps)
    ref = jne.percentiles(eigs, stat, ps)
    return got, ref


@pytest.mark.parametrize("n", [1, 2, 3, 17, 1000, 65_537])
@pytest.mark.parametrize("stat", ["trace", "maxeig"])
def test_matches_host_rule(jne, engine, n, stat):
    import torch

    rng = np.random.default_rng(n)
    eigs = np.sort(rng.gamma(2.0, 3.0, size=(n, 5)), axis=1)[:, ::-1]
    got, ref = _both(jne, engine, torch, eigs, stat)
    assert got == ref


def test_ties_negative_values_and_signed_zero(jne, engine):
    import torch

    rng = np.random.default_rng(7)
    vals = rng.choice([-3.5, -1.0, -0.0, 0.0, 0.25, 2.0, 1e300, -1e-300], size=(4099, 1))
    for stat in ("trace", "maxeig"):
        got, ref = _both(jne, engine, torch, vals, stat, ps=[i / 20 for i in range(21)])
        assert got == ref


def test_many_percentiles_span_several_rank_groups(jne, engine):
    import torch

    rng = np.random.default_rng(11)
    eigs = rng.standard_normal((20_000, 3))
    ps = list(np.linspace(0.0, 1.0, 37))
    got, ref = _both(jne, engine, torch, eigs, "trace", ps)
    assert got == ref


def test_on_engine_output_large(jne, engine):
    import torch

    n, dim = 1_000_000, 4
    out = torch.empty((n, dim), dtype=torch.float64, device="cuda")
    engine.eigs_seeded_device(0, dim, 1000, 1, n, out.data_ptr(), precision=jne.PREC_MIXED)
    engine.sync()
    host = out.cpu().numpy()
    for stat in ("trace", "maxeig"):
        got = engine.percentiles_device(out.data_ptr(), n, dim, stat, PS)
        assert got == jne.percentiles(host, stat, PS)


def test_errors(jne, engine):
    import torch

    t = _dev(torch, np.array([[1.0, np.nan], [2.0, 3.0]]))
    with pytest.raises(jne.JneError) as ei:
        engine.percentiles_device(t.data_ptr(), 2, 2, "trace", [0.5])
    assert ei.value.code == jne.JNE_ERR_NUMERIC
    with pytest.raises(jne.JneError) as ei:
        engine.percentiles_device(t.data_ptr(), 2, 2, "trace", [1.01])
    assert ei.value.code == jne.JNE_ERR_ARG
    assert np.isnan(engine.percentiles_device(0, 0, 2, "trace", [0.5])[0])
