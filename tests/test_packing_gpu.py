"""Two-run packing of the mixed kernels for dims up to 4: odd run counts (the
last unit holds one run), explicit increments, ragged batches mixing packed
and unpacked requests, and agreement with the FP64 kernel."""
import numpy as np
import pytest

from conftest import normwise_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("n", [1, 2, 7, 64, 333])
def test_packed_runs_match_fp64(engine, jne, dim, n):
    for model in (0, 3, 4):
        mixed = engine.eigs_seeded(model, dim, 1500, 11, n, precision=jne.PREC_MIXED)
        fp64 = engine.eigs_seeded(model, dim, 1500, 11, n, precision=jne.PREC_FP64)
        assert mixed.shape == fp64.shape == (n, jne.eigen_count(model, dim))
        assert normwise_err(mixed, fp64, 1.0) < 2e-6, (model, dim, n)


def test_a_run_does_not_depend_on_its_partner(engine, jne):
    # run 8 is paired with run 7 (n = 9) or alone (seed_first = 8, n = 1)
    full = engine.eigs_seeded(2, 3, 2000, 1, 9, precision=jne.PREC_MIXED)
    alone = engine.eigs_seeded(2, 3, 2000, 9, 1, precision=jne.PREC_MIXED)
    shifted = engine.eigs_seeded(2, 3, 2000, 2, 8, precision=jne.PREC_MIXED)  # pairs (2,3), (4,5), ...
    assert np.array_equal(full[8], alone[0])
    assert np.array_equal(full[1:], shifted)


def test_packed_explicit_increments(engine, oracle, jne):
    dB, _ = engine.export_increments(2, 700, 1, 5)
    for model in range(5):
        ref = oracle.c_eigs_from_increments(model, dB)
        got = engine.eigs_from_increments(model, dB, precision=jne.PREC_MIXED)
        assert normwise_err(got, ref, 1.0) < 4e-6, model


def test_ragged_mix_of_packed_and_unpacked(engine, jne):
    import torch

    reqs = [dict(model=1, dim=2, steps=900, n_runs=77), dict(model=4, dim=9, steps=600, n_runs=31),
            dict(model=0, dim=4, steps=2500, n_runs=1), dict(model=3, dim=1, steps=400, n_runs=100),
            dict(model=2, dim=6, steps=800, n_runs=45)]
    outs = [torch.empty((r["n_runs"], jne.eigen_count(r["model"], r["dim"])), dtype=torch.float64, device="cuda")
            for r in reqs]
    engine.run_batch(reqs, [o.data_ptr() for o in outs])
    engine.sync()
    for r, o in zip(reqs, outs):
        single = engine.eigs_seeded(r["model"], r["dim"], r["steps"], 1, r["n_runs"], precision=jne.PREC_MIXED)
        assert np.array_equal(o.cpu().numpy(), single), r
