"""The mixed kernel's launch shapes and their autotuner: every shape (blocks
per SM, one or two runs per warp) gives the same bits; the tuner keeps the
fastest measured shape whose chunk meets the error bound on its sample; the
tuned mode reproduces the fixed-chunk results exactly, and the ragged path uses
the tuned chunk lengths too."""
import numpy as np
import pytest

from conftest import normwise_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,steps", [(2, 700), (3, 1300), (7, 900), (12, 2000)])
def test_every_launch_shape_gives_the_same_bits(jne, dim, steps):
    with jne.Engine(0) as eng:
        ref = eng.eigs_seeded(4, dim, steps, 1, 257, precision=jne.PREC_MIXED)
        for bps in (4, 6):
            for pack in (1, 0):
                eng.set_launch_shape(bps, pack)
                got = eng.eigs_seeded(4, dim, steps, 1, 257, precision=jne.PREC_MIXED)
                assert np.array_equal(got, ref), (bps, pack)


def test_tuner_keeps_the_fastest_shape_within_the_bound(jne):
    with jne.Engine(0) as eng:
        best, table = eng.autotune(6, 3000, max_rel_err=5e-7, sample_runs=256, time_runs=65536)
        timed = [t for t in table if t["ms"] >= 0]
        assert timed and all(t["max_rel_err"] <= 5e-7 or t["chunk"] == 32 for t in timed)
        assert all(t["max_rel_err"] > 5e-7 for t in table if t["ms"] < 0)
        assert best["ms"] == min(t["ms"] for t in timed)
        assert {(t["blocks_per_sm"], t["pack"]) for t in timed} == {(4, 1), (6, 1)}  # dim 6: never packed
        loose, table = eng.autotune(3, 3000, max_rel_err=1e-3, sample_runs=256, time_runs=65536)
        # 2048 steps (the class's lower edge) allow chunks up to 1024, all within 1e-3; dim 3 also times
        # the unpacked shapes
        assert sorted({t["chunk"] for t in table if t["ms"] >= 0}) == [32, 64, 128, 256, 512, 1024]
        assert {(t["blocks_per_sm"], t["pack"]) for t in table} == {(4, 1), (4, 0), (6, 1), (6, 0)}
        assert loose["max_rel_err"] <= 1e-3


def test_tuned_mode_equals_the_fixed_chunk(jne):
    with jne.Engine(0) as eng:
        chunk, err = eng.autotune_chunk(12, 5000, max_rel_err=8e-7, sample_runs=256)
        eng.set_chunk(jne.CHUNK_TUNED)
        tuned = eng.eigs_seeded(4, 12, 6000, 1, 300, precision=jne.PREC_MIXED)    # same class: [4096, 8192)
        other = eng.eigs_seeded(4, 12, 9000, 1, 300, precision=jne.PREC_MIXED)    # untuned class: default rule
        eng.set_chunk(chunk)
        fixed = eng.eigs_seeded(4, 12, 6000, 1, 300, precision=jne.PREC_MIXED)
        eng.set_chunk(0)
        default = eng.eigs_seeded(4, 12, 9000, 1, 300, precision=jne.PREC_MIXED)
        ref = eng.eigs_seeded(4, 12, 6000, 1, 300, precision=jne.PREC_FP64)
    assert np.array_equal(tuned, fixed)
    assert np.array_equal(other, default)
    assert normwise_err(tuned, ref, 1.0) < 2e-6


def test_ragged_batch_uses_tuned_chunks(jne):
    import torch

    reqs = [dict(model=m, dim=d, steps=t, n_runs=200) for m, d, t in ((0, 12, 3000), (3, 5, 1200), (4, 2, 700))]
    with jne.Engine(0) as eng:
        chunks = [eng.autotune_chunk(r["dim"], r["steps"], max_rel_err=1e-6, sample_runs=128)[0] for r in reqs]
        eng.set_chunk(jne.CHUNK_TUNED)
        outs = [torch.empty((r["n_runs"], jne.eigen_count(r["model"], r["dim"])), dtype=torch.float64,
                            device="cuda") for r in reqs]
        eng.run_batch(reqs, [o.data_ptr() for o in outs])
        eng.sync()
        for r, ch, o in zip(reqs, chunks, outs):
            eng.set_chunk(ch)
            single = eng.eigs_seeded(r["model"], r["dim"], r["steps"], 1, r["n_runs"], precision=jne.PREC_MIXED)
            assert np.array_equal(o.cpu().numpy(), single), (r, ch)


def test_tuner_arguments(jne):
    with jne.Engine(0) as eng:
        for args in ((12, 200, 5e-7, 64), (13, 5000, 5e-7, 64), (4, 5000, 0.0, 64), (4, 5000, 5e-7, 0)):
            with pytest.raises(jne.JneError) as ei:
                eng.autotune_chunk(*args)
            assert ei.value.code == jne.JNE_ERR_ARG
        for shape in ((5, 1), (4, 2), (8, 0)):
            with pytest.raises(jne.JneError) as ei:
                eng.set_launch_shape(*shape)
            assert ei.value.code == jne.JNE_ERR_ARG
