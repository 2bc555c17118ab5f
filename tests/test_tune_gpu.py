"""The chunk-length autotuner: the chunk it keeps meets the error bound on its
sample, the tuned mode reproduces the fixed-chunk results exactly, and the
ragged path uses the tuned lengths too."""
import numpy as np
import pytest

from conftest import normwise_err

pytestmark = pytest.mark.gpu


def test_tuner_respects_the_bound_and_grows_with_it(jne):
    with jne.Engine(0) as eng:
        tight, e_tight = eng.autotune_chunk(6, 3000, max_rel_err=5e-7, sample_runs=256)
        loose, e_loose = eng.autotune_chunk(6, 3000, max_rel_err=1e-3, sample_runs=256)
    assert tight in (32, 64, 128, 256, 512, 1024) and loose in (32, 64, 128, 256, 512, 1024)
    assert tight == 32 or e_tight <= 5e-7
    assert e_loose <= 1e-3 and loose >= tight
    assert loose == 1024  # 2048 steps (the class's lower edge) allow chunks up to 1024


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
