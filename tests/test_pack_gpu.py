"""The device-side record packer (jne_pack_records_device) and the .dat sink that uses it: the packed bytes
equal the host encoder's (jne_dat_append) and the format restatement's, byte for byte, across every ULEB128
length of the seed and up to the last u32 seed; nothing past the records is written; the .dat files of a
streamed batch are the same whether its records are packed on the GPU or encoded on the host."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_records(jne, tmp_path, seed_first, eigs):
    """The records jne_dat_append writes for seeds seed_first.. (the file minus its 18-byte header)."""
    path = str(tmp_path / f"host_{seed_first}_{eigs.shape[0]}_{eigs.shape[1]}.dat")
    if os.path.exists(path):
        os.remove(path)
    w = jne.DatWriter(path, 0, 2, 100)
    w.append(np.arange(seed_first, seed_first + eigs.shape[0], dtype=np.uint64).astype(np.uint32), eigs)
    w.abandon()
    return open(path, "rb").read()[18:]


def _device_records(jne, engine, seed_first, eigs, pad=64):
    """The records packed on the GPU into a buffer `pad` bytes longer than needed (filled with 0xAB first),
    and that tail, which must come back untouched."""
    import torch

    n, k = eigs.shape
    nbytes = jne.record_bytes(seed_first, n, k)
    d_eigs = torch.from_numpy(np.ascontiguousarray(eigs)).cuda()
    buf = torch.full((nbytes + pad,), 0xAB, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()  # the inputs are in place before the engine's stream reads them
    assert engine.pack_records_device(seed_first, n, k, d_eigs.data_ptr(), buf.data_ptr(), nbytes + pad) == nbytes
    engine.sync()
    out = buf.cpu().numpy().tobytes()
    return out[:nbytes], out[nbytes:]


@pytest.mark.parametrize("seed_first,n", [(1, 20_000), (100, 300), (16_000, 1000), (2**21 - 500, 1000),
                                          (2**28 - 7, 50), (2**32 - 40, 40), (0, 1), (5, 2)])
@pytest.mark.parametrize("k", [1, 2, 12, 13])
def test_packed_bytes_equal_host_encoding(jne, engine, tmp_path, seed_first, n, k):
    rng = np.random.default_rng(seed_first % 1000 + k)
    eigs = rng.standard_normal((n, k)) * 10.0 ** rng.integers(-300, 300, size=(n, k))
    eigs[0, 0] = np.nan if n > 3 else eigs[0, 0]  # any f64 bit pattern is carried as bytes
    got, tail = _device_records(jne, engine, seed_first, eigs)
    assert got == _host_records(jne, tmp_path, seed_first, eigs)
    assert tail == b"\xab" * len(tail)


def test_packed_bytes_equal_format_restatement(jne, engine, oracle):
    eigs = np.array([[1.0, 2.0], [3.0, 4.0], [5.5, -0.25], [7.0, 8.0]])
    for a in (126, 16382, 2**32 - 4):
        got, _ = _device_records(jne, engine, a, eigs)
        want = oracle.dat_bytes(0, 2, 100, [(a + r, list(eigs[r])) for r in range(4)], finished=False)[18:]
        assert got == want, a


def test_one_million_records(jne, engine, tmp_path):
    """A sink round's worth (2^20 records of 13 values, about 114 MB) in one launch."""
    n, k = 1 << 20, 13
    eigs = np.random.default_rng(3).standard_normal((n, k))
    got, _ = _device_records(jne, engine, 1, eigs)
    assert got == _host_records(jne, tmp_path, 1, eigs)


def test_packer_arguments(jne, engine):
    import torch

    eigs = torch.zeros((4, 2), dtype=torch.float64, device="cuda")
    buf = torch.zeros(256, dtype=torch.uint8, device="cuda")
    need = jne.record_bytes(1, 4, 2)
    for args in ((1, 4, 2, eigs.data_ptr(), buf.data_ptr() + 8, 200),   # not 16-byte aligned
                 (1, 4, 2, eigs.data_ptr(), buf.data_ptr(), need - 1),  # too small
                 (1, 4, 256, eigs.data_ptr(), buf.data_ptr(), 256),     # count beyond u8
                 (2**32 - 2, 4, 2, eigs.data_ptr(), buf.data_ptr(), 256),  # seeds past u32
                 (1, 4, 2, 0, buf.data_ptr(), 256)):                    # null input
        with pytest.raises(jne.JneError) as ei:
            engine.pack_records_device(*args)
        assert ei.value.code == jne.JNE_ERR_ARG
    assert engine.pack_records_device(1, 0, 2, 0, 0, 0) == 0  # nothing to pack: no launch


def test_dat_sink_device_packing_equals_host_encoding(jne, engine, tmp_path):
    """jne_run_batch_sink with the .dat sink: the files are byte-identical whether the records are packed on
    the GPU (the sink's default) or encoded on the host, across rounds and seed-length boundaries."""
    reqs = [dict(model=0, dim=12, steps=300, n_runs=5000, seed_first=16_000),
            dict(model=3, dim=2, steps=1000, n_runs=20_000, seed_first=100),
            dict(model=0, dim=12, steps=300, n_runs=700, seed_first=21_000),
            dict(model=2, dim=5, steps=257, n_runs=3, seed_first=2**32 - 3)]
    dev, host = tmp_path / "dev", tmp_path / "host"
    with jne.Engine(0, 128 << 20) as small:  # a 128 MiB budget: rounds of about 40k runs, so two rounds
        small.run_batch_to_dat(reqs, str(dev), device_pack=True)
        small.run_batch_to_dat(reqs, str(host), device_pack=False)
    names = sorted(os.listdir(dev))
    assert names == sorted(os.listdir(host)) and len(names) == 3
    for name in names:
        assert open(dev / name, "rb").read() == open(host / name, "rb").read(), name
    recs, model, dim, steps = jne.read_dat(str(dev / "eigenvalues_model3_dim2_steps1000.dat"))
    assert list(recs.seeds) == list(range(100, 20_100))
    assert np.array_equal(recs.eigs, engine.eigs_seeded(3, 2, 1000, 100, 20_000, precision=jne.PREC_MIXED))
    recs, model, dim, steps = jne.read_dat(str(dev / "eigenvalues_model0_dim12_steps300.dat"))
    assert sorted(recs.seeds) == list(range(16_000, 21_000)) + list(range(21_000, 21_700))
