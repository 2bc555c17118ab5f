"""EIGENVALS_V6 storage and the percentile rule through the C ABI (host code, no
GPU), checked byte for byte against the oracle's restatement of the format and
against the assertions of the reference's append_writer_test.rs."""
import os

import numpy as np
import pytest


@pytest.fixture
def tmp(tmp_path):
    return str(tmp_path)


def test_bytes_match_format_restatement(jne, oracle, tmp):
    path = os.path.join(tmp, "a.dat")
    recs = [(1, [1.0, 2.0]), (300, [3.0, 4.0]), (16384, [5.5, -0.25]), (2**32 - 1, [7.0, 8.0])]
    w = jne.DatWriter(path, 0, 2, 100)
    for s, e in recs:
        w.append_eigenvalues(s, e)
    w.finish()
    assert open(path, "rb").read() == oracle.dat_bytes(0, 2, 100, recs)


def test_roundtrip_basic(jne, tmp):  # append_writer_test.rs:5-31
    path = os.path.join(tmp, "basic.dat")
    w = jne.DatWriter(path, 0, 2, 100)
    w.append_eigenvalues(1, [1.0, 2.0])
    w.append_eigenvalues(2, [3.0, 4.0])
    w.finish()
    recs, model, dim, steps = jne.read_dat(path)
    assert (model, dim, steps) == (0, 2, 100)
    assert [(s, list(e)) for s, e in recs] == [(1, [1.0, 2.0]), (2, [3.0, 4.0])]


def test_incomplete_file_is_scanned(jne, oracle, tmp):  # append_writer_test.rs:66-93
    path = os.path.join(tmp, "inc.dat")
    w = jne.DatWriter(path, 2, 2, 150)
    w.append_eigenvalues(1, [1.0, 2.0])
    w.append_eigenvalues(2, [3.0, 4.0])
    w.abandon()
    recs, *_ = jne.read_dat(path)
    assert [(s, list(e)) for s, e in recs] == [(1, [1.0, 2.0]), (2, [3.0, 4.0])]
    # a record cut in the middle is dropped, as the reference's scan read does
    with open(path, "ab") as f:
        f.write(bytes([3, 2]) + b"\x00" * 11)
    recs, *_ = jne.read_dat(path)
    assert len(recs) == 2


def test_large_dataset_and_resume_append(jne, tmp):  # append_writer_test.rs:95-123
    path = os.path.join(tmp, "large.dat")
    w = jne.DatWriter(path, 3, 2, 500)
    seeds = np.arange(1, 1001)
    w.append(seeds, np.stack([seeds * 0.1, seeds * 0.2], axis=1))
    w.finish()
    recs, *_ = jne.read_dat(path)
    assert len(recs) == 1000 and recs[0][0] == 1 and list(recs[999][1]) == [100.0, 200.0]
    # reopen: the trailer is stripped, records continue, a new trailer counts all
    w = jne.DatWriter(path, 3, 2, 500)
    assert w.existing == 1000
    w.append([1001], np.array([[1.5, 2.5]]))
    w.finish()
    recs, *_ = jne.read_dat(path)
    assert len(recs) == 1001 and recs[1000][0] == 1001
    raw = open(path, "rb").read()
    assert raw[-17:-9] == b"EOF_MARK" and int.from_bytes(raw[-9:-1], "little") == 1001 and raw[-1] == 2


def test_eigenvalue_count_consistency(jne, tmp):  # append_writer_test.rs:125-144
    w = jne.DatWriter(os.path.join(tmp, "c.dat"), 0, 2, 100)
    w.append_eigenvalues(1, [1.0, 2.0])
    with pytest.raises(jne.DatError) as ei:
        w.append_eigenvalues(2, [3.0, 4.0, 5.0])
    assert "Eigenvalue count mismatch" in str(ei.value)
    w.abandon()


def test_eigenvalue_count_limits(jne, tmp):  # append_writer_test.rs:146-197
    w = jne.DatWriter(os.path.join(tmp, "o.dat"), 0, 255, 1000)
    with pytest.raises(jne.DatError) as ei:
        w.append_eigenvalues(1, list(range(300)))
    assert "Too many eigenvalues" in str(ei.value) and "exceeds maximum of 255" in str(ei.value)
    w.abandon()
    path = os.path.join(tmp, "b.dat")
    w = jne.DatWriter(path, 4, 255, 1000)
    w.append_eigenvalues(1, [float(i) for i in range(255)])
    w.finish()
    recs, *_ = jne.read_dat(path)
    assert len(recs) == 1 and len(recs[0][1]) == 255


def test_parameter_validation(jne, tmp):  # append_writer_test.rs:199-227
    path = os.path.join(tmp, "p.dat")
    w = jne.DatWriter(path, 1, 3, 100)
    w.append_eigenvalues(1, [1.0, 2.0, 3.0])
    w.finish()
    for args, text in (((2, 3, 100), "Model mismatch: file has model 1, expected 2"),
                       ((1, 4, 100), "Dimension mismatch: file has dim 3, expected 4"),
                       ((1, 3, 200), "Steps mismatch: file has steps 100, expected 200")):
        with pytest.raises(jne.DatError) as ei:
            jne.DatWriter(path, *args)
        assert text in str(ei.value)
    jne.DatWriter(path, 1, 3, 100).finish()


def test_foreign_magic_is_recreated_and_unreadable_errors(jne, tmp):
    path = os.path.join(tmp, "m.dat")
    open(path, "wb").write(b"EIGENVALS_V5" + bytes(40))
    with pytest.raises(jne.DatError) as ei:
        jne.read_dat(path)
    assert "magic header mismatch" in str(ei.value)
    w = jne.DatWriter(path, 0, 1, 10)  # writer.rs:116-150: incompatible format -> recreate
    assert w.existing == 0
    w.append_eigenvalues(1, [1.0])
    w.finish()
    assert len(jne.read_dat(path)[0]) == 1
    with pytest.raises(jne.DatError) as ei:
        jne.read_dat(os.path.join(tmp, "missing.dat"))
    assert ei.value.code == jne.JNE_ERR_IO


def test_header_only_file(jne, oracle, tmp):
    path = os.path.join(tmp, "h.dat")
    open(path, "wb").write(oracle.dat_bytes(0, 1, 10, [], finished=False))
    recs, model, dim, steps = jne.read_dat(path)
    assert len(recs) == 0 and (model, dim, steps) == (0, 1, 10)


def test_percentiles_match_rule(jne, oracle):
    rng = np.random.default_rng(5)
    eigs = np.sort(rng.gamma(2.0, 3.0, size=(501, 4)), axis=1)[:, ::-1]
    ps = [0.01, 0.05, 0.1, 0.5, 0.9, 0.95, 0.99, 0.0, 1.0]
    tr = jne.percentiles(eigs, "trace", ps)
    mx = jne.percentiles(eigs, "maxeig", ps)
    for p, a, b in zip(ps, tr, mx):
        assert abs(a - oracle.percentile_value(np.sort(eigs.sum(1)), p)) < 1e-12
        assert abs(b - oracle.percentile_value(np.sort(eigs.max(1)), p)) < 1e-12
    assert np.isnan(jne.percentiles(np.zeros((0, 3)), "trace", [0.5])[0])


def test_simulation_filenames(jne, tmp):  # filename_consistency.rs, simulation_test.rs:47-78
    for m in range(5):
        sim = jne.EigenvalueSimulation(m, 3, 500, 1000, data_dir=os.path.join(tmp, "data"))
        assert os.path.basename(sim.get_filename(m)) == f"eigenvalues_model{m}_dim3_steps500.dat"
    a = jne.EigenvalueSimulation(0, 5, 999, 100, data_dir=tmp).get_filename()
    b = jne.EigenvalueSimulation(0, 5, 999, 500, data_dir=tmp).get_filename()
    assert a == b and os.path.basename(a) == "eigenvalues_model0_dim5_steps999.dat"


def test_percentile_arguments_and_nan(jne):
    eigs = np.array([[3.0, 1.0], [2.0, 0.5]])
    with pytest.raises(jne.DatError):
        jne.percentiles(eigs, "trace", [1.5])   # the reference indexes past the end
    with pytest.raises(jne.DatError):
        jne.percentiles(eigs, "trace", [-0.1])
    bad = eigs.copy()
    bad[1, 0] = np.nan                            # the reference's sort panics on NaN
    with pytest.raises(jne.DatError) as ei:
        jne.percentiles(bad, "trace", [0.5])
    assert ei.value.code == jne.JNE_ERR_NUMERIC
    # the Max aggregator folds with f64::max, which skips NaN
    assert jne.percentiles(bad, "maxeig", [0.0, 1.0]) == [0.5, 3.0]


@pytest.mark.parametrize("finished", [True, False])
def test_large_file_parallel_decode(jne, tmp, finished):
    """> 65,536 records: the values are decoded by several host threads, from the
    trailer index (finished) or the scan index (interrupted)."""
    rng = np.random.default_rng(3)
    n, k = 300_001, 3
    seeds = rng.permutation(np.arange(1, 2 * n, 2, dtype=np.uint32))[:n]  # 1- to 3-byte ULEB128 seeds
    seeds[:3] = [1, 0xFFFFFFFF, 1 << 28]                                   # 1- and 5-byte seeds
    eigs = rng.standard_normal((n, k))
    path = os.path.join(tmp, f"big_{finished}.dat")
    w = jne.DatWriter(path, 1, 2, 64)
    w.append(seeds, eigs)
    w.finish() if finished else w.abandon()
    recs, model, dim, steps = jne.read_dat(path)
    assert (model, dim, steps) == (1, 2, 64)
    assert np.array_equal(np.asarray(recs.seeds, dtype=np.uint32), seeds)
    assert np.array_equal(recs.eigs, eigs)


_SHORT_WRITE_CHILD = r"""
import os, resource, signal, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import __graft_entry__ as entry
jne = entry.load_package()
path, limit = sys.argv[2], int(sys.argv[3])
w = jne.DatWriter(path, 0, 2, 100)           # header written before the limit applies
w.append(range(1, 3), np.ones((2, 2)))
signal.signal(signal.SIGXFSZ, signal.SIG_IGN)  # a write past the limit fails with EFBIG instead
resource.setrlimit(resource.RLIMIT_FSIZE, (limit, limit))
n = 100_000                                   # 2.7 MB of records in one block
try:
    w.append(range(3, 3 + n), np.arange(2 * n, dtype=float).reshape(n, 2))
except jne.DatError as e:
    print("IOERR", e.code)
w.abandon()
"""


def test_short_write_leaves_whole_records(jne, tmp):
    """A block write that the file system cuts short (here a file-size limit) leaves the file at a record
    boundary: every record in it reads back whole, with no partial record at the end."""
    import subprocess
    import sys

    from conftest import ROOT

    path = os.path.join(tmp, "short.dat")
    limit = 100_003  # not a record boundary (records of dim 2 take 19-22 bytes)
    out = subprocess.run([sys.executable, "-c", _SHORT_WRITE_CHILD, ROOT, path, str(limit)],
                         capture_output=True, text=True, timeout=120)
    assert f"IOERR {jne.JNE_ERR_IO}" in out.stdout, out.stdout + out.stderr
    size = os.path.getsize(path)
    assert size <= limit
    recs, model, dim, steps = jne.read_dat(path)  # no trailer: read by scanning
    n = len(recs.seeds)
    assert n > 1000
    assert list(recs.seeds[:3]) == [1, 2, 3]
    assert np.array_equal(recs.eigs[2:], np.arange(2 * (n - 2), dtype=float).reshape(n - 2, 2))
    # the file ends exactly after the last record: 18-byte header + records of 1-3 seed bytes + 1 + 16
    seeds = np.asarray(recs.seeds, dtype=np.int64)
    seed_bytes = 1 + (seeds >= 1 << 7) + (seeds >= 1 << 14) + (seeds >= 1 << 21)
    assert size == 18 + int(np.sum(seed_bytes + 17))


def test_dat_sink_host_side(jne, tmp):
    """jne_dat_sink_open/close and its write callback, driven directly (no GPU): records reach each
    request's simulation file in the order written, requests of the same (model, dim, steps) share a file,
    a non-OK status stops with that status, and close writes the trailers."""
    import ctypes

    L = jne.lib()
    reqs = (jne.Request * 3)(jne.Request(0, 2, 100, 1, 7, 1, 4), jne.Request(3, 2, 50, 1, 7, 1, 3),
                             jne.Request(0, 2, 100, 1, 7, 5, 2))
    sink = jne.Sink()
    assert L.jne_dat_sink_open(os.fsencode(tmp), reqs, 3, ctypes.byref(sink)) == jne.JNE_OK

    def write(req, seed_first, eigs, status=jne.JNE_OK):
        e = np.ascontiguousarray(eigs, dtype=np.float64)
        return sink.write(sink.user, req, seed_first, e.shape[0], e.shape[1],
                          e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), status)

    a = np.arange(8.0).reshape(4, 2)
    b = np.arange(9.0).reshape(3, 3) + 100
    c = np.arange(4.0).reshape(2, 2) + 50
    assert write(0, 1, a[:3]) == jne.JNE_OK
    assert write(1, 1, b) == jne.JNE_OK
    assert write(0, 4, a[3:]) == jne.JNE_OK
    assert write(2, 5, c) == jne.JNE_OK
    assert write(2, 7, c[:1], jne.JNE_ERR_NUMERIC) == jne.JNE_ERR_NUMERIC  # NaN rows are not written
    assert L.jne_dat_sink_close(ctypes.byref(sink), 1) == jne.JNE_OK
    recs, model, dim, steps = jne.read_dat(os.path.join(tmp, "eigenvalues_model0_dim2_steps100.dat"))
    assert (model, dim, steps) == (0, 2, 100)
    assert list(recs.seeds) == [1, 2, 3, 4, 5, 6]
    assert np.array_equal(recs.eigs, np.vstack([a, c]))
    recs, model, dim, steps = jne.read_dat(os.path.join(tmp, "eigenvalues_model3_dim2_steps50.dat"))
    assert list(recs.seeds) == [1, 2, 3] and np.array_equal(recs.eigs, b)
    assert open(os.path.join(tmp, "eigenvalues_model3_dim2_steps50.dat"), "rb").read()[-17:-9] == b"EOF_MARK"


def _record_part(oracle, seed_first, eigs):
    """The records of seeds seed_first.. in the oracle's restatement of the format (no header, no trailer)."""
    recs = [(seed_first + r, list(eigs[r])) for r in range(eigs.shape[0])]
    return oracle.dat_bytes(0, 2, 100, recs, finished=False)[18:]


def test_record_bytes_closed_form(jne, oracle):
    """jne_record_bytes against the ULEB128 lengths of the restatement, across every length threshold."""
    for a in (0, 1, 126, 127, 128, 16383, 16384, 2**21 - 2, 2**28 - 1, 2**32 - 3):
        for n in (0, 1, 2, 5, 300):
            if a + n > 2**32:
                continue
            for k in (1, 2, 13, 255):
                want = sum(len(oracle.uleb128_encode(a + r)) + 1 + 8 * k for r in range(n))
                assert jne.record_bytes(a, n, k) == want, (a, n, k)
    assert jne.record_bytes(2**32 - 1, 1, 3) == 5 + 1 + 24
    for bad in ((2**32 - 1, 2, 3), (0, -1, 3), (0, 1, 256), (0, 1, -1)):
        assert jne.record_bytes(*bad) == -1


def test_append_packed_matches_format_restatement(jne, oracle, tmp):
    """Packed records appended as they are give the file jne_dat_append gives (the restatement's bytes),
    with the same count checks."""
    rng = np.random.default_rng(5)
    eigs = rng.standard_normal((400, 2))
    a = 16200  # the seeds cross the 2- to 3-byte ULEB128 boundary at 16384
    recs = _record_part(oracle, a, eigs)
    split = jne.record_bytes(a, 150, 2)
    path = os.path.join(tmp, "p.dat")
    w = jne.DatWriter(path, 0, 2, 100)
    w.append_packed(a, 150, 2, recs[:split])
    w.append_packed(a + 150, 250, 2, recs[split:])
    w.append_packed(a + 400, 0, 2, b"")
    w.finish()
    assert open(path, "rb").read() == oracle.dat_bytes(0, 2, 100, [(a + r, list(eigs[r])) for r in range(400)])
    w = jne.DatWriter(path, 0, 2, 100)
    with pytest.raises(jne.DatError) as ei:  # the file holds 2 values per record
        w.append_packed(1, 1, 3, bytes(jne.record_bytes(1, 1, 3)))
    assert ei.value.code == jne.JNE_ERR_FORMAT and "count mismatch" in str(ei.value)
    with pytest.raises(ValueError):
        w.append_packed(1, 2, 2, recs[:10])
    w.abandon()


_SHORT_PACKED_CHILD = r"""
import os, resource, signal, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import __graft_entry__ as entry
jne, oracle = entry.load_package(), entry.load_oracle()
path, limit = sys.argv[2], int(sys.argv[3])
n = 100_000
eigs = np.arange(2 * n, dtype=float).reshape(n, 2)
recs = oracle.dat_bytes(0, 2, 100, [(3 + r, list(eigs[r])) for r in range(n)], finished=False)[18:]
w = jne.DatWriter(path, 0, 2, 100)
w.append(range(1, 3), np.ones((2, 2)))
signal.signal(signal.SIGXFSZ, signal.SIG_IGN)
resource.setrlimit(resource.RLIMIT_FSIZE, (limit, limit))
try:
    w.append_packed(3, n, 2, recs)
except jne.DatError as e:
    print("IOERR", e.code)
w.abandon()
"""


def test_short_packed_write_leaves_whole_records(jne, tmp):
    """A packed append cut short by the file system also leaves the file at a record boundary."""
    import subprocess
    import sys

    from conftest import ROOT

    path = os.path.join(tmp, "short_packed.dat")
    limit = 100_003
    out = subprocess.run([sys.executable, "-c", _SHORT_PACKED_CHILD, ROOT, path, str(limit)],
                         capture_output=True, text=True, timeout=120)
    assert f"IOERR {jne.JNE_ERR_IO}" in out.stdout, out.stdout + out.stderr
    size = os.path.getsize(path)
    assert size <= limit
    recs, model, dim, steps = jne.read_dat(path)
    n = len(recs.seeds)
    assert n > 1000 and list(recs.seeds[:3]) == [1, 2, 3]
    assert np.array_equal(recs.eigs[2:], np.arange(2 * (n - 2), dtype=float).reshape(n - 2, 2))
    assert size == 18 + jne.record_bytes(1, n, 2)
