"""EigenvalueSimulation end to end on the GPU: the assertions of the reference's
integration tests (src/tests/data_storage/integration/*.rs, simulation_test.rs)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def data_dir(tmp_path):
    return str(tmp_path / "data")


def sim(jne, engine, model, dim, steps, runs, data_dir, **kw):
    return jne.EigenvalueSimulation(model, dim, steps, runs, data_dir=data_dir, engine=engine, **kw)


def test_basic_simulation_api(jne, engine, data_dir):  # basic_api.rs:4-49
    s0 = sim(jne, engine, 0, 2, 101, 5, data_dir)
    fn = s0.get_filename(0)
    assert "model0" in fn and "dim2" in fn and "steps101" in fn and fn.endswith(".dat")
    for m in jne.JohansenModel.all_models():
        sim(jne, engine, m, 2, 101, 5, data_dir).run_simulation_quiet()
    assert os.path.exists(fn)
    data = s0.read_data()
    assert len(data) == 5
    for seed, eig in data:
        assert 1 <= seed <= 5 and len(eig) == 2
    srt = data.sorted_by_seed()
    assert list(srt.seeds) == sorted(srt.seeds)


def test_results_equal_direct_batch(jne, engine, data_dir):
    for prec in (jne.PREC_FP64, jne.PREC_MIXED):
        s = sim(jne, engine, 3, 4, 700, 37, data_dir + str(prec), precision=prec)
        s.run_simulation_quiet()
        d = s.read_data().sorted_by_seed()
        assert np.array_equal(d.eigs, engine.eigs_seeded(3, 4, 700, 1, 37, precision=prec))


def test_resumable(jne, engine, data_dir):  # resumable.rs:4-85
    s = sim(jne, engine, 0, 2, 103, 5, data_dir)
    s.run_simulation_quiet()
    data = s.read_data().sorted_by_seed()
    original = data.eigs.sum(1)
    # remove seeds 2 and 4 (helpers.rs:25-68 rewrites the file without them)
    keep = [i for i, sd in enumerate(data.seeds) if sd not in (2, 4)]
    os.remove(s.get_filename())
    w = jne.DatWriter(s.get_filename(), 0, 2, 103)
    w.append(data.seeds[keep], data.eigs[keep])
    w.finish()
    after = s.read_all_data()
    assert len(after) == 3 and not set(after.seeds) & {2, 4}
    with pytest.raises(jne.DatError):
        s.read_data()
    s.run_simulation_quiet()
    final = s.read_data().sorted_by_seed()
    assert list(final.seeds) == [1, 2, 3, 4, 5]
    assert np.max(np.abs(final.eigs.sum(1) - original)) < 1e-10


def test_read_data_error_handling(jne, engine, data_dir):  # simulation_test.rs:80-133
    s = sim(jne, engine, 0, 2, 201, 5, data_dir)
    with pytest.raises(jne.DatError):
        s.read_data()
    with pytest.raises(jne.DatError):
        s.read_all_data()
    sim(jne, engine, 0, 2, 201, 3, data_dir).run_simulation_quiet()
    with pytest.raises(jne.DatError) as ei:
        s.read_data()
    assert "expected 5 records, found 3 records" in str(ei.value)
    assert "Use `read_all_data()`" in str(ei.value)
    assert len(s.read_all_data()) == 3
    s.run_simulation_quiet()
    assert len(s.read_data()) == 5 and len(s.read_all_data()) == 5


def test_read_data_filters_seeds_beyond_num_runs(jne, engine, data_dir):  # simulation_test.rs:4-45
    sim(jne, engine, 0, 2, 10, 6, data_dir).run_simulation_quiet()
    s = sim(jne, engine, 0, 2, 10, 3, data_dir)
    assert len(s.read_all_data()) == 6
    d = s.read_data()
    assert len(d) == 3 and max(d.seeds) <= 3


def test_edge_case_single_run(jne, engine, data_dir):  # edge_cases.rs:4-22
    for m in range(5):
        sim(jne, engine, m, 2, 11, 1, data_dir).run_simulation_quiet()
    d = sim(jne, engine, 0, 2, 11, 1, data_dir).read_data()
    assert len(d) == 1 and d[0][0] == 1


def test_multiple_models_finite(jne, engine, data_dir):  # multiple_models.rs:4-47
    for m in range(5):
        s = sim(jne, engine, m, 2, 54, 3, data_dir)
        s.run_simulation_quiet()
        d = s.read_data()
        assert len(d) == 3
        assert all(len(e) >= 1 and np.all(np.isfinite(e)) for _, e in d)


def test_incompatible_file_is_recreated(jne, engine, data_dir):  # parallel_compute.rs:155-180
    s = sim(jne, engine, 1, 2, 77, 4, data_dir)
    fn = s.get_filename()
    w = jne.DatWriter(fn, 0, 2, 77)  # wrong model in the header
    w.append_eigenvalues(1, [1.0, 2.0])
    w.finish()
    s.run_simulation_quiet()
    recs, model, dim, steps = jne.read_dat(fn)
    assert (model, dim, steps) == (1, 2, 77) and len(recs) == 4 and recs.eigs.shape[1] == 3


def test_percentiles_from_simulation(jne, engine, data_dir):  # examples/library_usage_example.rs
    s = sim(jne, engine, 0, 5, 1000, 1000, data_dir)
    s.run_simulation_quiet()
    p = [0.5, 0.9, 0.95]
    d = s.read_data()
    assert s.calculate_trace_percentiles(p) == jne.percentiles(d.eigs, "trace", p)
    mx = s.calculate_maxeig_percentiles(p)
    assert mx == sorted(mx) and mx[0] > 0


@pytest.mark.parametrize("prec", [0, 1])
def test_all_models_in_one_pass_write_the_same_files(jne, engine, tmp_path, prec):
    """jne_simulation_run_models: one pass over the paths for every model, files byte-identical
    to one EigenvalueSimulation per model."""
    one, many = str(tmp_path / "one"), str(tmp_path / "many")
    for m in range(5):
        sim(jne, engine, m, 3, 600, 777, one, precision=prec).run_simulation_quiet()
    jne.run_simulations(range(5), 3, 600, 777, data_dir=many, precision=prec, engine=engine)
    for m in range(5):
        name = f"eigenvalues_model{m}_dim3_steps600.dat"
        assert open(os.path.join(one, name), "rb").read() == open(os.path.join(many, name), "rb").read()


def test_all_models_resume_from_different_points(jne, engine, data_dir):
    # model 1 already has 300 runs, model 4 has all 500, models 0 and 2 none
    sim(jne, engine, 1, 2, 400, 300, data_dir).run_simulation_quiet()
    sim(jne, engine, 4, 2, 400, 500, data_dir).run_simulation_quiet()
    jne.run_simulations([0, 1, 2, 4], 2, 400, 500, data_dir=data_dir, engine=engine)
    for m in (0, 1, 2, 4):
        d = sim(jne, engine, m, 2, 400, 500, data_dir).read_data().sorted_by_seed()
        assert list(d.seeds) == list(range(1, 501))
        assert np.array_equal(d.eigs, engine.eigs_seeded(m, 2, 400, 1, 500, precision=jne.PREC_MIXED))
    with pytest.raises(jne.DatError):
        jne.run_simulations([0, 0], 2, 400, 10, data_dir=data_dir, engine=engine)
