"""The command-line driver (flags of cli.rs:56-132, loop of main.rs:85-136)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "johansen-null-eigenspectra_gb300", "jne_gb300")


def run(*args, cwd=None):
    return subprocess.run([CLI, *args], capture_output=True, text=True, timeout=600, cwd=cwd)


@pytest.fixture(scope="module", autouse=True)
def built(jne):
    if not os.path.exists(CLI):
        pytest.fail("jne_gb300 is not built (run __graft_entry__.build())")


def test_help_and_version():
    r = run("--help")
    assert r.returncode == 0 and "--dim-start" in r.stdout and "--model <list>" in r.stdout
    r = run("--version")
    assert r.returncode == 0 and r.stdout.startswith("jne_gb300 version ")


@pytest.mark.parametrize("args, msg", [
    (["--steps"], "--steps parameter requires a value"),
    (["--runs", "12x"], "must be a positive integer"),
    (["--runs", "-5"], "must be a positive integer"),
    (["--dim-start", "5", "--dim-end", "3"], "cannot be greater than end"),
    (["--steps", "0"], "must be greater than 0"),
    (["--model", "0,7"], "invalid model number"),
    (["--model", " , "], "must not be empty"),
    (["--precision", "half"], "fp64 or mixed"),
    (["--dim", "13"], "not supported"),
    (["--frobnicate"], "unknown argument"),
])
def test_argument_errors(args, msg):
    r = run(*args)
    assert r.returncode == 1 and msg in r.stderr


@pytest.mark.gpu
def test_runs_writes_files_prints_tables_and_resumes(jne, tmp_path):
    d = str(tmp_path / "data")
    r = run("--dim", "2", "--steps", "1,000", "--runs", "3,000", "--model", "0,3", "--data-dir", d)
    assert r.returncode == 0, r.stderr
    assert r.stdout.count("Trace for model Model") == 2 and r.stdout.count("MaxEig for model Model") == 2
    assert "Total calculated 3,000 values" in r.stdout
    for m, k in ((0, 2), (3, 3)):
        recs, model, dim, steps = jne.read_dat(os.path.join(d, f"eigenvalues_model{m}_dim2_steps1000.dat"))
        assert (model, dim, steps) == (m, 2, 1000) and recs.eigs.shape == (3000, k)
        assert sorted(recs.seeds) == list(range(1, 3001))
        with jne.Engine(0) as eng:
            ref = eng.eigs_seeded(m, 2, 1000, 1, 3000, precision=jne.PREC_MIXED)
        order = np.argsort(recs.seeds)
        assert np.array_equal(recs.eigs[order], ref)
    r = run("--dim", "2", "--steps", "1000", "--runs", "3000", "--model", "0", "--data-dir", d)
    assert r.returncode == 0 and "already completed" in r.stdout
    r = run("--dim", "2", "--steps", "1000", "--runs", "3000", "--model", "0", "--data-dir", d, "--quiet")
    assert r.returncode == 0 and r.stdout == ""
