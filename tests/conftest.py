import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

import __graft_entry__ as entry  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def jne():
    return entry.load_package()


@pytest.fixture(scope="session")
def oracle():
    import jne_oracle

    if not os.path.exists(jne_oracle.LIB_PATH):
        import subprocess

        subprocess.run(["sh", os.path.join(ROOT, "oracle", "build.sh")], check=True)
    return jne_oracle


@pytest.fixture(scope="session")
def golden():
    from gen_golden import generated_increments, load_increments

    data = np.load(os.path.join(ROOT, "tests", "golden", "golden_eigs.npz"))
    cases = {}
    for key in data.files:
        if key.startswith("z_"):
            _, d, t = key.split("_")
            cases[(int(d[1:]), int(t[1:]))] = load_increments(data[key])
        elif key.startswith("gseed_"):  # stored as (runs, seed): increments regenerated
            _, d, t = key.split("_")
            dim, steps = int(d[1:]), int(t[1:])
            runs, seed = (int(x) for x in data[key])
            cases[(dim, steps)] = generated_increments(dim, steps, runs, seed)
    eigs = {}
    for key in data.files:
        if key.startswith("eig_") or key.startswith("geig_"):
            _, m, d, t = key.split("_")
            eigs[(int(m[1:]), int(d[1:]), int(t[1:]))] = data[key]
    return cases, eigs


@pytest.fixture(scope="session")
def engine(jne):
    eng = jne.Engine(0)
    yield eng
    eng.close()


def normwise_err(got: np.ndarray, ref: np.ndarray, floor: float = 0.0) -> float:
    """max_j |got - ref| / max(max_j |ref|, floor) per run, maximised over runs.

    floor = 0 is the plain normwise-relative error.  floor = 1 makes it absolute
    for runs whose largest eigenvalue is below 1: there the statistic comes from
    a cancelling Ito sum (S10 = (B_T^2 - sum dB^2)/2 in one dimension), so a
    fixed relative precision of the moments cannot bound its relative error,
    while every critical value the tables are used for is well above 1."""
    got = np.atleast_2d(got)
    ref = np.atleast_2d(ref)
    den = np.maximum(np.abs(ref).max(axis=1), floor)
    return float(np.max(np.abs(got - ref).max(axis=1) / den))
