"""The C-ABI library: builds, loads, exports every declared symbol, validates
arguments on the host, and fails loudly without a GPU.  No kernel runs here."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "jne.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(jne_[a-z0-9_]+)\s*\(", src)))


def test_header_and_python_binding_agree(jne):
    assert _declared_functions() == sorted(jne.EXPORTS)


def test_library_exports_every_declared_symbol(jne):
    lib = jne.lib()
    for name in _declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", jne.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(jne_[a-z0-9_]+)$", out, flags=re.M))
    assert set(_declared_functions()) <= exported


def test_eigen_count_and_version(jne):
    lib = jne.lib()
    assert lib.jne_version() >= 100
    for model in range(5):
        for dim in (1, 2, 12):
            assert lib.jne_eigen_count(model, dim) == jne.eigen_count(model, dim)
    assert lib.jne_eigen_count(5, 2) == -1
    assert lib.jne_eigen_count(0, 0) == -1


def test_null_arguments_are_rejected(jne):
    lib = jne.lib()
    assert lib.jne_open(0, 0, None) == jne.JNE_ERR_ARG
    assert lib.jne_set_chunk(None, 256) == jne.JNE_ERR_ARG
    assert lib.jne_eigs_seeded(None, 0, 2, 10, 1, 1, 1, 0, None) == jne.JNE_ERR_ARG
    assert lib.jne_last_error(None) == b"null context"
    lib.jne_close(None)  # no-op


def test_models_enum_mirrors_reference(jne):
    M = jne.JohansenModel
    assert [m.to_number() for m in M.all_models()] == [0, 1, 2, 3, 4]
    assert M.default() == M.InterceptNoTrendUnrestrictedIntercept
    assert str(M(0)) == "Model 0: No intercept, no trend"
    assert M.from_number(7) is None
    assert [m.has_trend() for m in M.all_models()] == [False, False, False, True, True]
    assert [m.has_intercept() for m in M.all_models()] == [False, True, True, True, True]


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU failure path")
def test_engine_fails_loudly_without_gpu(jne):
    with pytest.raises(jne.JneError) as ei:
        jne.Engine(0)
    assert ei.value.code == jne.JNE_ERR_CUDA
