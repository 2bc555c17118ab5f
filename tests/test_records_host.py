"""The device record packer's per-thread body (jne_pack_chunk) and the closed-form record arithmetic of
csrc/jne_records.h, run on the host against a plain record encoder (no GPU): a C++ checker compiled here, with
AddressSanitizer and UBSan when the toolchain has them."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "records_check", "check_records.cpp")


def _build(tmp_path):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "check_records")
    base = [cxx, "-std=c++17", "-O1", "-g", SRC, "-o", exe]
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all"]
    if subprocess.run(base[:-2] + san + ["-o", exe], capture_output=True).returncode != 0:
        res = subprocess.run(base, capture_output=True, text=True)  # no sanitizer runtime: plain build
        assert res.returncode == 0, res.stderr
    return exe


def test_packer_body_matches_plain_encoder(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    assert out.stdout.strip().endswith(" 0 failures"), out.stdout
