"""Builds and runs tests/cpp/test_dense.cpp: the C++ mirror of the reference's
DepthmapEstimator / DepthmapCleaner / DepthmapPruner over a keyframe sequence."""
import os
import subprocess

import pytest

from patchmatch_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp):
    exe = os.path.join(tmp, "test_dense")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "test_dense.cpp"), "-o", exe,
                           "-L" + _native.LIB_DIR, "-lpm_gb300", "-lpm_scene", "-Wl,-rpath," + _native.LIB_DIR])
    return exe


def test_cpp_mirror_compiles_and_links(built, tmp_path):
    assert os.path.exists(_build(str(tmp_path)))


@pytest.mark.gpu
def test_cpp_mirror_pipeline(built, tmp_path):
    exe = _build(str(tmp_path))
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
