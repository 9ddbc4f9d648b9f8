"""The reference's own host stages, built unmodified and driven by our harness.

TEST INFRASTRUCTURE ONLY.  build() compiles src/openvslam/depthmap.cc of the
reference, unmodified, from where it lies (PM_REFERENCE_ROOT, else its
checkout in the development container), against the OpenCV stand-in in
oracle/refshim_host, together with oracle/ref_host_harness.cc (ours), into
oracle/_ref/librefhost.so.  Where the reference sources are absent nothing is
built and available() is False; the golden fixture
tests/golden/ref_host_96x48.npz (made by tests/golden/make_golden_host.py)
carries the reference's outputs instead.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_ROOT = os.environ.get("PM_REFERENCE_ROOT", "/root/reference")
REFERENCE_CC = os.path.join(REFERENCE_ROOT, "src", "openvslam", "depthmap.cc")
LIB = os.path.join(HERE, "_ref", "librefhost.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build(force: bool = False):
    if not os.path.exists(REFERENCE_CC):
        return None
    src = os.path.join(HERE, "ref_host_harness.cc")
    shim = os.path.join(HERE, "refshim_host", "opencv2", "opencv.hpp")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(shim), os.path.getmtime(os.path.abspath(__file__))):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared",
                           "-I" + os.path.join(HERE, "refshim_host"), "-I" + os.path.join(CUDA, "include"),
                           "-I" + os.path.dirname(REFERENCE_CC), src, REFERENCE_CC, "-o", LIB,
                           # the package library, loaded RTLD_GLOBAL, exports the same dense::
                           # class names (it mirrors this interface): bind to our own copies
                           "-Wl,-Bsymbolic", "-L" + os.path.join(CUDA, "lib64"), "-lcudart"],
                          stdout=subprocess.DEVNULL, stderr=subprocess.STDOUT)
    return LIB


def available() -> bool:
    try:
        return build() is not None
    except (OSError, subprocess.CalledProcessError):
        return False


_lib = None
_fp, _dp, _u8p, _ip = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_uint8), C.POINTER(C.c_int)


def lib():
    global _lib
    if _lib is None:
        if build() is None:
            raise FileNotFoundError("reference sources not present")
        L = C.CDLL(LIB)
        L.rhh_postprocess.argtypes = [C.c_int, C.c_int, _fp, _fp, _dp, C.c_float, C.c_float, C.c_float]
        L.rhh_clean.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(_fp), _dp, _dp, C.c_float, C.c_int, _fp]
        L.rhh_prune.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(_fp), _dp, _dp, _u8p, C.c_float, _fp, _dp,
                                _u8p, _ip, C.c_int]
        L.rhh_prune.restype = C.c_int
        _lib = L
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def postprocess(depth, score, plane, min_depth=0.3, max_depth=20.0, min_score=0.1):
    """PostProcess (depthmap.cc:1169-1208) of the reference: (depth, score)."""
    H, W = depth.shape
    d = np.ascontiguousarray(depth, np.float32).copy()
    s = np.ascontiguousarray(score, np.float32).copy()
    pl = np.ascontiguousarray(plane, np.float64)
    lib().rhh_postprocess(W, H, _p(d, _fp), _p(s, _fp), _p(pl, _dp), min_depth, max_depth, min_score)
    return d, s


def clean(depths, R, t, thr, min_views=3):
    """DepthmapCleaner::Clean of the centre map (index len // 2)."""
    depths = [np.ascontiguousarray(d, np.float32) for d in depths]
    H, W = depths[0].shape
    arr = (_fp * len(depths))(*[_p(d, _fp) for d in depths])
    R = np.ascontiguousarray(R, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    out = np.zeros((H, W), np.float32)
    lib().rhh_clean(W, H, len(depths), arr, _p(R, _dp), _p(t, _dp), thr, min_views, _p(out, _fp))
    return out


def prune(depths, R, t, bgr, thr):
    """DepthmapPruner::Prune of map 0: (pruned depth, points (n, 3) f64, colours (n, 3), (row, col) (n, 2))."""
    depths = [np.ascontiguousarray(d, np.float32) for d in depths]
    H, W = depths[0].shape
    arr = (_fp * len(depths))(*[_p(d, _fp) for d in depths])
    R = np.ascontiguousarray(R, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    bgr = None if bgr is None else np.ascontiguousarray(bgr, np.uint8)
    cap = H * W
    pruned = np.zeros((H, W), np.float32)
    xyz = np.zeros((cap, 3), np.float64)
    cols = np.zeros((cap, 3), np.uint8)
    ij = np.zeros((cap, 2), np.int32)
    n = lib().rhh_prune(W, H, len(depths), arr, _p(R, _dp), _p(t, _dp), _p(bgr, _u8p), thr, _p(pruned, _fp),
                        _p(xyz, _dp), _p(cols, _u8p), _p(ij, _ip), cap)
    return pruned, xyz[:n], cols[:n], ij[:n]
