"""The reference's own CUDA kernels, built unmodified and driven by our harness.

TEST INFRASTRUCTURE ONLY.  build() compiles
  - src/openvslam/PatchMatchCuda.cu of the reference, unmodified, from where
    it lies (REFERENCE_SRC), into a device-only fatbin oracle/_ref/refpm_sm103a.fatbin,
    with the stand-in OpenCV header and the CUDA 13 compatibility header of
    oracle/refshim/ (only where the reference sources are present: the fatbin
    is built in the development container and carried to the GPU machine);
  - oracle/ref_harness.cu (our code) into oracle/_build/libref_harness.so.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# Where the reference project lies: PM_REFERENCE_ROOT, else its checkout in
# the development container (absent on machines that only run the tests).
REFERENCE_ROOT = os.environ.get("PM_REFERENCE_ROOT", "/root/reference")
REFERENCE_SRC = os.path.join(REFERENCE_ROOT, "src", "openvslam", "PatchMatchCuda.cu")
REF_DIR = os.path.join(HERE, "_ref")
FATBIN = os.path.join(REF_DIR, "refpm_sm103a.fatbin")
HARNESS_SRC = os.path.join(HERE, "ref_harness.cu")
HARNESS = os.path.join(HERE, "_build", "libref_harness.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build(force: bool = False):
    """Build the fatbin (when the reference sources exist) and the harness."""
    os.makedirs(os.path.dirname(HARNESS), exist_ok=True)
    if os.path.exists(REFERENCE_SRC) and (force or not os.path.exists(FATBIN)):
        os.makedirs(REF_DIR, exist_ok=True)
        subprocess.check_call([_nvcc(), "-std=c++17", "-O3", "-fatbin"] + ARCH +
                              ["-I" + os.path.join(HERE, "refshim"), "-include", "pm_ref_compat.h",
                               "-o", FATBIN, REFERENCE_SRC],
                              stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    if force or not os.path.exists(HARNESS) or os.path.getmtime(HARNESS) < os.path.getmtime(HARNESS_SRC):
        subprocess.check_call([_nvcc(), "-std=c++17", "-O2", "-shared", "-Xcompiler", "-fPIC"] + ARCH +
                              ["-o", HARNESS, HARNESS_SRC, "-lcuda"])
    return FATBIN if os.path.exists(FATBIN) else None


def available() -> bool:
    return os.path.exists(FATBIN)


_fp = C.POINTER(C.c_float)


class RefKernels:
    """One loaded copy of the reference kernels (process-wide state, like the reference)."""

    def __init__(self):
        build()
        if not available():
            raise FileNotFoundError(f"reference kernels not built ({FATBIN})")
        L = C.CDLL(HARNESS)
        L.rh_error.restype = C.c_char_p
        L.rh_load.argtypes = [C.c_char_p]
        L.rh_setup.argtypes = [C.c_int, C.c_int] + [_fp] * 9
        L.rh_bearings.argtypes = [_fp]
        L.rh_score.argtypes = [_fp, _fp, C.c_float]
        L.rh_run.argtypes = [C.c_int, C.c_float, C.c_float, _fp, _fp, _fp]
        L.rh_time_passes.argtypes = [C.c_int, _fp]
        L.rh_probe_texture.argtypes = [C.c_int, _fp, C.c_int, _fp]
        self.L = L
        self._check(L.rh_load(FATBIN.encode()))
        self.W = self.H = 0

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"reference harness: {self.L.rh_error().decode()}")

    @staticmethod
    def poses(R, t):
        """Reference host pose packing (depthmap.cc:577-665) for views 0, 1, 2."""
        R = np.asarray(R, np.float64).reshape(-1, 3, 3)
        t = np.asarray(t, np.float64).reshape(-1, 3)
        R1inv = R[0].T
        t1inv = -R1inv @ t[0]
        f = lambda a: np.ascontiguousarray(a, np.float32).reshape(-1)
        return f(R[1]), f(t[1]), f(R[2]), f(t[2]), f(R1inv), f(t1inv)

    def setup(self, images, R, t):
        imgs = [np.ascontiguousarray(im, np.float32) for im in images[:3]]
        H, W = imgs[0].shape
        self._keep = imgs
        ps = self.poses(R, t)
        self._keep_p = ps
        p = lambda a: a.ctypes.data_as(_fp)
        self._check(self.L.rh_setup(W, H, p(imgs[0]), p(imgs[1]), p(imgs[2]), *[p(a) for a in ps]))
        self.W, self.H = W, H

    def bearings(self):
        out = np.zeros((self.H, self.W, 3), np.float32)
        self._check(self.L.rh_bearings(out.ctypes.data_as(_fp)))
        return out

    def score(self, planes, fill=-7.0):
        planes = np.ascontiguousarray(planes, np.float32)
        out = np.zeros((self.H, self.W), np.float32)
        self._check(self.L.rh_score(planes.ctypes.data_as(_fp), out.ctypes.data_as(_fp), fill))
        return out

    def run(self, iterations, min_depth, max_depth):
        d = np.zeros((self.H, self.W), np.float32)
        pl = np.zeros((self.H, self.W, 3), np.float32)
        s = np.zeros((self.H, self.W), np.float32)
        self._check(self.L.rh_run(iterations, min_depth, max_depth, d.ctypes.data_as(_fp), pl.ctypes.data_as(_fp),
                                  s.ctypes.data_as(_fp)))
        return dict(depth=d, plane=pl, score=s)

    def time_passes(self, iterations):
        ms = C.c_float()
        self._check(self.L.rh_time_passes(iterations, C.byref(ms)))
        return ms.value

    def probe_texture(self, source, xy):
        xy = np.ascontiguousarray(xy, np.float32)
        out = np.zeros(len(xy), np.float32)
        self._check(self.L.rh_probe_texture(source, xy.ctypes.data_as(_fp), len(xy), out.ctypes.data_as(_fp)))
        return out
