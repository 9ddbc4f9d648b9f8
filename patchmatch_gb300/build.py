"""In-tree build of the native libraries (no CMake, no setuptools).

    python -m patchmatch_gb300.build

Compiles the CUDA densifier for sm_103a into ``_lib/libpm_gb300.so`` (one
translation unit per source-count variant, compiled in parallel) and the host
scene generator into ``_lib/libpm_scene.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(ROOT, "_build", "obj")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INC, "-I" + CSRC] + ARCH
MAX_SOURCES = 10


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _sources():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps += [os.path.join(INC, f) for f in os.listdir(INC)]
    units = []
    for f in ("pm_api.cu", "pm_batch.cu", "pm_prep.cu", "pm_post.cu", "pm_seed.cu", "pm_input.cu", "pm_fuse_noalloc.cu", "pm_dense.cpp", "pm_server.cpp", "pm_views.cpp", "pm_io.cpp"):
        units.append((os.path.join(CSRC, f), os.path.join(OBJ_DIR, os.path.splitext(f)[0] + ".o"), []))
    # the cost/sweep kernels flush subnormals to zero: no value on that path is
    # subnormal, and it keeps the approximate reciprocal/rsqrt/exp2 single
    # instructions (NaN handling is unaffected)
    for k in range(4):  # the batched executor's mixed kernel, one unit per image variant
        units.append((os.path.join(CSRC, "pm_batch_mixed.cu"), os.path.join(OBJ_DIR, f"pm_batch_mixed_k{k}.o"),
                      [f"-DPM_MIXED_KIND={k}", "-ftz=true"]))
    for s in range(1, MAX_SOURCES + 1):
        units.append((os.path.join(CSRC, "pm_inst.cu"), os.path.join(OBJ_DIR, f"pm_inst_s{s}.o"),
                      [f"-DPM_INST_S={s}", "-ftz=true"]))
    return units, deps


def _stale(obj, srcs):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_pm(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    units, deps = _sources()
    todo = [(src, obj, extra) for src, obj, extra in units if force or _stale(obj, [src] + deps)]
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_run, [nvcc] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]) for src, obj, extra in todo]
        for f in futs:
            out = f.result()
            if verbose and out.strip():
                print(out)
    lib = os.path.join(LIB_DIR, "libpm_gb300.so")
    objs = [obj for _, obj, _ in units]
    if force or todo or _stale(lib, objs):
        _run([nvcc, "-shared"] + ARCH + ["-o", lib] + objs)
    return lib


def build_scene(force: bool = False) -> str:
    """Host ray caster (g++/OpenMP) plus its device twin (nvcc), one library."""
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    src = os.path.join(CSRC, "scene.cpp")
    gsrc = os.path.join(CSRC, "scene_gpu.cu")
    lib = os.path.join(LIB_DIR, "libpm_scene.so")
    deps = [src, gsrc, os.path.join(INC, "pm_scene.h")]
    if force or _stale(lib, deps):
        o1 = os.path.join(OBJ_DIR, "scene.o")
        o2 = os.path.join(OBJ_DIR, "scene_gpu.o")
        _run(["g++", "-O2", "-fopenmp", "-fPIC", "-std=c++17", "-I" + INC, "-c", src, "-o", o1])
        _run([_nvcc()] + NVCC_FLAGS + ["-c", gsrc, "-o", o2])
        _run([_nvcc(), "-shared"] + ARCH + ["-o", lib, o1, o2, "-Xcompiler", "-fopenmp"])
    return lib


def build(force: bool = False, verbose: bool = False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_pm, force, None, verbose)
        b = ex.submit(build_scene, force)
        return a.result(), b.result()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
