"""Locating and loading the in-tree native libraries.

The CUDA densifier (``libpm_gb300.so``) and the host scene generator
(``libpm_scene.so``) are built in-tree into ``patchmatch_gb300/_lib`` by
``patchmatch_gb300.build``.  Loading fails loudly when a library is missing:
there is no pure-Python or CPU fallback for the densifier.
"""
from __future__ import annotations

import ctypes
import os

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
PM_LIB = os.path.join(LIB_DIR, "libpm_gb300.so")
SCENE_LIB = os.path.join(LIB_DIR, "libpm_scene.so")

_cache: dict = {}


class NativeLibraryMissing(RuntimeError):
    pass


def _load(path: str) -> ctypes.CDLL:
    if path in _cache:
        return _cache[path]
    if not os.path.exists(path):
        raise NativeLibraryMissing(
            f"{os.path.basename(path)} is not built ({path}); run "
            "`python -c 'import __graft_entry__ as g; g.build()'` or `python -m patchmatch_gb300.build`")
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    _cache[path] = lib
    return lib


def load_pm_lib() -> ctypes.CDLL:
    return _load(PM_LIB)


def load_scene_lib() -> ctypes.CDLL:
    return _load(SCENE_LIB)
