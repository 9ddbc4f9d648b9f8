"""CPU tests of the C-ABI library: it builds, loads without a GPU, and exports
every function include/pm_gb300.h declares.  No compute calls are made."""
import ctypes
import os
import re

import pytest

from patchmatch_gb300 import _native, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pm_[a-z_0-9]+)\s*\(", txt)))


def test_header_declarations_match_binding_list():
    assert _declared("pm_gb300.h") == sorted(native.EXPORTS)


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(_native.PM_LIB)
    missing = [s for s in _declared("pm_gb300.h") if not hasattr(lib, s)]
    assert not missing, missing


def test_scene_library_exports(built):
    lib = ctypes.CDLL(_native.SCENE_LIB)
    missing = [s for s in _declared("pm_scene.h") if not hasattr(lib, s)]
    assert not missing, missing


def test_params_default_and_status_strings(built):
    p = native.default_params()
    assert (p.patch_half, p.iterations, p.combine, p.seam) == (5, 8, native.COMBINE_FOLD, native.SEAM_CLAMP)
    assert p.sampler == native.SAMPLER_TEXTURE
    assert abs(p.sigma_color - 50) < 1e-6 and abs(p.sigma_x - 5) < 1e-6 and abs(p.min_score - 0.1) < 1e-6
    L = native.lib()
    assert L.pm_status_string(native.PM_EBUDGET).decode() == "HBM budget exceeded"


def test_request_bytes_scales(built):
    L = native.lib()
    a = L.pm_request_bytes(1920, 960, 6, native.IMAGE_U8)
    b = L.pm_request_bytes(1920, 960, 6, native.IMAGE_F16)
    c = L.pm_request_bytes(3840, 1920, 6, native.IMAGE_U8)
    assert b > a and 3.5 * a < c < 4.5 * a


def test_create_without_gpu_reports_error(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(native.PmError):
        native.Context(0)


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    monkeypatch.setattr(_native, "PM_LIB", str(tmp_path / "libpm_gb300.so"))
    monkeypatch.setattr(_native, "_cache", {})
    with pytest.raises(_native.NativeLibraryMissing):
        _native.load_pm_lib()
