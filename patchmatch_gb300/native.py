"""ctypes binding of the densifier's C ABI (``include/pm_gb300.h``).

Everything here calls straight into ``libpm_gb300.so``; there is no Python or
CPU implementation of the densifier to fall back to.  Arrays are numpy (host)
buffers unless a raw pointer (int) is passed.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._native import load_pm_lib

PM_OK, PM_EINVAL, PM_ENOMEM, PM_EBUDGET, PM_ETIMEOUT, PM_ECUDA, PM_ENOTREADY, PM_ECANCELLED, PM_ENOTBUILT = range(9)
COMBINE_FOLD, COMBINE_MAX, COMBINE_TOPK, COMBINE_FOLD_SEPARATE = 0, 1, 2, 3
SEAM_CLAMP, SEAM_WRAP, SEAM_ZERO = 0, 1, 2
INIT_LOGUNIFORM_HEMI, INIT_REF_UNIFORM = 0, 1
IMAGE_U8, IMAGE_F16 = 0, 1
SAMPLER_EXACT, SAMPLER_TEXTURE = 0, 1
BATCH_PERSISTENT, BATCH_LAUNCHES, BATCH_STREAMS, BATCH_MIXED = 0, 1, 2, 3
PROPAGATION_SMOOTH, PROPAGATION_PLAIN = 0, 1
ORDER_BGR, ORDER_RGB = 0, 1
MAX_SOURCES = 10

# Every exported symbol declared in include/pm_gb300.h.
EXPORTS = (
    "pm_params_default", "pm_create", "pm_destroy", "pm_last_error", "pm_status_string", "pm_launch_count",
    "pm_stream", "pm_probe_fp32_peak",
    "pm_densify", "pm_request_create", "pm_request_destroy", "pm_request_bytes", "pm_request_set_params",
    "pm_request_set_view", "pm_request_init", "pm_request_set_state", "pm_request_sweep", "pm_request_postprocess",
    "pm_batch_create", "pm_batch_add", "pm_batch_clear", "pm_batch_set_executor", "pm_batch_run",
    "pm_batch_synchronize", "pm_batch_stream", "pm_batch_tune", "pm_batch_destroy",
    "pm_score_view", "pm_depth_interval", "pm_write_ply", "pm_write_dense_msgpack",
    "pm_image_to_gray", "pm_image_resize", "pm_build_pyramid_f16",
    "pm_request_seed", "pm_request_set_prior", "pm_request_set_landmarks", "pm_request_seed_landmarks", "pm_result_bytes", "pm_result_create", "pm_result_snapshot",
    "pm_result_destroy", "pm_request_set_prior_result",
    "pm_request_run", "pm_request_read", "pm_request_read_async", "pm_request_synchronize", "pm_request_query",
    "pm_request_stream", "pm_request_depth_device",
    "pm_score_hypotheses", "pm_filter_consistency", "pm_fuse", "pm_fuse_noalloc",
    "pm_filter_consistency_device", "pm_fuse_workspace_bytes", "pm_fuse_device", "pm_probe_sfu_peak",
    "pm_probe_tex_peak",
    "pm_server_config_default", "pm_server_create", "pm_server_submit", "pm_server_wait", "pm_server_destroy",
    "pm_server_submit_landmarks", "pm_server_wait_dense", "pm_result_depth_device", "pm_server_finish",
)


class Params(C.Structure):
    _fields_ = [("patch_half", C.c_int), ("iterations", C.c_int), ("combine", C.c_int), ("top_k", C.c_int),
                ("seam", C.c_int), ("init_mode", C.c_int), ("image_format", C.c_int), ("postprocess", C.c_int),
                ("min_depth", C.c_float), ("max_depth", C.c_float), ("min_score", C.c_float),
                ("min_patch_sd", C.c_float), ("sigma_color", C.c_float), ("sigma_x", C.c_float),
                ("seed", C.c_uint32), ("keyframe_id", C.c_uint32), ("sampler", C.c_int), ("propagation", C.c_int)]


class View(C.Structure):
    _fields_ = [("gray", C.c_void_p), ("pitch_bytes", C.c_size_t), ("mask", C.c_void_p),
                ("R_cw", C.c_double * 9), ("t_cw", C.c_double * 3)]


class Maps(C.Structure):
    _fields_ = [("depth", C.c_void_p), ("score", C.c_void_p), ("plane", C.c_void_p), ("normal", C.c_void_p),
                ("best_view", C.c_void_p)]


class Points(C.Structure):
    _fields_ = [("capacity", C.c_int), ("count", C.c_int), ("xyz", C.c_void_p), ("bgr", C.c_void_p),
                ("ij", C.c_void_p)]


class ServerConfig(C.Structure):
    _fields_ = [("params", Params), ("cache_capacity", C.c_int), ("max_inflight", C.c_int),
                ("min_sources", C.c_int), ("max_sources", C.c_int), ("min_baseline", C.c_float),
                ("max_baseline", C.c_float), ("seed_from_prior", C.c_int), ("seeded_iterations", C.c_int),
                ("prior_lag", C.c_int), ("poll_us", C.c_int), ("coarse_to_fine", C.c_int),
                ("dense_output", C.c_int), ("clean_threshold", C.c_float), ("clean_min_views", C.c_int),
                ("clean_reproj_px", C.c_float), ("fuse_threshold", C.c_float), ("min_view_score", C.c_float)]


class BatchTuning(C.Structure):
    _fields_ = [("executor", C.c_int), ("grid_mult", C.c_int), ("ms", C.c_float), ("candidate_ms", C.c_float * 5)]


class ServedInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("n_sources", C.c_int), ("seeded", C.c_int), ("iterations", C.c_int),
                ("queue_ms", C.c_double), ("latency_ms", C.c_double), ("view_score", C.c_float)]


_vp, _sz = C.c_void_p, C.c_size_t


def lib():
    L = load_pm_lib()
    if getattr(L, "_pm_typed", False):
        return L
    L.pm_params_default.argtypes = [C.POINTER(Params)]
    L.pm_create.argtypes = [C.c_int, _sz, C.POINTER(_vp)]
    L.pm_destroy.argtypes = [_vp]
    L.pm_last_error.restype = C.c_char_p
    L.pm_last_error.argtypes = [_vp]
    L.pm_status_string.restype = C.c_char_p
    L.pm_status_string.argtypes = [C.c_int]
    L.pm_launch_count.restype = C.c_uint64
    L.pm_launch_count.argtypes = [_vp]
    L.pm_stream.restype = _vp
    L.pm_stream.argtypes = [_vp]
    L.pm_probe_fp32_peak.argtypes = [_vp, C.POINTER(C.c_double)]
    L.pm_probe_sfu_peak.argtypes = [_vp, C.POINTER(C.c_double)]
    L.pm_probe_tex_peak.argtypes = [_vp, C.POINTER(C.c_double)]
    L.pm_densify.argtypes = [_vp, C.c_int, C.c_int, C.POINTER(View), C.c_int, C.POINTER(Params), C.POINTER(Maps)]
    L.pm_request_create.argtypes = [_vp, C.c_int, C.c_int, C.c_int, C.POINTER(Params), C.POINTER(_vp)]
    L.pm_request_destroy.argtypes = [_vp]
    L.pm_request_bytes.restype = _sz
    L.pm_request_bytes.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
    L.pm_request_set_params.argtypes = [_vp, C.POINTER(Params)]
    L.pm_request_set_view.argtypes = [_vp, C.c_int, C.POINTER(View)]
    L.pm_request_init.argtypes = [_vp]
    L.pm_request_set_state.argtypes = [_vp, _vp, _vp]
    L.pm_request_sweep.argtypes = [_vp, C.c_int, C.c_int]
    L.pm_request_seed.argtypes = [_vp, _vp]
    L.pm_request_set_landmarks.argtypes = [_vp, _vp, C.c_int]
    L.pm_request_seed_landmarks.argtypes = [_vp, _vp, C.c_int]
    L.pm_result_bytes.restype = _sz
    L.pm_result_bytes.argtypes = [C.c_int, C.c_int]
    L.pm_result_create.argtypes = [_vp, C.c_int, C.c_int, C.POINTER(_vp)]
    L.pm_result_snapshot.argtypes = [_vp, _vp]
    L.pm_result_destroy.argtypes = [_vp]
    L.pm_request_set_prior_result.argtypes = [_vp, _vp]
    L.pm_request_set_prior.argtypes = [_vp, _vp]
    L.pm_request_postprocess.argtypes = [_vp]
    L.pm_request_run.argtypes = [_vp]
    L.pm_request_read.argtypes = [_vp, C.POINTER(Maps), C.c_int]
    L.pm_request_synchronize.argtypes = [_vp]
    L.pm_request_read_async.argtypes = [_vp, C.POINTER(Maps), C.c_int]
    L.pm_request_query.argtypes = [_vp]
    L.pm_request_stream.restype = _vp
    L.pm_request_stream.argtypes = [_vp]
    L.pm_request_depth_device.restype = _vp
    L.pm_request_depth_device.argtypes = [_vp]
    L.pm_score_hypotheses.argtypes = [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp]
    L.pm_filter_consistency.argtypes = [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, C.c_float,
                                        C.c_int, C.c_float, _vp]
    L.pm_fuse.argtypes = [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, C.c_float, _vp, C.POINTER(Points)]
    L.pm_fuse_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, C.c_float, _vp, _vp, _vp, _vp, _vp,
                                  _vp]
    L.pm_filter_consistency_device.argtypes = [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, C.c_float,
                                               C.c_int, C.c_float, _vp, _vp]
    L.pm_fuse_workspace_bytes.restype = C.c_size_t
    L.pm_fuse_workspace_bytes.argtypes = [C.c_int, C.c_int]
    L.pm_fuse_device.argtypes = [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, C.c_float, _vp, _vp, _vp, _vp,
                                 _vp, _vp, C.c_size_t, _vp]
    L.pm_batch_create.argtypes = [_vp, C.POINTER(_vp)]
    for f in ("pm_batch_clear", "pm_batch_run", "pm_batch_synchronize", "pm_batch_destroy"):
        getattr(L, f).argtypes = [_vp]
    L.pm_batch_add.argtypes = [_vp, _vp]
    L.pm_batch_set_executor.argtypes = [_vp, C.c_int, C.c_int]
    L.pm_batch_stream.restype = _vp
    L.pm_batch_stream.argtypes = [_vp]
    L.pm_batch_tune.argtypes = [_vp, C.POINTER(BatchTuning)]
    L.pm_score_view.argtypes = [_vp, _vp, _vp, C.c_int, _vp, _vp, C.c_int, C.POINTER(C.c_float),
                                C.POINTER(C.c_int)]
    L.pm_depth_interval.argtypes = [_vp, _vp, _vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.pm_image_to_gray.argtypes = [_vp, _vp, C.c_int, C.c_int, _sz, C.c_int, C.c_int, _vp, _sz]
    L.pm_image_resize.argtypes = [_vp, _vp, C.c_int, C.c_int, _sz, C.c_int, _vp, C.c_int, C.c_int, _sz]
    L.pm_build_pyramid_f16.argtypes = [_vp, _vp, C.c_int, C.c_int, _sz, C.c_int, C.c_int, _vp]
    L.pm_write_ply.argtypes = [C.c_char_p, C.POINTER(Points)]
    L.pm_write_dense_msgpack.argtypes = [C.c_char_p, C.POINTER(Points), C.c_uint64, C.c_uint32]
    L.pm_server_config_default.argtypes = [C.POINTER(ServerConfig)]
    L.pm_server_create.argtypes = [_vp, C.POINTER(ServerConfig), C.POINTER(_vp)]
    L.pm_server_submit.argtypes = [_vp, C.c_int, C.c_int, C.POINTER(View), C.POINTER(C.c_uint64)]
    L.pm_server_wait.argtypes = [_vp, C.c_uint64, C.c_int, C.POINTER(Maps), C.POINTER(ServedInfo)]
    L.pm_server_submit_landmarks.argtypes = [_vp, C.c_int, C.c_int, C.POINTER(View), _vp, _vp, C.c_int,
                                             C.POINTER(C.c_uint64)]
    L.pm_server_wait_dense.argtypes = [_vp, C.c_uint64, C.c_int, _vp, C.POINTER(Points)]
    L.pm_server_finish.argtypes = [_vp]
    L.pm_result_depth_device.restype = _vp
    L.pm_result_depth_device.argtypes = [_vp]
    L.pm_server_destroy.argtypes = [_vp]
    L._pm_typed = True
    return L


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
        return a.ctypes.data
    if hasattr(a, "data_ptr"):  # torch tensor
        return a.data_ptr()
    raise TypeError(type(a))


class PmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


def default_params(**kw) -> Params:
    p = Params()
    lib().pm_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def make_view(gray, R, t, mask=None, pitch_bytes: int = 0) -> View:
    v = View()
    v.gray = _ptr(gray)
    v.pitch_bytes = pitch_bytes
    v.mask = _ptr(mask)
    R = np.asarray(R, np.float64).reshape(9)
    t = np.asarray(t, np.float64).reshape(3)
    for a in range(9):
        v.R_cw[a] = R[a]
    for a in range(3):
        v.t_cw[a] = t[a]
    return v


def score_view(prev_center, cur_center, prev_ids, cur_ids, cur_xyz):
    """pm_score_view: (score, n_common)."""
    pc = np.ascontiguousarray(prev_center, np.float64)
    cc = np.ascontiguousarray(cur_center, np.float64)
    pi = np.ascontiguousarray(prev_ids, np.uint64)
    ci = np.ascontiguousarray(cur_ids, np.uint64)
    cx = np.ascontiguousarray(cur_xyz, np.float64).reshape(-1, 3)
    if cx.shape[0] != len(ci):
        raise ValueError("cur_ids and cur_xyz differ in length")
    sc, nc = C.c_float(), C.c_int()
    rc = lib().pm_score_view(_ptr(pc), _ptr(cc), _ptr(pi), len(pi), _ptr(ci), _ptr(cx), len(ci), C.byref(sc),
                             C.byref(nc))
    if rc != PM_OK:
        raise PmError(rc, "pm_score_view failed")
    return sc.value, nc.value


def _points(xyz, bgr):
    xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
    bgr = None if bgr is None else np.ascontiguousarray(bgr, np.uint8).reshape(-1, 3)
    if bgr is not None and bgr.shape[0] != xyz.shape[0]:
        raise ValueError("xyz and bgr differ in length")
    n = xyz.shape[0]
    return Points(n, n, xyz.ctypes.data if n else None, bgr.ctypes.data if (bgr is not None and n) else None,
                  None), (xyz, bgr)


def write_ply(path, xyz, bgr=None):
    """pm_write_ply: ASCII PLY of points (n x 3 FP64) and colours (n x 3 u8)."""
    pts, keep = _points(xyz, bgr)
    rc = lib().pm_write_ply(str(path).encode(), C.byref(pts))
    if rc != PM_OK:
        raise PmError(rc, f"pm_write_ply failed for {path}")


def write_dense_msgpack(path, xyz, bgr=None, first_id: int = 0, keyframe_id: int = 0):
    """pm_write_dense_msgpack: the dense map message of the points."""
    pts, keep = _points(xyz, bgr)
    rc = lib().pm_write_dense_msgpack(str(path).encode(), C.byref(pts), first_id, keyframe_id)
    if rc != PM_OK:
        raise PmError(rc, f"pm_write_dense_msgpack failed for {path}")


def depth_interval(R_cw, t_cw, xyz):
    """pm_depth_interval: (p10, p90, min_depth, max_depth)."""
    R = np.ascontiguousarray(R_cw, np.float64)
    t = np.ascontiguousarray(t_cw, np.float64)
    x = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
    out = [C.c_double() for _ in range(4)]
    rc = lib().pm_depth_interval(_ptr(R), _ptr(t), _ptr(x), x.shape[0], *[C.byref(o) for o in out])
    if rc != PM_OK:
        raise PmError(rc, "pm_depth_interval failed")
    return tuple(o.value for o in out)


class Context:
    """One CUDA stream + device buffers on one GPU (pm_ctx)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._L = lib()
        h = C.c_void_p()
        rc = self._L.pm_create(device, hbm_budget, C.byref(h))
        if rc != PM_OK:
            raise PmError(rc, f"pm_create failed: {self._L.pm_status_string(rc).decode()}")
        self.h = h.value

    def close(self):
        # pm_destroy refuses while requests, results or batches are alive; the
        # handle is then kept (their finalisers still need the context)
        if getattr(self, "h", None) and self._L.pm_destroy(self.h) == PM_OK:
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def check(self, rc: int):
        if rc != PM_OK:
            raise PmError(rc, self._L.pm_last_error(self.h).decode())

    @property
    def launches(self) -> int:
        return int(self._L.pm_launch_count(self.h))

    @property
    def stream_handle(self) -> int:
        """cudaStream_t of the context (for torch.cuda.ExternalStream)."""
        return int(self._L.pm_stream(self.h))

    # ---- input preparation (torch CUDA tensors in and out) ----
    def to_gray(self, img, order: int = 0):
        """(H, W, C) or (H, W) uint8 CUDA tensor -> (H, W) uint8 CUDA tensor."""
        import torch
        img = img.contiguous()
        H, W = img.shape[:2]
        ch = 1 if img.dim() == 2 else img.shape[2]
        out = torch.empty((H, W), dtype=torch.uint8, device=img.device)
        self.check(self._L.pm_image_to_gray(self.h, img.data_ptr(), W, H, W * ch, ch, order, out.data_ptr(), W))
        return out

    def resize(self, img, W: int, H: int):
        """Bilinear resize of a (h, w[, C]) uint8 CUDA tensor to (H, W[, C])."""
        import torch
        img = img.contiguous()
        h, w = img.shape[:2]
        ch = 1 if img.dim() == 2 else img.shape[2]
        out = torch.empty((H, W) + (() if img.dim() == 2 else (ch,)), dtype=torch.uint8, device=img.device)
        self.check(self._L.pm_image_resize(self.h, img.data_ptr(), w, h, w * ch, ch, out.data_ptr(), W, H, W * ch))
        return out

    def pyramid_f16(self, img, levels: int = 3):
        """FP16 pyramid of a (H, W) uint8 or float16 CUDA tensor: list of float16 tensors."""
        import torch
        img = img.contiguous()
        H, W = img.shape
        f16 = img.dtype == torch.float16
        outs, w, h = [], W, H
        for _ in range(levels):
            outs.append(torch.empty((h, w), dtype=torch.float16, device=img.device))
            w, h = (w + 1) // 2, (h + 1) // 2
        arr = (C.c_void_p * levels)(*[o.data_ptr() for o in outs])
        self.check(self._L.pm_build_pyramid_f16(self.h, img.data_ptr(), W, H, W * (2 if f16 else 1),
                                                IMAGE_F16 if f16 else IMAGE_U8, levels, arr))
        return outs

    def probe_fp32_peak(self) -> float:
        v = C.c_double()
        self.check(self._L.pm_probe_fp32_peak(self.h, C.byref(v)))
        return v.value

    def probe_sfu_peak(self) -> float:
        """Measured special-function (approximate reciprocal) throughput, Gop/s."""
        v = C.c_double()
        self.check(self._L.pm_probe_sfu_peak(self.h, C.byref(v)))
        return v.value

    def probe_tex_peak(self) -> float:
        """Measured bilinear texture-fetch throughput (L1-resident u8), Gfetch/s."""
        v = C.c_double()
        self.check(self._L.pm_probe_tex_peak(self.h, C.byref(v)))
        return v.value

    def last_error(self) -> str:
        return self._L.pm_last_error(self.h).decode()

    # ---- one-shot ----
    def densify(self, images, R, t, params: Params | None = None, mask=None, want=("depth", "score", "normal")):
        """images: list of (H, W) uint8 / float16 arrays, view 0 = reference."""
        params = params or default_params()
        H, W = images[0].shape
        views = (View * len(images))(*[make_view(np.ascontiguousarray(im), R[k], t[k], mask if k == 0 else None)
                                       for k, im in enumerate(images)])
        out, maps = _alloc_maps(H, W, want)
        self.check(self._L.pm_densify(self.h, W, H, views, len(images), C.byref(params), C.byref(maps)))
        return out

    def request(self, W: int, H: int, n_sources: int, params: Params | None = None) -> "Request":
        return Request(self, W, H, n_sources, params or default_params())

    # ---- filter / fuse ----
    def filter_consistency(self, depths, R, t, center: int, thr: float, min_consistent: int = 3,
                           reproj_px: float = 0.0):
        depths = [np.ascontiguousarray(d, np.float32) for d in depths]
        H, W = depths[0].shape
        arr = (C.c_void_p * len(depths))(*[d.ctypes.data for d in depths])
        R = np.ascontiguousarray(R, np.float64)
        t = np.ascontiguousarray(t, np.float64)
        out = np.zeros((H, W), np.float32)
        self.check(self._L.pm_filter_consistency(self.h, W, H, len(depths), C.cast(arr, C.c_void_p), _ptr(R),
                                                 _ptr(t), center, thr, min_consistent, reproj_px, _ptr(out)))
        return out

    def fuse(self, depths, R, t, bgr, thr: float):
        """Returns (pruned, xyz[n,3] f64, bgr[n,3] u8, ij[n,2] i32, mutated depths)."""
        depths = [np.ascontiguousarray(d, np.float32).copy() for d in depths]
        H, W = depths[0].shape
        arr = (C.c_void_p * len(depths))(*[d.ctypes.data for d in depths])
        R = np.ascontiguousarray(R, np.float64)
        t = np.ascontiguousarray(t, np.float64)
        pruned = np.zeros((H, W), np.float32)
        cap = H * W
        xyz = np.zeros((cap, 3), np.float64)
        cols = np.zeros((cap, 3), np.uint8)
        ij = np.zeros((cap, 2), np.int32)
        pts = Points(cap, 0, xyz.ctypes.data, cols.ctypes.data, ij.ctypes.data)
        bgr = None if bgr is None else np.ascontiguousarray(bgr, np.uint8)
        self.check(self._L.pm_fuse(self.h, W, H, len(depths), C.cast(arr, C.c_void_p), _ptr(R), _ptr(t), _ptr(bgr),
                                   thr, _ptr(pruned), C.byref(pts)))
        n = pts.count
        return pruned, xyz[:n], cols[:n], ij[:n], depths


    def filter_consistency_device(self, depth_ptrs, W: int, H: int, R, t, center: int, thr: float, out_ptr: int,
                                  min_consistent: int = 3, reproj_px: float = 0.0, stream: int = 0):
        """pm_filter_consistency_device: device pointers in and out, enqueued on `stream` (0: the context's)."""
        arr = (C.c_void_p * len(depth_ptrs))(*depth_ptrs)
        R = np.ascontiguousarray(R, np.float64)
        t = np.ascontiguousarray(t, np.float64)
        self.check(self._L.pm_filter_consistency_device(self.h, W, H, len(depth_ptrs), C.cast(arr, C.c_void_p),
                                                        _ptr(R), _ptr(t), center, thr, min_consistent, reproj_px,
                                                        out_ptr, stream or None))

    def fuse_device(self, depth_ptrs, W: int, H: int, R, t, thr: float, pruned_ptr: int, xyz_ptr: int, count_ptr: int,
                    workspace_ptr: int, workspace_bytes: int, bgr_ptr: int = 0, bgr_out_ptr: int = 0, ij_ptr: int = 0,
                    stream: int = 0):
        """pm_fuse_device: device pointers in and out, enqueued on `stream` (0: the context's)."""
        arr = (C.c_void_p * len(depth_ptrs))(*depth_ptrs)
        R = np.ascontiguousarray(R, np.float64)
        t = np.ascontiguousarray(t, np.float64)
        self.check(self._L.pm_fuse_device(self.h, W, H, len(depth_ptrs), C.cast(arr, C.c_void_p), _ptr(R), _ptr(t),
                                          bgr_ptr or None, thr, pruned_ptr, xyz_ptr, bgr_out_ptr or None,
                                          ij_ptr or None, count_ptr, workspace_ptr, workspace_bytes, stream or None))


def fuse_workspace_bytes(W: int, H: int) -> int:
    return int(lib().pm_fuse_workspace_bytes(W, H))


def _alloc_maps(H, W, want):
    out = {}
    maps = Maps()
    for name in want:
        if name in ("depth", "score"):
            a = np.zeros((H, W), np.float32)
        elif name in ("plane", "normal"):
            a = np.zeros((H, W, 3), np.float32)
        elif name == "best_view":
            a = np.zeros((H, W), np.int32)
        else:
            raise KeyError(name)
        out[name] = a
        setattr(maps, name, a.ctypes.data)
    if "depth" not in out:
        a = np.zeros((H, W), np.float32)
        out["depth"] = a
        maps.depth = a.ctypes.data
    return out, maps


class Request:
    """Device-resident state of one keyframe (pm_request)."""

    def __init__(self, ctx: Context, W: int, H: int, n_sources: int, params: Params):
        self.ctx, self.W, self.H, self.S = ctx, W, H, n_sources
        self._L = ctx._L
        self.params = params
        h = C.c_void_p()
        ctx.check(self._L.pm_request_create(ctx.h, W, H, n_sources, C.byref(params), C.byref(h)))
        self.h = h.value
        self._keep = {}

    def close(self):
        if getattr(self, "h", None):
            # fails (and keeps the request) while a batch still holds it
            self.ctx.check(self._L.pm_request_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params: Params):
        self.params = params
        self.ctx.check(self._L.pm_request_set_params(self.h, C.byref(params)))

    def set_view(self, k: int, gray, R, t, mask=None, pitch_bytes: int = 0):
        if isinstance(gray, np.ndarray):
            gray = np.ascontiguousarray(gray)
            self._keep[k] = (gray, mask)
        v = make_view(gray, R, t, mask, pitch_bytes)
        self.ctx.check(self._L.pm_request_set_view(self.h, k, C.byref(v)))

    def set_views(self, images, R, t, mask=None):
        for k, im in enumerate(images):
            self.set_view(k, im, R[k], t[k], mask if k == 0 else None)

    def init(self):
        self.ctx.check(self._L.pm_request_init(self.h))

    def set_state(self, planes, scores=None):
        planes = np.ascontiguousarray(planes, np.float32)
        scores = None if scores is None else np.ascontiguousarray(scores, np.float32)
        self.ctx.check(self._L.pm_request_set_state(self.h, _ptr(planes), _ptr(scores)))

    def sweep(self, first_half: int, n_half: int):
        self.ctx.check(self._L.pm_request_sweep(self.h, first_half, n_half))

    def seed(self, prior: "Request"):
        self.ctx.check(self._L.pm_request_seed(self.h, prior.h))

    def set_landmarks(self, xyz_world):
        """Stage SLAM landmarks (n x 3 world points) for seeding in run()."""
        xyz = np.ascontiguousarray(xyz_world, np.float64).reshape(-1, 3)
        self.ctx.check(self._L.pm_request_set_landmarks(self.h, _ptr(xyz), xyz.shape[0]))

    def seed_landmarks(self, xyz_world):
        """Seed the current state from SLAM landmarks now."""
        xyz = np.ascontiguousarray(xyz_world, np.float64).reshape(-1, 3)
        self.ctx.check(self._L.pm_request_seed_landmarks(self.h, _ptr(xyz), xyz.shape[0]))

    def set_prior(self, prior: "Request | Result | None"):
        self._prior = prior  # keep it alive
        if isinstance(prior, Result):
            self.ctx.check(self._L.pm_request_set_prior_result(self.h, prior.h))
        else:
            self.ctx.check(self._L.pm_request_set_prior(self.h, prior.h if prior is not None else None))

    def postprocess(self):
        self.ctx.check(self._L.pm_request_postprocess(self.h))

    def run(self):
        self.ctx.check(self._L.pm_request_run(self.h))

    def synchronize(self):
        self.ctx.check(self._L.pm_request_synchronize(self.h))

    @property
    def stream_handle(self) -> int:
        """cudaStream_t of the request (for torch.cuda.ExternalStream)."""
        return int(self._L.pm_request_stream(self.h))

    @property
    def depth_device_ptr(self) -> int:
        """Device address of the request's filtered depth map (H x W floats)."""
        return int(self._L.pm_request_depth_device(self.h))

    def done(self) -> bool:
        rc = self._L.pm_request_query(self.h)
        if rc == PM_ENOTREADY:
            return False
        self.ctx.check(rc)
        return True

    def read(self, raw: bool = False, want=("depth", "score", "plane", "normal", "best_view")):
        out, maps = _alloc_maps(self.H, self.W, want)
        self.ctx.check(self._L.pm_request_read(self.h, C.byref(maps), 1 if raw else 0))
        return out

    def score_hypotheses(self, ij, planes, per_source: bool = False):
        ij = np.ascontiguousarray(ij, np.int32)
        planes = np.ascontiguousarray(planes, np.float32)
        n = ij.shape[0]
        scores = np.zeros(n, np.float32)
        best = np.zeros(n, np.int32)
        ps = np.zeros((n, self.S), np.float32) if per_source else None
        self.ctx.check(self._L.pm_score_hypotheses(self.h, n, _ptr(ij), _ptr(planes), _ptr(scores), _ptr(best),
                                                   _ptr(ps)))
        return (scores, best, ps) if per_source else (scores, best)


class Result:
    """A retained keyframe result (pm_result): plane state + filtered depth + pose."""

    def __init__(self, ctx: Context, W: int, H: int):
        self.ctx, self.W, self.H = ctx, W, H
        self._L = ctx._L
        h = C.c_void_p()
        ctx.check(self._L.pm_result_create(ctx.h, W, H, C.byref(h)))
        self.h = h.value

    def snapshot(self, req: Request):
        self.ctx.check(self._L.pm_result_snapshot(self.h, req.h))

    def close(self):
        if getattr(self, "h", None):
            self._L.pm_result_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """The batched executor (pm_batch) over requests of one context."""

    def __init__(self, ctx: Context, requests=()):
        self.ctx = ctx
        self._L = ctx._L
        h = C.c_void_p()
        ctx.check(self._L.pm_batch_create(ctx.h, C.byref(h)))
        self.h = h.value
        self.requests = []
        for r in requests:
            self.add(r)

    def add(self, req: "Request"):
        self.ctx.check(self._L.pm_batch_add(self.h, req.h))
        self.requests.append(req)

    def clear(self):
        self.ctx.check(self._L.pm_batch_clear(self.h))
        self.requests = []

    def set_executor(self, executor: int, grid_mult: int = 1):
        self.ctx.check(self._L.pm_batch_set_executor(self.h, executor, grid_mult))

    def run(self):
        self.ctx.check(self._L.pm_batch_run(self.h))

    def synchronize(self):
        self.ctx.check(self._L.pm_batch_synchronize(self.h))

    @property
    def stream_handle(self) -> int:
        return int(self._L.pm_batch_stream(self.h))

    def tune(self) -> dict:
        t = BatchTuning()
        self.ctx.check(self._L.pm_batch_tune(self.h, C.byref(t)))
        return {"executor": t.executor, "grid_mult": t.grid_mult, "ms": t.ms,
                "candidate_ms": list(t.candidate_ms)}

    def close(self):
        if getattr(self, "h", None):
            self._L.pm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def server_config(**kw) -> ServerConfig:
    """Defaults of pm_server_config_default; keyword overrides, params=... for pm_params."""
    c = ServerConfig()
    lib().pm_server_config_default(C.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise AttributeError(k)
        setattr(c, k, v)
    return c


class Server:
    """The served request loop (pm_server) on one context."""

    def __init__(self, ctx: Context, cfg: ServerConfig | None = None):
        self.ctx = ctx
        self._L = ctx._L
        self.cfg = cfg or server_config()
        h = C.c_void_p()
        rc = self._L.pm_server_create(ctx.h, C.byref(self.cfg), C.byref(h))
        if rc != PM_OK:
            raise PmError(rc, "pm_server_create failed")
        self.h = h.value
        self.shape = {}
        self.dense_shape = {}

    def submit(self, gray, R, t) -> int:
        gray = np.ascontiguousarray(gray, np.uint8)
        H, W = gray.shape
        v = make_view(gray, R, t)
        tk = C.c_uint64()
        rc = self._L.pm_server_submit(self.h, W, H, C.byref(v), C.byref(tk))
        if rc != PM_OK:
            raise PmError(rc, "pm_server_submit failed")
        self.shape[tk.value] = (H, W)
        self.dense_shape[tk.value] = (H, W)
        return tk.value

    def submit_landmarks(self, gray, R, t, xyz, ids) -> int:
        """pm_server_submit_landmarks: the keyframe with its SLAM landmarks (world xyz, ids)."""
        gray = np.ascontiguousarray(gray, np.uint8)
        H, W = gray.shape
        v = make_view(gray, R, t)
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        ids = np.ascontiguousarray(ids, np.uint64)
        if len(ids) != len(xyz):
            raise ValueError("xyz and ids differ in length")
        tk = C.c_uint64()
        rc = self._L.pm_server_submit_landmarks(self.h, W, H, C.byref(v), _ptr(xyz), _ptr(ids), len(ids),
                                                C.byref(tk))
        if rc != PM_OK:
            raise PmError(rc, "pm_server_submit_landmarks failed")
        self.shape[tk.value] = (H, W)
        self.dense_shape[tk.value] = (H, W)
        return tk.value

    def wait_dense(self, ticket: int, timeout_ms: int = -1):
        """pm_server_wait_dense: (status, fused depth or None, xyz[n,3] f64 or None, ij[n,2] or None)."""
        H, W = self.dense_shape[ticket]
        depth = np.zeros((H, W), np.float32)
        cap = H * W
        xyz = np.zeros((cap, 3), np.float64)
        ij = np.zeros((cap, 2), np.int32)
        pts = Points(cap, 0, xyz.ctypes.data, None, ij.ctypes.data)
        rc = self._L.pm_server_wait_dense(self.h, ticket, timeout_ms, depth.ctypes.data, C.byref(pts))
        if rc != PM_ETIMEOUT:
            self.dense_shape.pop(ticket, None)
        if rc != PM_OK:
            return rc, None, None, None
        n = pts.count
        return rc, depth, xyz[:n], ij[:n]

    def wait(self, ticket: int, timeout_ms: int = -1, want_score: bool = False):
        """Returns (status, depth or None, score or None, info dict)."""
        H, W = self.shape[ticket]
        depth = np.zeros((H, W), np.float32)
        score = np.zeros((H, W), np.float32) if want_score else None
        m = Maps()
        m.depth = depth.ctypes.data
        m.score = score.ctypes.data if want_score else None
        info = ServedInfo()
        rc = self._L.pm_server_wait(self.h, ticket, timeout_ms, C.byref(m), C.byref(info))
        if rc != PM_ETIMEOUT:  # collected (or rejected): the ticket is gone
            self.shape.pop(ticket, None)
        d = {k: getattr(info, k) for k, _ in ServedInfo._fields_}
        ok = rc == PM_OK
        return rc, (depth if ok else None), (score if ok else None), d

    def finish(self):
        """pm_server_finish: end of stream, every result completes and stays collectable."""
        rc = self._L.pm_server_finish(self.h)
        if rc != PM_OK:
            raise PmError(rc, "pm_server_finish failed")

    def close(self):
        if getattr(self, "h", None):
            self._L.pm_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
