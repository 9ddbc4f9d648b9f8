"""ctypes bindings of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arm of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")

OR_MAX_VIEWS = 17
COMBINE_FOLD, COMBINE_MAX, COMBINE_TOPK, COMBINE_FOLD_SEPARATE = 0, 1, 2, 3
SEAM_CLAMP, SEAM_WRAP, SEAM_ZERO = 0, 1, 2
ARITH_F64, ARITH_F32_REF = 0, 1
INTERP_EXACT, INTERP_TEX8_RN, INTERP_TEX8_RZ = 0, 1, 2
PROP_SMOOTH, PROP_PLAIN = 0, 1
INIT_LOGUNIFORM_HEMI, INIT_REF_UNIFORM = 0, 1


def build(force: bool = False) -> str:
    """Compile liboracle.so with gcc (OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "pm_oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "pm_oracle.h"))):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
                               "-o", LIB, src, "-lm"])
    return LIB


class ORViews(C.Structure):
    _fields_ = [("W", C.c_int), ("H", C.c_int), ("n_src", C.c_int),
                ("ref", C.POINTER(C.c_float)),
                ("src", C.POINTER(C.c_float) * (OR_MAX_VIEWS - 1)),
                ("R", (C.c_double * 9) * OR_MAX_VIEWS),
                ("t", (C.c_double * 3) * OR_MAX_VIEWS)]


class ORCostParams(C.Structure):
    _fields_ = [("patch_half", C.c_int), ("combine", C.c_int), ("top_k", C.c_int), ("seam", C.c_int),
                ("arith", C.c_int), ("interp", C.c_int), ("sigma_color", C.c_float),
                ("sigma_x", C.c_float)]


class ORRunParams(C.Structure):
    _fields_ = [("cp", ORCostParams), ("iterations", C.c_int), ("min_depth", C.c_float),
                ("max_depth", C.c_float), ("seed", C.c_uint32), ("keyframe", C.c_uint32),
                ("init_mode", C.c_int), ("row_lo", C.c_int), ("row_hi", C.c_int), ("threads", C.c_int),
                ("propagation", C.c_int)]


_lib = None
_fp, _dp, _ip, _u8p = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint8)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.or_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.or_refine_normals.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _fp]
        L.or_bearing64.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp]
        L.or_bearing_ref_f32.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _fp]
        L.or_cost.restype = C.c_double
        L.or_cost.argtypes = [C.POINTER(ORViews), C.POINTER(ORCostParams), C.c_int, C.c_int, _dp, _dp,
                              C.POINTER(C.c_int)]
        L.or_cost_batch.argtypes = [C.POINTER(ORViews), C.POINTER(ORCostParams), C.c_int, _ip, _fp, _dp, _ip,
                                    _dp, C.c_int]
        L.or_patchmatch.restype = C.c_double
        L.or_patchmatch.argtypes = [C.POINTER(ORViews), C.POINTER(ORRunParams), _fp, _fp, _fp, _ip]
        L.or_sweeps.argtypes = [C.POINTER(ORViews), C.POINTER(ORRunParams), _fp, _fp, _fp, _ip, C.c_int, C.c_int]
        L.or_postprocess.argtypes = [C.c_int, C.c_int, C.c_int, _fp, _u8p, C.c_float, C.c_float, C.c_float,
                                     C.c_float, _fp, _fp]
        L.or_warp_prior.argtypes = [C.c_int, C.c_int, _fp, _fp, _dp, _dp, C.c_int, C.c_int, _dp, _dp, _fp]
        L.or_median3.argtypes = [C.c_int, C.c_int, _fp, _fp]
        L.or_clean.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(_fp), _dp, _dp, C.c_int, C.c_float,
                               C.c_int, C.c_float, _fp]
        L.or_prune.restype = C.c_int
        L.or_prune.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(_fp), _dp, _dp, _u8p, C.c_float, _fp,
                               _dp, _u8p, _ip]
        _lib = L
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


class Views:
    """Holds the float images alive while the oracle reads them."""

    def __init__(self, ref, srcs, R, t):
        self.ref = np.ascontiguousarray(ref, np.float32)
        self.srcs = [np.ascontiguousarray(s, np.float32) for s in srcs]
        H, W = self.ref.shape
        self.s = ORViews()
        self.s.W, self.s.H, self.s.n_src = W, H, len(self.srcs)
        self.s.ref = _p(self.ref, _fp)
        for k, s in enumerate(self.srcs):
            self.s.src[k] = _p(s, _fp)
        R = np.asarray(R, np.float64).reshape(-1, 9)
        t = np.asarray(t, np.float64).reshape(-1, 3)
        for k in range(len(self.srcs) + 1):
            for a in range(9):
                self.s.R[k][a] = R[k, a]
            for a in range(3):
                self.s.t[k][a] = t[k, a]

    @classmethod
    def from_request(cls, req, use_u8: bool = True):
        imgs = [v.gray_u8.astype(np.float32) if use_u8 else v.gray for v in req.views]
        return cls(imgs[0], imgs[1:], req.R, req.t)


def cost_params(patch_half=5, combine=COMBINE_FOLD, top_k=3, seam=SEAM_CLAMP, arith=ARITH_F64,
                interp=INTERP_EXACT, sigma_color=50.0, sigma_x=5.0):
    return ORCostParams(patch_half, combine, top_k, seam, arith, interp, sigma_color, sigma_x)


def cost_batch(views: Views, cp: ORCostParams, ij, planes, threads: int = 0, want_ncc: bool = False):
    ij = np.ascontiguousarray(ij, np.int32)
    planes = np.ascontiguousarray(planes, np.float32)
    n = ij.shape[0]
    scores = np.empty(n, np.float64)
    best = np.empty(n, np.int32)
    ncc = np.empty((n, views.s.n_src), np.float64) if want_ncc else None
    lib().or_cost_batch(C.byref(views.s), C.byref(cp), n, _p(ij, _ip), _p(planes, _fp), _p(scores, _dp),
                        _p(best, _ip), _p(ncc, _dp), threads)
    return (scores, best, ncc) if want_ncc else (scores, best)


def patchmatch(views: Views, cp: ORCostParams, iterations=8, min_depth=0.3, max_depth=20.0, seed=0,
               keyframe=0, init_mode=INIT_LOGUNIFORM_HEMI, row_lo=-1, row_hi=-1, threads=0, propagation=0):
    H, W = views.ref.shape
    rp = ORRunParams(cp, iterations, min_depth, max_depth, seed, keyframe, init_mode, row_lo, row_hi, threads,
                     propagation)
    plane = np.zeros((H, W, 3), np.float32)
    depth = np.zeros((H, W), np.float32)
    score = np.zeros((H, W), np.float32)
    best = np.zeros((H, W), np.int32)
    secs = lib().or_patchmatch(C.byref(views.s), C.byref(rp), _p(plane, _fp), _p(depth, _fp), _p(score, _fp),
                               _p(best, _ip))
    return dict(plane=plane, depth=depth, score=score, best=best, seconds=secs)


def sweeps(views: Views, cp: ORCostParams, plane, depth, score, best, first_half, n_half, seed=0, keyframe=0,
           row_lo=-1, row_hi=-1, threads=0, propagation=0):
    """Half-sweeps from a given state (arrays are copied, results returned)."""
    rp = ORRunParams(cp, 0, 0.3, 20.0, seed, keyframe, INIT_LOGUNIFORM_HEMI, row_lo, row_hi, threads, propagation)
    plane = np.ascontiguousarray(plane, np.float32).copy()
    depth = np.ascontiguousarray(depth, np.float32).copy()
    score = np.ascontiguousarray(score, np.float32).copy()
    best = np.ascontiguousarray(best, np.int32).copy()
    lib().or_sweeps(C.byref(views.s), C.byref(rp), _p(plane, _fp), _p(depth, _fp), _p(score, _fp), _p(best, _ip),
                    first_half, n_half)
    return dict(plane=plane, depth=depth, score=score, best=best)


def postprocess(ref, depth, score, patch_half=5, mask=None, min_patch_sd=0.0, min_depth=0.3, max_depth=20.0,
                min_score=0.1):
    H, W = depth.shape
    d = np.ascontiguousarray(depth, np.float32).copy()
    s = np.ascontiguousarray(score, np.float32).copy()
    r = np.ascontiguousarray(ref, np.float32)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().or_postprocess(W, H, patch_half, _p(r, _fp), _p(m, _u8p), min_patch_sd, min_depth, max_depth,
                         min_score, _p(d, _fp), _p(s, _fp))
    return d, s


def warp_prior(prev_plane, prev_depth, Rp, tp, W, H, Rn, tn):
    """Seeding candidates (H, W, 4): plane xyz + range (0 = none)."""
    Hp, Wp = prev_depth.shape
    pl = np.ascontiguousarray(prev_plane, np.float32)
    d = np.ascontiguousarray(prev_depth, np.float32)
    Rp, tp, Rn, tn = [np.ascontiguousarray(a, np.float64) for a in (Rp, tp, Rn, tn)]
    cand = np.zeros((H, W, 4), np.float32)
    lib().or_warp_prior(Wp, Hp, _p(pl, _fp), _p(d, _fp), _p(Rp, _dp), _p(tp, _dp), W, H, _p(Rn, _dp), _p(tn, _dp),
                        _p(cand, _fp))
    return cand


def landmark_candidates(R, t, W, H, xyz, mask=None):
    """Seeding candidates (H, W, 4) from SLAM landmarks: plane xyz + range
    (0 = none).  Restates DepthmapEstimator::PreInitSparsePCL2
    (depthmap.cc:361-432) in FP64: ReprojectEquirect (:143-161), nearest-pixel
    rounding int(x + 0.5) (:380-381), mask test (:384-386), range = |X_c|
    (:392), normal = -bearing and PlanePosFromDepthAndNormal_equirect
    (:130-141, :395-400).  Where several landmarks land on one pixel the
    nearest (then the lowest index) is kept; points rounding outside the image
    are skipped."""
    R = np.asarray(R, np.float64).reshape(3, 3)
    t = np.asarray(t, np.float64).reshape(3)
    cand = np.zeros((H, W, 4), np.float32)
    best = {}
    for k, p in enumerate(np.asarray(xyz, np.float64).reshape(-1, 3)):
        X = R @ p + t
        d = float(np.linalg.norm(X))
        if d < 1e-4:
            continue
        b = X / d
        lat = -np.arcsin(np.clip(b[1], -1.0, 1.0))
        lon = np.arctan2(b[0], b[2])
        x = W * (0.5 + lon / (2 * np.pi))
        y = H * (0.5 - lat / np.pi)
        x0, y0 = int(x + 0.5), int(y + 0.5)
        if not (0 <= x0 < W and 0 <= y0 < H):
            continue
        key = (y0, x0)
        df = float(np.float32(d))
        if key not in best or (df, k) < best[key]:
            best[key] = (df, k)
    for (y0, x0), (df, k) in best.items():
        if mask is not None and not mask[y0, x0]:
            continue
        bb = bearing64(W, H, y0, x0)
        den = -df * float(np.dot(bb, bb))
        if 0 <= den < 1e-5:
            den = 1e-5
        elif -1e-5 < den < 0:
            den = -1e-5
        cand[y0, x0, :3] = -bb / den
        cand[y0, x0, 3] = df
    return cand


def median3(x):
    H, W = x.shape
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(x)
    lib().or_median3(W, H, _p(x, _fp), _p(out, _fp))
    return out


def clean(depths, R, t, center, thr, min_consistent=3, reproj_px=0.0):
    depths = [np.ascontiguousarray(d, np.float32) for d in depths]
    H, W = depths[0].shape
    arr = (_fp * len(depths))(*[_p(d, _fp) for d in depths])
    R = np.ascontiguousarray(R, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    out = np.zeros((H, W), np.float32)
    lib().or_clean(W, H, len(depths), arr, _p(R, _dp), _p(t, _dp), center, thr, min_consistent, reproj_px,
                   _p(out, _fp))
    return out


def prune(depths, R, t, rgb, thr):
    """Returns (pruned_depth, points[n,3] f64, colors[n,3] u8, keypts[n,2] i32, mutated depths)."""
    depths = [np.ascontiguousarray(d, np.float32).copy() for d in depths]
    H, W = depths[0].shape
    arr = (_fp * len(depths))(*[_p(d, _fp) for d in depths])
    R = np.ascontiguousarray(R, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    pruned = np.zeros((H, W), np.float32)
    pts = np.zeros((H * W, 3), np.float64)
    cols = np.zeros((H * W, 3), np.uint8)
    kp = np.zeros((H * W, 2), np.int32)
    rgb = None if rgb is None else np.ascontiguousarray(rgb, np.uint8)
    n = lib().or_prune(W, H, len(depths), arr, _p(R, _dp), _p(t, _dp), _p(rgb, _u8p), thr, _p(pruned, _fp),
                       _p(pts, _dp), _p(cols, _u8p), _p(kp, _ip))
    return pruned, pts[:n], cols[:n], kp[:n], depths


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().or_philox4x32_10(c, k, o)
    return list(o)


def refine_normals(seed, keyframe, pixel, tag):
    out = np.empty(18, np.float32)
    lib().or_refine_normals(seed, keyframe, pixel, tag, _p(out, _fp))
    return out


def bearing64(W, H, i, j):
    b = (C.c_double * 3)()
    lib().or_bearing64(W, H, i, j, b)
    return np.array(list(b))


def bearing_ref_f32(W, H, i, j):
    b = (C.c_float * 3)()
    lib().or_bearing_ref_f32(W, H, i, j, b)
    return np.array(list(b), np.float32)


def gt_plane(depth, normal, W, H, i, j):
    """Plane vector pi = n / (n . (d b)) of the analytic surface at pixel (i, j)."""
    b = bearing64(W, H, i, j)
    n = np.asarray(normal, np.float64)
    return n / np.dot(n, depth * b)


def score_view(prev_center, cur_center, prev_ids, cur_ids, cur_xyz):
    """Neighbour view test (score_view, depthmap_computation_module.cc:147-198):
    fraction of common landmarks (matched by id, first occurrence) whose angle
    between the rays to the two camera centres lies in (pi/60, pi/6);
    0 when there is none.  Returns (score, n_common)."""
    prev = set(int(k) for k in prev_ids)
    seen = set()
    s, n = 0.0, 0
    pc = np.asarray(prev_center, np.float64)
    cc = np.asarray(cur_center, np.float64)
    for k, lm in zip(cur_ids, np.asarray(cur_xyz, np.float64).reshape(-1, 3)):
        k = int(k)
        if k not in prev or k in seen:
            continue
        seen.add(k)
        dp, dc = pc - lm, cc - lm
        theta = np.arccos(np.dot(dc, dp) / np.sqrt(np.dot(dc, dc) * np.dot(dp, dp)))
        if np.pi / 60 < theta < np.pi / 6:
            s += 1.0
        n += 1
    return (np.float32(s) / np.float32(n) if n else 0.0), n


def depth_interval(R_cw, t_cw, xyz):
    """Landmark range percentiles (keyframe::computePercentileDepth_10_90,
    data/keyframe.cc:428-455, ranges stored as float) and the densifier's
    interval [1e-5, 1.1 p90] (compute_depth_intervall,
    depthmap_computation_module.cc:123-131)."""
    R = np.asarray(R_cw, np.float64).reshape(3, 3)
    t = np.asarray(t_cw, np.float64).reshape(3)
    X = np.asarray(xyz, np.float64).reshape(-1, 3) @ R.T + t
    d = np.sort(np.linalg.norm(X, axis=1).astype(np.float32))
    n = len(d)
    p10, p90 = float(d[n // 10]), float(d[n // 10 * 9])
    return p10, p90, 1e-5, p90 * 1.1


def to_gray(img, rgb=False):
    """BT.601 gray in 14-bit fixed point, rounded (the fixed-point form of
    COLOR_BGR2GRAY used by util/image_converter.cc:8-39)."""
    img = np.asarray(img)
    if img.ndim == 2:
        return img.copy()
    c = img.astype(np.uint32)
    b, g, r = (c[..., 2], c[..., 1], c[..., 0]) if rgb else (c[..., 0], c[..., 1], c[..., 2])
    return ((r * 4899 + g * 9617 + b * 1868 + 8192) >> 14).astype(np.uint8)


def resize_linear(img, W, H):
    """Bilinear resize, pixel centres aligned, 11-bit weights, one rounding
    (the 8-bit linear resize scheme behind the thumbnails, data/frame.cc:53-54)."""
    img = np.asarray(img)
    h, w = img.shape[:2]
    ch = 1 if img.ndim == 2 else img.shape[2]
    src = img.reshape(h, w, ch).astype(np.int64)

    def axis(n_dst, n_src):
        f0 = (np.arange(n_dst, dtype=np.float32) + np.float32(0.5)) * np.float32(np.float32(n_src) / np.float32(n_dst)) \
            - np.float32(0.5)
        s = np.floor(f0).astype(np.int64)
        f = (f0 - s.astype(np.float32)).astype(np.float32)
        f[s < 0] = 0
        s[s < 0] = 0
        hi = s >= n_src - 1
        f[hi] = 0
        s[hi] = n_src - 1
        c1 = np.rint(f * np.float32(2048)).astype(np.int64)
        return s, np.minimum(s + 1, n_src - 1), 2048 - c1, c1

    sx, sx1, cx0, cx1 = axis(W, w)
    sy, sy1, cy0, cy1 = axis(H, h)
    a = src[sy][:, sx] * cx0[None, :, None] + src[sy][:, sx1] * cx1[None, :, None]
    b = src[sy1][:, sx] * cx0[None, :, None] + src[sy1][:, sx1] * cx1[None, :, None]
    v = (a * cy0[:, None, None] + b * cy1[:, None, None] + (1 << 21)) >> 22
    out = np.clip(v, 0, 255).astype(np.uint8)
    return out[..., 0] if img.ndim == 2 else out


def pyramid_f16(img, levels=3):
    """FP16 pyramid: level 0 = the image, then 2x2 means (edge repeated)."""
    out = [np.asarray(img).astype(np.float16)]
    for _ in range(1, levels):
        s = out[-1].astype(np.float32)
        h, w = s.shape
        ys = np.minimum(np.arange((h + 1) // 2) * 2 + np.array([[0], [1]]), h - 1)
        xs = np.minimum(np.arange((w + 1) // 2) * 2 + np.array([[0], [1]]), w - 1)
        t = s[ys[0]][:, xs[0]] + s[ys[0]][:, xs[1]] + s[ys[1]][:, xs[0]] + s[ys[1]][:, xs[1]]
        out.append((np.float32(0.25) * t).astype(np.float16))
    return out
