"""Seeded synthetic equirectangular scenes with analytic ground truth.

Thin ctypes layer over ``libpm_scene.so`` (``include/pm_scene.h``).  The
workloads mirror the densifier's benchmark configurations: a camera inside a
10 x 6 x 3 m textured room (optionally with boxes and a cylinder), or a long
hall of boxes traversed by a smooth trajectory.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._native import load_scene_lib

ROOM, ROOM_OBJECTS, HALL = 0, 1, 2

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_u8p = C.POINTER(C.c_uint8)


def _lib():
    lib = load_scene_lib()
    if not getattr(lib, "_pm_typed", False):
        lib.pm_scene_create.restype = C.c_void_p
        lib.pm_scene_create.argtypes = [C.c_int, C.c_uint32]
        lib.pm_scene_destroy.argtypes = [C.c_void_p]
        lib.pm_scene_poses.restype = C.c_int
        lib.pm_scene_poses.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.c_float, C.c_float,
                                       C.c_float, _dp, _dp]
        lib.pm_scene_trajectory_pose.restype = C.c_int
        lib.pm_scene_trajectory_pose.argtypes = [C.c_void_p, C.c_uint32, C.c_int, C.c_double,
                                                 C.c_double, _dp, _dp]
        lib.pm_scene_render_device.restype = C.c_int
        lib.pm_scene_render_device.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_float,
                                               C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.pm_scene_render_device_f32.restype = C.c_int
        lib.pm_scene_render_device_f32.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_float,
                                                   C.c_uint32, C.c_void_p, C.c_void_p]
        lib.pm_scene_render.restype = C.c_int
        lib.pm_scene_render.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_float,
                                        C.c_uint32, _fp, _u8p, _u8p, _fp, _fp]
        lib._pm_typed = True
    return lib


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


@dataclass
class View:
    """One rendered keyframe: images, pose (world->camera) and ground truth."""
    gray: np.ndarray          # (H, W) float32, 0..255
    gray_u8: np.ndarray       # (H, W) uint8
    rgb: np.ndarray           # (H, W, 3) uint8, BGR
    depth: np.ndarray         # (H, W) float32 range along the bearing
    normal: np.ndarray        # (H, W, 3) float32 camera-frame unit normal
    R: np.ndarray             # (3, 3) float64 R_cw
    t: np.ndarray             # (3,) float64 t_cw


class Scene:
    def __init__(self, kind: int = ROOM, seed: int = 0):
        self._lib = _lib()
        self.kind, self.seed = kind, seed
        self._h = self._lib.pm_scene_create(kind, seed)
        if not self._h:
            raise RuntimeError("pm_scene_create failed")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.pm_scene_destroy(h)
            self._h = None

    def poses(self, n_views: int, seed: int, bmin: float, bmax: float, yaw_deg: float):
        R = np.zeros((n_views, 3, 3), np.float64)
        t = np.zeros((n_views, 3), np.float64)
        rc = self._lib.pm_scene_poses(self._h, n_views, seed, bmin, bmax, yaw_deg, _ptr(R, _dp), _ptr(t, _dp))
        if rc:
            raise RuntimeError("pm_scene_poses failed")
        return R, t

    def trajectory_pose(self, seed: int, n_waypoints: int, duration_s: float, t_s: float):
        R = np.zeros((3, 3), np.float64)
        t = np.zeros(3, np.float64)
        rc = self._lib.pm_scene_trajectory_pose(self._h, seed, n_waypoints, duration_s, t_s,
                                                _ptr(R, _dp), _ptr(t, _dp))
        if rc:
            raise RuntimeError("pm_scene_trajectory_pose failed")
        return R, t

    def render_device(self, R, t, W: int, H: int, gray=None, depth=None, bgr=None, supersample: int = 2,
                      noise_sigma: float = 0.0, noise_seed: int = 0, stream: int = 0):
        """Render on the GPU into torch CUDA tensors (uint8 (H, W), float32 (H, W), uint8 (H, W, 3))."""
        R = np.ascontiguousarray(R, np.float64)
        t = np.ascontiguousarray(t, np.float64)
        p = lambda x: None if x is None else x.data_ptr()
        rc = self._lib.pm_scene_render_device(self._h, _ptr(R, _dp), _ptr(t, _dp), W, H, supersample, noise_sigma,
                                              noise_seed, p(gray), p(depth), p(bgr), stream)
        if rc:
            raise RuntimeError("pm_scene_render_device failed")

    def render_device_f32(self, R, t, W: int, H: int, gray, supersample: int = 2, noise_sigma: float = 0.0,
                          noise_seed: int = 0, stream: int = 0):
        """Unrounded intensities (float32 CUDA tensor (H, W)) on the GPU."""
        R = np.ascontiguousarray(R, np.float64)
        t = np.ascontiguousarray(t, np.float64)
        rc = self._lib.pm_scene_render_device_f32(self._h, _ptr(R, _dp), _ptr(t, _dp), W, H, supersample, noise_sigma,
                                                  noise_seed, gray.data_ptr(), stream)
        if rc:
            raise RuntimeError("pm_scene_render_device_f32 failed")

    def render(self, R, t, W: int, H: int, supersample: int = 2, noise_sigma: float = 0.0,
               noise_seed: int = 0) -> View:
        R = np.ascontiguousarray(R, np.float64)
        t = np.ascontiguousarray(t, np.float64)
        gray = np.empty((H, W), np.float32)
        gu8 = np.empty((H, W), np.uint8)
        rgb = np.empty((H, W, 3), np.uint8)
        depth = np.empty((H, W), np.float32)
        normal = np.empty((H, W, 3), np.float32)
        rc = self._lib.pm_scene_render(self._h, _ptr(R, _dp), _ptr(t, _dp), W, H, supersample,
                                       noise_sigma, noise_seed, _ptr(gray, _fp), _ptr(gu8, _u8p),
                                       _ptr(rgb, _u8p), _ptr(depth, _fp), _ptr(normal, _fp))
        if rc:
            raise RuntimeError("pm_scene_render failed")
        return View(gray, gu8, rgb, depth, normal, R.copy(), t.copy())


@dataclass
class Request:
    """A densification request: reference view + sources (view 0 is the reference)."""
    views: list
    W: int
    H: int
    seed: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def n_src(self) -> int:
        return len(self.views) - 1

    @property
    def R(self) -> np.ndarray:
        return np.stack([v.R for v in self.views])

    @property
    def t(self) -> np.ndarray:
        return np.stack([v.t for v in self.views])


def make_request(kind: int, W: int, H: int, n_src: int, seed: int = 0, bmin: float = 0.2,
                 bmax: float = 0.5, yaw_deg: float = 15.0, noise_sigma: float = 0.0,
                 supersample: int = 2, scene_seed: int | None = None) -> Request:
    """Render one request: scene `kind` (ROOM / ROOM_OBJECTS / HALL) at W x H with
    n_src sources offset bmin..bmax metres and +-yaw_deg degrees of yaw."""
    sc = Scene(kind, seed if scene_seed is None else scene_seed)
    R, t = sc.poses(n_src + 1, seed, bmin, bmax, yaw_deg)
    views = [sc.render(R[k], t[k], W, H, supersample, noise_sigma, seed * 131 + k) for k in range(n_src + 1)]
    return Request(views, W, H, seed, dict(kind=kind, bmin=bmin, bmax=bmax, yaw_deg=yaw_deg,
                                           noise_sigma=noise_sigma))


def config_request(cfg: int, seed: int = 0, W: int | None = None, H: int | None = None,
                   n_src: int | None = None) -> Request:
    """The benchmark workloads by number: 1 = 512x256 room with 4 sources,
    2 = 1920x960 room with objects and 6 sources, 3 = 3840x1920 room with 8
    sources and sigma-2 image noise.  W/H/n_src override the size."""
    if cfg == 1:
        return make_request(ROOM, W or 512, H or 256, n_src or 4, seed, 0.2, 0.5, 15.0)
    if cfg == 2:
        return make_request(ROOM_OBJECTS, W or 1920, H or 960, n_src or 6, seed, 0.1, 0.8, 15.0)
    if cfg == 3:
        return make_request(ROOM, W or 3840, H or 1920, n_src or 8, seed, 0.2, 0.5, 15.0, noise_sigma=2.0)
    raise ValueError(f"unknown workload {cfg}")


@dataclass
class Keyframe:
    """One keyframe of a served stream: arrival time, image, pose, ground truth."""
    t_s: float
    gray_u8: np.ndarray
    depth: np.ndarray
    R: np.ndarray
    t: np.ndarray

    @property
    def shape(self):
        return self.gray_u8.shape


def served_stream(seed: int = 0, duration_s: float = 60.0, rate_hz: float = 2.0, n_waypoints: int = 20,
                  sizes=((1920, 960), (3840, 1920)), p_sizes=(0.75, 0.25), t_end: float | None = None,
                  device: int = 0) -> list:
    """Keyframes as a SLAM front end emits them: Poisson arrivals at rate_hz
    along the hall scene's seeded smooth trajectory (duration_s seconds through
    n_waypoints waypoints), each at a size drawn from `sizes` with
    probabilities `p_sizes`.  Rendered on the GPU, returned on the host.
    t_end stops the stream early (seconds)."""
    import torch
    rng = np.random.default_rng(seed)
    sc = Scene(HALL, seed)
    end = duration_s if t_end is None else min(t_end, duration_s)
    times = []
    t = rng.exponential(1.0 / rate_hz)
    while t < end:
        times.append(t)
        t += rng.exponential(1.0 / rate_hz)
    which = rng.choice(len(sizes), size=len(times), p=np.asarray(p_sizes, float) / np.sum(p_sizes))
    out = []
    dev = torch.device("cuda", device)
    bufs = {}
    for k, (ts, w) in enumerate(zip(times, which)):
        W, H = sizes[w]
        if (W, H) not in bufs:
            bufs[(W, H)] = (torch.empty((H, W), dtype=torch.uint8, device=dev),
                            torch.empty((H, W), dtype=torch.float32, device=dev))
        g, d = bufs[(W, H)]
        R, tc = sc.trajectory_pose(seed, n_waypoints, duration_s, ts)
        sc.render_device(R, tc, W, H, gray=g, depth=d, stream=torch.cuda.current_stream(dev).cuda_stream)
        out.append(Keyframe(float(ts), g.cpu().numpy(), d.cpu().numpy(), R, tc))
    return out
