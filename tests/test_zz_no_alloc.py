"""pm_fuse_noalloc: point fusion for callers that cannot allocate device memory
(an externally pooled process, a real-time thread that must stay out of the
CUDA allocator, or one whose HBM is fully committed).  It must give what
pm_fuse gives, on caller-owned device buffers, call after call.  This file is
collected last on purpose; it passes alone and after the other tests."""
import ctypes as C

import numpy as np
import pytest

from patchmatch_gb300 import native, scene

pytestmark = pytest.mark.gpu


def _inputs(seed, W, H, n, drop):
    req = scene.make_request(scene.ROOM, W, H, n - 1, seed=seed, bmin=0.05, bmax=0.3)
    rng = np.random.default_rng(seed)
    depths = []
    for v in req.views:
        d = v.depth.copy()
        d[rng.random(d.shape) < drop] = 0
        depths.append(d)
    return req, depths


def _run_noalloc(depths, R, t, bgr, thr):
    import torch
    L = native.lib()
    H, W = depths[0].shape
    dev = [torch.from_numpy(d).cuda() for d in depths]
    dbgr = torch.from_numpy(np.ascontiguousarray(bgr)).cuda()
    pruned = torch.full((H, W), -5.0, device="cuda")          # poisoned: must be overwritten
    xyz = torch.full((H * W, 3), float("nan"), device="cuda")
    bgr_out = torch.zeros((H * W, 3), dtype=torch.uint8, device="cuda")
    ij = torch.full((H * W, 2), -1, dtype=torch.int32, device="cuda")
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    ptrs = (C.c_void_p * len(dev))(*[d.data_ptr() for d in dev])
    R = np.ascontiguousarray(R, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.pm_fuse_noalloc(W, H, len(dev), C.cast(ptrs, C.c_void_p), R.ctypes.data, t.ctypes.data, dbgr.data_ptr(),
                           thr, pruned.data_ptr(), xyz.data_ptr(), bgr_out.data_ptr(), ij.data_ptr(),
                           count.data_ptr(), stream)
    assert rc == native.PM_OK
    torch.cuda.synchronize()
    n = int(count.item())
    return (pruned.cpu().numpy(), xyz[:n].cpu().numpy(), bgr_out[:n].cpu().numpy(), ij[:n].cpu().numpy(),
            [d.cpu().numpy() for d in dev])


def test_noalloc_fuse_matches_pm_fuse_twice_in_a_row(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    ctx = native.Context(0)
    # two different calls in a row: the second must not see the first's state
    cases = [(41, 320, 160, 4, 0.05, 0.02), (42, 256, 128, 5, 0.15, 0.03)]
    for seed, W, H, n, drop, thr in cases:
        req, depths = _inputs(seed, W, H, n, drop)
        bgr = req.views[0].rgb
        p0, x0, c0, ij0, m0 = ctx.fuse(depths, req.R, req.t, bgr, thr)
        p1, x1, c1, ij1, m1 = _run_noalloc(depths, req.R, req.t, bgr, thr)
        assert np.array_equal(p0, p1)
        assert len(x0) == len(x1) > 0
        assert np.array_equal(ij0, ij1) and np.array_equal(c0, c1)
        assert np.allclose(x0, x1.astype(np.float64), rtol=0, atol=1e-6)
        for a, b in zip(m0, m1):
            assert np.array_equal(a, b)
    ctx.close()


def test_noalloc_fuse_at_the_maximum_size(built):
    """2048 x 1024 = PM_FUSE_NOALLOC_MAX_PIXELS: the compaction scan runs over
    more than 1024 blocks and fills the array's last block-count slot."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    ctx = native.Context(0)
    req, depths = _inputs(43, 2048, 1024, 3, 0.05)
    bgr = req.views[0].rgb
    p0, x0, c0, ij0, m0 = ctx.fuse(depths, req.R, req.t, bgr, 0.02)
    p1, x1, c1, ij1, m1 = _run_noalloc(depths, req.R, req.t, bgr, 0.02)
    assert np.array_equal(p0, p1)
    assert len(x0) == len(x1) > 0
    assert np.array_equal(ij0, ij1) and np.array_equal(c0, c1)
    assert np.allclose(x0, x1.astype(np.float64), rtol=0, atol=1e-6)
    for a, b in zip(m0, m1):
        assert np.array_equal(a, b)
    ctx.close()


def test_noalloc_rejects_oversize_and_bad_arguments(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    L = native.lib()
    big_w = 8192 + 1
    R = np.eye(3)[None].repeat(2, 0).copy()
    t = np.zeros((2, 3))
    dummy = torch.zeros(4, device="cuda")
    ptrs = (C.c_void_p * 2)(dummy.data_ptr(), dummy.data_ptr())
    args = (C.cast(ptrs, C.c_void_p), R.ctypes.data, t.ctypes.data, None, 0.02, dummy.data_ptr(), dummy.data_ptr(),
            None, None, dummy.data_ptr(), None)
    assert L.pm_fuse_noalloc(big_w, 16, 2, *args) == native.PM_EINVAL
    assert L.pm_fuse_noalloc(4096, 1024, 2, *args) == native.PM_EINVAL      # 2^22 pixels > 2^21
    assert L.pm_fuse_noalloc(64, 32, 0, *args) == native.PM_EINVAL
