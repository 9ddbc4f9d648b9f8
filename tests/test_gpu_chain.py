"""Filter and fusion on device-resident maps (pm_filter_consistency_device,
pm_fuse_device): the same results as the host-buffer calls, and chained
straight after densification from pm_request_depth_device without a host
round trip (the reference hands host cv::Mat copies between its estimator,
cleaner and pruner, depthmap_computation_module.cc:396-412)."""
import numpy as np
import pytest

from oracle import oracle as O
from patchmatch_gb300 import native, scene

pytestmark = pytest.mark.gpu


def _maps(seed, W, H, n, noise=0.004, drop=0.1):
    req = scene.make_request(scene.ROOM_OBJECTS, W, H, n - 1, seed=seed, bmin=0.1, bmax=0.4)
    rng = np.random.default_rng(seed)
    depths = []
    for v in req.views:
        d = v.depth * (1 + rng.normal(0, noise, v.depth.shape)).astype(np.float32)
        d[rng.random(d.shape) < drop] = 0
        depths.append(d.astype(np.float32))
    return req, depths


@pytest.mark.parametrize("reproj", [0.0, 1.0])
def test_device_filter_equals_host_filter(ctx, reproj):
    import torch
    req, depths = _maps(61, 320, 160, 5)
    host = ctx.filter_consistency(depths, req.R, req.t, center=2, thr=0.01, min_consistent=3, reproj_px=reproj)
    dev = [torch.from_numpy(d).cuda() for d in depths]
    out = torch.full((160, 320), -7.0, device="cuda")
    ctx.filter_consistency_device([d.data_ptr() for d in dev], 320, 160, req.R, req.t, 2, 0.01, out.data_ptr(),
                                  min_consistent=3, reproj_px=reproj,
                                  stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), host)
    o = O.clean(depths, req.R, req.t, center=2, thr=0.01, min_consistent=3, reproj_px=reproj)
    assert ((host > 0) == (o > 0)).mean() >= 0.999


def test_device_fuse_equals_host_fuse(ctx):
    import torch
    req, depths = _maps(62, 320, 160, 5, drop=0.05)
    bgr = req.views[0].rgb
    p0, x0, c0, ij0, m0 = ctx.fuse(depths, req.R, req.t, bgr, 0.02)
    W, H = 320, 160
    dev = [torch.from_numpy(d).cuda() for d in depths]
    ws_bytes = native.fuse_workspace_bytes(W, H)
    ws = torch.empty(ws_bytes + 256, dtype=torch.uint8, device="cuda")
    ws_ptr = (ws.data_ptr() + 255) & ~255
    pruned = torch.full((H, W), -5.0, device="cuda")
    xyz = torch.full((H * W, 3), float("nan"), device="cuda")
    cols = torch.zeros((H * W, 3), dtype=torch.uint8, device="cuda")
    ij = torch.full((H * W, 2), -1, dtype=torch.int32, device="cuda")
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    dbgr = torch.from_numpy(np.ascontiguousarray(bgr)).cuda()
    for _ in range(2):  # the workspace is reused: the second call must not see the first's state
        for d, h in zip(dev, depths):
            d.copy_(torch.from_numpy(h))
        ctx.fuse_device([d.data_ptr() for d in dev], W, H, req.R, req.t, 0.02, pruned.data_ptr(), xyz.data_ptr(),
                        count.data_ptr(), ws_ptr, ws_bytes, bgr_ptr=dbgr.data_ptr(), bgr_out_ptr=cols.data_ptr(),
                        ij_ptr=ij.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        n = int(count.item())
        assert n == len(x0) > 0
        assert np.array_equal(pruned.cpu().numpy(), p0)
        assert np.array_equal(ij[:n].cpu().numpy(), ij0) and np.array_equal(cols[:n].cpu().numpy(), c0)
        assert np.allclose(xyz[:n].cpu().numpy().astype(np.float64), x0, rtol=0, atol=1e-6)
        for a, b in zip(dev, m0):
            assert np.array_equal(a.cpu().numpy(), b)


def test_device_fuse_rejects_small_or_unaligned_workspace(ctx):
    import torch
    W, H = 64, 32
    d = torch.zeros((H, W), device="cuda")
    ws_bytes = native.fuse_workspace_bytes(W, H)
    ws = torch.empty(ws_bytes + 512, dtype=torch.uint8, device="cuda")
    base = (ws.data_ptr() + 255) & ~255
    R = np.stack([np.eye(3)] * 2)
    t = np.zeros((2, 3))
    with pytest.raises(native.PmError) as e:
        ctx.fuse_device([d.data_ptr()] * 2, W, H, R, t, 0.02, d.data_ptr(), d.data_ptr(), d.data_ptr(), base,
                        ws_bytes - 1)
    assert e.value.status == native.PM_EINVAL
    with pytest.raises(native.PmError) as e:
        ctx.fuse_device([d.data_ptr()] * 2, W, H, R, t, 0.02, d.data_ptr(), d.data_ptr(), d.data_ptr(), base + 16,
                        ws_bytes)
    assert e.value.status == native.PM_EINVAL


def test_chain_from_resident_requests(ctx):
    """Five keyframes densified and left on the device; the centre's
    consistency filter reads their filtered depths in place and equals the
    host-buffer filter over the same maps read back."""
    import torch
    sc = scene.Scene(scene.ROOM_OBJECTS, 63)
    W, H = 384, 192
    poses = [sc.trajectory_pose(9, 8, 10.0, 1.0 + 0.2 * k) for k in range(7)]
    views = [sc.render(R, t, W, H) for R, t in poses]
    reqs = []
    for k in range(1, 6):
        idx = [k, k - 1, k + 1]
        r = ctx.request(W, H, 2, native.default_params(iterations=4, keyframe_id=k))
        r.set_views([views[q].gray_u8 for q in idx], np.stack([views[q].R for q in idx]),
                    np.stack([views[q].t for q in idx]))
        r.run()
        reqs.append(r)
    for r in reqs:
        r.synchronize()
    ptrs = [r.depth_device_ptr for r in reqs]
    R = np.stack([views[k].R for k in range(1, 6)])
    t = np.stack([views[k].t for k in range(1, 6)])
    out = torch.zeros((H, W), device="cuda")
    ctx.filter_consistency_device(ptrs, W, H, R, t, 2, 0.01, out.data_ptr(), min_consistent=3, reproj_px=1.0)
    torch.cuda.synchronize()
    host_maps = [r.read()["depth"] for r in reqs]
    ref = ctx.filter_consistency(host_maps, R, t, center=2, thr=0.01, min_consistent=3, reproj_px=1.0)
    got = out.cpu().numpy()
    assert np.array_equal(got, ref)
    assert (got > 0).mean() > 0.15  # 4 sweeps, 2 sources, 1 % agreement of 3 of 5 views
    for r in reqs:
        r.close()


def test_gpu_filter_and_fuse_equal_reference_host_golden(ctx):
    """The GPU consistency filter and fusion against the reference's own
    host Clean and Prune (golden fixture of depthmap.cc compiled unmodified):
    keep decisions equal, kept depths and pixel indices identical."""
    import os
    fix = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_host_96x48.npz")
    if not os.path.exists(fix):
        pytest.skip("golden fixture not generated")
    gold = dict(np.load(fix))
    for case in (0, 1):
        d = list(gold[f"c{case}_depths"])
        R, t = gold[f"c{case}_R"], gold[f"c{case}_t"]
        thr_c, thr_p = (float(x) for x in gold[f"c{case}_thr"])
        g = ctx.filter_consistency(d, R, t, center=2, thr=thr_c, min_consistent=3)
        ref = gold[f"c{case}_clean"]
        assert ((g > 0) == (ref > 0)).mean() >= 0.999, case
        both = (g > 0) & (ref > 0)
        assert np.array_equal(g[both], ref[both])
        pruned, xyz, cols, ij, _ = ctx.fuse(d, R, t, gold[f"c{case}_bgr"], thr_p)
        assert ((pruned > 0) == (gold[f"c{case}_pruned"] > 0)).mean() >= 0.999, case
        common = np.intersect1d(ij[:, 0] * 96 + ij[:, 1], gold[f"c{case}_ij"][:, 0] * 96 + gold[f"c{case}_ij"][:, 1])
        assert len(common) >= 0.999 * max(len(ij), len(gold[f"c{case}_ij"]))
