"""CPU tests of the oracle (the parity checker) and of the scene generator.

These pin the oracle's restatement on properties the reference's own code
implies: analytic bearings, NCC of the true surface close to 1, scale
invariance of the plane warp, the median filter, the consistency filter on a
perfect scene, and the sequential pruning order.  The comparison against the
reference kernels' own outputs lives in test_golden.py.
"""
import numpy as np
import pytest

from oracle import oracle as O
from patchmatch_gb300 import scene


@pytest.fixture(scope="module")
def room():
    O.build()
    return scene.make_request(scene.ROOM, 128, 64, 3, seed=5)


def test_philox_deterministic_and_distinct():
    a = O.philox([0, 0, 0, 0], [0, 0])
    b = O.philox([0, 0, 0, 0], [0, 0])
    c = O.philox([1, 0, 0, 0], [0, 0])
    d = O.philox([0, 0, 0, 0], [1, 0])
    assert a == b and a != c and a != d
    # statistical sanity of the refinement normals
    z = np.concatenate([O.refine_normals(0, 0, p, 1) for p in range(4000)])
    assert abs(z.mean()) < 0.03 and abs(z.std() - 1.0) < 0.03


def test_bearing_convention():
    W, H = 64, 32
    # lon = 0 at column W/2 (forward, +z); lat = 0 at row H/2
    assert np.allclose(O.bearing64(W, H, H // 2, W // 2), [0, 0, 1])
    # column 3W/4: lon = +pi/2 -> +x
    assert np.allclose(O.bearing64(W, H, H // 2, 3 * W // 4), [1, 0, 0], atol=1e-12)
    # row 0: lat = +pi/2 -> -y (up)
    assert np.allclose(O.bearing64(W, H, 0, W // 2), [0, -1, 0], atol=1e-12)


def test_true_plane_scores_high(room):
    v0 = room.views[0]
    V = O.Views.from_request(room)
    rng = np.random.default_rng(0)
    ij = np.stack([rng.integers(6, 58, 300), rng.integers(6, 122, 300)], 1).astype(np.int32)
    gt = np.array([O.gt_plane(v0.depth[i, j], v0.normal[i, j], 128, 64, i, j) for i, j in ij], np.float32)
    s, _ = O.cost_batch(V, O.cost_params(), ij, gt)
    assert np.median(s) > 0.9
    bad, _ = O.cost_batch(V, O.cost_params(), ij, gt * 3.0)
    assert np.median(bad) < np.median(s) - 0.2


def test_f32_reference_arithmetic_close_to_exact(room):
    V = O.Views.from_request(room)
    rng = np.random.default_rng(1)
    ij = np.stack([rng.integers(6, 58, 500), rng.integers(6, 122, 500)], 1).astype(np.int32)
    v0 = room.views[0]
    gt = np.array([O.gt_plane(v0.depth[i, j], v0.normal[i, j], 128, 64, i, j) for i, j in ij], np.float32)
    planes = gt * rng.uniform(0.9, 1.1, (500, 1)).astype(np.float32)
    s64, _, n64 = O.cost_batch(V, O.cost_params(), ij, planes, want_ncc=True)
    s32, _, n32 = O.cost_batch(V, O.cost_params(arith=O.ARITH_F32_REF), ij, planes, want_ncc=True)
    assert np.median(np.abs(n64 - n32)) < 1e-5


def test_combine_modes(room):
    V = O.Views.from_request(room)
    ij = np.array([[30, 60]], np.int32)
    v0 = room.views[0]
    pl = O.gt_plane(v0.depth[30, 60], v0.normal[30, 60], 128, 64, 30, 60).astype(np.float32)[None]
    _, _, ncc = O.cost_batch(V, O.cost_params(), ij, pl, want_ncc=True)
    mx, b = O.cost_batch(V, O.cost_params(combine=O.COMBINE_MAX), ij, pl)
    assert np.isclose(mx[0], ncc[0].max()) and b[0] == int(np.argmax(ncc[0]))
    tk, _ = O.cost_batch(V, O.cost_params(combine=O.COMBINE_TOPK, top_k=2), ij, pl)
    assert np.isclose(tk[0], np.sort(ncc[0])[::-1][:2].mean())
    fs, _ = O.cost_batch(V, O.cost_params(combine=O.COMBINE_FOLD_SEPARATE), ij, pl)
    score = -1.0
    for s2 in ncc[0]:
        score = 0.5 * (score + s2) if abs((score - s2) / s2) < 0.25 else max(score, s2)
    assert np.isclose(fs[0], score)


def test_median3_replicate_border():
    rng = np.random.default_rng(2)
    x = rng.random((9, 13)).astype(np.float32)
    m = O.median3(x)
    p = np.pad(x, 1, mode="edge")
    ref = np.median(np.stack([p[di:di + 9, dj:dj + 13] for di in range(3) for dj in range(3)]), 0)
    assert np.array_equal(m, ref.astype(np.float32))


def test_clean_keeps_consistent_truth():
    req = scene.make_request(scene.ROOM, 128, 64, 4, seed=8)
    depths = [v.depth for v in req.views]
    out = O.clean(depths, req.R, req.t, center=0, thr=0.01, min_consistent=3)
    kept = (out > 0).mean()
    assert kept > 0.8
    # a corrupted centre map loses its corrupted pixels
    bad = depths[0].copy()
    bad[20:30, 40:60] *= 1.3
    out2 = O.clean([bad] + depths[1:], req.R, req.t, center=0, thr=0.01, min_consistent=3)
    assert (out2[20:30, 40:60] > 0).mean() < 0.05


def test_prune_removes_duplicates_in_order():
    req = scene.make_request(scene.ROOM, 128, 64, 2, seed=9, bmin=0.05, bmax=0.1)
    depths = [v.depth for v in req.views]
    pruned, pts, cols, kp, mutated = O.prune(depths, req.R, req.t, req.views[0].rgb, 0.02)
    # the same surface seen from nearby cameras: most head pixels either win
    # (and zero the duplicates in the later maps) or are dropped
    assert len(pts) > 0
    zeroed = sum(int(((d > 0) & (m == 0)).sum()) for d, m in zip(depths[1:], mutated[1:]))
    assert zeroed > 0
    assert np.all(pruned[kp[:, 0], kp[:, 1]] > 0)
    # raster order of emitted points
    lin = kp[:, 0] * 128 + kp[:, 1]
    assert np.all(np.diff(lin) > 0)


def test_scene_ground_truth_consistent():
    req = scene.make_request(scene.ROOM_OBJECTS, 160, 80, 1, seed=1)
    v = req.views[0]
    assert np.isfinite(v.depth).all() and v.depth.min() > 0.1
    assert np.allclose(np.linalg.norm(v.normal, axis=2), 1.0, atol=1e-5)
    assert v.gray_u8.std() > 20


def test_landmark_candidates_restatement():
    """A landmark on the bearing of pixel (i, j) at range d gives that pixel
    the camera-facing plane b / d; nearer landmarks win shared pixels; points
    behind 1e-4 m or rounding outside the image give nothing."""
    W, H = 64, 32
    R = np.eye(3)
    t = np.zeros(3)
    b = O.bearing64(W, H, 10, 20)
    pts = np.array([3.0 * b, 2.0 * b, [0.0, 0.0, 5e-5]])
    c = O.landmark_candidates(R, t, W, H, pts)
    assert c[10, 20, 3] == np.float32(2.0)
    assert np.allclose(c[10, 20, :3], b / 2.0, rtol=1e-6)
    assert (c[..., 3] > 0).sum() == 1


def test_host_cost_border_reads_zero(room):
    """OR_SEAM_ZERO restates the reference host cost's border
    (LinearInterpolation, depthmap.cc:34-38): a sample whose footprint leaves
    [0, W-1) x [0, H-1) reads 0.  Hypotheses whose samples all stay inside
    score the same as with a clamped border; at the seam columns they differ."""
    H, W = room.H, room.W
    V = O.Views.from_request(room)
    v0 = room.views[0]
    ij = np.array([[H // 2, W // 2], [H // 2, 6], [H // 2, W - 7], [H // 3, W - 7]], np.int32)
    planes = np.array([O.gt_plane(v0.depth[i, j], v0.normal[i, j], W, H, i, j) for i, j in ij], np.float32)
    _, _, z = O.cost_batch(V, O.cost_params(seam=O.SEAM_ZERO, combine=O.COMBINE_MAX), ij, planes, want_ncc=True)
    _, _, c = O.cost_batch(V, O.cost_params(seam=O.SEAM_CLAMP, combine=O.COMBINE_MAX), ij, planes, want_ncc=True)
    assert np.allclose(z[0], c[0], rtol=0, atol=1e-12)  # image centre: every sample inside
    assert np.abs(z[1:] - c[1:]).max() > 1e-3           # at the seam the border decides


def test_smallest_window_skips_neighbours_outside_the_image():
    """With patch_half = 1 the active region starts 2 pixels from the border;
    the oracle's propagation skips the candidates that fall outside the image
    (a full run touches every border pixel and stays finite)."""
    req = scene.make_request(scene.ROOM, 64, 32, 2, seed=3)
    o = O.patchmatch(O.Views.from_request(req), O.cost_params(patch_half=1), iterations=2)
    d = o["depth"]
    assert np.isfinite(d).all() and (d[2:30, 2:62] > 0).all()
