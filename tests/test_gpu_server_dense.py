"""The served loop's dense output (consistency filter + fusion over the
stream), its landmark input (view test, depth interval, seeding) and its
failure paths (timed-out waits, cancellation on destroy, a producer that
never collects).  The reference's densification and fusion threads are the
model: depthmap_computation_module.cc:205-472, dense_pointcloud_module.cc:
100-175, and their stop/reset handling, depthmap_computation_module.cc:498-615."""
import threading
import time

import numpy as np
import pytest

from patchmatch_gb300 import native, scene

pytestmark = pytest.mark.gpu

W, H = 384, 192


@pytest.fixture(scope="module")
def views():
    sc = scene.Scene(scene.ROOM_OBJECTS, 71)
    out = []
    for k in range(13):
        R, t = sc.trajectory_pose(6, 8, 12.0, 0.5 + 0.3 * k)
        out.append(sc.render(R, t, W, H))
    return out


def _cfg(inflight=4, **kw):
    p = native.default_params(iterations=4)
    base = dict(params=p, max_inflight=inflight, min_sources=2, max_sources=4, prior_lag=4, seeded_iterations=2,
                min_baseline=0.02, max_baseline=3.0)
    base.update(kw)
    return native.server_config(**base)


def test_dense_output_equals_the_host_chain(ctx, views):
    """Each keyframe's fused depth and points equal pm_filter_consistency over
    the five densified keyframes centred on it and pm_fuse over the five
    cleaned maps headed by it, run on the host-read depths in ticket order
    (the cleaner's and pruner's queues, depthmap.cc:1229-1377,1405-1696)."""
    srv = native.Server(ctx, _cfg(dense_output=1))
    tks = [srv.submit(v.gray_u8, v.R, v.t) for v in views]
    res = [srv.wait(tk) for tk in tks]
    srv.finish()  # end of stream: the tail's windows complete too
    dense = [srv.wait_dense(tk) for tk in tks]
    with pytest.raises(native.PmError) as e:  # the stream has ended
        srv.submit(views[0].gray_u8, views[0].R, views[0].t)
    assert e.value.status == native.PM_ECANCELLED
    srv.close()
    ok = [k for k, r in enumerate(res) if r[0] == native.PM_OK]
    assert len(ok) >= 9
    for k, r in enumerate(res):
        if r[0] != native.PM_OK:
            assert dense[k][0] == r[0]  # never densified: the same status
    cfg = _cfg(dense_output=1)
    # the cleaner: centre of each window of five densified keyframes
    cleaned = []
    for c in range(2, len(ok) - 2):
        win = ok[c - 2:c + 3]
        d = ctx.filter_consistency([res[k][1] for k in win], np.stack([views[k].R for k in win]),
                                   np.stack([views[k].t for k in win]), center=2, thr=cfg.clean_threshold,
                                   min_consistent=cfg.clean_min_views, reproj_px=cfg.clean_reproj_px)
        cleaned.append((ok[c], d))
    # the pruner: head of each window of five cleaned maps, later maps edited in place
    fused = {}
    maps = [d for _, d in cleaned]
    for h in range(0, len(cleaned) - 4):
        idx = [cleaned[h + q][0] for q in range(5)]
        pruned, xyz, _, ij, mutated = ctx.fuse(maps[h:h + 5], np.stack([views[k].R for k in idx]),
                                               np.stack([views[k].t for k in idx]), None, cfg.fuse_threshold)
        maps[h + 1:h + 5] = mutated[1:]
        fused[idx[0]] = (pruned, xyz, ij)
    assert len(fused) >= 1
    for k in range(len(views)):
        st, d, xyz, ij = dense[k]
        if k in fused:
            assert st == native.PM_OK, k
            pruned, hx, hij = fused[k]
            assert np.array_equal(d, pruned), k
            assert np.array_equal(ij, hij), k
            assert np.allclose(xyz, hx, rtol=0, atol=1e-6), k
            assert len(xyz) > 0
        elif res[k][0] == native.PM_OK:
            # the first two and the last keyframes: their windows never fill
            assert st == native.PM_ENOTREADY, (k, st)


def _landmarks(view, n, rng):
    """n world points on the scene surface seen from `view` and their ids
    (the pixel index), as SLAM landmarks."""
    i = rng.integers(8, H - 8, n)
    j = rng.integers(8, W - 8, n)
    d = view.depth[i, j].astype(np.float64)
    lat = -np.pi * (i / H - 0.5)
    lon = 2 * np.pi * (j / W - 0.5)
    b = np.stack([np.cos(lat) * np.sin(lon), -np.sin(lat), np.cos(lat) * np.cos(lon)], 1)
    Xc = b * d[:, None]
    Xw = (Xc - view.t[None]) @ view.R  # R^T (X_c - t)
    return Xw, (i * W + j).astype(np.uint64)


def test_landmark_view_test_and_seeding(ctx, views):
    """Each keyframe with landmarks is scored against the previous joined one
    (pm_score_view): a repeat of the previous position sees every common
    landmark at a triangulation angle of 0 and is dropped; the server's
    decisions and scores equal the host view test replayed in order, and
    joined keyframes are densified with their landmark seeds."""
    rng = np.random.default_rng(3)
    xyz, ids = _landmarks(views[0], 400, rng)
    srv = native.Server(ctx, _cfg(inflight=1, min_sources=1))
    order = [0, 0, 3, 6, 6, 9, 12]  # repeats have no baseline
    tks = [srv.submit_landmarks(views[k].gray_u8, views[k].R, views[k].t, xyz, ids) for k in order]
    res = [srv.wait(tk) for tk in tks]
    srv.close()
    centre = lambda v: -v.R.T @ v.t
    prev = None
    joined = 0
    for k, r in zip(order, res):
        v = views[k]
        if prev is None:
            assert r[3]["view_score"] == pytest.approx(-1.0)  # nothing to compare with
            prev = v
            continue
        score, _ = native.score_view(centre(prev), centre(v), ids, ids, xyz)
        assert r[3]["view_score"] == pytest.approx(score, abs=1e-6)
        if score > 0.25:
            prev = v
            joined += 1
            assert r[0] in (native.PM_OK, native.PM_ENOTREADY)
        else:
            assert r[0] == native.PM_ENOTREADY
    assert res[1][0] == native.PM_ENOTREADY and res[1][3]["view_score"] <= 0.25
    assert joined >= 2
    ok = [r for r in res if r[0] == native.PM_OK]
    assert ok
    for r in ok:
        assert np.isfinite(r[1]).all() and (r[1] > 0).mean() > 0.2


def test_wait_times_out_and_ticket_stays_collectable(ctx):
    """A 1 ms wait on a 1920x960 keyframe still on the GPU returns
    PM_ETIMEOUT; the ticket can be collected afterwards."""
    req = scene.config_request(2, seed=5)
    srv = native.Server(ctx, _cfg(inflight=1, min_sources=4, params=native.default_params(iterations=8)))
    for v in req.views[1:5]:
        srv.submit(v.gray_u8, v.R, v.t)
    tk = srv.submit(req.views[0].gray_u8, req.views[0].R, req.views[0].t)
    st, _, _, _ = srv.wait(tk, timeout_ms=1)
    assert st == native.PM_ETIMEOUT
    st, d, _, info = srv.wait(tk)
    assert st == native.PM_OK and d is not None and info["n_sources"] == 4
    srv.close()


def test_destroy_cancels_queued_keyframes_and_waits_for_waiters(ctx):
    """Destroy while keyframes are queued: those not yet on the GPU complete
    with PM_ECANCELLED (a thread blocked on one returns it), the ones on the
    GPU finish, and destroy returns only after the waiting thread has left."""
    req = scene.config_request(2, seed=6)
    # every keyframe a full 8-sweep run (no prior, no coarse-to-fine): about 60 ms each, one at a time
    srv = native.Server(ctx, _cfg(inflight=1, min_sources=1, params=native.default_params(iterations=8),
                                  seed_from_prior=0, coarse_to_fine=0))
    tks = [srv.submit(v.gray_u8, v.R, v.t) for _ in range(3) for v in req.views]
    got = {}

    def waiter(tk):
        got[tk] = srv._L.pm_server_wait(srv.h, tk, -1, None, None)

    th = threading.Thread(target=waiter, args=(tks[-1],))
    th.start()
    time.sleep(0.2)  # the waiter is inside pm_server_wait before destroy starts
    srv._L.pm_server_destroy(srv.h)  # returns only once the waiter has left pm_server_wait
    srv.h = None
    th.join(5.0)
    assert not th.is_alive()
    assert got[tks[-1]] == native.PM_ECANCELLED


def test_producer_that_never_collects_does_not_block(ctx, views):
    """One producer submits and never waits (nor returns to the server); the
    worker keeps serving another producer's keyframes."""
    srv = native.Server(ctx, _cfg(inflight=2))
    stalled = threading.Event()

    def lazy_producer():
        for v in views[:3]:
            srv.submit(v.gray_u8, v.R, v.t)
        stalled.wait(5.0)

    th = threading.Thread(target=lazy_producer)
    th.start()
    t0 = time.perf_counter()
    tks = [srv.submit(v.gray_u8, v.R, v.t) for v in views[3:9]]
    res = [srv.wait(tk, timeout_ms=20000) for tk in tks]
    assert time.perf_counter() - t0 < 20.0
    assert all(r[0] in (native.PM_OK, native.PM_ENOTREADY) for r in res)
    assert sum(r[0] == native.PM_OK for r in res) >= 4
    stalled.set()
    th.join()
    srv.close()


def test_short_points_buffer_leaves_the_ticket_collectable(ctx, views):
    """pm_server_wait_dense with a points buffer smaller than the fused cloud
    returns PM_EINVAL with the count and writes nothing; the same ticket is
    then collected with a buffer of that size and equals the full-size read
    of a second, identical server."""
    import ctypes as C
    outs, sel = [], None
    for short in (True, False):
        srv = native.Server(ctx, _cfg(dense_output=1))
        tks = [srv.submit(v.gray_u8, v.R, v.t) for v in views]
        for tk in tks:
            srv.wait(tk)
        srv.finish()
        depth = np.zeros((H, W), np.float32)
        if short:
            # the first ticket with a fused cloud (the stream's first keyframes have none)
            xyz1 = np.full((1, 3), 7.0)
            ij1 = np.full((1, 2), 7, np.int32)
            for sel, tk in enumerate(tks):
                pts = native.Points(1, 0, xyz1.ctypes.data, None, ij1.ctypes.data)
                rc = srv._L.pm_server_wait_dense(srv.h, tk, -1, depth.ctypes.data, C.byref(pts))
                if rc != native.PM_ENOTREADY:
                    break
            assert rc == native.PM_EINVAL and pts.count > 1
            assert (xyz1 == 7.0).all() and (ij1 == 7).all() and (depth == 0).all()
            n = pts.count
        else:
            n = H * W
        tk = tks[sel]
        xyz = np.zeros((n, 3), np.float64)
        ij = np.zeros((n, 2), np.int32)
        pts = native.Points(n, 0, xyz.ctypes.data, None, ij.ctypes.data)
        assert srv._L.pm_server_wait_dense(srv.h, tk, -1, depth.ctypes.data, C.byref(pts)) == native.PM_OK
        outs.append((depth.copy(), xyz[:pts.count].copy(), ij[:pts.count].copy()))
        srv.close()
    (d0, x0, i0), (d1, x1, i1) = outs
    assert len(x0) > 1 and np.array_equal(d0, d1) and np.array_equal(i0, i1) and np.array_equal(x0, x1)


def test_finish_and_destroy_from_two_threads(ctx, views):
    """A thread blocked in pm_server_finish while another destroys the server:
    destroy returns only after finish has, and both succeed."""
    srv = native.Server(ctx, _cfg(inflight=1, dense_output=1))
    for v in views[:6]:
        srv.submit(v.gray_u8, v.R, v.t)
    got = {}
    th = threading.Thread(target=lambda: got.setdefault("finish", srv._L.pm_server_finish(srv.h)))
    th.start()
    time.sleep(0.05)
    assert srv._L.pm_server_destroy(srv.h) == native.PM_OK
    srv.h = None
    th.join(10.0)
    assert not th.is_alive() and got["finish"] == native.PM_OK
