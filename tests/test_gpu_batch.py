"""The batched executor (pm_batch): requests of uneven size, source count,
sampler and propagation rule densified together give exactly the maps of
pm_request_run, whichever executor runs them."""
import numpy as np
import pytest

from patchmatch_gb300 import native, scene

pytestmark = pytest.mark.gpu

SPECS = [  # (W, H, sources, seed, extra params)
    (256, 128, 2, 1, {}),
    (384, 192, 3, 2, {}),
    (256, 128, 2, 3, {}),
    (320, 160, 4, 4, {"sampler": native.SAMPLER_EXACT}),
    (192, 96, 3, 5, {"propagation": native.PROPAGATION_PLAIN}),
    (512, 256, 5, 6, {"iterations": 3}),
]


@pytest.fixture(scope="module")
def batch_requests():
    return [scene.make_request(scene.ROOM_OBJECTS, W, H, S, seed=seed) for W, H, S, seed, _ in SPECS]


def _make(ctx, reqs):
    out = []
    for (W, H, S, seed, extra), req in zip(SPECS, reqs):
        kw = {"iterations": 2, **extra}
        p = native.default_params(seed=seed, keyframe_id=seed, **kw)
        r = ctx.request(W, H, S, p)
        r.set_views([v.gray_u8 for v in req.views], req.R, req.t)
        out.append(r)
    return out


def test_batch_equals_individual_runs(ctx, batch_requests):
    rs = _make(ctx, batch_requests)
    alone = []
    for r in rs:
        r.run()
        alone.append(r.read(want=("depth", "score", "plane")))
    b = native.Batch(ctx, rs)
    for executor, mult in ((native.BATCH_PERSISTENT, 1), (native.BATCH_PERSISTENT, 2), (native.BATCH_LAUNCHES, 1),
                           (native.BATCH_STREAMS, 1), (native.BATCH_MIXED, 1)):
        b.set_executor(executor, mult)
        b.run()
        for r, a in zip(rs, alone):
            got = r.read(want=("depth", "score", "plane"))
            for k in ("depth", "score", "plane"):
                assert np.array_equal(got[k], a[k]), (executor, mult, k, r.W, r.S)
    t = b.tune()
    print("tuning:", t)
    assert t["executor"] in (native.BATCH_PERSISTENT, native.BATCH_LAUNCHES, native.BATCH_STREAMS,
                             native.BATCH_MIXED) and t["ms"] > 0
    b.run()
    assert np.array_equal(rs[1].read(want=("depth",))["depth"], alone[1]["depth"])
    # new views (another scene, other poses) on a request: every executor follows
    other = scene.make_request(scene.ROOM, 256, 128, 2, seed=9)
    rs[0].set_views([v.gray_u8 for v in other.views], other.R, other.t)
    rs[0].run()
    solo = rs[0].read(want=("depth",))["depth"]
    for executor in (native.BATCH_PERSISTENT, native.BATCH_LAUNCHES, native.BATCH_STREAMS, native.BATCH_MIXED):
        b.set_executor(executor, 1)
        b.run()
        assert np.array_equal(rs[0].read(want=("depth",))["depth"], solo), executor
    b.close()
    for r in rs:
        r.close()


def _landmarks(view, W, H, n, rng):
    i = rng.integers(8, H - 8, n)
    j = rng.integers(8, W - 8, n)
    d = view.depth[i, j].astype(np.float64)
    lat = -np.pi * (i / H - 0.5)
    lon = 2 * np.pi * (j / W - 0.5)
    b = np.stack([np.cos(lat) * np.sin(lon), -np.sin(lat), np.cos(lat) * np.cos(lon)], 1)
    return (b * d[:, None] - view.t[None]) @ view.R


def test_seeded_batch_equals_individual_runs(ctx):
    """Seeded requests in a batch: a coarse-to-fine chain (the full-size
    request seeded from a half-size request of the same batch), a request
    seeded from SLAM landmarks, one from a retained result and one from a
    request outside the batch.  Every executor gives the maps of the same
    requests run one at a time in dependency order, bit for bit."""
    sc = scene.Scene(scene.ROOM_OBJECTS, 44)
    R, t = sc.poses(4, 44, 0.2, 0.5, 15.0)
    full = [sc.render(R[k], t[k], 512, 256) for k in range(4)]
    half = [sc.render(R[k], t[k], 256, 128) for k in range(4)]
    other = scene.make_request(scene.ROOM_OBJECTS, 384, 192, 3, seed=45)

    def req(W, H, views, Rs, ts, it, kf):
        r = ctx.request(W, H, len(views) - 1, native.default_params(iterations=it, keyframe_id=kf, seed=kf))
        r.set_views([v.gray_u8 for v in views], Rs, ts)
        return r

    coarse = req(256, 128, half, R, t, 6, 1)
    fine = req(512, 256, full, R, t, 2, 2)
    fine.set_prior(coarse)
    lmk = req(512, 256, full, R, t, 2, 3)
    lmk.set_landmarks(_landmarks(full[0], 512, 256, 300, np.random.default_rng(1)))
    outside = req(384, 192, other.views, other.R, other.t, 3, 4)
    from_req = req(384, 192, other.views, other.R, other.t, 2, 5)
    from_req.set_prior(outside)
    res = native.Result(ctx, 384, 192)
    from_res = req(384, 192, other.views, other.R, other.t, 2, 6)
    from_res.set_prior(res)
    plain = req(256, 128, half, R, t, 3, 7)
    outside.run()
    res.snapshot(outside)
    outside.synchronize()
    batch = [coarse, fine, lmk, from_req, from_res, plain]
    alone = []
    for r in batch:  # dependency order: the coarse pass before the fine one
        r.run()
        r.synchronize()
        alone.append(r.read(raw=True, want=("depth", "score", "plane")))
    b = native.Batch(ctx, batch)
    for executor, mult in ((native.BATCH_PERSISTENT, 1), (native.BATCH_LAUNCHES, 1), (native.BATCH_STREAMS, 1),
                           (native.BATCH_MIXED, 1)):
        b.set_executor(executor, mult)
        b.run()
        b.synchronize()
        for r, a in zip(batch, alone):
            got = r.read(raw=True, want=("depth", "score", "plane"))
            for k in ("depth", "score", "plane"):
                assert np.array_equal(got[k], a[k]), (executor, k, r.W, r.S)
    b.close()
    for r in batch + [outside]:
        r.close()
    res.close()


def test_batch_rejects_a_cycle_of_priors(ctx, batch_requests):
    rs = _make(ctx, batch_requests[:2])
    rs[0].set_prior(rs[1])
    rs[1].set_prior(rs[0])
    b = native.Batch(ctx, rs)
    with pytest.raises(native.PmError) as e:
        b.run()
    assert e.value.status == native.PM_EINVAL
    rs[0].set_prior(None)
    rs[1].set_prior(None)
    b.run()
    b.synchronize()
    with pytest.raises(native.PmError):
        b.add(rs[0])  # already in the batch
    b.close()
    for r in rs:
        r.close()


def test_request_in_a_batch_cannot_be_destroyed(ctx):
    """pm_request_destroy refuses a request a batch still holds (the batch
    would run on freed memory); clearing the batch releases it."""
    req = scene.make_request(scene.ROOM, 128, 64, 2, seed=5)
    r = ctx.request(128, 64, 2, native.default_params(iterations=2))
    r.set_views([v.gray_u8 for v in req.views], req.R, req.t)
    b = native.Batch(ctx, [r])
    with pytest.raises(native.PmError) as e:
        r.close()
    assert e.value.status == native.PM_EINVAL
    b.run()
    b.synchronize()
    b.clear()
    r.close()
    b.close()


@pytest.mark.parametrize("fmt", [native.IMAGE_U8, native.IMAGE_F16])
def test_banded_tile_order_equals_one_cta_per_tile(ctx, fmt):
    """Wide texture-sampled requests (source row bytes W x texel bytes x S of
    at least 30,000: here 2048 x 2 x 8 for FP16, 3840 x 1 x 8 for u8) run their
    sweeps in the banded persistent tile order; the persistent batch executor
    takes (request, tile) items from its own queue in raster order.  Tiles of
    a half-sweep are independent, so the maps are identical bit for bit."""
    W = 2048 if fmt == native.IMAGE_F16 else 3840
    H, S = W // 2, 8
    req = scene.make_request(scene.ROOM_OBJECTS, W, H, S, seed=31)
    r = ctx.request(W, H, S, native.default_params(iterations=2, image_format=fmt))
    imgs = [v.gray.astype(np.float16) if fmt == native.IMAGE_F16 else v.gray_u8 for v in req.views]
    r.set_views(imgs, req.R, req.t)
    r.run()
    banded = r.read(raw=True)
    b = native.Batch(ctx, [r])
    b.set_executor(native.BATCH_PERSISTENT, 1)
    b.run()
    b.synchronize()
    per_tile = r.read(raw=True)
    b.close()
    r.close()
    for k in ("plane", "score", "depth"):
        assert np.array_equal(banded[k], per_tile[k]), k
