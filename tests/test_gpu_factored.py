"""The factored warp of the tile kernel (9 and 10 sources) and the direct
rotation (fewer sources), through the C ABI.

The tile kernel stages per-column and per-row factors of M_r b in shared
memory; the fixed-hypothesis kernel evaluates the same factored arithmetic
from the trig tables.  So the tile kernel's init scores of each pixel's own
plane must equal the fixed-hypothesis scores of the same planes bit for bit,
at every source count and with either sampler; and half-sweeps from an
identical state must pick the oracle's planes as they do with fewer sources.
"""
import numpy as np
import pytest

from oracle import oracle as O
from patchmatch_gb300 import native, scene

pytestmark = pytest.mark.gpu

W, H = 192, 96


def _request(ctx, req, **kw):
    p = native.default_params(**kw)
    r = ctx.request(req.W, req.H, req.n_src, p)
    r.set_views([v.gray_u8 for v in req.views], req.R, req.t)
    return r


@pytest.mark.parametrize("sampler", [native.SAMPLER_EXACT, native.SAMPLER_TEXTURE])
@pytest.mark.parametrize("n_src,w,h", [(4, W, H), (8, W, H), (10, W, H), (9, 131, 67)])
def test_tile_scores_equal_fixed_hypothesis_scores(ctx, n_src, w, h, sampler):
    """131x67 leaves the last tile column and row partly off the image, where
    the staged factors of off-image columns and rows are 0."""
    req = scene.make_request(scene.ROOM_OBJECTS, w, h, n_src, seed=60 + n_src, bmin=0.1, bmax=0.6)
    r = _request(ctx, req, sampler=sampler, iterations=0, postprocess=0)
    r.init()
    g = r.read(raw=True)
    ph = 5
    ii, jj = np.mgrid[ph + 1:h - ph, ph + 1:w - ph]
    ij = np.stack([ii.ravel(), jj.ravel()], 1).astype(np.int32)
    planes = np.ascontiguousarray(g["plane"][ii.ravel(), jj.ravel(), :3], np.float32)
    s, best = r.score_hypotheses(ij, planes)
    r.close()
    tile = g["score"][ii.ravel(), jj.ravel()]
    same = (s == tile) | (np.isnan(s) & np.isnan(tile))
    print(f"S={n_src} sampler={sampler}: identical scores {same.mean():.6f} of {len(s)}")
    assert same.all()
    assert (best == g["best_view"][ii.ravel(), jj.ravel()]).all()


@pytest.mark.parametrize("n_src", [9, 10])
def test_factored_half_sweeps_match_oracle(ctx, n_src):
    """One red and one black half-sweep from an identical state with the
    factored warp: the chosen planes match the FP64 oracle's except where two
    candidate scores tie to within FP32-vs-FP64 error (>= 98 %, as with the
    direct rotation)."""
    req = scene.make_request(scene.ROOM, W, H, n_src, seed=70 + n_src)
    r = _request(ctx, req, sampler=native.SAMPLER_EXACT, iterations=0, postprocess=0)
    r.init()
    s0 = r.read(raw=True)
    V = O.Views.from_request(req)
    o = O.sweeps(V, O.cost_params(), s0["plane"], s0["depth"], s0["score"], s0["best_view"], 0, 2)
    r.set_state(s0["plane"], s0["score"])
    r.sweep(0, 2)
    g = r.read(raw=True)
    r.close()
    interior = np.zeros((H, W), bool)
    interior[6:H - 5, 6:W - 5] = True
    same = np.all(np.abs(g["plane"] - o["plane"]) <= 1e-4 * np.abs(o["plane"]) + 1e-7, axis=2)[interior]
    print(f"S={n_src}: half-sweep identical-plane fraction {same.mean():.5f}")
    assert same.mean() >= 0.98
