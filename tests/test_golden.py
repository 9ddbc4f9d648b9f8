"""Oracle against golden vectors produced by the reference's own CUDA kernels
(tests/golden/make_golden.py runs PatchMatchCuda.cu, compiled unmodified, on a
GB300).  CPU only: replays the stored inputs through the oracle."""
import os

import numpy as np
import pytest

from oracle import oracle as O

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kernels_128x64.npz")


@pytest.fixture(scope="module")
def gold():
    if not os.path.exists(FIX):
        pytest.skip("golden fixture not generated")
    O.build()
    return dict(np.load(FIX))


def _interior(H, W, ph=5):
    m = np.zeros((H, W), bool)
    m[ph + 1:H - ph, ph + 1:W - ph] = True
    return m


def test_bearing_table_matches_reference(gold):
    b = gold["bearings"]
    H, W, _ = b.shape
    ours = np.array([[O.bearing_ref_f32(W, H, i, j) for j in range(W)] for i in range(H)])
    assert np.abs(ours - b).max() < 2e-7
    exact = np.array([[O.bearing64(W, H, i, j) for j in range(W)] for i in range(H)])
    assert np.abs(exact - b).max() < 1e-6


def test_texture_border_is_clamp(gold):
    """The reference requests cudaAddressModeWrap with unnormalised
    coordinates; the hardware clamps (wrap needs normalised coordinates), so
    the oracle's SEAM_CLAMP is the reference behaviour."""
    src = gold["images"][1].astype(np.float32)
    H, W = src.shape
    xy = gold["probe_xy"]
    got = gold["probe"]
    # texture coordinate x samples texel centres at k + 0.5; clamp-to-edge
    u = np.clip(xy[:, 0] - 0.5, 0, W - 1)
    v = np.clip(xy[:, 1] - 0.5, 0, H - 1)
    x0 = np.floor(u).astype(int)
    y0 = np.floor(v).astype(int)
    x1 = np.minimum(x0 + 1, W - 1)
    y1 = np.minimum(y0 + 1, H - 1)
    ax, ay = u - x0, v - y0
    clamp = (1 - ay) * ((1 - ax) * src[y0, x0] + ax * src[y0, x1]) + ay * ((1 - ax) * src[y1, x0] + ax * src[y1, x1])
    assert np.abs(clamp - got).max() < 1.0  # 8-bit texture weights


@pytest.mark.parametrize("interp", [O.INTERP_TEX8_RN, O.INTERP_TEX8_RZ, O.INTERP_EXACT])
def test_cost_replays_reference_kernel(gold, interp):
    """ScorePlaneDepth_ on fixed planes: the oracle in the reference's float
    arithmetic with texture-unit (8-bit) interpolation weights reproduces the
    reference kernel's scores; exact interpolation differs only by the
    texture weight quantisation."""
    imgs = gold["images"].astype(np.float32)
    H, W = imgs[0].shape
    V = O.Views(imgs[0], imgs[1:], gold["R"], gold["t"])
    m = _interior(H, W)
    ii, jj = np.nonzero(m)
    ij = np.stack([ii, jj], 1).astype(np.int32)
    planes = gold["planes"][ii, jj]
    ref = gold["scores"][ii, jj]
    ours, _ = O.cost_batch(V, O.cost_params(arith=O.ARITH_F32_REF, interp=interp), ij, planes)
    err = np.abs(ours - ref)
    print(f"interp={interp}: median {np.median(err):.2e} p99 {np.quantile(err, .99):.2e} max {err.max():.2e}")
    if interp == O.INTERP_EXACT:
        assert np.median(err) < 2e-3
    else:
        assert np.median(err) < 1e-4
