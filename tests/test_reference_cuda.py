"""The product against the reference's own CUDA path (PatchMatchCuda.cu compiled
unmodified into oracle/_ref, launched by oracle/ref_harness.cu).

The reference supports exactly two sources and seeds cuRAND from clock64(),
so its runs are not reproducible; converged maps are compared.  Skipped when
the reference kernels were not built (their sources live outside this
repository)."""
import numpy as np
import pytest

from oracle import oracle as O
from patchmatch_gb300 import native, scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rk(built):
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip("reference kernels not built")
    return refkernels.RefKernels()


def test_reference_cost_matches_oracle_tex8(rk):
    """ScorePlaneDepth_ of the reference vs the oracle's float replay with
    texture-unit interpolation weights, on fresh hypotheses."""
    req = scene.make_request(scene.ROOM, 256, 128, 2, seed=31)
    imgs = [v.gray_u8.astype(np.float32) for v in req.views]
    rk.setup(imgs, req.R, req.t)
    rng = np.random.default_rng(4)
    v0 = req.views[0]
    H, W = 128, 256
    P = np.zeros((H, W, 3), np.float32)
    for i in range(H):
        for j in range(W):
            P[i, j] = O.gt_plane(v0.depth[i, j], v0.normal[i, j], W, H, i, j)
    P *= rng.uniform(0.9, 1.1, (H, W, 1)).astype(np.float32)
    ref = rk.score(P)
    m = np.zeros((H, W), bool)
    m[6:H - 5, 6:W - 5] = True
    ii, jj = np.nonzero(m)
    ij = np.stack([ii, jj], 1).astype(np.int32)
    V = O.Views(imgs[0], imgs[1:], req.R, req.t)
    errs = {}
    for interp in (O.INTERP_TEX8_RN, O.INTERP_TEX8_RZ, O.INTERP_EXACT):
        o, _ = O.cost_batch(V, O.cost_params(arith=O.ARITH_F32_REF, interp=interp), ij, P[ii, jj])
        errs[interp] = np.abs(o - ref[ii, jj])
        print(f"interp {interp}: median {np.median(errs[interp]):.2e} p99 {np.quantile(errs[interp], .99):.2e}")
    assert min(errs, key=lambda k: np.median(errs[k])) == O.INTERP_TEX8_RN
    assert np.median(errs[O.INTERP_TEX8_RN]) < 1e-4


def test_converged_depth_agrees_with_reference_gpu_path(rk, ctx):
    """Full runs at 512x256 with the reference's two sources and fold rule:
    fraction of pixels valid in both whose depths agree within 1 %."""
    req = scene.make_request(scene.ROOM, 512, 256, 2, seed=32)
    imgs = [v.gray_u8 for v in req.views]
    rk.setup([im.astype(np.float32) for im in imgs], req.R, req.t)
    iters = 8
    ref = rk.run(iters, 0.3, 20.0)
    p = native.default_params(iterations=iters, postprocess=0, init_mode=native.INIT_REF_UNIFORM)
    r = ctx.request(512, 256, 2, p)
    r.set_views(imgs, req.R, req.t)
    r.run()
    ours = r.read(raw=True)
    gt = req.views[0].depth
    m = np.zeros((256, 512), bool)
    m[6:251, 6:507] = True
    # pixels both methods resolved (score above the post-filter's 0.1 floor)
    both = m & (ref["score"] > 0.1) & (ours["score"] > 0.1)
    agree = (np.abs(ours["depth"] - ref["depth"]) / ref["depth"] < 0.01)[both].mean()
    acc_ref = (np.abs(ref["depth"] - gt) / gt < 0.01)[both].mean()
    acc_ours = (np.abs(ours["depth"] - gt) / gt < 0.01)[both].mean()
    print(f"resolved {both.mean():.3f} agree1% {agree:.4f} ref-acc1% {acc_ref:.4f} ours-acc1% {acc_ours:.4f}")
    assert agree >= 0.9
    assert acc_ours >= acc_ref - 0.02
    r.close()
