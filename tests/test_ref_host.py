"""The oracle's restatements of the reference's host stages against the
reference's own code: PostProcess, DepthmapCleaner::Clean and
DepthmapPruner::Prune of src/openvslam/depthmap.cc, compiled unmodified
against a minimal OpenCV stand-in (oracle/refhost.py).  Checked live where
the reference sources exist and against the golden fixture generated from
them (tests/golden/make_golden_host.py) everywhere."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from patchmatch_gb300 import scene

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_host_96x48.npz")


@pytest.fixture(scope="module")
def gold():
    if not os.path.exists(FIX):
        pytest.skip("golden fixture not generated")
    return dict(np.load(FIX))


@pytest.mark.parametrize("case", [0, 1])
def test_oracle_clean_equals_reference_golden(gold, case):
    d = list(gold[f"c{case}_depths"])
    thr = float(gold[f"c{case}_thr"][0])
    o = O.clean(d, gold[f"c{case}_R"], gold[f"c{case}_t"], center=2, thr=thr, min_consistent=3)
    assert np.array_equal(o, gold[f"c{case}_clean"])
    assert (o > 0).mean() > 0.3


@pytest.mark.parametrize("case", [0, 1])
def test_oracle_prune_equals_reference_golden(gold, case):
    d = list(gold[f"c{case}_depths"])
    thr = float(gold[f"c{case}_thr"][1])
    pruned, xyz, cols, ij, _ = O.prune(d, gold[f"c{case}_R"], gold[f"c{case}_t"], gold[f"c{case}_bgr"], thr)
    assert np.array_equal(pruned, gold[f"c{case}_pruned"])
    assert np.array_equal(ij, gold[f"c{case}_ij"]) and np.array_equal(cols, gold[f"c{case}_colors"])
    assert len(xyz) > 0 and np.abs(xyz - gold[f"c{case}_xyz"]).max() < 1e-5  # metres


@pytest.mark.parametrize("case", [0, 1])
def test_oracle_postprocess_equals_reference_golden(gold, case):
    d, s = gold[f"c{case}_post_in_depth"], gold[f"c{case}_post_in_score"]
    ref = np.zeros_like(d)  # the variance mask is off: intensities are not read
    od, osc = O.postprocess(ref, d, s, patch_half=1, min_depth=0.3, max_depth=20.0, min_score=0.1)
    assert np.array_equal(od, gold[f"c{case}_post_depth"])
    assert np.array_equal(osc, gold[f"c{case}_post_score"])
    assert (od > 0).mean() > 0.3


def test_oracle_equals_reference_host_code_live():
    """Fresh inputs through the reference's compiled host stages and the
    oracle (skipped where the reference sources are absent)."""
    from oracle import refhost
    if not refhost.available():
        pytest.skip("reference sources not present")
    for seed in (11, 12):
        req = scene.make_request(scene.ROOM_OBJECTS, 128, 64, 4, seed=seed, bmin=0.05, bmax=0.5)
        rng = np.random.default_rng(seed)
        d = [(v.depth * (1 + rng.normal(0, 0.006, v.depth.shape))).astype(np.float32) for v in req.views]
        for x in d:
            x[rng.random(x.shape) < 0.08] = 0
        for thr in (0.01, 0.05):
            assert np.array_equal(refhost.clean(d, req.R, req.t, thr, 3),
                                  O.clean(d, req.R, req.t, center=2, thr=thr, min_consistent=3))
            rp = refhost.prune(d, req.R, req.t, req.views[0].rgb, thr)
            op = O.prune(d, req.R, req.t, req.views[0].rgb, thr)
            assert np.array_equal(rp[0], op[0]) and np.array_equal(rp[3], op[3])
            assert np.abs(rp[1] - op[1]).max() < 1e-5
