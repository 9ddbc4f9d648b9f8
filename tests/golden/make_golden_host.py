"""Generate tests/golden/ref_host_96x48.npz: inputs and outputs of the
reference's own host stages (PostProcess, DepthmapCleaner::Clean,
DepthmapPruner::Prune of src/openvslam/depthmap.cc, compiled unmodified by
oracle/refhost.py) on seeded synthetic depth maps, so that the oracle and the
GPU stages can be checked against them where the reference is absent.

    python tests/golden/make_golden_host.py [out_dir]     (needs the reference sources)
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refhost  # noqa: E402
from patchmatch_gb300 import scene  # noqa: E402

W, H = 96, 48


def inputs(seed):
    req = scene.make_request(scene.ROOM_OBJECTS, W, H, 4, seed=seed, bmin=0.1, bmax=0.4)
    rng = np.random.default_rng(seed)
    depths = []
    for v in req.views:
        d = (v.depth * (1 + rng.normal(0, 0.004, v.depth.shape))).astype(np.float32)
        d[rng.random(d.shape) < 0.1] = 0
        depths.append(d)
    return req, np.stack(depths), rng


def main(out_dir):
    if not refhost.available():
        raise SystemExit("the reference sources are needed to generate this fixture")
    out = {}
    for case, (seed, thr_c, thr_p) in enumerate([(3, 0.01, 0.02), (4, 0.03, 0.08)]):
        req, depths, rng = inputs(seed)
        out[f"c{case}_depths"] = depths
        out[f"c{case}_R"] = req.R
        out[f"c{case}_t"] = req.t
        out[f"c{case}_bgr"] = req.views[0].rgb
        out[f"c{case}_thr"] = np.array([thr_c, thr_p])
        out[f"c{case}_clean"] = refhost.clean(list(depths), req.R, req.t, thr_c, 3)
        pr, xyz, cols, ij = refhost.prune(list(depths), req.R, req.t, req.views[0].rgb, thr_p)
        out[f"c{case}_pruned"], out[f"c{case}_xyz"], out[f"c{case}_colors"], out[f"c{case}_ij"] = pr, xyz, cols, ij
        # post-filter input: zero outside rows/cols [1, N-5) (the oracle's window at patch_half 1)
        d = (req.views[0].depth * (1 + rng.normal(0, 0.02, (H, W)))).astype(np.float32)
        d[rng.random(d.shape) < 0.05] = 0
        s = rng.uniform(-0.2, 1.0, (H, W)).astype(np.float32)
        win = np.zeros((H, W), bool)
        win[1:H - 5, 1:W - 5] = True
        d[~win] = 0
        s[~win] = -1
        plane = np.zeros((H, W, 3))
        plane[..., 2] = 1.0
        out[f"c{case}_post_in_depth"], out[f"c{case}_post_in_score"] = d, s
        out[f"c{case}_post_depth"], out[f"c{case}_post_score"] = refhost.postprocess(d, s, plane, 0.3, 20.0, 0.1)
    path = os.path.join(out_dir, "ref_host_96x48.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
