"""Generate golden vectors from the reference's own CUDA kernels.

Runs PatchMatchCuda.cu of the reference (compiled unmodified into
oracle/_ref/refpm_sm103a.fatbin by oracle/refkernels.py) on a GPU and stores
small fixtures that the CPU tests replay against the oracle:

  ref_kernels_128x64.npz
    images (3, 64, 128) u8      reference view + 2 sources (seeded room scene)
    R (3, 3, 3), t (3, 3)       world->camera poses
    bearings (64, 128, 3) f32   output of ComputeBearingsEquirect_
    planes (64, 128, 3) f32     fixed plane hypotheses (perturbed ground truth)
    scores (64, 128) f32        output of ScorePlaneDepth_ on those planes
    probe_xy (n, 2), probe (n,) linear-filtered texture reads of source 1 past
                                the image borders (the hardware border policy)

    python tests/golden/make_golden.py [out_dir]     (needs a GPU and the fatbin;
                                                      default out_dir: tests/golden)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle import refkernels  # noqa: E402
from patchmatch_gb300 import scene  # noqa: E402


def planes_for(req, seed):
    H, W = req.H, req.W
    v0 = req.views[0]
    rng = np.random.default_rng(seed)
    P = np.zeros((H, W, 3), np.float32)
    for i in range(H):
        for j in range(W):
            P[i, j] = O.gt_plane(v0.depth[i, j], v0.normal[i, j], W, H, i, j)
    scale = rng.uniform(0.85, 1.15, (H, W, 1)).astype(np.float32)
    tilt = rng.normal(0, 0.1, (H, W, 3)).astype(np.float32) * np.linalg.norm(P, axis=2, keepdims=True)
    return (P * scale + tilt * (rng.random((H, W, 1)) < 0.5)).astype(np.float32)


def main():
    req = scene.make_request(scene.ROOM, 128, 64, 2, seed=21)
    rk = refkernels.RefKernels()
    imgs = [v.gray_u8 for v in req.views]
    rk.setup([im.astype(np.float32) for im in imgs], req.R, req.t)
    planes = planes_for(req, 0)
    scores = rk.score(planes)
    bearings = rk.bearings()
    xs = np.array([-1.0, -0.5, 0.0, 0.25, 0.5, 1.0, 126.5, 127.0, 127.25, 127.5, 127.75, 128.0, 128.5, 129.0, 130.0])
    probe_xy = np.stack(np.meshgrid(xs, np.array([10.5, 30.25])), -1).reshape(-1, 2).astype(np.float32)
    probe = rk.probe_texture(1, probe_xy)
    out_dir = sys.argv[1] if len(sys.argv) > 1 else HERE
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "ref_kernels_128x64.npz")
    np.savez_compressed(out, images=np.stack(imgs), R=req.R, t=req.t, bearings=bearings, planes=planes,
                        scores=scores, probe_xy=probe_xy, probe=probe)
    print("wrote", out)


if __name__ == "__main__":
    main()
