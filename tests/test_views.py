"""Neighbour geometry on the host (pm_score_view, pm_depth_interval) against
the oracle's restatement of the reference (CPU only)."""
import numpy as np
import pytest

from oracle import oracle as O
from patchmatch_gb300 import native


def _landmarks(rng, n, spread=8.0):
    return rng.uniform(-spread, spread, (n, 3))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_score_view_matches_oracle(built, seed):
    rng = np.random.default_rng(seed)
    xyz = _landmarks(rng, 500)
    ids = rng.permutation(100000)[:500].astype(np.uint64)
    prev_ids = np.concatenate([ids[:350], rng.integers(200000, 300000, 80).astype(np.uint64)])
    cur_sel = rng.permutation(500)[:420]
    cur_ids, cur_xyz = ids[cur_sel], xyz[cur_sel]
    pc = np.array([0.0, 0.0, 0.0])
    cc = rng.normal(0, 1.0, 3)
    s, n = native.score_view(pc, cc, prev_ids, cur_ids, cur_xyz)
    so, no = O.score_view(pc, cc, prev_ids, cur_ids, cur_xyz)
    assert n == no == len(set(prev_ids.tolist()) & set(cur_ids.tolist()))
    assert s == pytest.approx(so, abs=1e-7)
    assert 0.0 < s < 1.0


def test_score_view_edges(built):
    pc, cc = np.zeros(3), np.array([1.0, 0, 0])
    # nothing in common -> 0 (the reference would divide 0 by 0)
    assert native.score_view(pc, cc, [1, 2], [3], [[0, 0, 5.0]]) == (0.0, 0)
    # duplicates of one id count once; a landmark at 5 m seen across 1 m: ~11 degrees -> inside
    s, n = native.score_view(pc, cc, [7], [7, 7], [[0.5, 0, 5.0], [0.5, 0, 5.0]])
    assert (s, n) == (1.0, 1)
    # far landmark: angle below 3 degrees -> outside
    assert native.score_view(pc, cc, [7], [7], [[0.5, 0, 50.0]])[0] == 0.0
    with pytest.raises(ValueError):
        native.score_view(pc, cc, [1], [1], np.zeros((0, 3)))  # ids without positions
    L = native.lib()
    assert L.pm_score_view(None, None, None, 0, None, None, 0, None, None) == native.PM_EINVAL


def test_depth_interval_matches_oracle(built):
    rng = np.random.default_rng(5)
    for n in (1, 9, 10, 11, 1234):
        xyz = _landmarks(rng, n)
        R = np.linalg.qr(rng.normal(size=(3, 3)))[0]
        t = rng.normal(size=3)
        got = native.depth_interval(R, t, xyz)
        exp = O.depth_interval(R, t, xyz)
        assert got == pytest.approx(exp, rel=1e-12)
        assert got[2] == 1e-5 and got[3] == pytest.approx(1.1 * got[1])
    with pytest.raises(native.PmError):
        native.depth_interval(np.eye(3), np.zeros(3), np.zeros((0, 3)))
