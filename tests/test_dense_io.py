"""Dense map output (pm_write_ply, pm_write_dense_msgpack) and the message
reader / PLY exporter (CPU only)."""
import numpy as np
import pytest

from patchmatch_gb300 import dense_io, native


def _cloud(n=257, seed=0):
    rng = np.random.default_rng(seed)
    return rng.normal(0, 3, (n, 3)), rng.integers(0, 256, (n, 3)).astype(np.uint8)


def _read_ply(path):
    with open(path) as f:
        lines = f.read().splitlines()
    end = lines.index("end_header")
    header = lines[:end + 1]
    rows = [l.split() for l in lines[end + 1:]]
    return header, np.array([[float(v) for v in r[:3]] for r in rows]), np.array([[int(v) for v in r[3:]] for r in rows])


def test_ply_round_trip(built, tmp_path):
    xyz, bgr = _cloud()
    p = tmp_path / "cloud.ply"
    native.write_ply(p, xyz, bgr)
    header, x, c = _read_ply(p)
    assert header[:3] == ["ply", "format ascii 1.0", f"element vertex {len(xyz)}"]
    assert header[3:9] == ["property float x", "property float y", "property float z", "property uchar red",
                           "property uchar green", "property uchar blue"]
    assert np.abs(x - xyz).max() <= 5e-7  # fixed notation, 6 decimals
    assert np.array_equal(c, bgr)
    native.write_ply(p, xyz)  # no colours: white
    assert (_read_ply(p)[2] == 255).all()
    native.write_ply(p, np.zeros((0, 3)))
    assert _read_ply(p)[1].size == 0


def test_dense_msgpack_layout(built, tmp_path):
    xyz, bgr = _cloud(40)
    p = tmp_path / "map.msg_dense"
    native.write_dense_msgpack(p, xyz, bgr, first_id=7, keyframe_id=3)
    msg = dense_io.read_dense_msg(p)
    assert list(msg) == ["cameras", "keyframes", "landmarks"]
    lms = msg["landmarks"]
    assert list(lms) == sorted(str(7 + k) for k in range(40))  # JSON-object key order
    for k in range(40):
        rec = lms[str(7 + k)]
        assert list(rec) == ["1st_keyfrm", "color", "n_fnd", "n_vis", "pos_w", "ref_keyfrm"]
        assert rec["pos_w"] == list(xyz[k]) and rec["color"] == [float(v) for v in bgr[k]]
        assert rec["1st_keyfrm"] == rec["ref_keyfrm"] == 3
    mp = pytest.importorskip("msgpack")
    with open(p, "rb") as f:
        assert mp.unpackb(f.read(), raw=False) == msg


def test_msg_to_ply_matches_reference_exporter_format(built, tmp_path):
    xyz, bgr = _cloud(12, seed=3)
    p = tmp_path / "map.msg_dense"
    native.write_dense_msgpack(p, xyz, bgr, first_id=0)
    out = dense_io.msg_to_ply(p)
    with open(out) as f:
        lines = f.read().splitlines()
    body = lines[lines.index("end_header") + 1:]
    order = sorted(range(12), key=str)  # records in key order
    for line, k in zip(body, order):
        assert line == "{:.4f} {:.4f} {:.4f} {} {} {}".format(*xyz[k], *bgr[k])
    out2 = dense_io.msg_to_ply(p, tmp_path / "w.ply", nocolor=True)
    with open(out2) as f:
        assert f.read().splitlines()[-1].endswith(" 255 255 255")


def test_write_errors(built, tmp_path):
    with pytest.raises(native.PmError):
        native.write_ply(tmp_path / "no" / "such" / "dir.ply", np.zeros((1, 3)))
    with pytest.raises(ValueError):
        native.write_ply(tmp_path / "x.ply", np.zeros((2, 3)), np.zeros((1, 3)))
