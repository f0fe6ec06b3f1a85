"""Scene ingestion and image output (host only)."""
import numpy as np
import pytest


def test_obj_load_faces_and_index_forms(rt, tmp_path):
    p = tmp_path / "m.obj"
    p.write_text("""# comment
o first
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vt 0 0
vn 0 0 1
usemtl x
f 1/1/1 2/1/1 3/1/1 4/1/1
o second
v 0 0 1
v 1 0 1
v 0 1 1
f -3//1 -2//1 -1//1
f 5 6 7
""")
    t = rt.load_obj(p, material=3)
    assert len(t) == 4
    v = lambda i, k: tuple(t[i][k][:3])
    # quad fanned from its first vertex: (1,2,3), (1,3,4)
    assert (v(0, "v0"), v(0, "v1"), v(0, "v2")) == ((0, 0, 0), (1, 0, 0), (1, 1, 0))
    assert (v(1, "v0"), v(1, "v1"), v(1, "v2")) == ((0, 0, 0), (1, 1, 0), (0, 1, 0))
    assert (v(2, "v0"), v(2, "v1"), v(2, "v2")) == ((0, 0, 1), (1, 0, 1), (0, 1, 1))
    assert np.array_equal(t[2:3].view(np.uint8), t[3:4].view(np.uint8))
    assert set(t["materialIndex"]) == {3}
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 2 3\n")
    with pytest.raises(rt.RtError):
        rt.load_obj(bad)
    with pytest.raises(rt.RtError) as e:
        rt.load_obj(tmp_path / "missing.obj")
    assert e.value.status == 8


def test_model_matrix_is_translate_ry_rx_rz_scale(rt):
    tr, rot, sc = (1.5, -2.0, 0.25), (0.3, -1.1, 2.0), (2.0, 0.5, 3.0)
    m = rt.model_matrix(tr, rot, sc)["m"][0].reshape(4, 4).T.astype(np.float64)  # row-major view
    x, y, z = rot

    def R(axis, a):
        c, s = np.cos(a), np.sin(a)
        return {"x": np.array([[1, 0, 0], [0, c, -s], [0, s, c]]), "y": np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]]),
                "z": np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])}[axis]

    ref = np.eye(4)
    ref[:3, :3] = R("y", y) @ R("x", x) @ R("z", z) @ np.diag(sc)
    ref[:3, 3] = tr
    assert np.allclose(m, ref, atol=1e-6)


def test_write_images(rt, tmp_path):
    w, h = 5, 3
    img = np.zeros((h, w, 4), np.float32)
    img[0, 0, :3] = (1.0, 0.5, 0.0)
    img[2, 4, :3] = (0.0, 0.25, 1.0)
    rt.write_image(tmp_path / "a.ppm", img, w, h)
    data = (tmp_path / "a.ppm").read_bytes()
    header = b"P6\n5 3\n255\n"
    assert data.startswith(header)
    px = np.frombuffer(data[len(header):], np.uint8).reshape(h, w, 3)
    assert tuple(px[0, 0]) == (255, 128, 0) and tuple(px[2, 4]) == (0, 64, 255)
    rt.write_image(tmp_path / "a.pfm", img, w, h)
    d = (tmp_path / "a.pfm").read_bytes()
    hdr = b"PF\n5 3\n-1.0\n"
    f = np.frombuffer(d[len(hdr):], "<f4").reshape(h, w, 3)
    assert np.array_equal(f[::-1], img[..., :3])  # bottom row first
