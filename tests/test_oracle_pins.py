"""Pin the C++ oracle to the reference's own golden images and test vectors.

Each test restates one test of the retrofire tree (file:line given) against
the fixtures that tests/golden/make_goldens.py extracted from it.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from retrofire_gb300 import mat
from retrofire_gb300.rand import Xorshift64

FLAT, GOURAUD, TEXTURED, TEX_GOURAUD, GOURAUD_SRGB = range(5)
REPEAT_POT, CLAMP, ONCE = range(3)
ARGB, XRGB, RGBA, BGRA = range(4)


def rgba(r, g, b, a=0xFF):
    return r | (g << 8) | (b << 16) | (a << 24)


@pytest.fixture(scope="module")
def vectors(golden_dir):
    with open(os.path.join(golden_dir, "reference_vectors.json")) as f:
        return json.load(f)


def xrgb_to_rgb(img):
    return np.stack([(img >> 16) & 0xFF, (img >> 8) & 0xFF, img & 0xFF], -1).astype(np.uint8)


def textured_quad_scene():
    """core/tests/rendering.rs:10-40."""
    verts = np.array([[-1, -1, 0, 0, 0], [1, -1, 0, 0, 1],
                      [-1, 1, 0, 1, 0], [1, 1, 0, 1, 1]], np.float32)
    faces = np.array([[0, 1, 2], [3, 2, 1]], np.uint32)
    y, x = np.mgrid[0:8, 0:8]
    xor = ((x ^ y) & 1).astype(np.uint32)
    tex = (0x7F * xor) | ((0xFF * (1 - xor)) << 16)  # rgba(0x7F*xor, 0, 0xFF*(1-xor), 0)
    project = mat.perspective(1.0, 1.0, 0.1, 1000.0)
    mvp = mat.then(mat.translate3(0.0, 0.0, 1.0), project)
    vp = mat.viewport(0, 0, 256, 256)
    return verts, faces, tex.astype(np.uint32), mvp, vp


def test_textured_quad_bit_exact(golden_dir):
    """rendering.rs:18-60: Buf2<Color3> 256x256 equals textured_quad.ppm."""
    verts, faces, tex, mvp, vp = textured_quad_scene()
    d = O.make_draw(verts, faces, TEXTURED, mvp, tex=tex, sampler=CLAMP)
    color = np.zeros((256, 256), np.uint32)
    st = O.render([d], vp, color, None, {}, pixfmt=XRGB)
    rgb = xrgb_to_rgb(color)
    gold = np.load(os.path.join(golden_dir, "textured_quad.npz"))["rgb"]
    assert tuple(rgb[0, 0]) == (0, 0, 0xFF)
    assert tuple(rgb[255, 0]) == (0x7F, 0, 0)
    assert tuple(rgb[0, 255]) == (0x7F, 0, 0)
    assert np.array_equal(rgb, gold)
    assert st.prims_i == 2 and st.prims_o == 2 and st.frags_o == 256 * 256


def hello_tri_scene():
    """core/examples/hello_tri.rs:4-35 (fp feature: linear-space Gouraud)."""
    cols = np.array([[1.0, 0.0, 0.0], [0.0, 0.8, 0.0], [0.4, 0.4, 1.0]], np.float32)
    lin = np.power(cols, np.float32(2.2)).astype(np.float32)  # to_linear, per vertex
    pos = np.array([[-1, 1, 0], [1, 1, 0], [0, -1, 0]], np.float32)
    verts = np.concatenate([pos, lin], 1)
    w, h = 640, 480
    mvp = mat.then(mat.translate3(0.0, 0.0, 2.0),
                   mat.perspective(1.0, np.float32(w) / np.float32(h), 0.1, 1000.0))
    vp = mat.viewport(0, h, w, 0)
    return verts, np.array([[0, 1, 2]], np.uint32), mvp, vp


def test_hello_tri_coverage_exact_color_1lsb(golden_dir):
    """hello_tri.rs:47-57 + core/triangle.ppm: coverage exact, colour +-1 LSB
    (the per-fragment powf goes through the platform libm)."""
    verts, faces, mvp, vp = hello_tri_scene()
    d = O.make_draw(verts, faces, GOURAUD_SRGB, mvp)
    color = np.zeros((480, 640), np.uint32)
    O.render([d], vp, color, None, {}, pixfmt=RGBA)
    r, g, b, a = (color >> 24) & 0xFF, (color >> 16) & 0xFF, (color >> 8) & 0xFF, color & 0xFF
    assert (int(r[240, 320]), int(g[240, 320]), int(b[240, 320]), int(a[240, 320])) == (151, 128, 187, 255)
    gold = np.load(os.path.join(golden_dir, "triangle.npz"))["rgb"].astype(np.int32)
    ours = np.stack([r, g, b], -1).astype(np.int32)
    assert np.array_equal(a == 255, gold.any(-1)), "coverage differs"
    assert np.abs(ours - gold).max() <= 1


def test_shared_edge_no_gaps_or_overdraw(vectors):
    """raster.rs:325-368."""
    pts = np.array([[8, 0, 0], [0, 6, 0], [14, 10, 0], [20, 3, 0]], np.float32)
    buf = np.zeros((10, 20), np.int32)
    for tri in ([0, 1, 2], [0, 2, 3]):
        rows, _ = O.tri_fill(pts[tri], np.zeros((3, 1), np.float32))
        for y, x0, x1, _ in rows:
            buf[int(y), int(x0):int(x1)] += 1
    s = "".join("\n" + "".join(str(v) for v in r) for r in buf)
    assert s == vectors["shared_edge"]


def test_gradient_digits(vectors):
    """raster.rs:370-401: per-fragment varying digits, exact."""
    pts = np.array([[15, 2, 1.0], [2, 8, 1.0], [26, 14, 1.0]], np.float32)
    val = np.array([[0.0], [1.0], [0.5]], np.float32)
    rows, frags = O.tri_fill(pts, val, zdiv_mask=1)
    s, fi = "\n", 0
    for y, x0, x1, cnt in rows:
        s += " " * max(1, int(x0))  # format!("{:w$}", " ")
        for f in frags[fi:fi + int(cnt), 0]:
            s += str(int(np.clip(np.floor(np.float32(10.0) * f), 0, 255)))  # as u8
        fi += int(cnt)
        s += "\n"
    assert fi == len(frags)
    assert s == vectors["gradient"]


def test_clip_all_cases_histogram(vectors):
    """clip.rs:665-719: every in/out combination of 5^3 points per vertex."""
    xs = np.array([-2.0, -1.0, 0.0, 1.0, 2.0], np.float32)
    X, Y, Z = np.meshgrid(xs, xs, xs, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel(), np.ones(125, np.float32)], 1)
    hist = np.zeros(8, np.int64)
    allok = True
    bc = np.broadcast_to
    for a in range(125):
        tris = np.empty((125, 125, 3, 4), np.float32)
        tris[:, :, 0] = pts[a]
        tris[:, :, 1] = bc(pts[:, None, :], (125, 125, 4))
        tris[:, :, 2] = bc(pts[None, :, :], (125, 125, 4))
        counts, ok = O.clip_batch(tris.reshape(-1, 12))
        allok &= ok
        hist += np.bincount(counts, minlength=8)[:8]
    assert allok, "clip returned an out-of-bounds vertex"
    assert hist.sum() == 5 ** 9
    assert hist.tolist() == vectors["clip_histogram"]


def test_clip_unit_cases():
    """clip.rs:587-663: inside, outside, quad and heptagon results."""
    def tri(a, b, c):
        return np.array([a + [1.0], b + [1.0], c + [1.0]], np.float32)
    c, _ = O.clip_batch(tri([-1, -1, -1], [1, 1, 0], [0, 1, 1]))
    assert c.tolist() == [1]
    c, _ = O.clip_batch(tri([2, 2, 2], [2, -2, 0], [0, -1, 2]))
    assert c.tolist() == [0]
    c, _ = O.clip_batch(tri([0, 0, 0], [2, 0, 0], [0, 0, 2]))
    assert c.tolist() == [2]
    c, ok = O.clip_batch(tri([-1.5, 0, 0], [0, 0, -1.5], [2, 0, 2]))
    assert c.tolist() == [5] and ok


def test_samplers():
    """tex.rs:381-418."""
    tex = np.array([[rgba(0xFF, 0, 0, 0), rgba(0, 0xFF, 0, 0)],
                    [rgba(0, 0, 0xFF, 0), rgba(0xFF, 0xFF, 0, 0)]], np.uint32)
    R, G, B, Yl = rgba(0xFF, 0, 0, 0), rgba(0, 0xFF, 0, 0), rgba(0, 0, 0xFF, 0), rgba(0xFF, 0xFF, 0, 0)
    s = lambda k, u, v: O.sample(tex, k, u, v)
    assert [s(REPEAT_POT, -0.1, 0.0), s(REPEAT_POT, 0.0, -0.1)] == [G, B]
    assert [s(REPEAT_POT, 1.0, 0.0), s(REPEAT_POT, 0.0, 1.0)] == [R, R]
    assert [s(REPEAT_POT, 4.8, 0.2), s(REPEAT_POT, 0.2, 4.8)] == [G, B]
    assert [s(CLAMP, -1.0, 0.0), s(CLAMP, 0.0, -1.0)] == [R, R]
    assert [s(CLAMP, 1.5, 0.0), s(CLAMP, 0.0, 1.5), s(CLAMP, 1.5, 1.5)] == [G, B, Yl]
    assert [s(ONCE, 0, 0), s(ONCE, 0.5, 0), s(ONCE, 0, 0.5), s(ONCE, 0.5, 0.5)] == [R, G, B, Yl]


def test_pixfmt():
    """pixfmt.rs:152-205."""
    col = rgba(0x11, 0x22, 0x33, 0x44)
    assert O.pack(col, RGBA) == 0x11223344
    assert O.pack(col, ARGB) == 0x44112233
    assert O.pack(col, BGRA) == 0x33221144
    assert O.pack(col, XRGB) == 0x00112233


def test_matrices():
    """mat.rs:1843-1862."""
    m = mat.viewport(20, 10, 620, 470)
    assert mat.apply_point(m, [-1.0, -1.0, 0.2])[:3].tolist() == [20.0, 10.0, np.float32(0.2)]
    assert mat.apply_point(m, [1.0, 1.0, 0.6])[:3].tolist() == [620.0, 470.0, np.float32(0.6)]
    p = mat.perspective(0.8, 2.0, 0.1, 100.0)
    lbn = mat.apply_point(p, [-0.125, -0.0625, 0.1])
    rtf = mat.apply_point(p, [125.0, 62.5, 100.0])
    assert np.allclose(lbn / lbn[3], [-1, -1, -1, 1], atol=1e-5)
    assert np.allclose(rtf / rtf[3], [1, 1, 1, 1], atol=1e-5)


def test_rand_kats():
    """rand.rs:133-137 and rand.rs:314-318."""
    g = Xorshift64(11223344556677889900)
    assert [g.next_bits() for _ in range(3)] == [7782624861773764242, 6203733934162558527,
                                                 13009646309496342147]
    g = Xorshift64()
    assert [float(g.uniform(-1.0, 1.0)) for _ in range(3)] == [
        float(np.float32(0.19692874)), float(np.float32(-0.7686298)), float(np.float32(0.91969657))]


def test_oracle_depth_sort_orders_by_mean_clip_z():
    """render.rs:209-219 in the oracle: one render() call of three
    triangles covering the same pixels, at clip-space z 0.2, 0.5, 0.8 and
    w 1, 2, 3 (x, y scaled by w), submitted in that order, no depth test:
    the depth buffer keeps 1/w of the triangle drawn last.  Unsorted and
    front to back that is the far one (w 3); back to front the near one."""
    import numpy as np
    from oracle import oracle as O
    from retrofire_gb300 import mat
    verts = []
    for z, w in ((0.2, 1.0), (0.5, 2.0), (0.8, 3.0)):
        verts += [[-0.8 * w, -0.8 * w, z, w], [0.8 * w, -0.8 * w, z, w], [0.0, 0.8 * w, z, w]]
    verts = np.array(verts, np.float32)
    faces = np.arange(9, dtype=np.uint32).reshape(3, 3)
    vp = mat.viewport(0, 64, 64, 0)
    for sort, last_w in ((0, 3.0), (1, 3.0), (2, 1.0)):
        col = np.zeros((64, 64), np.uint32)
        dep = np.zeros((64, 64), np.float32)
        d = O.make_draw(verts, faces, 0, pos_dim=4, flat_rgba=0xFFFFFFFF)
        st = O.render([d], vp, col, dep, dict(depth_test=0, face_cull=0, depth_sort=sort))
        assert st.prims_o == 3
        assert dep[32, 32] == np.float32(1.0) / np.float32(last_w), (sort, dep[32, 32])
