"""Line primitives on the GPU (rf_render_lines) against the oracle's
render() of Edge<usize>: coverage, depth, colour and stats bit-exact."""
import numpy as np
import pytest

import retrofire_gb300 as rf
from oracle import oracle as O
from retrofire_gb300 import mat, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def both(verts, lines, shader, vp, w, h, mvp=None, pos_dim=3, ctx=None, tex=None, pixfmt=rf.ARGB8888,
         depth=True, pre_tris=None, device=None):
    """(gpu color, gpu depth, gpu stats), (oracle color, depth, stats)."""
    ctx = ctx or rf.Context()
    cd = dict(depth_test=ctx.depth_test, color_write=ctx.color_write, depth_write=ctx.depth_write,
              face_cull=ctx.face_cull)
    dev = device or rf.Device()
    oc = np.zeros((h, w), np.uint32)
    od = np.zeros((h, w), np.float32) if depth else None
    O.clear(oc, od, pixfmt)
    try:
        tg = rf.Framebuf(w, h, pixfmt, depth, device=dev)
        tg.clear()
        t = rf.Texture(tex, device=dev) if tex is not None else None
        if pre_tris is not None:  # a triangle draw first, into the same target
            pv, pf, pmvp = pre_tris
            pm = rf.Mesh(pv, pf, device=dev)
            rf.render(pm, None, rf.Shader.gouraud(), pmvp, vp, tg, rf.Context())
            O.render([O.make_draw(pv, pf, rf.GOURAUD, pmvp)], vp, oc, od, {}, pixfmt=pixfmt)
            pm.close()
        lm = rf.Lines(verts, lines, pos_dim=pos_dim, device=dev)
        sh = rf.Shader(shader, texture=t)
        st = rf.render_lines(lm, sh, mvp, vp, tg, ctx)
        c, d = tg.read()
        ost = O.render_lines(verts, lines, shader, vp, oc, od, cd, mvp=mvp, pos_dim=pos_dim,
                             tex=tex, pixfmt=pixfmt)
        lm.close()
        if t is not None:
            t.close()
        tg.close()
        return (c, d, st), (oc, od, ost)
    finally:
        if device is None:
            dev.close()


def check(g, o, what=""):
    gc, gd, gs = g
    oc, od, os_ = o
    assert np.array_equal(gc, oc), "%s colour: %d px differ" % (what, (gc != oc).sum())
    if gd is not None:
        assert np.array_equal(gd.view(np.uint32), od.view(np.uint32)), what + " depth"
    g_ = {k: v for k, v in gs.as_dict().items() if k in os_.as_dict()}
    assert g_ == os_.as_dict(), "%s stats %r %r" % (what, g_, os_.as_dict())


def wire(n, seed, attrs="col"):
    v, f = scenes.grid_mesh(n, seed, attrs)
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    return v, e


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_grid_wireframe(seed):
    v, e = wire(24, seed)
    mvp = scenes.orbit_camera(seed, 320, 240)
    g, o = both(v, e, rf.GOURAUD, mat.viewport(0, 240, 320, 0), 320, 240, mvp=mvp)
    assert o[2].frags_i > 1000
    check(g, o, "seed %d" % seed)


def random_lines(n, seed):
    """Clip-space lines: mostly inside, some crossing planes or behind the
    eye, some axis-aligned, some degenerate points."""
    rng = np.random.default_rng(seed)
    p = rng.uniform(-1.4, 1.4, size=(2 * n, 4)).astype(np.float32)
    p[:, 3] = rng.uniform(0.5, 2.0, size=2 * n)
    p[:, :3] *= p[:, 3:4]
    p[::7, 3] *= -1.0                      # behind the eye
    p[1::11, 1] = p[0::11, 1][: len(p[1::11])]  # horizontal in clip space
    p[3::13, 0] = p[2::13, 0][: len(p[3::13])]  # vertical
    p[5::17] = p[4::17][: len(p[5::17])]   # points
    col = rng.uniform(0, 1, size=(2 * n, 3)).astype(np.float32)
    return np.concatenate([p, col], 1), np.arange(2 * n, dtype=np.uint32).reshape(n, 2)


@pytest.mark.parametrize("depth_test", [rf.DEPTH_LESS, rf.DEPTH_NONE, rf.DEPTH_GREATER, rf.DEPTH_EQUAL])
@pytest.mark.parametrize("cull", [rf.CULL_BACK, rf.CULL_FRONT])
def test_random_clip_space_lines(depth_test, cull):
    v, li = random_lines(3000, 5 + depth_test + 7 * cull)
    ctx = rf.Context(depth_test=depth_test, face_cull=cull)
    g, o = both(v, li, rf.GOURAUD, mat.viewport(0, 0, 256, 200), 256, 200, pos_dim=4, ctx=ctx)
    check(g, o, "depth %d cull %d" % (depth_test, cull))


@pytest.mark.parametrize("pixfmt", [rf.ARGB8888, rf.RGBA8888])
def test_textured_and_colour_only(pixfmt):
    v, e = wire(16, 4, "col_uv")
    uv = np.ascontiguousarray(v[:, [0, 1, 2, 6, 7]])  # positions + texcoords
    mvp = scenes.orbit_camera(9, 200, 160)
    tex = scenes.checker_texture(64)
    g, o = both(uv, e, rf.TEXTURED, mat.viewport(0, 160, 200, 0), 200, 160, mvp=mvp, tex=tex,
                pixfmt=pixfmt)
    check(g, o, "textured")
    g, o = both(v[:, :6], e, rf.GOURAUD, mat.viewport(0, 160, 200, 0), 200, 160, mvp=mvp,
                depth=False, pixfmt=pixfmt)
    check(g, o, "colour-only")


def test_lines_over_a_surface():
    """Lines depth-tested against triangles rendered before them."""
    gv, gf = scenes.grid_mesh(20, 6)
    v, e = wire(10, 7)
    v = v.copy()
    v[:, 1] += 0.02  # just above the surface in places
    mvp = scenes.orbit_camera(11, 320, 240)
    g, o = both(v, e, rf.GOURAUD, mat.viewport(0, 240, 320, 0), 320, 240, mvp=mvp,
                pre_tris=(gv, gf, mvp))
    check(g, o, "over surface")


def test_viewport_larger_than_target():
    v, li = random_lines(500, 21)
    g, o = both(v, li, rf.GOURAUD, mat.viewport(0, 0, 400, 300), 300, 200, pos_dim=4)
    assert o[2].oob > 0
    check(g, o, "oversized viewport")


def test_pending_clear_and_counts():
    v, e = wire(8, 2)
    dev = rf.Device()
    try:
        lm = rf.Lines(v, e, device=dev)
        tg = rf.Framebuf(120, 90, device=dev)
        tg.clear(0xFF102030)
        st = rf.render_lines(lm, rf.Shader.gouraud(), scenes.orbit_camera(3, 120, 90),
                             mat.viewport(0, 90, 120, 0), tg)
        c, _ = tg.read()
        assert st.calls == 1 and st.prims_i == len(e) and st.verts_o == 3 * st.prims_o
        assert (c == O.pack(0xFF102030, 0)).sum() > 0  # the clear landed under the lines
        with pytest.raises(rf.RfError):  # line meshes are not triangle meshes
            rf.render_draws([(lm, rf.Shader.gouraud(), None)], mat.viewport(0, 90, 120, 0), tg)
        lm.close()
        tg.close()
    finally:
        dev.close()
