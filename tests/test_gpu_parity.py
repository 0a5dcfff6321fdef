"""GPU parity: the CUDA path (through the C ABI) against the oracle.

Coverage, depth and stats must be bit-exact; colour bit-exact for every
shader but GOURAUD_SRGB (powf, +-1 LSB per 8-bit channel).
"""
import os

import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import mat, scenes
from rfhelp import DrawSpec, assert_parity, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def both(draws, vp, w, h, **kw):
    gkw = {k: v for k, v in kw.items() if k in ("ctx", "pixfmt", "depth", "clear", "prefill",
                                                "tile", "per_call")}
    okw = {k: v for k, v in kw.items() if k in ("ctx", "pixfmt", "depth", "clear", "prefill")}
    return gpu_render(draws, vp, w, h, **gkw), oracle_render(draws, vp, w, h, **okw)


# ------------------------------------------------------------ goldens ---

def test_textured_quad_golden(golden_dir):
    """core/tests/rendering.rs:18-60 on the GPU: bit-exact to the PPM."""
    from test_oracle_pins import textured_quad_scene, xrgb_to_rgb
    verts, faces, tex, mvp, vp = textured_quad_scene()
    d = DrawSpec(verts, faces, rf.TEXTURED, mvp, tex=tex, sampler=rf.CLAMP)
    g, o = both([d], vp, 256, 256, pixfmt=rf.XRGB8888, depth=False, clear=False)
    gold = np.load(os.path.join(golden_dir, "textured_quad.npz"))["rgb"]
    assert np.array_equal(xrgb_to_rgb(g[0]), gold)
    assert_parity(g, o)


def test_hello_tri_golden(golden_dir):
    """core/examples/hello_tri.rs: centre pixel, coverage exact, +-1 LSB."""
    from test_oracle_pins import hello_tri_scene
    verts, faces, mvp, vp = hello_tri_scene()
    d = DrawSpec(verts, faces, rf.GOURAUD_SRGB, mvp)
    g, o = both([d], vp, 640, 480, pixfmt=rf.RGBA8888, depth=False, clear=False)
    col = g[0]
    r, gg, b, a = (col >> 24) & 255, (col >> 16) & 255, (col >> 8) & 255, col & 255
    assert abs(int(r[240, 320]) - 151) <= 1 and abs(int(gg[240, 320]) - 128) <= 1
    assert abs(int(b[240, 320]) - 187) <= 1 and int(a[240, 320]) == 255
    gold = np.load(os.path.join(golden_dir, "triangle.npz"))["rgb"].astype(np.int32)
    assert np.array_equal(a == 255, gold.any(-1))
    assert np.abs(np.stack([r, gg, b], -1).astype(np.int32) - gold).max() <= 1
    assert_parity(g, o, color_tol=1)


# ------------------------------------------------------- benchmark scenes ---

@pytest.mark.parametrize("seed", list(range(1, 13)))
def test_textured_cube(seed):
    s = scenes.textured_cube(seed=seed)
    d = DrawSpec(s["verts"], s["faces"], rf.TEXTURED, s["mvp"], tex=s["tex"])
    g, o = both([d], s["vp"], s["w"], s["h"])
    assert_parity(g, o, what="cube seed %d" % seed)


@pytest.mark.parametrize("seed,ntri,w,h", [(2, 3000, 640, 360), (5, 2000, 333, 77),
                                           (6, 20000, 1920, 1080)])
def test_fill_stress(seed, ntri, w, h):
    s = scenes.fill_stress(ntri=ntri, w=w, h=h, seed=seed)
    d = DrawSpec(s["verts"], s["faces"], rf.GOURAUD, pos_dim=4)
    g, o = both([d], s["vp"], w, h)
    assert g[2].frags_i > 0
    assert_parity(g, o, what="fill seed %d" % seed)


def test_instanced_cubes_multi_draw():
    s = scenes.instanced_cubes(ninst=300, w=480, h=270, tex_size=256)
    draws = [DrawSpec(s["verts"], s["faces"], rf.TEX_GOURAUD, s["mvps"][i], tex=s["tex"])
             for i in range(len(s["mvps"]))]
    g, o = both(draws, s["vp"], s["w"], s["h"])
    assert g[2].prims_o > 0
    assert_parity(g, o, what="instanced multi-draw")
    g2 = gpu_render(draws[:60], s["vp"], s["w"], s["h"], per_call=True)
    o2 = oracle_render(draws[:60], s["vp"], s["w"], s["h"])
    assert_parity(g2, o2, what="instanced per-call")


# ------------------------------------------------------------ context ---

def small_fill(seed=11, ntri=1500, w=300, h=200):
    s = scenes.fill_stress(ntri=ntri, w=w, h=h, seed=seed)
    return [DrawSpec(s["verts"], s["faces"], rf.GOURAUD, pos_dim=4)], s["vp"], w, h


@pytest.mark.parametrize("depth_test", [rf.DEPTH_NONE, rf.DEPTH_LESS, rf.DEPTH_EQUAL,
                                        rf.DEPTH_GREATER])
@pytest.mark.parametrize("color_write,depth_write", [(True, True), (True, False), (False, True)])
def test_context_depth_modes(depth_test, color_write, depth_write):
    draws, vp, w, h = small_fill()
    ctx = rf.Context(depth_test=depth_test, color_write=color_write, depth_write=depth_write,
                     face_cull=rf.CULL_NONE)
    rng = np.random.default_rng(depth_test)
    pre = (rng.integers(0, 1 << 32, (h, w), dtype=np.uint64).astype(np.uint32),
           np.where(rng.random((h, w)) < 0.3, np.float32(0.5), np.float32(0.3)).astype(np.float32))
    g, o = both(draws, vp, w, h, ctx=ctx, prefill=pre, clear=False)
    assert_parity(g, o, what="depth_test=%d cw=%d dw=%d" % (depth_test, color_write, depth_write))


@pytest.mark.parametrize("cull", [rf.CULL_NONE, rf.CULL_BACK, rf.CULL_FRONT])
def test_face_cull(cull):
    s = scenes.textured_cube(seed=4)
    d = DrawSpec(s["verts"], s["faces"], rf.TEXTURED, s["mvp"], tex=s["tex"])
    g, o = both([d], s["vp"], s["w"], s["h"], ctx=rf.Context(face_cull=cull))
    assert_parity(g, o)


@pytest.mark.parametrize("fmt", [rf.ARGB8888, rf.XRGB8888, rf.RGBA8888, rf.BGRA8888])
def test_pixel_formats(fmt):
    draws, vp, w, h = small_fill(seed=3)
    g, o = both(draws, vp, w, h, pixfmt=fmt, ctx=rf.Context(color_clear=0x80402010))
    assert_parity(g, o)


def test_colour_only_target():
    draws, vp, w, h = small_fill(seed=4)
    g, o = both(draws, vp, w, h, depth=False)
    assert g[1] is None
    assert_parity(g, o)


# ------------------------------------------------------ shaders/samplers ---

def uv_plane(umax=3.0, n=6, shift=-1.3):
    """A grid of textured quads with uv outside [0,1] (negative too)."""
    xs = np.linspace(-1.5, 1.5, n + 1, dtype=np.float32)
    verts, faces = [], []
    for j in range(n + 1):
        for i in range(n + 1):
            verts.append([xs[i], xs[j], 0.3 * xs[i], shift + umax * i / n, shift + umax * j / n])
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            faces += [[a, a + 1, a + n + 1], [a + 1, a + n + 2, a + n + 1]]
    return np.array(verts, np.float32), np.array(faces, np.uint32)


@pytest.mark.parametrize("sampler", [rf.REPEAT_POT, rf.CLAMP, rf.ONCE])
@pytest.mark.parametrize("shader", [rf.TEXTURED, rf.TEX_GOURAUD])
def test_samplers(sampler, shader):
    verts, faces = uv_plane(shift=0.0 if sampler == rf.ONCE else -1.3,
                            umax=1.0 if sampler == rf.ONCE else 3.0)
    if shader == rf.TEX_GOURAUD:
        rng = np.random.default_rng(5)
        col = rng.uniform(0, 1, (len(verts), 3)).astype(np.float32)
        verts = np.concatenate([verts[:, :3], col, verts[:, 3:]], 1)
    tex = scenes.noise_texture(32, seed=9)
    mvp = mat.then(mat.translate3(0.0, 0.0, 3.0), mat.perspective(1.2, 4.0 / 3.0, 0.1, 50.0))
    d = DrawSpec(verts, faces, shader, mvp, tex=tex, sampler=sampler)
    g, o = both([d], mat.viewport(0, 0, 400, 300), 400, 300, ctx=rf.Context(face_cull=rf.CULL_NONE))
    assert_parity(g, o)


def test_flat_and_mixed_shaders():
    s = scenes.textured_cube(seed=8)
    verts3 = s["verts"][:, :3]
    d0 = DrawSpec(verts3, s["faces"], rf.FLAT, s["mvp"], flat_rgba=0xFF3366CC)
    m2 = mat.then(mat.translate3(0.4, 0.2, 0.5), s["mvp"])
    d1 = DrawSpec(s["verts"], s["faces"], rf.TEXTURED, m2, tex=s["tex"])
    g, o = both([d0, d1, d0], s["vp"], s["w"], s["h"], ctx=rf.Context(face_cull=rf.CULL_NONE))
    assert_parity(g, o)


# ---------------------------------------------------------- tiling ---

@pytest.mark.parametrize("tile", [(8, 1), (16, 2), (32, 4), (64, 8), (32, 1)])
def test_tilings_agree(tile):
    draws, vp, w, h = small_fill(seed=12, ntri=4000, w=517, h=301)
    g, o = both(draws, vp, w, h, tile=tile)
    assert_parity(g, o, what="tile %r" % (tile,))


@pytest.mark.parametrize("tile,depth", [((32, 4), True), ((64, 8), True), ((32, 4), False),
                                        ((64, 2), False)])
def test_bulk_write_back(tile, depth):
    """A target whose rows start 16-byte aligned (width a multiple of 4):
    its tiles of whole 32-column blocks go back to memory as bulk copies,
    one 128-byte row per lane, with and without a depth buffer; the edge
    tiles (520 = 16 x 32 + 8) take the per-pixel path beside them."""
    draws, vp, w, h = small_fill(seed=13, ntri=3000, w=520, h=300)
    g, o = both(draws, vp, w, h, tile=tile, depth=depth)
    assert_parity(g, o, what="tile %r depth %r" % (tile, depth))


# ------------------------------------------------------------ edge cases ---

def test_empty_and_degenerate():
    w, h = 160, 120
    vp = mat.viewport(0, 0, w, h)
    rng = np.random.default_rng(1)
    P = rng.uniform(-1, 1, (12, 3)).astype(np.float32)
    col = rng.uniform(0, 1, (12, 3)).astype(np.float32)
    verts = np.concatenate([np.concatenate([P, np.ones((12, 1), np.float32)], 1), col], 1)
    faces = np.array([[0, 0, 0], [0, 1, 1], [2, 3, 2], [4, 5, 6], [7, 8, 9]], np.uint32)
    verts[7, :3] = verts[8, :3] = verts[9, :3] * np.float32(0.5)  # collinear-ish
    draws = [DrawSpec(verts, faces, rf.GOURAUD, pos_dim=4),
             DrawSpec(verts, np.zeros((0, 3), np.uint32), rf.GOURAUD, pos_dim=4)]
    g, o = both(draws, vp, w, h, ctx=rf.Context(face_cull=rf.CULL_NONE))
    assert_parity(g, o)


def test_nonfinite_and_w_zero():
    w, h = 128, 96
    vp = mat.viewport(0, 0, w, h)
    v = np.array([[0, 0, 0, 0, 1, 0, 0], [0.5, 0.5, 0, 1, 0, 1, 0], [-0.5, 0.5, 0, 1, 0, 0, 1],
                  [np.nan, 0, 0, 1, 1, 1, 1], [0.2, -0.3, 0.1, 1, 1, 0, 1], [0.3, 0.3, 0, 1, 0, 1, 1],
                  [np.inf, 0, 0, 1, 0, 0, 0], [0.1, 0.9, 0, 1, 1, 1, 0], [0.9, 0.1, 0, 1, 1, 0, 0]],
                 np.float32)
    faces = np.array([[0, 1, 2], [3, 4, 5], [6, 7, 8], [4, 5, 7]], np.uint32)
    d = DrawSpec(v, faces, rf.GOURAUD, pos_dim=4)
    g, o = both([d], vp, w, h, ctx=rf.Context(face_cull=rf.CULL_NONE))
    assert_parity(g, o)


def test_nonfinite_and_out_of_range_colours():
    """Colour varyings that are NaN, infinite, negative or above 1: the
    `(256 * c) as u8` of each channel saturates and takes NaN to 0."""
    w, h = 96, 64
    vp = mat.viewport(0, 0, w, h)
    v = np.array([[-0.9, -0.9, 0.1, 1, np.nan, -1.0, 2.0], [0.9, -0.8, 0.2, 1, 0.5, 3.0, np.inf],
                  [0.0, 0.9, 0.3, 1, 0.2, -np.inf, 0.5],
                  [-0.5, 0.5, 0.5, 1, 1e30, -1e30, 0.99], [0.8, 0.8, 0.5, 1, -0.001, 1.01, 0.0],
                  [0.7, -0.7, 0.5, 1, 0.996, 0.004, -0.0]], np.float32)
    faces = np.array([[0, 1, 2], [3, 4, 5]], np.uint32)
    d = DrawSpec(v, faces, rf.GOURAUD, pos_dim=4)
    for ctx in (rf.Context(face_cull=rf.CULL_NONE), rf.Context(face_cull=rf.CULL_NONE, depth_test=rf.DEPTH_NONE)):
        g, o = both([d], vp, w, h, ctx=ctx)
        assert o[2]["frags_o"] > 0
        assert_parity(g, o)


def test_near_plane_and_fullscreen():
    w, h = 400, 300
    vp = mat.viewport(0, 0, w, h)
    v = np.array([[-3, -3, -2, 1, 1, 0, 0], [3, -3, 0.5, 1, 0, 1, 0], [0, 5, 2.5, 1, 0, 0, 1],
                  [-1, -1, 0.2, 1, 1, 1, 0], [1, -1, 0.2, 1, 0, 1, 1], [-1, 1, 0.2, 1, 1, 0, 1],
                  [1, 1, 0.2, 1, 0.5, 0.5, 0.5]], np.float32)
    faces = np.array([[0, 1, 2], [3, 4, 5], [4, 6, 5]], np.uint32)
    d = DrawSpec(v, faces, rf.GOURAUD, pos_dim=4)
    g, o = both([d], vp, w, h, ctx=rf.Context(face_cull=rf.CULL_NONE))
    assert_parity(g, o)


def test_viewport_out_of_target_counts_oob():
    """A viewport larger than the target: the reference panics on those
    scanlines; here they are dropped and counted identically."""
    draws, _, w, h = small_fill(seed=7, ntri=800, w=200, h=150)
    vp = mat.viewport(-40, -30, 260, 190)
    g, o = both(draws, vp, w, h)
    assert o[2]["oob"] > 0
    assert_parity(g, o)


def test_flipped_viewport_and_tiny_targets():
    draws, _, _, _ = small_fill(seed=9, ntri=300, w=64, h=64)
    for (w, h) in [(1, 1), (3, 70), (70, 3), (33, 31)]:
        g, o = both(draws, mat.viewport(0, h, w, 0), w, h, ctx=rf.Context(face_cull=rf.CULL_FRONT))
        assert_parity(g, o, what="%dx%d" % (w, h))


# -------------------------------------------------------- clear / state ---

def test_clear_then_read_without_render():
    dev = rf.Device()
    tg = rf.Framebuf(50, 40, rf.ARGB8888, True, device=dev)
    tg.clear(0x11223344, 2.0)  # Color4 bytes r=0x44 g=0x33 b=0x22 a=0x11
    c, d = tg.read()
    assert (c == 0x11443322).all() and (d == np.float32(0.5)).all()
    tg.close()
    dev.close()


def test_renders_accumulate_like_sequential_calls():
    draws, vp, w, h = small_fill(seed=21, ntri=1000, w=240, h=160)
    more, _, _, _ = small_fill(seed=22, ntri=1000, w=240, h=160)
    dev = rf.Device()
    tg = rf.Framebuf(w, h, device=dev)
    tg.clear()
    meshes = [rf.Mesh(d.verts, d.faces, pos_dim=4, device=dev) for d in draws + more]
    ctx = rf.Context()
    for m in meshes:
        rf.render(m, None, rf.Shader.gouraud(), None, vp, tg, ctx)
    c, d = tg.read()
    oc, od, ost = oracle_render(draws + more, vp, w, h)
    assert np.array_equal(c, oc) and np.array_equal(d.view(np.uint32), od.view(np.uint32))
    assert ctx.stats.as_dict() == dict(ost, objs_i=0, objs_o=0)
    for m in meshes:
        m.close()
    tg.close()
    dev.close()


def test_async_stats_accumulate():
    draws, vp, w, h = small_fill(seed=23, ntri=500, w=128, h=128)
    dev = rf.Device()
    tg = rf.Framebuf(w, h, device=dev)
    m = rf.Mesh(draws[0].verts, draws[0].faces, pos_dim=4, device=dev)
    for _ in range(3):
        tg.clear()
        rf.render_draws([(m, rf.Shader.gouraud(), None)], vp, tg, sync_stats=False)
    st = dev.take_stats()
    _, _, ost = oracle_render(draws, vp, w, h)
    assert st.frags_i == 3 * ost["frags_i"] and st.prims_o == 3 * ost["prims_o"]
    assert st.calls == 3
    m.close()
    tg.close()
    dev.close()


def test_call_stats_exclude_queued_work():
    """A call made with a stats pointer reports its own render() stats only
    (render.rs:206), even after frames queued without stats; those stay for
    rf_ctx_take_stats, which does not report the synchronous call again."""
    draws, vp, w, h = small_fill(seed=24, ntri=400, w=128, h=96)
    dev = rf.Device()
    tg = rf.Framebuf(w, h, device=dev)
    m = rf.Mesh(draws[0].verts, draws[0].faces, pos_dim=4, device=dev)
    _, _, ost = oracle_render(draws, vp, w, h)
    for _ in range(2):
        tg.clear()
        rf.render_draws([(m, rf.Shader.gouraud(), None)], vp, tg, sync_stats=False)
    tg.clear()
    st = rf.render_draws([(m, rf.Shader.gouraud(), None)], vp, tg, sync_stats=True)
    assert {k: st.as_dict()[k] for k in ost} == ost
    rest = dev.take_stats()
    assert rest.calls == 2 and rest.frags_i == 2 * ost["frags_i"]
    m.close()
    tg.close()
    dev.close()


def test_bad_arguments():
    dev = rf.Device()
    with pytest.raises(rf.RfError) as e:
        rf.Mesh(np.zeros((3, 5), np.float32), np.array([[0, 1, 3]]), device=dev)
    assert e.value.code == 2
    tex = rf.Texture(np.zeros((3, 5), np.uint32), device=dev)
    tg = rf.Framebuf(8, 8, device=dev)
    m = rf.Mesh(np.zeros((3, 5), np.float32), np.array([[0, 1, 2]]), device=dev)
    with pytest.raises(rf.RfError) as e:
        rf.render(m, None, rf.Shader.textured(tex, rf.REPEAT_POT), None, mat.viewport(0, 0, 8, 8), tg)
    assert e.value.code == 3  # SamplerRepeatPot::new panics on non-pot sizes
    with pytest.raises(rf.RfError) as e:
        rf.render(m, None, rf.Shader.gouraud(), None, mat.viewport(0, 0, 8, 8), tg)
    assert e.value.code == 2  # attribute count does not match the shader
    for o in (m, tex, tg):
        o.close()
    dev.close()


def test_text_mesh_renders_like_the_oracle():
    """A text mesh (text.rs: quads from an atlas) through the textured path
    with the clamp sampler."""
    from retrofire_gb300 import text
    atl = text.Atlas(scenes.noise_texture(128, 5)[:64], 8, 8)
    t = text.Text(atl)
    t.write("retrofire on\na GB300 !")
    v, f = t.mesh()
    mvp = np.array([[1 / 64, 0, 0, -1], [0, -1 / 32, 0, 1], [0, 0, 0, 0.5], [0, 0, 0, 1]], np.float32)
    d = DrawSpec(v, f, rf.TEXTURED, mvp, tex=atl.texels, sampler=rf.CLAMP)
    g, o = both([d], mat.viewport(0, 0, 256, 128), 256, 128, ctx=rf.Context(face_cull=rf.CULL_NONE))
    assert o[2]["frags_o"] > 1000
    assert_parity(g, o)
