"""rf_render_noalloc: rendering without any device allocation.

Some callers of this library may not allocate device memory while they
render: a frame loop held to a fixed, pre-reserved memory budget, or a
plugin inside a host application that owns every allocation and only lends
the plugin the buffers it reads and fills.  rf_render_noalloc serves them:
the caller passes its own device buffers for the mesh, texture and target,
and the library's temporaries live in a fixed scratch area compiled into it.

This test calls it through the C ABI twice in a row (plus a third call that
repeats the first, so nothing left in the shared scratch area by the second
call can leak), each time on caller-owned device buffers, and checks every
result against the allocating entry point rf_render and against the oracle
(the reference's CPU path restated): colour, depth and stats must match bit
for bit, the tolerance all parity tests here use for these shaders.  It also
checks that inputs beyond the stated limits are refused.  The file is named
so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import scenes

from rfhelp import DrawSpec, oracle_render

pytestmark = pytest.mark.gpu

BAD_ARG = 2
OVER_BUDGET = 5


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def cube_case():
    s = scenes.textured_cube(seed=3)
    return dict(verts=s["verts"], faces=s["faces"], shader=rf.TEXTURED, mvp=s["mvp"],
                tex=s["tex"], vp=s["vp"], w=s["w"], h=s["h"], pos_dim=3)


def fill_case():
    s = scenes.fill_stress(ntri=1000, w=300, h=200, seed=31)
    return dict(verts=s["verts"], faces=s["faces"], shader=rf.GOURAUD,
                mvp=np.eye(4, dtype=np.float32), tex=None, vp=s["vp"], w=300, h=200, pos_dim=4)


def with_allocating_entry_point(c):
    """The same frame through rf_render (device handles, library-owned scratch)."""
    dev = rf.Device()
    tg = rf.Framebuf(c["w"], c["h"], rf.ARGB8888, True, device=dev)
    tex = rf.Texture(c["tex"], device=dev) if c["tex"] is not None else None
    tg.clear()
    mesh = rf.Mesh(c["verts"], c["faces"], pos_dim=c["pos_dim"], device=dev)
    st = rf.render(mesh, None, rf.Shader(c["shader"], texture=tex), c["mvp"], c["vp"], tg)
    col, dep = tg.read()
    for o in (mesh, tex, tg):
        if o is not None:
            o.close()
    dev.close()
    return col, dep, st.as_dict()


def with_noalloc_entry_point(c):
    """The frame through rf_render_noalloc on caller-owned device buffers."""
    import torch
    dv = torch.from_numpy(np.ascontiguousarray(c["verts"], np.float32)).cuda()
    di = torch.from_numpy(np.ascontiguousarray(c["faces"], np.uint32).view(np.int32)).cuda()
    dt = None
    if c["tex"] is not None:
        dt = torch.from_numpy(np.ascontiguousarray(c["tex"], np.uint32).view(np.int32)).cuda()
    col = torch.zeros((c["h"], c["w"]), dtype=torch.int32, device="cuda")
    dep = torch.zeros((c["h"], c["w"]), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    mvp = (C.c_float * 16)(*[float(x) for x in np.asarray(c["mvp"], np.float32).reshape(-1)])
    vp = (C.c_float * 16)(*[float(x) for x in np.asarray(c["vp"], np.float32).reshape(-1)])
    fl = rf.Context().flags()
    clear_rgba = C.c_uint32(0xFF000000)
    depth_clear = C.c_float(float("inf"))
    st = rf.CStats()
    nattr = c["verts"].shape[1] - c["pos_dim"]
    th, tw = (c["tex"].shape if c["tex"] is not None else (0, 0))
    code = rf.lib().rf_render_noalloc(
        dv.data_ptr(), c["verts"].shape[0], c["pos_dim"], nattr, di.data_ptr(),
        c["faces"].shape[0], c["shader"], mvp, 0, dt.data_ptr() if dt is not None else None,
        tw, th, rf.REPEAT_POT, vp, col.data_ptr(), dep.data_ptr(), c["w"], c["h"], rf.ARGB8888,
        C.byref(fl), C.byref(clear_rgba), C.byref(depth_clear), None, C.byref(st))
    assert code == 0, "rf_render_noalloc returned %d" % code
    torch.cuda.synchronize()
    return (col.cpu().numpy().view(np.uint32), dep.cpu().numpy(),
            rf.Stats.from_c(st).as_dict())


def with_oracle(c):
    """The same frame through the oracle (render.rs:134-207 restated)."""
    d = DrawSpec(c["verts"], c["faces"], c["shader"], c["mvp"], pos_dim=c["pos_dim"],
                 tex=c["tex"])
    return oracle_render([d], c["vp"], c["w"], c["h"])


def assert_same(a, b, what):
    assert np.array_equal(a[0], b[0]), what + ": colour differs"
    assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32)), what + ": depth differs"
    sa = {k: a[2][k] for k in b[2]}
    assert sa == b[2], what + ": stats differ %r vs %r" % (sa, b[2])


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls():
    cases = [("textured cube", cube_case()), ("gouraud fill", fill_case()),
             ("textured cube again", cube_case())]
    expected = {name: with_allocating_entry_point(c) for name, c in cases}
    oracle = {name: with_oracle(c) for name, c in cases}
    for name, c in cases:
        got = with_noalloc_entry_point(c)
        assert got[2]["frags_i"] > 0
        assert_same(got, expected[name], name + " vs rf_render")
        assert_same(got, oracle[name], name + " vs the oracle")


def test_noalloc_refuses_inputs_beyond_its_limits():
    fl = rf.Context().flags()
    m = (C.c_float * 16)()
    L = rf.lib()
    args = dict(nverts=3, ntri=1, w=64, h=64)

    def call(nverts, ntri, w, h):
        return L.rf_render_noalloc(C.c_void_p(16), nverts, 3, 3, C.c_void_p(16), ntri,
                                   rf.GOURAUD, m, 0, None, 0, 0, 0, m, C.c_void_p(16),
                                   C.c_void_p(16), w, h, rf.ARGB8888, C.byref(fl), None, None,
                                   None, None)
    assert call(**dict(args, ntri=1025)) == OVER_BUDGET
    assert call(**dict(args, nverts=4097)) == OVER_BUDGET
    assert call(**dict(args, w=1025)) == OVER_BUDGET
    assert call(**dict(args, h=1025)) == OVER_BUDGET
    assert call(**dict(args, nverts=0)) == BAD_ARG  # triangles with no vertices
