"""The Python mirror of the reference API without a GPU: Context defaults
and flags (ctx.rs:11-126), Stats accumulation (stats.rs:16-40) and the
uniforms a Shader passes through the C ABI."""
import numpy as np
import pytest

import retrofire_gb300 as rf


def test_context_defaults_are_context_default():
    c = rf.Context()
    assert c.color_clear == 0xFF000000          # rgba(0, 0, 0, 255), ctx.rs:117
    assert c.depth_clear == float("inf")        # the depth buffer gets 1/inf = 0
    assert (c.face_cull, c.depth_test) == (rf.CULL_BACK, rf.DEPTH_LESS)
    f = c.flags()
    assert (f.depth_test, f.color_write, f.depth_write, f.face_cull) == (rf.DEPTH_LESS, 1, 1, rf.CULL_BACK)
    g = rf.Context(depth_test=rf.DEPTH_GREATER, color_write=False, depth_write=0,
                   face_cull=rf.CULL_NONE).flags()
    assert (g.depth_test, g.color_write, g.depth_write, g.face_cull) == (rf.DEPTH_GREATER, 0, 0, rf.CULL_NONE)


def test_depth_sort_flag():
    """Context::depth_sort defaults to None (ctx.rs:117-126) and travels in
    rf_context_flags."""
    assert rf.Context().flags().depth_sort == rf.SORT_NONE
    assert rf.Context(depth_sort=None).flags().depth_sort == rf.SORT_NONE
    assert rf.Context(depth_sort=rf.SORT_BACK_TO_FRONT).flags().depth_sort == 2
    assert rf.Context(depth_sort=rf.SORT_FRONT_TO_BACK).flags().depth_sort == 1


def test_stats_accumulate():
    a = rf.Stats(calls=1, prims_i=12, frags_i=100, frags_o=40)
    a += rf.Stats(calls=2, prims_i=3, frags_i=5, objs_i=4, objs_o=3)
    assert a.as_dict() == {"calls": 3, "prims_i": 15, "prims_o": 0, "verts_i": 0, "verts_o": 0,
                           "frags_i": 105, "frags_o": 40, "oob": 0, "objs_i": 4, "objs_o": 3}
    cs = rf.CStats()
    cs.frags_i, cs.oob = 7, 2
    s = rf.Stats.from_c(cs)
    assert (s.frags_i, s.oob, s.calls) == (7, 2, 0)


class _Tex:
    handle = 42


def test_shader_uniforms():
    m = np.arange(16, dtype=np.float32).reshape(4, 4)
    u = rf.Shader.tex_gouraud(_Tex(), sampler=rf.CLAMP).uniforms(m)
    assert list(u.mvp) == list(range(16))       # row-major, as Matrix.0
    assert (u.texture, u.sampler, u.flat_rgba) == (42, rf.CLAMP, 0)
    u = rf.Shader.flat(0x80FF0001).uniforms(None)
    assert list(u.mvp) == list(np.eye(4, dtype=np.float32).reshape(-1))
    assert (u.flat_rgba, u.texture) == (0x80FF0001, 0)
    assert rf.Shader.gouraud().kind == rf.GOURAUD and rf.Shader.gouraud_srgb().kind == rf.GOURAUD_SRGB
    assert rf.NATTR == {rf.FLAT: 0, rf.GOURAUD: 3, rf.TEXTURED: 2, rf.TEX_GOURAUD: 5,
                        rf.GOURAUD_SRGB: 3}
