"""Shared helpers for the parity tests: render one scene through the CUDA
library (through its C ABI) and through the oracle, and compare."""
import numpy as np

import retrofire_gb300 as rf
from oracle import oracle as O

NAN_SAFE = np.uint32


class DrawSpec:
    def __init__(self, verts, faces, shader, mvp=None, pos_dim=3, flat_rgba=0, tex=None,
                 sampler=rf.REPEAT_POT):
        self.verts = np.ascontiguousarray(verts, np.float32)
        self.faces = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
        self.shader, self.mvp, self.pos_dim = shader, mvp, pos_dim
        self.flat_rgba, self.tex, self.sampler = flat_rgba, tex, sampler


def ctx_dict(ctx):
    return dict(depth_test=ctx.depth_test, color_write=ctx.color_write,
                depth_write=ctx.depth_write, face_cull=ctx.face_cull, depth_sort=ctx.depth_sort)


def gpu_render(draws, vp, w, h, ctx=None, pixfmt=rf.ARGB8888, depth=True, clear=True,
               prefill=None, tile=None, per_call=False, device=None):
    """Returns (color, depth, Stats).  clear: Frame::clear with the context's
    clear values first; prefill: (color, depth) written into the target."""
    ctx = ctx or rf.Context()
    dev = device or rf.Device()
    if tile:
        dev.set_tiling(*tile)
    tg = rf.Framebuf(w, h, pixfmt, depth, device=dev)
    texes = {}
    meshes = []
    try:
        if prefill is not None:
            tg.write(*prefill)
        if clear:
            tg.clear(ctx.color_clear, ctx.depth_clear)
        items = []
        for d in draws:
            m = rf.Mesh(d.verts, d.faces, pos_dim=d.pos_dim, device=dev)
            meshes.append(m)
            tex = None
            if d.tex is not None:
                key = id(d.tex)
                if key not in texes:
                    texes[key] = rf.Texture(d.tex, device=dev)
                tex = texes[key]
            items.append((m, rf.Shader(d.shader, d.flat_rgba, tex, d.sampler), d.mvp))
        st = rf.Stats()
        if per_call:
            for m, sh, mvp in items:
                st += rf.render(m, None, sh, mvp, vp, tg, ctx)
        else:
            st += rf.render_draws(items, vp, tg, ctx)
        col, dep = tg.read()
        return col, dep, st
    finally:
        for m in meshes:
            m.close()
        for t in texes.values():
            t.close()
        tg.close()
        if device is None:
            dev.close()


def oracle_render(draws, vp, w, h, ctx=None, pixfmt=rf.ARGB8888, depth=True, clear=True,
                  prefill=None):
    ctx = ctx or rf.Context()
    col = np.zeros((h, w), np.uint32)
    dep = np.zeros((h, w), np.float32) if depth else None
    if prefill is not None:
        if prefill[0] is not None:
            col[...] = prefill[0]
        if depth and prefill[1] is not None:
            dep[...] = prefill[1]
    if clear:
        O.clear(col, dep, pixfmt, ctx.color_clear, ctx.depth_clear)
    ods = [O.make_draw(d.verts, d.faces, d.shader, d.mvp, pos_dim=d.pos_dim,
                       flat_rgba=d.flat_rgba, tex=d.tex, sampler=d.sampler) for d in draws]
    st = O.render(ods, vp, col, dep, ctx_dict(ctx), pixfmt=pixfmt)
    return col, dep, st.as_dict()


def channels(img):
    return np.stack([(img >> s) & 0xFF for s in (24, 16, 8, 0)], -1).astype(np.int32)


def assert_parity(gpu, ref, color_tol=0, what=""):
    """Depth and stats bit-exact; colour exact (or within color_tol LSB per
    channel, with identical coverage judged by the depth/colour writes)."""
    gc, gd, gs = gpu
    oc, od, os_ = ref
    report = []
    if gd is not None or od is not None:
        db = np.ascontiguousarray(gd).view(np.uint32) != np.ascontiguousarray(od).view(np.uint32)
        if db.any():
            y, x = np.argwhere(db)[0]
            report.append("depth: %d px differ, first (%d,%d) gpu=%r ref=%r"
                          % (db.sum(), x, y, gd[y, x], od[y, x]))
    if color_tol == 0:
        cb = gc != oc
        if cb.any():
            y, x = np.argwhere(cb)[0]
            report.append("color: %d px differ, first (%d,%d) gpu=%08x ref=%08x"
                          % (cb.sum(), x, y, gc[y, x], oc[y, x]))
    else:
        diff = np.abs(channels(gc) - channels(oc)).max(-1)
        bad = diff > color_tol
        if bad.any():
            y, x = np.argwhere(bad)[0]
            report.append("color: %d px beyond %d LSB, first (%d,%d)" % (bad.sum(), color_tol, x, y))
    gsd = gs.as_dict() if hasattr(gs, "as_dict") else gs
    gsd = {k: gsd[k] for k in os_}  # the counters the oracle's render() keeps
    if gsd != os_:
        report.append("stats: gpu=%r ref=%r" % (gsd, os_))
    assert not report, (what + ": " if what else "") + "; ".join(report)
