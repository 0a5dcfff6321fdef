"""ctypes front for the C++ oracle (test infrastructure only).

Mirrors the call shape of the product's `render()` so the parity tests can
run the same scene through both: `render(draws, viewport, target, ctx)`
renders a list of draws in order into numpy colour/depth buffers, exactly as
that many consecutive retrofire `render()` calls would (render.rs:134-207).
"""
import ctypes as C

import numpy as np

from . import build as _build

_lib = None


class Draw(C.Structure):
    _fields_ = [("verts", C.POINTER(C.c_float)), ("nverts", C.c_uint32),
                ("pos_dim", C.c_uint32), ("nattr", C.c_uint32),
                ("idx", C.POINTER(C.c_uint32)), ("ntri", C.c_uint32),
                ("shader", C.c_int32), ("mvp", C.c_float * 16),
                ("flat_rgba", C.c_uint32), ("tex", C.POINTER(C.c_uint32)),
                ("tw", C.c_uint32), ("th", C.c_uint32), ("sampler", C.c_int32)]


class Ctx(C.Structure):
    _fields_ = [("depth_test", C.c_int32), ("color_write", C.c_int32),
                ("depth_write", C.c_int32), ("face_cull", C.c_int32), ("depth_sort", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in
                ("calls", "prims_i", "prims_o", "verts_i", "verts_o",
                 "frags_i", "frags_o", "oob")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        fp = C.POINTER(C.c_float)
        u32p = C.POINTER(C.c_uint32)
        L.rfo_render.argtypes = [C.POINTER(Draw), fp, u32p, fp, C.c_uint32,
                                 C.c_uint32, C.c_int32, C.POINTER(Ctx), C.POINTER(Stats)]
        L.rfo_render.restype = None
        L.rfo_clear.argtypes = [u32p, fp, C.c_uint32, C.c_uint32, C.c_int32, u32p, fp]
        L.rfo_clear.restype = None
        L.rfo_pack.argtypes = [C.c_uint32, C.c_int32]
        L.rfo_pack.restype = C.c_uint32
        L.rfo_clip_batch.argtypes = [C.c_uint32, fp, fp, u32p, fp, fp]
        L.rfo_clip_batch.restype = C.c_int32
        L.rfo_tri_fill.argtypes = [fp, fp, C.c_uint32, C.c_uint32,
                                   C.POINTER(C.c_uint64), C.c_uint32, fp,
                                   C.c_uint64, C.POINTER(C.c_uint64)]
        L.rfo_tri_fill.restype = C.c_uint32
        L.rfo_sample.argtypes = [u32p, C.c_uint32, C.c_uint32, C.c_int32, C.c_float, C.c_float]
        L.rfo_sample.restype = C.c_uint32
        L.rfo_render_lines.argtypes = [C.POINTER(Draw), u32p, C.c_uint32, fp, u32p, fp,
                                       C.c_uint32, C.c_uint32, C.c_int32, C.POINTER(Ctx),
                                       C.POINTER(Stats)]
        L.rfo_render_lines.restype = None
        L.rfo_bbox_status.argtypes = [fp, C.c_uint32, C.c_uint32, fp]
        L.rfo_bbox_status.restype = C.c_int32
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _u32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def make_draw(verts, idx, shader, mvp=None, pos_dim=3, flat_rgba=0, tex=None,
              sampler=0):
    """Build an oracle Draw; keeps references to the arrays it points at."""
    verts = np.ascontiguousarray(verts, np.float32)
    idx = np.ascontiguousarray(idx, np.uint32).reshape(-1)
    d = Draw()
    d.verts = _fp(verts)
    d.nverts = verts.shape[0]
    d.pos_dim = pos_dim
    d.nattr = verts.shape[1] - pos_dim
    d.idx = _u32p(idx)
    d.ntri = idx.size // 3
    d.shader = shader
    m = np.eye(4, dtype=np.float32) if mvp is None else np.asarray(mvp, np.float32)
    d.mvp[:] = [float(x) for x in m.reshape(-1)]
    d.flat_rgba = flat_rgba
    if tex is not None:
        tex = np.ascontiguousarray(tex, np.uint32)
        d.tex = _u32p(tex)
        d.th, d.tw = tex.shape
    d.sampler = sampler
    d._keep = (verts, idx, tex)
    return d


def render(draws, viewport, color, depth, ctx, pixfmt=0, stats=None):
    """Render the draws in order into color (u32 HxW) and depth (f32 HxW or None)."""
    L = lib()
    h, w = color.shape
    vp = np.ascontiguousarray(viewport, np.float32).reshape(-1)
    st = stats if stats is not None else Stats()
    c = Ctx(ctx.get("depth_test", 1), int(ctx.get("color_write", True)),
            int(ctx.get("depth_write", True)), ctx.get("face_cull", 1), ctx.get("depth_sort", 0))
    dp = _fp(depth) if depth is not None else C.POINTER(C.c_float)()
    for d in draws:
        L.rfo_render(C.byref(d), _fp(vp), _u32p(color), dp, w, h, pixfmt,
                     C.byref(c), C.byref(st))
    return st


def clear(color, depth, pixfmt=0, clear_rgba=0xFF000000, depth_clear=float("inf")):
    L = lib()
    h, w = color.shape
    cr = (C.c_uint32 * 1)(clear_rgba) if clear_rgba is not None else None
    dc = (C.c_float * 1)(depth_clear) if depth_clear is not None else None
    L.rfo_clear(_u32p(color), _fp(depth) if depth is not None else C.POINTER(C.c_float)(),
                w, h, pixfmt, C.cast(cr, C.POINTER(C.c_uint32)) if cr else None,
                C.cast(dc, C.POINTER(C.c_float)) if dc else None)


def pack(rgba, pixfmt):
    return lib().rfo_pack(rgba, pixfmt)


def clip_batch(pos, attr=None):
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 12)
    n = pos.shape[0]
    counts = np.zeros(n, np.uint32)
    at = None if attr is None else np.ascontiguousarray(attr, np.float32)
    ok = lib().rfo_clip_batch(n, _fp(pos), _fp(at) if at is not None else None,
                              _u32p(counts), None, None)
    return counts, bool(ok)


def tri_fill(screen, attr, zdiv_mask=0, max_rows=4096, max_frags=1 << 20):
    screen = np.ascontiguousarray(screen, np.float32).reshape(3, 3)
    attr = np.ascontiguousarray(attr, np.float32).reshape(3, -1)
    na = attr.shape[1]
    rows = np.zeros((max_rows, 4), np.uint64)
    frags = np.zeros((max_frags, max(na, 1)), np.float32)
    nf = C.c_uint64(0)
    nr = lib().rfo_tri_fill(_fp(screen), _fp(attr), na, zdiv_mask,
                            rows.ctypes.data_as(C.POINTER(C.c_uint64)), max_rows,
                            _fp(frags), max_frags, C.byref(nf))
    return rows[:nr], frags[:nf.value, :na]


def sample(tex, sampler, u, v):
    tex = np.ascontiguousarray(tex, np.uint32)
    th, tw = tex.shape
    return lib().rfo_sample(_u32p(tex), tw, th, sampler, u, v)


__all__ = ["Draw", "Ctx", "Stats", "make_draw", "render", "clear", "pack",
           "clip_batch", "tri_fill", "sample", "lib"]


VISIBLE, CLIPPED, HIDDEN = 0, 1, 2


def bbox_status(verts, mvp, pos_dim=3):
    """BBox::of the positions, then BBox::visibility under mvp (scene.rs):
    VISIBLE, CLIPPED or HIDDEN."""
    v = np.ascontiguousarray(verts, np.float32)
    m = np.ascontiguousarray(mvp, np.float32).reshape(-1)
    return int(lib().rfo_bbox_status(_fp(v), v.shape[0], v.shape[1], _fp(m)))


def render_lines(verts, lines, shader, viewport, color, depth, ctx, mvp=None, pos_dim=3,
                 flat_rgba=0, tex=None, sampler=0, pixfmt=0, stats=None):
    """One render() call of Edge<usize> primitives: `lines` (n, 2) vertex
    index pairs (raster.rs line(), clip.rs line clipping)."""
    L = lib()
    h, w = color.shape
    d = make_draw(verts, np.zeros((0, 3), np.uint32), shader, mvp, pos_dim, flat_rgba, tex, sampler)
    li = np.ascontiguousarray(lines, np.uint32).reshape(-1)
    vp = np.ascontiguousarray(viewport, np.float32).reshape(-1)
    st = stats if stats is not None else Stats()
    c = Ctx(ctx.get("depth_test", 1), int(ctx.get("color_write", True)),
            int(ctx.get("depth_write", True)), ctx.get("face_cull", 1), 0)
    dp = _fp(depth) if depth is not None else C.POINTER(C.c_float)()
    L.rfo_render_lines(C.byref(d), _u32p(li), li.size // 2, _fp(vp), _u32p(color), dp, w, h,
                       pixfmt, C.byref(c), C.byref(st))
    return st
