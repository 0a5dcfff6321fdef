"""retrofire_gb300 — retrofire's triangle render path on a GB300 (sm_103a).

Python host mirror of the reference's rendering surface over the C ABI of
librfgpu (include/rfgpu.h):

    render(prims, verts, shader, uniform, to_screen, target, ctx)
        core/src/render.rs:134-207
    Context                      core/src/render/ctx.rs:11-126
    Framebuf / Colorbuf          core/src/render/target.rs:35-44
    shader kinds                 core/src/render/shader.rs (fixed family)
    Texture + samplers           core/src/render/tex.rs
    Stats                        core/src/render/stats.rs:16-40

Meshes, textures and targets live on the device; ``render`` uploads the
given vertex/index arrays (a fresh mesh per call, like the reference's
borrowed slices) unless a ``Mesh`` handle is passed.  There is no CPU
fallback: without the CUDA library every entry point raises.
"""
import ctypes as C
import os

import numpy as np

from . import mat  # noqa: F401  (host-side matrix helpers)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "librfgpu.so")

# Shader kinds, samplers, pixel formats, depth tests, face culling
# (mirrors of include/rfgpu.h).
FLAT, GOURAUD, TEXTURED, TEX_GOURAUD, GOURAUD_SRGB = range(5)
REPEAT_POT, CLAMP, ONCE = range(3)
ARGB8888, XRGB8888, RGBA8888, BGRA8888 = range(4)
DEPTH_NONE, DEPTH_LESS, DEPTH_EQUAL, DEPTH_GREATER = range(4)
CULL_NONE, CULL_BACK, CULL_FRONT = range(3)
# Context::depth_sort (ctx.rs:39): None, Some(FrontToBack), Some(BackToFront)
SORT_NONE, SORT_FRONT_TO_BACK, SORT_BACK_TO_FRONT = range(3)
NATTR = {FLAT: 0, GOURAUD: 3, TEXTURED: 2, TEX_GOURAUD: 5, GOURAUD_SRGB: 3}

STAGES = ("vertex", "clip", "scan", "setup", "raster")
OBJ_POSITION, OBJ_NORMAL, OBJ_TEXCOORD, OBJ_NORMAL_TEXCOORD = range(4)

STATUS = {0: "ok", 1: "bad handle", 2: "bad argument", 3: "non power-of-two texture",
          4: "out of device memory", 5: "over budget", 6: "overflow", 7: "timeout",
          8: "cuda error", 9: "no cuda device"}


class RfError(RuntimeError):
    def __init__(self, code, what=""):
        super().__init__("%s: %s (%d)" % (what, STATUS.get(code, "?"), code))
        self.code = code


class Uniforms(C.Structure):
    _fields_ = [("mvp", C.c_float * 16), ("flat_rgba", C.c_uint32), ("sampler", C.c_uint32),
                ("texture", C.c_uint64)]


class Flags(C.Structure):
    _fields_ = [("depth_test", C.c_int32), ("color_write", C.c_int32),
                ("depth_write", C.c_int32), ("face_cull", C.c_int32), ("depth_sort", C.c_int32)]


class CStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("calls", "prims_i", "prims_o", "verts_i", "verts_o",
                                          "frags_i", "frags_o", "oob", "objs_i", "objs_o")]


# rf_draw flags
DRAW_CULL_BBOX = 1


class Draw(C.Structure):
    _fields_ = [("mesh", C.c_uint64), ("shader", C.c_int32), ("flags", C.c_uint32),
                ("uniforms", Uniforms)]


class Job(C.Structure):
    _fields_ = [("target", C.c_uint64), ("ndraws", C.c_uint32), ("draws", C.POINTER(Draw)),
                ("viewport", C.c_float * 16), ("flags", Flags)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_batch", C.c_uint32),
                ("inflight", C.c_uint32), ("staging_bytes", C.c_uint64),
                ("max_batch_tris", C.c_uint64)]


class Request(C.Structure):
    _fields_ = [("ndraws", C.c_uint32), ("draws", C.POINTER(Draw)), ("viewport", C.c_float * 16),
                ("flags", Flags), ("w", C.c_uint32), ("h", C.c_uint32), ("pixfmt", C.c_int32),
                ("has_depth", C.c_int32), ("clear_rgba", C.c_uint32), ("depth_clear", C.c_float),
                ("color_out", C.POINTER(C.c_uint32)), ("depth_out", C.POINTER(C.c_float))]


class Result(C.Structure):
    _fields_ = [("status", C.c_int32), ("batch_size", C.c_uint32), ("batch_id", C.c_uint64),
                ("queue_ms", C.c_double), ("render_ms", C.c_double), ("total_ms", C.c_double),
                ("stats", CStats), ("gpu_start_ns", C.c_uint64), ("gpu_end_ns", C.c_uint64),
                ("pipeline", C.c_uint32), ("reserved_", C.c_uint32)]


# Exported symbols of include/rfgpu.h with their ctypes signatures.
_P = C.c_void_p
_SIGS = {
    "rf_ctx_create": [_P, C.POINTER(_P)],
    "rf_ctx_destroy": [_P],
    "rf_ctx_sync": [_P],
    "rf_ctx_take_stats": [_P, C.POINTER(CStats)],
    "rf_ctx_set_tiling": [_P, C.c_uint32, C.c_uint32],
    "rf_ctx_set_online_tuning": [_P, C.c_int32],
    "rf_ctx_last_tiling": [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)],
    "rf_mesh_upload": [_P, C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.c_uint32,
                       C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint64)],
    "rf_mesh_update": [_P, C.c_uint64, C.POINTER(C.c_float), C.POINTER(C.c_uint32)],
    "rf_mesh_update_async": [_P, C.c_uint64, C.POINTER(C.c_float), C.POINTER(C.c_uint32)],
    "rf_target_read_async": [_P, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_float)],
    "rf_mesh_destroy": [_P, C.c_uint64],
    "rf_ctx_set_timing": [_P, C.c_int32],
    "rf_ctx_stage_ms": [_P, C.POINTER(C.c_double), C.POINTER(C.c_uint32)],
    "rf_texture_upload": [_P, C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32,
                          C.POINTER(C.c_uint64)],
    "rf_texture_destroy": [_P, C.c_uint64],
    "rf_target_create": [_P, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32,
                         C.POINTER(C.c_uint64)],
    "rf_target_destroy": [_P, C.c_uint64],
    "rf_target_clear": [_P, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_float)],
    "rf_target_write": [_P, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_float)],
    "rf_target_read": [_P, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_float)],
    "rf_render": [_P, C.c_uint64, C.c_int32, C.POINTER(Uniforms), C.POINTER(C.c_float),
                  C.c_uint64, C.POINTER(Flags), C.POINTER(CStats)],
    "rf_render_draws": [_P, C.POINTER(Draw), C.c_uint32, C.POINTER(C.c_float), C.c_uint64,
                        C.POINTER(Flags), C.POINTER(CStats)],
    "rf_render_batch": [_P, C.POINTER(Job), C.c_uint32, C.POINTER(CStats)],
    "rf_lines_upload": [_P, C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.c_uint32,
                        C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint64)],
    "rf_render_lines": [_P, C.c_uint64, C.c_int32, C.POINTER(Uniforms), C.POINTER(C.c_float),
                        C.c_uint64, C.POINTER(Flags), C.POINTER(CStats)],
    "rf_ctx_device": [_P, C.POINTER(C.c_int32)],
    "rf_mesh_info": [_P, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                     C.POINTER(C.c_uint32)],
    "rf_server_create": [_P, C.POINTER(ServerConfig), C.POINTER(_P)],
    "rf_server_submit": [_P, C.POINTER(Request), C.POINTER(C.c_uint64)],
    "rf_server_wait": [_P, C.c_uint64, C.c_uint32, C.POINTER(Result)],
    "rf_server_counts": [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)],
    "rf_server_destroy": [_P],
    "rf_server_memory": [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)],
    "rf_obj_parse": [C.c_char_p, C.c_size_t, C.c_int32, C.POINTER(C.POINTER(C.c_float)),
                     C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.POINTER(C.c_uint32)),
                     C.POINTER(C.c_uint32), C.c_char_p, C.c_size_t],
    "rf_mesh_load_obj": [_P, C.c_char_p, C.c_size_t, C.c_int32, C.POINTER(C.c_uint64)],
    "rf_ctx_set_graphs": [_P, C.c_int32],
    "rf_ctx_counts": [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)],
    "rf_ctx_autotune": [_P, C.POINTER(Job), C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32),
                        C.POINTER(C.c_uint32), C.POINTER(C.c_float)],
    # device pointers throughout; see include/rfgpu.h
    "rf_render_noalloc": [_P, C.c_uint32, C.c_uint32, C.c_uint32, _P, C.c_uint32, C.c_int32,
                          C.POINTER(C.c_float), C.c_uint32, _P, C.c_uint32, C.c_uint32,
                          C.c_uint32, C.POINTER(C.c_float), _P, _P, C.c_uint32, C.c_uint32,
                          C.c_int32, C.POINTER(Flags), C.POINTER(C.c_uint32),
                          C.POINTER(C.c_float), _P, C.POINTER(CStats)],
}

_lib = None


def lib():
    """Load librfgpu.so (built by retrofire_gb300.build); raise if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("librfgpu.so is not built (%s); run "
                               "`python -m retrofire_gb300.build`" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, argt in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = argt
            fn.restype = C.c_int32
        L.rf_status_str.argtypes = [C.c_int32]
        L.rf_status_str.restype = C.c_char_p
        L.rf_ctx_last_error.argtypes = [_P]
        L.rf_ctx_last_error.restype = C.c_char_p
        L.rf_obj_free.argtypes = [_P]
        L.rf_obj_free.restype = None
        _lib = L
    return _lib


def _check(code, what):
    if code != 0:
        raise RfError(code, what)


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _u32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


class Stats:
    """Stats (stats.rs:16-40): calls and per-stage Throughput in/out."""
    FIELDS = ("calls", "prims_i", "prims_o", "verts_i", "verts_o", "frags_i", "frags_o", "oob",
              "objs_i", "objs_o")

    def __init__(self, **kw):
        for f in self.FIELDS:
            setattr(self, f, int(kw.get(f, 0)))

    @classmethod
    def from_c(cls, cs):
        return cls(**{f: getattr(cs, f) for f in cls.FIELDS})

    def __iadd__(self, o):
        for f in self.FIELDS:
            setattr(self, f, getattr(self, f) + getattr(o, f))
        return self

    def as_dict(self):
        return {f: getattr(self, f) for f in self.FIELDS}

    def __repr__(self):
        return "Stats(%s)" % ", ".join("%s=%d" % kv for kv in self.as_dict().items())


class Context:
    """Context (ctx.rs:11-126); defaults equal Context::default()."""

    def __init__(self, color_clear=0xFF000000, depth_clear=float("inf"), face_cull=CULL_BACK,
                 depth_test=DEPTH_LESS, color_write=True, depth_write=True, depth_sort=SORT_NONE):
        self.depth_sort = SORT_NONE if depth_sort is None else depth_sort  # SORT_*
        self.color_clear = color_clear    # Color4 as r|g<<8|b<<16|a<<24, or None
        self.depth_clear = depth_clear    # f32 or None
        self.face_cull = face_cull
        self.depth_test = depth_test
        self.color_write = color_write
        self.depth_write = depth_write
        self.stats = Stats()

    def flags(self):
        return Flags(self.depth_test, int(bool(self.color_write)), int(bool(self.depth_write)),
                     self.face_cull, self.depth_sort)


class Device:
    """One rf_ctx: a CUDA stream plus the handles created on it."""

    def __init__(self, stream=None):
        p = _P()
        _check(lib().rf_ctx_create(stream, C.byref(p)), "rf_ctx_create")
        self.ptr = p

    def close(self):
        if self.ptr:
            lib().rf_ctx_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        _check(lib().rf_ctx_sync(self.ptr), "rf_ctx_sync")

    def last_error(self):
        """The CUDA call and message behind the last "cuda error" or "out of
        device memory" status of this device ("" if none)."""
        return lib().rf_ctx_last_error(self.ptr).decode()

    def set_tiling(self, tile_w=0, warps=0):
        _check(lib().rf_ctx_set_tiling(self.ptr, tile_w, warps), "rf_ctx_set_tiling")

    def set_online_tuning(self, enable=True):
        _check(lib().rf_ctx_set_online_tuning(self.ptr, int(bool(enable))),
               "rf_ctx_set_online_tuning")

    def last_tiling(self):
        """(tile width, warps per block) of the last frame."""
        tw, wp = C.c_uint32(), C.c_uint32()
        _check(lib().rf_ctx_last_tiling(self.ptr, C.byref(tw), C.byref(wp)), "rf_ctx_last_tiling")
        return tw.value, wp.value

    def set_timing(self, enable=True):
        _check(lib().rf_ctx_set_timing(self.ptr, int(bool(enable))), "rf_ctx_set_timing")

    def stage_ms(self):
        """Per-stage GPU milliseconds summed over the timed renders since the
        last call, and the number of renders: ({stage: ms}, frames)."""
        out = (C.c_double * 5)()
        fr = C.c_uint32()
        _check(lib().rf_ctx_stage_ms(self.ptr, out, C.byref(fr)), "rf_ctx_stage_ms")
        return dict(zip(STAGES, list(out))), fr.value

    def set_graphs(self, enable=True):
        _check(lib().rf_ctx_set_graphs(self.ptr, int(bool(enable))), "rf_ctx_set_graphs")

    def counts(self):
        """{kernels, graph_launches, graphs_cached} of this context so far."""
        k, n, c = C.c_uint64(), C.c_uint64(), C.c_uint32()
        _check(lib().rf_ctx_counts(self.ptr, C.byref(k), C.byref(n), C.byref(c)), "rf_ctx_counts")
        return {"kernels": k.value, "graph_launches": n.value, "graphs_cached": c.value}

    def take_stats(self):
        cs = CStats()
        _check(lib().rf_ctx_take_stats(self.ptr, C.byref(cs)), "rf_ctx_take_stats")
        return Stats.from_c(cs)


_default_device = None


def default_device():
    global _default_device
    if _default_device is None:
        _default_device = Device()
    return _default_device


class Mesh:
    """Device-resident Mesh (geom/mesh.rs:24-30): vertex array + Tri<usize> faces.

    verts: (n, pos_dim + nattr) float32, pos_dim 3 (model space) or 4 (clip
    space, passed through the vertex shader unchanged)."""

    def __init__(self, verts, faces, pos_dim=3, device=None):
        self.dev = device or default_device()
        v = np.ascontiguousarray(verts, np.float32)
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1)
        if v.ndim != 2 or v.shape[1] < pos_dim:
            raise ValueError("verts must be (n, pos_dim + nattr)")
        self.nverts, self.ntri = v.shape[0], f.size // 3
        self.pos_dim, self.nattr = pos_dim, v.shape[1] - pos_dim
        h = C.c_uint64()
        _check(lib().rf_mesh_upload(self.dev.ptr, _fp(v), v.shape[0], pos_dim, self.nattr,
                                    _u32p(f), self.ntri, C.byref(h)), "rf_mesh_upload")
        self.handle = h.value

    def update(self, verts=None, faces=None):
        """rf_mesh_update: same-sized arrays, uploaded in place."""
        v = None if verts is None else np.ascontiguousarray(verts, np.float32)
        f = None if faces is None else np.ascontiguousarray(faces, np.uint32)
        _check(lib().rf_mesh_update(self.dev.ptr, self.handle, _fp(v) if v is not None else None,
                                    _u32p(f) if f is not None else None), "rf_mesh_update")

    def update_async(self, verts=None, faces=None):
        """rf_mesh_update_async: the arrays must stay alive and unchanged
        until Device.sync (page-locked memory for overlap)."""
        _check(lib().rf_mesh_update_async(self.dev.ptr, self.handle,
                                          _fp(verts) if verts is not None else None,
                                          _u32p(faces) if faces is not None else None),
               "rf_mesh_update_async")

    def close(self):
        if self.handle and self.dev.ptr:
            lib().rf_mesh_destroy(self.dev.ptr, self.handle)
        self.handle = 0


class Lines(Mesh):
    """A device line mesh: verts as for Mesh, lines (n, 2) vertex index
    pairs (Edge<usize>, geom/prim.rs)."""

    def __init__(self, verts, lines, pos_dim=3, device=None):
        self.dev = device or default_device()
        v = np.ascontiguousarray(verts, np.float32)
        li = np.ascontiguousarray(lines, np.uint32).reshape(-1)
        self.nverts, self.ntri = v.shape[0], li.size // 2
        self.pos_dim, self.nattr = pos_dim, v.shape[1] - pos_dim
        h = C.c_uint64()
        _check(lib().rf_lines_upload(self.dev.ptr, _fp(v), v.shape[0], pos_dim, self.nattr,
                                     _u32p(li), self.ntri, C.byref(h)), "rf_lines_upload")
        self.handle = h.value


def render_lines(lines, shader, uniform, to_screen, target, ctx=None):
    """render() of line primitives (Edge<usize>): lines is a Lines mesh."""
    ctx = ctx or Context()
    vp = np.ascontiguousarray(to_screen, np.float32).reshape(-1)
    u = shader.uniforms(uniform)
    fl = ctx.flags()
    cs = CStats()
    _check(lib().rf_render_lines(target.dev.ptr, lines.handle, shader.kind, C.byref(u), _fp(vp),
                                 target.handle, C.byref(fl), C.byref(cs)), "rf_render_lines")
    st = Stats.from_c(cs)
    ctx.stats += st
    return st


class Texture:
    """Texture<Buf2<Color4>> (tex.rs:33-37); texels (h, w) u32 = bytes r,g,b,a."""

    def __init__(self, texels, device=None):
        self.dev = device or default_device()
        t = np.ascontiguousarray(texels, np.uint32)
        self.h, self.w = t.shape
        h = C.c_uint64()
        _check(lib().rf_texture_upload(self.dev.ptr, _u32p(t), self.w, self.h, C.byref(h)),
               "rf_texture_upload")
        self.handle = h.value

    def close(self):
        if self.handle and self.dev.ptr:
            lib().rf_texture_destroy(self.dev.ptr, self.handle)
        self.handle = 0


class Framebuf:
    """Framebuf<Colorbuf<Buf2<u32>, fmt>, Buf2<f32>> (target.rs:35-44) on the
    device; with depth=False a colour-only Colorbuf (target.rs:187-202)."""

    def __init__(self, w, h, pixfmt=ARGB8888, depth=True, device=None):
        self.dev = device or default_device()
        self.w, self.h, self.pixfmt, self.has_depth = w, h, pixfmt, depth
        hd = C.c_uint64()
        _check(lib().rf_target_create(self.dev.ptr, w, h, pixfmt, int(depth), C.byref(hd)),
               "rf_target_create")
        self.handle = hd.value

    def clear(self, color_clear=0xFF000000, depth_clear=float("inf")):
        """Frame::clear (front/src/lib.rs:103-120); None skips a buffer."""
        cc = (C.c_uint32 * 1)(color_clear) if color_clear is not None else None
        dc = (C.c_float * 1)(depth_clear) if depth_clear is not None else None
        _check(lib().rf_target_clear(self.dev.ptr, self.handle,
                                     C.cast(cc, C.POINTER(C.c_uint32)) if cc else None,
                                     C.cast(dc, C.POINTER(C.c_float)) if dc else None),
               "rf_target_clear")

    def write(self, color=None, depth=None):
        c = None if color is None else np.ascontiguousarray(color, np.uint32)
        d = None if depth is None else np.ascontiguousarray(depth, np.float32)
        _check(lib().rf_target_write(self.dev.ptr, self.handle, _u32p(c) if c is not None else None,
                                     _fp(d) if d is not None else None), "rf_target_write")

    def read(self):
        color = np.empty((self.h, self.w), np.uint32)
        depth = np.empty((self.h, self.w), np.float32) if self.has_depth else None
        _check(lib().rf_target_read(self.dev.ptr, self.handle, _u32p(color),
                                    _fp(depth) if depth is not None else None), "rf_target_read")
        return color, depth

    def read_async(self, color, depth=None):
        """rf_target_read_async into caller arrays (h, w) uint32 / float32;
        valid after Device.sync."""
        _check(lib().rf_target_read_async(self.dev.ptr, self.handle, _u32p(color),
                                          _fp(depth) if depth is not None else None),
               "rf_target_read_async")

    def close(self):
        if self.handle and self.dev.ptr:
            lib().rf_target_destroy(self.dev.ptr, self.handle)
        self.handle = 0


class Shader:
    """A member of the fixed shader family with its non-matrix uniforms."""

    def __init__(self, kind, flat_rgba=0, texture=None, sampler=REPEAT_POT):
        self.kind, self.flat_rgba, self.texture, self.sampler = kind, flat_rgba, texture, sampler

    @classmethod
    def flat(cls, rgba):
        return cls(FLAT, flat_rgba=rgba)

    @classmethod
    def gouraud(cls):
        return cls(GOURAUD)

    @classmethod
    def gouraud_srgb(cls):
        return cls(GOURAUD_SRGB)

    @classmethod
    def textured(cls, texture, sampler=REPEAT_POT):
        return cls(TEXTURED, texture=texture, sampler=sampler)

    @classmethod
    def tex_gouraud(cls, texture, sampler=REPEAT_POT):
        return cls(TEX_GOURAUD, texture=texture, sampler=sampler)

    def uniforms(self, mvp):
        u = Uniforms()
        m = np.eye(4, dtype=np.float32) if mvp is None else np.asarray(mvp, np.float32)
        u.mvp[:] = [float(x) for x in m.reshape(-1)]
        u.flat_rgba = self.flat_rgba
        u.sampler = self.sampler
        u.texture = self.texture.handle if self.texture is not None else 0
        return u


def render(prims, verts, shader, uniform, to_screen, target, ctx=None, pos_dim=3):
    """render() (render.rs:134-207).

    prims: Mesh, or (n, 3) vertex indices with verts (n, pos_dim + nattr);
    uniform: the 4x4 mvp (ProjMat3); to_screen: the 4x4 viewport matrix;
    target: Framebuf; ctx: Context (stats are added into ctx.stats)."""
    ctx = ctx or Context()
    dev = target.dev
    own = not isinstance(prims, Mesh)
    mesh = Mesh(verts, prims, pos_dim=pos_dim, device=dev) if own else prims
    try:
        vp = np.ascontiguousarray(to_screen, np.float32).reshape(-1)
        u = shader.uniforms(uniform)
        fl = ctx.flags()
        cs = CStats()
        _check(lib().rf_render(dev.ptr, mesh.handle, shader.kind, C.byref(u), _fp(vp),
                               target.handle, C.byref(fl), C.byref(cs)), "rf_render")
        st = Stats.from_c(cs)
        ctx.stats += st
        return st
    finally:
        if own:
            mesh.close()


def render_draws(draws, to_screen, target, ctx=None, sync_stats=True):
    """Several render() calls into one target, in order, as one GPU pass.

    draws: list of (Mesh, Shader, mvp) or (Mesh, Shader, mvp, flags), flags
    DRAW_CULL_BBOX for object-level frustum culling."""
    ctx = ctx or Context()
    arr = (Draw * len(draws))()
    for i, dr in enumerate(draws):
        mesh, shader, mvp = dr[:3]
        arr[i].mesh = mesh.handle
        arr[i].shader = shader.kind
        arr[i].flags = dr[3] if len(dr) > 3 else 0
        arr[i].uniforms = shader.uniforms(mvp)
    vp = np.ascontiguousarray(to_screen, np.float32).reshape(-1)
    fl = ctx.flags()
    cs = CStats()
    _check(lib().rf_render_draws(target.dev.ptr, arr, len(draws), _fp(vp), target.handle,
                                 C.byref(fl), C.byref(cs) if sync_stats else None),
           "rf_render_draws")
    st = Stats.from_c(cs)
    ctx.stats += st
    return st


class Scene:
    """One job of a batch: a target, its Context flags and viewport, and the
    render() calls into it, in order.  draws: list of (Mesh, Shader, mvp).
    The C draw records are built once, at first use; set_draws replaces
    them (for a scene whose matrices change between frames)."""

    def __init__(self, target, draws, to_screen, ctx=None):
        self.target, self.ctx = target, ctx or Context()
        self.to_screen = np.ascontiguousarray(to_screen, np.float32).reshape(-1)
        self.set_draws(draws)

    def set_draws(self, draws):
        self.draws = list(draws)
        self._arr = None

    def _draw_array(self):
        if self._arr is None:
            arr = (Draw * max(1, len(self.draws)))()
            if self.draws:
                mvps = np.zeros((len(self.draws), 16), np.float32)
                for i, dr in enumerate(self.draws):
                    mesh, shader, mvp = dr[:3]
                    arr[i].mesh = mesh.handle
                    arr[i].shader = shader.kind
                    arr[i].flags = dr[3] if len(dr) > 3 else 0
                    arr[i].uniforms = shader.uniforms(None)
                    if mvp is not None:
                        mvps[i] = np.asarray(mvp, np.float32).reshape(-1)
                    else:
                        mvps[i] = np.eye(4, dtype=np.float32).reshape(-1)
                # the 16 mvp floats of every record in one strided copy
                raw = np.ctypeslib.as_array(C.cast(arr, C.POINTER(C.c_uint8)),
                                            (len(self.draws) * C.sizeof(Draw),))
                rec = raw.reshape(len(self.draws), C.sizeof(Draw))
                off = Draw.uniforms.offset + Uniforms.mvp.offset
                rec[:, off:off + 64] = mvps.view(np.uint8).reshape(-1, 64)
            self._arr = arr
        return self._arr


def _jobs(scenes):
    jobs = (Job * len(scenes))()
    keep = []
    for j, sc in zip(jobs, scenes):
        arr = sc._draw_array()
        keep.append(arr)
        j.target = sc.target.handle
        j.ndraws = len(sc.draws)
        j.draws = C.cast(arr, C.POINTER(Draw))
        j.viewport[:] = [float(x) for x in sc.to_screen]
        j.flags = sc.ctx.flags()
    return jobs, keep


def render_batch(scenes, device=None, sync_stats=True):
    """rf_render_batch: every scene rendered as one pass over all targets.
    Returns one Stats per scene (added into each scene's ctx.stats), or None
    when sync_stats is false (the work is only queued)."""
    if not scenes:
        return []
    dev = device or scenes[0].target.dev
    jobs, keep = _jobs(scenes)
    out = (CStats * len(scenes))() if sync_stats else None
    _check(lib().rf_render_batch(dev.ptr, jobs, len(scenes),
                                 C.cast(out, C.POINTER(CStats)) if out is not None else None),
           "rf_render_batch")
    del keep
    if out is None:
        return None
    res = []
    for sc, cs in zip(scenes, out):
        st = Stats.from_c(cs)
        sc.ctx.stats += st
        res.append(st)
    return res


def autotune(scenes, reps=3, device=None):
    """rf_ctx_autotune over a batch: returns (tile_w, warps, best_ms) and
    keeps that tiling on the device context; the targets are unchanged."""
    dev = device or scenes[0].target.dev
    jobs, keep = _jobs(scenes)
    tw, wp, ms = C.c_uint32(), C.c_uint32(), C.c_float()
    _check(lib().rf_ctx_autotune(dev.ptr, jobs, len(scenes), reps, C.byref(tw), C.byref(wp),
                                 C.byref(ms)), "rf_ctx_autotune")
    del keep
    return tw.value, wp.value, ms.value


class Server:
    """rf_server: continuous batching over `inflight` pipelines (worker
    threads with their own streams) that read the device context's meshes
    and textures, under a device-memory budget.  While it runs, make no
    other call on that Device."""

    WAIT_FOREVER = 0xFFFFFFFF

    def __init__(self, device, hbm_budget_bytes=0, max_batch=0, inflight=0, staging_bytes=0,
                 max_batch_tris=0):
        self.dev = device
        cfg = ServerConfig(hbm_budget_bytes, max_batch, inflight, staging_bytes, max_batch_tris)
        p = _P()
        _check(lib().rf_server_create(device.ptr, C.byref(cfg), C.byref(p)), "rf_server_create")
        self.ptr = p
        self._keep = {}

    def submit(self, draws, to_screen, w, h, ctx=None, pixfmt=ARGB8888, depth=True,
               color_out=None, depth_out=None, read_depth=None):
        """Queue a scene; returns a ticket.  draws: list of (Mesh, Shader,
        mvp).  depth: the target has a depth buffer (Framebuf) or not
        (Colorbuf); read_depth (default: depth) copies it out too.
        color_out / depth_out: (h, w) uint32 / float32 host arrays that
        receive the image (allocated here when None)."""
        read_depth = depth if read_depth is None else (read_depth and depth)
        ctx = ctx or Context()
        arr = (Draw * max(1, len(draws)))()
        for i, dr in enumerate(draws):
            mesh, shader, mvp = dr[:3]
            arr[i].mesh = mesh.handle
            arr[i].shader = shader.kind
            arr[i].flags = dr[3] if len(dr) > 3 else 0
            arr[i].uniforms = shader.uniforms(mvp)
        if color_out is None:
            color_out = np.empty((h, w), np.uint32)
        if read_depth and depth_out is None:
            depth_out = np.empty((h, w), np.float32)
        q = Request()
        q.ndraws = len(draws)
        q.draws = C.cast(arr, C.POINTER(Draw))
        q.viewport[:] = [float(x) for x in np.asarray(to_screen, np.float32).reshape(-1)]
        q.flags = ctx.flags()
        q.w, q.h, q.pixfmt, q.has_depth = w, h, pixfmt, int(bool(depth))
        cc = 0xFF000000 if ctx.color_clear is None else ctx.color_clear
        q.clear_rgba = cc
        q.depth_clear = float("inf") if ctx.depth_clear is None else ctx.depth_clear
        q.color_out = _u32p(color_out)
        q.depth_out = _fp(depth_out) if read_depth else None
        t = C.c_uint64()
        _check(lib().rf_server_submit(self.ptr, C.byref(q), C.byref(t)), "rf_server_submit")
        self._keep[t.value] = (color_out, depth_out if read_depth else None)
        return t.value

    def wait(self, ticket, timeout_ms=WAIT_FOREVER):
        """(color, depth, result dict) of a request; raises RfError with
        code 7 on timeout.  result["status"] is the request's own status."""
        r = Result()
        _check(lib().rf_server_wait(self.ptr, ticket, timeout_ms, C.byref(r)), "rf_server_wait")
        col, dep = self._keep.pop(ticket)
        res = {"status": r.status, "batch_size": r.batch_size, "batch_id": r.batch_id,
               "queue_ms": r.queue_ms, "render_ms": r.render_ms, "total_ms": r.total_ms,
               "stats": Stats.from_c(r.stats), "gpu_start_ns": r.gpu_start_ns,
               "gpu_end_ns": r.gpu_end_ns, "pipeline": r.pipeline}
        return col, dep, res

    def counts(self):
        b, c, q = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().rf_server_counts(self.ptr, C.byref(b), C.byref(c), C.byref(q)),
               "rf_server_counts")
        return {"batches": b.value, "completed": c.value, "queued": q.value}

    def memory(self):
        """Admission charges in flight now, their peak, and the most batches
        in flight at once."""
        c, pk, pi = C.c_uint64(), C.c_uint64(), C.c_uint32()
        _check(lib().rf_server_memory(self.ptr, C.byref(c), C.byref(pk), C.byref(pi)),
               "rf_server_memory")
        return {"charged": c.value, "peak_charged": pk.value, "peak_inflight": pi.value}

    def close(self):
        if self.ptr:
            lib().rf_server_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ObjError(ValueError):
    pass


def parse_obj(text, attrs=OBJ_POSITION):
    """Wavefront OBJ text (str or bytes) -> (verts (n, 3 + nattr) float32,
    faces (m, 3) uint32), like retrofire's reader (geom/src/io.rs).  Runs
    in the library on the host; raises ObjError with the reader's message."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    vp, ip = C.POINTER(C.c_float)(), C.POINTER(C.c_uint32)()
    nv, na, nt = C.c_uint32(), C.c_uint32(), C.c_uint32()
    err = C.create_string_buffer(256)
    code = lib().rf_obj_parse(data, len(data), attrs, C.byref(vp), C.byref(nv), C.byref(na),
                              C.byref(ip), C.byref(nt), err, 256)
    if code == 2 and err.value:
        raise ObjError(err.value.decode())
    _check(code, "rf_obj_parse")
    try:
        w = 3 + na.value
        verts = np.ctypeslib.as_array(vp, (nv.value * w,)).copy().reshape(nv.value, w) \
            if nv.value else np.zeros((0, w), np.float32)
        faces = np.ctypeslib.as_array(ip, (nt.value * 3,)).copy().reshape(nt.value, 3) \
            if nt.value else np.zeros((0, 3), np.uint32)
    finally:
        lib().rf_obj_free(C.cast(vp, _P))
        lib().rf_obj_free(C.cast(ip, _P))
    return verts, faces
