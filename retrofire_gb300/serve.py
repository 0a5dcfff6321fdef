"""Serving helpers over rf_server (include/rfgpu.h): preload a mesh set on a
device context, turn a request stream into scenes, and drive a server with
Poisson arrivals while recording each request's latency.

No counterpart in the reference, which renders one frame per call on the
caller's thread (core/src/render.rs:134).
"""
import threading
import time

import numpy as np

from . import (ARGB8888, GOURAUD, TEX_GOURAUD, TEXTURED, Context, Mesh, Server, Shader, Texture,
               scenes)

SHADERS = {"textured": TEXTURED, "gouraud": GOURAUD, "tex_gouraud": TEX_GOURAUD}


class MeshSet:
    """The preloaded handles of a serving workload: one Mesh per entry of
    `meshes` ((name, shader, builder) as scenes.SERVING_MESHES) and one
    power-of-two texture shared by the textured shaders."""

    def __init__(self, device, meshes=scenes.SERVING_MESHES, tex_size=256, seed=9):
        self.device = device
        self.entries = []
        self.texels = scenes.noise_texture(tex_size, seed)
        self.texture = Texture(self.texels, device=device)
        for name, shader, build in meshes:
            v, f = build()
            m = Mesh(v, f, pos_dim=3, device=device)
            kind = SHADERS[shader]
            sh = Shader(kind, texture=self.texture if kind in (TEXTURED, TEX_GOURAUD) else None)
            self.entries.append((name, m, sh, v, f))

    def draws(self, req):
        _, m, sh, _, _ = self.entries[req["mesh"]]
        return [(m, sh, req["mvp"])]

    def close(self):
        for e in self.entries:
            e[1].close()
        self.texture.close()


def run_load(server, meshset, requests, realtime=True, pixfmt=ARGB8888, depth=True,
             read_depth=None):
    """Submits `requests` (scenes.serving_requests) to `server` at their
    arrival offsets (or all at once when realtime is False) from one thread
    while this thread collects the results.  Returns (results, wall_s) with
    results[i] = (color, depth, result dict)."""
    tickets = [None] * len(requests)
    errors = []

    def producer():
        try:
            t0 = time.perf_counter()
            for i, r in enumerate(requests):
                if realtime:
                    dt = r["t"] - (time.perf_counter() - t0)
                    if dt > 0:
                        time.sleep(dt)
                tickets[i] = server.submit(meshset.draws(r), r["vp"], r["w"], r["h"],
                                           ctx=Context(), pixfmt=pixfmt, depth=depth,
                                           read_depth=read_depth)
        except Exception as e:  # surfaced to the caller below
            errors.append(e)

    t0 = time.perf_counter()
    th = threading.Thread(target=producer)
    th.start()
    out = [None] * len(requests)
    for i in range(len(requests)):
        while tickets[i] is None and th.is_alive():
            time.sleep(0.0002)
        if tickets[i] is None:
            break
        out[i] = server.wait(tickets[i])
    th.join()
    if errors:
        raise errors[0]
    return out, time.perf_counter() - t0


def run_per_frame(device, meshset, requests, realtime=True, depth=True, read_depth=False):
    """The plain per-frame drop-in serving the same stream: one thread takes
    the requests in arrival order and, for each, clears a target of its
    size (with a depth buffer when `depth`), renders it with one
    rf_render_draws and reads the image back (colour, and depth when
    read_depth) before taking the next.  Latency runs from the request's
    arrival to its image being in host memory.  Returns (results, wall_s)
    shaped like run_load's (batch_size 1)."""
    from . import Framebuf, render_draws
    targets = {}
    out = []
    ctx = Context()
    t0 = time.perf_counter()
    for r in requests:
        arrival = t0 + r["t"] if realtime else time.perf_counter()
        if realtime:
            dt = arrival - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
        start = time.perf_counter()
        key = (r["w"], r["h"])
        if key not in targets:
            targets[key] = Framebuf(r["w"], r["h"], ARGB8888, depth, device=device)
        tg = targets[key]
        tg.clear(ctx.color_clear, ctx.depth_clear)
        st = render_draws(meshset.draws(r), r["vp"], tg, ctx, sync_stats=True)
        col, dep = tg.read() if (depth and read_depth) else (_read_color(tg), None)
        done = time.perf_counter()
        out.append((col, dep, {"status": 0, "batch_size": 1,
                               "queue_ms": 1e3 * max(0.0, start - arrival),
                               "render_ms": 1e3 * (done - start),
                               "total_ms": 1e3 * (done - arrival), "stats": st}))
    wall = time.perf_counter() - t0
    for tg in targets.values():
        tg.close()
    return out, wall


def _read_color(tg):
    from . import _check, _u32p, lib
    color = np.empty((tg.h, tg.w), np.uint32)
    _check(lib().rf_target_read(tg.dev.ptr, tg.handle, _u32p(color), None), "rf_target_read")
    return color


def latency_summary(results):
    """p50 / p99 / mean of total_ms and queue_ms, and mean batch size."""
    tot = np.array([r[2]["total_ms"] for r in results])
    q = np.array([r[2]["queue_ms"] for r in results])
    bs = np.array([r[2]["batch_size"] for r in results])
    return {"p50_ms": float(np.percentile(tot, 50)), "p99_ms": float(np.percentile(tot, 99)),
            "mean_ms": float(tot.mean()), "queue_p50_ms": float(np.percentile(q, 50)),
            "queue_p99_ms": float(np.percentile(q, 99)), "mean_batch": float(bs.mean()),
            "max_batch": int(bs.max())}
