"""The measured workloads beyond the headline frame, as lists of scenes.

A scene is a dict: w, h, vp (viewport matrix) and draws, each draw a dict of
verts, faces, shader, mvp, pos_dim and tex (texels or None); draws that
share a vertex array share one device mesh.

  cube    640x480 textured cube, seed-drawn rotation (latency case)
  cubes   1920x1080, 10,000 instanced tex x Gouraud cubes, one render()
          call per instance (demos/src/bin/crates.rs:114-133 idiom)
  batch   256 uneven independent scenes (scenes.batch_scenes)
  serve   the first requests of the serving stream as scenes
"""
import ctypes as C
import functools
import time

import numpy as np

from . import (GOURAUD, TEX_GOURAUD, TEXTURED, Framebuf, Mesh, Scene, Shader, Texture, scenes)


def _draw(verts, faces, shader, mvp=None, pos_dim=3, tex=None):
    return dict(verts=verts, faces=faces, shader=shader, mvp=mvp, pos_dim=pos_dim, tex=tex)


def _from_batch_entry(sc):
    if sc["kind"] == "fill":
        draws = [_draw(sc["verts"], sc["faces"], GOURAUD, None, 4)]
    else:
        draws = [_draw(sc["verts"], sc["faces"], TEX_GOURAUD, m, 3, sc["tex"]) for m in sc["mvps"]]
    return dict(w=sc["w"], h=sc["h"], vp=sc["vp"], draws=draws)


@functools.lru_cache(maxsize=None)
def scenes_for(name):
    if name == "cube":
        c = scenes.textured_cube(seed=1, w=640, h=480)
        return [dict(w=640, h=480, vp=c["vp"],
                     draws=[_draw(c["verts"], c["faces"], TEXTURED, c["mvp"], 3, c["tex"])])]
    if name == "cubes":
        s = scenes.instanced_cubes(ninst=10_000, w=1920, h=1080, seed=3, tex_size=1024)
        s["kind"] = "cubes"
        return [_from_batch_entry(s)]
    if name == "batch":
        return [_from_batch_entry(s) for s in scenes.batch_scenes(256, seed=4)]
    if name == "serve":
        built = [(sh, b()) for _, sh, b in scenes.SERVING_MESHES]
        tex = scenes.noise_texture(256, 9)
        kinds = {"textured": TEXTURED, "gouraud": GOURAUD, "tex_gouraud": TEX_GOURAUD}
        out = []
        for r in scenes.serving_requests(60, 2000.0, seed=2100):
            sh, (v, f) = built[r["mesh"]]
            k = kinds[sh]
            out.append(dict(w=r["w"], h=r["h"], vp=r["vp"],
                            draws=[_draw(v, f, k, r["mvp"], 3, tex if k != GOURAUD else None)]))
        return out
    raise ValueError(name)


def describe(name):
    return {
        "cube": {"workload": "textured_cube_640x480", "triangles": 12, "scenes": 1,
                 "shader": "textured (repeat-pot 64x64 checker)"},
        "cubes": {"workload": "instanced_cubes_1080p_10k", "triangles": 120_000, "draws": 10_000,
                  "scenes": 1, "shader": "tex x gouraud (1024x1024 noise)"},
        "batch": {"workload": "uneven_batch_256", "scenes": 256,
                  "sizes": "W 64..1920, H 64..1080, 12..200k triangles, log-uniform",
                  "recipes": "fill-stress or instanced cubes by coin flip"},
        "serve": {"workload": "serving_poisson", "scenes": 60},
    }[name]


def cpu_sample_indices(name, workers=1):
    """Scenes the oracle renders for the CPU baseline (about 5-30 s of one
    core; one share per worker)."""
    n = len(scenes_for(name))
    if name == "cube":
        return [0] * (2000 * workers)
    if name == "cubes":
        return [0] * workers
    if name == "batch":
        return list(range(n))
    return list(range(n)) * max(1, workers // 4)


def upload(scs, dev):
    meshes, texes, targets, out = {}, {}, [], []
    for sc in scs:
        tg = Framebuf(sc["w"], sc["h"], device=dev)
        tg.clear()
        targets.append(tg)
        items = []
        for d in sc["draws"]:
            key = (id(d["verts"]), id(d["faces"]), d["pos_dim"])
            if key not in meshes:
                meshes[key] = (Mesh(d["verts"], d["faces"], pos_dim=d["pos_dim"], device=dev),
                               d["verts"], d["faces"])
            tex = None
            if d["tex"] is not None:
                if id(d["tex"]) not in texes:
                    texes[id(d["tex"])] = Texture(d["tex"], device=dev)
                tex = texes[id(d["tex"])]
            items.append((meshes[key][0], Shader(d["shader"], texture=tex), d["mvp"]))
        out.append(Scene(tg, items, sc["vp"]))
    return {"scenes": out, "targets": targets, "meshes": meshes, "textures": texes}


def e2e(objs, dev, steps, warmup, objs2=None):
    """Per step from host buffers (pinned): every mesh's vertices and
    indices uploaded, every target cleared, the batch rendered, every
    target's colour + depth read back.  The steps are streamed over two
    device copies of the scenes (objs, objs2: rf_mesh_update_async /
    rf_target_read_async on the library's copy streams), so one step's
    copies overlap the other copy's rendering; the time is the wall clock to
    the final sync.  One step done synchronously (upload, render, read back)
    gives the latency percentiles.  Returns seconds over `steps`, the bytes
    each way per step and the latencies."""
    import torch
    from . import render_batch
    sets = [objs] + ([objs2] if objs2 is not None else [])
    host = {}  # the pinned copy of every mesh's arrays, shared by the sets
    pins, outs = [], []
    h2d = d2h = 0
    for o in sets:
        pin = []
        for key, (m, v, f) in o["meshes"].items():
            if key not in host:
                pv = torch.from_numpy(np.ascontiguousarray(v, np.float32)).pin_memory()
                pf = torch.from_numpy(np.ascontiguousarray(f, np.uint32).view(np.int32)).pin_memory()
                host[key] = (pv, pf, pv.numpy(), pf.numpy().view(np.uint32))
                h2d += pv.numel() * 4 + pf.numel() * 4
            pin.append((m, host[key][2], host[key][3]))
        pins.append(pin)
        out = []
        for tg in o["targets"]:
            c = torch.empty((tg.h, tg.w), dtype=torch.int32).pin_memory()
            d = torch.empty((tg.h, tg.w), dtype=torch.float32).pin_memory()
            out.append((tg, c, d, c.numpy().view(np.uint32), d.numpy()))
        outs.append(out)
    d2h = sum(8 * tg.w * tg.h for tg in objs["targets"])
    from . import _fp, _u32p, lib

    def render(k):
        for tg in sets[k]["targets"]:
            tg.clear()
        render_batch(sets[k]["scenes"], device=dev, sync_stats=False)

    def streamed(n):
        for m, v, f in pins[0]:
            m.update_async(v, f)
        for i in range(n):
            k = i % len(sets)
            render(k)
            if i + 1 < n:
                for m, v, f in pins[(i + 1) % len(sets)]:
                    m.update_async(v, f)
            for tg, _, _, c, d in outs[k]:
                tg.read_async(c, d)
        dev.sync()

    def sync_step():
        for m, v, f in pins[0]:
            m.update(v, f)
        render(0)
        for tg, _, _, c, d in outs[0]:
            code = lib().rf_target_read(dev.ptr, tg.handle, _u32p(c), _fp(d))
            if code:
                raise RuntimeError("rf_target_read: %d" % code)

    streamed(max(2, warmup))
    t0 = time.perf_counter()
    streamed(steps)
    wall = time.perf_counter() - t0
    lat = []
    for _ in range(max(3, min(steps, 20))):
        t1 = time.perf_counter()
        sync_step()
        lat.append(time.perf_counter() - t1)
    ms = sorted(x * 1e3 for x in lat)
    return {"seconds": wall, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "mode": "streamed over %d device copies of the scenes, async copies on the library's "
                    "copy streams, wall clock to the final sync" % len(sets),
            "latency_ms": {"p50": ms[len(ms) // 2], "p99": ms[min(len(ms) - 1, int(0.99 * len(ms)))],
                           "note": "one synchronous step: upload, render, read back"}}


def render_per_frame(scenes_, device, sync_stats=False):
    """The plain per-frame drop-in over a batch's scenes: one
    rf_render_draws (one frame of render() calls into one target) per
    scene, in order, on the device's stream.  Returns each scene's Stats
    when sync_stats is set."""
    from . import CStats, Stats, _check, _fp, lib
    L = lib()
    out = []
    for sc in scenes_:
        arr = sc._draw_array()
        fl = sc.ctx.flags()
        cs = CStats() if sync_stats else None
        _check(L.rf_render_draws(device.ptr, arr, len(sc.draws), _fp(sc.to_screen),
                                 sc.target.handle, C.byref(fl), C.byref(cs) if cs else None),
               "rf_render_draws")
        if sync_stats:
            out.append(Stats.from_c(cs))
    return out if sync_stats else None


def target_digests(targets):
    """blake2b of every target's colour and depth bytes (read back)."""
    import hashlib
    out = []
    for tg in targets:
        c, d = tg.read()
        h = hashlib.blake2b(c.tobytes(), digest_size=16)
        if d is not None:
            h.update(d.tobytes())
        out.append(h.hexdigest())
    return out


def close(objs):
    for m, _, _ in objs["meshes"].values():
        m.close()
    for t in objs["textures"].values():
        t.close()
    for tg in objs["targets"]:
        tg.close()
