#!/usr/bin/env python
"""Benchmark: fragments/s of the fill-rate stress frame on one GB300.

Workload (the largest single-GPU configuration of the reference's benchmark
set that renders one frame): 1920x1080 ARGB8888 colour + f32 depth target,
100,000 Gouraud triangles given in clip space (screen area log-uniform in
1..1e4 px^2, ~5% crossing the near/far plane), depth test on, default
Context.  A step = Frame::clear + one render() of the whole mesh.

value   fragments (Stats.frags.i) per second with the mesh resident in HBM,
        timed with CUDA events around each step on the library's stream; an
        L2 flush (512 MiB write) runs between steps, outside the timed span.
        The frame's launches are replayed as one CUDA graph; the stage times
        and the roofline come from as many steps before them with the
        library's per-stage events (those run without replay).
e2e     the same metric through the C ABI with host buffers: per step the
        mesh is uploaded from pinned host memory, the target cleared and
        rendered, and its colour + depth read back to pinned memory; steps
        are streamed over four contexts (four CUDA streams, two device meshes
        and targets each, async copies on the contexts' copy streams), so
        neighbouring frames and their copies overlap, and timed by the wall
        clock to the final sync over at least 200 frames.
roofline  achieved = algorithmic bytes of the tile rasteriser per frame
        (4 frags.i + 8 frags.o + 8 W H) / its CUDA-event time; peak = the
        measured HBM copy bandwidth.
batch   the metric's own comparison on the 256 uneven scenes: one
        rf_render_batch per step (CUDA graphs on) against the plain per-frame
        drop-in, one rf_render_draws per scene, on the same targets, timed the
        same way (CUDA events, L2 flush between steps); both legs' images and
        stats are compared bit for bit before timing.
serve   a Poisson request stream at a fixed rate through rf_server (continuous
        batching) against the plain per-frame loop (one request at a time:
        clear, rf_render_draws, read back): frames/s and p50/p99 latency from
        arrival to the image in host memory.

--impl reference times the reference's CPU path (the C++ oracle, a
restatement of retrofire's render(); Rust is not available here) on the
host cores, frame-parallel across all of them.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, NTRI, SEED = 1920, 1080, 100_000, 2
# Frames the library's online tiling needs per frame shape before it keeps
# the fastest tile width (one warm-up + one per width), run before warm-up.
TUNE_FRAMES = 5
WORKLOAD = "fill_stress_1080p_100k_gouraud"
METRIC = "frags/s"


def config(extra=None):
    c = {"workload": WORKLOAD, "target": "%dx%d ARGB8888 + f32 depth" % (W, H),
         "triangles": NTRI, "shader": "gouraud", "seed": SEED,
         "l2": "flushed between steps (512 MiB write)", "parallelism": "replicas"}
    c.update(extra or {})
    return c


def max_over_ranks(ms, world, device):
    """The slowest rank's time (every rank gets it).  Replicas only: the
    path has no exchange step, so this is the one collective."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, world, total_ms):
    """Whole-job rate of `world` replicas that each processed
    `units_per_rank` units, timed by the slowest rank."""
    return units_per_rank * world / (total_ms / 1e3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------ CPU side ---

def _oracle_frames(args):
    """Worker: render `n` frames of the workload with the oracle; returns
    (seconds, frags_i per frame)."""
    n, ntri = args
    sys.path.insert(0, ROOT)
    import numpy as np
    from oracle import oracle as O
    from retrofire_gb300 import scenes
    s = scenes.fill_stress(ntri=ntri, w=W, h=H, seed=SEED)
    d = O.make_draw(s["verts"], s["faces"], 1, pos_dim=4)
    col = np.zeros((H, W), np.uint32)
    dep = np.zeros((H, W), np.float32)
    fr = 0
    t0 = time.perf_counter()
    for _ in range(n):
        O.clear(col, dep)
        st = O.render([d], s["vp"], col, dep, {})
        fr = st.frags_i
    return time.perf_counter() - t0, fr


def cpu_rate(frames_per_worker, workers):
    """frags/s of the oracle, `workers` processes (spawned) in parallel."""
    if workers == 1:
        t, fr = _oracle_frames((frames_per_worker, NTRI))
        return fr * frames_per_worker / t, t
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        pool.map(_oracle_frames, [(0, 1000)] * workers)  # import + build warm-up
        t0 = time.perf_counter()
        res = pool.map(_oracle_frames, [(frames_per_worker, NTRI)] * workers)
        wall = time.perf_counter() - t0
    fr = res[0][1]
    return fr * frames_per_worker * workers / wall, wall


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import build as obuild
    obuild.build()
    cores = os.cpu_count() or 1
    times = []
    _, fr = _oracle_frames((1, NTRI))
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_oracle_frames, [(0, 1000)] * cores)
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_oracle_frames, [(1, NTRI)] * cores)
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                times.append(dt)
    total = sum(times)
    value = fr * cores * len(times) / total
    line = {"metric": METRIC, "value": value, "unit": "frags/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": config({"frames_per_step": cores}),
            "cpu_baseline": {"value": value, "unit": "frags/s", "cores": cores, "kind": "port",
                             "sample": "%d frames per step, one per core, %d timed steps"
                                       % (cores, len(times))},
            "e2e": {"value": value, "unit": "frags/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------ GPU side ---

class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of the tile rasteriser from the committed ncu
    summary (profiles/k_raster_fill_1080p.txt), or None."""
    p = os.path.join(ROOT, "profiles", "k_raster_fill_1080p.txt")
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def run_e2e(args, rf, dev, mesh, tg, sh, ctx, vp, s, frags_i, world):
    """The metric through the C ABI with host buffers in and out.  Every
    step uploads its mesh from page-locked host memory and reads its colour
    and depth target back into page-locked memory.  Steps are streamed over
    four contexts (four CUDA streams), each with two device meshes and
    targets: rf_mesh_update_async / rf_target_read_async run on the
    contexts' copy streams while the other contexts' frames render, so
    neighbouring frames' kernels and copies overlap on the device (1080p
    fill frame: 267 G frags/s over two contexts, 286 G over three, 290 G
    over four).  The value is the wall-clock rate up to the final
    sync.  A synchronous step (upload, render, read back, one at a time, one
    context) gives the latency.  --e2e-contexts sets how many contexts the
    frames rotate over."""
    import ctypes as C
    import numpy as np
    import torch
    pin_v = torch.from_numpy(s["verts"]).pin_memory()
    pin_i = torch.from_numpy(s["faces"].astype(np.int32)).pin_memory()
    vnp, inp = pin_v.numpy(), pin_i.numpy().view(np.uint32)

    def pinned_out():
        c = torch.empty((H, W), dtype=torch.int32).pin_memory()
        d = torch.empty((H, W), dtype=torch.float32).pin_memory()
        return (c, d, c.numpy().view(np.uint32), d.numpy())

    nctx = max(1, args.e2e_contexts)
    extra = []
    for _ in range(nctx - 1):
        d = rf.Device()
        d.set_tiling(*dev.last_tiling())  # the tile width the first context settled on
        d.set_graphs(True)  # every context replays each frame's launches as one graph
        extra.append(d)
    devs = [dev] + extra
    own = []  # the objects created here (closed at the end)
    slots = []  # (device, mesh, target, pinned outputs): frames rotate over the contexts
    for b in range(2):
        for d in devs:
            if d is dev and b == 0:
                m, t = mesh, tg
            else:
                m = rf.Mesh(s["verts"], s["faces"], pos_dim=4, device=d)
                t = rf.Framebuf(W, H, rf.ARGB8888, True, device=d)
                own += [m, t]
            slots.append((d, m, t, pinned_out()))
    L = rf.lib()

    def streamed(n):
        slots[0][1].update_async(vnp, inp)
        for i in range(n):
            _, m, t, o = slots[i % len(slots)]
            t.clear(ctx.color_clear, ctx.depth_clear)
            rf.render_draws([(m, sh, None)], vp, t, ctx, sync_stats=False)
            if i + 1 < n:
                slots[(i + 1) % len(slots)][1].update_async(vnp, inp)
            t.read_async(o[2], o[3])
        for d in devs:
            d.sync()

    def sync_step():
        mesh.update(vnp, inp)
        tg.clear(ctx.color_clear, ctx.depth_clear)
        rf.render_draws([(mesh, sh, None)], vp, tg, ctx, sync_stats=False)
        o = slots[0][3]
        code = L.rf_target_read(dev.ptr, tg.handle, o[2].ctypes.data_as(C.POINTER(C.c_uint32)),
                                o[3].ctypes.data_as(C.POINTER(C.c_float)))
        if code:
            raise rf.RfError(code, "rf_target_read")

    streamed(max(len(slots), args.warmup))  # (every slot at least once)
    # every slot renders the same frame: their read-backs agree bit for bit
    ref = None
    for _, _, _, o in slots:
        h = hash(o[2].tobytes()) ^ hash(o[3].tobytes())
        if ref is not None and h != ref:
            raise RuntimeError("streamed frames differ between contexts")
        ref = h
    # (at least 200 frames: the wall clock of a few milliseconds of frames
    # varies by several per cent from run to run)
    nfr = max(args.steps, 200)
    t0 = time.perf_counter()
    streamed(nfr)
    wall = time.perf_counter() - t0
    for d in devs:
        d.take_stats()
    lat = []
    for _ in range(max(3, min(args.steps, 20))):
        t1 = time.perf_counter()
        sync_step()
        lat.append(time.perf_counter() - t1)
    for o in own:
        o.close()
    for d in extra:
        d.close()
    lat_ms = sorted(x * 1e3 for x in lat)
    total_ms = max_over_ranks(1e3 * wall, world, "cuda")
    return {"value": replica_rate(frags_i * nfr, world, total_ms), "unit": "frags/s", "frames": nfr,
            "h2d_bytes_per_step": int(s["verts"].nbytes + s["faces"].nbytes),
            "d2h_bytes_per_step": int(2 * 4 * W * H),
            "mode": "streamed over %d contexts (%d CUDA streams) with two device meshes and "
                    "targets each, async copies on the contexts' copy streams, CUDA graph "
                    "replay, wall clock to the final sync" % (nctx, nctx),
            "latency_ms": {"p50": lat_ms[len(lat_ms) // 2],
                           "p99": lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))],
                           "note": "one synchronous step on one context: upload, render, "
                                   "read back"}}


def batch_leg(args, dev, stream, flush, local):
    """C4 batched vs the plain per-frame drop-in (see the module doc)."""
    import torch
    import retrofire_gb300 as rf
    from retrofire_gb300 import workloads
    scs = workloads.scenes_for("batch")
    objs = workloads.upload(scs, dev)
    batch = objs["scenes"]
    targets = objs["targets"]

    def clear_all():
        for tg in targets:
            tg.clear()

    # Parity of the two legs (untimed): every scene's image and stats.
    clear_all()
    st_b = rf.render_batch(batch, device=dev)
    dig_b = workloads.target_digests(targets)
    clear_all()
    st_f = workloads.render_per_frame(batch, dev, sync_stats=True)
    dig_f = workloads.target_digests(targets)
    bad_img = [i for i, (a, b) in enumerate(zip(dig_b, dig_f)) if a != b]
    bad_st = [i for i, (a, b) in enumerate(zip(st_b, st_f)) if a.as_dict() != b.as_dict()]
    same = not bad_img and not bad_st
    mismatch = None if same else {
        "images": bad_img[:16], "n_images": len(bad_img), "stats": bad_st[:16], "n_stats": len(bad_st),
        "first_stats": [st_b[bad_st[0]].as_dict(), st_f[bad_st[0]].as_dict()] if bad_st else None}
    frags_i = sum(x.frags_i for x in st_b)
    frags_o = sum(x.frags_o for x in st_b)
    px = sum(sc["w"] * sc["h"] for sc in scs)
    ntri = sum(len(d["faces"]) for sc in scs for d in sc["draws"])

    def timed(step, graphs):
        dev.set_graphs(graphs)
        for _ in range(TUNE_FRAMES):  # online tiling settles per frame shape (untimed)
            step()
        step_ms, _, launches, clk = device_time(dev, stream, step, args.steps, args.warmup, flush,
                                                local, stages=False)
        dev.set_graphs(False)
        ms = sum(step_ms) / len(step_ms)
        return {"ms_per_step": ms, "frags_per_s": frags_i / (ms / 1e3),
                "tris_per_s": ntri / (ms / 1e3), "frames_per_s": len(scs) / (ms / 1e3),
                "gpu_launches_per_step": launches / args.steps, "clocks": clk}

    def batched():
        clear_all()
        rf.render_batch(batch, device=dev, sync_stats=False)

    def per_frame():
        clear_all()
        workloads.render_per_frame(batch, dev)

    b = timed(batched, True)
    b.update(graphs=True, tile_w=dev.last_tiling()[0], calls_per_step=1)  # (read right after its steps)
    f = timed(per_frame, False)
    f.update(graphs=False, calls_per_step=len(scs))
    peak, peak_kind = measured_peak()
    alg = 4 * frags_i + 8 * frags_o + 8 * px
    workloads.close(objs)
    return {"workload": "uneven_batch_256", "scenes": len(scs), "triangles": ntri,
            "frags_i_per_step": frags_i, "frags_o_per_step": frags_o,
            "batched": b, "per_frame": f,
            "batched_vs_per_frame": f["ms_per_step"] / b["ms_per_step"],
            "batched_model_gbs": alg / (b["ms_per_step"] / 1e3) / 1e9,
            "peak_gbs": peak, "peak_kind": peak_kind,
            "parity_checked": {"batched_equals_per_frame": bool(same), "scenes": len(scs),
                               "mismatch": mismatch,
                               "what": "colour + depth images (blake2b) and per-scene stats, "
                                       "bit for bit",
                               "oracle": "every scene bit-exact against the oracle in "
                                         "tests/test_gpu_fullsize.py"},
            "l2": "flushed between steps (512 MiB write)" if flush is not None else "not flushed"}


def serve_leg(args, dev):
    """C5 served vs the plain per-frame request loop at one rate."""
    import retrofire_gb300 as rf
    from retrofire_gb300 import scenes, serve
    rate = args.serve_rate
    n = max(50, int(rate * args.duration))
    reqs = scenes.serving_requests(n, rate, seed=100 + int(rate))
    ms = serve.MeshSet(dev)
    warm = scenes.serving_requests(60, rate, seed=7)
    out = {"rate_per_s": rate, "requests": n, "duration_s": args.duration,
           "meshes": [m[0] for m in scenes.SERVING_MESHES],
           "resolutions": scenes.SERVING_RESOLUTIONS,
           "target": "ARGB8888 + f32 depth, depth test on (Context::default)",
           "readback": "colour to host per request"}
    srv = rf.Server(dev, hbm_budget_bytes=64 << 30, inflight=args.inflight)
    try:
        serve.run_load(srv, ms, warm, realtime=False, read_depth=False)
        res, wall = serve.run_load(srv, ms, reqs, realtime=True, read_depth=False)
        mem = srv.memory()
    finally:
        srv.close()
    s = serve.latency_summary(res)
    fr = sum(r[2]["stats"].frags_i for r in res)
    out["served"] = dict(s, frames_per_s=n / wall, frags_per_s=fr / wall, inflight=args.inflight,
                         peak_inflight=mem["peak_inflight"], peak_charged_gb=mem["peak_charged"] / 1e9)
    serve.run_per_frame(dev, ms, warm, realtime=False)
    res_f, wall_f = serve.run_per_frame(dev, ms, reqs, realtime=True)  # depth targets, colour read
    sf = serve.latency_summary(res_f)
    fr_f = sum(r[2]["stats"].frags_i for r in res_f)
    out["per_frame"] = dict(sf, frames_per_s=n / wall_f, frags_per_s=fr_f / wall_f)
    same = all(np.array_equal(a[0], b[0]) for a, b in zip(res, res_f)) and \
        all(a[2]["stats"].as_dict() == b[2]["stats"].as_dict() for a, b in zip(res, res_f))
    out["parity_checked"] = {"served_equals_per_frame": bool(same), "requests": n,
                             "what": "colour images and stats of every request, bit for bit"}
    out["served_vs_per_frame"] = {"frames_per_s": out["served"]["frames_per_s"] /
                                  out["per_frame"]["frames_per_s"],
                                  "p99_ms": out["per_frame"]["p99_ms"] / out["served"]["p99_ms"]}
    ms.close()
    return out


def run_gpu(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import retrofire_gb300 as rf
    from retrofire_gb300 import scenes

    cpu = None
    if rank == 0 and not args.no_cpu:
        # Single-threaded oracle on a bounded sample (the reference renders
        # on one thread), measured before the GPU work starts.
        r1, t1 = cpu_rate(args.cpu_frames, 1)
        cpu = {"value": r1, "unit": "frags/s", "cores": 1, "kind": "port",
               "sample": "%d full frames of the workload, single thread, %.1f s"
                         % (args.cpu_frames, t1)}

    s = scenes.fill_stress(ntri=NTRI, w=W, h=H, seed=SEED)
    stream = torch.cuda.Stream()
    dev = rf.Device(stream.cuda_stream)
    if args.tile or args.warps:
        dev.set_tiling(args.tile, args.warps)
    mesh = rf.Mesh(s["verts"], s["faces"], pos_dim=4, device=dev)
    tg = rf.Framebuf(W, H, rf.ARGB8888, True, device=dev)
    sh = rf.Shader.gouraud()
    ctx = rf.Context()
    vp = s["vp"]
    flush = None if args.no_flush else torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def step(sync_stats=False):
        tg.clear(ctx.color_clear, ctx.depth_clear)
        return rf.render_draws([(mesh, sh, None)], vp, tg, ctx, sync_stats=sync_stats)

    st = step(sync_stats=True)  # one frame for the per-frame stats
    frags_i, frags_o = st.frags_i, st.frags_o
    if not args.tile:
        for _ in range(TUNE_FRAMES):  # online tiling settles (setup, untimed)
            step()
    def timed(n, stage_events):
        """n steps, each bracketed by CUDA events on the library's stream,
        the L2 flushed before each; with stage_events the library also
        records its per-stage events (which turns graph replay off)."""
        dev.set_timing(stage_events)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(n)]
        clocks = Clocks(local)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        k0 = dev.counts()["kernels"]
        clocks.start()
        with torch.cuda.stream(stream):
            for i in range(n):
                if flush is not None:
                    flush.fill_(i & 0xFF)
                evs[i][0].record(stream)
                step()
                evs[i][1].record(stream)
        torch.cuda.synchronize()
        clk = clocks.stop()
        launches = dev.counts()["kernels"] - k0
        stage = dev.stage_ms() if stage_events else None
        dev.set_timing(False)
        return [a.elapsed_time(b) for a, b in evs], launches, clk, stage

    # Per-stage CUDA events first (the raster kernel's time for the
    # roofline), then the timed steps proper with graph replay: the frame's
    # launch sequence is captured once and replayed by one graph launch.
    for _ in range(args.warmup):
        step()
    dev.sync()
    dev.stage_ms()  # discard warm-up timings
    _, _, _, (stage, nfr) = timed(args.steps, True)
    tiling = dev.last_tiling()  # the timed frames' tile width and warps
    dev.set_graphs(True)
    for _ in range(args.warmup):
        step()
    g0 = dev.counts()["graph_launches"]
    step_ms, launches, clk, _ = timed(args.steps, False)
    graph_launches = dev.counts()["graph_launches"] - g0
    total_ms = max_over_ranks(sum(step_ms), world, "cuda")
    ms = total_ms / args.steps
    value = replica_rate(frags_i * args.steps, world, total_ms)

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, rf, dev, mesh, tg, sh, ctx, vp, s, frags_i, world)

    bleg = sleg = None
    others = {}
    if rank == 0 and not args.no_others:
        for name in ("cube", "cubes"):
            others[name] = workload_leg(args, name, stream, flush, local)
    if rank == 0 and not args.no_batch:
        bleg = batch_leg(args, dev, stream, flush, local)
    if rank == 0 and not args.no_serve:
        sleg = serve_leg(args, rf.Device())
    if world > 1:
        torch.distributed.barrier()

    if rank == 0:
        peak, peak_kind = measured_peak()
        raster_ms = stage["raster"] / max(nfr, 1)
        alg_bytes = 4 * frags_i + 8 * frags_o + 8 * W * H
        achieved = alg_bytes / (raster_ms / 1e3) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": "frags/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded fill-rate stress scene)",
            "config": config({"tile_w": tiling[0], "warps_per_block": tiling[1],
                              "tiling": "explicit" if args.tile else
                              "online per frame shape, settled before the warm-up",
                              "launch": "CUDA graph replay of the frame (%d graph launches "
                                        "in the timed steps); the stage times and the "
                                        "roofline come from as many steps before them with "
                                        "per-stage events, which run without replay"
                                        % graph_launches}),
            "tris_per_s": NTRI * args.steps * world / (total_ms / 1e3),
            "frames_per_s": args.steps * world / (total_ms / 1e3),
            "frags_o_per_frame": frags_o, "frags_i_per_frame": frags_i,
            "stage_ms_per_frame": {k: v / max(nfr, 1) for k, v in stage.items()},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": ncu_traffic(),
                         "kernel": "k_raster", "peak_kind": peak_kind,
                         "alg_bytes_per_launch": alg_bytes},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk,
            "batch": bleg,
            "serve": sleg,
            "cube": others.get("cube"),
            "cubes": others.get("cubes"),
        }
        print(json.dumps(line))
    for o in (mesh, tg):
        o.close()
    dev.close()
    if world > 1:
        torch.distributed.destroy_process_group()


# ------------------------------------------------- further workloads ---
#
# --workload picks one of the reference's other configurations; each prints
# one JSON line with the same keys as the default; the headline line is the
# default workload's.

def _oracle_scene(sc):
    """Renders one bench scene dict with the oracle; returns Stats."""
    import numpy as np
    from oracle import oracle as O
    col = np.zeros((sc["h"], sc["w"]), np.uint32)
    dep = np.zeros((sc["h"], sc["w"]), np.float32)
    O.clear(col, dep)
    ods = [O.make_draw(d["verts"], d["faces"], d["shader"], d["mvp"], pos_dim=d["pos_dim"],
                       tex=d.get("tex")) for d in sc["draws"]]
    return O.render(ods, sc["vp"], col, dep, {})


def _oracle_scenes(args):
    """Worker: (seconds, frags_i, n) of the oracle over the given scenes."""
    sys.path.insert(0, ROOT)
    from retrofire_gb300 import workloads
    name, idx = args
    scs = workloads.scenes_for(name)
    fr = 0
    t0 = time.perf_counter()
    for i in idx:
        fr += _oracle_scene(scs[i]).frags_i
    return time.perf_counter() - t0, fr, len(idx)


def cpu_sample(name, idx, workers):
    """frags/s and items/s of the oracle over scenes `idx` of a workload."""
    if workers == 1:
        t, fr, n = _oracle_scenes((name, idx))
        return fr / t, n / t, t
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    parts = [idx[k::workers] for k in range(workers)]
    with ctx.Pool(workers) as pool:
        pool.map(_oracle_scenes, [(name, [])] * workers)
        t0 = time.perf_counter()
        res = pool.map(_oracle_scenes, [(name, p) for p in parts])
        wall = time.perf_counter() - t0
    fr = sum(r[1] for r in res)
    return fr / wall, len(idx) / wall, wall


def device_time(dev, stream, step, steps, warmup, flush, local, stages=True):
    import torch
    for _ in range(warmup):
        step()
    dev.sync()
    dev.stage_ms()
    if stages:
        dev.set_timing(True)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    clocks = Clocks(local)
    torch.cuda.synchronize()
    k0 = dev.counts()["kernels"]
    clocks.start()
    with torch.cuda.stream(stream):
        for i in range(steps):
            if flush is not None:
                flush.fill_(i & 0xFF)
            evs[i][0].record(stream)
            step()
            evs[i][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = dev.counts()["kernels"] - k0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    stage, nfr = dev.stage_ms()
    dev.set_timing(False)
    return step_ms, {k: v / max(nfr, 1) for k, v in stage.items()}, launches, clk


def measure_workload(args, name, scs, dev, stream, flush, local, world):
    """Upload one of the further configurations (C1 cube / C3 cubes / C4
    batch) to dev and time it: per-step device times with CUDA events, the
    stage times, and the streamed end-to-end seconds.  The caller closes
    the returned scenes (objs) and turns the seconds into a rate."""
    import retrofire_gb300 as rf
    from retrofire_gb300 import workloads
    objs = workloads.upload(scs, dev)
    batch = objs["scenes"]
    st = rf.render_batch(batch, device=dev)  # per-scene stats of one step
    frags_i = sum(x.frags_i for x in st)
    frags_o = sum(x.frags_o for x in st)
    px = sum(sc["w"] * sc["h"] for sc in scs)
    graphs = name == "cube"
    if graphs:
        dev.set_graphs(True)

    def step():
        for tg in objs["targets"]:
            tg.clear()
        rf.render_batch(batch, device=dev, sync_stats=False)

    if not args.tile:
        for _ in range(TUNE_FRAMES):  # online tiling settles (setup, untimed)
            step()
    if world > 1:
        import torch
        torch.distributed.barrier()
    step_ms, stage, launches, clk = device_time(dev, stream, step, args.steps, args.warmup,
                                                flush, local, stages=not graphs)
    e2e = None
    if not args.no_e2e:
        objs2 = workloads.upload(scs, dev)  # a second device copy to stream over
        e2e = workloads.e2e(objs, dev, args.steps, max(1, args.warmup), objs2)
        workloads.close(objs2)
    return {"objs": objs, "frags_i": frags_i, "frags_o": frags_o, "px": px, "graphs": graphs,
            "step_ms": step_ms, "stage": stage, "launches": launches, "clk": clk, "e2e": e2e}


def workload_leg(args, name, stream, flush, local):
    """The default line's summary of C1 (textured cube) or C3 (instanced
    cubes) on a fresh device of its own: device time per frame, the raster
    stage, and the streamed end-to-end rate with one synchronous frame's
    latency."""
    import retrofire_gb300 as rf
    from retrofire_gb300 import workloads
    dev = rf.Device(stream.cuda_stream)
    scs = workloads.scenes_for(name)
    m = measure_workload(args, name, scs, dev, stream, flush, local, 1)
    ms = sum(m["step_ms"]) / len(m["step_ms"])
    out = {"workload": workloads.describe(name)["workload"], "graphs": m["graphs"],
           "tile_w": dev.last_tiling()[0], "ms_per_frame": ms,
           "frags_per_s": m["frags_i"] / (ms / 1e3), "frags_i_per_frame": m["frags_i"],
           "raster_ms": m["stage"].get("raster") if m["stage"] and not m["graphs"] else None,
           "gpu_launches_per_frame": m["launches"] / max(1, args.steps), "clocks": m["clk"]}
    e2e = m["e2e"]
    if e2e is not None:
        out["e2e"] = {"frags_per_s": m["frags_i"] * args.steps / e2e.pop("seconds"),
                      "latency_ms": e2e.get("latency_ms"),
                      "h2d_bytes_per_frame": e2e.get("h2d_bytes_per_step"),
                      "d2h_bytes_per_frame": e2e.get("d2h_bytes_per_step")}
    workloads.close(m["objs"])
    dev.close()
    return out


def run_workload(args):
    """C1 cube / C3 cubes / C4 batch on one GPU (replicas for N > 1)."""
    import numpy as np
    import torch
    import retrofire_gb300 as rf
    from retrofire_gb300 import workloads
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    name = args.workload
    scs = workloads.scenes_for(name)
    cpu = None
    if rank == 0 and not args.no_cpu:
        idx = workloads.cpu_sample_indices(name)
        fr, it, t = cpu_sample(name, idx, 1)
        cpu = {"value": fr, "unit": "frags/s", "cores": 1, "kind": "port",
               "items_per_s": it,
               "sample": "%d of the workload's %d scenes, single thread, %.1f s"
                         % (len(idx), len(scs), t)}
    stream = torch.cuda.Stream()
    dev = rf.Device(stream.cuda_stream)
    if args.tile or args.warps:
        dev.set_tiling(args.tile, args.warps)
    flush = None if args.no_flush else torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    m = measure_workload(args, name, scs, dev, stream, flush, local, world)
    objs, frags_i, frags_o, px, graphs = m["objs"], m["frags_i"], m["frags_o"], m["px"], m["graphs"]
    step_ms, stage, launches, clk, e2e = m["step_ms"], m["stage"], m["launches"], m["clk"], m["e2e"]
    total_ms = max_over_ranks(sum(step_ms), world, "cuda")
    if e2e is not None:
        e2e_ms = max_over_ranks(1e3 * e2e.pop("seconds"), world, "cuda")
        e2e["value"] = replica_rate(frags_i * args.steps, world, e2e_ms)
        e2e["unit"] = "frags/s"
    if rank == 0:
        peak, peak_kind = measured_peak()
        roof = None
        if stage.get("raster"):
            alg = 4 * frags_i + 8 * frags_o + 8 * px
            ach = alg / (stage["raster"] / 1e3) / 1e9
            roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                    "frac": ach / peak, "traffic": None, "kernel": "k_raster",
                    "peak_kind": peak_kind, "alg_bytes_per_launch": alg}
        line = {
            "metric": METRIC, "value": replica_rate(frags_i * args.steps, world, total_ms),
            "unit": "frags/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": dict(workloads.describe(name), graphs=graphs, tile_w=dev.last_tiling()[0],
                           l2="flushed between steps (512 MiB write)" if flush is not None
                           else "not flushed"),
            "items_per_s": len(scs) * args.steps * world / (total_ms / 1e3),
            "frags_i_per_step": frags_i, "frags_o_per_step": frags_o,
            "stage_ms_per_step": stage if not graphs else None,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches, "clocks": clk,
        }
        print(json.dumps(line))
    workloads.close(objs)
    dev.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_serve(args):
    """C5: Poisson request stream through rf_server; requests/s and latency."""
    import torch
    import retrofire_gb300 as rf
    from retrofire_gb300 import scenes, serve
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = rf.Device()
    ms = serve.MeshSet(dev)
    lines = []
    for rate in args.rates:
        reqs = scenes.serving_requests(int(rate * args.duration), float(rate), seed=100 + int(rate))
        srv = rf.Server(dev, hbm_budget_bytes=64 << 30, inflight=args.inflight)
        serve.run_load(srv, ms, reqs[:40], realtime=False, read_depth=False)  # warm-up
        clocks = Clocks(local)
        clocks.start()
        res, wall = serve.run_load(srv, ms, reqs, realtime=True, read_depth=False)
        clk = clocks.stop()
        s = serve.latency_summary(res)
        d2h = sum(4 * r["w"] * r["h"] for r in reqs) // len(reqs)  # colour read back per request
        lines.append((rate, len(reqs), wall, s, srv.counts(), clk, d2h))
        srv.close()
    cpu = None
    if rank == 0 and not args.no_cpu:
        fr, it, t = cpu_sample("serve", list(range(60)), 1)
        cpu = {"value": it, "unit": "requests/s", "cores": 1, "kind": "port",
               "sample": "60 requests of the stream rendered by the oracle, single thread, %.1f s" % t}
    if rank == 0:
        rate, n, wall, s, c, clk, d2h = lines[-1]
        h2d = 0  # meshes are preloaded handles; a request uploads only its draw records
        line = {"metric": "requests/s", "value": n / wall, "unit": "requests/s", "n_gpus": world,
                "steps": n, "warmup": 40, "ms_per_step": 1e3 * wall / n, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded Poisson request stream)",
                "config": {"workload": "serving_poisson", "rate_per_s": rate,
                           "duration_s": args.duration, "hbm_budget_gb": 64,
                           "meshes": [m[0] for m in scenes.SERVING_MESHES],
                           "resolutions": scenes.SERVING_RESOLUTIONS,
                           "readback": "colour to host per request"},
                "latency_ms": {"p50": s["p50_ms"], "p99": s["p99_ms"]},
                "per_rate": [{"rate": r, "served_per_s": nn / w, **ss, **cc}
                             for r, nn, w, ss, cc, _, _ in lines],
                "e2e": {"value": n / wall, "unit": "requests/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "cpu_baseline": cpu, "roofline": None, "gpu_launches": None, "clocks": clk}
        print(json.dumps(line))
    ms.close()
    dev.close()


def run_reference_workload(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import build as obuild
    obuild.build()
    sys.path.insert(0, ROOT)
    from retrofire_gb300 import workloads
    name = args.workload
    cores = os.cpu_count() or 1
    idx = workloads.cpu_sample_indices(name, cores)
    times, frs, its = [], [], []
    for i in range(args.warmup + args.steps):
        fr, it, t = cpu_sample(name, idx, cores)
        if i >= args.warmup:
            times.append(t)
            frs.append(fr)
            its.append(it)
    metric, unit = ("requests/s", "requests/s") if name == "serve" else (METRIC, "frags/s")
    value = (sum(its) if name == "serve" else sum(frs)) / len(times)
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference", "config": workloads.describe(name),
            "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "kind": "port",
                             "sample": "%d scenes per step over %d cores" % (len(idx), cores)},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--warps", type=int, default=0)
    ap.add_argument("--cpu-frames", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling)")
    ap.add_argument("--e2e-contexts", type=int, default=4,
                    help="contexts (CUDA streams) the end-to-end leg streams its frames over")
    ap.add_argument("--no-flush", action="store_true", help="no L2 flush buffer (profiling)")
    ap.add_argument("--workload", default="fill", choices=["fill", "cube", "cubes", "batch", "serve"],
                    help="fill: the headline frame (default); cube: 640x480 textured cube "
                         "(latency, CUDA graphs); cubes: 10k instanced cubes, one draw each; "
                         "batch: 256 uneven scenes in one pass; serve: Poisson request stream")
    ap.add_argument("--rates", type=float, nargs="+", default=[200.0, 1000.0, 2000.0])
    ap.add_argument("--duration", type=float, default=2.0)
    ap.add_argument("--serve-rate", type=float, default=1000.0,
                    help="request rate of the default line's served-vs-per-frame leg")
    ap.add_argument("--inflight", type=int, default=2, help="serving pipelines")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-vs-per-frame leg")
    ap.add_argument("--no-serve", action="store_true", help="skip the served-vs-per-frame leg")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the default line's textured-cube and instanced-cubes legs")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # --gpus N without a launcher: start N replicas (one process per GPU)
        # the way the multi-GPU runs are launched, and report their line.
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
               "--nproc-per-node", str(args.gpus), "--master-addr", "127.0.0.1",
               "--master-port", str(29500 + os.getpid() % 1000), os.path.abspath(__file__)] + sys.argv[1:]
        sys.exit(subprocess.call(cmd))
    if args.impl == "reference":
        if args.workload == "fill":
            run_reference(args)
        else:
            run_reference_workload(args)
        return
    import __graft_entry__
    __graft_entry__.build()
    if args.workload == "fill":
        run_gpu(args)
    elif args.workload == "serve":
        run_serve(args)
    else:
        run_workload(args)


if __name__ == "__main__":
    main()
