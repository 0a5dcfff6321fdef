"""The serving loop (rf_server): continuous batching must not change any
request's result.  Every request's image and stats equal the oracle's
render() of its scene on a cleared target and the same request served
alone; a request submitted while another batch is on the device overlaps
it there; admission keeps the charges in flight within the budget and
refuses what the budget cannot hold; a bad request fails alone."""
import time

import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import mat, scenes, serve
from rfhelp import DrawSpec, assert_parity, oracle_render

pytestmark = pytest.mark.gpu

SMALL = scenes.SERVING_MESHES[:4]  # up to 33k triangles: the oracle stays fast
RES = ((320, 240, 0.5), (640, 480, 0.3), (200, 150, 0.2))


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def oracle_of(ms, req):
    _, _, sh, v, f = ms.entries[req["mesh"]]
    d = DrawSpec(v, f, sh.kind, req["mvp"], tex=ms.texels if sh.texture is not None else None)
    return oracle_render([d], req["vp"], req["w"], req["h"])


def test_mix_equals_alone_and_oracle():
    dev = rf.Device()
    ms = serve.MeshSet(dev, SMALL)
    reqs = scenes.serving_requests(40, 1000.0, seed=12, meshes=SMALL, resolutions=RES)
    x = 17
    srv = rf.Server(dev)
    try:
        alone = serve.run_load(srv, ms, [reqs[x]], realtime=False)[0][0]
        assert alone[2]["batch_size"] == 1 and alone[2]["status"] == 0
        mixed, _ = serve.run_load(srv, ms, reqs, realtime=False)
        assert max(r[2]["batch_size"] for r in mixed) > 1, "no request was batched"
        mx = mixed[x]
        assert np.array_equal(alone[0], mx[0])
        assert np.array_equal(alone[1].view(np.uint32), mx[1].view(np.uint32))
        assert alone[2]["stats"].as_dict() == mx[2]["stats"].as_dict()
        for i, (r, (c, d, res)) in enumerate(zip(reqs, mixed)):
            assert res["status"] == 0
            assert_parity((c, d, res["stats"]), oracle_of(ms, r), what="request %d" % i)
    finally:
        srv.close()
        ms.close()
        dev.close()


def charge(w, h, ntri, nverts, depth=True):
    """The admission charge of one request (include/rfgpu.h): target,
    scratch per triangle and vertex, tile masks at 8x32-pixel tiles."""
    tiles = ((w + 7) // 8) * ((h + 31) // 32)
    mw = (ntri + 31) // 32
    return (w * h * 4 * (2 if depth else 1) + ntri * 5632 + nverts * 24
            + tiles * (mw + (mw + 31) // 32) * 4)


def test_budget_bounds_batches():
    """A budget that holds two requests: no batch is larger, the charges in
    flight over all pipelines never exceed it, and results are unchanged."""
    dev = rf.Device()
    ms = serve.MeshSet(dev, SMALL[:2])
    reqs = scenes.serving_requests(12, 1000.0, seed=13, meshes=SMALL[:2],
                                   resolutions=((320, 240, 1.0),))
    one = max(charge(320, 240, len(e[4]), len(e[3])) for e in ms.entries)
    budget = 2 * one + 1000
    srv = rf.Server(dev, hbm_budget_bytes=budget, inflight=3)
    try:
        res, _ = serve.run_load(srv, ms, reqs, realtime=False)
        assert max(r[2]["batch_size"] for r in res) <= 2
        m = srv.memory()
        assert 0 < m["peak_charged"] <= budget and m["charged"] == 0
        for i, (r, (c, d, st)) in enumerate(zip(reqs, res)):
            assert_parity((c, d, st["stats"]), oracle_of(ms, r), what="request %d" % i)
    finally:
        srv.close()
        ms.close()
        dev.close()


def test_request_overlaps_batch_in_flight():
    """A request submitted while another pipeline's batch is on the GPU is
    admitted at once and its GPU work overlaps that batch's (the global-timer
    stamps at each batch's start and end intersect); its image equals the
    same request served alone and the oracle, and so does the big one's."""
    dev = rf.Device()
    ms = serve.MeshSet(dev)  # grid500k is entry 4
    big = dict(mesh=4, w=1920, h=1080, mvp=scenes.orbit_camera(77, 1920, 1080),
               vp=mat.viewport(0, 1080, 1920, 0))
    small = dict(mesh=0, w=320, h=240, mvp=scenes.orbit_camera(78, 320, 240),
                 vp=mat.viewport(0, 240, 320, 0))
    srv = rf.Server(dev, max_batch=1, inflight=2)
    try:
        def sub(r):
            return srv.submit(ms.draws(r), r["vp"], r["w"], r["h"])
        # Both pipelines see both shapes first (arenas sized, tiling settled).
        for _ in range(6):
            ts = [sub(big), sub(small)]
            for t in ts:
                srv.wait(t)
        alone = srv.wait(sub(small))
        overlapped = False
        for _ in range(5):
            tb = sub(big)
            t0 = time.perf_counter()
            while srv.counts()["queued"] and time.perf_counter() - t0 < 5.0:
                time.sleep(0.0001)
            tsm = sub(small)
            cs, ds, rs = srv.wait(tsm)
            cb, db, rb = srv.wait(tb)
            assert rs["status"] == 0 and rb["status"] == 0
            assert rs["batch_size"] == 1 and rb["batch_size"] == 1
            assert np.array_equal(cs, alone[0])
            assert np.array_equal(ds.view(np.uint32), alone[1].view(np.uint32))
            assert rs["stats"].as_dict() == alone[2]["stats"].as_dict()
            if (rs["pipeline"] != rb["pipeline"]
                    and max(rs["gpu_start_ns"], rb["gpu_start_ns"])
                    < min(rs["gpu_end_ns"], rb["gpu_end_ns"])):
                overlapped = True
                break
        assert overlapped, "no overlap: small %r big %r" % (
            (rs["pipeline"], rs["gpu_start_ns"], rs["gpu_end_ns"]),
            (rb["pipeline"], rb["gpu_start_ns"], rb["gpu_end_ns"]))
        assert srv.memory()["peak_inflight"] >= 2
        assert_parity((cs, ds, rs["stats"]), oracle_of(ms, small), what="small request")
        assert_parity((cb, db, rb["stats"]), oracle_of(ms, big), what="big request")
    finally:
        srv.close()
        ms.close()
        dev.close()


def test_over_budget_and_bad_request():
    dev = rf.Device()
    ms = serve.MeshSet(dev, SMALL[:2])
    srv = rf.Server(dev, hbm_budget_bytes=4 << 20)
    try:
        reqs = scenes.serving_requests(6, 1000.0, seed=14, meshes=SMALL[:2],
                                       resolutions=((160, 120, 1.0),))
        with pytest.raises(rf.RfError) as e:  # 1920x1080 with depth: 16.6 MB
            srv.submit(ms.draws(reqs[0]), reqs[0]["vp"], 1920, 1080)
        assert e.value.code == 5
        # A request whose mesh handle is bad, between good ones.
        bad = rf.Mesh(np.zeros((3, 6), np.float32), np.array([[0, 1, 2]]), device=dev)
        bad_handle = bad.handle
        bad.close()

        class Dead:
            handle = bad_handle

        tickets = []
        for i, r in enumerate(reqs):
            draws = ms.draws(r) if i != 3 else [(Dead(), ms.entries[1][2], r["mvp"])]
            tickets.append(srv.submit(draws, r["vp"], r["w"], r["h"]))
        for i, (t, r) in enumerate(zip(tickets, reqs)):
            c, d, res = srv.wait(t)
            if i == 3:
                assert res["status"] == 1
            else:
                assert res["status"] == 0
                assert_parity((c, d, res["stats"]), oracle_of(ms, r), what="request %d" % i)
        with pytest.raises(rf.RfError) as e:
            srv.wait(tickets[0])  # already collected
        assert e.value.code == 2
        assert srv.counts()["completed"] == len(reqs)
    finally:
        srv.close()
        ms.close()
        dev.close()


def test_poisson_stream_realtime():
    """A short real-time Poisson stream; latencies are recorded and every
    result matches the oracle."""
    dev = rf.Device()
    ms = serve.MeshSet(dev, SMALL)
    reqs = scenes.serving_requests(60, 600.0, seed=15, meshes=SMALL, resolutions=RES)
    srv = rf.Server(dev)
    try:
        res, wall = serve.run_load(srv, ms, reqs, realtime=True)
        s = serve.latency_summary(res)
        assert s["p99_ms"] >= s["p50_ms"] > 0.0
        for i, (r, (c, d, st)) in enumerate(zip(reqs, res)):
            assert_parity((c, d, st["stats"]), oracle_of(ms, r), what="request %d" % i)
    finally:
        srv.close()
        ms.close()
        dev.close()
