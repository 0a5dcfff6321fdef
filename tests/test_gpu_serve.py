"""The serving loop (rf_server): continuous batching must not change any
request's result.  Every request's image and stats equal the oracle's
render() of its scene on a cleared target and the same request served
alone; admission refuses what the budget cannot hold; a bad request fails
alone."""
import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import scenes, serve
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


def test_budget_bounds_batches():
    """A budget that holds about two requests splits the stream into
    batches of at most that many; results are unchanged."""
    dev = rf.Device()
    ms = serve.MeshSet(dev, SMALL[:2])
    reqs = scenes.serving_requests(12, 1000.0, seed=13, meshes=SMALL[:2],
                                   resolutions=((320, 240, 1.0),))
    one = 320 * 240 * 8 + 128 * rf_bytes_per_tri() + 81 * 24
    srv = rf.Server(dev, hbm_budget_bytes=2 * one + 1000)
    try:
        res, _ = serve.run_load(srv, ms, reqs, realtime=False)
        assert max(r[2]["batch_size"] for r in res) <= 2
        for i, (r, (c, d, st)) in enumerate(zip(reqs, res)):
            assert_parity((c, d, st["stats"]), oracle_of(ms, r), what="request %d" % i)
    finally:
        srv.close()
        ms.close()
        dev.close()


def rf_bytes_per_tri():
    return 5632


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
