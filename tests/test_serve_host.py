"""Host side of the serving workload (no GPU): the request stream's
arrival process and mix, the camera and mesh builders, and the load driver
(arrival pacing, result order, error propagation) over a stand-in server."""
import time

import numpy as np

import retrofire_gb300 as rf
from retrofire_gb300 import mat, scenes
from oracle import oracle as O


def test_poisson_arrivals_and_mix():
    reqs = scenes.serving_requests(20000, 1000.0, seed=3)
    t = np.array([r["t"] for r in reqs])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert np.all(gaps > 0)
    assert abs(gaps.mean() - 1e-3) < 5e-5                   # rate 1000 / s
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.05      # exponential: cv = 1
    res = [(r["w"], r["h"]) for r in reqs]
    for (w, h, p) in scenes.SERVING_RESOLUTIONS:
        assert abs(res.count((w, h)) / len(res) - p) < 0.02
    mi = np.bincount([r["mesh"] for r in reqs], minlength=len(scenes.SERVING_MESHES))
    share = mi / len(reqs)                                  # uniform over the mesh set
    assert np.all(np.abs(share - 1.0 / len(scenes.SERVING_MESHES)) < 0.02)


def test_request_stream_is_seeded():
    a = scenes.serving_requests(50, 500.0, seed=7)
    b = scenes.serving_requests(50, 500.0, seed=7)
    for x, y in zip(a, b):
        assert x["t"] == y["t"] and x["mesh"] == y["mesh"] and (x["w"], x["h"]) == (y["w"], y["h"])
        assert np.array_equal(x["mvp"], y["mvp"])


def test_serving_meshes_sizes_and_winding():
    sizes = []
    for name, shader, build in scenes.SERVING_MESHES:
        v, f = build()
        sizes.append(len(f))
        assert f.max() < len(v)
        nattr = {"textured": 2, "gouraud": 3, "tex_gouraud": 5}[shader]
        assert v.shape[1] == 3 + nattr
    assert sizes[0] == 12 and sizes[-1] == 500_000
    # Grid triangles face +y: seen from above they wind counter-clockwise
    # on screen, so the default back-face cull keeps them.
    v, f = scenes.grid_mesh(4, 1)
    p = v[:, [0, 2]]
    a, b, c = p[f[:, 0]], p[f[:, 1]], p[f[:, 2]]
    cross = (b - a)[:, 0] * (c - a)[:, 1] - (b - a)[:, 1] * (c - a)[:, 0]
    assert np.all(cross > 0) or np.all(cross < 0)


def test_orbit_camera_keeps_grid_visible():
    """A request of the stream draws most of a small grid with the default
    context (the oracle, CPU)."""
    v, f = scenes.grid_mesh(8, 1)
    hit = 0
    for seed in range(10):
        mvp = scenes.orbit_camera(seed, 320, 240)
        d = O.make_draw(v, f, rf.GOURAUD, mvp, pos_dim=3)
        col = np.zeros((240, 320), np.uint32)
        dep = np.zeros((240, 320), np.float32)
        O.clear(col, dep)
        st = O.render([d], mat.viewport(0, 240, 320, 0), col, dep, {})
        hit += st.prims_o >= 100
    assert hit >= 8


class _FakeServer:
    """Stands in for rf.Server on the host: tickets in submission order,
    results carrying the submit time, an error planted at one request."""

    def __init__(self, fail_at=None):
        self.sub, self.fail_at, self.n = {}, fail_at, 0

    def submit(self, draws, vp, w, h, ctx=None, pixfmt=0, depth=True, read_depth=None):
        if self.n == self.fail_at:
            raise rf.RfError(2, "rf_server_submit")
        self.n += 1
        self.sub[self.n] = (time.perf_counter(), w, h, draws)
        return self.n

    def wait(self, ticket):
        t, w, h, draws = self.sub.pop(ticket)
        res = {"total_ms": 1.0 + ticket, "queue_ms": 0.5, "batch_size": 1 + ticket % 3,
               "submitted": t, "draws": draws}
        return np.zeros((h, w), np.uint32), None, res


class _FakeMeshSet:
    def draws(self, req):
        return [("mesh%d" % req["mesh"], None, req["mvp"])]


def test_run_load_paces_arrivals_and_keeps_order():
    from retrofire_gb300 import serve
    reqs = scenes.serving_requests(40, 400.0, seed=11)
    srv = _FakeServer()
    t0 = time.perf_counter()
    out, wall = serve.run_load(srv, _FakeMeshSet(), reqs, realtime=True)
    assert len(out) == len(reqs) and wall >= reqs[-1]["t"] * 0.95
    for i, (r, (c, d, res)) in enumerate(zip(reqs, out)):
        assert c.shape == (r["h"], r["w"]) and res["draws"][0][0] == "mesh%d" % r["mesh"]
        # submitted no earlier than its arrival offset
        assert res["submitted"] - t0 >= r["t"] - 1e-3
    s = serve.latency_summary(out)
    assert s["p50_ms"] == np.percentile([2.0 + i for i in range(40)], 50)
    assert s["max_batch"] == 3 and s["queue_p99_ms"] == 0.5


def test_run_load_surfaces_a_submit_error():
    from retrofire_gb300 import serve
    reqs = scenes.serving_requests(10, 1000.0, seed=12)
    try:
        serve.run_load(_FakeServer(fail_at=4), _FakeMeshSet(), reqs, realtime=False)
    except rf.RfError as e:
        assert e.code == 2
    else:
        raise AssertionError("the producer's error was not raised")
