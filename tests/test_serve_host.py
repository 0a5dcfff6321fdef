"""Host side of the serving workload (no GPU): the request stream's
arrival process and mix, the camera and mesh builders."""
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
