"""Parity at the measured workloads' full sizes: the CUDA path against the
oracle on the exact inputs the benchmark renders (coverage, depth, colour
and stats bit-exact).

  fill stress   1920x1080, 100,000 Gouraud triangles (the headline frame)
  cubes         1920x1080, 10,000 instanced tex x Gouraud cubes, one draw each
  batch         the 256 uneven scenes, rendered as one batch
  serving       a sample of the request stream (meshes up to 500 k triangles)
"""
import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import scenes, serve, workloads
from rfhelp import DrawSpec, assert_parity, oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def specs_of(sc):
    return [DrawSpec(d["verts"], d["faces"], d["shader"], d["mvp"], pos_dim=d["pos_dim"],
                     tex=d["tex"]) for d in sc["draws"]]


def render_and_compare(name, frames=1):
    """Renders a workload's scenes with the library (as the benchmark does,
    online tiling included) `frames` times and compares the last frame of
    every scene with the oracle."""
    scs = workloads.scenes_for(name)
    dev = rf.Device()
    objs = workloads.upload(scs, dev)
    try:
        for _ in range(frames):
            for tg in objs["targets"]:
                tg.clear()
            stats = rf.render_batch(objs["scenes"], device=dev)
        for i, (sc, tg, st) in enumerate(zip(scs, objs["targets"], stats)):
            c, d = tg.read()
            assert_parity((c, d, st), oracle_render(specs_of(sc), sc["vp"], sc["w"], sc["h"]),
                          what="%s scene %d" % (name, i))
    finally:
        workloads.close(objs)
        dev.close()


def test_fill_stress_full_frame():
    s = scenes.fill_stress()
    d = DrawSpec(s["verts"], s["faces"], rf.GOURAUD, None, pos_dim=4)
    dev = rf.Device()
    try:
        tg = rf.Framebuf(1920, 1080, device=dev)
        mesh = rf.Mesh(s["verts"], s["faces"], pos_dim=4, device=dev)
        ref = oracle_render([d], s["vp"], 1920, 1080)
        # the first frames run the online tiling trials: every width must agree
        for frame in range(6):
            tg.clear()
            st = rf.render_draws([(mesh, rf.Shader.gouraud(), None)], s["vp"], tg)
            c, dep = tg.read()
            assert_parity((c, dep, st), ref, what="frame %d (tile %d)" % (frame, dev.last_tiling()[0]))
        mesh.close()
        tg.close()
    finally:
        dev.close()


def test_instanced_cubes_full_frame():
    render_and_compare("cubes")


def test_uneven_batch_full():
    render_and_compare("batch", frames=2)


def test_serving_sample_full_meshes():
    """60 requests of the stream (every preloaded mesh, 500 k triangles
    included) served in batches; each equals the oracle's render."""
    dev = rf.Device()
    ms = serve.MeshSet(dev)
    reqs = scenes.serving_requests(60, 2000.0, seed=2100)
    srv = rf.Server(dev)
    try:
        res, _ = serve.run_load(srv, ms, reqs, realtime=False)
        for i, (r, (c, d, out)) in enumerate(zip(reqs, res)):
            assert out["status"] == 0
            _, _, sh, v, f = ms.entries[r["mesh"]]
            spec = DrawSpec(v, f, sh.kind, r["mvp"], tex=ms.texels if sh.texture is not None else None)
            assert_parity((c, d, out["stats"]), oracle_render([spec], r["vp"], r["w"], r["h"]),
                          what="request %d (mesh %s)" % (i, ms.entries[r["mesh"]][0]))
    finally:
        srv.close()
        ms.close()
        dev.close()
