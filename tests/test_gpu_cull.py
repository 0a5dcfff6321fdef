"""Object-level frustum culling (RF_DRAW_CULL_BBOX): a flagged draw whose
bounding box is Hidden is a render() call that is never made (the
per-object loop of demos/src/bin/crates.rs:114-133); the result equals the
oracle rendering every other draw, and objs_i / objs_o count as that loop
does."""
import numpy as np
import pytest

import retrofire_gb300 as rf
from oracle import oracle as O
from retrofire_gb300 import scenes
from rfhelp import DrawSpec, assert_parity, oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def cull_case(seed, n=400, w=320, h=240):
    s = scenes.instanced_cubes(ninst=n, w=w, h=h, seed=seed, tex_size=64)
    flagged = [i % 5 != 0 for i in range(n)]
    status = [O.bbox_status(s["verts"], m) for m in s["mvps"]]
    drawn = [not (f and st == O.HIDDEN) for f, st in zip(flagged, status)]
    return s, flagged, drawn


def expected(s, drawn):
    specs = [DrawSpec(s["verts"], s["faces"], rf.TEX_GOURAUD, m, tex=s["tex"])
             for m, d in zip(s["mvps"], drawn) if d]
    return oracle_render(specs, s["vp"], s["w"], s["h"])


@pytest.mark.parametrize("seed", [9, 10])
def test_culled_draws_are_skipped(seed):
    s, flagged, drawn = cull_case(seed)
    assert sum(not d for d in drawn) > 20  # the case really culls
    dev = rf.Device()
    try:
        mesh = rf.Mesh(s["verts"], s["faces"], device=dev)
        tex = rf.Texture(s["tex"], device=dev)
        sh = rf.Shader.tex_gouraud(tex)
        tg = rf.Framebuf(s["w"], s["h"], device=dev)
        tg.clear()
        draws = [(mesh, sh, m, rf.DRAW_CULL_BBOX if f else 0) for m, f in zip(s["mvps"], flagged)]
        st = rf.render_draws(draws, s["vp"], tg)
        c, d = tg.read()
        assert_parity((c, d, st), expected(s, drawn))
        assert st.objs_i == sum(flagged)
        assert st.objs_o == sum(f and dr for f, dr in zip(flagged, drawn))
        for o in (mesh, tex, tg):
            o.close()
    finally:
        dev.close()


def test_culling_in_a_batch_and_a_graph():
    cases = [cull_case(seed, n=150, w=200, h=150) for seed in (11, 12)]
    dev = rf.Device()
    dev.set_graphs(True)
    try:
        objs, scs = [], []
        for s, flagged, _ in cases:
            mesh = rf.Mesh(s["verts"], s["faces"], device=dev)
            tex = rf.Texture(s["tex"], device=dev)
            tg = rf.Framebuf(s["w"], s["h"], device=dev)
            objs += [mesh, tex, tg]
            sh = rf.Shader.tex_gouraud(tex)
            draws = [(mesh, sh, m, rf.DRAW_CULL_BBOX if f else 0) for m, f in zip(s["mvps"], flagged)]
            scs.append(rf.Scene(tg, draws, s["vp"]))
        for _ in range(2):  # the second frame replays the graph
            for sc in scs:
                sc.target.clear()
            stats = rf.render_batch(scs, device=dev)
            for (s, flagged, drawn), sc, st in zip(cases, scs, stats):
                c, d = sc.target.read()
                assert_parity((c, d, st), expected(s, drawn))
                assert (st.objs_i, st.objs_o) == (sum(flagged),
                                                  sum(f and dr for f, dr in zip(flagged, drawn)))
        for o in objs:
            o.close()
    finally:
        dev.close()
