"""Context::depth_sort on the GPU (render.rs:180-182, 209-219) against the
oracle: every render() call's clipped triangles ordered by their mean
clip-space z under f32::total_cmp, front to back or back to front, before
setup.  Both sides sort stably (triangles of equal depth keep their clipped
order, where the reference's sort_unstable_by leaves it unspecified), so
coverage, depth, colour and stats are compared bit for bit whatever the
ties.  The painter's-algorithm case (no depth test) makes the order
visible in every pixel."""
import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import scenes
from rfhelp import DrawSpec, assert_parity, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def both(draws, vp, w, h, ctx, **kw):
    return gpu_render(draws, vp, w, h, ctx=ctx, **kw), oracle_render(draws, vp, w, h, ctx=ctx)


@pytest.mark.parametrize("sort", [rf.SORT_FRONT_TO_BACK, rf.SORT_BACK_TO_FRONT])
@pytest.mark.parametrize("depth_test", [rf.DEPTH_NONE, rf.DEPTH_LESS])
def test_fill_scene_sorted(sort, depth_test):
    """3,000 fill-stress triangles, ~5% of them clipped into fans."""
    s = scenes.fill_stress(ntri=3000, w=640, h=360, seed=21)
    d = DrawSpec(s["verts"], s["faces"], rf.GOURAUD, pos_dim=4)
    ctx = rf.Context(depth_sort=sort, depth_test=depth_test)
    g, o = both([d], s["vp"], 640, 360, ctx)
    assert g[2].prims_o > 3000  # clipped fans take part in the sort
    assert_parity(g, o, what="sort %d depth %d" % (sort, depth_test))


def test_sorted_differs_from_unsorted():
    """Without a depth test the order shows: front-to-back, back-to-front
    and submission order give three different images."""
    s = scenes.fill_stress(ntri=1500, w=320, h=200, seed=22)
    d = DrawSpec(s["verts"], s["faces"], rf.GOURAUD, pos_dim=4)
    imgs = []
    for sort in (rf.SORT_NONE, rf.SORT_FRONT_TO_BACK, rf.SORT_BACK_TO_FRONT):
        ctx = rf.Context(depth_sort=sort, depth_test=rf.DEPTH_NONE)
        g, o = both([d], s["vp"], 320, 200, ctx)
        assert_parity(g, o, what="sort %d" % sort)
        imgs.append(g[0])
    assert not np.array_equal(imgs[0], imgs[1]) and not np.array_equal(imgs[1], imgs[2])


@pytest.mark.parametrize("tile", [(8, 4), (32, 8)])
def test_sorted_per_draw_and_textured(tile):
    """Several render() calls into one target: each call's triangles are
    sorted on their own (the calls stay in order); instanced textured
    cubes with a perspective camera, clipped by the near plane."""
    s = scenes.instanced_cubes(ninst=60, w=400, h=300, seed=23, tex_size=64)
    draws = [DrawSpec(s["verts"], s["faces"], rf.TEX_GOURAUD, m, tex=s["tex"]) for m in s["mvps"]]
    ctx = rf.Context(depth_sort=rf.SORT_BACK_TO_FRONT, depth_test=rf.DEPTH_NONE,
                     face_cull=rf.CULL_NONE)
    g, o = both(draws, s["vp"], 400, 300, ctx, tile=tile)
    assert_parity(g, o, what="tile %r" % (tile,))


def test_batch_mixes_sorted_and_unsorted_jobs():
    """One batch: a sorted scene next to an unsorted one; each equals the
    oracle and the same scene rendered alone."""
    dev = rf.Device()
    a = scenes.fill_stress(ntri=800, w=200, h=150, seed=24)
    b = scenes.fill_stress(ntri=900, w=180, h=120, seed=25)
    ctxs = [rf.Context(depth_sort=rf.SORT_FRONT_TO_BACK, depth_test=rf.DEPTH_NONE),
            rf.Context(depth_test=rf.DEPTH_NONE)]
    objs = []
    try:
        scs = []
        for sc, ctx in zip((a, b), ctxs):
            m = rf.Mesh(sc["verts"], sc["faces"], pos_dim=4, device=dev)
            tg = rf.Framebuf(sc["w"], sc["h"], device=dev)
            tg.clear()
            objs += [m, tg]
            scs.append(rf.Scene(tg, [(m, rf.Shader.gouraud(), None)], sc["vp"], ctx))
        st = rf.render_batch(scs, device=dev)
        for sc, ctx, scene, stats in zip((a, b), ctxs, scs, st):
            col, dep = scene.target.read()
            d = DrawSpec(sc["verts"], sc["faces"], rf.GOURAUD, pos_dim=4)
            assert_parity((col, dep, stats), oracle_render([d], sc["vp"], sc["w"], sc["h"], ctx=ctx))
    finally:
        for o in objs:
            o.close()
        dev.close()
