"""The rasteriser's work list: a tile far more crowded than a resident
warp's share of the frame is walked as four row slices by different warps,
and heavy tiles start first.  Results must equal the oracle bit for bit
whatever the split: a crowd of tiny triangles in one corner tile, over a
spread of larger ones, at every tile width."""
import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import mat
from rfhelp import DrawSpec, assert_parity, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def crowd_scene(seed, w=256, h=128, ncrowd=3000, nspread=300):
    """Clip-space Gouraud triangles: ncrowd of 1-4 px inside the
    pixel box [40, 70) x [20, 50), then nspread of 4-60 px anywhere; depths
    and colours random, submission order fixed by the seed."""
    rng = np.random.default_rng(seed)

    def tris(n, x0, x1, y0, y1, smin, smax):
        c = np.stack([rng.uniform(x0, x1, n), rng.uniform(y0, y1, n)], 1)
        off = rng.uniform(-1.0, 1.0, (n, 3, 2)) * rng.uniform(smin, smax, (n, 1, 1))
        return c[:, None, :] + off

    px = np.concatenate([tris(ncrowd, 40, 70, 20, 50, 1.0, 4.0), tris(nspread, 0, w, 0, h, 4.0, 60.0)])
    n = len(px)
    wv = rng.uniform(1.0, 4.0, (n, 3))  # screen depth 1/w varies per vertex
    clip = np.empty((n, 3, 4))
    clip[..., 0] = (px[..., 0] / (w / 2.0) - 1.0) * wv
    clip[..., 1] = (px[..., 1] / (h / 2.0) - 1.0) * wv
    clip[..., 2] = rng.uniform(-0.9, 0.9, (n, 3)) * wv
    clip[..., 3] = wv
    col = rng.uniform(0.0, 1.0, (n, 3, 3))
    verts = np.concatenate([clip, col], -1).reshape(-1, 7).astype(np.float32)
    faces = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    return [DrawSpec(verts, faces, rf.GOURAUD, pos_dim=4)], mat.viewport(0, 0, w, h), w, h


@pytest.mark.parametrize("tile", [(8, 4), (16, 4), (32, 4), (64, 2)])
@pytest.mark.parametrize("seed", [1, 2])
def test_crowded_tile_matches_oracle(tile, seed):
    draws, vp, w, h = crowd_scene(seed)
    g = gpu_render(draws, vp, w, h, tile=tile)
    o = oracle_render(draws, vp, w, h)
    assert o[2]["frags_i"] > 5000
    assert_parity(g, o, what="tile %r seed %d" % (tile, seed))


@pytest.mark.parametrize("cull", [rf.CULL_NONE, rf.CULL_FRONT])
def test_crowded_tile_other_contexts(cull):
    """The generic kernel (depth test Greater) and another cull mode over the
    same crowd."""
    draws, vp, w, h = crowd_scene(7)
    ctx = rf.Context(depth_clear=0.5, face_cull=cull, depth_test=rf.DEPTH_GREATER)
    g = gpu_render(draws, vp, w, h, ctx=ctx, tile=(8, 4))
    o = oracle_render(draws, vp, w, h, ctx=ctx)
    assert_parity(g, o, what="cull %d" % cull)
