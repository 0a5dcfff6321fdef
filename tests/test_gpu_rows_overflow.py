"""The row-record buffer too small for a frame: the triangles whose records
do not fit are rasterised from their setup records instead -- the large
ones by the warp-per-triangle binning kernel, the small ones (at most 16
rows) handed over to it by the group kernels -- and the image and stats
stay those of the oracle.  The next frame on the same device has grown the
buffer and takes the regular path."""
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


def overflow_scene(seed=21, ntall=300, nsmall=2000, w=128, h=4096):
    """ntall full-height slivers first (about 4,096 rows of 9 words each,
    ~11 M words: more than the 4 M-word buffer a fresh context starts with
    for this triangle count), then nsmall triangles of 2 to 16 rows, whose
    records come after the slivers' and so find no room."""
    rng = np.random.default_rng(seed)
    verts, faces = [], []

    def tri(p):
        k = len(verts)
        for (x, y) in p:
            verts.append([x, y, rng.uniform(-0.9, 0.9), 1.0] + list(rng.uniform(0, 1, 3)))
        faces.append([k, k + 1, k + 2])

    for _ in range(ntall):
        x = rng.uniform(-0.95, 0.85)
        tri([(x, -1.2), (x + rng.uniform(0.05, 0.15), -1.2), (x + rng.uniform(0, 0.1), 1.2)])
    row = 2.0 / h
    for _ in range(nsmall):
        x, y = rng.uniform(-1, 0.9), rng.uniform(-1, 0.99)
        rows = rng.integers(2, 17)
        tri([(x, y), (x + rng.uniform(0.02, 0.1), y + 0.3 * rows * row), (x + 0.03, y + rows * row)])
    return np.array(verts, np.float32), np.array(faces, np.uint32), w, h


def test_rows_overflow_first_frame_then_grown():
    verts, faces, w, h = overflow_scene()
    d = DrawSpec(verts, faces, rf.GOURAUD, pos_dim=4)
    vp = mat.viewport(0, 0, w, h)
    ctx = rf.Context(face_cull=rf.CULL_NONE)
    o = oracle_render([d], vp, w, h, ctx=ctx)
    assert o[2]["frags_i"] > 0
    dev = rf.Device()  # a fresh context: its row buffer starts small
    try:
        for frame in range(2):
            g = gpu_render([d], vp, w, h, ctx=ctx, device=dev)
            assert_parity(g, o, what="frame %d" % frame)
    finally:
        dev.close()
