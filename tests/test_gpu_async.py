"""Streaming copies (rf_mesh_update_async, rf_target_read_async): frames
pipelined over two meshes and two targets give, frame by frame, what the
oracle renders; an upload queued right after a render does not change that
render, and a read queued before the next render into a target returns the
earlier frame."""
import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import scenes
from rfhelp import DrawSpec, assert_parity, oracle_render

pytestmark = pytest.mark.gpu

W, H, N = 320, 240, 3000


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def pinned(a):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    return t, t.numpy()


def frame_scene(seed):
    return scenes.fill_stress(ntri=N, w=W, h=H, seed=seed, amax=400.0)


def oracle_of(s):
    return oracle_render([DrawSpec(s["verts"], s["faces"], rf.GOURAUD, None, pos_dim=4)],
                         s["vp"], W, H)


def test_pipelined_frames_match_the_oracle():
    import torch
    frames = [frame_scene(100 + i) for i in range(6)]
    ins = [pinned(f["verts"]) for f in frames]
    outs = [(pinned(np.zeros((H, W), np.uint32)), pinned(np.zeros((H, W), np.float32)))
            for _ in frames]
    dev = rf.Device()
    try:
        faces = frames[0]["faces"]
        meshes = [rf.Mesh(frames[0]["verts"], faces, pos_dim=4, device=dev) for _ in range(2)]
        tgs = [rf.Framebuf(W, H, device=dev) for _ in range(2)]
        sh = rf.Shader.gouraud()
        stats = []
        meshes[0].update_async(ins[0][1])
        for i, f in enumerate(frames):
            k = i % 2
            tgs[k].clear()
            stats.append(rf.render_draws([(meshes[k], sh, None)], f["vp"], tgs[k], sync_stats=False))
            if i + 1 < len(frames):
                meshes[1 - k].update_async(ins[i + 1][1])  # next frame's input overlaps
            tgs[k].read_async(outs[i][0][1], outs[i][1][1])
        dev.sync()
        for i, f in enumerate(frames):
            c, d = outs[i][0][1], outs[i][1][1]
            oc, od, _ = oracle_of(f)
            assert np.array_equal(c, oc), "frame %d colour" % i
            assert np.array_equal(d.view(np.uint32), od.view(np.uint32)), "frame %d depth" % i
        tot = dev.take_stats()
        assert tot.frags_i == sum(oracle_of(f)[2]["frags_i"] for f in frames)
        for o in meshes + tgs:
            o.close()
    finally:
        dev.close()


def test_upload_waits_for_the_render_that_reads_the_mesh():
    a, b = frame_scene(7), frame_scene(8)
    pa, pb = pinned(a["verts"]), pinned(b["verts"])
    oc = pinned(np.zeros((H, W), np.uint32))
    od = pinned(np.zeros((H, W), np.float32))
    dev = rf.Device()
    try:
        mesh = rf.Mesh(a["verts"], a["faces"], pos_dim=4, device=dev)
        tg = rf.Framebuf(W, H, device=dev)
        tg.clear()
        st = rf.render_draws([(mesh, rf.Shader.gouraud(), None)], a["vp"], tg, sync_stats=False)
        mesh.update_async(pb[1])          # must not reach the render queued before it
        tg.read_async(oc[1], od[1])
        dev.sync()
        assert_parity((oc[1].copy(), od[1].copy(), dev.take_stats()), oracle_of(a))
        tg.clear()                         # the next render sees the new content
        st = rf.render_draws([(mesh, rf.Shader.gouraud(), None)], b["vp"], tg)
        c, d = tg.read()
        assert_parity((c, d, st), oracle_of(b))
        del pa
        mesh.close()
        tg.close()
    finally:
        dev.close()


def test_read_waits_before_the_next_render_into_the_target():
    a, b = frame_scene(9), frame_scene(10)
    oc = pinned(np.zeros((H, W), np.uint32))
    od = pinned(np.zeros((H, W), np.float32))
    dev = rf.Device()
    try:
        ma = rf.Mesh(a["verts"], a["faces"], pos_dim=4, device=dev)
        mb = rf.Mesh(b["verts"], b["faces"], pos_dim=4, device=dev)
        tg = rf.Framebuf(W, H, device=dev)
        tg.clear()
        rf.render_draws([(ma, rf.Shader.gouraud(), None)], a["vp"], tg, sync_stats=False)
        tg.read_async(oc[1], od[1])       # frame a
        tg.clear()
        rf.render_draws([(mb, rf.Shader.gouraud(), None)], b["vp"], tg, sync_stats=False)
        dev.sync()
        ac, ad, _ = oracle_of(a)
        assert np.array_equal(oc[1], ac) and np.array_equal(od[1].view(np.uint32), ad.view(np.uint32))
        c, d = tg.read()
        bc, bd, _ = oracle_of(b)
        assert np.array_equal(c, bc) and np.array_equal(d.view(np.uint32), bd.view(np.uint32))
        for o in (ma, mb, tg):
            o.close()
    finally:
        dev.close()
