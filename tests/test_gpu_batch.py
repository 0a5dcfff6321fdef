"""Batched scenes, CUDA-graph replay and the tiling autotuner, against the
oracle and against rendering each scene alone.

A batch (rf_render_batch) is one pass of the pipeline over many targets;
its result for every scene must equal that scene rendered by itself
(rf_render_draws) and the oracle's render() loop over the scene's draws:
coverage, depth, colour and stats bit-exact.
"""
import numpy as np
import pytest

import retrofire_gb300 as rf
from retrofire_gb300 import mat, scenes
from rfhelp import DrawSpec, assert_parity, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


class SceneSpec:
    def __init__(self, draws, vp, w, h, ctx=None, pixfmt=rf.ARGB8888, depth=True, clear=True,
                 prefill=None):
        self.draws, self.vp, self.w, self.h = draws, vp, w, h
        self.ctx = ctx or rf.Context()
        self.pixfmt, self.depth, self.clear, self.prefill = pixfmt, depth, clear, prefill

    def oracle(self):
        return oracle_render(self.draws, self.vp, self.w, self.h, ctx=self.ctx,
                             pixfmt=self.pixfmt, depth=self.depth, clear=self.clear,
                             prefill=self.prefill)

    def alone(self, dev):
        return gpu_render(self.draws, self.vp, self.w, self.h, ctx=self.ctx, pixfmt=self.pixfmt,
                          depth=self.depth, clear=self.clear, prefill=self.prefill, device=dev)


def from_generated(sc):
    """A batch_scenes() entry as a SceneSpec (draws share one vertex array)."""
    if sc.get("kind", "cubes" if "mvps" in sc else "fill") == "fill":
        d = [DrawSpec(sc["verts"], sc["faces"], rf.GOURAUD, None, pos_dim=4)]
    else:
        d = [DrawSpec(sc["verts"], sc["faces"], rf.TEX_GOURAUD, m, tex=sc["tex"])
             for m in sc["mvps"]]
        faces = d[0].faces
        for x in d:  # one device mesh for all instances
            x.verts, x.faces = d[0].verts, faces
    return SceneSpec(d, sc["vp"], sc["w"], sc["h"])


class Batch:
    """Device-side objects of a batch of SceneSpecs on one rf_ctx."""

    def __init__(self, specs, dev):
        self.dev, self.specs = dev, specs
        self.meshes, self.texes, self.targets, self.scenes = {}, {}, [], []
        for sp in specs:
            tg = rf.Framebuf(sp.w, sp.h, sp.pixfmt, sp.depth, device=dev)
            self.targets.append(tg)
            items = []
            for d in sp.draws:
                key = (id(d.verts), id(d.faces), d.pos_dim)
                if key not in self.meshes:
                    self.meshes[key] = rf.Mesh(d.verts, d.faces, pos_dim=d.pos_dim, device=dev)
                tex = None
                if d.tex is not None:
                    if id(d.tex) not in self.texes:
                        self.texes[id(d.tex)] = rf.Texture(d.tex, device=dev)
                    tex = self.texes[id(d.tex)]
                items.append((self.meshes[key], rf.Shader(d.shader, d.flat_rgba, tex, d.sampler),
                              d.mvp))
            self.scenes.append(rf.Scene(tg, items, sp.vp, sp.ctx))
        self.reset()

    def reset(self):
        for sp, tg in zip(self.specs, self.targets):
            if sp.prefill is not None:
                tg.write(*sp.prefill)
            if sp.clear:
                tg.clear(sp.ctx.color_clear, sp.ctx.depth_clear)

    def render(self, sync_stats=True):
        return rf.render_batch(self.scenes, device=self.dev, sync_stats=sync_stats)

    def read(self):
        return [tg.read() for tg in self.targets]

    def close(self):
        for o in list(self.meshes.values()) + list(self.texes.values()) + self.targets:
            o.close()


def cube_spec(seed, w=640, h=480, **kw):
    c = scenes.textured_cube(seed=seed, w=w, h=h)
    return SceneSpec([DrawSpec(c["verts"], c["faces"], rf.TEXTURED, c["mvp"], tex=c["tex"])],
                     c["vp"], w, h, **kw)


def fill_spec(ntri, w, h, seed, **kw):
    s = scenes.fill_stress(ntri=ntri, w=w, h=h, seed=seed, amax=max(4.0, 1e4 * w * h / 2073600.0))
    return SceneSpec([DrawSpec(s["verts"], s["faces"], rf.GOURAUD, None, pos_dim=4)], s["vp"],
                     w, h, **kw)


def mixed_specs():
    rng = np.random.default_rng(11)
    flat = scenes.fill_stress(ntri=300, w=200, h=120, seed=5, amax=400.0)
    fverts = np.ascontiguousarray(flat["verts"][:, :4])
    pre_c = rng.integers(0, 1 << 32, size=(90, 130), dtype=np.uint64).astype(np.uint32)
    pre_d = rng.uniform(0.0, 1.0, size=(90, 130)).astype(np.float32)
    return [
        fill_spec(2000, 320, 240, 1),
        cube_spec(3),
        fill_spec(40, 64, 64, 2),
        SceneSpec([DrawSpec(fverts, flat["faces"], rf.FLAT, None, pos_dim=4,
                            flat_rgba=0xFF3366CC)], flat["vp"], 200, 120),
        cube_spec(4, 333, 211, ctx=rf.Context(depth_test=rf.DEPTH_GREATER, face_cull=rf.CULL_NONE),
                  clear=False, prefill=None),
        fill_spec(500, 130, 90, 3, ctx=rf.Context(color_write=False), clear=False,
                  prefill=(pre_c, pre_d)),
        fill_spec(800, 257, 129, 4, depth=False, pixfmt=rf.RGBA8888),
        cube_spec(5, 96, 1000, pixfmt=rf.BGRA8888),
        from_generated(scenes.instanced_cubes(ninst=60, w=300, h=200, seed=9, tex_size=64)),
    ]


def test_batch_equals_oracle_and_alone():
    specs = mixed_specs()
    dev = rf.Device()
    b = Batch(specs, dev)
    try:
        stats = b.render()
        outs = b.read()
        for i, (sp, (c, d), st) in enumerate(zip(specs, outs, stats)):
            assert_parity((c, d, st), sp.oracle(), what="scene %d vs oracle" % i)
            ac, ad, ast = sp.alone(dev)
            assert np.array_equal(c, ac), "scene %d colour differs from its lone render" % i
            if d is not None:
                assert np.array_equal(d.view(np.uint32), ad.view(np.uint32)), i
            assert st.as_dict() == ast.as_dict(), i
    finally:
        b.close()
        dev.close()


@pytest.mark.parametrize("seed", [21, 22])
def test_batch_uneven_recipe(seed):
    """The uneven-batch recipe (log-uniform sizes, fill or instanced cubes)."""
    specs = [from_generated(s) for s in
             scenes.batch_scenes(nscenes=24, seed=seed, max_tris=6000, wmax=700, hmax=500)]
    dev = rf.Device()
    b = Batch(specs, dev)
    try:
        stats = b.render()
        for i, (sp, (c, d), st) in enumerate(zip(specs, b.read(), stats)):
            assert_parity((c, d, st), sp.oracle(), what="scene %d" % i)
    finally:
        b.close()
        dev.close()


@pytest.mark.parametrize("tile", [(8, 4), (16, 8), (64, 4)])
def test_batch_tilings(tile):
    specs = mixed_specs()[:6]
    dev = rf.Device()
    dev.set_tiling(*tile)
    b = Batch(specs, dev)
    try:
        stats = b.render()
        for i, (sp, (c, d), st) in enumerate(zip(specs, b.read(), stats)):
            assert_parity((c, d, st), sp.oracle(), what="scene %d tile %r" % (i, tile))
    finally:
        b.close()
        dev.close()


def test_batch_stats_accumulate_without_sync():
    specs = mixed_specs()[:4]
    dev = rf.Device()
    b = Batch(specs, dev)
    try:
        assert b.render(sync_stats=False) is None
        tot = dev.take_stats().as_dict()
        exp = {}
        for sp in specs:
            for k, v in sp.oracle()[2].items():
                exp[k] = exp.get(k, 0) + v
        assert tot == dict(exp, objs_i=0, objs_o=0)
        assert dev.take_stats().as_dict() == {k: 0 for k in tot}
    finally:
        b.close()
        dev.close()


def test_batch_empty_scene_and_duplicates():
    dev = rf.Device()
    specs = [fill_spec(100, 64, 48, 7), SceneSpec([], mat.viewport(0, 0, 32, 16), 32, 16)]
    b = Batch(specs, dev)
    try:
        stats = b.render()
        assert stats[1].as_dict() == rf.Stats().as_dict()
        c, d = b.targets[1].read()  # the pending clear lands on the read
        assert (c == 0xFF000000).all() and (d == 0.0).all()
        assert_parity((*b.targets[0].read(), stats[0]), specs[0].oracle())
        dup = [b.scenes[0], rf.Scene(b.targets[0], [], specs[0].vp)]
        with pytest.raises(rf.RfError) as e:
            rf.render_batch(dup, device=dev)
        assert e.value.code == 2
    finally:
        b.close()
        dev.close()


def test_graph_replay_same_shape():
    """Frames of one shape replay one captured graph; every frame still
    equals the oracle (the per-frame matrices travel as data)."""
    dev = rf.Device()
    dev.set_graphs(True)
    dev.set_online_tuning(False)  # one tile width: one graph
    try:
        for seed in range(30, 36):
            g = cube_spec(seed).alone(dev)
            assert_parity(g, cube_spec(seed).oracle(), what="seed %d" % seed)
        cnt = dev.counts()
        assert cnt["graphs_cached"] == 1
        assert cnt["graph_launches"] == 6
        # per frame: nine render kernels and the mesh upload's two
        # bounding-box kernels
        assert cnt["kernels"] == 6 * (9 + 2)
    finally:
        dev.close()


def test_graph_replay_batches_and_growth():
    """Batches of one shape replay; a larger frame grows the scratch (the
    cached graphs are dropped) and the smaller shape is captured again."""
    dev = rf.Device()
    dev.set_graphs(True)
    try:
        for rnd in range(3):
            specs = [cube_spec(40 + rnd), fill_spec(700, 300, 200, 50 + rnd)]
            b = Batch(specs, dev)
            try:
                stats = b.render()
                for i, (sp, (c, d), st) in enumerate(zip(specs, b.read(), stats)):
                    assert_parity((c, d, st), sp.oracle(), what="round %d scene %d" % (rnd, i))
            finally:
                b.close()
            if rnd == 1:
                big = fill_spec(30000, 800, 600, 99)
                assert_parity(big.alone(dev), big.oracle(), what="big")
        assert dev.counts()["graph_launches"] == 4
    finally:
        dev.close()


def test_autotune_leaves_targets_unchanged():
    specs = mixed_specs()[:6]
    dev = rf.Device()
    b = Batch(specs, dev)
    try:
        tw, wp, ms = rf.autotune(b.scenes, reps=1, device=dev)
        assert tw in (8, 16, 32, 64) and wp in (4, 8) and ms > 0.0
        assert dev.take_stats().as_dict() == rf.Stats().as_dict()
        stats = b.render()  # the targets still hold their prefill / pending clear
        for i, (sp, (c, d), st) in enumerate(zip(specs, b.read(), stats)):
            assert_parity((c, d, st), sp.oracle(), what="scene %d after autotune" % i)
    finally:
        b.close()
        dev.close()


def test_online_tiling_trials_then_keeps_fastest():
    """Online tiling: a warm-up frame, one timed frame per tile width, then
    the fastest; every frame equals the oracle."""
    dev = rf.Device()
    sp = fill_spec(3000, 400, 300, 61)
    ref = sp.oracle()
    seen = []
    try:
        for _ in range(8):
            assert_parity(sp.alone(dev), ref, what="frame %d" % len(seen))
            seen.append(dev.last_tiling()[0])
        assert seen[:5] == [8, 8, 16, 32, 64]
        assert seen[5] in (8, 16, 32, 64) and seen[5] == seen[6] == seen[7]
        dev.set_tiling(16, 4)  # an explicit width ends the tuning
        assert_parity(sp.alone(dev), ref)
        assert dev.last_tiling() == (16, 4)
    finally:
        dev.close()
