"""The seeded synthetic workloads have the shapes, sizes and value
distributions of the benchmark recipes they stand in for: the fill-stress
frame (log-uniform screen areas 1..1e4 px^2, ~5 % crossing the near or far
plane, every triangle front-facing), the instanced cubes and the uneven
batch.  Host only."""
import numpy as np
import pytest

from retrofire_gb300 import scenes


@pytest.fixture(scope="module")
def fill():
    return scenes.fill_stress()


def _screen(s):
    v = s["verts"].reshape(-1, 3, 7).astype(np.float64)
    w = v[..., 3]
    ndc = v[..., :2] / w[..., None]
    sx = (ndc[..., 0] + 1.0) * s["w"] / 2.0
    sy = (ndc[..., 1] + 1.0) * s["h"] / 2.0
    return v, w, sx, sy


def test_fill_shapes_and_seed(fill):
    assert fill["verts"].shape == (300_000, 7) and fill["verts"].dtype == np.float32
    assert fill["faces"].shape == (100_000, 3)
    assert np.array_equal(fill["faces"].ravel(), np.arange(300_000))
    again = scenes.fill_stress()
    assert np.array_equal(again["verts"], fill["verts"])
    other = scenes.fill_stress(seed=3)
    assert not np.array_equal(other["verts"], fill["verts"])
    np.testing.assert_array_equal(fill["vp"][:2, 3], [960.0, 540.0])


def test_fill_area_distribution(fill):
    _, w, sx, sy = _screen(fill)
    assert (w > 0).all() and w.min() >= 0.8 and w.max() <= 4.8
    ux, uy = sx[:, 1] - sx[:, 0], sy[:, 1] - sy[:, 0]
    vx, vy = sx[:, 2] - sx[:, 0], sy[:, 2] - sy[:, 0]
    area = 0.5 * (ux * vy - uy * vx)
    assert area.min() > 0.99 and area.max() < 1.0001e4
    # log-uniform on [1, 1e4]: mean (1e4 - 1) / ln 1e4, median 100
    assert area.mean() == pytest.approx((1e4 - 1.0) / np.log(1e4), rel=0.03)
    assert np.mean(area < 100.0) == pytest.approx(0.5, abs=0.01)


def test_fill_front_facing(fill):
    """Tri::winding (geom/prim.rs:288-294): z = (-u.y) v.x + u.x v.y < 0 is
    clockwise, a back face under the default cull.  None is."""
    _, _, sx, sy = _screen(fill)
    ux, uy = sx[:, 1] - sx[:, 0], sy[:, 1] - sy[:, 0]
    vx, vy = sx[:, 2] - sx[:, 0], sy[:, 2] - sy[:, 0]
    assert ((-uy) * vx + ux * vy >= 0.0).all()


def test_fill_plane_crossings(fill):
    v, w, _, _ = _screen(fill)
    z = v[..., 2]
    crossing = (np.abs(z) > w).any(1)
    assert crossing.mean() == pytest.approx(0.05, abs=0.005)
    # one or two vertices beyond the plane, never all three
    k = (np.abs(z) > w).sum(1)
    assert set(np.unique(k[crossing])) == {1, 2}


def test_instanced_cubes_recipe():
    s = scenes.instanced_cubes(ninst=500)
    assert s["mvps"].shape == (500, 4, 4)
    assert s["verts"].shape == (24, 8)      # position, face colour, UV
    assert s["faces"].shape == (12, 3)
    assert s["tex"].shape == (1024, 1024) and (s["tex"] >> 24 == 0xFF).all()
    assert (s["verts"][:, 6:] >= 0).all() and (s["verts"][:, 6:] <= 1).all()


def test_batch_recipe():
    b = scenes.batch_scenes()
    assert len(b) == 256
    kinds = [s["kind"] for s in b]
    assert 0.35 < kinds.count("fill") / 256 < 0.65
    assert all(64 <= s["w"] <= 1920 and 64 <= s["h"] <= 1080 for s in b)
    tris = [len(s["faces"]) if s["kind"] == "fill" else 12 * len(s["mvps"]) for s in b]
    assert min(tris) >= 12 and max(tris) <= 200_000
    # log-uniform counts: about half the scenes below the geometric middle
    assert 0.35 < np.mean(np.array(tris) < np.sqrt(12 * 200_000)) < 0.65
    again = scenes.batch_scenes(nscenes=4)
    assert [s["w"] for s in again] == [s["w"] for s in b[:4]]


def test_first_person_camera():
    """FirstPerson (render/cam.rs:403-418) restated: the camera position maps
    to the view-space origin, the looked-at point onto the +z axis at its
    distance, world up stays up; Camera composes view then projection."""
    from retrofire_gb300 import mat
    for eye, tgt in (([0.0, 2.0, -110.0], [0.0, 0.0, 0.0]), ([3.0, 1.5, 2.0], [0.5, 0.0, -0.2])):
        fp = mat.FirstPerson(eye)
        fp.look_at(tgt)
        v = fp.world_to_view()
        o = mat.apply_point(v, eye)
        assert np.allclose(o[:3], 0.0, atol=1e-4)
        t = mat.apply_point(v, tgt)
        dist = np.linalg.norm(np.subtract(tgt, eye))
        assert np.allclose(t[:2], 0.0, atol=1e-4 * dist) and abs(t[2] - dist) < 1e-4 * dist
        up = v[:3, :3] @ np.array([0.0, 1.0, 0.0], np.float32)
        assert up[1] > 0.9
    cam = (mat.Camera((640, 480)).with_transform(fp).viewport((0, 640), (480, 0))
           .perspective(lambda a: mat.focal_ratio_horizontal(np.pi / 3.0), 0.1, 100.0))
    assert cam.dims == (640, 480)
    assert np.array_equal(cam.viewport_m, mat.viewport(0, 480, 640, 0))
    assert np.array_equal(cam.world_to_project(), mat.then(fp.world_to_view(), cam.project))
