"""Object-level culling on the host side: the oracle's restatement of
BBox::of + BBox::visibility (render/scene.rs) on simple known cases."""
import numpy as np

from oracle import oracle as O
from retrofire_gb300 import mat, scenes


def cam(z):
    """Unit cube translated to z, camera at the origin looking along +z."""
    proj = mat.perspective(mat.focal_ratio_horizontal(np.pi / 2), 1.0, 0.1, 100.0)
    return mat.then(mat.translate3(0.0, 0.0, z), proj)


def test_box_status_cases():
    v, _ = scenes.cube_mesh(1.0)
    assert O.bbox_status(v, cam(5.0)) == O.VISIBLE
    assert O.bbox_status(v, cam(-5.0)) == O.HIDDEN      # behind the camera
    assert O.bbox_status(v, cam(0.0)) == O.CLIPPED      # around the eye: crosses near
    assert O.bbox_status(v, cam(200.0)) == O.HIDDEN     # beyond far


def test_box_is_the_position_extent():
    v, _ = scenes.cube_mesh(1.0)
    far = np.array(v)
    far[0, :3] = [0.0, 0.0, -1000.0]  # one vertex far behind: the box now crosses
    assert O.bbox_status(far, cam(5.0)) == O.CLIPPED
    nan = np.array(v)
    nan[1, 0] = np.nan  # f32::min / max ignore NaN
    assert O.bbox_status(nan, cam(5.0)) == O.VISIBLE
