"""Texture atlases and text meshes (tex.rs Atlas, text.rs Text / bake):
known answers from the reference's definitions."""
import numpy as np
import pytest

from retrofire_gb300 import text
from retrofire_gb300.scenes import noise_texture

f32 = np.float32


def atlas():
    return text.Atlas(noise_texture(128, 3)[:64], 8, 8)  # 16 x 8 glyphs of 8x8


def test_rect_and_coords():
    a = atlas()
    assert a.rect(0) == ((0, 0), (8, 8))
    assert a.rect(17) == ((8, 8), (16, 16))
    tl, tr, bl, br = a.coords(17)
    assert tl == (f32(8) / f32(128), f32(8) / f32(64)) and br == (f32(16) / f32(128), f32(16) / f32(64))
    assert tr == (br[0], tl[1]) and bl == (tl[0], br[1])
    assert a.coords(200)[3][1] > 1.0  # no bounds check, like the reference
    with pytest.raises(IndexError):
        a.get(200)


def test_text_geometry():
    t = text.Text(atlas())
    t.write("ab\nc")
    v, f = t.mesh()
    assert v.shape == (12, 5) and f.tolist() == [[0, 1, 3], [0, 3, 2], [4, 5, 7], [4, 7, 6],
                                                 [8, 9, 11], [8, 11, 10]]
    assert v[0, :3].tolist() == [0, 0, 0] and v[4, :3].tolist() == [8, 0, 0]
    assert v[8, :3].tolist() == [0, 8, 0] and v[11, :3].tolist() == [8, 16, 0]
    assert tuple(v[0, 3:]) == atlas().coords(ord("a"))[0]
    t.clear()
    t.write(b"x")
    assert t.mesh()[0].shape == (4, 5) and t.cursor == (8.0, 0.0)


def test_bake():
    a = atlas()
    b = text.bake(b"hi\nyou", a)
    assert b.shape == (16, 24)
    assert np.array_equal(b[0:8, 8:16], a.get(ord("i")))
    assert np.array_equal(b[8:16, 16:24], a.get(ord("u")))
    assert (b[0:8, 16:24] == 0).all()  # short row: default texels
    assert text.bake(b"", a).shape == (0, 0)
