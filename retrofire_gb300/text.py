"""Texture atlases and text meshes (host side), restating retrofire's
Atlas (core/src/render/tex.rs:141-185) and Text (core/src/render/text.rs).

A text is geometry: one quad (two triangles) per character, positioned on a
grid of glyph cells and textured from the atlas; it renders through the
ordinary textured path (text samples with SamplerClamp, text.rs: sample).
"""
import numpy as np

f32 = np.float32


class Atlas:
    """Atlas with Layout::Grid { sub_dims: (gw, gh) } over a texture
    (texels (h, w) u32, Color4 bytes r,g,b,a)."""

    def __init__(self, texels, glyph_w, glyph_h):
        self.texels = np.ascontiguousarray(texels, np.uint32)
        self.gw, self.gh = int(glyph_w), int(glyph_h)

    @property
    def width(self):
        return self.texels.shape[1]

    @property
    def height(self):
        return self.texels.shape[0]

    def rect(self, i):
        """Top-left and bottom-right pixel corners of sub-texture i
        (tex.rs:147-157)."""
        per_row = self.width // self.gw
        x0, y0 = i % per_row * self.gw, i // per_row * self.gh
        return (x0, y0), (x0 + self.gw, y0 + self.gh)

    def get(self, i):
        """The texels of sub-texture i (tex.rs:163-166)."""
        (x0, y0), (x1, y1) = self.rect(i)
        if x1 > self.width or y1 > self.height:
            raise IndexError("sub-texture %d is out of bounds" % i)
        return self.texels[y0:y1, x0:x1]

    def coords(self, i):
        """Texture coordinates of sub-texture i: top-left, top-right,
        bottom-left, bottom-right (tex.rs:175-184); f32 divisions by the
        texture's width and height (kept as f32 by Texture)."""
        tw, th = f32(self.width), f32(self.height)
        (x0, y0), (x1, y1) = self.rect(i)
        u0, v0 = f32(x0) / tw, f32(y0) / th
        u1, v1 = f32(x1) / tw, f32(y1) / th
        return [(u0, v0), (u1, v0), (u0, v1), (u1, v1)]


class Text:
    """Text (text.rs): write characters, get a Mesh<TexCoord> (verts
    (n, 5): x, y, z, u, v; faces (m, 3))."""

    def __init__(self, font):
        self.font = font
        self.clear()

    def clear(self):
        self.cursor = (f32(0.0), f32(0.0))
        self._verts, self._faces = [], []

    def _write_char(self, idx):
        gw, gh = f32(self.font.gw), f32(self.font.gh)
        tl, tr, bl, br = self.font.coords(idx)
        x, y = self.cursor
        l = len(self._verts)
        self._verts += [(x, y, f32(0), *tl), (f32(x + gw), y, f32(0), *tr),
                        (x, f32(y + gh), f32(0), *bl), (f32(x + gw), f32(y + gh), f32(0), *br)]
        self._faces += [(l, l + 1, l + 3), (l, l + 3, l + 2)]
        self.cursor = (f32(x + gw), y)

    def write(self, data):
        """io::Write (bytes) or fmt::Write (str): one glyph per byte / char;
        a newline moves the cursor to the start of the next row."""
        seq = data if isinstance(data, (bytes, bytearray)) else [ord(c) for c in data]
        gh = f32(self.font.gh)
        for b in seq:
            if b == 0x0A:
                self.cursor = (f32(0.0), f32(self.cursor[1] + gh))
            else:
                self._write_char(int(b))
        return len(data)

    def mesh(self):
        v = np.array(self._verts, np.float32).reshape(-1, 5)
        f = np.array(self._faces, np.uint32).reshape(-1, 3)
        return v, f


def bake(s, font):
    """text.rs bake: the glyphs of s (bytes; rows split at newlines) copied
    into one buffer of num_cols * gw by num_rows * gh texels."""
    rows = bytes(s).split(b"\n")
    num_rows, num_cols = len(rows), max(len(r) for r in rows)
    if num_rows == 0 or num_cols == 0:
        return np.zeros((0, 0), np.uint32)
    buf = np.zeros((num_rows * font.gh, num_cols * font.gw), np.uint32)
    for r, row in enumerate(rows):
        for c, ch in enumerate(row):
            buf[r * font.gh:(r + 1) * font.gh, c * font.gw:(c + 1) * font.gw] = font.get(ch)
    return buf
