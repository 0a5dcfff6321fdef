"""Mesh ingestion: the library's OBJ reader (rf_obj_parse, host code)
against the behaviour of retrofire's reader (geom/src/io.rs) and a Python
restatement of it; one GPU test renders a loaded OBJ against the oracle."""
import numpy as np
import pytest

import retrofire_gb300 as rf


@pytest.fixture(scope="module", autouse=True)
def built():
    from retrofire_gb300 import build
    build.build()


def test_triangles_comments_and_skipped_items():
    v, f = rf.parse_obj("# a comment\n\ng group\ns 1\nmtllib x.mtl\nusemtl m\n"
                        "v 0 0 0\nv 1 0 0\r\nv\t0 1 0 1.0\n\n f 1 2 3 \n")
    assert v.shape == (3, 3) and f.tolist() == [[0, 1, 2]]
    assert v.tolist() == [[0, 0, 0], [1, 0, 0], [0, 1, 0]]


def test_quad_split_and_first_use_order():
    v, f = rf.parse_obj("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 4 3 2 1\nf 1 2 4\n")
    # quad [a,b,c,d] -> [a,b,c], [a,c,d]; vertices numbered as first used
    assert f.tolist() == [[0, 1, 2], [0, 2, 3], [3, 2, 0]]
    assert v.tolist() == [[0, 1, 0], [1, 1, 0], [1, 0, 0], [0, 0, 0]]


def test_vertices_are_index_triples():
    src = ("v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nvn 0 0 -1\nvt 0 0\nvt 1 1\n"
           "f 1/1/1 2/1/1 3/2/1\nf 1/1/2 3/2/1 2/1/1\n")
    v, f = rf.parse_obj(src, rf.OBJ_NORMAL_TEXCOORD)
    assert v.shape == (4, 8)  # 1/1/2 is a new vertex, the rest repeat
    assert f.tolist() == [[0, 1, 2], [3, 2, 1]]
    assert v[0].tolist() == [0, 0, 0, 0, 0, 1, 0, 0]
    assert v[3].tolist() == [0, 0, 0, 0, 0, -1, 0, 0]
    vp, fp = rf.parse_obj(src)  # positions only: still keyed by the triple
    assert vp.shape == (4, 3) and fp.tolist() == f.tolist()
    vn, _ = rf.parse_obj(src, rf.OBJ_NORMAL)
    vt, _ = rf.parse_obj(src, rf.OBJ_TEXCOORD)
    assert vn.shape == (4, 6) and vt.shape == (4, 5)
    assert vt[2].tolist() == [0, 1, 0, 1, 1]


def test_position_normal_without_texcoord():
    v, f = rf.parse_obj("v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n", rf.OBJ_NORMAL)
    assert v.shape == (3, 6) and (v[:, 3:] == [0, 0, 1]).all()


def test_float_formats():
    v, _ = rf.parse_obj("v 1e3 -0.5 .25\nv 5. +2 -0\nv 1.5E-2 3 4\nf 1 2 3\n")
    assert v[0].tolist() == [1000.0, -0.5, 0.25]
    assert v[1].tolist() == [5.0, 2.0, 0.0] and np.signbit(v[1, 2])
    assert v[2, 0] == np.float32(0.015)


def test_float_words_and_range():
    """Rust's f32::from_str: inf / infinity / nan in any case, with a sign;
    out-of-range decimals round to +-inf or +-0."""
    v, _ = rf.parse_obj("v inf -Infinity NaN\nv 1e50 -1e-50 +.5\nv 3.4028235e38 1e-45 7\nf 1 2 3\n")
    assert np.isposinf(v[0, 0]) and np.isneginf(v[0, 1]) and np.isnan(v[0, 2])
    assert np.isposinf(v[1, 0]) and v[1, 1] == 0.0 and np.signbit(v[1, 1]) and v[1, 2] == 0.5
    assert v[2, 0] == np.finfo(np.float32).max and v[2, 1] == np.float32(1e-45)


@pytest.mark.parametrize("tok", ["0x1p3", "0X10", ".", "e5", "1e", "1.5e+", "--1", "1..2", "1e5.5",
                                 "nan(1)", "infinit", "1_000", "1f", ",5"])
def test_float_syntax_rejected(tok):
    """Forms Rust's f32 parser rejects (hexadecimal, C's nan payloads, a
    missing mantissa or exponent) are invalid numeric values here too."""
    with pytest.raises(rf.ObjError) as e:
        rf.parse_obj("v %s 0 0\n" % tok)
    assert "invalid numeric" in str(e.value)


@pytest.mark.parametrize("src", ["", "   \n\t\n", "# only\n# comments\n"])
def test_empty_inputs(src):
    v, f = rf.parse_obj(src)
    assert v.shape == (0, 3) and f.shape == (0, 3)


@pytest.mark.parametrize("src,attrs,msg", [
    ("xyz 1 2 3\n", rf.OBJ_POSITION, "unsupported item"),
    ("f\n", rf.OBJ_POSITION, "unexpected end"),
    ("v 1 2\n", rf.OBJ_POSITION, "unexpected end"),
    ("v 1 a 3\n", rf.OBJ_POSITION, "invalid numeric"),
    ("v 0 0 0\nv 1 0 0\nf 1 2 3\n", rf.OBJ_POSITION, "vertex index out of bounds"),
    ("v 0 0 0\nf 0 1 1\n", rf.OBJ_POSITION, "index 0"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nf 1/1 2/2 3/1\n", rf.OBJ_TEXCOORD, "texcoord index out"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//2 3//1\n", rf.OBJ_NORMAL, "normal index out"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", rf.OBJ_TEXCOORD, "missing vertex attribute"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\nf 1 2 3\n", rf.OBJ_POSITION,
     "not all faces have normals"),
])
def test_errors(src, attrs, msg):
    with pytest.raises(rf.ObjError) as e:
        rf.parse_obj(src, attrs)
    assert msg in str(e.value)


def restated(src, attrs):
    """Python restatement of the reader for well-formed input."""
    coords, norms, texcs, faces = [], [], [], []
    for line in src.split("\n"):
        t = line.split()
        if not t or t[0].startswith("#") or t[0] in ("g", "s", "mtllib", "usemtl"):
            continue
        if t[0] == "v":
            coords.append([np.float32(x) for x in t[1:4]])
        elif t[0] == "vn":
            norms.append([np.float32(x) for x in t[1:4]])
        elif t[0] == "vt":
            texcs.append([np.float32(x) for x in t[1:3]])
        elif t[0] == "f":
            idx = []
            for g in t[1:5]:
                p = g.split("/")
                idx.append((int(p[0]) - 1, int(p[1]) - 1 if len(p) > 1 and p[1] else None,
                            int(p[2]) - 1 if len(p) > 2 else None))
            faces.append(idx[:3])
            if len(idx) == 4:
                faces.append([idx[0], idx[2], idx[3]])
    seen, verts, out = {}, [], []
    for tri in faces:
        row = []
        for key in tri:
            if key not in seen:
                seen[key] = len(verts)
                a = list(coords[key[0]])
                if attrs in (rf.OBJ_NORMAL, rf.OBJ_NORMAL_TEXCOORD):
                    a += norms[key[2]]
                if attrs in (rf.OBJ_TEXCOORD, rf.OBJ_NORMAL_TEXCOORD):
                    a += texcs[key[1]]
                verts.append(a)
            row.append(seen[key])
        out.append(row)
    return np.array(verts, np.float32), np.array(out, np.uint32)


def random_obj(seed, n=40):
    """A random well-formed OBJ (values exact in f32), triangles and quads."""
    rng = np.random.default_rng(seed)
    lines = ["# generated"]
    q = lambda a: " ".join("%.10g" % x for x in a)
    for _ in range(n):
        lines.append("v " + q(rng.integers(-4096, 4096, 3) / 1024.0))
    for _ in range(n // 2):
        lines.append("vn " + q(rng.integers(-1024, 1024, 3) / 1024.0))
        lines.append("vt " + q(rng.integers(0, 1024, 2) / 1024.0))
    for _ in range(3 * n):
        k = 4 if rng.random() < 0.3 else 3
        g = ["%d/%d/%d" % (rng.integers(1, n + 1), rng.integers(1, n // 2 + 1),
                           rng.integers(1, n // 2 + 1)) for _ in range(k)]
        lines.append("f " + " ".join(g))
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("attrs", [rf.OBJ_POSITION, rf.OBJ_NORMAL, rf.OBJ_TEXCOORD,
                                   rf.OBJ_NORMAL_TEXCOORD])
def test_matches_restatement(seed, attrs):
    src = random_obj(seed)
    v, f = rf.parse_obj(src, attrs)
    rv, rfc = restated(src, attrs)
    assert np.array_equal(f, rfc)
    assert np.array_equal(v.view(np.uint32), rv.view(np.uint32))


@pytest.mark.gpu
def test_loaded_obj_renders_like_the_oracle():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from oracle import oracle as O
    from retrofire_gb300 import mat, scenes
    # a closed grid surface written out as OBJ text with per-vertex normals
    gv, gf = scenes.grid_mesh(24, 3)
    lines = ["v %.9g %.9g %.9g" % tuple(p) for p in gv[:, :3]]
    lines += ["vn %.9g %.9g %.9g" % tuple(c) for c in gv[:, 3:6]]
    lines += ["f %d//%d %d//%d %d//%d" % (a + 1, a + 1, b + 1, b + 1, c + 1, c + 1) for a, b, c in gf]
    src = "\n".join(lines) + "\n"
    verts, faces = rf.parse_obj(src, rf.OBJ_NORMAL)
    dev = rf.Device()
    try:
        h = rf.C.c_uint64()
        data = src.encode()
        assert rf.lib().rf_mesh_load_obj(dev.ptr, data, len(data), rf.OBJ_NORMAL, rf.C.byref(h)) == 0
        mesh = rf.Mesh.__new__(rf.Mesh)
        mesh.dev, mesh.handle = dev, h.value
        tg = rf.Framebuf(320, 240, device=dev)
        tg.clear()
        mvp = scenes.orbit_camera(5, 320, 240)
        vp = mat.viewport(0, 240, 320, 0)
        st = rf.render_draws([(mesh, rf.Shader.gouraud(), mvp)], vp, tg)
        c, d = tg.read()
        col = np.zeros((240, 320), np.uint32)
        dep = np.zeros((240, 320), np.float32)
        O.clear(col, dep)
        ost = O.render([O.make_draw(verts, faces, rf.GOURAUD, mvp, pos_dim=3)], vp, col, dep, {})
        assert np.array_equal(c, col) and np.array_equal(d.view(np.uint32), dep.view(np.uint32))
        assert st.as_dict() == dict(ost.as_dict(), objs_i=0, objs_o=0) and st.frags_i > 0
        mesh.close()
        tg.close()
    finally:
        dev.close()
