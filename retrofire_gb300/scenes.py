"""Seeded synthetic scenes with the shapes of the benchmark workloads.

  textured_cube    640x480, one textured cube (24 verts / 12 tris), 64x64
                   checker, seed-drawn Euler angles, camera 4 units away.
  fill_stress      1920x1080, N independent Gouraud triangles given in clip
                   space, screen area log-uniform in [1, 1e4] px^2, ~5% with
                   one or two vertices beyond the near or far plane.
  instanced_cubes  1920x1080, N textured x Gouraud cubes on a 200x200 floor,
                   first-person camera, one 1024x1024 noise texture; one draw
                   (render() call) per instance.

Everything is generated on the host with numpy from an explicit seed; the
reference's own Xorshift64 drives the cube angles (rand.rs:118-183).
"""
import numpy as np

from . import mat
from .rand import Xorshift64

f32 = np.float32
TWO_PI = f32(2.0 * np.pi)

# geom/src/solids/platonic.rs:131-183 Box tables.
_BOX_COORDS = np.array([[0, 0, 0], [0, 0, 1], [0, 1, 0], [0, 1, 1],
                        [1, 0, 0], [1, 0, 1], [1, 1, 0], [1, 1, 1]], f32)
_BOX_NORMS = np.array([[-1, 0, 0], [1, 0, 0], [0, -1, 0], [0, 1, 0], [0, 0, -1], [0, 0, 1]], f32)
_BOX_UVS = np.array([[0, 0], [1, 0], [0, 1], [1, 1]], f32)
_BOX_VERTS = [(0b011, 0, 0), (0b010, 0, 1), (0b001, 0, 2), (0b000, 0, 3),
              (0b110, 1, 0), (0b111, 1, 1), (0b100, 1, 2), (0b101, 1, 3),
              (0b000, 2, 0), (0b100, 2, 1), (0b001, 2, 2), (0b101, 2, 3),
              (0b011, 3, 0), (0b111, 3, 1), (0b010, 3, 2), (0b110, 3, 3),
              (0b010, 4, 0), (0b110, 4, 1), (0b000, 4, 2), (0b100, 4, 3),
              (0b111, 5, 0), (0b011, 5, 1), (0b101, 5, 2), (0b001, 5, 3)]
BOX_FACES = np.array([[0, 1, 3], [0, 3, 2], [4, 5, 7], [4, 7, 6], [8, 9, 11], [8, 11, 10],
                      [12, 13, 15], [12, 15, 14], [16, 17, 19], [16, 19, 18],
                      [20, 21, 23], [20, 23, 22]], np.uint32)


def cube_mesh(side_len, attrs="uv"):
    """Cube{side_len}.build() as Box(-s/2..s/2) (platonic.rs:191-241).

    attrs: "uv" -> (pos, TexCoord); "none" -> pos only; "col_uv" ->
    (Color3f from the face normal, TexCoord) in the solids.rs:70-79 idiom."""
    dim = f32(side_len) / f32(2.0)
    lo, hi = -dim, dim
    rows = []
    for pos_i, norm_i, uv_i in _BOX_VERTS:
        c = _BOX_COORDS[pos_i]
        p = [f32(lo + f32(f32(hi - lo) * c[k])) for k in range(3)]  # lerp
        n = _BOX_NORMS[norm_i]
        uv = list(_BOX_UVS[uv_i])
        if attrs == "uv":
            rows.append(p + uv)
        elif attrs == "col_uv":
            diffuse = f32(max(f32(n[2] + f32(0.2)), f32(0.2)) * f32(0.8))
            col = [f32(diffuse * f32(f32(0.45) * f32(n[k] + f32(1.1)))) for k in range(3)]
            rows.append(p + col + uv)
        else:
            rows.append(p)
    return np.array(rows, f32), BOX_FACES.copy()


def checker_texture(n=64, cell=8):
    """n x n RGBA8 checker, white/black cells of `cell` px, alpha 255."""
    y, x = np.mgrid[0:n, 0:n]
    on = ((x // cell) ^ (y // cell)) & 1
    return np.where(on == 1, np.uint32(0xFFFFFFFF), np.uint32(0xFF000000)).astype(np.uint32)


def noise_texture(n=1024, seed=7):
    rng = np.random.default_rng(seed)
    return (rng.integers(0, 1 << 24, size=(n, n), dtype=np.uint32) | np.uint32(0xFF000000))


def textured_cube(seed=1, w=640, h=480):
    """The plain single-frame case: returns dict(verts, faces, tex, mvp, vp)."""
    g = Xorshift64(seed)
    a, b, c = (g.uniform(0.0, TWO_PI) for _ in range(3))
    m = mat.then(mat.then(mat.rotate_x(a), mat.rotate_y(b)), mat.rotate_z(c))
    m = mat.then(m, mat.translate3(0.0, 0.0, 4.0))
    proj = mat.perspective(mat.focal_ratio_horizontal(np.pi / 3.0), f32(w) / f32(h), 0.1, 100.0)
    mvp = mat.then(m, proj)
    verts, faces = cube_mesh(2.0, "uv")
    return dict(verts=verts, faces=faces, tex=checker_texture(), mvp=mvp,
                vp=mat.viewport(0, 0, w, h), w=w, h=h)


def fill_stress(ntri=100_000, w=1920, h=1080, seed=2, cross_frac=0.05, amin=1.0, amax=1e4):
    """Clip-space Gouraud triangles (pos_dim 4 + rgb).  Returns dict(verts,
    faces, vp, w, h); verts are (3*ntri, 7) float32, faces (ntri, 3)."""
    rng = np.random.default_rng(seed)
    n = ntri
    centre = rng.uniform(-1.0, 1.0, size=(n, 2))
    wt = rng.uniform(1.0, 4.0, size=n)
    area = np.exp(rng.uniform(0.0, np.log(amax / amin), size=n)) * amin
    # Random CCW shape: three points on the unit circle at increasing angles
    # (Dirichlet gaps, so slivers are rare), then a random rotation and an
    # anisotropic stretch (determinant > 0 keeps the winding), then scaled
    # to the drawn area.
    th0 = rng.uniform(0.0, 2 * np.pi, size=n)
    gaps = rng.dirichlet([2.0, 2.0, 2.0], size=n) * 2 * np.pi
    th = np.stack([th0, th0 + gaps[:, 0], th0 + gaps[:, 0] + gaps[:, 1]], 1)
    px = np.stack([np.cos(th), np.sin(th)], -1)  # (n, 3, 2)
    phi = rng.uniform(0.0, 2 * np.pi, size=n)
    stretch = np.exp(rng.uniform(-0.7, 0.7, size=n))
    rot = np.stack([np.stack([np.cos(phi), -np.sin(phi)], -1),
                    np.stack([np.sin(phi), np.cos(phi)], -1)], -2)  # (n, 2, 2)
    px = px * np.stack([stretch, 1.0 / stretch], -1)[:, None, :]
    px = np.einsum("nij,nkj->nki", rot, px)
    u = px[:, 1] - px[:, 0]
    v = px[:, 2] - px[:, 0]
    a0 = 0.5 * (u[:, 0] * v[:, 1] - u[:, 1] * v[:, 0])
    px *= np.sqrt(area / a0)[:, None, None]
    ndc = centre[:, None, :] + px / np.array([w / 2.0, h / 2.0])
    zn = rng.uniform(-0.9, 0.9, size=(n, 3))
    cross = rng.random(n) < cross_frac
    ncross = np.where(rng.random(n) < 0.5, 1, 2)
    side = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    for k in range(3):
        sel = cross & (k < ncross)
        zn[sel, k] = side[sel] * rng.uniform(1.05, 2.0, size=sel.sum())
    wv = wt[:, None] * rng.uniform(0.8, 1.2, size=(n, 3))
    clip = np.empty((n, 3, 4))
    clip[..., 0] = ndc[..., 0] * wv
    clip[..., 1] = ndc[..., 1] * wv
    clip[..., 2] = zn * wv
    clip[..., 3] = wv
    col = rng.uniform(0.0, 1.0, size=(n, 3, 3))
    verts = np.concatenate([clip, col], -1).reshape(-1, 7).astype(f32)
    faces = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    return dict(verts=verts, faces=faces, vp=mat.viewport(0, 0, w, h), w=w, h=h, pos_dim=4)


def first_person_camera(eye, target, w, h, focal_ratio_of_aspect, near, far):
    """Camera::new((w, h)) with a FirstPerson transform at `eye` looking at
    `target`, the viewport flipped to y-down rows as demos/src/bin/crates.rs
    sets it ((0..w, h..0)), and a perspective projection
    (render/cam.rs:146-224).  Returns the Camera."""
    fp = mat.FirstPerson(eye)
    fp.look_at(target)
    return (mat.Camera((w, h)).with_transform(fp).viewport((0, w), (h, 0))
            .perspective(focal_ratio_of_aspect, near, far))


def instanced_cubes(ninst=10_000, w=1920, h=1080, seed=3, tex_size=1024):
    """Returns dict(verts, faces, tex, mvps (ninst,4,4), vp, w, h)."""
    rng = np.random.default_rng(seed)
    scale = rng.uniform(0.5, 2.0, size=ninst)
    tx = rng.uniform(-100.0, 100.0, size=ninst)
    tz = rng.uniform(-100.0, 100.0, size=ninst)
    yaw = rng.uniform(0.0, 2 * np.pi, size=ninst)
    # demos/src/bin/crates.rs:51-54: FirstPerson camera, Fov::Diagonal(90 deg),
    # near..far 0.1..1000; here at (0, 2, -110) looking at the origin.
    cam = first_person_camera([0.0, 2.0, -110.0], [0.0, 0.0, 0.0], w, h,
                              lambda a: mat.focal_ratio_diagonal(np.pi / 2.0, a), 0.1, 1000.0)
    vp_proj = cam.world_to_project()
    sc = np.zeros((ninst, 4, 4), f32)
    sc[:, 0, 0] = sc[:, 1, 1] = sc[:, 2, 2] = scale
    sc[:, 3, 3] = 1.0
    sn, cs = np.sin(yaw).astype(f32), np.cos(yaw).astype(f32)
    ry = np.zeros((ninst, 4, 4), f32)
    ry[:, 0, 0], ry[:, 0, 2], ry[:, 2, 0], ry[:, 2, 2] = cs, sn, -sn, cs
    ry[:, 1, 1] = ry[:, 3, 3] = 1.0
    tr = np.tile(np.eye(4, dtype=f32), (ninst, 1, 1))
    tr[:, 0, 3], tr[:, 1, 3], tr[:, 2, 3] = tx, (scale / 2.0), tz
    model = mat.then(mat.then(sc, ry), tr)
    mvps = mat.then(model, vp_proj)
    verts, faces = cube_mesh(1.0, "col_uv")
    return dict(verts=verts, faces=faces, tex=noise_texture(tex_size, seed + 100), mvps=mvps,
                vp=cam.viewport_m, w=w, h=h)


def batch_scenes(nscenes=256, seed=4, min_tris=12, max_tris=200_000, wmin=64, wmax=1920,
                 hmin=64, hmax=1080):
    """Uneven batch of independent scenes: target W and H log-uniform in
    [wmin, wmax] x [hmin, hmax], triangle count log-uniform in [min_tris,
    max_tris], and by coin flip either the fill-stress recipe (Gouraud
    clip-space triangles; the area range scaled by the target's share of a
    1920x1080 frame) or the instanced-cube recipe (tex x Gouraud, one draw
    per cube, triangle count / 12 cubes, texture 64^2..1024^2).

    Returns a list of dicts with kind ("fill" | "cubes"), w, h, vp and the
    fields of fill_stress / instanced_cubes."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nscenes):
        w = int(round(np.exp(rng.uniform(np.log(wmin), np.log(wmax)))))
        h = int(round(np.exp(rng.uniform(np.log(hmin), np.log(hmax)))))
        t = int(round(np.exp(rng.uniform(np.log(min_tris), np.log(max_tris)))))
        s = int(rng.integers(1, 1 << 30))
        if rng.random() < 0.5:
            amax = max(4.0, 1e4 * (w * h) / (1920.0 * 1080.0))
            sc = fill_stress(ntri=max(1, t), w=w, h=h, seed=s, amax=amax)
            sc["kind"] = "fill"
        else:
            tex = 1 << int(rng.integers(6, 11))
            sc = instanced_cubes(ninst=max(1, t // 12), w=w, h=h, seed=s, tex_size=tex)
            sc["kind"] = "cubes"
        out.append(sc)
    return out


def grid_mesh(n, seed=0, attrs="col"):
    """Heightfield over [-1, 1]^2 in x/z: (n+1)^2 vertices, 2 n^2 triangles,
    y a seeded sum of four sine waves, colour from height.  attrs "col"
    (Gouraud, 3 attributes) or "col_uv" (tex x Gouraud: colour, then UV
    repeating 4 times across the grid).  Returns (verts, faces)."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-1.0, 1.0, n + 1)
    X, Z = np.meshgrid(xs, xs)
    k = rng.uniform(1.0, 4.0, size=(4, 2))
    ph = rng.uniform(0.0, 2 * np.pi, size=4)
    Y = sum(np.sin(k[i, 0] * np.pi * X + k[i, 1] * np.pi * Z + ph[i]) for i in range(4)) * 0.04
    t = (Y - Y.min()) / max(1e-9, float(Y.max() - Y.min()))
    col = np.stack([0.2 + 0.6 * t, 0.5 + 0.3 * (1 - t), 0.3 + 0.2 * np.cos(3 * t)], -1)
    cols = [X, Y, Z, col[..., 0], col[..., 1], col[..., 2]]
    if attrs == "col_uv":
        cols += [(X + 1.0) * 2.0, (Z + 1.0) * 2.0]
    verts = np.stack(cols, -1).reshape(-1, len(cols)).astype(f32)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    v00 = (i * (n + 1) + j).reshape(-1)
    v01, v10 = v00 + 1, v00 + n + 1
    v11 = v10 + 1
    faces = np.concatenate([np.stack([v00, v11, v01], -1), np.stack([v00, v10, v11], -1)])
    return verts, faces.astype(np.uint32)


# Preloaded mesh set of the serving workload: (name, shader, mesh builder).
SERVING_MESHES = (
    ("cube12", "textured", lambda: cube_mesh(1.6, "uv")),
    ("grid128", "gouraud", lambda: grid_mesh(8, 1)),
    ("grid2k", "tex_gouraud", lambda: grid_mesh(32, 2, "col_uv")),
    ("grid33k", "gouraud", lambda: grid_mesh(128, 3)),
    ("grid500k", "tex_gouraud", lambda: grid_mesh(500, 4, "col_uv")),
)
SERVING_RESOLUTIONS = ((320, 240, 0.4), (640, 480, 0.3), (1280, 720, 0.2), (1920, 1080, 0.1))


def orbit_camera(seed, w, h, dist=(2.4, 3.6), pitch=(0.35, 1.0)):
    """Per-request camera: yaw U[0, 2 pi), pitch and distance uniform in the
    given ranges, looking at the origin; horizontal FOV 60 degrees, near /
    far 0.1..100.  Returns the 4x4 view-projection matrix."""
    rng = np.random.default_rng(seed)
    yaw = rng.uniform(0.0, 2 * np.pi)
    pt = rng.uniform(*pitch)
    d = rng.uniform(*dist)
    eye = [d * np.cos(pt) * np.sin(yaw), d * np.sin(pt), -d * np.cos(pt) * np.cos(yaw)]
    cam = first_person_camera(eye, [0.0, 0.0, 0.0], w, h,
                              lambda a: mat.focal_ratio_horizontal(np.pi / 3.0), 0.1, 100.0)
    return cam.world_to_project()


def serving_requests(n, rate, seed=5, meshes=SERVING_MESHES, resolutions=SERVING_RESOLUTIONS):
    """n requests with Poisson arrivals at `rate` per second: dicts with
    t (arrival offset, s), mesh (index into meshes), w, h, mvp, vp."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    p = np.array([r[2] for r in resolutions])
    ri = rng.choice(len(resolutions), size=n, p=p / p.sum())
    mi = rng.integers(0, len(meshes), size=n)
    cs = rng.integers(1, 1 << 30, size=n)
    out = []
    for k in range(n):
        w, h = resolutions[ri[k]][:2]
        out.append(dict(t=float(t[k]), mesh=int(mi[k]), w=w, h=h,
                        mvp=orbit_camera(int(cs[k]), w, h), vp=mat.viewport(0, h, w, 0)))
    return out
