"""Host-side matrix setup in f32 with retrofire's arithmetic.

Matrices are 4x4 row-major float32 arrays (``Matrix.0[row][col]``,
core/src/math/mat.rs:77-80).  Every product folds its dot products from
0.0 in index order like ``vec::dot`` (core/src/math/vec.rs:231-238), so a
matrix composed here has the same bits as the reference's ``then`` /
``compose`` (mat.rs:268-299) given the same factors.  Trigonometry
(``rotate_*``) goes through numpy's float32 sin/cos; the result is shared
by the CUDA path and the oracle, so it never affects parity.
"""
import numpy as np

f32 = np.float32


def _dot(a, b):
    acc = f32(0.0)
    for x, y in zip(a, b):
        acc = f32(acc + f32(f32(x) * f32(y)))
    return acc


def compose(m, n):
    """m.compose(n): apply n first, then m (mat.rs:268-283).

    Element (j, i) is dot(m[j], column i of n) folded from 0.0 in k order;
    works on stacks of matrices (..., 4, 4)."""
    m = np.asarray(m, f32)
    n = np.asarray(n, f32)
    acc = np.zeros(np.broadcast_shapes(m.shape, n.shape), f32)
    for k in range(4):
        acc = (acc + m[..., :, k, None] * n[..., None, k, :]).astype(f32)
    return acc


def then(m, n):
    """m.then(n) == n.compose(m) (mat.rs:284-299)."""
    return compose(n, m)


def translate3(x, y, z):
    """mat.rs:1078-1085."""
    m = np.eye(4, dtype=f32)
    m[0, 3], m[1, 3], m[2, 3] = f32(x), f32(y), f32(z)
    return m


def scale3(x, y, z):
    return np.diag([f32(x), f32(y), f32(z), f32(1.0)]).astype(f32)


def _sc(a):
    a = f32(a)
    return f32(np.sin(a)), f32(np.cos(a))


def rotate_x(a):
    """mat.rs:1147-1156 (angle in radians)."""
    s, c = _sc(a)
    return np.array([[1, 0, 0, 0], [0, c, -s, 0], [0, s, c, 0], [0, 0, 0, 1]], f32)


def rotate_y(a):
    """mat.rs:1168-1177."""
    s, c = _sc(a)
    return np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]], f32)


def rotate_z(a):
    """mat.rs:1187-1196."""
    s, c = _sc(a)
    return np.array([[c, -s, 0, 0], [s, c, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], f32)


def perspective(focal_ratio, aspect_ratio, near, far):
    """mat.rs:1255-1277; panics become ValueError."""
    fr, ar, n, fa = f32(focal_ratio), f32(aspect_ratio), f32(near), f32(far)
    if not (fr > 0 and ar > 0 and n > 0 and fa > n):
        raise ValueError("perspective: parameters must be positive and far > near")
    e00 = fr
    e11 = f32(e00 * ar)
    e22 = f32(f32(fa + n) / f32(fa - n))
    e23 = f32(f32(f32(f32(2.0) * fa) * n) / f32(n - fa))
    return np.array([[e00, 0, 0, 0], [0, e11, 0, 0], [0, 0, e22, e23], [0, 0, 1, 0]], f32)


def viewport(x0, y0, x1, y1):
    """viewport(pt2(x0, y0)..pt2(x1, y1)) (mat.rs:1304-1315)."""
    x0, y0, x1, y1 = f32(x0), f32(y0), f32(x1), f32(y1)
    dx = f32(f32(x1 - x0) / f32(2.0))
    dy = f32(f32(y1 - y0) / f32(2.0))
    return np.array([[dx, 0, 0, f32(x0 + dx)], [0, dy, 0, f32(y0 + dy)],
                     [0, 0, 1, 0], [0, 0, 0, 1]], f32)


def apply_point(m, p):
    """Mat4 . Point3 (mat.rs:929-950) or ProjMat3 . Point3 (mat.rs:952-973)."""
    h = [f32(p[0]), f32(p[1]), f32(p[2]), f32(1.0)]
    m = np.asarray(m, f32)
    return np.array([_dot(m[r], h) for r in range(4)], f32)


def focal_ratio_diagonal(fov_rad, aspect):
    """Fov::Diagonal (cam.rs:118-143)."""
    ratio = f32(1.0) / f32(np.tan(f32(fov_rad) / f32(2.0)))
    diag = f32(np.sqrt(f32(1.0) + f32(f32(1.0) / f32(aspect)) / f32(aspect)))
    return f32(ratio * diag)


def focal_ratio_horizontal(fov_rad):
    """Fov::Horizontal (cam.rs:130)."""
    return f32(f32(1.0) / f32(np.tan(f32(fov_rad) / f32(2.0))))


# ---- vectors, angles and the camera (render/cam.rs) ------------------------

def cross(a, b):
    """Vec3::cross (vec.rs:555-566)."""
    a = [f32(x) for x in a]
    b = [f32(x) for x in b]
    return np.array([f32(f32(a[1] * b[2]) - f32(a[2] * b[1])),
                     f32(f32(a[2] * b[0]) - f32(a[0] * b[2])),
                     f32(f32(a[0] * b[1]) - f32(a[1] * b[0]))], f32)


def normalize(v):
    """Vector::normalize (vec.rs:151-162): v * len_sqr.powf(-0.5) (std)."""
    v = np.asarray(v, f32)
    ls = _dot(v, v)
    if not np.isfinite(ls) or abs(float(ls)) <= 1e-12:
        raise ValueError("cannot normalize a near-zero or non-finite vector")
    return (v * f32(np.power(ls, f32(-0.5), dtype=f32))).astype(f32)


def from_linear(i, j, k):
    """Mat4::from_linear (mat.rs:532-560): the basis vectors as columns."""
    m = np.eye(4, dtype=f32)
    m[:3, 0], m[:3, 1], m[:3, 2] = i, j, k
    return m


def orient_z(new_z, x):
    """orient_z (mat.rs:1112-1132): new_y = (new_z x x).normalize(),
    new_x = new_y x new_z."""
    new_y = normalize(cross(new_z, x))
    return from_linear(cross(new_y, new_z), new_y, np.asarray(new_z, f32))


def spherical_to_cart(r, az, alt):
    """SphericalVec::to_cart (angle.rs:362-376)."""
    sa, ca = f32(np.sin(f32(alt))), f32(np.cos(f32(alt)))
    sz, cz = f32(np.sin(f32(az))), f32(np.cos(f32(az)))
    r = f32(r)
    return np.array([f32(r * f32(cz * ca)), f32(r * sa), f32(r * f32(-sz * ca))], f32)


def cart_to_spherical(v):
    """Vec3::to_spherical (angle.rs:452-458): (r, az, alt)."""
    x, y, z = (f32(c) for c in v)
    az = f32(np.arctan2(-z, x))
    alt = f32(np.arctan2(y, f32(np.sqrt(f32(f32(x * x) + f32(z * z))))))
    r = f32(np.sqrt(_dot([x, y, z], [x, y, z])))
    return r, az, alt


def _wrap(a, lo, hi):
    """Angle::wrap (angle.rs:224-227): lo + rem_euclid(a - lo, hi - lo)."""
    a, lo, hi = f32(a), f32(lo), f32(hi)
    d = f32(hi - lo)
    r = f32(np.fmod(f32(a - lo), d))
    if r < 0:
        r = f32(r + abs(d))
    return f32(lo + r)


TAU = f32(2.0 * np.pi)


class FirstPerson:
    """FirstPerson camera transform (cam.rs:71-76, 403-418, 322-430)."""

    def __init__(self, pos=(0.0, 0.0, 0.0)):
        self.pos = np.asarray(pos, f32)
        self.heading = (f32(0.0), f32(0.0), f32(0.0))  # SphericalVec::default: (r, az, alt)

    def rotate_to(self, az, alt):
        """cam.rs rotate_to: azimuth wrapped to [-1/2, 1/2) turn, altitude
        clamped to [-1/4, 1/4] turn."""
        half, quarter = f32(TAU * f32(0.5)), f32(TAU * f32(0.25))
        self.heading = (f32(1.0), _wrap(az, -half, half),
                        f32(min(max(f32(alt), -quarter), quarter)))

    def look_at(self, pt):
        """Centers the view on a world-space point (cam.rs look_at)."""
        d = (np.asarray(pt, f32) - self.pos).astype(f32)
        _, az, alt = cart_to_spherical(d)
        self.rotate_to(az, alt)

    def world_to_view(self):
        """Transform::world_to_view for FirstPerson (cam.rs:403-418)."""
        r, az, alt = self.heading
        fwd_move = spherical_to_cart(1.0, az, 0.0)
        fwd = spherical_to_cart(r, az, alt)
        right = cross([0.0, 1.0, 0.0], fwd_move)
        inv_origin = translate3(-self.pos[0], -self.pos[1], -self.pos[2])
        inv_orient = orient_z(fwd, right).T.copy()
        return then(inv_origin, inv_orient)


class Camera:
    """Camera (cam.rs:146-254): dims, viewport, projection and a transform."""

    def __init__(self, dims):
        w, h = dims
        self.dims = (int(w), int(h))
        self.viewport_m = viewport(0, 0, w, h)        # Camera::new
        self.project = np.eye(4, dtype=f32)
        self.transform = None

    def with_transform(self, tf):
        self.transform = tf
        return self

    def viewport(self, xs, ys):
        """Camera::viewport((l..r, t..b)): bounds intersected with the
        target, dims = their extent (cam.rs:170-188)."""
        w, h = self.dims
        l, r = xs
        t, b = ys
        l, r = min(max(l, 0), w), min(max(r, 0), w)
        t, b = min(max(t, 0), h), min(max(b, 0), h)
        self.dims = (abs(r - l), abs(b - t))
        self.viewport_m = viewport(l, t, r, b)
        return self

    def perspective(self, focal_ratio_of_aspect, near, far):
        """Camera::perspective (cam.rs:198-205); focal_ratio_of_aspect maps
        the aspect ratio to Fov::focal_ratio."""
        aspect = f32(f32(self.dims[0]) / f32(self.dims[1]))
        self.project = perspective(focal_ratio_of_aspect(aspect), aspect, near, far)
        return self

    def world_to_project(self):
        """world_to_view().then(&project) (cam.rs:222-224)."""
        return then(self.transform.world_to_view(), self.project)

    def model_to_project(self, to_world):
        """The uniform Camera::render passes: to_world.then(world_to_project)."""
        return then(to_world, self.world_to_project())
