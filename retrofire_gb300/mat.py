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
