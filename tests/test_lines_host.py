"""Line primitives in the oracle (render() of Edge<usize>: clip.rs line
clipping, raster.rs line()): known answers worked out from the algorithm
(the reference has no line test)."""
import numpy as np

import retrofire_gb300 as rf
from oracle import oracle as O

W, H = 24, 16
# to_screen: screen = 10 ndc + 12 in x, 8 ndc + 8 in y (depth = 1/w)
VP = np.array([[10, 0, 0, 12], [0, 8, 0, 8], [0, 0, 1, 0], [0, 0, 0, 1]], np.float32)


def ndc(x, y):
    return (x - 12.0) / 10.0, (y - 8.0) / 8.0


def draw(segs, colors=None, ctx=None, z=None):
    """segs: list of ((x0, y0), (x1, y1)) in screen pixels; clip-space
    vertices with w = 1 and per-vertex colour; returns (pixels, color, st)."""
    verts, lines = [], []
    for i, (a, b) in enumerate(segs):
        for k, p in enumerate((a, b)):
            x, y = ndc(*p)
            col = colors[i][k] if colors else (0.5, 0.25, 0.75)
            zz = 0.0 if z is None else z[i]
            verts.append([x, y, zz, 1.0, *col])
        lines.append([2 * i, 2 * i + 1])
    color = np.zeros((H, W), np.uint32)
    depth = np.zeros((H, W), np.float32)
    O.clear(color, depth)
    st = O.render_lines(np.array(verts, np.float32), np.array(lines), rf.GOURAUD, VP, color, depth,
                        ctx or {}, pos_dim=4)
    ys, xs = np.nonzero(color != 0xFF000000)
    return sorted(zip(xs.tolist(), ys.tolist())), color, st


def test_horizontal_and_vertical_pixels():
    px, _, st = draw([((2.2, 3.7), (9.6, 3.7))])
    # x from round_up_to_half(2.2) = 2.5 (as usize 2) to 10.5 (10): 2..9 on row 3
    assert px == [(x, 3) for x in range(2, 10)]
    assert (st.frags_i, st.frags_o, st.prims_o, st.verts_o) == (8, 8, 1, 3)
    px, _, st = draw([((5.3, 1.2), (5.3, 6.8))])
    # y from 1.5 (1) to 7.5 (7): rows 1..6 in column 5
    assert px == sorted((5, y) for y in range(1, 7))


def test_shallow_line_steps_y_per_column():
    px, _, _ = draw([((2.2, 2.2), (11.2, 4.2))])  # dy/dx = 2/9
    ys = dict(px)
    # x from 2.5 (2) to 11.5 (11); y starts at 2.2 + (2.5 - 2.2) 2/9 and steps
    assert sorted(ys) == list(range(2, 11))
    assert ys[2] == 2 and ys[10] == 4
    assert all(ys[x + 1] - ys[x] in (0, 1) for x in range(2, 10))


def test_clipped_at_the_frustum_side():
    px, _, _ = draw([((1.2, 2.2), (11.2, 4.2))])  # x = 1.2 lies outside (ndc -1.08)
    assert min(x for x, _ in px) == 2             # starts at the left plane, x = 2.0


def test_first_vertex_varyings_and_depth():
    # after line()'s swap the vertex with the smaller y is v0: here the
    # second, blue one gives every pixel of the tall line its colour
    px, col, _ = draw([((5.3, 6.8), (5.3, 1.2))], colors=[[(1.0, 0.0, 0.0), (0.0, 0.0, 1.0)]])
    assert set(col[y, x] for x, y in px) == {O.pack((255 << 24) | (255 << 16), 0)}
    # a wide line drawn right to left: the left end (after the second swap)
    px, col, _ = draw([((9.6, 3.7), (2.2, 3.9))], colors=[[(1.0, 0.0, 0.0), (0.0, 1.0, 0.0)]])
    assert set(col[y, x] for x, y in px) == {O.pack((255 << 24) | (255 << 8), 0)}


def test_depth_ties_keep_the_first_line():
    segs = [((2.2, 3.7), (9.6, 3.7)), ((2.2, 3.7), (9.6, 3.7))]
    cols = [[(1.0, 0.0, 0.0)] * 2, [(0.0, 1.0, 0.0)] * 2]
    px, col, st = draw(segs, colors=cols)
    assert st.frags_i == 16 and st.frags_o == 8  # Less: equal depth fails
    assert set(col[y, x] for x, y in px) == {O.pack((255 << 24) | 255, 0)}


def test_front_culling_drops_lines_and_clipping():
    _, _, st = draw([((2.2, 3.7), (9.6, 3.7))], ctx={"face_cull": rf.CULL_FRONT})
    assert (st.prims_i, st.prims_o, st.frags_i) == (1, 0, 0)
    # a line from inside to beyond the far plane is clipped at it, not dropped
    verts = np.array([[0.0, 0.0, 0.5, 1.0, 1, 1, 1], [0.5, 0.0, 3.0, 1.0, 1, 1, 1]], np.float32)
    color = np.zeros((H, W), np.uint32)
    depth = np.zeros((H, W), np.float32)
    O.clear(color, depth)
    st = O.render_lines(verts, np.array([[0, 1]]), rf.GOURAUD, VP, color, depth, {}, pos_dim=4)
    assert st.prims_o == 1 and 0 < st.frags_i < 5
    both_out = np.array([[0.0, 0.0, 2.0, 1.0, 1, 1, 1], [0.5, 0.0, 3.0, 1.0, 1, 1, 1]], np.float32)
    st = O.render_lines(both_out, np.array([[0, 1]]), rf.GOURAUD, VP, color, depth, {}, pos_dim=4)
    assert st.prims_o == 0
