"""Pins the CPU oracle (no GPU).

1. The reference's own known-answer tests, src/geometry.rs:196-234.
2. Hand-derived micro cases of draw_triangle (src/rasterizer.rs:48-93): coverage, the
   loose 2*max.x range, depth ties, the wrapped id = y*w + 2x, the id+1 half cell, the
   newline sentinel, back-facing and degenerate triangles.
3. A second, independent restatement in numpy float32 scalars (small cases only)
   compared with the C oracle on seeded random triangles.
4. The banded multi-threaded oracle equals the sequential one.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
import workloads as W

F = np.float32
BLANK = ord(" ")


def cell(ch, rgb):
    return ord(ch) | (rgb[0] << 8) | (rgb[1] << 16) | (rgb[2] << 24)


# ---------------------------------------------------------------------------------- KATs
DEFAULT_TRI = [1.0, -1.0, -1.0, 1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 1.0, -1.0, 1.0]


def test_kat_aabb():
    """src/geometry.rs:196-206"""
    mn, mx = O.triangle_aabb(DEFAULT_TRI)
    assert mn.tolist() == [-1.0, -1.0, -1.0, 1.0]
    assert mx.tolist() == [1.0, 1.0, 1.0, 1.0]


def test_kat_transform():
    """src/geometry.rs:208-220: Matrix4::new_translation(&Vector3::new(1,1,1))."""
    T = np.array([[1, 0, 0, 1], [0, 1, 0, 1], [0, 0, 1, 1], [0, 0, 0, 1]], np.float32)
    v = O.triangle_mul(DEFAULT_TRI, T)
    mn, mx = O.triangle_aabb(v.reshape(-1))
    assert mn.tolist() == [0.0, 0.0, 0.0, 1.0]
    assert mx.tolist() == [2.0, 2.0, 2.0, 1.0]


def test_kat_normal():
    """src/geometry.rs:222-234"""
    n = O.triangle_normal([-1, 1, 0, 1, 0, 1, 1, 1, 1, 1, 0, 1])
    assert n.tolist() == [0.0, 1.0, 0.0, 0.0]


def test_default_shader_ramp():
    """src/rasterizer.rs:5-27 with f32 thresholds."""
    cases = {-1.0: ".", 0.2: ".", float(np.nextafter(F(0.2), F(1))): ":", 0.3: ":", 0.4: "-",
             0.5: "=", 0.6: "+", 0.7: "*", 0.8: "#", 0.9: "%", 1.0: "@",
             float(np.nextafter(F(1.0), F(2))): " ", float("nan"): " ", float("inf"): " "}
    for s, ch in cases.items():
        assert O.default_shader(s) == ch, s


def test_viewport_transform_and_extent():
    """src/context.rs:104-133: scale = min(h, w/2)/ext/2, translation (w/4, h/2)."""
    assert O.scene_extent([[0.5, 2.0, -3.0], [1.5, float("nan"), 0.25]]) == 2.0
    assert O.scene_extent(np.zeros((0, 3))) == 0.0
    U = O.viewport_transform(160, 48, 1.0)
    assert U.tolist() == [[24.0, 0, 0, 40.0], [0, -24.0, 0, 24.0], [0, 0, 24.0, 0], [0, 0, 0, 1.0]]
    U = O.viewport_transform(3840, 2160, 1.25)
    s = F(F(F(1920.0) / F(1.25)) / F(2.0))
    assert U[0, 0] == s and U[1, 1] == -s and U[0, 3] == 960.0 and U[1, 3] == 1080.0


def test_euler_rotation_matches_nalgebra_formula():
    """Rotation3::from_euler_angles(roll, pitch, yaw): Rz(yaw)*Ry(pitch)*Rx(roll)."""
    for angles in [(0.5, math.pi, 0.0), (0.1, 0.2, 0.3), (0.0, 0.0, 0.0)]:
        R = O.euler_rotation(*angles).astype(np.float64)
        r, p, y = angles
        Rx = np.array([[1, 0, 0], [0, math.cos(r), -math.sin(r)], [0, math.sin(r), math.cos(r)]])
        Ry = np.array([[math.cos(p), 0, math.sin(p)], [0, 1, 0], [-math.sin(p), 0, math.cos(p)]])
        Rz = np.array([[math.cos(y), -math.sin(y), 0], [math.sin(y), math.cos(y), 0], [0, 0, 1]])
        np.testing.assert_allclose(R[:3, :3], Rz @ Ry @ Rx, atol=2e-7)
        assert R[3].tolist() == [0, 0, 0, 1] and R[:3, 3].tolist() == [0, 0, 0]


def test_cli_rotation_slots():
    """src/inputs.rs:131-149: --yaw feeds roll, pi is added to the pitch in f32."""
    r, p, y = W.cli_rotation(yaw=0.5)
    assert r == 0.5 and y == 0.0 and p == float(F(math.pi))


# ----------------------------------------------------------------- hand-derived micro cases
I4 = np.eye(4, dtype=np.float32)


def draw(tris, w, h, image, U=I4, R=I4):
    """tris: list of (v9, rgb)."""
    o = O.Oracle(w, h, image, U)
    M = O.mat4_mul(U, R)
    for v, rgb in tris:
        o.draw_triangle(v, rgb, M)
    return o.frame()


def test_single_triangle_coverage():
    # screen-space triangle (1,1) (5,1) (1,5): w0 = 24-4(px+py), w1 = 4(px-1), w2 = 4(py-1).
    # Loose range: x in [1, ceil(min(10, 15))) = [1,10), y in [1, ceil(min(5, 7))) = [1,5).
    # Covered iff px + py <= 6.  z = 0.5 everywhere; shade = 1*(1/16)*16 = 1.0 -> '@'.
    f = draw([([1, 1, 0.5, 5, 1, 0.5, 1, 5, 0.5], (10, 20, 30))], 16, 8, False)
    cov = {(x, y) for y in range(1, 5) for x in range(1, 10) if x + y <= 6}
    assert f.fragments == len(cov) == 14
    assert f.candidates == 4 * 9
    exp_z = np.full(16 * 8, np.finfo(np.float32).max, np.float32)
    exp_c = np.full(16 * 8, BLANK, np.uint32)
    for x, y in cov:
        i = y * 16 + 2 * x
        exp_z[i] = 0.5
        exp_c[i] = exp_c[i + 1] = cell("@", (10, 20, 30))
    assert np.array_equal(f.z, exp_z)
    assert np.array_equal(f.cells, exp_c)


def test_back_facing_and_degenerate_write_nothing_but_newlines():
    # clockwise (back-facing) triangle: all three edge functions can't be >= 0
    back = ([1, 1, 0, 1, 5, 0, 5, 1, 0], (1, 2, 3))
    # degenerate: collinear on y = x, orient = 0, a = 1/0 = inf.  The samples on the line
    # have w0 = w1 = w2 = 0 (covered) but z = v1z + inf*0 = NaN, which never passes z < zbuf.
    diag = ([1, 1, 0, 3, 3, 1, 5, 5, 2], (4, 5, 6))
    f = draw([back, diag], 12, 8, True)
    assert (f.z == np.finfo(np.float32).max).all()
    # newline sentinels: rows [1,5) of both triangles (written even without coverage)
    nl = [i for i, c in enumerate(f.cells) if c & 0xFF == ord("\n")]
    assert nl == [y * 12 + 1 for y in range(1, 5)]
    assert f.fragments == 4   # (1,1) (2,2) (3,3) (4,4)
    assert f.candidates == 4 * 9 + 4 * 9


def test_depth_tie_first_writer_wins_and_minus_zero():
    # Two identical triangles at z = 0 then a third at z = -0.0: ties keep the first.
    t = [1, 1, 0, 5, 1, 0, 1, 5, 0]
    tneg = [1, 1, -0.0, 5, 1, -0.0, 1, 5, -0.0]
    f = draw([(t, (1, 1, 1)), (t, (2, 2, 2)), (tneg, (3, 3, 3))], 16, 8, False)
    i = 1 * 16 + 2 * 1
    assert f.winner[i] == 0 and f.cells[i] == cell("@", (1, 1, 1))
    # a nearer triangle later wins
    tnear = [1, 1, -1, 5, 1, -1, 1, 5, -1]
    f = draw([(t, (1, 1, 1)), (tnear, (9, 9, 9))], 16, 8, False)
    assert f.winner[i] == 1 and f.z[i] == -1.0 and f.cells[i] == cell("@", (9, 9, 9))


def test_wrapped_cell_and_half_cell():
    # w = 8: sample x >= 4 writes depth cell y*8 + 2x = (y+1)*8 + (2x-8) in the next row.
    # Triangle A (1,1)(6,1)(1,4): covered row 1: x 1..6, row 2: x 1..4, row 3: x 1..2.
    # All at z = 0: in row 2, x=1 targets id 18 = the wrapped (5,1) sample's cell -> tie,
    # the earlier (5,1) write stays.
    A = ([1, 1, 0, 6, 1, 0, 1, 4, 0], (7, 7, 7))
    f = draw([A], 8, 6, False)
    assert f.winner[2 * 8 + 0] == 0      # (4,1) wrapped
    assert f.winner[2 * 8 + 2] == 0      # (5,1) wrapped; (1,2) tied and lost
    z = f.z.reshape(6, 8)
    assert z[1, 2] == 0 and z[1, 4] == 0 and z[1, 6] == 0 and z[1, 0] == np.finfo(np.float32).max
    # the id+1 half cell of the last cell of row 1 (id 15 is odd: never a depth target for
    # even w), so frame cell 16 is written only by (4,1).
    assert f.cells[16] == cell("@", (7, 7, 7))


def test_half_cell_later_writer_overrides_neighbour():
    # Two triangles: B (later, farther) writes cell c; A (earlier, nearer) wrote c-1 ...
    # with even w, depth cells are even so id+1 is odd and never a depth cell: the
    # frame cell id+1 takes the later of its left neighbour's writes only.
    # With odd w = 9 the wrapped samples land on odd cells: cell c gets a depth write
    # from a wrapped sample AND the id+1 write of cell c-1.
    w, h = 9, 6
    # A (1,2)(3,2)(1,3): row 2 only, covered x = 1..3 -> depth ids 20, 22, 24 (z = 5)
    # B (5,1)(6,1)(5,2): row 1 only, covered x = 5, 6 -> wrapped ids 19, 21 (odd cells)
    A = ([1, 2, 5, 3, 2, 5, 1, 3, 5], (1, 0, 0))
    B = ([5, 1, 1, 6, 1, 1, 5, 2, 1], (0, 2, 0))
    f = draw([A, B], w, h, False)
    assert [int(f.winner[i]) for i in range(18, 26)] == [-1, 1, 0, 1, 0, -1, 0, -1]
    # frame cells 19..22 come from B (its id and id+1 writes are later than A's),
    # 23..25 from A.
    b, a = f.cells[19] >> 8, f.cells[24] >> 8
    assert b == (2 << 8) and a == 1
    assert [int(c >> 8) for c in f.cells[19:26]] == [b, b, b, b, a, a, a]


def test_newline_sentinel_order():
    # image mode: after each row y of a triangle's range, cell y*w+1 = '\n'.  A later
    # triangle's row write at y*w+1 comes from a wrapped sample of row y-1 (w even:
    # x = w/2).  Draw order decides.
    w, h = 8, 6
    # T0 wraps (4,1) -> id 16 = 2*8+0 ; its id+1 = 17 = 2*8+1 = newline cell of row 2
    T0 = ([1, 1, 0, 6, 1, 0, 1, 4, 0], (5, 5, 5))
    f = draw([T0], w, h, True)
    # rows [1,4): newline at 9, 17, 25; row 2's newline comes after (4,1)'s id+1 write
    assert f.cells[17] & 0xFF == ord("\n")
    assert f.cells[9] & 0xFF == ord("\n")
    # now a later triangle whose only range row is 1 and which writes id 16/17 again
    T1 = ([4, 1, -1, 5, 1, -1, 4, 1.5, -1], (6, 6, 6))
    f = draw([T0, T1], w, h, True)
    # T1 rows [1, ceil(1.5)=2) -> newline at 9 only; its (4,1) sample is nearer -> writes 16,17
    assert f.cells[17] == cell("@", (6, 6, 6)) or f.cells[17] & 0xFF != ord("\n")
    assert f.cells[9] & 0xFF == ord("\n")
    assert len(f.cells) == w * h + h and (f.cells[w * h:] == BLANK).all()


# --------------------------------------------------- independent numpy-scalar restatement
def py_draw(tris, w, h, image, M):
    """src/rasterizer.rs:48-93 restated with numpy float32 scalars (small cases only)."""
    zb = [F(np.finfo(np.float32).max)] * (w * h)
    fb = [BLANK] * (w * h + (h if image else 0))
    frags = 0
    for t, (v, rgb) in enumerate(tris):
        V = []
        for k in range(3):
            p = [F(v[3 * k]), F(v[3 * k + 1]), F(v[3 * k + 2]), F(1.0)]
            out = []
            for i in range(4):
                acc = F(M[i][0]) * p[0]
                for j in range(1, 4):
                    acc = F(M[i][j]) * p[j] + acc
                out.append(acc)
            V.append(out)

        def orient(a, b, c):
            return (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0])

        def usize(f):
            return 0 if not (f > 0) else int(f)

        mnx = min(V[0][0], V[1][0], V[2][0]); mny = min(V[0][1], V[1][1], V[2][1])
        mxx = max(V[0][0], V[1][0], V[2][0]); mxy = max(V[0][1], V[1][1], V[2][1])
        x0 = usize(np.ceil(max(mnx, F(1)))); y0 = usize(np.ceil(max(mny, F(1))))
        x1 = usize(np.ceil(min(mxx * F(2), F(w - 1)))); y1 = usize(np.ceil(min(mxy, F(h - 1))))
        with np.errstate(all="ignore"):
            a = F(1) / orient(V[0], V[1], V[2])
            e1 = [V[1][i] - V[0][i] for i in range(3)]
            e2 = [V[2][i] - V[0][i] for i in range(3)]
            nx = e1[1] * e2[2] - e1[2] * e2[1]
            ny = e1[2] * e2[0] - e1[0] * e2[2]
            nz = e1[0] * e2[1] - e1[1] * e2[0]
            n = np.sqrt(F(0) + ((nx * nx + nz * nz) + (ny * ny + F(0) * F(0))))
            nzh = nz / n
            for y in range(y0, y1):
                for x in range(x0, x1):
                    p = [F(x), F(y)]
                    w0 = orient(V[1], V[2], p); w1 = orient(V[2], V[0], p); w2 = orient(V[0], V[1], p)
                    if w0 >= 0 and w1 >= 0 and w2 >= 0:
                        frags += 1
                        shade = nzh * a * (w0 + w1 + w2)
                        z = V[0][2] + a * (w1 * (V[1][2] - V[0][2]) + w2 * (V[2][2] - V[0][2]))
                        i = y * w + 2 * x
                        if z < zb[i]:
                            zb[i] = z
                            c = cell(O.default_shader(float(shade)), rgb)
                            fb[i] = fb[i + 1] = c
                if image:
                    fb[y * w + 1] = ord("\n")
    return np.array(fb, np.uint32), np.array(zb, np.float32), frags


@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_numpy_restatement(seed):
    rng = np.random.default_rng(100 + seed)
    w = int(rng.integers(5, 23))
    h = int(rng.integers(4, 14))
    image = bool(seed % 2)
    tris = []
    for k in range(25):
        c = rng.uniform(-0.2, 1.2, size=3) * [w / 2, h, 1]
        v = (c + rng.normal(0, 2.5, size=(3, 3))).astype(np.float32)
        if k % 7 == 3:
            v[2] = v[0] + (v[1] - v[0]) * 2   # collinear
        if k % 5 == 1:
            v[:, 2] = np.float32(0.25)        # depth ties
        tris.append((v.reshape(-1).tolist(), tuple(int(t) for t in rng.integers(0, 256, 3))))
    R = O.euler_rotation(0.0, float(rng.uniform(-0.1, 0.1)), 0.0)
    U = np.eye(4, dtype=np.float32)
    U[2, 2] = 1.0
    M = O.mat4_mul(U, R)
    f = draw(tris, w, h, image, U=U, R=R)
    cells, z, frags = py_draw(tris, w, h, image, M)
    assert f.fragments == frags
    assert np.array_equal(f.cells, cells)
    assert np.array_equal(f.z.view(np.uint32), z.view(np.uint32))


# ------------------------------------------------------------------- banded == sequential
@pytest.mark.parametrize("w,h,image", [(160, 48, True), (161, 49, False), (97, 40, True), (8, 6, True)])
def test_banded_equals_sequential(w, h, image):
    m = W.soup(3000, seed=w + h, n_large=20, sigma=0.05)
    R = O.euler_rotation(0.4, float(W.PI_F32) + np.float32(0.3), 0.2)
    U = O.viewport_transform(w, h, O.scene_extent([m["bbox_max"]]))
    a = O.Oracle(w, h, image, U)
    a.draw_mesh(m["x"], m["y"], m["z"], m["rgb"], R)
    a.draw_mesh(m["x"][:300], m["y"][:300], m["z"][:300], m["rgb"][:100], R)
    b = O.Oracle(w, h, image, U)
    b.draw_mesh(m["x"], m["y"], m["z"], m["rgb"], R, threads=5)
    b.draw_mesh(m["x"][:300], m["y"][:300], m["z"][:300], m["rgb"][:100], R, threads=3)
    fa, fb_ = a.frame(), b.frame()
    assert fa.fragments == fb_.fragments and fa.candidates == fb_.candidates
    assert np.array_equal(fa.cells, fb_.cells)
    assert np.array_equal(fa.z.view(np.uint32), fb_.z.view(np.uint32))
    assert np.array_equal(fa.winner, fb_.winner)
