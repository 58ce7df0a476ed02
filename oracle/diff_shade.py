"""f64 CPU reference of the differentiable shading and its adjoint -- test infrastructure.

The reference renderer has no differentiable path; its only shading quantity is the
screen-space normal's z picked per triangle (src/rasterizer.rs:76).  The shaded image
used by the GPU's sloth_batch_shade is, for the winning sample (x, y) of each depth cell
(the oracle's winner and winner_xy buffers, i.e. the reference's depth test) and its
triangle A, B, C after the f32 matrix M = utransform * transform:

    rgb = (b0*c(A) + b1*c(B) + b2*c(C)) * clamp(unit((B-A) x (C-A)) . L, 0, 1)

with b_i the 2-D barycentric weights of (x, y).  This module evaluates it and its
vector-Jacobian product in float64 with numpy, for visibility held fixed; the tests check
the adjoint against central finite differences of the forward here, and the GPU's f32
adjoint against this one.  Only tests and benchmarks import it.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

NO_HIT = 0xFFFFFFFF


@dataclass
class View:
    """One frame's fixed visibility: per depth cell the winning triangle (-1: none) and
    its sample point, plus the f32 matrix the GPU uses (utransform*transform)."""
    M: np.ndarray          # (4, 4)
    winner: np.ndarray     # (nz,) int, frame-local triangle or -1
    winner_xy: np.ndarray  # (nz,) uint32, x | y << 16


def _hits(view: View):
    cells = np.nonzero(view.winner >= 0)[0]
    t = view.winner[cells].astype(np.int64)
    xy = view.winner_xy[cells].astype(np.int64)
    return cells, t, (xy & 0xFFFF).astype(np.float64), (xy >> 16).astype(np.float64)


def _screen(pos: np.ndarray, M: np.ndarray) -> np.ndarray:
    M = np.asarray(M, np.float64)
    return pos @ M[:3, :3].T + M[:3, 3]


def _tri_ids(idx: np.ndarray | None, t: np.ndarray):
    if idx is None:
        return 3 * t, 3 * t + 1, 3 * t + 2
    idx = np.asarray(idx).reshape(-1, 3).astype(np.int64)
    return idx[t, 0], idx[t, 1], idx[t, 2]


def _terms(pos, vrgb, light, idx, view: View):
    cells, t, px, py = _hits(view)
    S = _screen(np.asarray(pos, np.float64), view.M)
    i0, i1, i2 = _tri_ids(idx, t)
    A, B, C = S[i0], S[i1], S[i2]
    o = (B[:, 0] - A[:, 0]) * (C[:, 1] - A[:, 1]) - (B[:, 1] - A[:, 1]) * (C[:, 0] - A[:, 0])
    n = np.cross(B - A, C - A)
    nl = np.sqrt((n * n).sum(1))
    ok = (o != 0) & (nl > 0)
    o_s = np.where(ok, o, 1.0)
    nl_s = np.where(ok, nl, 1.0)
    w0 = (C[:, 0] - B[:, 0]) * (py - B[:, 1]) - (C[:, 1] - B[:, 1]) * (px - B[:, 0])
    w1 = (A[:, 0] - C[:, 0]) * (py - C[:, 1]) - (A[:, 1] - C[:, 1]) * (px - C[:, 0])
    w2 = (B[:, 0] - A[:, 0]) * (py - A[:, 1]) - (B[:, 1] - A[:, 1]) * (px - A[:, 0])
    b = np.stack([w0, w1, w2], 1) / o_s[:, None]
    V = np.asarray(vrgb, np.float64)
    c0, c1, c2 = V[i0], V[i1], V[i2]
    col = b[:, 0:1] * c0 + b[:, 1:2] * c1 + b[:, 2:3] * c2
    nh = n / nl_s[:, None]
    L = np.asarray(light, np.float64)
    ndl = nh @ L
    s = np.clip(ndl, 0.0, 1.0)
    return dict(cells=cells, t=t, px=px, py=py, A=A, B=B, C=C, o=o_s, ok=ok, n=n, nl=nl_s, nh=nh, ndl=ndl,
                s=s, b=b, c0=c0, c1=c1, c2=c2, col=col, ids=(i0, i1, i2), L=L)


def shade(pos, vrgb, light, idx, view: View) -> np.ndarray:
    """(nz, 3) float64 shaded image of one view."""
    T = _terms(pos, vrgb, light, idx, view)
    out = np.zeros((view.winner.size, 3))
    rgb = T["col"] * T["s"][:, None]
    rgb[~T["ok"]] = 0.0
    out[T["cells"]] = rgb
    return out


def shade_vjp(pos, vrgb, light, idx, view: View, grad_rgb: np.ndarray):
    """(d pos, d vrgb, d light) of sum(grad_rgb * shade(...)) for one view."""
    T = _terms(pos, vrgb, light, idx, view)
    go = np.asarray(grad_rgb, np.float64).reshape(-1, 3)[T["cells"]]
    go = np.where(T["ok"][:, None], go, 0.0)
    s, ndl, b = T["s"], T["ndl"], T["b"]
    gcol = go * s[:, None]                                       # d loss / d col
    gs = np.where((ndl > 0) & (ndl < 1), (go * T["col"]).sum(1), 0.0)
    # colours
    gc = [gcol * b[:, k:k + 1] for k in range(3)]
    # barycentrics b_i = w_i / o
    gb = np.stack([(gcol * T["c0"]).sum(1), (gcol * T["c1"]).sum(1), (gcol * T["c2"]).sum(1)], 1)
    gw = gb / T["o"][:, None]
    go_ = -(gb * b).sum(1) / T["o"]                               # d loss / d o
    A, B, C, px, py = T["A"], T["B"], T["C"], T["px"], T["py"]
    gA = np.zeros_like(A)
    gB = np.zeros_like(B)
    gC = np.zeros_like(C)

    def orient_grad(P, Q, Rx, Ry, g, gP, gQ, gR=None):
        # orient(P, Q, R) = (Qx-Px)(Ry-Py) - (Qy-Py)(Rx-Px)
        gP[:, 0] += g * (Q[:, 1] - Ry)
        gP[:, 1] += g * (Rx - Q[:, 0])
        gQ[:, 0] += g * (Ry - P[:, 1])
        gQ[:, 1] += g * (P[:, 0] - Rx)
        if gR is not None:
            gR[:, 0] += g * (P[:, 1] - Q[:, 1])
            gR[:, 1] += g * (Q[:, 0] - P[:, 0])

    orient_grad(B, C, px, py, gw[:, 0], gB, gC)
    orient_grad(C, A, px, py, gw[:, 1], gC, gA)
    orient_grad(A, B, px, py, gw[:, 2], gA, gB)
    orient_grad(A, B, C[:, 0], C[:, 1], go_, gA, gB, gC)
    # shade factor: s = unit(n) . L, n = (B-A) x (C-A)
    nh, nl, L = T["nh"], T["nl"], T["L"]
    gn = gs[:, None] * (L[None, :] - ndl[:, None] * nh) / nl[:, None]
    e1, e2 = B - A, C - A
    ge1, ge2 = np.cross(e2, gn), np.cross(gn, e1)
    gB += ge1
    gC += ge2
    gA -= ge1 + ge2
    glight = (gs[:, None] * nh).sum(0)
    # screen -> object: object gradient = M3^T screen gradient
    M3 = np.asarray(view.M, np.float64)[:3, :3]
    P = np.asarray(pos)
    gpos = np.zeros((P.shape[0], 3))
    gv = np.zeros((np.asarray(vrgb).shape[0], 3))
    for k, gk in enumerate((gA, gB, gC)):
        np.add.at(gpos, T["ids"][k], gk @ M3)
        np.add.at(gv, T["ids"][k], gc[k])
    return gpos, gv, glight


def interior_cells(pos, idx, view: View, margin: float = 1.0) -> np.ndarray:
    """Mask over depth cells: a winner whose sample lies at least `margin` pixels (in the
    screen's x, y) inside every edge of its triangle."""
    cells, t, px, py = _hits(view)
    S = _screen(np.asarray(pos, np.float64), view.M)
    i0, i1, i2 = _tri_ids(idx, t)
    V = [S[i0], S[i1], S[i2]]
    o = (V[1][:, 0] - V[0][:, 0]) * (V[2][:, 1] - V[0][:, 1]) - (V[1][:, 1] - V[0][:, 1]) * (V[2][:, 0] - V[0][:, 0])
    sign = np.sign(o)
    ok = sign != 0
    for a, c in ((0, 1), (1, 2), (2, 0)):
        P, Q = V[a], V[c]
        w = (Q[:, 0] - P[:, 0]) * (py - P[:, 1]) - (Q[:, 1] - P[:, 1]) * (px - P[:, 0])
        ln = np.hypot(Q[:, 0] - P[:, 0], Q[:, 1] - P[:, 1])
        ok &= (w * sign) >= margin * ln
    mask = np.zeros(view.winner.size, bool)
    mask[cells[ok]] = True
    return mask
