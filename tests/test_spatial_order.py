"""The order in which setup takes an indexed mesh's triangles (sloth_spatial_order, host
only): checked on the CPU against a numpy restatement of its rule (Morton code of the
centroid in the box of the finite centroids, stable in index order), as a permutation,
with non-finite vertices and bad indices, and for the locality it is there for."""
import numpy as np
import pytest

import sloth_gpu as S
import workloads as W


def restated_codes(x, y, z, idx):
    i = np.asarray(idx, np.int64).reshape(-1, 3)
    with np.errstate(invalid="ignore", over="ignore"):
        c = [(v[i[:, 0]] + v[i[:, 1]]) + v[i[:, 2]] for v in (x, y, z)]   # f32, left to right
    finite = np.isfinite(c[0]) & np.isfinite(c[1]) & np.isfinite(c[2])
    code = np.zeros(i.shape[0], np.int64)
    q = []
    for s in c:
        fin = np.isfinite(s)
        lo = np.float64(s[fin].min()) if fin.any() else np.inf
        hi = np.float64(s[fin].max()) if fin.any() else -np.inf
        with np.errstate(invalid="ignore", over="ignore"):
            f = (s.astype(np.float64) - lo) / (hi - lo) if hi > lo else np.zeros(s.size)
            qa = np.where(f <= 0.0, 0, np.where(f >= 1.0, 1023, np.nan_to_num(f * 1024.0))).astype(np.int64)
        q.append(qa)
    for b in range(10):
        for a in range(3):
            code |= ((q[a] >> b) & 1) << (3 * b + a)
    code[~finite] = 0
    return code


def restated_order(x, y, z, idx):
    return np.argsort(restated_codes(x, y, z, idx), kind="stable").astype(np.uint32)


def shuffled(m, seed):
    rng = np.random.default_rng(seed)
    idx = m["idx"][rng.permutation(m["idx"].shape[0])]
    return m["x"], m["y"], m["z"], np.ascontiguousarray(idx, np.uint32)


def test_matches_restatement_and_is_a_permutation():
    for seed, m in enumerate([W.displaced_icosphere(3, seed=1), W.uv_sphere(), W.displaced_icosphere(5, seed=2)]):
        x, y, z, idx = shuffled(m, seed)
        got = S.spatial_order(x, y, z, idx)
        assert np.array_equal(np.sort(got), np.arange(idx.shape[0], dtype=np.uint32))
        assert np.array_equal(got, restated_order(x, y, z, idx))


def test_non_finite_centroids_go_first_in_index_order():
    m = W.displaced_icosphere(2, seed=4)
    x, y, z, idx = shuffled(m, 9)
    x = x.copy()
    y = y.copy()
    bad = np.unique(idx[[3, 50, 51, 200]].reshape(-1))[:3]
    x[bad[0]] = np.nan
    y[bad[1]] = np.inf
    z = z.copy()
    z[bad[2]] = np.float32(3e38)   # finite; its triangles stretch the box along z
    got = S.spatial_order(x, y, z, idx)
    assert np.array_equal(got, restated_order(x, y, z, idx))
    # the non-finite triangles take code 0: they come first, in index order, among the
    # triangles of the box's lowest cell
    nonfin = np.nonzero(np.isin(idx, bad[:2]).any(1))[0]
    codes = restated_codes(x, y, z, idx)
    pos = np.nonzero(np.isin(got, nonfin))[0]
    assert np.all(np.diff(got[pos].astype(np.int64)) > 0)
    assert np.all(codes[got[:pos.max() + 1]] == 0)


def test_ties_keep_index_order_and_degenerate_boxes():
    # every triangle the same: one code, the identity order
    x = np.array([0.0, 1.0, 0.0], np.float32)
    y = np.array([0.0, 0.0, 1.0], np.float32)
    z = np.zeros(3, np.float32)
    idx = np.tile(np.array([0, 1, 2], np.uint32), (17, 1))
    assert np.array_equal(S.spatial_order(x, y, z, idx), np.arange(17, dtype=np.uint32))
    assert S.spatial_order(x, y, z, np.zeros((0, 3), np.uint32)).size == 0


def test_rejects_out_of_range_indices():
    x = y = z = np.zeros(3, np.float32)
    with pytest.raises(S.SlothError):
        S.spatial_order(x, y, z, np.array([[0, 1, 3]], np.uint32))


def test_neighbours_in_the_order_lie_close_together():
    m = W.displaced_icosphere(5, seed=3)
    x, y, z, idx = m["x"], m["y"], m["z"], m["idx"]
    cen = np.stack([x[idx].mean(1), y[idx].mean(1), z[idx].mean(1)], 1)
    step = lambda o: float(np.linalg.norm(np.diff(cen[o], axis=0), axis=1).mean())
    own = step(np.arange(idx.shape[0]))
    ordered = step(S.spatial_order(x, y, z, idx))
    assert ordered < own / 10, (ordered, own)
