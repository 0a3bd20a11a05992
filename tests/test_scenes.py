"""The synthetic workloads themselves (no GPU): sizes, orientation, pins."""
import numpy as np

import scenes


def test_delaunay_sheet_is_a_valid_oriented_mesh():
    rng = np.random.default_rng(0)
    for n_tri in (600, 5000):
        s = scenes.delaunay_sheet(n_tri, rng)
        tri, X = s["tri"], s["X"].reshape(-1, 2)
        assert 0.8 * n_tri <= len(tri) <= 1.25 * n_tri
        a, b, c = X[tri[:, 0]], X[tri[:, 1]], X[tri[:, 2]]
        area = 0.5 * ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))
        assert (area > 0).all()
        assert abs(area.sum() - 1.0) < 1e-9          # the triangles tile the square
        assert len(np.unique(tri)) == s["n"]          # every node is used
        assert X.min() >= 0 and X.max() <= 1
        corners = s["fixed"][::3] // 3
        assert np.allclose(X[corners], [[0, 1], [1, 1]])
        # the density grows along x: more nodes in the right half
        assert (X[:, 0] > 0.5).sum() > 1.3 * (X[:, 0] < 0.5).sum()
        h = s["hinge"]
        assert len(h) > 0 and h.min() >= 0 and h.max() < s["n"]


def test_delaunay_batch_layout():
    B = scenes.delaunay_batch(3, tri_lo=300, tri_hi=900, seed=1)
    off = B["node_off"]
    assert len(off) == 4 and off[-1] * 3 == B["x"].size == B["v"].size
    for k, s in enumerate(B["sheets"]):
        f = B["fixed"][6 * k:6 * k + 6]
        assert np.array_equal(f, s["fixed"] + 3 * off[k])
