"""The EOL assembly oracle (orc_forces_fill_eol, oracle/assemble.cpp) on the
CPU:

* with no EOL node it is bit-identical to the non-EOL fill;
* with EOL nodes its f, M and MDK over the 3N + 2E DOFs equal an
  independent dense assembly of T' E T from the oracle's element routines,
  where T maps a vertex's Eulerian DOFs to -F (the face's deformation
  gradient, or the mean of the two adjacent faces' for a hinge) — the
  transforms of fillEOLInertia / fillEOLMembrane / fillEOLBending
  (Forces.cpp:177-329, 580-683) — with the reference's quirk that a hinge
  touching an EOL node also adds its bending force.
"""
import numpy as np
import pytest

import oracle as O
import scenes


def _F(x, X, i0, i1, i2):
    Dx = np.stack([x[3 * i1:3 * i1 + 3] - x[3 * i0:3 * i0 + 3],
                   x[3 * i2:3 * i2 + 3] - x[3 * i0:3 * i0 + 3]], 1)
    DX = np.stack([X[2 * i1:2 * i1 + 2] - X[2 * i0:2 * i0 + 2],
                   X[2 * i2:2 * i2 + 2] - X[2 * i0:2 * i0 + 2]], 1)
    return Dx @ np.linalg.inv(DX)


def _upper(K, nv):
    """The element matrix as the reference reads it: upper blocks, mirrored."""
    U = K.copy()
    for v in range(nv):
        for w in range(v):
            U[3 * v:3 * v + 3, 3 * w:3 * w + 3] = K[3 * w:3 * w + 3, 3 * v:3 * v + 3].T
    return U


def _dense(x, X, tri, hinge, eol_nodes, mat, grav, h):
    n = len(x) // 3
    E = len(eol_nodes)
    idx = -np.ones(n, int)
    idx[eol_nodes] = np.arange(E)
    nd = 3 * n + 2 * E
    A = np.zeros((nd, nd)); M = np.zeros((nd, nd)); f = np.zeros(nd)
    dh2 = mat.damping_b * h * h

    def T_of(verts, F):
        T = np.zeros((3 * len(verts), nd))
        cols = []
        for a, v in enumerate(verts):
            T[3 * a:3 * a + 3, 3 * v:3 * v + 3] = np.eye(3)
            if idx[v] >= 0:
                c = 3 * n + 2 * idx[v]
                T[3 * a:3 * a + 3, c:c + 2] = -F
        return T

    for t in np.asarray(tri).reshape(-1, 3):
        x9 = np.concatenate([x[3 * v:3 * v + 3] for v in t])
        X6 = np.concatenate([X[2 * v:2 * v + 2] for v in t])
        P, Q = O.face_frame(x9, X6)
        _, fm, Km = O.membrane(x9, X6, mat.e, mat.nu, P, Q)
        _, fi, Mi = O.inertial(x9, X6, grav, mat.density)
        Km, Mi = _upper(Km.T, 3), _upper(Mi.T, 3)  # column-major reads
        T = T_of(t, _F(x, X, *t))
        A += T.T @ (Mi + dh2 * Km) @ T
        M += T.T @ Mi @ T
        f += T.T @ (fm + fi)
    for hg in np.asarray(hinge).reshape(-1, 4):
        x12 = np.concatenate([x[3 * v:3 * v + 3] for v in hg])
        X8 = np.concatenate([X[2 * v:2 * v + 2] for v in hg])
        _, fb, Kb = O.bending(x12, X8, mat.beta)
        Kb = _upper(Kb.T, 4)
        Fm = (_F(x, X, hg[0], hg[1], hg[2]) + _F(x, X, hg[0], hg[1], hg[3])) / 2
        T = T_of(hg, Fm)
        A += T.T @ (dh2 * Kb) @ T
        if (idx[hg] >= 0).any():
            f += T.T @ fb
    return f, M, A


def test_no_eol_is_the_plain_fill():
    s = scenes.sheet(6)
    x = s["x"] + np.random.default_rng(0).normal(0, 0.01, s["x"].size)
    a = O.Forces(x, s["X"], s["tri"], s["hinge"], O.material(), scenes.GRAV, scenes.H)
    b = O.ForcesEOL(x, s["X"], s["tri"], s["hinge"], O.material(), scenes.GRAV, scenes.H, [])
    for w in (0, 1):
        assert (a.csr(w) != b.csr(w)).nnz == 0
    assert np.array_equal(a.f(), b.f())


@pytest.mark.parametrize("seed", [1, 2])
def test_eol_fill_is_the_transformed_assembly(seed):
    s = scenes.sheet(5)
    rng = np.random.default_rng(seed)
    x = s["x"] + rng.normal(0, 0.02, s["x"].size)
    x[2::3] += rng.normal(0, 0.05, s["n"])
    eol = np.sort(rng.choice(s["n"], 9, replace=False))
    mat = O.material()
    F = O.ForcesEOL(x, s["X"], s["tri"], s["hinge"], mat, scenes.GRAV, scenes.H, eol)
    f, M, A = _dense(x, s["X"], s["tri"], s["hinge"], eol, mat, scenes.GRAV, scenes.H)
    rel = lambda p, q: np.abs(p - q).max() / np.abs(q).max()
    assert rel(F.csr(1).toarray(), A) <= 1e-12
    assert rel(F.csr(0).toarray(), M) <= 1e-12
    assert rel(F.f(), f) <= 1e-12
