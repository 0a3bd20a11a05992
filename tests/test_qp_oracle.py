"""The contact-QP oracle (oracle/qp_ref.py) on the CPU:

* on small random strictly convex QPs its active-set answer equals the one
  found by enumerating every active set (the KKT point is unique);
* on a drape snapshot with box contacts it satisfies the KKT conditions to
  round-off;
* the library's host-side row builder eolc_contact_rows produces exactly the
  oracle's restatement of Constraints.cpp:422-468.
"""
import ctypes
import itertools

import numpy as np
import pytest
import scipy.sparse as sp

import oracle as O
import qp_ref
import scenes


def _enumerate(A, b, C, d):
    """Exact minimiser by trying every active set (small m only)."""
    n, m = A.shape[0], C.shape[0]
    best = None
    for k in range(m + 1):
        for W in itertools.combinations(range(m), k):
            W = list(W)
            K = np.block([[A, C[W].T], [C[W], np.zeros((k, k))]]) if k else A
            try:
                sol = np.linalg.solve(K, np.concatenate([-b, d[W]]))
            except np.linalg.LinAlgError:
                continue
            v, lw = sol[:n], sol[n:]
            if (lw >= -1e-12).all() and (C @ v - d <= 1e-10).all():
                obj = 0.5 * v @ A @ v + b @ v
                if best is None or obj < best[0] - 1e-14:
                    best = (obj, v)
    return best[1]


@pytest.mark.parametrize("seed", range(6))
def test_active_set_matches_enumeration(seed):
    rng = np.random.default_rng(seed)
    n, m = 12, 5
    Q = rng.normal(size=(n, n))
    A = Q @ Q.T + n * np.eye(n)
    b = rng.normal(size=n) * 3
    C = rng.normal(size=(m, n))
    d = rng.normal(size=m) * 0.3
    v, lam, _ = qp_ref.solve_qp(sp.csr_matrix(A), b, [], [], sp.csr_matrix(C), d)
    ve = _enumerate(A, b, C, d)
    assert np.abs(v - ve).max() <= 1e-9 * max(1, np.abs(ve).max())
    assert (lam >= 0).all()


def _drape_problem(quads=24, snap=14, seed=0):
    x0, X, tri, center, snaps = scenes.drape_positions(quads, 40)
    x = snaps[snap]
    n = len(x) // 3
    hinge = O.hinges(n, tri)
    box = O.axis_box(center, (0.4, 0.4, 0.2))
    cons = O.cd2(x, tri, [box], threshold=1e-3)
    F = O.Forces(x, X, tri, hinge, O.material(), scenes.GRAV, scenes.H)
    rng = np.random.default_rng(seed)
    v = rng.normal(0, 0.05, 3 * n)
    v[2::3] -= 0.5
    return F, F.rhs(v, scenes.H), cons, n


def test_oracle_kkt_on_drape_contacts():
    F, b, cons, n = _drape_problem()
    C, d = qp_ref.contact_rows(cons, n)
    assert C.shape[0] > 20
    A = F.csr(1)
    v, lam, _ = qp_ref.solve_qp(A, b, [], [], C, d)
    stat, feas, comp = qp_ref.kkt_residuals(A, b, [], v, C, d, lam)
    assert stat <= 1e-9 and feas <= 1e-12 and comp <= 1e-9, (stat, feas, comp)
    assert (lam > 0).sum() > 0


def test_contact_rows_match_oracle():
    import eolc
    F, b, cons, n = _drape_problem(snap=9)
    F2, b2, cons2, _ = _drape_problem(snap=14)
    cons = list(cons) + list(cons2)
    kinds = {(c.count1, c.count2) for c in cons}
    assert {(1, 3), (2, 2), (3, 1)} <= kinds
    C_ref, d_ref = qp_ref.contact_rows(cons, n)
    # the oracle's contacts re-typed as the library's struct (same layout)
    lib_cons = [eolc.Contact.from_buffer_copy(bytes(c)) for c in cons]
    C, d = eolc.contact_rows(lib_cons, n)
    # same rows (column order inside a row is immaterial)
    C, C_ref = C.copy(), C_ref.copy()
    C.sort_indices()
    C_ref.sort_indices()
    assert C.shape == C_ref.shape
    assert np.array_equal(C.indptr, C_ref.indptr)
    assert np.array_equal(C.indices, C_ref.indices)
    assert np.array_equal(C.data, C_ref.data)
    assert np.array_equal(d, d_ref)


def test_contact_rows_capacity_and_kinds():
    """eolc_contact_rows (host only): rows only for the three kinds of
    Constraints.cpp:422-468, in contact order, and EOLC_CAPACITY with the
    needed count when the buffers are short."""
    import ctypes
    import eolc
    F, b, cons, n = _drape_problem(snap=9)
    cons = list(cons)
    lib_cons = [eolc.Contact.from_buffer_copy(bytes(c)) for c in cons]
    odd = eolc.Contact.from_buffer_copy(bytes(cons[0]))
    odd.count1, odd.count2 = 2, 1  # no row for this kind
    lib_cons.insert(1, odd)
    C, d = eolc.contact_rows(lib_cons, n)
    assert C.shape[0] == len(cons)
    arr = (eolc.Contact * len(lib_cons))(*lib_cons)
    ptr = np.zeros(3, np.int32)
    col = np.zeros(18, np.int32)
    val = np.zeros(18)
    dd = np.zeros(2)
    m = ctypes.c_int()
    st = eolc.lib.eolc_contact_rows(ctypes.cast(arr, ctypes.c_void_p), len(lib_cons), 2,
                                    eolc._i(ptr), eolc._i(col), eolc._d(val), eolc._d(dd),
                                    ctypes.byref(m))
    assert st == eolc.CAPACITY and m.value == len(cons)
    assert ptr[0] == 0 and ptr[1] > 0  # the rows that fit are written
