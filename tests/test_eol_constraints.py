"""Constraints::fill for EOL meshes on the CPU (Constraints.cpp:135-468):

* the library's host-side row builder eolc_constraint_rows produces the
  oracle's restatement (oracle/eol_ref.py) row for row, in the reference's
  order, on the box-edge sheet in every branch — locally flat and bent edge
  nodes, boundary and interior Eulerian rows, corner and point-obstacle
  nodes (flat and bent), rotated boxes, CD2 contact rows with the EOL nodes'
  contacts skipped;
* it reports capacity and rejects bad tables;
* the oracle's QP with equality rows (solve_qp_eq) equals the minimiser found
  by enumerating active sets on small random QPs, and an oracle EOL step
  keeps its equality rows and contacts.
"""
import itertools

import numpy as np
import pytest

import eol_ref as R
import eolc
import oracle as O
import scenes


def _boxes(s, rot=0.0):
    """The scene's box as (oracle Box, library Box); rot: rotation about z
    applied to the frame (the rows only read the table, so any frame will do
    for the builders' comparison)."""
    E1 = np.eye(4)
    c, sn = np.cos(rot), np.sin(rot)
    E1[:3, :3] = [[c, -sn, 0], [sn, c, 0], [0, 0, 1]]
    E1[:3, 3] = s["box_center"]
    flat = list(E1.flatten(order="F"))
    ob = O.axis_box(s["box_center"], s["box_dim"])
    for k in range(16):
        ob.E1[k] = flat[k]
    return ob, eolc.Box(s["box_dim"], flat)


def _compare(s, x, u, corner, cd, preserve, rot=0.0, point_normals=None, contacts=()):
    ob, lb = _boxes(s, rot)
    Aeq, beq, C, d = R.constraint_rows(x, u, s["tri"], s["edges"], s["eol"], corner, cd, preserve,
                                       [ob], point_normals, contacts)
    lc = [eolc.Contact.from_buffer_copy(bytes(c)) for c in contacts]
    E, I = eolc.constraint_rows(x, u, s["tri"], s["edges"], s["eol"], corner, cd, preserve,
                                [lb], point_normals, lc)
    n, ne = s["n"], len(s["eol"])
    idx = eolc.eol_reference_index(n, ne)
    nd = 3 * (n + ne)
    Eg, Ig = E.csr(nd)[:, idx], I.csr(nd)[:, idx]
    assert (E.m, I.m) == (Aeq.shape[0], C.shape[0])
    tol = 1e-15
    assert np.abs((Eg - Aeq).toarray()).max(initial=0.0) <= tol
    assert np.abs((Ig - C).toarray()).max(initial=0.0) <= tol
    assert not E.rhs.any() and not I.rhs.any()
    # no row of the builder touches a padded Eulerian DOF
    pad = set((3 * (n + np.arange(ne)) + 2).tolist())
    assert not pad & set(E.col.tolist()) and not pad & set(I.col.tolist())
    return Aeq, C


def test_rows_flat_sheet_on_box_edge():
    s = scenes.eol_edge_sheet(10)
    ob, _ = _boxes(s)
    contacts = O.cd2(s["x"], s["tri"], [ob], threshold=1e-3)
    Aeq, C = _compare(s, s["x"], s["X"], s["corner"], s["cd"], s["preserve"], contacts=contacts)
    ne = len(s["eol"])
    # flat edge nodes: one node-normal inequality and one flat equality each,
    # plus one Eulerian equality; the EOL nodes' contacts are skipped
    assert Aeq.shape[0] == 2 * ne
    n_kept = sum(1 for c in contacts if c.verts2[0] not in set(s["eol"].tolist()))
    assert C.shape[0] == ne + n_kept
    assert n_kept < len(contacts)
    # the contacts as one ctypes array (eolc Context.cd2(array=True)) give the same rows
    lc = [eolc.Contact.from_buffer_copy(bytes(c)) for c in contacts]
    arr = (eolc.Contact * len(lc))(*lc)
    _, lb = _boxes(s)
    E1, I1 = eolc.constraint_rows(s["x"], s["X"], s["tri"], s["edges"], s["eol"], s["corner"],
                                  s["cd"], s["preserve"], [lb], None, lc)
    E2, I2 = eolc.constraint_rows(s["x"], s["X"], s["tri"], s["edges"], s["eol"], s["corner"],
                                  s["cd"], s["preserve"], [lb], None, arr)
    for a, b in ((E1, E2), (I1, I2)):
        assert all(np.array_equal(p, q) for p, q in
                   ((a.ptr, b.ptr), (a.col, b.col), (a.val, b.val), (a.rhs, b.rhs)))


# jitter amplitudes that bend 11, 1 and 7 of the 11 EOL nodes past 0.1 rad
@pytest.mark.parametrize("seed,amp", [(1, 0.02), (2, 0.002), (3, 0.004)])
def test_rows_bent_nodes_and_interior_directions(seed, amp):
    s = scenes.eol_edge_sheet(10)
    rng = np.random.default_rng(seed)
    x = s["x"] + rng.normal(0, amp, s["x"].size)
    u = s["X"] + rng.normal(0, 0.01, s["X"].size)     # interior directions differ
    pres = (rng.random(len(s["edges"])) < 0.3).astype(np.int32) | s["preserve"]
    _compare(s, x, u, s["corner"], s["cd"], pres, rot=0.3 * seed)


@pytest.mark.parametrize("bend", [0.0, 0.05])
def test_rows_corner_and_point_nodes(bend):
    s = scenes.eol_edge_sheet(10)
    rng = np.random.default_rng(4)
    x = s["x"] + rng.normal(0, bend, s["x"].size)
    ne = len(s["eol"])
    pn = np.array([[0.0, 0.0, 1.0], [0.6, 0.0, 0.8]])
    corner = -np.ones(ne, np.int32)
    corner[0], corner[1], corner[ne - 1] = 0, 1, 2 + 3     # two points, one box corner
    cd = s["cd"] + 2                                        # two point columns come first
    Aeq, C = _compare(s, x, s["X"], corner, cd, s["preserve"], rot=0.7, point_normals=pn)
    assert Aeq.shape[0] > 0 and C.shape[0] > 0


def test_rows_capacity_and_bad_arguments():
    s = scenes.eol_edge_sheet(6)
    ne = len(s["eol"])
    x, u = eolc._f64(s["x"]), eolc._f64(s["X"])
    tri, edges = eolc._i32(s["tri"]), eolc._i32(s["edges"])
    eol, corner, cd = eolc._i32(s["eol"]), eolc._i32(s["corner"]), eolc._i32(s["cd"])
    pres = eolc._i32(s["preserve"])
    _, lb = _boxes(s)
    barr = (eolc.Box * 1)(lb)

    def call(cap_e, cap_i, cd_arr=cd):
        mesh = eolc.EolMesh(s["n"], eolc._d(x), eolc._d(u), eolc._i(tri), len(tri),
                            eolc._i(edges), eolc._i(pres), len(edges), eolc._i(eol),
                            eolc._i(corner), eolc._i(cd_arr), ne)
        bufs = []
        for cap in (cap_e, cap_i):
            a = (np.zeros(cap + 1, np.int32), np.zeros(9 * max(cap, 1), np.int32),
                 np.zeros(9 * max(cap, 1)), np.zeros(max(cap, 1)))
            bufs.append((eolc.Rows(0, cap, eolc._i(a[0]), eolc._i(a[1]), eolc._d(a[2]),
                                   eolc._d(a[3])), a))
        st = eolc.lib.eolc_constraint_rows(mesh, barr, None, 1, None, 0, None, 0, 0.0, bufs[0][0],
                                           bufs[1][0])
        return st, bufs[0][0].n_rows, bufs[1][0].n_rows, bufs

    st, me, mi, _ = call(100, 100)
    assert st == eolc.OK and (me, mi) == (2 * ne, ne)
    st, me2, mi2, bufs = call(3, 100)
    assert st == eolc.CAPACITY and (me2, mi2) == (me, mi)
    assert bufs[0][1][0][3] > 0                 # the rows that fit are written
    st, *_ = call(100, 100, eolc._i32(np.full(ne, 20, np.int32)))  # one box: columns 0..19
    assert st == eolc.BAD_ARG


def _enumerate_eq(A, b, E, e, C, d):
    n, m, me = A.shape[0], C.shape[0], E.shape[0]
    best = None
    for k in range(m + 1):
        for W in itertools.combinations(range(m), k):
            G = np.vstack([E, C[list(W)]])
            K = np.block([[A, G.T], [G, np.zeros((len(G), len(G)))]])
            sol = np.linalg.solve(K, np.concatenate([-b, e, d[list(W)]]))
            v, lw = sol[:n], sol[n + me:]
            if (lw >= -1e-12).all() and (C @ v - d <= 1e-10).all():
                obj = 0.5 * v @ A @ v + b @ v
                if best is None or obj < best[0] - 1e-14:
                    best = (obj, v)
    return best[1]


@pytest.mark.parametrize("seed", range(6))
def test_qp_with_equality_rows_matches_enumeration(seed):
    rng = np.random.default_rng(seed)
    n, me, m = 9, 2, 5
    B = rng.normal(size=(n, n))
    A = B @ B.T + 0.5 * np.eye(n)
    b = rng.normal(size=n)
    E, e = rng.normal(size=(me, n)), rng.normal(size=me)
    C, d = rng.normal(size=(m, n)), rng.normal(size=m) * 0.3
    v, le, li, _ = R.solve_qp_eq(A, b, [], [], E, e, C, d)
    ve = _enumerate_eq(A, b, E, e, C, d)
    assert np.abs(v - ve).max() <= 1e-10 * max(1.0, np.abs(ve).max())
    assert np.abs(E @ v - e).max() <= 1e-10
    assert np.abs(A @ v + b + E.T @ le + C.T @ li).max() <= 1e-9
    assert (li >= 0).all()


def test_oracle_eol_step_keeps_rows():
    s = scenes.eol_edge_sheet(8)
    ob, _ = _boxes(s)
    x, u = s["x"].copy(), s["X"].copy()
    n, ne = s["n"], len(s["eol"])
    v = np.zeros(3 * n + 2 * ne)
    mat, g, h = O.material(), scenes.GRAV, scenes.H
    for _ in range(3):
        contacts = O.cd2(x, s["tri"], [ob], threshold=1e-3)
        rows = R.constraint_rows(x, u, s["tri"], s["edges"], s["eol"], s["corner"], s["cd"],
                                 s["preserve"], [ob], None, contacts)
        u0 = u.copy()
        R.step(x, u, v, s["tri"], s["hinge"], s["eol"], mat, g, h, s["fixed"], s["fixed_vel"],
               rows)
        Aeq, _, C, _ = rows
        vm = np.abs(v).max()
        assert np.abs(Aeq @ v).max() <= 1e-10 * vm
        assert (C @ v).max() <= 1e-10 * vm
        # only the EOL nodes' material coordinates move
        moved = np.flatnonzero(np.abs(u - u0).reshape(-1, 2).max(1) > 0)
        assert set(moved.tolist()) <= set(s["eol"].tolist())
    assert np.abs(v[3 * n:]).max() > 0  # material flows across the edge


def test_constraints_mirror_builds_the_reference_rows():
    """eolc.Constraints.fill: the EOL equalities then the pins' unit rows in
    Aeq (beq = 0.99 v + c), the EOL inequalities then the contact rows in
    Aineq, all in the extended layout."""
    s = scenes.eol_edge_sheet(8)
    ob, lb = _boxes(s)
    rng = np.random.default_rng(9)
    x = s["x"] + rng.normal(0, 1e-3, s["x"].size)
    n, ne = s["n"], len(s["eol"])
    v = rng.normal(0, 0.1, 3 * (n + ne))
    fvel = rng.normal(0, 0.01, len(s["fixed"]))
    con = O.cd2(x, s["tri"], [ob], threshold=1e-3)
    lc = [eolc.Contact.from_buffer_copy(bytes(c)) for c in con]
    C = eolc.Constraints(None).fill(x, s["X"], v, s["tri"], s["edges"], s["eol"], s["corner"],
                                    s["cd"], s["preserve"], [lb], fixed_dofs=s["fixed"],
                                    fixed_vel=fvel, contacts=lc)
    Aeq, _, Ai, _ = R.constraint_rows(x, s["X"], s["tri"], s["edges"], s["eol"], s["corner"],
                                      s["cd"], s["preserve"], [ob], None, con)
    idx = eolc.eol_reference_index(n, ne)
    me = Aeq.shape[0]
    assert C.Aeq.shape[0] == me + len(s["fixed"]) and C.hasFixed and C.hasCollisions
    assert np.abs((C.Aeq[:me][:, idx] - Aeq).toarray()).max() <= 1e-15
    pins = C.Aeq[me:].toarray()
    assert (pins[np.arange(len(s["fixed"])), s["fixed"]] == 1).all() and pins.sum() == len(s["fixed"])
    assert np.array_equal(C.beq[me:], 0.99 * v[s["fixed"]] + fvel)
    assert np.abs((C.Aineq[:, idx] - Ai).toarray()).max() <= 1e-15


@pytest.mark.parametrize("amp", [0.0, 0.004, 0.05])
def test_rows_on_moving_boxes(amp):
    """Boxes with Box::v (spinning and translating): the right-hand sides of
    Constraints.cpp:165-172 and :270-277 on edge nodes (flat and bent) and
    corner nodes (flat and bent), against the oracle's Rigid::integrate and
    point velocities; a box at rest keeps zero right-hand sides."""
    s = scenes.eol_edge_sheet(10)
    rng = np.random.default_rng(11)
    x = s["x"] + rng.normal(0, amp, s["x"].size)
    ne = len(s["eol"])
    corner = s["corner"].copy()
    corner[0], corner[-1] = 20 + 5, 20 + 7           # corners of the second box
    cd = s["cd"].copy()
    ob0, lb0 = _boxes(s, rot=0.2)
    ob1, lb1 = _boxes(s, rot=-0.4)
    vel = np.array([[0.3, -0.2, 0.5, 0.05, 0.02, -0.1],   # box 0: spin and drift
                    [0.0, 0.0, 0.0, 0.0, 0.0, 0.2]])      # box 1: translation only
    h = scenes.H
    Aeq, beq, Ai, bi = R.constraint_rows(x, s["X"], s["tri"], s["edges"], s["eol"], corner, cd,
                                         s["preserve"], [ob0, ob1], None, (), vel, h)
    E, I = eolc.constraint_rows(x, s["X"], s["tri"], s["edges"], s["eol"], corner, cd,
                                s["preserve"], [lb0, lb1], None, (), vel, h)
    idx = eolc.eol_reference_index(s["n"], ne)
    nd = 3 * (s["n"] + ne)
    assert np.abs((E.csr(nd)[:, idx] - Aeq).toarray()).max() <= 1e-15
    assert np.abs((I.csr(nd)[:, idx] - Ai).toarray()).max() <= 1e-15
    scale = max(np.abs(beq).max(), np.abs(bi).max())
    assert scale > 0.01                                # the motion reaches the rows
    assert np.abs(E.rhs - beq).max() <= 1e-13 * scale
    assert np.abs(I.rhs - bi).max() <= 1e-13 * scale
    # the same boxes at rest: zero right-hand sides
    E0, I0 = eolc.constraint_rows(x, s["X"], s["tri"], s["edges"], s["eol"], corner, cd,
                                  s["preserve"], [lb0, lb1], None, (), np.zeros((2, 6)), h)
    assert not E0.rhs.any() and not I0.rhs.any()


def test_rigid_integrate_matches_the_exponential_map():
    """The oracle's Rigid::integrate is the rigid motion exp(h [w v]) applied
    after E0 (checked against scipy's matrix exponential of the twist)."""
    import scipy.linalg as sl
    rng = np.random.default_rng(2)
    for _ in range(5):
        phi = rng.normal(size=6)
        E0 = np.eye(4)
        E0[:3, :3] = sl.expm(np.cross(np.eye(3), rng.normal(size=3)))
        E0[:3, 3] = rng.normal(size=3)
        w, v = phi[:3], phi[3:]
        T = np.zeros((4, 4))
        T[:3, :3] = np.cross(np.eye(3), w)
        T[:3, 3] = v
        h = 0.01
        assert np.abs(R.rigid_integrate(E0, phi, h) - E0 @ sl.expm(h * T)).max() <= 1e-12


def test_rows_of_the_flat_box_edge_sheet_by_hand():
    """The rows Constraints.cpp:263-403 give on a flat 4x4-quad sheet whose
    middle node column lies on the +x/+z edge of an axis-aligned box, worked
    out by hand from the reference's expressions: every EOL node is flat
    (all normals +z), so it gets the inequality -n = (0, 0, -1) and the
    equality -(n x t) = (1, 0, 0) with t = +y (the edge's third table
    direction); the Eulerian row is (0, -1) at the two boundary nodes (the
    border expression with the first boundary edge, (u_y - u'_y, -u_x - u'_x)
    normalised) and at the interior ones (the preserved edges' unit
    directions toward the end nearer the material origin, summed and
    normalised).  Both the library and the oracle must give exactly these."""
    s = scenes.eol_edge_sheet(4)
    n, ne = s["n"], len(s["eol"])
    nd = 3 * (n + ne)
    eq = np.zeros((2 * ne, nd))
    iq = np.zeros((ne, nd))
    for k, a in enumerate(s["eol"]):
        eq[2 * k, 3 * a] = 1.0                      # -(n x t) on the node
        eq[2 * k + 1, 3 * (n + k) + 1] = -1.0       # the Eulerian row (0, -1)
        iq[k, 3 * a + 2] = -1.0                     # -n on the node
    ob, lb = _boxes(s)
    E, I = eolc.constraint_rows(s["x"], s["X"], s["tri"], s["edges"], s["eol"], s["corner"],
                                s["cd"], s["preserve"], [lb], None, ())
    assert np.array_equal(E.csr(nd).toarray(), eq)
    assert np.array_equal(I.csr(nd).toarray(), iq)
    Aeq, _, Ai, _ = R.constraint_rows(s["x"], s["X"], s["tri"], s["edges"], s["eol"], s["corner"],
                                      s["cd"], s["preserve"], [ob], None, ())
    idx = eolc.eol_reference_index(n, ne)
    assert np.array_equal(Aeq.toarray(), eq[:, idx])
    assert np.array_equal(Ai.toarray(), iq[:, idx])


def test_corner_rows_by_hand():
    """A flat node tagged with corner 5 (+x, -y, +z) of an axis-aligned box
    (Constraints.cpp:148-215): the table normal nor = (1, -1, 1)/sqrt(3) as
    the inequality -nor, and the equalities o1 = (0, -nor_z, nor_y) =
    (0, -1, -1)/sqrt(3) and o2 = (o1 x nor)/|o1 x nor| = (-2, -1, 1)/sqrt(6);
    no Eulerian row."""
    s = scenes.eol_edge_sheet(4)
    n, ne = s["n"], len(s["eol"])
    corner = s["corner"].copy()
    corner[0] = 5
    _, lb = _boxes(s)
    E, I = eolc.constraint_rows(s["x"], s["X"], s["tri"], s["edges"], s["eol"], corner, s["cd"],
                                s["preserve"], [lb], None, ())
    a = int(s["eol"][0])
    nd = 3 * (n + ne)
    Ed, Id = E.csr(nd).toarray(), I.csr(nd).toarray()
    r3, r6 = 1 / np.sqrt(3), 1 / np.sqrt(6)
    assert np.abs(Id[0, 3 * a:3 * a + 3] - [-r3, r3, -r3]).max() <= 1e-15
    assert np.abs(Ed[0, 3 * a:3 * a + 3] - [0, -r3, -r3]).max() <= 1e-15
    assert np.abs(Ed[1, 3 * a:3 * a + 3] - [-2 * r6, -r6, r6]).max() <= 1e-15
    assert not Ed[:2, 3 * n:].any()               # the corner node has no Eulerian row
    assert E.m == 2 * ne and I.m == ne            # 2 + 1 rows for it and for each other
