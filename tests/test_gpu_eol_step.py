"""Stepping an EOL mesh on the GPU against the oracle (oracle/eol_ref.py):
the sheet lying on a box with its edge-line nodes as EOL nodes
(scenes.eol_edge_sheet), where the hanging half pulls material over the box
edge through the EOL nodes' Eulerian DOFs.

* eolc_cd2 on a topology with EOL nodes returns the oracle's contact set,
  bit for bit (CD2 sees the mesh nodes only, Collisions.cpp:55-78);
* eolc_velocity_solve_qp with the rows of eolc_constraint_rows (EOL
  equalities and inequalities, CD2 contact rows) equals the oracle's exact
  QP (FP64 within 1e-7 of max|v|, mixed within 1e-5), with its equality rows
  satisfied;
* consecutive eolc_step_eol steps track the oracle's Cloth::step of the EOL
  mesh — x, the material coordinates u of the EOL nodes and v in the
  reference's 3N + 2E layout (FP64 within 1e-7, mixed within 1e-5 of the
  largest velocity or displacement);
* the same with the EOL line's end nodes tagged as box-corner nodes and its
  middle node on a point obstacle (the corner and point branches of
  Constraints.cpp:148-262; the rows read only the tagged table column, so
  the box stays the one whose edges lie off the sheet: box edges crossing
  the cloth give edge-edge rows that depend on vertex-face rows, on which
  the augmented Lagrangian's multipliers converge too slowly);
* GeneralizedSolver.velocitySolve (eolc.py) with the reference's Aeq —
  pinned unit rows and the EOL rows together — equals the QP entry point;
* steps on a moving box (Box::v: a spin and a lift), whose rows carry the
  moving-obstacle right-hand sides, track the oracle (FP64 solved to rel_tol
  1e-10: the QP stops on its infeasibility, 10 rel_tol max|v|, which with
  non-zero right-hand sides leaves ~1e-6 of max|v| at rel_tol 1e-8);
* EOL steps with the topology rebuilt before every step (as after each
  remesh) equal the steps on one topology: bit for bit in FP64, within the
  solve tolerance in mixed precision (the resident solver's patches are cut
  from the material coordinates at the first solve after a topology change,
  and the EOL nodes' material coordinates move every step);
* a row on a padded Eulerian DOF is rejected.
"""
import numpy as np
import pytest

import eol_ref as R
import oracle as O
import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


def _setup(eolc, quads=10):
    s = scenes.eol_edge_sheet(quads)
    ctx = eolc.Context(0)
    ctx.set_topology_eol(s["n"], s["tri"], s["hinge"], s["eol"])
    ob = O.axis_box(s["box_center"], s["box_dim"])
    lb = eolc.Box(s["box_dim"], list(ob.E1))
    return s, ctx, ob, lb


def _rows_both(eolc, s, ctx, ob, lb, x, u):
    contacts = ctx.cd2(x, [lb], threshold=1e-3)
    E, I = eolc.constraint_rows(x, u, s["tri"], s["edges"], s["eol"], s["corner"], s["cd"],
                                s["preserve"], [lb], None, contacts)
    ref = R.constraint_rows(x, u, s["tri"], s["edges"], s["eol"], s["corner"], s["cd"],
                            s["preserve"], [ob], None, O.cd2(x, s["tri"], [ob], threshold=1e-3))
    return E, I, ref, contacts


def test_cd2_on_eol_topology_matches_oracle(eolc):
    s, ctx, ob, lb = _setup(eolc)
    rng = np.random.default_rng(5)
    x = s["x"] + rng.normal(0, 3e-4, s["x"].size)
    got = ctx.cd2(x, [lb], threshold=1e-3, raw=True)
    ref = O.cd2(x, s["tri"], [ob], threshold=1e-3, raw=True)
    assert len(got) > 0 and got == ref


@pytest.mark.parametrize("precision", [0, 1])
def test_qp_matches_oracle(eolc, precision):
    s, ctx, ob, lb = _setup(eolc)
    n, ne = s["n"], len(s["eol"])
    idx = eolc.eol_reference_index(n, ne)
    x, u = s["x"].copy(), s["X"].copy()
    # a state with motion: two oracle steps from rest
    v = np.zeros(3 * n + 2 * ne)
    mat_o, g, h = O.material(), scenes.GRAV, scenes.H
    for _ in range(2):
        rows = R.constraint_rows(x, u, s["tri"], s["edges"], s["eol"], s["corner"], s["cd"],
                                 s["preserve"], [ob], None, O.cd2(x, s["tri"], [ob], threshold=1e-3))
        R.step(x, u, v, s["tri"], s["hinge"], s["eol"], mat_o, g, h, s["fixed"], s["fixed_vel"],
               rows)
    E, I, ref, _ = _rows_both(eolc, s, ctx, ob, lb, x, u)
    Aeq, e, C, d = ref
    mat = eolc.Material(**scenes.material_c1())
    f, M, MDK = ctx.forces_fill(x, u, mat, g, h, precision)
    vx = np.zeros(3 * (n + ne))
    vx[idx] = v
    b = -(eolc.bsr_to_csr(ctx, M) @ vx + h * f)
    beq = 0.99 * v[s["fixed"]]
    F = O.ForcesEOL(x, u, s["tri"], s["hinge"], mat_o, g, h, s["eol"])
    b_ref = -(F.csr(0) @ v + h * F.f())
    vr, ler, lir, _ = R.solve_qp_eq(F.csr(1), b_ref, s["fixed"], beq, Aeq, e, C, d)
    opts = eolc.SolveOpts(precision=precision)
    vg, le, li, info = ctx.velocity_solve_qp(b, s["fixed"], beq, E, I, opts, v0=vx)
    assert info.status == eolc.OK
    vm = np.abs(vr).max()
    err = np.abs(vg[idx] - vr).max() / vm
    eq_viol = np.abs(Aeq @ vg[idx]).max() / vm
    print("precision %d: %d solves, %d iterations, %d active, v err %.2e, |Aeq v| %.2e"
          % (precision, info.solves, info.iterations, info.n_active, err, eq_viol))
    assert err <= (1e-7 if precision == 0 else 1e-5)
    assert eq_viol <= 1e-8
    assert not vg[3 * (n + np.arange(ne)) + 2].any()
    assert (li >= 0).all() and info.n_active == int((li > 0).sum())


@pytest.mark.parametrize("precision,precond", [(0, 0), (1, 0), (1, 3)])
def test_steps_track_oracle(eolc, precision, precond):
    s, ctx, ob, lb = _setup(eolc)
    n, ne = s["n"], len(s["eol"])
    idx = eolc.eol_reference_index(n, ne)
    mat, mat_o, g, h = eolc.Material(**scenes.material_c1()), O.material(), scenes.GRAV, scenes.H
    xg, ug, vg = s["x"].copy(), s["X"].copy(), np.zeros(3 * (n + ne))
    xo, uo, vo = s["x"].copy(), s["X"].copy(), np.zeros(3 * n + 2 * ne)
    tol = 1e-7 if precision == 0 else 1e-5
    opts = eolc.SolveOpts(precision=precision, precond=precond)  # Jacobi or patch PCG
    for k in range(4):
        E, I, _, _ = _rows_both(eolc, s, ctx, ob, lb, xg, ug)
        info = ctx.step_eol(xg, ug, vg, mat, g, h, s["fixed"], s["fixed_vel"], E, I, opts)
        assert info.status == eolc.OK
        rows = R.constraint_rows(xo, uo, s["tri"], s["edges"], s["eol"], s["corner"], s["cd"],
                                 s["preserve"], [ob], None,
                                 O.cd2(xo, s["tri"], [ob], threshold=1e-3))
        R.step(xo, uo, vo, s["tri"], s["hinge"], s["eol"], mat_o, g, h, s["fixed"],
               s["fixed_vel"], rows)
        vm = np.abs(vo).max()
        ev = np.abs(vg[idx] - vo).max() / vm
        ex = np.abs(xg - xo).max() / (h * vm)
        eu = np.abs(ug - uo).max() / (h * vm)
        print("step %d: %d ineq rows, %d active, %d solves, v %.2e x %.2e u %.2e"
              % (k, I.m, info.n_active, info.solves, ev, ex, eu))
        assert ev <= tol and ex <= tol and eu <= tol
    # material crossed the edge: the EOL nodes' u moved, nothing else did
    moved = np.flatnonzero(np.abs(ug - s["X"]).reshape(-1, 2).max(1) > 0)
    assert len(moved) > 0 and set(moved.tolist()) <= set(s["eol"].tolist())


@pytest.mark.parametrize("precision", [0, 1])
def test_corner_and_point_nodes_step(eolc, precision):
    s = scenes.eol_edge_sheet(10)
    n, ne = s["n"], len(s["eol"])
    idx = eolc.eol_reference_index(n, ne)
    ctx = eolc.Context(0)
    ctx.set_topology_eol(n, s["tri"], s["hinge"], s["eol"])
    ob = O.axis_box(s["box_center"], s["box_dim"])
    lb = eolc.Box(s["box_dim"], list(ob.E1))
    mid = ne // 2
    pts, nrm = s["x"].reshape(-1, 3)[s["eol"][mid]].copy(), np.array([0.0, 0.0, 1.0])
    corner = s["corner"].copy()
    # the line's ends on corners 5 (+x, -y, +z) and 7 (+x, +y, +z); the
    # point obstacle's column comes first
    corner[0], corner[-1], corner[mid] = 1 + 5, 1 + 7, 0
    cd = s["cd"] + 1
    mat, mat_o, g, h = eolc.Material(**scenes.material_c1()), O.material(), scenes.GRAV, scenes.H
    xg, ug, vg = s["x"].copy(), s["X"].copy(), np.zeros(3 * (n + ne))
    xo, uo, vo = s["x"].copy(), s["X"].copy(), np.zeros(3 * n + 2 * ne)
    tol = 1e-7 if precision == 0 else 1e-5
    kinds = set()
    for k in range(3):
        con = ctx.cd2(xg, [lb], points=pts, normals=nrm, threshold=1e-3)
        kinds |= {(c.count1, c.count2, c.source > 0) for c in con}
        E, I = eolc.constraint_rows(xg, ug, s["tri"], s["edges"], s["eol"], corner, cd,
                                    s["preserve"], [lb], nrm, con)
        info = ctx.step_eol(xg, ug, vg, mat, g, h, s["fixed"], s["fixed_vel"], E, I,
                            eolc.SolveOpts(precision=precision))
        assert info.status == eolc.OK
        co = O.cd2(xo, s["tri"], [ob], points=pts, normals=nrm, threshold=1e-3)
        rows = R.constraint_rows(xo, uo, s["tri"], s["edges"], s["eol"], corner, cd,
                                 s["preserve"], [ob], nrm, co)
        R.step(xo, uo, vo, s["tri"], s["hinge"], s["eol"], mat_o, g, h, s["fixed"],
               s["fixed_vel"], rows)
        vm = np.abs(vo).max()
        ev = np.abs(vg[idx] - vo).max() / vm
        ex = np.abs(xg - xo).max() / (h * vm)
        eu = np.abs(ug - uo).max() / (h * vm)
        print("step %d: %d eq, %d ineq rows, v %.2e x %.2e u %.2e" % (k, E.m, I.m, ev, ex, eu))
        assert ev <= tol and ex <= tol and eu <= tol
    assert {(3, 1, True), (1, 3, False)} <= kinds  # box vertex-face, point-face
    # the corner nodes' material coordinates move freely (no Eulerian row)
    assert np.abs(ug.reshape(-1, 2)[s["eol"][[0, -1]]] - s["X"].reshape(-1, 2)[s["eol"][[0, -1]]]).max() > 0


def test_generalized_solver_takes_eol_rows(eolc):
    s, ctx, ob, lb = _setup(eolc)
    n, ne = s["n"], len(s["eol"])
    mat = eolc.Material(**scenes.material_c1())
    x, u = s["x"].copy(), s["X"].copy()
    E, I, _, _ = _rows_both(eolc, s, ctx, ob, lb, x, u)
    forces = eolc.Forces(ctx, eolc.PREC_FP64)
    forces.fill(x, u, mat, scenes.GRAV, scenes.H)
    b = -scenes.H * forces.f
    nd = 3 * (n + ne)
    # the reference's Aeq: the EOL equality rows, then addFixed's unit rows
    import scipy.sparse as sp
    pins = sp.csr_matrix((np.ones(len(s["fixed"])), (np.arange(len(s["fixed"])), s["fixed"])),
                         shape=(len(s["fixed"]), nd))
    Aeq = sp.vstack([E.csr(nd), pins]).tocsr()
    beq = np.concatenate([E.rhs, np.zeros(len(s["fixed"]))])
    gs = eolc.GeneralizedSolver(ctx, eolc.SolveOpts(precision=0))
    v = np.zeros(nd)
    assert gs.velocitySolve(True, True, forces.MDK, b, Aeq, beq, I.csr(nd), I.rhs, v)
    vq, _, _, info = ctx.velocity_solve_qp(b, s["fixed"], np.zeros(len(s["fixed"])), E, I,
                                           eolc.SolveOpts(precision=0))
    assert info.status == eolc.OK
    assert np.abs(v - vq).max() <= 1e-12 * np.abs(vq).max()


@pytest.mark.parametrize("precision", [0, 1])
def test_steps_on_moving_box(eolc, precision):
    s, ctx, ob, lb = _setup(eolc)
    n, ne = s["n"], len(s["eol"])
    idx = eolc.eol_reference_index(n, ne)
    vel = np.array([0.0, 0.2, 0.0, 0.0, 0.0, 0.05])  # spin about y, lift 5 cm/s
    mat, mat_o, g, h = eolc.Material(**scenes.material_c1()), O.material(), scenes.GRAV, scenes.H
    xg, ug, vg = s["x"].copy(), s["X"].copy(), np.zeros(3 * (n + ne))
    xo, uo, vo = s["x"].copy(), s["X"].copy(), np.zeros(3 * n + 2 * ne)
    tol = 1e-7 if precision == 0 else 1e-5
    opts = eolc.SolveOpts(precision=precision, rel_tol=1e-10 if precision == 0 else 1e-8)
    for k in range(3):
        con = ctx.cd2(xg, [lb], threshold=1e-3, array=True)
        E, I = eolc.constraint_rows(xg, ug, s["tri"], s["edges"], s["eol"], s["corner"], s["cd"],
                                    s["preserve"], [lb], None, con, vel[None, :], h)
        assert np.abs(E.rhs).max() > 0 and np.abs(I.rhs).max() > 0
        info = ctx.step_eol(xg, ug, vg, mat, g, h, s["fixed"], s["fixed_vel"], E, I, opts)
        assert info.status == eolc.OK
        rows = R.constraint_rows(xo, uo, s["tri"], s["edges"], s["eol"], s["corner"], s["cd"],
                                 s["preserve"], [ob], None,
                                 O.cd2(xo, s["tri"], [ob], threshold=1e-3), vel[None, :], h)
        R.step(xo, uo, vo, s["tri"], s["hinge"], s["eol"], mat_o, g, h, s["fixed"],
               s["fixed_vel"], rows)
        vm = np.abs(vo).max()
        ev = np.abs(vg[idx] - vo).max() / vm
        ex = np.abs(xg - xo).max() / (h * vm)
        eu = np.abs(ug - uo).max() / (h * vm)
        print("moving box step %d: v %.2e x %.2e u %.2e" % (k, ev, ex, eu))
        assert ev <= tol and ex <= tol and eu <= tol


@pytest.mark.parametrize("precision", [0, 1])
def test_steps_after_topology_refresh(eolc, precision):
    s, ctx, ob, lb = _setup(eolc)
    n, ne = s["n"], len(s["eol"])
    mat, g, h = eolc.Material(**scenes.material_c1()), scenes.GRAV, scenes.H
    opts = eolc.SolveOpts(precision=precision)
    runs = []
    for refresh in (False, True):
        c = eolc.Context(0)
        c.set_topology_eol(n, s["tri"], s["hinge"], s["eol"])
        x, u, v = s["x"].copy(), s["X"].copy(), np.zeros(3 * (n + ne))
        for _ in range(3):
            if refresh:
                c.set_topology_eol(n, s["tri"], s["hinge"], s["eol"])
            con = c.cd2(x, [lb], threshold=1e-3, array=True)
            E, I = eolc.constraint_rows(x, u, s["tri"], s["edges"], s["eol"], s["corner"],
                                        s["cd"], s["preserve"], [lb], None, con)
            assert c.step_eol(x, u, v, mat, g, h, s["fixed"], s["fixed_vel"], E, I,
                              opts).status == eolc.OK
        runs.append((x, u, v))
    if precision == 0:
        for a, b in zip(*runs):
            assert np.array_equal(a, b)
    else:
        (x0, u0, v0), (x1, u1, v1) = runs
        vm = np.abs(v0).max()
        assert np.abs(v1 - v0).max() <= 1e-5 * vm
        assert max(np.abs(x1 - x0).max(), np.abs(u1 - u0).max()) <= 1e-5 * h * vm


def test_row_on_padded_dof_rejected(eolc):
    s, ctx, ob, lb = _setup(eolc, quads=6)
    n, ne = s["n"], len(s["eol"])
    mat = eolc.Material(**scenes.material_c1())
    f, M, MDK = ctx.forces_fill(s["x"], s["X"], mat, scenes.GRAV, scenes.H, 0)
    bad = eolc.RowSet([0, 1], [3 * n + 2], [1.0], [0.0])
    with pytest.raises(eolc.EolcError) as e:
        ctx.velocity_solve_qp(-scenes.H * f, s["fixed"], np.zeros(len(s["fixed"])), bad, None,
                              eolc.SolveOpts(precision=0))
    assert e.value.status == eolc.BAD_ARG
