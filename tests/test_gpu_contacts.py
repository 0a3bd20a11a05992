"""Contact-constrained velocity solve on the GPU (eolc_velocity_solve_ineq)
against the exact QP oracle (oracle/qp_ref.py): the minimiser of
1/2 v'MDK v + b'v with pinned DOFs and the contact rows of
Constraints.cpp:422-468 built from the library's own CD2 contacts.

Tolerances: the QP minimiser is unique, so v is compared directly — FP64
path 1e-7 relative (linear solves to rel-res 1e-10), mixed path 1e-5 (FP32
matrix); the multipliers of the FP64 path within 1e-5 of the largest; every
answer feasible to the solver's own stopping bound.
"""
import numpy as np
import pytest

import oracle as O
import qp_ref
import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


def _problem(eolc, quads, snap, precision, pins=False, seed=0):
    x0, X, tri, center, snaps = scenes.drape_positions(quads, 40)
    x = snaps[snap]
    n = len(x) // 3
    hinge = O.hinges(n, tri)
    ctx = eolc.Context(0)
    ctx.set_topology(n, tri, hinge)
    mat = eolc.Material(**scenes.material_c1())
    f, M, MDK = ctx.forces_fill(x, X, mat, scenes.GRAV, scenes.H, precision)
    box = O.axis_box(center, (0.4, 0.4, 0.2))
    cons = ctx.cd2(x, boxes=[eolc.Box(box.dim, box.E1)], threshold=1e-3)
    C, d = eolc.contact_rows(cons, n)
    F = O.Forces(x, X, tri, hinge, O.material(), scenes.GRAV, scenes.H)
    rng = np.random.default_rng(seed)
    v = rng.normal(0, 0.05, 3 * n)
    v[2::3] -= 0.5
    b = F.rhs(v, scenes.H)
    if pins:
        ids = O.corner_ids(quads + 1, quads + 1)
        fixed = np.array([3 * ids[k] + c for k in (3, 4) for c in range(3)], np.int32)
        beq = 0.99 * v[fixed]
    else:
        fixed, beq = np.zeros(0, np.int32), np.zeros(0)
    A = eolc.bsr_to_csr(ctx, MDK)  # the matrix the GPU solves with
    return ctx, A, b, fixed, beq, C, d, cons


def _relmax(a, b):
    return np.abs(a - b).max() / max(1e-300, np.abs(b).max())


@pytest.mark.parametrize("snap,pins", [(14, False), (9, True), (24, True)])
def test_fp64_matches_exact_qp(eolc, snap, pins):
    ctx, A, b, fixed, beq, C, d, cons = _problem(eolc, 24, snap, eolc.PREC_FP64, pins)
    assert C.shape[0] > 20
    opts = eolc.SolveOpts(rel_tol=1e-10, precision=eolc.PREC_FP64)
    v, lam, info = ctx.velocity_solve_ineq(b, fixed, beq, C, d, opts)
    vo, lo, _ = qp_ref.solve_qp(A, b, fixed, beq, C, d)
    print("rows %d active %d (oracle %d), solves %d, updates %d, PCG iterations %d, "
          "v err %.2e, lambda err %.2e, violation %.1e"
          % (C.shape[0], info.n_active, (lo > 0).sum(), info.solves, info.outer, info.iterations,
             _relmax(v, vo), np.abs(lam - lo).max() / lo.max(), info.max_violation))
    assert info.status == eolc.OK
    assert _relmax(v, vo) <= 1e-7
    assert np.abs(lam - lo).max() <= 1e-5 * lo.max()
    assert info.max_violation <= 1e-9
    assert (lam >= 0).all()
    if len(fixed):
        assert np.array_equal(v[fixed], beq)


@pytest.mark.parametrize("precond", [0, 1, 2, 3])
def test_mixed_matches_exact_qp(eolc, precond):
    ctx, A, b, fixed, beq, C, d, cons = _problem(eolc, 24, 24, eolc.PREC_MIXED, True)
    if precond == eolc.PC_LEARNED:
        import os
        lpc = eolc.LearnedPC(0, seed=1)
        w = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                         "eol-cloth_gb300", "weights", "lpc.npy")
        if os.path.exists(w):
            lpc.set_params(np.load(w))
        lpc.attach(ctx)
    opts = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED, precond=precond,
                          fallback_factor=0)
    v, lam, info = ctx.velocity_solve_ineq(b, fixed, beq, C, d, opts)
    vo, lo, _ = qp_ref.solve_qp(A, b, fixed, beq, C, d)
    print("precond %d: solves %d, updates %d, PCG iterations %d, v err %.2e"
          % (precond, info.solves, info.outer, info.iterations, _relmax(v, vo)))
    assert info.status == eolc.OK
    assert _relmax(v, vo) <= 1e-5
    assert info.max_violation <= 1e-7


def test_without_rows_equals_plain_solve(eolc):
    ctx, A, b, fixed, beq, C, d, cons = _problem(eolc, 16, 12, eolc.PREC_FP64, True)
    opts = eolc.SolveOpts(rel_tol=1e-10, precision=eolc.PREC_FP64)
    empty = (np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    v, lam, info = ctx.velocity_solve_ineq(b, fixed, beq, empty, np.zeros(0), opts)
    v2, _ = ctx.velocity_solve(b, fixed, beq, opts)
    assert info.status == eolc.OK and info.solves == 1
    assert _relmax(v, v2) <= 1e-9


def test_inactive_rows_change_nothing(eolc):
    """Rows that the unconstrained solution satisfies strictly leave it as is."""
    ctx, A, b, fixed, beq, C, d, cons = _problem(eolc, 16, 12, eolc.PREC_FP64, True)
    opts = eolc.SolveOpts(rel_tol=1e-10, precision=eolc.PREC_FP64)
    v0, _ = ctx.velocity_solve(b, fixed, beq, opts)
    dd = C @ v0 + 1.0  # slack of 1 on every row
    v, lam, info = ctx.velocity_solve_ineq(b, fixed, beq, C, dd, opts)
    assert info.status == eolc.OK and info.n_active == 0
    assert not lam.any()
    assert _relmax(v, v0) <= 1e-8  # two solves to rel-res 1e-10


def test_results_are_reproducible(eolc):
    ctx, A, b, fixed, beq, C, d, cons = _problem(eolc, 24, 14, eolc.PREC_MIXED, False)
    opts = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED)
    r1 = ctx.velocity_solve_ineq(b, fixed, beq, C, d, opts)
    r2 = ctx.velocity_solve_ineq(b, fixed, beq, C, d, opts)
    assert np.array_equal(r1[0], r2[0]) and np.array_equal(r1[1], r2[1])


def test_rows_outside_the_pattern_are_rejected(eolc):
    ctx, A, b, fixed, beq, C, d, cons = _problem(eolc, 16, 12, eolc.PREC_FP64, False)
    n = A.shape[0] // 3
    import scipy.sparse as sp
    bad = sp.csr_matrix(([1.0, -1.0], ([0, 0], [0, 3 * (n - 1)])), shape=(1, 3 * n))
    with pytest.raises(eolc.EolcError) as e:
        ctx.velocity_solve_ineq(b, fixed, beq, bad, np.zeros(1),
                                eolc.SolveOpts(precision=eolc.PREC_FP64))
    assert e.value.status == eolc.BAD_ARG


def test_generalized_solver_with_collisions(eolc):
    """The reference-facing velocitySolve(fixed, collisions, ...) routes the
    contact rows to the QP solve."""
    ctx, A, b, fixed, beq, C, d, cons = _problem(eolc, 24, 14, eolc.PREC_MIXED, True)
    import scipy.sparse as sp
    Aeq = sp.csr_matrix((np.ones(len(fixed)), (np.arange(len(fixed)), fixed)),
                        shape=(len(fixed), A.shape[0]))
    gs = eolc.GeneralizedSolver(ctx, eolc.SolveOpts(precision=eolc.PREC_MIXED))
    v = np.zeros(A.shape[0])
    assert gs.velocitySolve(True, True, None, b, Aeq, beq, C, d, v)
    vo, lo, _ = qp_ref.solve_qp(A, b, fixed, beq, C, d)
    assert _relmax(v, vo) <= 1e-5


def _oracle_contact_step(x, X, v, tri, hinge, box, fixed, fixed_vel):
    """Cloth::step with collisions on the CPU: pins from v, CD2 rows,
    Forces::fill, exact QP, x += h v."""
    n = len(x) // 3
    cons = O.cd2(x, tri, [box], threshold=1e-3)
    C, d = qp_ref.contact_rows(cons, n)
    F = O.Forces(x, X, tri, hinge, O.material(), scenes.GRAV, scenes.H)
    b = F.rhs(v, scenes.H)
    beq = (1 - 0.01) * v[fixed] + fixed_vel
    vn, lam, _ = qp_ref.solve_qp(F.csr(1), b, fixed, beq, C, d)
    return x + scenes.H * vn, vn, C.shape[0]


@pytest.mark.parametrize("precision,tol", [(0, 1e-7), (1, 1e-5)])
def test_contact_steps_track_the_oracle(eolc, precision, tol):
    """Cloth::step with the QP: each GPU step against the CPU step from the
    same state, for three steps of a pinned sheet falling onto a box."""
    quads = 24
    x0, X, tri, center, snaps = scenes.drape_positions(quads, 40)
    n = len(x0) // 3
    hinge = O.hinges(n, tri)
    box = O.axis_box(center, (0.4, 0.4, 0.2))
    ids = O.corner_ids(quads + 1, quads + 1)
    fixed = np.array([3 * ids[k] + c for k in (3, 4) for c in range(3)], np.int32)
    fixed_vel = np.zeros(len(fixed))
    ctx = eolc.Context(0)
    ctx.set_topology(n, tri, hinge)
    mat = eolc.Material(**scenes.material_c1())
    rng = np.random.default_rng(4)
    x = snaps[14].copy()
    v = rng.normal(0, 0.02, 3 * n)
    v[2::3] -= 0.4
    tol_pcg = 1e-10 if precision == 0 else 1e-8
    opts = eolc.SolveOpts(rel_tol=tol_pcg, precision=precision)
    rows = []
    for k in range(3):
        xo, vo, m = _oracle_contact_step(x, X, v, tri, hinge, box, fixed, fixed_vel)
        xg, vg = x.copy(), v.copy()
        info = ctx.step_contacts(xg, X, vg, mat, scenes.GRAV, scenes.H, fixed, fixed_vel,
                                 boxes=[eolc.Box(box.dim, box.E1)], threshold=1e-3, opts=opts)
        assert info.status == eolc.OK
        rows.append((m, info.n_active, info.solves))
        assert _relmax(vg, vo) <= tol, (k, _relmax(vg, vo))
        assert np.abs(xg - xo).max() <= scenes.H * tol * np.abs(vo).max() + 1e-15
        x, v = xg, vg
    print("rows / active / solves per step:", rows)
    assert all(m > 0 for m, _, _ in rows)


def test_carried_multipliers_change_the_path_not_the_answer(eolc):
    """eolc_step_contacts starts each persisting contact from the previous
    call's multiplier: the same step repeated from the same state gives the
    same velocities (FP64, 1e-8) in fewer linear solves."""
    quads = 24
    x0, X, tri, center, snaps = scenes.drape_positions(quads, 40)
    n = len(x0) // 3
    hinge = O.hinges(n, tri)
    box = O.axis_box(center, (0.4, 0.4, 0.2))
    ids = O.corner_ids(quads + 1, quads + 1)
    fixed = np.array([3 * ids[k] + c for k in (3, 4) for c in range(3)], np.int32)
    ctx = eolc.Context(0)
    ctx.set_topology(n, tri, hinge)
    mat = eolc.Material(**scenes.material_c1())
    v0 = np.random.default_rng(4).normal(0, 0.02, 3 * n)
    v0[2::3] -= 0.4
    opts = eolc.SolveOpts(rel_tol=1e-10, precision=eolc.PREC_FP64)
    out = []
    for k in range(2):
        x, v = snaps[14].copy(), v0.copy()
        info = ctx.step_contacts(x, X, v, mat, scenes.GRAV, scenes.H, fixed, np.zeros(len(fixed)),
                                 boxes=[eolc.Box(box.dim, box.E1)], threshold=1e-3, opts=opts)
        assert info.status == eolc.OK
        out.append((v, info.solves))
    print("solves cold %d, warm %d" % (out[0][1], out[1][1]))
    assert _relmax(out[1][0], out[0][0]) <= 1e-8
    assert out[1][1] < out[0][1]
    ctx.clear_contact_multipliers()
    x, v = snaps[14].copy(), v0.copy()
    info = ctx.step_contacts(x, X, v, mat, scenes.GRAV, scenes.H, fixed, np.zeros(len(fixed)),
                             boxes=[eolc.Box(box.dim, box.E1)], threshold=1e-3, opts=opts)
    assert info.solves == out[0][1]


def test_dropped_sheet_contact_trajectory(eolc):
    """Consecutive Cloth::steps with contacts on the configuration-2 sheet:
    128x128 quads (positions jittered N(0, 1e-4), seed 2), unpinned, dropped
    flat onto the 0.4 x 0.4 x 0.2 box whose top face starts 0.05 m below it
    (mixed precision, patch-PCG to rel-res 1e-8, multipliers carried from
    step to step).  Every step converges with every contact row satisfied to
    the QP's bound, the first contacts arrive when free fall says (semi-
    implicit Euler: g h^2 k (k + 1) / 2 = 0.05 - 1e-3 at k = 20), and the
    sheet's centre then rests on the box top.  Per-step velocities against
    the exact QP are tested on the 24x24 drape above."""
    quads = 128
    r = quads + 1
    x0, X, tri = eolc.sheet_mesh(r, r)
    n = len(x0) // 3
    hinge = eolc.mesh_hinges(tri)
    box = O.axis_box([0.5, 0.5, -0.15], (0.4, 0.4, 0.2))
    ctx = eolc.Context(0)
    ctx.set_topology(n, tri, hinge)
    mat = eolc.Material(**scenes.material_c1())
    x = x0 + np.random.default_rng(2).normal(0.0, 1e-4, x0.size)
    v = np.zeros(3 * n)
    none = np.zeros(0, np.int32)
    opts = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED, precond=eolc.PC_PATCH,
                          degree=5)
    active = []
    for k in range(40):
        info = ctx.step_contacts(x, X, v, mat, scenes.GRAV, scenes.H, none, np.zeros(0),
                                 boxes=[eolc.Box(box.dim, box.E1)], threshold=1e-3, opts=opts)
        assert info.status == eolc.OK, k
        assert info.max_violation <= 1e-6, (k, info.max_violation)
        active.append(info.n_active)
    print("active contact rows per step:", active)
    assert max(active[:19]) == 0 and min(active[21:]) > 0
    centre = x.reshape(-1, 3)[(r // 2) * r + r // 2]
    assert abs(centre[2] - (-0.05)) <= 2e-3, centre
