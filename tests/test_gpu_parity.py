"""GPU parity tests through the C ABI (libeolc.so) against the CPU oracle.

Tolerances:
  * FP64 path: f, M and MDK BSR values within 1e-10 relative (max-norm);
    velocities of an FP64 solve at tol 1e-12 within 1e-10 of the oracle's
    direct solution.
  * mixed path (FP32 matrix assembly / PCG, FP64 forces and right-hand side,
    FP64 dots + FP64 refinement residual): final FP64 relative residual
    <= 1e-8 on its own system; its error against the FP64 oracle is measured
    and bounded (1e-5 relative on v).
  * collisions: contact list bit-identical, order included.
"""
import numpy as np
import pytest

import oracle as O
import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


@pytest.fixture(scope="module")
def ctx(eolc):
    return eolc.Context(0)


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def gpu_material(eolc, **kw):
    m = scenes.material_c1()
    m.update(kw)
    return eolc.Material(**m)


def oracle_material(**kw):
    m = scenes.material_c1()
    m.update(kw)
    return O.material(**m)


def deformed(x, seed, amp=0.01):
    rng = np.random.default_rng(seed)
    return x + rng.normal(0, amp, x.size)


@pytest.mark.parametrize("builder,res", [("grid2", 21), ("grid2", 6), ("gridc", 7)])
def test_forces_fill_fp64_matches_oracle(eolc, ctx, builder, res):
    x, X, tri = getattr(O, builder)(res, res)
    hinge = O.hinges(len(x) // 3, tri)
    ctx.set_topology(len(x) // 3, tri, hinge)
    for seed in range(3):
        xd = deformed(x, seed) if seed else x
        f, M, MDK = ctx.forces_fill(xd, X, gpu_material(eolc), scenes.GRAV, scenes.H, eolc.PREC_FP64)
        F = O.Forces(xd, X, tri, hinge, oracle_material(), scenes.GRAV, scenes.H)
        assert relmax(f, F.f()) <= 1e-10
        Mg = eolc.bsr_to_csr(ctx, M)
        Kg = eolc.bsr_to_csr(ctx, MDK)
        assert abs(Mg - F.csr(0)).max() <= 1e-10 * abs(F.csr(0)).max()
        assert abs(Kg - F.csr(1)).max() <= 1e-10 * abs(F.csr(1)).max()
        # same sparsity pattern as the reference's setFromTriplets result
        assert Kg.nnz == F.csr(1).nnz


def test_forces_fill_mixed_close_to_fp64(eolc, ctx):
    s = scenes.sheet(20)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    xd = deformed(s["x"], 4)
    f, _, MDK = ctx.forces_fill(xd, s["X"], gpu_material(eolc), scenes.GRAV, scenes.H, eolc.PREC_MIXED)
    F = O.Forces(xd, s["X"], s["tri"], s["hinge"], oracle_material(), scenes.GRAV, scenes.H)
    assert relmax(f, F.f()) <= 1e-5
    assert abs(eolc.bsr_to_csr(ctx, MDK) - F.csr(1)).max() <= 1e-5 * abs(F.csr(1)).max()


def test_bsr_pattern_counts(eolc, ctx):
    """20x20 quads: 441 nodes, 800 triangles, 1160 hinges, 5241 blocks."""
    s = scenes.sheet(20)
    assert len(s["tri"]) == 800 and len(s["hinge"]) == 1160
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    rp, ci = ctx.bsr_pattern()
    assert len(ci) == 5241 and rp[-1] == 5241


@pytest.mark.parametrize("precond", [0, 1])
def test_velocity_solve_fp64_matches_direct(eolc, ctx, precond):
    s = scenes.sheet(20)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    xd = deformed(s["x"], 5, 0.005)
    v0 = np.random.default_rng(1).normal(0, 0.1, xd.size)
    F = O.Forces(xd, s["X"], s["tri"], s["hinge"], oracle_material(), scenes.GRAV, scenes.H)
    b = F.rhs(v0, scenes.H)
    beq = 0.99 * v0[s["fixed"]]
    vd = F.solve_direct(b, s["fixed"], beq)
    ctx.forces_fill(xd, s["X"], gpu_material(eolc), scenes.GRAV, scenes.H, eolc.PREC_FP64)
    opts = eolc.SolveOpts(rel_tol=1e-12, precision=eolc.PREC_FP64, precond=precond)
    v, info = ctx.velocity_solve(b, s["fixed"], beq, opts)
    assert info.status == eolc.OK and info.rel_res <= 1e-12
    assert relmax(v, vd) <= 1e-10


@pytest.mark.parametrize("precond", [0, 1])
def test_velocity_solve_mixed_reaches_fp64_residual(eolc, ctx, precond):
    s = scenes.sheet(24)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    xd = deformed(s["x"], 6, 0.003)
    v0 = np.random.default_rng(2).normal(0, 0.1, xd.size)
    ctx.forces_fill(xd, s["X"], gpu_material(eolc), scenes.GRAV, scenes.H, eolc.PREC_MIXED)
    F = O.Forces(xd, s["X"], s["tri"], s["hinge"], oracle_material(), scenes.GRAV, scenes.H)
    b = F.rhs(v0, scenes.H)
    beq = 0.99 * v0[s["fixed"]]
    opts = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED, precond=precond)
    v, info = ctx.velocity_solve(b, s["fixed"], beq, opts)
    assert info.status == eolc.OK
    assert info.rel_res <= 1e-8
    assert info.refinements >= 1
    # the residual against the FP32-assembled system, recomputed here in FP64
    _, _, MDK32 = ctx.forces_fill(xd, s["X"], gpu_material(eolc), scenes.GRAV, scenes.H,
                                  eolc.PREC_MIXED)
    A = eolc.bsr_to_csr(ctx, MDK32)
    free = np.setdiff1d(np.arange(xd.size), s["fixed"])
    vf = v.copy()
    r = (-b - A @ vf)[free]
    rhs = (-b - A[:, s["fixed"]] @ beq)[free]
    assert np.linalg.norm(r) <= 1.05e-8 * np.linalg.norm(rhs)
    # error against the FP64 oracle solution (only the FP32 matrix differs)
    vd = F.solve_direct(b, s["fixed"], beq)
    assert relmax(v, vd) <= 1e-5


def _oracle_step_direct(F, v, fixed, fixed_vel):
    b = F.rhs(v, scenes.H)
    beq = (1 - 0.01) * v[fixed] + fixed_vel
    return F.solve_direct(b, fixed, beq)


def test_config1_100_steps_fp64_per_step(eolc, ctx):
    """Configuration 1 (20x20 quads, corners 3 and 4 pinned, 100 FP64 steps).
    Every step starts both sides from the oracle's state (the drape amplifies
    a 1e-13 difference to ~1e-8 within 100 steps, oracle against itself):
    f and MDK within 1e-10, the new velocity within 1e-10 of the oracle's
    direct FP64 solve and the new positions within 1e-12."""
    s = scenes.sheet(20)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    mat_g, mat_o = gpu_material(eolc), oracle_material()
    opts = eolc.SolveOpts(rel_tol=1e-13, precision=eolc.PREC_FP64)
    xo, vo = s["x"].copy(), np.zeros(3 * s["n"])
    worst_v = worst_x = worst_f = worst_k = 0.0
    for k in range(100):
        F = O.Forces(xo, s["X"], s["tri"], s["hinge"], mat_o, scenes.GRAV, scenes.H)
        f, _, MDK = ctx.forces_fill(xo, s["X"], mat_g, scenes.GRAV, scenes.H, eolc.PREC_FP64)
        worst_f = max(worst_f, relmax(f, F.f()))
        K = F.csr(1)
        worst_k = max(worst_k, abs(eolc.bsr_to_csr(ctx, MDK) - K).max() / abs(K).max())
        xg, vg = xo.copy(), vo.copy()
        info = ctx.step(xg, s["X"], vg, mat_g, scenes.GRAV, scenes.H, s["fixed"],
                        s["fixed_vel"], opts)
        assert info.status == eolc.OK and info.rel_res <= 1e-13
        vo = _oracle_step_direct(F, vo, s["fixed"], s["fixed_vel"])
        xo = xo + scenes.H * vo
        worst_v = max(worst_v, relmax(vg, vo))
        worst_x = max(worst_x, np.abs(xg - xo).max())
    assert worst_f <= 1e-10 and worst_k <= 1e-10, (worst_f, worst_k)
    assert worst_v <= 1e-10, worst_v
    assert worst_x <= 1e-12, worst_x


def test_config1_mixed_per_step_error_vs_fp64(eolc, ctx):
    """Mixed path on the configuration-1 states: FP64 residual <= 1e-8 every
    step; stated error against the FP64 oracle velocity <= 1e-5 relative (FP32
    matrix, FP64 forces and right-hand side)."""
    s = scenes.sheet(20)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    opts = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED)
    xo, vo = s["x"].copy(), np.zeros(3 * s["n"])
    worst = 0.0
    for k in range(100):
        F = O.Forces(xo, s["X"], s["tri"], s["hinge"], oracle_material(), scenes.GRAV, scenes.H)
        xg, vg = xo.copy(), vo.copy()
        info = ctx.step(xg, s["X"], vg, gpu_material(eolc), scenes.GRAV, scenes.H, s["fixed"],
                        s["fixed_vel"], opts)
        assert info.status == eolc.OK and info.rel_res <= 1e-8
        vo = _oracle_step_direct(F, vo, s["fixed"], s["fixed_vel"])
        xo = xo + scenes.H * vo
        worst = max(worst, relmax(vg, vo))
    print("worst mixed velocity error vs FP64 oracle: %.2e" % worst)
    assert worst <= 1e-5, worst


def test_short_free_run_tracks_oracle(eolc, ctx):
    """Free-running FP64 trajectories agree to 1e-10 over the first 20 steps,
    before the drape's sensitivity takes over."""
    s = scenes.sheet(20)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    opts = eolc.SolveOpts(rel_tol=1e-13, precision=eolc.PREC_FP64)
    xg, vg = s["x"].copy(), np.zeros(3 * s["n"])
    xo, vo = s["x"].copy(), np.zeros(3 * s["n"])
    for k in range(20):
        ctx.step(xg, s["X"], vg, gpu_material(eolc), scenes.GRAV, scenes.H, s["fixed"],
                 s["fixed_vel"], opts)
        F = O.Forces(xo, s["X"], s["tri"], s["hinge"], oracle_material(), scenes.GRAV, scenes.H)
        vo = _oracle_step_direct(F, vo, s["fixed"], s["fixed_vel"])
        xo = xo + scenes.H * vo
    assert relmax(vg, vo) <= 1e-10 and np.abs(xg - xo).max() <= 1e-12


def test_resident_steps_equal_host_steps(eolc, ctx):
    s = scenes.sheet(16)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    opts = eolc.SolveOpts(precision=eolc.PREC_MIXED)
    mat = gpu_material(eolc)
    xa, va = s["x"].copy(), np.zeros(3 * s["n"])
    for _ in range(5):
        ctx.step(xa, s["X"], va, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"], opts)
    ctx.state_upload(s["x"], s["X"], np.zeros(3 * s["n"]))
    ctx.step_resident(5, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"], opts)
    xb, vb = ctx.state_download()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_runs_are_bit_reproducible(eolc, ctx):
    s = scenes.sheet(30)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    opts = eolc.SolveOpts(precision=eolc.PREC_MIXED)
    outs = []
    for _ in range(2):
        x, v = s["x"].copy(), np.zeros(3 * s["n"])
        for _ in range(3):
            ctx.step(x, s["X"], v, gpu_material(eolc), scenes.GRAV, scenes.H, s["fixed"],
                     s["fixed_vel"], opts)
        outs.append((x, v))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


# ---------------------------------------------------------------- collisions
def _box(eolc, center, dim):
    ob = O.axis_box(center, dim)
    return ob, eolc.Box(list(ob.dim), list(ob.E1))


def test_collisions_small_bit_exact(eolc, ctx):
    x0, X, tri, center, snaps = scenes.drape_positions(24, 12, seed=3, box_dim=(0.4, 0.4, 0.2))
    ctx.set_topology(len(x0) // 3, tri, O.hinges(len(x0) // 3, tri))
    ob, gb = _box(eolc, center, (0.4, 0.4, 0.2))
    kinds = set()
    for x in snaps:
        want = O.cd2(x, tri, boxes=[ob], threshold=1e-3)
        got = ctx.cd2(x, boxes=[gb], threshold=1e-3)
        assert eolc.contacts_equal(got, want), (len(got), len(want))
        kinds |= {(c.count1, c.count2) for c in want}
    assert (3, 1) in kinds and (2, 2) in kinds


def test_collisions_points_and_two_boxes_bit_exact(eolc, ctx):
    x0, X, tri, center, snaps = scenes.drape_positions(16, 4, seed=5)
    ctx.set_topology(len(x0) // 3, tri, O.hinges(len(x0) // 3, tri))
    rng = np.random.default_rng(0)
    pts = np.column_stack([rng.uniform(0, 1, 40), rng.uniform(0, 1, 40),
                           rng.uniform(-0.06, -0.03, 40)])
    nrm = np.tile([0.0, 0.0, 1.0], (40, 1))
    ob1, gb1 = _box(eolc, center, (0.4, 0.4, 0.2))
    ob2, gb2 = _box(eolc, [0.85, 0.2, center[2]], (0.2, 0.3, 0.2))
    for x in snaps:
        want = O.cd2(x, tri, boxes=[ob1, ob2], points=pts, normals=nrm, threshold=2e-3)
        got = ctx.cd2(x, boxes=[gb1, gb2], points=pts, normals=nrm, threshold=2e-3)
        assert eolc.contacts_equal(got, want), (len(got), len(want))


def test_collisions_empty_and_capacity(eolc, ctx):
    x0, X, tri, center, snaps = scenes.drape_positions(8, 1)
    ctx.set_topology(len(x0) // 3, tri, O.hinges(len(x0) // 3, tri))
    # box far away: no contacts
    _, far = _box(eolc, [5.0, 5.0, 5.0], (0.4, 0.4, 0.2))
    assert ctx.cd2(x0, boxes=[far]) == []
    assert ctx.cd2(x0) == []
    # capacity too small: status CAPACITY with the needed count
    x0, X, tri, center, snaps = scenes.drape_positions(24, 12, seed=3)
    ctx.set_topology(len(x0) // 3, tri, O.hinges(len(x0) // 3, tri))
    ob, gb = _box(eolc, center, (0.4, 0.4, 0.2))
    x = snaps[-1]
    n = len(O.cd2(x, tri, boxes=[ob]))
    assert n > 2
    with pytest.raises(eolc.EolcError) as e:
        ctx.cd2(x, boxes=[gb], capacity=1)
    assert e.value.status == eolc.CAPACITY


def test_nonfinite_inputs_are_reported(eolc, ctx):
    s = scenes.sheet(8)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    x = s["x"].copy()
    x[5] = np.nan
    _, gb = _box(eolc, [0.5, 0.5, -0.15], (0.4, 0.4, 0.2))
    with pytest.raises(eolc.EolcError) as e:
        ctx.cd2(x, boxes=[gb])
    assert e.value.status == eolc.NONFINITE
    v = np.zeros(3 * s["n"])
    with pytest.raises(eolc.EolcError) as e:
        ctx.step(x, s["X"], v, gpu_material(eolc), scenes.GRAV, scenes.H, s["fixed"],
                 s["fixed_vel"], eolc.SolveOpts(precision=eolc.PREC_MIXED))
    assert e.value.status == eolc.NONFINITE
    # the context stays usable
    x = s["x"].copy()
    ctx.step(x, s["X"], v, gpu_material(eolc), scenes.GRAV, scenes.H, s["fixed"],
             s["fixed_vel"], eolc.SolveOpts(precision=eolc.PREC_MIXED))
