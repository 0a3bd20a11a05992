"""Patch-local preconditioner (EOLC_PC_PATCH): same FP64 relative residual as
Jacobi-PCG, the same velocities, and far fewer iterations.

The comparison is the Jacobi path (itself checked against the oracle's Eigen-style
CG and direct solve in test_gpu_parity.py) and, on the small sheet, the
oracle's direct solve.
"""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


def _ctx(eolc, s):
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    return ctx


@pytest.mark.parametrize("quads", [20, 64])
def test_patch_steps_match_jacobi_steps(eolc, quads):
    s = scenes.sheet(quads)
    ctx = _ctx(eolc, s)
    mat = eolc.Material(**scenes.material_c1())
    rng = np.random.default_rng(quads)
    # a jitter of 6% of the edge length keeps MDK positive definite
    x = s["x"] + rng.normal(0, 0.06 / quads, s["x"].size)
    v = np.zeros_like(x)
    for step in range(4):
        xj, vj = x.copy(), v.copy()
        xp, vp = x.copy(), v.copy()
        ij = ctx.step(xj, s["X"], vj, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_JACOBI))
        ip = ctx.step(xp, s["X"], vp, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_PATCH))
        assert ip.status == eolc.OK and ip.rel_res <= 1e-8
        assert np.abs(vp - vj).max() <= 1e-5 * np.abs(vj).max()
        assert np.abs(xp - xj).max() <= 1e-7
        print("step %d: Jacobi %d iterations, patch %d" % (step, ij.iterations, ip.iterations))
        x, v = xj, vj


@pytest.mark.parametrize("quads", [40, 128])
def test_coarse_correction_keeps_solution_and_cuts_iterations(eolc, quads):
    """Two-level patch preconditioner (default) against the one-level one
    (no_coarse=1): the same velocities to the FP64 criterion's accuracy,
    and fewer iterations at 128^2 (42 aggregates of patches)."""
    s = scenes.sheet(quads)
    ctx = _ctx(eolc, s)
    mat = eolc.Material(**scenes.material_c1())
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    its2, its1 = [], []
    for step in range(3):
        xa, va = x.copy(), v.copy()
        i2 = ctx.step(xa, s["X"], va, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_PATCH))
        i1 = ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_PATCH, no_coarse=1))
        assert i2.status == eolc.OK and i2.rel_res <= 1e-8
        assert i1.status == eolc.OK and i1.rel_res <= 1e-8
        assert np.abs(va - v).max() <= 1e-5 * np.abs(v).max()
        its2.append(i2.iterations)
        its1.append(i1.iterations)
    print("two-level %s, one-level %s" % (its2, its1))
    if quads >= 128:
        assert np.mean(its2) <= 0.75 * np.mean(its1)


def test_lagged_coarse_operator_converges(eolc):
    """Coarse operator rebuilt every 3 solves (eolc_set_coarse_refresh): the
    reused ones still give converged steps matching the fresh ones."""
    s = scenes.sheet(64)
    ctx = _ctx(eolc, s)
    lag = _ctx(eolc, s)
    lag.set_coarse_refresh(3)
    mat = eolc.Material(**scenes.material_c1())
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    xl, vl = x.copy(), v.copy()
    for step in range(5):
        i1 = ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_PATCH))
        i2 = lag.step(xl, s["X"], vl, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_PATCH))
        assert i1.status == eolc.OK and i2.status == eolc.OK and i2.rel_res <= 1e-8
        assert np.abs(vl - v).max() <= 1e-5 * np.abs(v).max()
        print("step %d: fresh %d iterations, lagged %d" % (step, i1.iterations, i2.iterations))
    with pytest.raises(eolc.EolcError):
        lag.set_coarse_refresh(0)


def test_patch_solve_matches_direct_solve(eolc):
    import oracle as O
    s = scenes.sheet(20)
    ctx = _ctx(eolc, s)
    mat = eolc.Material(**scenes.material_c1())
    rng = np.random.default_rng(3)
    x = s["x"] + rng.normal(0, 0.003, s["x"].size)
    v = rng.normal(0, 0.1, x.size)
    ctx.forces_fill(x, s["X"], mat, scenes.GRAV, scenes.H, eolc.PREC_MIXED, want_M=False)
    F = O.Forces(x, s["X"], s["tri"], s["hinge"], O.material(), scenes.GRAV, scenes.H)
    b = F.rhs(v, scenes.H)
    beq = 0.99 * v[s["fixed"]]
    vd = F.solve_direct(b, s["fixed"], beq)
    vp, info = ctx.velocity_solve(b, s["fixed"], beq,
                                  eolc.SolveOpts(precond=eolc.PC_PATCH, rel_tol=1e-10))
    assert info.status == eolc.OK
    # the mixed path solves the FP32-rounded matrix: agreement to its accuracy
    assert np.abs(vp - vd).max() <= 1e-4 * np.abs(vd).max()


def test_patch_needs_far_fewer_iterations(eolc):
    s = scenes.sheet(128)
    ctx = _ctx(eolc, s)
    mat = eolc.Material(**scenes.material_c1())
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    its_j, its_p = [], []
    for step in range(3):
        xp, vp = x.copy(), v.copy()
        ij = ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_JACOBI))
        ip = ctx.step(xp, s["X"], vp, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                      eolc.SolveOpts(precond=eolc.PC_PATCH))
        assert ip.status == eolc.OK and ip.rel_res <= 1e-8
        its_j.append(ij.iterations)
        its_p.append(ip.iterations)
    print("Jacobi %s, patch %s" % (its_j, its_p))
    assert np.mean(its_p) <= 0.5 * np.mean(its_j)


@pytest.mark.parametrize("degree", [1, 3, 16])
def test_patch_degrees_converge(eolc, degree):
    s = scenes.sheet(40)
    ctx = _ctx(eolc, s)
    mat = eolc.Material(**scenes.material_c1())
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    info = ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                    eolc.SolveOpts(precond=eolc.PC_PATCH, degree=degree))
    assert info.status == eolc.OK and info.rel_res <= 1e-8


def test_patch_argument_errors(eolc):
    s = scenes.sheet(8)
    ctx = _ctx(eolc, s)
    mat = eolc.Material(**scenes.material_c1())
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    for opts in (eolc.SolveOpts(precond=eolc.PC_PATCH, precision=eolc.PREC_FP64),
                 eolc.SolveOpts(precond=eolc.PC_PATCH, degree=65)):
        with pytest.raises(eolc.EolcError) as e:
            ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"], opts)
        assert e.value.status == eolc.BAD_ARG


def test_patch_rejects_meshes_beyond_shared_memory(eolc):
    s = scenes.sheet(320)  # 103,041 nodes: > 464 per SM on a 152-SM device
    ctx = _ctx(eolc, s)
    mat = eolc.Material(**scenes.material_c1())
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    with pytest.raises(eolc.EolcError) as e:
        ctx.step(x, s["X"], v, mat, scenes.GRAV, scenes.H, s["fixed"], s["fixed_vel"],
                 eolc.SolveOpts(precond=eolc.PC_PATCH))
    assert e.value.status == eolc.BAD_ARG
