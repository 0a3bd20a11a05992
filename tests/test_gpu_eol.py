"""EOL assembly branches on the GPU (eolc_set_topology_eol + eolc_forces_fill)
against the oracle's Forces::fill with EOL nodes (orc_forces_fill_eol):
f, M and MDK over the 3N + 2E DOFs of the reference, read out of the
library's extended block rows (Eulerian node k at block row N + k, DOFs 0
and 1; DOF 2 padding).  FP64 within 1e-10 relative, the mixed path's FP32
MDK within 1e-5; the padded DOF is inert; a pinned solve of the EOL system
matches a direct FP64 solve; the entry points that need one position per
block row refuse EOL topologies."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl

import oracle as O
import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


def _case(eolc, quads, n_eol, seed, amp):
    s = scenes.sheet(quads)
    rng = np.random.default_rng(seed)
    x = s["x"] + rng.normal(0, amp, s["x"].size)
    eol = rng.choice(s["n"], n_eol, replace=False)  # EoL_index order is arbitrary
    ctx = eolc.Context(0)
    ctx.set_topology_eol(s["n"], s["tri"], s["hinge"], eol)
    ref = O.ForcesEOL(x, s["X"], s["tri"], s["hinge"], O.material(), scenes.GRAV, scenes.H, eol)
    idx = eolc.eol_reference_index(s["n"], n_eol)
    return s, x, eol, ctx, ref, idx


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("quads,n_eol,seed", [(6, 9, 1), (12, 30, 2), (20, 80, 3)])
def test_fp64_fill_matches_oracle(eolc, quads, n_eol, seed):
    s, x, eol, ctx, ref, idx = _case(eolc, quads, n_eol, seed, 0.02)
    mat = eolc.Material(**scenes.material_c1())
    f, M, MDK = ctx.forces_fill(x, s["X"], mat, scenes.GRAV, scenes.H, eolc.PREC_FP64)
    A = eolc.bsr_to_csr(ctx, MDK)
    Mm = eolc.bsr_to_csr(ctx, M)
    Ar, Mr = A[idx][:, idx].toarray(), Mm[idx][:, idx].toarray()
    print("MDK %.1e  M %.1e  f %.1e" % (_rel(Ar, ref.csr(1).toarray()),
                                        _rel(Mr, ref.csr(0).toarray()), _rel(f[idx], ref.f())))
    assert _rel(Ar, ref.csr(1).toarray()) <= 1e-10
    assert _rel(Mr, ref.csr(0).toarray()) <= 1e-10
    assert _rel(f[idx], ref.f()) <= 1e-10
    # padded DOFs: zero force and mass, MDK identity on them
    pad = 3 * (s["n"] + np.arange(n_eol)) + 2
    assert not f[pad].any()
    assert np.abs(Mm[pad]).max() == 0
    Ad = A.toarray()
    assert np.array_equal(Ad[np.ix_(pad, pad)], np.eye(n_eol))
    others = np.setdiff1d(np.arange(A.shape[0]), pad)
    assert np.abs(Ad[np.ix_(pad, others)]).max() == 0


def test_mixed_fill_matches_oracle(eolc):
    s, x, eol, ctx, ref, idx = _case(eolc, 12, 30, 4, 0.02)
    mat = eolc.Material(**scenes.material_c1())
    f, M, MDK = ctx.forces_fill(x, s["X"], mat, scenes.GRAV, scenes.H, eolc.PREC_MIXED)
    A = eolc.bsr_to_csr(ctx, MDK)[idx][:, idx].toarray()
    assert _rel(A, ref.csr(1).toarray()) <= 1e-5
    assert _rel(f[idx], ref.f()) <= 1e-10  # forces stay FP64


# The EOL system alone can be indefinite (the reference solves it only
# under its EOL equality rows, Constraints.cpp:300-412): the free case uses a
# mesh whose reduced matrix is positive definite (checked on the CPU, cond
# ~1.4e3); the pinned case fixes every Eulerian DOF to nonzero values, which
# exercises the x-X blocks through the right-hand side.
@pytest.mark.parametrize("case", ["free", "pinned"])
@pytest.mark.parametrize("precision,precond", [(0, 0), (1, 1), (1, 3)])
def test_pinned_solve_matches_direct(eolc, case, precision, precond):
    if case == "free":
        s, x, eol, ctx, ref, idx = _case(eolc, 6, 9, 1, 0.05)
    else:
        s, x, eol, ctx, ref, idx = _case(eolc, 12, 30, 5, 0.05)
    n, E = s["n"], len(eol)
    mat = eolc.Material(**scenes.material_c1())
    ctx.forces_fill(x, s["X"], mat, scenes.GRAV, scenes.H, precision)
    rng = np.random.default_rng(6)
    v0 = rng.normal(0, 0.1, len(idx))
    b = -(ref.csr(0) @ v0 + scenes.H * ref.f())  # b = -(M v + h f), Cloth.cpp:345
    fixed_ref = np.array(s["fixed"], np.int64)  # corners: same index in both layouts
    if case == "pinned":
        fixed_ref = np.concatenate([fixed_ref, 3 * n + np.arange(2 * E)])
    beq = 0.99 * v0[fixed_ref]
    A = ref.csr(1).tocsc()
    free = np.setdiff1d(np.arange(len(idx)), fixed_ref)
    vd = np.zeros(len(idx))
    vd[fixed_ref] = beq
    vd[free] = spl.spsolve(A[free][:, free], -b[free] - A[free][:, fixed_ref] @ beq)
    bx = np.zeros(3 * ctx.n_nodes)
    bx[idx] = b
    tol = 1e-12 if precision == 0 else 1e-8
    v, info = ctx.velocity_solve(bx, idx[fixed_ref].astype(np.int32), beq,
                                 eolc.SolveOpts(rel_tol=tol, precision=precision, precond=precond))
    assert info.status == eolc.OK
    err = _rel(v[idx], vd)
    print("%s precision %d precond %d: %d iterations, v err %.2e" % (case, precision, precond,
                                                                      info.iterations, err))
    assert err <= (1e-8 if precision == 0 else 1e-4)
    assert not v[3 * (n + np.arange(E)) + 2].any()


def test_other_entry_points_refuse_eol(eolc):
    s, x, eol, ctx, ref, idx = _case(eolc, 6, 5, 7, 0.02)
    mat = eolc.Material(**scenes.material_c1())
    with pytest.raises(eolc.EolcError) as e:
        ctx.step(x.copy(), s["X"], np.zeros(3 * s["n"]), mat, scenes.GRAV, scenes.H,
                 s["fixed"], s["fixed_vel"])
    assert e.value.status == eolc.BAD_ARG
    assert ctx.cd2(x) == []  # CD2 runs on the mesh nodes (no obstacles here)
    with pytest.raises(eolc.EolcError):
        ctx.export_obj_text(0)
    # a plain topology afterwards works as before
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    f, M, MDK = ctx.forces_fill(x, s["X"], mat, scenes.GRAV, scenes.H, eolc.PREC_FP64)
    F = O.Forces(x, s["X"], s["tri"], s["hinge"], O.material(), scenes.GRAV, scenes.H)
    assert _rel(eolc.bsr_to_csr(ctx, MDK).toarray(), F.csr(1).toarray()) <= 1e-10
