"""Shared-memory tiled assembly of M and MDK (tile_blocks_kernel): parity
with the oracle's Forces::fill (Forces.cpp:331-930: triplets summed in
insertion order) on an irregular mesh whose rows have uneven valence and span
many tiles, and, at the full 256 x 256-quad size, the properties that do not
need the oracle: a matrix symmetric to the rounding of its precision (each
element block (a, b), a > b, is the transpose of the evaluated (b, a), and
both sums run over the same elements in the same order; the block formula
is compiled once per local row, so the two evaluations may round a last bit
differently), bit-identical results run to run, and the FP32 matrix within
FP32 rounding of the FP64 one (1e-5 of the largest entry, as the mixed parity
tests against the oracle)."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle as O
import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eolc():
    import __graft_entry__ as g
    g.build_lib()
    import eolc as E
    return E


def _mat(eolc):
    return eolc.Material(**scenes.material_c1())


def test_irregular_mesh_fill_matches_oracle(eolc):
    rng = np.random.default_rng(21)
    s = scenes.delaunay_sheet(6000, rng)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    x = s["x"] + rng.normal(0, 2e-3, s["x"].size)
    F = O.Forces(x, s["X"], s["tri"], s["hinge"], O.material(**scenes.material_c1()),
                 scenes.GRAV, scenes.H)
    M0, K0 = F.csr(0), F.csr(1)
    f, M, MDK = ctx.forces_fill(x, s["X"], _mat(eolc), scenes.GRAV, scenes.H, eolc.PREC_FP64)
    assert abs(eolc.bsr_to_csr(ctx, M) - M0).max() <= 1e-10 * abs(M0).max()
    assert abs(eolc.bsr_to_csr(ctx, MDK) - K0).max() <= 1e-10 * abs(K0).max()
    f32, _, MDK32 = ctx.forces_fill(x, s["X"], _mat(eolc), scenes.GRAV, scenes.H,
                                    eolc.PREC_MIXED, want_M=False)
    assert abs(eolc.bsr_to_csr(ctx, MDK32) - K0).max() <= 1e-5 * abs(K0).max()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_full_size_matrix_symmetric_and_reproducible(eolc, precision):
    s = scenes.sheet(256)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    rng = np.random.default_rng(5)
    x = s["x"] + rng.normal(0, 1e-3, s["x"].size)
    prec = eolc.PREC_MIXED if precision == "mixed" else eolc.PREC_FP64
    _, _, A = ctx.forces_fill(x, s["X"], _mat(eolc), scenes.GRAV, scenes.H, prec, want_M=False)
    _, _, B = ctx.forces_fill(x, s["X"], _mat(eolc), scenes.GRAV, scenes.H, prec, want_M=False)
    assert np.array_equal(A, B)  # no atomics: bit-reproducible
    rp, ci = ctx.bsr_pattern()
    row = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    blk = A.reshape(-1, 3, 3)
    where = {(int(i), int(j)): k for k, (i, j) in enumerate(zip(row, ci))}
    partner = np.array([where[(int(j), int(i))] for i, j in zip(row, ci)])
    eps = 1e-6 if precision == "mixed" else 1e-14
    asym = np.abs(blk - blk[partner].transpose(0, 2, 1)).max()
    assert asym <= eps * np.abs(blk).max(), asym
    K = eolc.bsr_to_csr(ctx, A)
    if precision == "mixed":
        _, _, D = ctx.forces_fill(x, s["X"], _mat(eolc), scenes.GRAV, scenes.H, eolc.PREC_FP64,
                                  want_M=False)
        Kd = eolc.bsr_to_csr(ctx, D)
        assert abs(K - Kd).max() <= 1e-5 * abs(Kd).max()  # the mixed parity tolerance
