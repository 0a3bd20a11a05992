"""Generate tests/golden/trace_c1.npz: the oracle's 100-step run of the 20 x 20
quad sheet (441 nodes, 800 triangles, 1,160 hinges; corners 3 and 4 pinned;
rho 0.1, E 50, nu 0.3, beta 1e-5, damping (0, 1); h 5e-3; Jacobi CG to a
relative residual of 1e-8; from rest).

Stored per step: the CG iteration count and relative residual, and weighted
checksums of f, M and MDK (the sum of every entry times a fixed pseudo-random
weight, so that any changed entry moves them); at the checkpoint steps the
positions and velocities themselves.  The fixture is a regression trace of
the oracle's whole Cloth::step (Forces::fill, pins, solve, x += h v): its
element math is pinned separately to the reference's own routines
(elements.npz).

Usage (from the repository root):
    python tests/golden/make_trace.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for sub in ("oracle", "tests"):
    sys.path.insert(0, os.path.join(ROOT, sub))
import oracle as O  # noqa: E402
import scenes  # noqa: E402

OUT = os.path.join(HERE, "trace_c1.npz")
QUADS = 20
STEPS = 100
CHECKPOINTS = (1, 2, 5, 10, 25, 50, 100)
WEIGHT_SEED = 20180814


def weights(n, salt):
    return np.random.default_rng([WEIGHT_SEED, salt]).uniform(-1.0, 1.0, n)


def checksums(F):
    """(f, M, MDK) weighted sums; the CSR layouts are canonical (sorted
    columns, duplicates summed), so entry k of data is a fixed (row, col)."""
    f = F.f()
    M, K = F.csr(0), F.csr(1)
    return np.array([f @ weights(f.size, 0), M.data @ weights(M.nnz, 1),
                     K.data @ weights(K.nnz, 2), np.abs(K.data).sum()])


def run():
    s = scenes.sheet(QUADS)
    mat = O.material(**scenes.material_c1())
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    iters, rres, sums = [], [], []
    xs, vs = [], []
    for k in range(1, STEPS + 1):
        F = O.Forces(x, s["X"], s["tri"], s["hinge"], mat, scenes.GRAV, scenes.H)
        sums.append(checksums(F))
        del F
        it, rr = O.step(x, s["X"], v, s["tri"], s["hinge"], mat, scenes.GRAV, scenes.H,
                        s["fixed"], s["fixed_vel"], tol=1e-8)
        iters.append(it)
        rres.append(rr)
        if k in CHECKPOINTS:
            xs.append(x.copy())
            vs.append(v.copy())
    return dict(checkpoints=np.array(CHECKPOINTS), iters=np.array(iters), rel_res=np.array(rres),
                fill_sums=np.array(sums), x=np.array(xs), v=np.array(vs))


def main():
    np.savez_compressed(OUT, **run())
    print("wrote", OUT)


if __name__ == "__main__":
    main()
