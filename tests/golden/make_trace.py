"""Generate tests/golden/trace_c1.npz: the oracle's 100-step run of the 20 x 20
quad sheet (441 nodes, 800 triangles, 1,160 hinges; corners 3 and 4 pinned;
rho 0.1, E 50, nu 0.3, beta 1e-5, damping (0, 1); h 5e-3; Jacobi CG to a
relative residual of 1e-8; from rest).

Stored per step: the CG iteration count and relative residual, and weighted
checksums of f, M and MDK (the sum of every entry times a weight hashed from
its row and column with integer arithmetic, so that any changed entry moves
them, explicit zeros do not, and every machine computes the same weights);
at the checkpoint steps the positions and velocities themselves.  Pairs of
consecutive checkpoints (1-2, 5-6, 50-51) give single steps to replay.

The fixture is a regression trace of the oracle's whole Cloth::step
(Forces::fill, pins, solve, x += h v) and the library's parity fixture on
the GPU (tests/test_gpu_trace.py); the oracle's element math is pinned
separately to the reference's own routines (elements.npz).

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
CHECKPOINTS = (1, 2, 5, 6, 10, 25, 50, 51, 100)


def weights(rows, cols):
    """A weight in [-0.5, 0.5) per (row, col): a multiplicative hash in
    64-bit integers, exact on every machine."""
    r = np.asarray(rows, np.uint64)
    c = np.asarray(cols, np.uint64)
    h = (r * np.uint64(0x9E3779B97F4A7C15) + c * np.uint64(0xC2B2AE3D27D4EB4F)
         + np.uint64(0x165667B19E3779F9))
    h ^= h >> np.uint64(29)
    h *= np.uint64(0xBF58476D1CE4E5B9)
    h ^= h >> np.uint64(32)
    return (h >> np.uint64(11)).astype(np.float64) / 2.0 ** 53 - 0.5


def checksums(f, M, K):
    """(weighted sum, sum of |entries|) of f, M and MDK (scipy sparse)."""
    out = [f @ weights(np.arange(f.size), np.zeros(f.size, np.int64)), np.abs(f).sum()]
    for A in (M, K):
        A = A.tocoo()
        out += [A.data @ weights(A.row, A.col), np.abs(A.data).sum()]
    return np.array(out)


def run():
    s = scenes.sheet(QUADS)
    mat = O.material(**scenes.material_c1())
    x, v = s["x"].copy(), np.zeros(3 * s["n"])
    iters, rres, sums = [], [], []
    xs, vs = [], []
    for k in range(1, STEPS + 1):
        F = O.Forces(x, s["X"], s["tri"], s["hinge"], mat, scenes.GRAV, scenes.H)
        sums.append(checksums(F.f(), F.csr(0), F.csr(1)))
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
