"""Generate the collision golden vectors in tests/golden/cd_ref.npz.

Runs the reference's OWN collision detection — src/boxTriCollision.cpp and
src/raytri.cpp compiled unmodified against the minimal Eigen shim in
oracle/eigen_shim/, with the CD2 wrapper oracle/ref_cd.cpp, by
oracle/build_ref.sh into oracle/_ref/libeolc_ref_cd.so — on seeded drape
scenes and stores positions, obstacles and the contact records (the
library's eolc_contact layout, bytes).  The committed .npz pins the oracle's
restated CD2 (tests/test_oracle_golden.py) and the library's eolc_cd2
(tests/test_gpu_c2.py) on machines where the reference sources are absent.

Scenes (tests/scenes.py drapes, threshold 1e-3 unless stated):
  drape24   24 x 24 quads, seed 3, 12 snapshots, the 0.4 x 0.4 x 0.2 box;
  points16  16 x 16 quads, seed 5, 4 snapshots, 40 point obstacles and two
            boxes, threshold 2e-3;
  drape128  128 x 128 quads, seed 2024, snapshots 100 and 199 of the
            200-step drape of configuration 2 (edge-edge and corner
            contacts; vertex-face contacts).

Usage (from the repository root, where the reference sources are present):
    oracle/build_ref.sh && python tests/golden/make_cd_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for sub in ("oracle", "tests", "eol-cloth_gb300"):
    sys.path.insert(0, os.path.join(ROOT, sub))
import oracle as O  # noqa: E402  (record layouts and box frames)
import scenes as S  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "libeolc_ref_cd.so")
OUT = os.path.join(HERE, "cd_ref.npz")


def ref_cd2(L, x, tri, boxes, points=None, normals=None, threshold=1e-3):
    """The reference's CD2 on these positions: the contact records' bytes."""
    tri = np.ascontiguousarray(tri, np.int32)
    n = len(x) // 3
    pts = np.zeros(3) if points is None else np.ascontiguousarray(points, np.float64)
    nrm = np.zeros(3) if normals is None else np.ascontiguousarray(normals, np.float64)
    npts = 0 if points is None else len(pts.reshape(-1, 3))
    barr = (O.Box * max(1, len(boxes)))(*boxes)
    cap = 4 * n + 64
    out = (O.Contact * cap)()
    k = L.ref_cd2(n, O.dp(x), O.ip(tri), len(tri), barr, len(boxes), O.dp(pts), O.dp(nrm),
                  npts, ctypes.c_double(threshold), out, cap)
    assert k <= cap
    return np.frombuffer(ctypes.string_at(out, ctypes.sizeof(O.Contact) * k), np.uint8)


def box_arrays(boxes):
    return (np.array([list(b.dim) for b in boxes]), np.array([list(b.E1) for b in boxes]))


def main():
    L = ctypes.CDLL(REF)
    out = {}

    def store(name, tri, xs, boxes, threshold, points=None, normals=None):
        cons = [ref_cd2(L, x, tri, boxes, points, normals, threshold) for x in xs]
        dims, E1s = box_arrays(boxes)
        out.update({name + "_tri": np.asarray(tri, np.int32), name + "_x": np.array(xs),
                    name + "_dim": dims, name + "_E1": E1s,
                    name + "_thr": np.array(threshold),
                    name + "_n": np.array([len(c) // ctypes.sizeof(O.Contact) for c in cons]),
                    name + "_contacts": np.concatenate(cons)})
        if points is not None:
            out.update({name + "_pts": np.asarray(points), name + "_nrm": np.asarray(normals)})
        print(name, "contacts per snapshot", out[name + "_n"].tolist())

    x0, X, tri, center, snaps = S.drape_positions(24, 12, seed=3)
    store("drape24", tri, snaps, [O.axis_box(center, (0.4, 0.4, 0.2))], 1e-3)
    x0, X, tri, center, snaps = S.drape_positions(16, 4, seed=5)
    rng = np.random.default_rng(0)
    pts = np.column_stack([rng.uniform(0, 1, 40), rng.uniform(0, 1, 40),
                           rng.uniform(-0.06, -0.03, 40)])
    nrm = np.tile([0.0, 0.0, 1.0], (40, 1))
    boxes = [O.axis_box(center, (0.4, 0.4, 0.2)), O.axis_box([0.85, 0.2, center[2]], (0.2, 0.3, 0.2))]
    store("points16", tri, snaps, boxes, 2e-3, pts, nrm)
    x0, X, tri, center, snaps = S.drape_positions(128, 200, seed=2024)
    store("drape128", tri, [snaps[100], snaps[199]], [O.axis_box(center, (0.4, 0.4, 0.2))], 1e-3)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
