"""Generate the element golden vectors in tests/golden/elements.npz.

Runs the reference's OWN element routines (ComputeMembrane, ComputeBending,
ComputeInertial, intersect_triangle3_inc), compiled in place from the
reference sources by oracle/build_ref.sh into oracle/_ref/libeolc_ref.so, on
seeded inputs and stores inputs + outputs.  The committed .npz pins the
oracle's restated element math (tests/test_oracle_golden.py) on machines
where the reference sources are absent.

Usage (from the repository root, where the reference sources are present):
    oracle/build_ref.sh && python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402  (face frame used to build consistent P, Q)

REF = os.path.join(ROOT, "oracle", "_ref", "libeolc_ref.so")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "elements.npz")
_D = ctypes.POINTER(ctypes.c_double)


def dp(a):
    return a.ctypes.data_as(_D)


def main():
    L = ctypes.CDLL(REF)
    rng = np.random.default_rng(20181108)
    out = {}

    # ---- membrane: P, Q from the face frame of Forces.cpp:355-368 --------
    cases = []
    for k in range(96):
        X = rng.uniform(0, 0.05, 6)
        if k % 8 == 7:  # clockwise material triangle (negative signed area)
            X[2:4], X[4:6] = X[4:6].copy(), X[2:4].copy()
        x = np.concatenate([np.append(X[2 * i:2 * i + 2], 0.0) for i in range(3)])
        th = rng.uniform(0, 2 * np.pi)
        Rz = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
        S = np.eye(3) + rng.normal(0, 0.2 if k % 3 else 0.02, (3, 3))
        x = (x.reshape(3, 3) @ (Rz @ S).T).ravel() + rng.normal(0, 0.002, 9)
        if k % 16 == 5:  # inverted in-plane configuration (det Fbar < 0)
            x = x.reshape(3, 3); x[:, 0] *= -1; x = x.ravel()
        cases.append((x, X))
    mx, mX, mP, mQ, mW, mf, mK, me, mnu = [], [], [], [], [], [], [], [], []
    for i, (x, X) in enumerate(cases):
        P, Q = O.face_frame(x, X)
        e = [50.0, 20.0, 100.0, 5e3][i % 4]
        nu = [0.3, 0.01, 0.45, 0.2][(i // 4) % 4]
        W = np.zeros(1); f = np.zeros(9); K = np.zeros(81)
        L.ref_membrane(dp(x), dp(X), ctypes.c_double(e), ctypes.c_double(nu),
                       dp(P), dp(Q), dp(W), dp(f), dp(K))
        mx.append(x); mX.append(X); mP.append(P); mQ.append(Q)
        mW.append(W[0]); mf.append(f); mK.append(K); me.append(e); mnu.append(nu)
    out.update(mem_x=np.array(mx), mem_X=np.array(mX), mem_P=np.array(mP),
               mem_Q=np.array(mQ), mem_e=np.array(me), mem_nu=np.array(mnu),
               mem_W=np.array(mW), mem_f=np.array(mf), mem_K=np.array(mK))

    # ---- bending: hinge stencil x0-x1 edge, x2 / x3 apexes -----------------
    bx, bX, bb, bW, bf, bK = [], [], [], [], [], []
    for k in range(96):
        h = rng.uniform(0.005, 0.05)
        X = np.array([0, 0, h, 0, 0.5 * h, 0.8 * h, 0.4 * h, -0.7 * h])
        X = X + rng.normal(0, 0.1 * h, 8)
        x = np.concatenate([np.append(X[2 * i:2 * i + 2], 0.0) for i in range(4)])
        if k % 4 == 0:  # nearly flat
            x = x + rng.normal(0, 1e-4 * h, 12)
        elif k % 4 == 1:  # strongly folded
            x[11] += rng.uniform(0.5, 2.0) * h
            x[8] -= rng.uniform(0.5, 2.0) * h
        else:
            x = x + rng.normal(0, 0.2 * h, 12)
        beta = [1e-5, 1e-3, 1.0][k % 3]
        W = np.zeros(1); f = np.zeros(12); K = np.zeros(144)
        L.ref_bending(dp(x), dp(X), ctypes.c_double(beta), dp(W), dp(f), dp(K))
        bx.append(x); bX.append(X); bb.append(beta); bW.append(W[0]); bf.append(f); bK.append(K)
    out.update(bend_x=np.array(bx), bend_X=np.array(bX), bend_beta=np.array(bb),
               bend_W=np.array(bW), bend_f=np.array(bf), bend_K=np.array(bK))

    # ---- inertial -----------------------------------------------------------
    ix, iX, ig, irho, iW, i_f, iM = [], [], [], [], [], [], []
    for k in range(32):
        X = rng.uniform(0, 0.1, 6)
        x = rng.normal(0, 0.1, 9)
        g = rng.normal(0, 5, 3) if k % 2 else np.array([0.0, 0.0, -9.8])
        rho = [0.1, 0.05, 1.3, 1e-3][k % 4]
        W = np.zeros(1); f = np.zeros(9); M = np.zeros(81)
        L.ref_inertial(dp(x), dp(X), dp(g), ctypes.c_double(rho), dp(W), dp(f), dp(M))
        ix.append(x); iX.append(X); ig.append(g); irho.append(rho)
        iW.append(W[0]); i_f.append(f); iM.append(M)
    out.update(iner_x=np.array(ix), iner_X=np.array(iX), iner_g=np.array(ig),
               iner_rho=np.array(irho), iner_W=np.array(iW), iner_f=np.array(i_f),
               iner_M=np.array(iM))

    # ---- ray-triangle (inclusive-border variant used by intersect_square) --
    ro, rd, rv, rhit, rtuv = [], [], [], [], []
    for k in range(512):
        v = rng.uniform(-1, 1, 9)
        o = rng.uniform(-1, 1, 3)
        if k % 4 == 0:  # aim at a point on or near an edge / vertex
            a, b = rng.uniform(0, 1, 2)
            w = [a, b, 1 - a - b] if k % 8 == 0 else [0.0, b, 1 - b]
            tgt = w[0] * v[0:3] + w[1] * v[3:6] + w[2] * v[6:9]
            d = tgt - o
        elif k % 4 == 1:  # parallel to the triangle plane
            n = np.cross(v[3:6] - v[0:3], v[6:9] - v[0:3])
            d = np.cross(n, rng.normal(size=3))
        else:
            tgt = rng.dirichlet([1, 1, 1]) @ v.reshape(3, 3)
            d = (tgt - o) * rng.uniform(0.2, 3)
        tuv = np.full(3, np.nan)
        hit = L.ref_raytri(dp(o), dp(d), dp(v[0:3].copy()), dp(v[3:6].copy()),
                           dp(v[6:9].copy()), dp(tuv))
        ro.append(o); rd.append(d); rv.append(v); rhit.append(hit); rtuv.append(tuv)
    out.update(ray_o=np.array(ro), ray_d=np.array(rd), ray_v=np.array(rv),
               ray_hit=np.array(rhit, np.int32), ray_tuv=np.array(rtuv))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, {k: v.shape for k, v in out.items() if k.endswith(("_K", "_hit"))})


if __name__ == "__main__":
    main()
