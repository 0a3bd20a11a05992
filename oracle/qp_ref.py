"""Oracle of the contact-constrained velocity solve — TEST INFRASTRUCTURE ONLY
(tests/ and bench.py's CPU baseline compare against it).

GeneralizedSolver::velocitySolve with collisions (GeneralizedSolver.cpp:
138-170) hands Mosek or Gurobi the QP of QuadProg.h (MATLAB quadprog
convention, QuadProg.h:8-9):

    min_v 1/2 v' MDK v + b' v   s.t.   Aeq v = beq,   Aineq v <= bineq.

Neither solver is available, and the QP is strictly convex (MDK is SPD), so
its minimiser v is unique and any exact QP method reproduces what they
return; the multipliers are unique when the active rows are independent.
This oracle is a primal active-set method on the sparse KKT system
(scipy's sparse LU, FP64), with the pinned DOFs eliminated exactly as the
equality rows of addFixed (Constraints.cpp:114-119).

contact_rows() restates the inequality rows that Constraints::fill builds
from the CD2 contacts of a non-EOL mesh (Constraints.cpp:422-468): box face
against cloth vertex -> -nor1 on the vertex; edge against edge -> -nor2 w_j
on the two cloth vertices; box corner or point against cloth face -> -nor2
w_j on the three cloth vertices; bineq = 0.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def contact_rows(contacts, n_nodes):
    """(Aineq as CSR over the 3N DOFs, bineq) in contact order."""
    rows, cols, vals = [], [], []
    m = 0
    for c in contacts:
        if c.count1 == 3 and c.count2 == 1:
            terms = [(c.verts2[0], -np.array(c.nor1[:]))]
        elif c.count1 == 2 and c.count2 == 2:
            terms = [(c.verts2[j], -np.array(c.nor2[:]) * c.weights2[j]) for j in range(2)]
        elif c.count1 == 1 and c.count2 == 3:
            terms = [(c.verts2[j], -np.array(c.nor2[:]) * c.weights2[j]) for j in range(3)]
        else:
            continue
        for vtx, g in terms:
            for k in range(3):
                rows.append(m)
                cols.append(3 * vtx + k)
                vals.append(g[k])
        m += 1
    C = sp.csr_matrix((vals, (rows, cols)), shape=(m, 3 * n_nodes))
    return C, np.zeros(m)


def solve_qp(A, b, fixed_dofs, beq, C, d, max_iter=None):
    """Exact minimiser of 1/2 v'Av + b'v s.t. v[fixed] = beq, C v <= d.

    Returns (v, lam, iterations); lam >= 0 are the inequality multipliers
    (A v + b + C' lam = 0 on the free DOFs)."""
    A = sp.csr_matrix(A)
    n = A.shape[0]
    C = sp.csr_matrix(C)
    m = C.shape[0]
    fixed = np.asarray(fixed_dofs, np.int64)
    free = np.setdiff1d(np.arange(n), fixed)
    vfix = np.zeros(n)
    vfix[fixed] = beq
    Aff = A[free][:, free].tocsc()
    rhs = -(b + A @ vfix)[free]
    Cf = C[:, free].tocsr()
    dd = d - C @ vfix
    scale = max(1.0, float(np.abs(rhs).max()))
    W = []
    max_iter = max_iter or 5 * m + 20
    for it in range(max_iter):
        if W:
            K = sp.bmat([[Aff, Cf[W].T], [Cf[W], None]]).tocsc()
            sol = spla.spsolve(K, np.concatenate([rhs, dd[W]]))
            vf, lw = sol[:len(free)], sol[len(free):]
        else:
            vf, lw = spla.spsolve(Aff, rhs), np.zeros(0)
        if len(lw) and lw.min() < -1e-13 * max(scale, np.abs(lw).max()):
            W.pop(int(np.argmin(lw)))
            continue
        viol = Cf @ vf - dd
        if W:
            viol[W] = -np.inf
        k = int(np.argmax(viol)) if m else 0
        if m == 0 or viol[k] <= 1e-13 * max(1.0, np.abs(vf).max()):
            v = vfix.copy()
            v[free] = vf
            lam = np.zeros(m)
            lam[W] = np.maximum(lw, 0.0)
            return v, lam, it
        W.append(k)
    raise RuntimeError("active set did not converge in %d iterations" % max_iter)


def kkt_residuals(A, b, fixed_dofs, v, C, d, lam):
    """Relative stationarity, feasibility and complementarity of (v, lam)."""
    n = A.shape[0]
    free = np.setdiff1d(np.arange(n), np.asarray(fixed_dofs, np.int64))
    g = (A @ v + b + C.T @ lam)[free]
    r = C @ v - d
    sv = max(1e-300, np.abs(v).max())
    return (np.abs(g).max() / max(1e-300, np.abs(b[free]).max()),
            max(0.0, r.max(initial=0.0)) / sv,
            np.abs(lam * r).max(initial=0.0) / max(1e-300, np.abs(lam).max(initial=0.0) * sv))
