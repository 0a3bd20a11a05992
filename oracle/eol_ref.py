"""Oracle of an EOL step's constraint rows and QP — TEST INFRASTRUCTURE ONLY
(tests/ compare the library against it; nothing in the product imports it).

constraint_rows() restates Constraints::fill for a mesh with EOL nodes
(Constraints.cpp:135-468, boxes at rest or moving) in the reference's DOF
layout: the 3N Lagrangian DOFs, then two Eulerian DOFs per EOL node at
3N + 2k (EoL_index k).  It reads the mesh the way ArcSim's objects hold it:

  * Vert::adjf of a node = its faces in ascending order (Mesh::add(Face),
    mesh.cpp:365-378, appends each face to its vertices' lists);
  * Node::adje = its edges in mesh.edges order (Mesh::add(Edge), :336-342);
  * Face::n = normalize((x1 - x0) x (x2 - x0)) (compute_ws_data, :135-139);
  * Node::n = normal<WS>(node) (geometry.cpp:302-316);
  * get_angle(u, v) = acos(clamp(dot(u^, v^), -1, 1)) (geometry.cpp:392-394);
  * is_seam_or_boundary(edge) = an edge with fewer than two faces
    (util.cpp:146-150; one vertex per node, so no seams);
  * normalisation of a zero vector leaves it zero (ArcSim normalize,
    vectors.hpp:111, and Eigen's normalized()).

The constraint table follows Constraints::updateTable (:76-105) with the box
tables of Box.cpp:25-72 (face normals rotated by E1, corner normals from the
three edges' six faces, per edge its two faces and the face along it).  A
node on a moving box (Box::v = (w, v) not zero) gets the right-hand sides of
:165-172 and :270-277 from its point's velocity over the step,
xdot = (Rigid::integrate(E1, Box::v, h) xl - E1 xl) / h with xl = E1^-1 x
(Rigid.cpp:79-111, restated with numpy's matrix products).

solve_qp_eq() extends qp_ref.solve_qp with general equality rows: a primal
active-set method on the sparse KKT system whose working set always holds
the equality rows (zero rows, 0 = 0, are dropped).

step() is Cloth::step (Cloth.cpp:359-413) of an EOL mesh without remeshing:
pins beq = 0.99 v + c (addFixed, Constraints.cpp:114-119), Forces::fill with
the EOL branches (the oracle's orc_forces_fill_eol), b = -(M v + h f)
(Cloth.cpp:345), the QP, x += h v and u += h vE (Cloth.cpp:394-410).
"""
import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle as O

FACE_NORMALS = [(1.0, 0.0, 0.0), (-1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, -1.0, 0.0),
                (0.0, 0.0, 1.0), (0.0, 0.0, -1.0)]                      # Box.cpp:25-32
EDGE_FACES = [(1, 3), (1, 5), (1, 4), (1, 2), (3, 5), (3, 4), (0, 3), (2, 5), (0, 5), (2, 4),
              (0, 4), (0, 2)]                                            # Box.cpp:34-47
EDGE_TAN = [4, 2, 2, 4, 0, 0, 4, 0, 2, 0, 2, 4]                          # Box.cpp:49-62
VERT_EDGES = [(0, 1, 4), (0, 2, 5), (1, 3, 7), (2, 3, 9), (4, 6, 8), (5, 6, 10), (7, 8, 11),
              (9, 10, 11)]                                               # Box.cpp:64-72


def _norm(v):
    return math.sqrt(sum(c * c for c in v))


def _normalize(v):
    n = _norm(v)
    return [c / n for c in v] if n > 0 else list(v)


def _cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _dot(a, b):
    return sum(p * q for p, q in zip(a, b))


def constraint_table(boxes, point_normals):
    """9 x (n_points + 20 n_boxes) table of Constraints::updateTable."""
    pn = np.zeros((0, 3)) if point_normals is None else np.asarray(point_normals).reshape(-1, 3)
    cols = []
    for p in pn:
        cols.append(list(p) + [0.0] * 6)
    for box in boxes:
        E1 = np.array(list(box.E1)).reshape(4, 4, order="F")
        R = E1[:3, :3]
        fn = [[sum(R[i, k] * f[k] for k in range(3)) for i in range(3)] for f in FACE_NORMALS]
        for p in range(8):
            c = [0.0, 0.0, 0.0]
            for i in range(3):
                for j in range(2):
                    n = fn[EDGE_FACES[VERT_EDGES[p][i]][j]]
                    c = [c[k] + n[k] for k in range(3)]
            cols.append(_normalize([ck / 6.0 for ck in c]) + [0.0] * 6)
        for e in range(12):
            cols.append(fn[EDGE_FACES[e][0]] + fn[EDGE_FACES[e][1]] + fn[EDGE_TAN[e]])
    return np.array(cols, np.float64).reshape(-1, 9)


def rigid_integrate(E0, phi, h):
    """Rigid::integrate (Rigid.cpp:79-111): E0 times the screw motion of
    phi = (w, v) over h (Rodrigues rotation when |w| > 1e-10)."""
    w, v = np.array(phi[:3], float), np.array(phi[3:], float)
    P = np.eye(4)
    P[:3, 3] = h * v
    wlen = np.linalg.norm(w)
    if wlen > 1e-10:
        w, v = w / wlen, v / wlen
        K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
        c, s = np.cos(wlen * h), np.sin(wlen * h)
        R = c * np.eye(3) + s * K + (1 - c) * np.outer(w, w)
        P[:3, :3] = R
        P[:3, 3] = (w @ v) * wlen * h * w + (np.eye(3) - R) @ np.cross(w, v)
    return E0 @ P


def point_velocity(E1, phi, h, x):
    """xdot of Constraints.cpp:168-170 for a point x on a moving box."""
    Einv = np.eye(4)
    Einv[:3, :3] = E1[:3, :3].T
    Einv[:3, 3] = -E1[:3, :3].T @ E1[:3, 3]
    xl = Einv @ np.append(np.asarray(x, float), 1.0)
    return ((rigid_integrate(E1, phi, h) @ xl - E1 @ xl) / h)[:3]


class _Mesh:
    """The ArcSim adjacency that Constraints::fill walks."""

    def __init__(self, x, u, tri, edges, preserve):
        self.x = np.asarray(x, np.float64).reshape(-1, 3)
        self.u = np.asarray(u, np.float64).reshape(-1, 2)
        self.tri = np.asarray(tri, np.int64).reshape(-1, 3)
        self.edges = np.asarray(edges, np.int64).reshape(-1, 2)
        self.preserve = (np.zeros(len(self.edges), np.int64) if preserve is None
                         else np.asarray(preserve, np.int64))
        n = len(self.x)
        self.adjf = [[] for _ in range(n)]
        for f, t in enumerate(self.tri):
            for a in t:
                self.adjf[int(a)].append(f)
        self.adje = [[] for _ in range(n)]
        for e, (a, b) in enumerate(self.edges):
            self.adje[int(a)].append(e)
            self.adje[int(b)].append(e)
        count = {}
        for t in self.tri:
            for i in range(3):
                k = tuple(sorted((int(t[i]), int(t[(i + 1) % 3]))))
                count[k] = count.get(k, 0) + 1
        self.boundary = [count.get(tuple(sorted((int(a), int(b)))), 0) < 2 for a, b in self.edges]

    def face_n(self, f):
        x0, x1, x2 = (list(self.x[int(v)]) for v in self.tri[f])
        return _normalize(_cross([x1[k] - x0[k] for k in range(3)],
                                 [x2[k] - x0[k] for k in range(3)]))

    def node_n(self, a):
        n = [0.0, 0.0, 0.0]
        for f in self.adjf[a]:
            v = [int(t) for t in self.tri[f]]
            j = v.index(a)
            xa = list(self.x[a])
            e1 = [self.x[v[(j + 1) % 3]][k] - xa[k] for k in range(3)]
            e2 = [self.x[v[(j + 2) % 3]][k] - xa[k] for k in range(3)]
            c = _cross(e1, e2)
            s = 2 * _dot(e1, e1) * _dot(e2, e2)
            n = [n[k] + c[k] / s for k in range(3)]
        return _normalize(n)

    def flat(self, a, limit):
        fs = self.adjf[a]
        n0 = _normalize(self.face_n(fs[0]))
        for f in fs[1:]:
            n1 = _normalize(self.face_n(f))
            if math.acos(min(max(_dot(n0, n1), -1.0), 1.0)) > limit:
                return False
        return True


def constraint_rows(x, u, tri, edges, eol_nodes, corner_id, cd_edge, preserve=None, boxes=(),
                    point_normals=None, contacts=(), box_velocity=None, h=0.0):
    """(Aeq, beq, Aineq, bineq) of Constraints::fill without the pins, over
    the reference's 3N + 2E DOFs, rows in the reference's order.
    box_velocity: None or per box Box::v (w, v); h: the step."""
    M = _Mesh(x, u, tri, edges, preserve)
    N = len(M.x)
    n_eol = len(eol_nodes)
    eol_index = {int(a): k for k, a in enumerate(eol_nodes)}
    n_points = 0 if point_normals is None else len(np.asarray(point_normals).reshape(-1, 3))
    boxes = list(boxes)
    T = constraint_table(boxes, point_normals)
    eq, iq, beq, bineq = [], [], [], []

    def xdot(col, a):
        """The node's point velocity on the moving box of column col, or None."""
        if col < n_points or box_velocity is None:
            return None
        b = (col - n_points) // 20
        phi = np.asarray(box_velocity, float).reshape(-1, 6)[b]
        if np.linalg.norm(phi[:3]) == 0.0 and np.linalg.norm(phi[3:]) == 0.0:
            return None
        E1 = np.array(list(boxes[b].E1)).reshape(4, 4, order="F")
        return point_velocity(E1, phi, h, M.x[a])

    def node_row(rows, a, g, value=0.0):
        rows.append([(3 * a + c, g[c]) for c in range(3)])
        (beq if rows is eq else bineq).append(value)

    for a in range(N):
        if a not in eol_index:
            continue
        k = eol_index[a]
        cid = int(corner_id[k])
        if cid >= 0:                                       # :148-262
            nor = list(T[cid, 0:3])
            o1 = [0.0, -nor[2], nor[1]]
            o2 = _normalize(_normalize(_cross(o1, nor)))
            xd = xdot(cid, a)
            r = (lambda g, sgn: 0.0 if xd is None else sgn * float(np.dot(g, xd)))
            if M.flat(a, 0.5) or cid < n_points:
                node_row(iq, a, [-c for c in nor], value=r(nor, -1))
                node_row(eq, a, o1, value=r(o1, 1))
                node_row(eq, a, o2, value=r(o2, 1))
            else:
                node_row(iq, a, [-c for c in nor], value=r(nor, -1))
                node_row(iq, a, [-c for c in o1], value=r(o1, 1))
                node_row(iq, a, [-c for c in o2], value=r(o2, 1))
            continue
        cd = int(cd_edge[k])                               # :263-415
        xd = xdot(cd, a)
        r = (lambda g: 0.0 if xd is None else -float(np.dot(g, xd)))
        if M.flat(a, 0.1):
            n = M.node_n(a)
            fc = _cross(n, list(T[cd, 6:9]))
            node_row(iq, a, [-c for c in n], value=r(n))
            node_row(eq, a, [-c for c in fc], value=r(fc))
        else:
            node_row(iq, a, [-c for c in T[cd, 0:3]], value=r(T[cd, 0:3]))
            node_row(iq, a, [-c for c in T[cd, 3:6]], value=r(T[cd, 3:6]))
        bnd = [e for e in M.adje[a] if M.boundary[e]]
        if bnd:
            e = bnd[0]
            o = int(M.edges[e][1]) if int(M.edges[e][0]) == a else int(M.edges[e][0])
            g = _normalize([M.u[a][1] - M.u[o][1], -M.u[a][0] - M.u[o][0]])
        else:
            t = [0.0, 0.0]
            for e in M.adje[a]:
                if not M.preserve[e]:
                    continue
                n0, n1 = int(M.edges[e][0]), int(M.edges[e][1])
                u0, u1 = list(M.u[n0]) + [0.0], list(M.u[n1]) + [0.0]
                if _norm(u0) > _norm(u1):
                    d = _normalize([u1[0] - u0[0], u1[1] - u0[1]])
                else:
                    d = _normalize([u0[0] - u1[0], u0[1] - u1[1]])
                t = [t[0] + d[0], t[1] + d[1]]
            g = _normalize(t)
        eq.append([(3 * N + 2 * k, g[0]), (3 * N + 2 * k + 1, g[1])])
        beq.append(0.0)
    for c in contacts:                                     # :422-468
        if c.count1 == 3 and c.count2 == 1:
            terms = [(c.verts2[0], [-v for v in c.nor1])]
        elif c.count1 == 2 and c.count2 == 2:
            terms = [(c.verts2[j], [-v * c.weights2[j] for v in c.nor2]) for j in range(2)]
        elif c.count1 == 1 and c.count2 == 3:
            terms = [(c.verts2[j], [-v * c.weights2[j] for v in c.nor2]) for j in range(3)]
        else:
            continue
        if any(int(vtx) in eol_index for vtx, _ in terms):
            continue
        iq.append([(3 * int(vtx) + i, g[i]) for vtx, g in terms for i in range(3)])
        bineq.append(0.0)
    n_dofs = 3 * N + 2 * n_eol

    def csr(rows):
        r = [i for i, row in enumerate(rows) for _ in row]
        cidx = [d for row in rows for d, _ in row]
        v = [g for row in rows for _, g in row]
        return sp.csr_matrix((v, (r, cidx)), shape=(len(rows), n_dofs))

    return csr(eq), np.array(beq, float), csr(iq), np.array(bineq, float)


def solve_qp_eq(A, b, fixed_dofs, beq, Aeq, e, C, d, max_iter=None):
    """Exact minimiser of 1/2 v'Av + b'v s.t. v[fixed] = beq, Aeq v = e,
    C v <= d (primal active set; equality rows always in the working set).
    Returns (v, lam_eq, lam_ineq, iterations): A v + b + Aeq' lam_eq +
    C' lam_ineq = 0 on the free DOFs, lam_ineq >= 0."""
    A = sp.csr_matrix(A)
    n = A.shape[0]
    Aeq, C = sp.csr_matrix(Aeq), sp.csr_matrix(C)
    keep = np.flatnonzero(np.abs(Aeq).sum(axis=1).A1 > 0)
    fixed = np.asarray(fixed_dofs, np.int64)
    free = np.setdiff1d(np.arange(n), fixed)
    vfix = np.zeros(n)
    vfix[fixed] = beq
    Aff = A[free][:, free].tocsc()
    rhs = -(b + A @ vfix)[free]
    Ef = Aeq[keep][:, free].tocsr()
    ee = (np.asarray(e, np.float64) - Aeq @ vfix)[keep]
    Cf = C[:, free].tocsr()
    dd = d - C @ vfix
    m, me = C.shape[0], len(keep)
    scale = max(1.0, float(np.abs(rhs).max()))
    W = []
    max_iter = max_iter or 5 * m + 20
    for it in range(max_iter):
        G = sp.vstack([Ef, Cf[W]]).tocsr() if W else Ef
        K = sp.bmat([[Aff, G.T], [G, None]]).tocsc() if G.shape[0] else Aff
        sol = spla.spsolve(K, np.concatenate([rhs, ee, dd[W]]))
        vf, le, lw = sol[:len(free)], sol[len(free):len(free) + me], sol[len(free) + me:]
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
            lam_eq = np.zeros(Aeq.shape[0])
            lam_eq[keep] = le
            lam = np.zeros(m)
            lam[W] = np.maximum(lw, 0.0)
            return v, lam_eq, lam, it
        W.append(k)
    raise RuntimeError("active set did not converge in %d iterations" % max_iter)


def step(x, u, v, tri, hinge, eol_nodes, mat, grav, h, fixed_dofs, fixed_vel, rows):
    """One EOL Cloth::step in the reference layout: x (3N), u (2N) and v
    (3N + 2E) are updated in place; rows = (Aeq, beq, Aineq, bineq) of
    constraint_rows on the step's state.  Returns (lam_eq, lam_ineq)."""
    F = O.ForcesEOL(x, u, tri, hinge, mat, grav, h, eol_nodes)
    M, MDK, f = F.csr(0), F.csr(1), F.f()
    b = -(M @ v + h * f)
    fixed = np.asarray(fixed_dofs, np.int64)
    beq = (1 - 0.01) * v[fixed] + np.asarray(fixed_vel, np.float64)
    Aeq, e, C, d = rows
    vn, le, li, _ = solve_qp_eq(MDK, b, fixed, beq, Aeq, e, C, d)
    v[:] = vn
    N = len(x) // 3
    x += h * v[:3 * N]
    for k, a in enumerate(eol_nodes):
        u[2 * a] = u[2 * a] + h * v[3 * N + 2 * k]
        u[2 * a + 1] = u[2 * a + 1] + h * v[3 * N + 2 * k + 1]
    return le, li
