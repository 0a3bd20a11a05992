"""ctypes front end of the CPU oracle (oracle/*.cpp -> oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY.  tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use it to compare against; the product library never imports it.
The C++ sources restate the reference's hot path (file:line citations in each
function); see oracle/oracle.h for what is pinned and how.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SOURCES = ["mesh.cpp", "elements.cpp", "assemble.cpp", "collide.cpp", "export.cpp"]


def build(force=False):
    """Compile the oracle with FP contraction off (same results on x86/Arm)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    hdrs = [os.path.join(HERE, h) for h in ("oracle.h", "vec3.h")]
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= t for s in srcs + hdrs):
            return LIB_PATH
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-o", LIB_PATH] + srcs
    subprocess.check_call(cmd)
    return LIB_PATH


class Contact(ctypes.Structure):
    """Layout of eolc_contact (include/eolc.h)."""
    _fields_ = [
        ("dist", ctypes.c_double),
        ("nor1", ctypes.c_double * 3),
        ("nor2", ctypes.c_double * 3),
        ("pos1", ctypes.c_double * 3),
        ("pos2", ctypes.c_double * 3),
        ("pos1_", ctypes.c_double * 3),
        ("weights1", ctypes.c_double * 3),
        ("weights2", ctypes.c_double * 3),
        ("edge_dir", ctypes.c_double * 3),
        ("count1", ctypes.c_int),
        ("count2", ctypes.c_int),
        ("verts1", ctypes.c_int * 3),
        ("verts2", ctypes.c_int * 3),
        ("tri1", ctypes.c_int),
        ("tri2", ctypes.c_int),
        ("edge1", ctypes.c_int * 3),
        ("n_edge1", ctypes.c_int),
        ("edge2", ctypes.c_int),
        ("source", ctypes.c_int),
    ]


class Box(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_double * 3), ("E1", ctypes.c_double * 16)]


class Material(ctypes.Structure):
    _fields_ = [("density", ctypes.c_double), ("e", ctypes.c_double),
                ("nu", ctypes.c_double), ("beta", ctypes.c_double),
                ("damping_a", ctypes.c_double), ("damping_b", ctypes.c_double)]


_lib = None
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_forces_fill.restype = ctypes.c_void_p
        L.orc_forces_fill.argtypes = [ctypes.c_int, _D, _D, _I, ctypes.c_int, _I,
                                      ctypes.c_int, ctypes.POINTER(Material), _D,
                                      ctypes.c_double]
        L.orc_forces_free.argtypes = [ctypes.c_void_p]
        L.orc_forces_nnz.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_forces_csr.argtypes = [ctypes.c_void_p, ctypes.c_int, _I, _I, _D]
        L.orc_forces_f.argtypes = [ctypes.c_void_p, _D]
        L.orc_rhs.argtypes = [ctypes.c_void_p, _D, ctypes.c_double, _D]
        L.orc_velocity_solve.argtypes = [ctypes.c_void_p, _D, _I, _D, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_int, _D, _D]
        L.orc_velocity_solve_direct.argtypes = [ctypes.c_void_p, _D, _I, _D,
                                                ctypes.c_int, _D]
        L.orc_step.argtypes = [ctypes.c_int, _D, _D, _D, _I, ctypes.c_int, _I,
                               ctypes.c_int, ctypes.POINTER(Material), _D,
                               ctypes.c_double, _I, _D, ctypes.c_int,
                               ctypes.c_double, ctypes.c_int, _D]
        L.orc_cd2.argtypes = [ctypes.c_int, _D, _I, ctypes.c_int,
                              ctypes.POINTER(Box), ctypes.c_int, _D, _D,
                              ctypes.c_int, ctypes.c_double,
                              ctypes.POINTER(Contact), ctypes.c_int]
        L.orc_create_edges.argtypes = [ctypes.c_int, _D, _I, ctypes.c_int, _I,
                                       ctypes.c_int]
        L.orc_hinges.argtypes = [ctypes.c_int, _I, ctypes.c_int, _I, ctypes.c_int]
        L.orc_forces_fill_eol.restype = ctypes.c_void_p
        L.orc_forces_fill_eol.argtypes = [ctypes.c_int, _D, _D, _I, ctypes.c_int, _I,
                                          ctypes.c_int, ctypes.POINTER(Material), _D,
                                          ctypes.c_double, _I, ctypes.c_int]
        L.orc_obj_text.argtypes = [ctypes.c_int, _D, _D, _I, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_char_p, ctypes.c_longlong,
                                   ctypes.POINTER(ctypes.c_longlong)]
        L.orc_node_normals.argtypes = [ctypes.c_int, _D, _I, ctypes.c_int, _D]
        for name in ("orc_grid2_build", "orc_gridc_build"):
            getattr(L, name).argtypes = [ctypes.c_int, ctypes.c_int, _D, _D, _D, _I]
        _lib = L
    return _lib


def dp(a):
    return a.ctypes.data_as(_D)


def ip(a):
    return a.ctypes.data_as(_I)


# JSON-file corner convention of simulationSettings*.json: corner1 (0,0),
# corner2 (1,0), corner3 (0,1), corner4 (1,1) as (x, y, z, X, Y).
UNIT_CORNERS = np.array([[0, 0, 0, 0, 0], [1, 0, 0, 1, 0],
                         [0, 1, 0, 0, 1], [1, 1, 0, 1, 1]], dtype=np.float64)


def grid2(r0, r1, corners=UNIT_CORNERS):
    """Two-triangle-per-quad grid of r0 x r1 nodes -> (x, X, tri)."""
    n, t = r0 * r1, 2 * (r0 - 1) * (r1 - 1)
    x = np.zeros(3 * n); X = np.zeros(2 * n); tri = np.zeros(3 * t, np.int32)
    c = np.ascontiguousarray(corners, dtype=np.float64).ravel()
    lib().orc_grid2_build(r0, r1, dp(c), dp(x), dp(X), ip(tri))
    return x, X, tri.reshape(-1, 3)


def gridc(r0, r1, corners=UNIT_CORNERS):
    """The reference's centre-node grid (Cloth.cpp:63-126)."""
    n, t = r0 * r1 + (r0 - 1) * (r1 - 1), 4 * (r0 - 1) * (r1 - 1)
    x = np.zeros(3 * n); X = np.zeros(2 * n); tri = np.zeros(3 * t, np.int32)
    c = np.ascontiguousarray(corners, dtype=np.float64).ravel()
    lib().orc_gridc_build(r0, r1, dp(c), dp(x), dp(X), ip(tri))
    return x, X, tri.reshape(-1, 3)


def hinges(n_nodes, tri):
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    cap = 3 * len(tri)
    out = np.zeros(4 * cap, np.int32)
    n = lib().orc_hinges(n_nodes, ip(tri), len(tri), ip(out), cap)
    return out[:4 * n].reshape(-1, 4)


def corner_ids(r0, r1):
    """Pinned corner node ids of load_clothset (parseParams.cpp:298-305)."""
    return {1: 0, 2: r0 * (r1 - 1), 3: r0 * r1 - 1, 4: r0 - 1}


def membrane(x9, X6, e, nu, P6, Q4):
    W = np.zeros(1); f = np.zeros(9); K = np.zeros(81)
    lib().orc_membrane(dp(x9), dp(X6), ctypes.c_double(e), ctypes.c_double(nu),
                       dp(P6), dp(Q4), dp(W), dp(f), dp(K))
    return W[0], f, K.reshape(9, 9)


def face_frame(x9, X6):
    P = np.zeros(6); Q = np.zeros(4)
    lib().orc_face_frame(dp(x9), dp(X6), dp(P), dp(Q))
    return P, Q


def inertial(x9, X6, g, rho):
    W = np.zeros(1); f = np.zeros(9); M = np.zeros(81)
    g = np.ascontiguousarray(g, dtype=np.float64)
    lib().orc_inertial(dp(x9), dp(X6), dp(g), ctypes.c_double(rho), dp(W), dp(f), dp(M))
    return W[0], f, M.reshape(9, 9)


def bending(x12, X8, beta):
    W = np.zeros(1); f = np.zeros(12); K = np.zeros(144)
    lib().orc_bending(dp(x12), dp(X8), ctypes.c_double(beta), dp(W), dp(f), dp(K))
    return W[0], f, K.reshape(12, 12)


def raytri(orig, d, v0, v1, v2):
    tuv = np.zeros(3)
    arr = [np.ascontiguousarray(a, dtype=np.float64) for a in (orig, d, v0, v1, v2)]
    hit = lib().orc_raytri(*[dp(a) for a in arr], dp(tuv))
    return hit, tuv


def material(density=0.1, e=50.0, nu=0.3, beta=1e-5, damping=(0.0, 1.0)):
    return Material(density, e, nu, beta, damping[0], damping[1])


class Forces:
    """Forces::fill result: f, M and MDK as scipy CSR (3N x 3N)."""

    def __init__(self, x, X, tri, hinge, mat, grav, h):
        self.n_nodes = len(x) // 3
        tri = np.ascontiguousarray(tri, dtype=np.int32)
        hinge = np.ascontiguousarray(hinge, dtype=np.int32)
        g = np.ascontiguousarray(grav, dtype=np.float64)
        L = lib()
        self._h = L.orc_forces_fill(self.n_nodes, dp(x), dp(X), ip(tri), len(tri),
                                    ip(hinge), len(hinge), ctypes.byref(mat), dp(g),
                                    ctypes.c_double(h))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_forces_free(self._h)
            self._h = None

    @property
    def n_dofs(self):
        return 3 * self.n_nodes + 2 * getattr(self, "n_eol", 0)

    def f(self):
        out = np.zeros(self.n_dofs)
        lib().orc_forces_f(self._h, dp(out))
        return out

    def csr(self, which):
        import scipy.sparse as sp
        n = self.n_dofs
        nnz = lib().orc_forces_nnz(self._h, which)
        rp = np.zeros(n + 1, np.int32); c = np.zeros(nnz, np.int32); v = np.zeros(nnz)
        lib().orc_forces_csr(self._h, which, ip(rp), ip(c), dp(v))
        return sp.csr_matrix((v, c, rp), shape=(n, n))

    def rhs(self, v, h):
        b = np.zeros(3 * self.n_nodes)
        lib().orc_rhs(self._h, dp(np.ascontiguousarray(v, dtype=np.float64)),
                      ctypes.c_double(h), dp(b))
        return b

    def solve(self, b, fixed_dofs, beq, tol=1e-8, max_iter=100000):
        fixed_dofs = np.ascontiguousarray(fixed_dofs, dtype=np.int32)
        beq = np.ascontiguousarray(beq, dtype=np.float64)
        v = np.zeros(3 * self.n_nodes); rr = np.zeros(1)
        it = lib().orc_velocity_solve(self._h, dp(b), ip(fixed_dofs), dp(beq),
                                      len(fixed_dofs), ctypes.c_double(tol), max_iter,
                                      dp(v), dp(rr))
        return v, it, rr[0]

    def solve_direct(self, b, fixed_dofs, beq):
        fixed_dofs = np.ascontiguousarray(fixed_dofs, dtype=np.int32)
        beq = np.ascontiguousarray(beq, dtype=np.float64)
        v = np.zeros(3 * self.n_nodes)
        rc = lib().orc_velocity_solve_direct(self._h, dp(b), ip(fixed_dofs), dp(beq),
                                             len(fixed_dofs), dp(v))
        if rc != 0:
            raise RuntimeError("direct solve failed (%d)" % rc)
        return v


class ForcesEOL(Forces):
    """Forces::fill with EOL nodes: eol_nodes[k] is the node of EoL_index k;
    f, M, MDK over the 3N + 2E DOFs (Eulerian DOFs of k at 3N + 2k)."""

    def __init__(self, x, X, tri, hinge, mat, grav, h, eol_nodes):
        self.n_nodes = len(x) // 3
        self.n_eol = len(eol_nodes)
        idx = -np.ones(self.n_nodes, np.int32)
        idx[np.asarray(eol_nodes, np.int64)] = np.arange(self.n_eol, dtype=np.int32)
        tri = np.ascontiguousarray(tri, dtype=np.int32)
        hinge = np.ascontiguousarray(hinge, dtype=np.int32)
        g = np.ascontiguousarray(grav, dtype=np.float64)
        self._h = lib().orc_forces_fill_eol(self.n_nodes, dp(x), dp(X), ip(tri), len(tri),
                                            ip(hinge), len(hinge), ctypes.byref(mat), dp(g),
                                            ctypes.c_double(h), ip(idx), self.n_eol)


def step(x, X, v, tri, hinge, mat, grav, h, fixed_dofs, fixed_vel, tol=1e-8,
         max_iter=100000):
    """One Cloth::step; x and v (float64 arrays) are updated in place."""
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    hinge = np.ascontiguousarray(hinge, dtype=np.int32)
    fixed_dofs = np.ascontiguousarray(fixed_dofs, dtype=np.int32)
    fixed_vel = np.ascontiguousarray(fixed_vel, dtype=np.float64)
    g = np.ascontiguousarray(grav, dtype=np.float64)
    rr = np.zeros(1)
    it = lib().orc_step(len(x) // 3, dp(x), dp(X), dp(v), ip(tri), len(tri),
                        ip(hinge), len(hinge), ctypes.byref(mat), dp(g),
                        ctypes.c_double(h), ip(fixed_dofs), dp(fixed_vel),
                        len(fixed_dofs), ctypes.c_double(tol), max_iter, dp(rr))
    return it, rr[0]


def axis_box(center, dim):
    """Axis-aligned box obstacle: E1 = translation to center."""
    E1 = np.eye(4)
    E1[:3, 3] = center
    return Box((ctypes.c_double * 3)(*dim),
               (ctypes.c_double * 16)(*E1.flatten(order="F")))


def cd2(x, tri, boxes=(), points=None, normals=None, threshold=1e-3, cap=None, raw=False):
    """CD2 (Collisions.cpp:55-78) of the restated boxTriCollision: the
    contact list, or with raw=True the contacts' bytes in order."""
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    n_nodes = len(x) // 3
    pts = np.zeros(3) if points is None else np.ascontiguousarray(points, np.float64)
    nrm = np.zeros(3) if normals is None else np.ascontiguousarray(normals, np.float64)
    npts = 0 if points is None else len(pts.reshape(-1, 3))
    boxes = list(boxes)
    barr = (Box * max(1, len(boxes)))(*boxes)
    cap = cap or (4 * n_nodes + 64)
    out = (Contact * cap)()
    n = lib().orc_cd2(n_nodes, dp(x), ip(tri), len(tri), barr, len(boxes), dp(pts),
                      dp(nrm), npts, ctypes.c_double(threshold), out, cap)
    if n > cap:
        return cd2(x, tri, boxes, points, normals, threshold, cap=n, raw=raw)
    if raw:
        return ctypes.string_at(out, ctypes.sizeof(Contact) * n)
    return [out[k] for k in range(n)]


def create_edges(x, tri):
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    cap = 3 * len(tri)
    out = np.zeros(6 * cap, np.int32)
    n = lib().orc_create_edges(len(x) // 3, dp(x), ip(tri), len(tri), ip(out), cap)
    return out[:6 * n].reshape(-1, 6)


def obj_text(x, X, tri, frame=0, time=0.0):
    """The (Cloth2D, Cloth3D) OBJ files of one frame as bytes, formatted as
    BrenderManager::exportBrender + Cloth::exportBrender write them."""
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    x = np.ascontiguousarray(x, np.float64)
    X = np.ascontiguousarray(X, np.float64)
    n = len(x) // 3
    ln = (ctypes.c_longlong * 2)()
    lib().orc_obj_text(n, dp(x), dp(X), ip(tri), len(tri.reshape(-1, 3)), frame,
                       ctypes.c_double(time), None, 0, ln)
    buf = ctypes.create_string_buffer(ln[0] + ln[1])
    assert lib().orc_obj_text(n, dp(x), dp(X), ip(tri), len(tri.reshape(-1, 3)), frame,
                              ctypes.c_double(time), buf, ln[0] + ln[1], ln) == 0
    raw = buf.raw
    return raw[:ln[0]], raw[ln[0]:ln[0] + ln[1]]


def node_normals(x, tri):
    """ArcSim normal<WS> of every node, FP64 (3N)."""
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    x = np.ascontiguousarray(x, np.float64)
    out = np.zeros(len(x))
    lib().orc_node_normals(len(x) // 3, dp(x), ip(tri), len(tri.reshape(-1, 3)), dp(out))
    return out
