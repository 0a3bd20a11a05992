"""Python front end of libeolc.so (the GB300 hot path of EOL-Cloth).

Two layers:
  * Context: a thin ctypes binding of the C ABI in include/eolc.h.
  * Forces / GeneralizedSolver / Cloth / CD2: the reference's call surface
    (src/Forces.h:26-45, src/GeneralizedSolver.h:26-30, src/Cloth.h:75-76,
    src/Collisions.h:9-11) on top of it, with numpy/scipy containers where
    the reference has Eigen ones.

There is no CPU fallback: importing this module without a built
libeolc.so raises, and every call goes to the GPU.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libeolc.so")

(OK, NOT_CONVERGED, BREAKDOWN, NONFINITE, TIMEOUT, BAD_ARG, CUDA_ERROR, CAPACITY, NO_TOPOLOGY,
 IO_ERROR) = range(10)
PREC_FP64, PREC_MIXED = 0, 1
PC_JACOBI, PC_BLOCK_JACOBI, PC_LEARNED, PC_PATCH = 0, 1, 2, 3
STATUS_NAMES = ["OK", "NOT_CONVERGED", "BREAKDOWN", "NONFINITE", "TIMEOUT", "BAD_ARG",
                "CUDA_ERROR", "CAPACITY", "NO_TOPOLOGY", "IO_ERROR"]


class EolcError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else status, msg))
        self.status = status


class Material(ctypes.Structure):
    """src/Cloth.h:28-35."""
    _fields_ = [("density", ctypes.c_double), ("e", ctypes.c_double), ("nu", ctypes.c_double),
                ("beta", ctypes.c_double), ("damping_a", ctypes.c_double),
                ("damping_b", ctypes.c_double)]

    def __init__(self, density=0.05, e=50.0, nu=0.01, beta=1e-5, damping=(0.0, 1.0)):
        # defaults of load_matset (parseParams.cpp:193-201)
        super().__init__(density, e, nu, beta, damping[0], damping[1])


class SolveOpts(ctypes.Structure):
    _fields_ = [("rel_tol", ctypes.c_double), ("max_iter", ctypes.c_int),
                ("precision", ctypes.c_int), ("precond", ctypes.c_int),
                ("fallback_factor", ctypes.c_int), ("degree", ctypes.c_int),
                ("streamed", ctypes.c_int), ("no_coarse", ctypes.c_int)]

    def __init__(self, rel_tol=1e-8, max_iter=100000, precision=PREC_MIXED,
                 precond=PC_JACOBI, fallback_factor=2, degree=0, streamed=0, no_coarse=0):
        super().__init__(rel_tol, max_iter, precision, precond, fallback_factor, degree, streamed,
                         no_coarse)


class SolveInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int),
                ("refinements", ctypes.c_int), ("used_fallback", ctypes.c_int),
                ("rel_res", ctypes.c_double), ("solve_kernel_ms", ctypes.c_double),
                ("assemble_ms", ctypes.c_double)]


class IneqInfo(ctypes.Structure):
    """Layout of eolc_ineq_info (include/eolc.h)."""
    _fields_ = [("status", ctypes.c_int), ("solves", ctypes.c_int), ("outer", ctypes.c_int),
                ("iterations", ctypes.c_int), ("n_active", ctypes.c_int),
                ("max_violation", ctypes.c_double), ("rel_res", ctypes.c_double),
                ("solve_kernel_ms", ctypes.c_double), ("fallbacks", ctypes.c_int)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("n_failed", ctypes.c_int), ("config", ctypes.c_int),
                ("steps", ctypes.c_int), ("iterations", ctypes.c_longlong),
                ("max_iterations", ctypes.c_int), ("n_fallback", ctypes.c_int),
                ("max_rel_res", ctypes.c_double), ("step_ms", ctypes.c_double)]


class Box(ctypes.Structure):
    """Box obstacle: full dimensions and 4x4 frame (column-major)."""
    _fields_ = [("dim", ctypes.c_double * 3), ("E1", ctypes.c_double * 16)]

    def __init__(self, dim, E1):
        super().__init__((ctypes.c_double * 3)(*list(dim)), (ctypes.c_double * 16)(*list(E1)))


class Contact(ctypes.Structure):
    """eolc_contact, mirroring btc::Collision (boxTriCollision.h:49-110)."""
    _fields_ = [
        ("dist", ctypes.c_double), ("nor1", ctypes.c_double * 3), ("nor2", ctypes.c_double * 3),
        ("pos1", ctypes.c_double * 3), ("pos2", ctypes.c_double * 3),
        ("pos1_", ctypes.c_double * 3), ("weights1", ctypes.c_double * 3),
        ("weights2", ctypes.c_double * 3), ("edge_dir", ctypes.c_double * 3),
        ("count1", ctypes.c_int), ("count2", ctypes.c_int), ("verts1", ctypes.c_int * 3),
        ("verts2", ctypes.c_int * 3), ("tri1", ctypes.c_int), ("tri2", ctypes.c_int),
        ("edge1", ctypes.c_int * 3), ("n_edge1", ctypes.c_int), ("edge2", ctypes.c_int),
        ("source", ctypes.c_int)]


_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_V = ctypes.c_void_p


class Rows(ctypes.Structure):
    """eolc_rows: constraint rows in CSR over the DOFs of the block rows."""
    _fields_ = [("n_rows", ctypes.c_int), ("capacity", ctypes.c_int), ("ptr", _I),
                ("col", _I), ("val", _D), ("rhs", _D)]


class EolMesh(ctypes.Structure):
    """eolc_eol_mesh: the mesh state Constraints::fill reads."""
    _fields_ = [("n_nodes", ctypes.c_int), ("x", _D), ("u", _D), ("tri", _I),
                ("n_tri", ctypes.c_int), ("edges", _I), ("preserve", _I),
                ("n_edges", ctypes.c_int), ("eol_nodes", _I), ("corner_id", _I),
                ("cd_edge", _I), ("n_eol", ctypes.c_int)]

# Every symbol the C ABI exports (include/eolc.h).
EXPORTS = ["eolc_version", "eolc_launch_count", "eolc_create", "eolc_destroy", "eolc_last_error", "eolc_set_stream",
           "eolc_set_topology", "eolc_bsr_pattern", "eolc_forces_fill", "eolc_velocity_solve",
           "eolc_step", "eolc_state_upload", "eolc_state_download", "eolc_step_resident",
           "eolc_cd2", "eolc_velocity_solve_static", "eolc_lpc_create", "eolc_lpc_destroy",
           "eolc_lpc_last_error", "eolc_lpc_num_params", "eolc_lpc_get_params",
           "eolc_lpc_set_params", "eolc_lpc_loss_grad", "eolc_lpc_add_system",
           "eolc_lpc_num_systems", "eolc_lpc_clear_systems", "eolc_lpc_train",
           "eolc_attach_preconditioner", "eolc_set_jacobi_reference",
           "eolc_set_topology_batched", "eolc_set_instance_materials", "eolc_step_batched",
           "eolc_batch_num_configs", "eolc_batch_config_name", "eolc_batch_set_config",
           "eolc_batch_autotune", "eolc_set_learned_refresh", "eolc_set_coarse_refresh",
           "eolc_batch_set_jacobi_reference", "eolc_lpc_blocks", "eolc_export_obj",
           "eolc_export_obj_text", "eolc_velocity_solve_ineq", "eolc_contact_rows",
           "eolc_step_contacts", "eolc_set_topology_device", "eolc_topology_arrays",
           "eolc_edge_list", "eolc_set_topology_eol", "eolc_clear_contact_multipliers",
           "eolc_velocity_solve_qp", "eolc_constraint_rows", "eolc_step_eol",
           "eolc_set_wait_limit"]


def load_library(path=LIB_PATH):
    if not os.path.exists(path):
        raise ImportError("libeolc.so is not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    L.eolc_version.restype = ctypes.c_int
    L.eolc_launch_count.argtypes = [_V]
    L.eolc_launch_count.restype = ctypes.c_longlong
    L.eolc_create.argtypes = [ctypes.POINTER(_V), ctypes.c_int]
    L.eolc_destroy.argtypes = [_V]
    L.eolc_destroy.restype = None
    L.eolc_last_error.argtypes = [_V]
    L.eolc_last_error.restype = ctypes.c_char_p
    L.eolc_set_stream.argtypes = [_V, _V]
    L.eolc_set_topology.argtypes = [_V, ctypes.c_int, _I, ctypes.c_int, _I, ctypes.c_int]
    L.eolc_bsr_pattern.argtypes = [_V, _I, _I, _I]
    L.eolc_forces_fill.argtypes = [_V, _D, _D, ctypes.POINTER(Material), _D, ctypes.c_double,
                                   ctypes.c_int, _D, _D, _D]
    L.eolc_velocity_solve.argtypes = [_V, _D, _I, _D, ctypes.c_int, ctypes.POINTER(SolveOpts),
                                      _D, ctypes.POINTER(SolveInfo)]
    L.eolc_step.argtypes = [_V, _D, _D, _D, ctypes.POINTER(Material), _D, ctypes.c_double, _I,
                            _D, ctypes.c_int, ctypes.POINTER(SolveOpts),
                            ctypes.POINTER(SolveInfo)]
    L.eolc_state_upload.argtypes = [_V, _D, _D, _D]
    L.eolc_state_download.argtypes = [_V, _D, _D]
    L.eolc_step_resident.argtypes = [_V, ctypes.c_int, ctypes.POINTER(Material), _D,
                                     ctypes.c_double, _I, _D, ctypes.c_int,
                                     ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveInfo)]
    L.eolc_cd2.argtypes = [_V, _D, ctypes.POINTER(Box), ctypes.c_int, _D, _D, ctypes.c_int,
                           ctypes.c_double, ctypes.POINTER(Contact), ctypes.c_int, _I]
    L.eolc_velocity_solve_static.argtypes = [ctypes.c_int, _I, _I, _V, _V, _I, _D, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_int, _V,
                                             ctypes.POINTER(SolveInfo), _V]
    _F = ctypes.POINTER(ctypes.c_float)
    L.eolc_lpc_create.argtypes = [ctypes.POINTER(_V), ctypes.c_int, ctypes.c_uint]
    L.eolc_lpc_destroy.argtypes = [_V]
    L.eolc_lpc_destroy.restype = None
    L.eolc_lpc_last_error.argtypes = [_V]
    L.eolc_lpc_last_error.restype = ctypes.c_char_p
    L.eolc_lpc_num_params.argtypes = [_V]
    L.eolc_lpc_get_params.argtypes = [_V, _F]
    L.eolc_lpc_set_params.argtypes = [_V, _F]
    L.eolc_lpc_loss_grad.argtypes = [_V, _V, _I, ctypes.c_int, _F, ctypes.c_int, _D, _F]
    L.eolc_lpc_add_system.argtypes = [_V, _V, _I, ctypes.c_int, _F, ctypes.c_int]
    L.eolc_lpc_num_systems.argtypes = [_V]
    L.eolc_lpc_blocks.argtypes = [_V, _V, _I, ctypes.c_int, _F]
    L.eolc_lpc_clear_systems.argtypes = [_V]
    L.eolc_lpc_train.argtypes = [_V, ctypes.c_int, ctypes.c_float, ctypes.c_uint, _D]
    L.eolc_attach_preconditioner.argtypes = [_V, _V]
    L.eolc_set_jacobi_reference.argtypes = [_V, ctypes.c_int]
    L.eolc_set_learned_refresh.argtypes = [_V, ctypes.c_int]
    L.eolc_set_coarse_refresh.argtypes = [_V, ctypes.c_int]
    L.eolc_set_wait_limit.argtypes = [_V, ctypes.c_longlong]
    L.eolc_batch_set_jacobi_reference.argtypes = [_V, _I, ctypes.c_int]
    L.eolc_set_topology_batched.argtypes = [_V, ctypes.c_int, _I, _I, _I, _I, _I]
    L.eolc_set_instance_materials.argtypes = [_V, ctypes.POINTER(Material), ctypes.c_int]
    L.eolc_step_batched.argtypes = [_V, ctypes.c_int, _D, ctypes.c_double, _I, _D, ctypes.c_int,
                                    ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveInfo),
                                    ctypes.POINTER(BatchInfo)]
    L.eolc_batch_num_configs.argtypes = []
    L.eolc_batch_config_name.argtypes = [ctypes.c_int]
    L.eolc_batch_set_config.argtypes = [_V, ctypes.c_int]
    L.eolc_batch_autotune.argtypes = [_V, _D, ctypes.c_double, _I, _D, ctypes.c_int,
                                      ctypes.POINTER(SolveOpts), _I, _D]
    L.eolc_export_obj.argtypes = [_V, ctypes.c_char_p, ctypes.c_int, ctypes.c_double]
    L.eolc_velocity_solve_ineq.argtypes = [_V, _D, _I, _D, ctypes.c_int, ctypes.c_int, _I, _I, _D,
                                           _D, ctypes.POINTER(SolveOpts), _D, _D,
                                           ctypes.POINTER(IneqInfo)]
    L.eolc_set_topology_device.argtypes = [_V, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_int]
    L.eolc_topology_arrays.argtypes = [_V, _I, _I, _I, _I, _I, _I, _I]
    L.eolc_edge_list.argtypes = [_V, _I, ctypes.c_int, _I]
    L.eolc_clear_contact_multipliers.argtypes = [_V]
    L.eolc_set_topology_eol.argtypes = [_V, ctypes.c_int, _I, ctypes.c_int, _I, ctypes.c_int,
                                        _I, ctypes.c_int]
    L.eolc_step_contacts.argtypes = [_V, _D, _D, _D, ctypes.POINTER(Material), _D,
                                     ctypes.c_double, _I, _D, ctypes.c_int, ctypes.POINTER(Box),
                                     ctypes.c_int, _D, _D, ctypes.c_int, ctypes.c_double,
                                     ctypes.POINTER(SolveOpts), ctypes.POINTER(IneqInfo)]
    L.eolc_contact_rows.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _I, _I, _D, _D,
                                    _I]
    L.eolc_velocity_solve_qp.argtypes = [_V, _D, _I, _D, ctypes.c_int, ctypes.POINTER(Rows),
                                         ctypes.POINTER(Rows), ctypes.POINTER(SolveOpts), _D, _D,
                                         _D, ctypes.POINTER(IneqInfo)]
    L.eolc_constraint_rows.argtypes = [ctypes.POINTER(EolMesh), ctypes.POINTER(Box), _D,
                                       ctypes.c_int, _D, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_int, ctypes.c_double, ctypes.POINTER(Rows),
                                       ctypes.POINTER(Rows)]
    L.eolc_step_eol.argtypes = [_V, _D, _D, _D, ctypes.POINTER(Material), _D, ctypes.c_double,
                                _I, _D, ctypes.c_int, ctypes.POINTER(Rows), ctypes.POINTER(Rows),
                                ctypes.POINTER(SolveOpts), ctypes.POINTER(IneqInfo)]
    L.eolc_export_obj_text.argtypes = [_V, ctypes.c_int, ctypes.c_double, ctypes.c_char_p,
                                       ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    for name in EXPORTS:
        if not hasattr(L, name):
            raise ImportError("libeolc.so lacks %s" % name)
        getattr(L, name).restype = getattr(L, name).restype
    for name in EXPORTS:
        if name not in ("eolc_version", "eolc_destroy", "eolc_last_error", "eolc_launch_count",
                        "eolc_lpc_destroy", "eolc_lpc_last_error", "eolc_batch_config_name"):
            getattr(L, name).restype = ctypes.c_int
    L.eolc_batch_config_name.restype = ctypes.c_char_p
    return L


lib = load_library()


def _d(a):
    return a.ctypes.data_as(_D)


def _i(a):
    return a.ctypes.data_as(_I)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Context:
    """One device, one stream, one topology."""

    def __init__(self, device=0):
        h = _V()
        st = lib.eolc_create(ctypes.byref(h), device)
        if st != OK:
            raise EolcError(st, "eolc_create(%d) failed" % device)
        self._h = h
        self.n_nodes = 0

    def __del__(self):
        if getattr(self, "_h", None):
            lib.eolc_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def launch_count(self):
        return lib.eolc_launch_count(self._h)

    def set_stream(self, stream_handle):
        """Run on an external cudaStream_t (an integer handle), e.g. torch's."""
        self._check(lib.eolc_set_stream(self._h, _V(stream_handle)))

    def _check(self, st):
        if st != OK:
            raise EolcError(st, lib.eolc_last_error(self._h).decode())

    def set_topology(self, n_nodes, tri, hinge):
        tri, hinge = _i32(tri), _i32(hinge)
        self._tri = tri
        self._check(lib.eolc_set_topology(self._h, n_nodes, _i(tri), len(tri.reshape(-1, 3)),
                                          _i(hinge), len(hinge.reshape(-1, 4))))
        self.n_nodes = n_nodes

    def set_topology_eol(self, n_nodes, tri, hinge, eol_nodes):
        """eolc_set_topology_eol: EOL node k = eol_nodes[k] gets an Eulerian
        block row n_nodes + k (see eol_reference_index)."""
        tri, hinge, eol = _i32(tri), _i32(hinge), _i32(eol_nodes)
        self._tri = tri
        self._check(lib.eolc_set_topology_eol(self._h, n_nodes, _i(tri), len(tri.reshape(-1, 3)),
                                              _i(hinge), len(hinge.reshape(-1, 4)),
                                              _i(eol if len(eol) else np.zeros(1, np.int32)),
                                              len(eol)))
        self.n_nodes = n_nodes + len(eol)  # block rows (mesh nodes + Eulerian nodes)
        self.n_real = n_nodes

    def set_topology_device(self, n_nodes, tri_ptr, n_tri, hinge_ptr, n_hinge):
        """eolc_set_topology_device: tri / hinge as device addresses (e.g.
        torch CUDA int32 tensors' data_ptr())."""
        self._check(lib.eolc_set_topology_device(self._h, n_nodes, ctypes.c_void_p(tri_ptr), n_tri,
                                                 ctypes.c_void_p(hinge_ptr), n_hinge))
        self.n_nodes = n_nodes

    def topology_arrays(self):
        """The device topology: dict of rowptr, colidx, cptr, contrib,
        nf_ptr, nf_list (eolc_topology_arrays)."""
        sizes = np.zeros(4, np.int32)
        self._check(lib.eolc_topology_arrays(self._h, None, None, None, None, None, None,
                                             _i(sizes)))
        n, nb, nc, nf = (int(v) for v in sizes)
        out = dict(rowptr=np.zeros(n + 1, np.int32), colidx=np.zeros(max(1, nb), np.int32),
                   cptr=np.zeros(nb + 1, np.int32), contrib=np.zeros(max(1, nc), np.int32),
                   nf_ptr=np.zeros(n + 1, np.int32), nf_list=np.zeros(max(1, nf), np.int32))
        self._check(lib.eolc_topology_arrays(self._h, _i(out["rowptr"]), _i(out["colidx"]),
                                             _i(out["cptr"]), _i(out["contrib"]),
                                             _i(out["nf_ptr"]), _i(out["nf_list"]), _i(sizes)))
        out["colidx"] = out["colidx"][:nb]
        out["contrib"] = out["contrib"][:nc]
        out["nf_list"] = out["nf_list"][:nf]
        return out

    def edge_list(self):
        """CD2's cloth edges (eolc_edge_list): (E, 4) int32 rows
        (v0, v1, face0, face1 or -1)."""
        n = ctypes.c_int()
        st = lib.eolc_edge_list(self._h, None, 0, ctypes.byref(n))
        if st not in (OK, CAPACITY):
            self._check(st)
        out = np.zeros((max(1, n.value), 4), np.int32)
        self._check(lib.eolc_edge_list(self._h, _i(out), n.value, ctypes.byref(n)))
        return out[:n.value]

    def bsr_pattern(self):
        nb = ctypes.c_int()
        self._check(lib.eolc_bsr_pattern(self._h, ctypes.byref(nb), None, None))
        rp = np.zeros(self.n_nodes + 1, np.int32)
        ci = np.zeros(nb.value, np.int32)
        self._check(lib.eolc_bsr_pattern(self._h, None, _i(rp), _i(ci)))
        return rp, ci

    def forces_fill(self, x, X, mat, grav, h, precision=PREC_FP64, want_M=True):
        """Forces::fill: returns f (3N), M and MDK BSR values (n_blocks x 9)."""
        x, X, g = _f64(x), _f64(X), _f64(grav)
        nb = len(self.bsr_pattern()[1])
        f = np.zeros(3 * self.n_nodes)
        M = np.zeros(nb * 9) if want_M else None
        MDK = np.zeros(nb * 9)
        self._check(lib.eolc_forces_fill(self._h, _d(x), _d(X), ctypes.byref(mat), _d(g), h,
                                         precision, _d(f), _d(M) if want_M else None, _d(MDK)))
        return f, M, MDK

    def velocity_solve(self, b, fixed_dofs, beq, opts=None, v0=None):
        opts = opts or SolveOpts()
        b, fixed_dofs, beq = _f64(b), _i32(fixed_dofs), _f64(beq)
        v = np.zeros(3 * self.n_nodes) if v0 is None else _f64(v0).copy()
        info = SolveInfo()
        st = lib.eolc_velocity_solve(self._h, _d(b), _i(fixed_dofs), _d(beq), len(fixed_dofs),
                                     ctypes.byref(opts), _d(v), ctypes.byref(info))
        self._check(st)
        return v, info

    def velocity_solve_ineq(self, b, fixed_dofs, beq, Aineq, bineq, opts=None, v0=None):
        """Contact-constrained solve (eolc_velocity_solve_ineq): Aineq a scipy
        sparse matrix over the 3N DOFs (or (indptr, indices, data)), bineq its
        right-hand side.  Returns (v, lambda, IneqInfo)."""
        opts = opts or SolveOpts()
        b, fixed_dofs, beq = _f64(b), _i32(fixed_dofs), _f64(beq)
        if isinstance(Aineq, tuple):
            ptr, col, val = (_i32(Aineq[0]), _i32(Aineq[1]), _f64(Aineq[2]))
        else:
            import scipy.sparse as sp
            A = sp.csr_matrix(Aineq)
            ptr, col, val = _i32(A.indptr), _i32(A.indices), _f64(A.data)
        m = len(ptr) - 1
        d = _f64(bineq) if m > 0 else np.zeros(1)
        v = np.zeros(3 * self.n_nodes) if v0 is None else _f64(v0).copy()
        lam = np.zeros(max(1, m))
        info = IneqInfo()
        st = lib.eolc_velocity_solve_ineq(self._h, _d(b), _i(fixed_dofs), _d(beq),
                                          len(fixed_dofs), m, _i(ptr),
                                          _i(col if len(col) else np.zeros(1, np.int32)),
                                          _d(val if len(val) else np.zeros(1)), _d(d),
                                          ctypes.byref(opts), _d(v), _d(lam), ctypes.byref(info))
        self._check(st)
        return v, lam[:m], info

    def velocity_solve_qp(self, b, fixed_dofs, beq, eq=None, ineq=None, opts=None, v0=None):
        """The QP with equality and inequality rows (eolc_velocity_solve_qp)
        on the last fill's MDK; eq / ineq are RowSet (or None).  b, v over the
        block rows' DOFs (the extended layout on an EOL topology).  Returns
        (v, lambda_eq, lambda_ineq, IneqInfo)."""
        opts = opts or SolveOpts()
        b, fixed_dofs, beq = _f64(b), _i32(fixed_dofs), _f64(beq)
        eq = eq or RowSet.empty()
        ineq = ineq or RowSet.empty()
        re, ri = eq.as_c(), ineq.as_c()
        v = np.zeros(3 * self.n_nodes) if v0 is None else _f64(v0).copy()
        le, li = np.zeros(max(1, eq.m)), np.zeros(max(1, ineq.m))
        info = IneqInfo()
        st = lib.eolc_velocity_solve_qp(self._h, _d(b), _i(fixed_dofs), _d(beq),
                                        len(fixed_dofs), ctypes.byref(re), ctypes.byref(ri),
                                        ctypes.byref(opts), _d(v), _d(le), _d(li),
                                        ctypes.byref(info))
        self._check(st)
        return v, le[:eq.m], li[:ineq.m], info

    def step_eol(self, x, u, v, mat, grav, h, fixed_dofs, fixed_vel, eq=None, ineq=None,
                 opts=None):
        """Cloth::step of an EOL mesh (eolc_step_eol) with the rows of
        Constraints::fill (constraint_rows); x (3N), u (2N) and v (extended
        layout) are updated in place.  Returns the QP's IneqInfo."""
        opts = opts or SolveOpts()
        fixed_dofs, fixed_vel = _i32(fixed_dofs), _f64(fixed_vel)
        eq = eq or RowSet.empty()
        ineq = ineq or RowSet.empty()
        re, ri = eq.as_c(), ineq.as_c()
        info = IneqInfo()
        st = lib.eolc_step_eol(self._h, _d(x), _d(u), _d(v), ctypes.byref(mat), _d(_f64(grav)), h,
                               _i(fixed_dofs), _d(fixed_vel), len(fixed_dofs), ctypes.byref(re),
                               ctypes.byref(ri), ctypes.byref(opts), ctypes.byref(info))
        self._check(st)
        return info

    def step_contacts(self, x, X, v, mat, grav, h, fixed_dofs, fixed_vel, boxes=(), points=None,
                      normals=None, threshold=1e-3, opts=None):
        """Cloth::step with the contact QP (eolc_step_contacts); x, v updated
        in place.  Returns the QP's IneqInfo."""
        opts = opts or SolveOpts()
        fixed_dofs, fixed_vel = _i32(fixed_dofs), _f64(fixed_vel)
        boxes = list(boxes)
        barr = (Box * max(1, len(boxes)))(*boxes)
        pts = _f64(points) if points is not None else np.zeros(3)
        nrm = _f64(normals) if normals is not None else np.zeros(3)
        npts = 0 if points is None else len(pts.reshape(-1, 3))
        info = IneqInfo()
        st = lib.eolc_step_contacts(self._h, _d(x), _d(_f64(X)), _d(v), ctypes.byref(mat),
                                    _d(_f64(grav)), h, _i(fixed_dofs), _d(fixed_vel),
                                    len(fixed_dofs), barr, len(boxes), _d(pts), _d(nrm), npts,
                                    threshold, ctypes.byref(opts), ctypes.byref(info))
        self._check(st)
        return info

    def clear_contact_multipliers(self):
        self._check(lib.eolc_clear_contact_multipliers(self._h))

    def step(self, x, X, v, mat, grav, h, fixed_dofs, fixed_vel, opts=None):
        """Cloth::step on host arrays; x, v updated in place."""
        opts = opts or SolveOpts()
        assert x.dtype == np.float64 and v.dtype == np.float64
        assert x.flags.c_contiguous and v.flags.c_contiguous
        X, g = _f64(X), _f64(grav)
        fixed_dofs, fixed_vel = _i32(fixed_dofs), _f64(fixed_vel)
        info = SolveInfo()
        st = lib.eolc_step(self._h, _d(x), _d(X), _d(v), ctypes.byref(mat), _d(g), h,
                           _i(fixed_dofs), _d(fixed_vel), len(fixed_dofs), ctypes.byref(opts),
                           ctypes.byref(info))
        self._check(st)
        return info

    def state_upload(self, x, X, v):
        self._check(lib.eolc_state_upload(self._h, _d(_f64(x)), _d(_f64(X)), _d(_f64(v))))

    def state_download(self):
        x = np.zeros(3 * self.n_nodes); v = np.zeros(3 * self.n_nodes)
        self._check(lib.eolc_state_download(self._h, _d(x), _d(v)))
        return x, v

    def step_resident(self, n_steps, mat, grav, h, fixed_dofs, fixed_vel, opts=None):
        opts = opts or SolveOpts()
        fixed_dofs, fixed_vel = _i32(fixed_dofs), _f64(fixed_vel)
        info = SolveInfo()
        st = lib.eolc_step_resident(self._h, n_steps, ctypes.byref(mat), _d(_f64(grav)), h,
                                    _i(fixed_dofs), _d(fixed_vel), len(fixed_dofs),
                                    ctypes.byref(opts), ctypes.byref(info))
        self._check(st)
        return info

    def cd2(self, x, boxes=(), points=None, normals=None, threshold=1e-3, capacity=None,
            raw=False, array=False):
        """CD2 contact list (point obstacles first, then each box); raw=True
        returns the contacts' bytes (eolc_contact records, in order),
        array=True a ctypes array of them (no per-contact objects: pass it to
        constraint_rows as is)."""
        x = _f64(x)
        boxes = list(boxes)
        barr = (Box * max(1, len(boxes)))(*boxes)
        pts = _f64(points) if points is not None else np.zeros(3)
        nrm = _f64(normals) if normals is not None else np.zeros(3)
        npts = 0 if points is None else len(pts.reshape(-1, 3))
        cap = capacity if capacity is not None else 4 * self.n_nodes + 64
        out = (Contact * max(1, cap))()
        n = ctypes.c_int()
        st = lib.eolc_cd2(self._h, _d(x), barr, len(boxes), _d(pts), _d(nrm), npts, threshold,
                          out, cap, ctypes.byref(n))
        if st == CAPACITY and capacity is None:
            return self.cd2(x, boxes, points, normals, threshold, capacity=n.value, raw=raw,
                            array=array)
        self._check(st)
        if raw:
            return ctypes.string_at(out, ctypes.sizeof(Contact) * n.value)
        if array:
            return (Contact * n.value).from_buffer(out)
        return [out[k] for k in range(n.value)]

    # ---- OBJ export ------------------------------------------------------------
    def export_obj(self, export_dir, frame, time=0.0):
        """Writes <dir>/<frame>_Cloth2D.obj and <dir>/<frame>_Cloth3D.obj from
        the device state (positions of the last upload or step)."""
        self._check(lib.eolc_export_obj(self._h, os.fsencode(export_dir), frame, time))

    def export_obj_text(self, frame, time=0.0):
        """The two files' bytes: (Cloth2D, Cloth3D)."""
        ln = (ctypes.c_size_t * 2)()
        self._check(lib.eolc_export_obj_text(self._h, frame, time, None, 0, ln))
        buf = ctypes.create_string_buffer(ln[0] + ln[1])
        self._check(lib.eolc_export_obj_text(self._h, frame, time, buf, ln[0] + ln[1], ln))
        raw = buf.raw
        return raw[:ln[0]], raw[ln[0]:ln[0] + ln[1]]

    # ---- batches -------------------------------------------------------------
    def set_topology_batched(self, sheets):
        """sheets: list of (n_nodes, tri, hinge) with instance-local node ids.
        Returns the node offsets (instance k owns nodes off[k]..off[k+1]-1)."""
        node_off, tri_off, hinge_off, tris, hinges = [0], [0], [0], [], []
        for n, tri, hinge in sheets:
            tri, hinge = _i32(tri).reshape(-1, 3), _i32(hinge).reshape(-1, 4)
            tris.append(tri + node_off[-1])
            hinges.append(hinge + node_off[-1])
            node_off.append(node_off[-1] + n)
            tri_off.append(tri_off[-1] + len(tri))
            hinge_off.append(hinge_off[-1] + len(hinge))
        tri = _i32(np.concatenate(tris))
        hinge = _i32(np.concatenate(hinges)) if hinge_off[-1] else np.zeros((1, 4), np.int32)
        node_off, tri_off, hinge_off = _i32(node_off), _i32(tri_off), _i32(hinge_off)
        self._tri = tri
        self._check(lib.eolc_set_topology_batched(self._h, len(sheets), _i(node_off), _i(tri),
                                                  _i(tri_off), _i(hinge), _i(hinge_off)))
        self.n_nodes = int(node_off[-1])
        self.node_off = node_off
        return node_off

    def set_instance_materials(self, mats):
        arr = (Material * len(mats))(*mats)
        self._check(lib.eolc_set_instance_materials(self._h, arr, len(mats)))

    def step_batched(self, n_steps, grav, h, fixed_dofs, fixed_vel, opts=None):
        """n_steps batched steps on the resident state; returns (BatchInfo,
        per-instance SolveInfo list).  Raises on a failed instance solve."""
        opts = opts or SolveOpts()
        fixed_dofs, fixed_vel = _i32(fixed_dofs), _f64(fixed_vel)
        n_inst = len(self.node_off) - 1
        infos = (SolveInfo * n_inst)()
        tot = BatchInfo()
        st = lib.eolc_step_batched(self._h, n_steps, _d(_f64(grav)), h, _i(fixed_dofs),
                                   _d(fixed_vel), len(fixed_dofs), ctypes.byref(opts), infos,
                                   ctypes.byref(tot))
        self._check(st)
        return tot, [infos[k] for k in range(n_inst)]

    def set_learned_refresh(self, solves):
        self._check(lib.eolc_set_learned_refresh(self._h, solves))

    def set_wait_limit(self, polls):
        """Polls before a device wait of this context's solves gives up with
        TIMEOUT (eolc_set_wait_limit; 0 restores the default)."""
        self._check(lib.eolc_set_wait_limit(self._h, polls))

    def set_coarse_refresh(self, solves):
        """Rebuild the patch preconditioner's coarse operator every `solves`
        solves (eolc_set_coarse_refresh)."""
        self._check(lib.eolc_set_coarse_refresh(self._h, solves))

    def batch_set_jacobi_reference(self, iters):
        iters = _i32(iters)
        self._check(lib.eolc_batch_set_jacobi_reference(self._h, _i(iters), len(iters)))

    def batch_set_config(self, config):
        self._check(lib.eolc_batch_set_config(self._h, config))

    def batch_autotune(self, grav, h, fixed_dofs, fixed_vel, opts=None):
        """Returns (chosen configuration, ms per configuration)."""
        opts = opts or SolveOpts()
        fixed_dofs, fixed_vel = _i32(fixed_dofs), _f64(fixed_vel)
        ms = np.zeros(batch_num_configs())
        chosen = ctypes.c_int()
        self._check(lib.eolc_batch_autotune(self._h, _d(_f64(grav)), h, _i(fixed_dofs),
                                            _d(fixed_vel), len(fixed_dofs), ctypes.byref(opts),
                                            ctypes.byref(chosen), _d(ms)))
        return chosen.value, ms


def batch_num_configs():
    return lib.eolc_batch_num_configs()


def batch_config_name(config):
    return lib.eolc_batch_config_name(config).decode()


class LearnedPC:
    """The learned block-sparse approximate inverse (see include/eolc.h)."""

    def __init__(self, device=0, seed=0):
        h = _V()
        st = lib.eolc_lpc_create(ctypes.byref(h), device, seed)
        if st != OK:
            raise EolcError(st, "eolc_lpc_create failed")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            lib.eolc_lpc_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def _check(self, st):
        if st != OK:
            raise EolcError(st, lib.eolc_lpc_last_error(self._h).decode())

    def num_params(self):
        return lib.eolc_lpc_num_params(self._h)

    def get_params(self):
        out = np.zeros(self.num_params(), np.float32)
        self._check(lib.eolc_lpc_get_params(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params()
        self._check(lib.eolc_lpc_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def loss_grad(self, ctx, fixed_dofs, probes):
        fixed_dofs = _i32(fixed_dofs)
        probes = np.ascontiguousarray(probes, dtype=np.float32)
        k = probes.shape[0]
        grad = np.zeros(self.num_params(), np.float32)
        loss = ctypes.c_double()
        st = lib.eolc_lpc_loss_grad(self._h, ctx.handle, _i(fixed_dofs), len(fixed_dofs),
                                    probes.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), k,
                                    ctypes.byref(loss), grad.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        self._check(st)
        return loss.value, grad

    def add_system(self, ctx, fixed_dofs, probes):
        fixed_dofs = _i32(fixed_dofs)
        probes = np.ascontiguousarray(probes, dtype=np.float32)
        self._check(lib.eolc_lpc_add_system(self._h, ctx.handle, _i(fixed_dofs), len(fixed_dofs),
                                            probes.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                            probes.shape[0]))

    def blocks(self, ctx, fixed_dofs):
        """G (n_blocks x 9) for the context's current FP32 MDK."""
        fixed_dofs = _i32(fixed_dofs)
        nb = len(ctx.bsr_pattern()[1])
        G = np.zeros(nb * 9, np.float32)
        self._check(lib.eolc_lpc_blocks(self._h, ctx.handle, _i(fixed_dofs), len(fixed_dofs),
                                        G.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return G.reshape(-1, 9)

    def num_systems(self):
        return lib.eolc_lpc_num_systems(self._h)

    def clear_systems(self):
        self._check(lib.eolc_lpc_clear_systems(self._h))

    def train(self, epochs, lr=1e-3, seed=0):
        losses = np.zeros(epochs)
        self._check(lib.eolc_lpc_train(self._h, epochs, lr, seed, _d(losses)))
        return losses

    def attach(self, ctx):
        ctx._check(lib.eolc_attach_preconditioner(ctx.handle, self._h))
        ctx._lpc = self  # keep the network alive while attached


# ---------------------------------------------------------------------------
# Mesh input (host side, numpy): the sheets the benchmark scenes use
# ---------------------------------------------------------------------------
# Corner convention of the scene files (simulationSettings*.json): corner1
# (0, 0), corner2 (1, 0), corner3 (0, 1), corner4 (1, 1), rows (x, y, z, X, Y).
UNIT_CORNERS = np.array([[0, 0, 0, 0, 0], [1, 0, 0, 1, 0],
                         [0, 1, 0, 0, 1], [1, 1, 0, 1, 1]], dtype=np.float64)


def sheet_mesh(r0, r1, corners=UNIT_CORNERS):
    """Grid of r0 x r1 nodes with two triangles per quad -> (x, X, tri).
    Node k = i r1 + j sits at the bilinear blend of the four corners, blended
    as Cloth::build blends them (Cloth.cpp:63-76: (1 - s) a + s b per
    component, first along i, then along j); quad (i, j) gives the triangles
    (k, k + 1, k + r1 + 1) and (k, k + r1 + 1, k + r1)."""
    c = np.asarray(corners, np.float64).reshape(4, 5)
    u = np.arange(r0) / (r0 - 1.0)
    v = np.arange(r1) / (r1 - 1.0)

    def blend(s, a, b):
        return (1 - s)[:, None] * a[None, :] + s[:, None] * b[None, :]

    a0, a1 = blend(u, c[0], c[2]), blend(u, c[1], c[3])  # (r0, 5) each
    pts = (1 - v)[None, :, None] * a0[:, None, :] + v[None, :, None] * a1[:, None, :]
    pts = pts.reshape(-1, 5)
    x = np.ascontiguousarray(pts[:, :3]).ravel()
    X = np.ascontiguousarray(pts[:, 3:]).ravel()
    i, j = np.meshgrid(np.arange(r0 - 1), np.arange(r1 - 1), indexing="ij")
    k0 = (i * r1 + j).ravel()
    t = np.empty((2 * len(k0), 3), np.int32)
    t[0::2] = np.stack([k0, k0 + 1, k0 + r1 + 1], 1)
    t[1::2] = np.stack([k0, k0 + r1 + 1, k0 + r1], 1)
    return x, X, t


def mesh_hinges(tri):
    """Bending hinges (x0, x1, x2, x3) of a triangle list, one per edge with
    two faces, in ArcSim's edge order (Mesh::add(Face), mesh.cpp:356-378):
    each face, in order, creates its missing edges (v[i], v[i+1]); a face
    registers on side 0 of its edge (v[i+1], v[i+2]) when that edge's first
    node is v[i+1], else on side 1 (a later face overwrites).  x0, x1 are the
    edge's nodes, x2 / x3 the other vertex of the side-0 / side-1 face
    (Forces.cpp:687-697)."""
    tri = np.asarray(tri, np.int64).reshape(-1, 3)
    nf = len(tri)
    if nf == 0:
        return np.zeros((0, 4), np.int32)
    a = tri.ravel()                          # v[i] of (face, i)
    b = tri[:, [1, 2, 0]].ravel()            # v[i+1]
    key = np.minimum(a, b) * (int(tri.max()) + 1) + np.maximum(a, b)
    uk, first, inv = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")          # edges in creation order
    rank = np.empty(len(uk), np.int64)
    rank[order] = np.arange(len(uk))
    eid = rank[inv]                                    # edge of (face, i) = (v[i], v[i+1])
    n0, n1 = a[first[order]], b[first[order]]
    # face f registers on edge (v[i+1], v[i+2]) = the edge created at slot
    # (f, i+1); its side follows whether n0 is v[i+1]
    f = np.repeat(np.arange(nf), 3)
    slot_next = (np.arange(3 * nf).reshape(nf, 3)[:, [1, 2, 0]]).ravel()
    e_reg = eid[slot_next]
    first_node = a[slot_next]
    side0 = n0[e_reg] == first_node
    f0 = np.full(len(uk), -1, np.int64)
    f1 = np.full(len(uk), -1, np.int64)
    np.maximum.at(f0, e_reg[side0], f[side0])
    np.maximum.at(f1, e_reg[~side0], f[~side0])
    keep = (f0 >= 0) & (f1 >= 0)
    e0, e1 = n0[keep], n1[keep]

    def other(fa):  # get_other_vert (mesh.hpp:276-280)
        v = tri[fa]
        pick = np.where((v[:, 0] != e0) & (v[:, 0] != e1), v[:, 0],
                        np.where((v[:, 1] != e0) & (v[:, 1] != e1), v[:, 1], v[:, 2]))
        return pick

    return np.stack([e0, e1, other(f0[keep]), other(f1[keep])], 1).astype(np.int32)


def mesh_edges(tri):
    """The edges of a triangle list in ArcSim's mesh.edges order
    (Mesh::add(Face), mesh.cpp:356-363: each face, in order, creates its
    missing edges (v[i], v[i+1])): (n_edges, 2) int32 of Edge::n[0], n[1]."""
    tri = np.asarray(tri, np.int64).reshape(-1, 3)
    if len(tri) == 0:
        return np.zeros((0, 2), np.int32)
    a = tri.ravel()
    b = tri[:, [1, 2, 0]].ravel()
    key = np.minimum(a, b) * (int(tri.max()) + 1) + np.maximum(a, b)
    _, first = np.unique(key, return_index=True)
    first = np.sort(first)
    return np.stack([a[first], b[first]], 1).astype(np.int32)


class RowSet:
    """Constraint rows as CSR arrays (ptr, col, val) with right-hand sides."""

    def __init__(self, ptr, col, val, rhs):
        self.ptr, self.col, self.val, self.rhs = _i32(ptr), _i32(col), _f64(val), _f64(rhs)

    @staticmethod
    def empty():
        return RowSet(np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), np.zeros(0))

    @staticmethod
    def from_csr(A, rhs):
        import scipy.sparse as sp
        A = sp.csr_matrix(A)
        return RowSet(A.indptr, A.indices, A.data, rhs)

    @property
    def m(self):
        return len(self.ptr) - 1

    def csr(self, n_dofs):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.ptr), shape=(self.m, n_dofs))

    def as_c(self):
        """An eolc_rows view of the arrays (kept alive by this object)."""
        self._col = self.col if len(self.col) else np.zeros(1, np.int32)
        self._val = self.val if len(self.val) else np.zeros(1)
        self._rhs = self.rhs if len(self.rhs) else np.zeros(1)
        return Rows(self.m, self.m, _i(self.ptr), _i(self._col), _d(self._val), _d(self._rhs))


def constraint_rows(x, u, tri, edges, eol_nodes, corner_id, cd_edge, preserve=None, boxes=(),
                    point_normals=None, contacts=(), box_velocity=None, h=0.0):
    """Constraints::fill for an EOL mesh (eolc_constraint_rows, host only):
    (equality RowSet, inequality RowSet) over the extended layout.
    box_velocity: None (boxes at rest) or (n_boxes, 6) Box::v, angular then
    linear; h: the step (needed with moving boxes)."""
    x, u, tri, edges = _f64(x), _f64(u), _i32(tri), _i32(edges)
    eol, cid, cde = _i32(eol_nodes), _i32(corner_id), _i32(cd_edge)
    pres = None if preserve is None else _i32(preserve)
    n = len(x) // 3
    one = np.zeros(1, np.int32)
    mesh = EolMesh(n, _d(x), _d(u), _i(tri), len(tri.reshape(-1, 3)),
                   _i(edges if len(edges) else one), _i(pres) if pres is not None else None,
                   len(edges.reshape(-1, 2)), _i(eol if len(eol) else one),
                   _i(cid if len(cid) else one), _i(cde if len(cde) else one), len(eol))
    boxes = list(boxes)
    barr = (Box * max(1, len(boxes)))(*boxes)
    bv = None if box_velocity is None or not boxes else _f64(box_velocity)
    pn = np.zeros(3) if point_normals is None else _f64(point_normals)
    npts = 0 if point_normals is None else len(pn.reshape(-1, 3))
    if isinstance(contacts, ctypes.Array) and len(contacts) > 0:
        carr = contacts  # eolc_contact records already in one array
    else:
        contacts = list(contacts)
        carr = (Contact * max(1, len(contacts)))(*contacts)
    cap_e, cap_i = 3 * len(eol) + 1, 3 * len(eol) + len(contacts) + 1
    while True:
        bufs = []
        for cap in (cap_e, cap_i):
            ptr, col = np.zeros(cap + 1, np.int32), np.zeros(9 * cap, np.int32)
            val, rhs = np.zeros(9 * cap), np.zeros(cap)
            bufs.append((Rows(0, cap, _i(ptr), _i(col), _d(val), _d(rhs)), ptr, col, val, rhs))
        st = lib.eolc_constraint_rows(ctypes.byref(mesh), barr, _d(bv) if bv is not None else None,
                                      len(boxes), _d(pn), npts,
                                      ctypes.cast(carr, ctypes.c_void_p), len(contacts), h,
                                      ctypes.byref(bufs[0][0]), ctypes.byref(bufs[1][0]))
        if st == CAPACITY:
            cap_e, cap_i = max(cap_e, bufs[0][0].n_rows), max(cap_i, bufs[1][0].n_rows)
            continue
        if st != OK:
            raise EolcError(st, "eolc_constraint_rows: bad arguments")
        out = []
        for R, ptr, col, val, rhs in bufs:
            m = R.n_rows
            q = int(ptr[m])
            out.append(RowSet(ptr[:m + 1].copy(), col[:q].copy(), val[:q].copy(), rhs[:m].copy()))
        return out[0], out[1]


def corner_ids(r0, r1):
    """Node ids of the pinned corners 1-4 of a scene's cloth
    (parseParams.cpp:298-305)."""
    return {1: 0, 2: r0 * (r1 - 1), 3: r0 * r1 - 1, 4: r0 - 1}


def contact_rows(contacts, n_nodes):
    """Inequality rows of Constraints::fill from CD2 contacts
    (Constraints.cpp:422-468) via eolc_contact_rows: (scipy CSR over the 3N
    DOFs, bineq)."""
    import scipy.sparse as sp
    n = len(contacts)
    arr = (Contact * max(1, n))(*contacts)
    ptr = np.zeros(n + 1, np.int32)
    col = np.zeros(max(1, 9 * n), np.int32)
    val = np.zeros(max(1, 9 * n))
    d = np.zeros(max(1, n))
    m = ctypes.c_int()
    st = lib.eolc_contact_rows(ctypes.cast(arr, ctypes.c_void_p), n, n, _i(ptr), _i(col), _d(val),
                               _d(d), ctypes.byref(m))
    if st != OK:
        raise EolcError(st, "eolc_contact_rows failed")
    m = m.value
    C = sp.csr_matrix((val[:ptr[m]], col[:ptr[m]], ptr[:m + 1]), shape=(m, 3 * n_nodes))
    return C, d[:m].copy()


def eol_reference_index(n_real, n_eol):
    """For each DOF of the reference's EOL system (3N Lagrangian, then 2 per
    EOL node), its DOF in the library's extended layout (Eulerian node k's
    DOFs 0, 1 at 3 (N + k))."""
    k = np.arange(n_eol)
    eul = np.stack([3 * (n_real + k), 3 * (n_real + k) + 1], 1).ravel()
    return np.concatenate([np.arange(3 * n_real), eul]).astype(np.int64)


def bsr_to_csr(ctx, vals):
    """3x3 BSR values (n_blocks x 9, row-major blocks) -> scipy CSR."""
    import scipy.sparse as sp
    rp, ci = ctx.bsr_pattern()
    return sp.bsr_matrix((np.asarray(vals).reshape(-1, 3, 3), ci, rp),
                         shape=(3 * ctx.n_nodes, 3 * ctx.n_nodes)).tocsr()


_CONTACT_FIELDS = [f[0] for f in Contact._fields_]


def contact_tuple(c):
    out = []
    for name in _CONTACT_FIELDS:
        v = getattr(c, name)
        if hasattr(v, "__len__"):
            out.append(tuple(np.asarray(list(v)).view(np.int64 if isinstance(v[0], float) else np.int32).tolist()
                             if isinstance(v[0], float) else list(v)))
        else:
            out.append(np.float64(v).view(np.int64).item() if isinstance(v, float) else v)
    return tuple(tuple(o) if isinstance(o, list) else o for o in out)


def contacts_equal(a, b):
    """Bitwise equality of two contact lists (order included)."""
    if len(a) != len(b):
        return False
    return all(contact_tuple(x) == contact_tuple(y) for x, y in zip(a, b))


# ---------------------------------------------------------------------------
# Reference call surface
# ---------------------------------------------------------------------------
class Forces:
    """Forces (src/Forces.h:26-45): fill() computes f, M and MDK on the GPU."""

    def __init__(self, ctx, precision=PREC_FP64):
        self.ctx = ctx
        self.precision = precision
        self.f = None
        self.M = None
        self.MDK = None

    def fill(self, x, X, mat, grav, h):
        """Forces::fill (Forces.cpp:912-930) for node positions x and
        material coordinates X of the context's topology."""
        f, M, MDK = self.ctx.forces_fill(x, X, mat, grav, h, self.precision)
        self.f = f
        self.M = bsr_to_csr(self.ctx, M)
        self.MDK = bsr_to_csr(self.ctx, MDK)


class Constraints:
    """Constraints (src/Constraints.h): fill() builds Aeq, beq, Aineq, bineq
    as Constraints::fill does (Constraints.cpp:135-513), over the context's
    DOFs (the extended layout on an EOL topology): the EOL nodes' rows and
    the CD2 contact rows through eolc_constraint_rows, then the pinned DOFs'
    unit rows with beq = 0.99 v + c (addFixed, :114-119, :472-496).  Row
    order is the reference's: Aeq = EOL equalities, then pins; Aineq = EOL
    inequalities, then contacts."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.hasFixed = False
        self.hasCollisions = False
        self.Aeq = self.beq = self.Aineq = self.bineq = None

    def fill(self, x, u, v, tri, edges, eol_nodes, corner_id, cd_edge, preserve=None,
             boxes=(), points=None, normals=None, fixed_dofs=(), fixed_vel=(),
             threshold=1e-3, contacts=None, box_velocity=None, h=0.0):
        """contacts: the CD2 contact list of x (None: eolc_cd2 on this
        context).  v: current velocities (the pins' beq).  box_velocity, h:
        moving boxes (Box::v per box) and the step."""
        import scipy.sparse as sp
        if contacts is None:
            contacts = self.ctx.cd2(x, boxes, points, normals, threshold)
        E, I = constraint_rows(x, u, tri, edges, eol_nodes, corner_id, cd_edge, preserve,
                               boxes, normals, contacts, box_velocity, h)
        nd = len(v)
        fixed = _i32(fixed_dofs)
        pins = sp.csr_matrix((np.ones(len(fixed)), (np.arange(len(fixed)), fixed)),
                             shape=(len(fixed), nd))
        self.Aeq = sp.vstack([E.csr(nd), pins]).tocsr()
        self.beq = np.concatenate([E.rhs, 0.99 * _f64(v)[fixed] + _f64(fixed_vel)])
        self.Aineq = I.csr(nd)
        self.bineq = I.rhs.copy()
        self.hasFixed = len(fixed) > 0
        self.hasCollisions = I.m > 0
        return self


class GeneralizedSolver:
    """GeneralizedSolver (src/GeneralizedSolver.h): velocitySolve on the GPU,
    with or without contact rows."""

    def __init__(self, ctx, opts=None):
        self.ctx = ctx
        self.opts = opts or SolveOpts()
        self.last_info = None

    def velocitySolve(self, fixedPoints, collisions, MDK, b, Aeq, beq, Aineq, bineq, v):
        """Same arguments as GeneralizedSolver::velocitySolve
        (GeneralizedSolver.cpp:107-173).  MDK must be the matrix of the
        context's last fill (it stays resident on the GPU); DOFs are the
        context's block rows (the extended layout on an EOL topology).  The
        unit rows of Aeq (pinned DOFs, Constraints.cpp:114-119) become fixed
        DOFs; any other Aeq rows (the EOL rows of Constraints.cpp:147-415)
        go to eolc_velocity_solve_qp with Aineq.  With collisions=True the QP
        with Aineq v <= bineq (which the reference hands to Mosek/Gurobi) is
        solved on the GPU as well.  v is the initial guess and is overwritten
        in place."""
        import scipy.sparse as sp
        fixed = np.zeros(0, np.int32)
        beqv = np.zeros(0)
        general = None
        if fixedPoints and Aeq is not None and Aeq.shape[0] > 0:
            A = sp.csr_matrix(Aeq)
            A.sort_indices()
            beq_all = np.asarray(beq, dtype=np.float64)
            unit = (np.diff(A.indptr) == 1)
            unit[unit] = A.data[A.indptr[:-1][unit]] == 1.0
            fixed = A.indices[A.indptr[:-1][unit]].astype(np.int32)
            beqv = beq_all[unit]
            if not unit.all():
                general = RowSet.from_csr(A[~unit], beq_all[~unit])
        if general is not None:
            ineq = (RowSet.from_csr(Aineq, bineq) if collisions and Aineq is not None
                    and Aineq.shape[0] > 0 else None)
            out, self.lambda_eq, lam, info = self.ctx.velocity_solve_qp(
                b, fixed, beqv, general, ineq, self.opts, v0=v)
            if ineq is not None:
                self.lambda_ineq = lam
        elif collisions and Aineq is not None and Aineq.shape[0] > 0:
            out, self.lambda_ineq, info = self.ctx.velocity_solve_ineq(
                b, fixed, beqv, Aineq, bineq, self.opts, v0=v)
        else:
            out, info = self.ctx.velocity_solve(b, fixed, beqv, self.opts, v0=v)
        v[:] = out
        self.last_info = info
        return info.status == OK


def CD2(ctx, x, boxes=(), points=None, normals=None, threshold=1e-3):
    """CD2 (Collisions.cpp:55-78): contacts of the cloth (context topology,
    positions x) with point obstacles and boxes, in the reference's order."""
    return ctx.cd2(x, boxes, points, normals, threshold)


class BrenderManager:
    """Per-frame OBJ export (src/BrenderManager.h:15-45): set_export_dir,
    get_frame and export_brender(time), which writes the frame's files and
    then advances the frame counter.  Unlike the reference's singleton, one
    manager per cloth context; obstacle shapes are not exported."""

    def __init__(self, ctx, export_dir="."):
        self.ctx = ctx
        self.export_dir = export_dir
        self.frame = 0

    def set_export_dir(self, export_dir):
        self.export_dir = export_dir

    def get_frame(self):
        return self.frame

    def export_brender(self, time=0.0):
        self.ctx.export_obj(self.export_dir, self.frame, time)
        self.frame += 1
