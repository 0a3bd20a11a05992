"""The velocity solve that allocates nothing on the device.

Callers that cannot call cudaMalloc on their step path (an interactive
stepping loop, where cudaMalloc/cudaFree may synchronize the device and take
milliseconds; a host framework that keeps all device memory in its own pool)
use eolc_velocity_solve_static: the same mixed-precision Jacobi PCG as
eolc_velocity_solve, with its scratch in one fixed device array inside the
library.  This file is collected last so that a failure here does not stop
the rest of a -x run.  The buffers the caller passes are allocated by the
test itself (torch), never by the entry point.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
import scenes

pytestmark = pytest.mark.gpu


def test_static_solve_matches_context_solve_twice():
    import torch
    import __graft_entry__ as g
    g.build_lib()
    import eolc

    s = scenes.sheet(40)
    ctx = eolc.Context(0)
    ctx.set_topology(s["n"], s["tri"], s["hinge"])
    mat = eolc.Material(**scenes.material_c1())
    rng = np.random.default_rng(11)
    x = s["x"] + rng.normal(0, 0.003, s["x"].size)
    v0 = rng.normal(0, 0.05, s["x"].size)
    _, _, MDK = ctx.forces_fill(x, s["X"], mat, scenes.GRAV, scenes.H, eolc.PREC_MIXED)
    F = O.Forces(x, s["X"], s["tri"], s["hinge"], O.material(**scenes.material_c1()),
                 scenes.GRAV, scenes.H)
    b = F.rhs(v0, scenes.H)
    beq = 0.99 * v0[s["fixed"]]
    opts = eolc.SolveOpts(rel_tol=1e-8, precision=eolc.PREC_MIXED, precond=eolc.PC_JACOBI)
    v_ref, info_ref = ctx.velocity_solve(b, s["fixed"], beq, opts)
    assert info_ref.status == eolc.OK

    rowptr, colidx = ctx.bsr_pattern()
    dev = torch.device("cuda", 0)
    mdk_d = torch.tensor(MDK.astype(np.float32), device=dev)  # FP32 values, exact
    b_d = torch.tensor(b, dtype=torch.float64, device=dev)
    fixed = np.ascontiguousarray(s["fixed"], dtype=np.int32)
    beq = np.ascontiguousarray(beq, dtype=np.float64)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        v_d = torch.full((3 * s["n"],), float("nan"), dtype=torch.float64, device=dev)
        info = eolc.SolveInfo()
        st = eolc.lib.eolc_velocity_solve_static(
            s["n"], rowptr.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
            colidx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ctypes.c_void_p(mdk_d.data_ptr()),
            ctypes.c_void_p(b_d.data_ptr()), fixed.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
            beq.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(fixed), 1e-8, 100000,
            ctypes.c_void_p(v_d.data_ptr()), ctypes.byref(info), ctypes.c_void_p(stream.cuda_stream))
        assert st == eolc.OK, (call, st)
        assert info.status == eolc.OK and info.rel_res <= 1e-8
        v = v_d.cpu().numpy()
        # both solves reach an FP64 relative residual of 1e-8 on the same
        # system; the mixed-path tolerance of the other tests applies
        assert np.abs(v - v_ref).max() <= 1e-6 * np.abs(v_ref).max(), call


def test_static_solve_rejects_oversized_systems():
    import __graft_entry__ as g
    g.build_lib()
    import eolc
    n = 16385  # one row past the limit
    rowptr = np.arange(n + 1, dtype=np.int32)
    colidx = np.arange(n, dtype=np.int32)
    info = eolc.SolveInfo()
    st = eolc.lib.eolc_velocity_solve_static(
        n, rowptr.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
        colidx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ctypes.c_void_p(1),
        ctypes.c_void_p(1), None, None, 0, 1e-8, 10, ctypes.c_void_p(1), ctypes.byref(info), None)
    assert st == eolc.CAPACITY
