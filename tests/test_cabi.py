"""CPU checks of the C ABI library: it loads and exports every symbol that
include/eolc.h declares (no compute calls: this host has no GPU), and the
ctypes mirrors of the structs have the C layout."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "eolc.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(eolc_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build_lib()
    return g.LIB


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    syms = declared_symbols()
    assert len(syms) >= 14
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_lists_all_exports(built):
    import eolc
    assert sorted(eolc.EXPORTS) == declared_symbols()


def test_struct_layouts_match_c(built, tmp_path):
    """sizeof / offsetof of the ABI structs compiled by the C compiler."""
    import eolc
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stddef.h>\n#include <stdio.h>\n#include "%s"\n'
        'int main(void){printf("%%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu'
        ' %%zu %%zu %%zu %%zu %%zu\\n",'
        ' sizeof(eolc_contact), offsetof(eolc_contact, count1), offsetof(eolc_contact, source),'
        ' sizeof(eolc_box), sizeof(eolc_material), sizeof(eolc_solve_opts),'
        ' sizeof(eolc_solve_info), sizeof(eolc_batch_info), offsetof(eolc_batch_info, iterations),'
        ' offsetof(eolc_batch_info, step_ms), sizeof(eolc_ineq_info),'
        ' offsetof(eolc_ineq_info, max_violation), sizeof(eolc_rows), offsetof(eolc_rows, rhs),'
        ' sizeof(eolc_eol_mesh), offsetof(eolc_eol_mesh, edges), offsetof(eolc_eol_mesh, n_eol));'
        ' return 0;}\n'
        % HEADER)
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    want = [ctypes.sizeof(eolc.Contact), eolc.Contact.count1.offset, eolc.Contact.source.offset,
            ctypes.sizeof(eolc.Box), ctypes.sizeof(eolc.Material), ctypes.sizeof(eolc.SolveOpts),
            ctypes.sizeof(eolc.SolveInfo), ctypes.sizeof(eolc.BatchInfo),
            eolc.BatchInfo.iterations.offset, eolc.BatchInfo.step_ms.offset,
            ctypes.sizeof(eolc.IneqInfo), eolc.IneqInfo.max_violation.offset,
            ctypes.sizeof(eolc.Rows), eolc.Rows.rhs.offset, ctypes.sizeof(eolc.EolMesh),
            eolc.EolMesh.edges.offset, eolc.EolMesh.n_eol.offset]
    assert got == want


def test_library_reports_missing_device_cleanly(built):
    """Without a GPU, eolc_create fails with a status instead of aborting."""
    import eolc
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    h = ctypes.c_void_p()
    st = eolc.lib.eolc_create(ctypes.byref(h), 0)
    assert st == eolc.CUDA_ERROR and not h.value
