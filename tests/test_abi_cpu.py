"""The C-ABI library loads and exports every entry point of include/gales_asm.h; the
ctypes descriptors match the C layouts; host-only helpers agree with the Python
mirror.  No GPU compute is called here."""
import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gales_asm.h"


@pytest.fixture(scope="module")
def lib(gm):
    b = __import__("importlib").import_module("gales-multi-fluid_gb300.build")
    b.build()
    return gm.abi.lib()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gales_\w+)\s*\(", text)))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    for n in ["gales_asm_create", "gales_asm_assemble", "gales_asm_residual", "gales_asm_vjp",
              "gales_asm_pattern", "gales_asm_destroy", "gales_asm_last_error", "gales_asm_element_blocks"]:
        assert n in names


def test_library_exports_every_declared_symbol(lib, gm):
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) == set(gm.abi.EXPORTED)


def test_struct_layouts_match_c(gm, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "sz.c"
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "{HEADER}"\n'
                   'int main(){printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(gales_mesh_desc),'
                   'sizeof(gales_chemical_desc), sizeof(gales_material_desc), sizeof(gales_side_bc),'
                   'sizeof(gales_setup_desc), offsetof(gales_setup_desc, side_bc),'
                   'offsetof(gales_setup_desc, dirichlet_mask));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run([cc, str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    a = gm.abi
    assert out == [C.sizeof(a.MeshDesc), C.sizeof(a.ChemicalDesc), C.sizeof(a.MaterialDesc),
                   C.sizeof(a.SideBC), C.sizeof(a.SetupDesc), a.SetupDesc.side_bc.offset,
                   a.SetupDesc.dirichlet_mask.offset]


def test_solver_and_magma_struct_layouts_match_c(gm, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "sz2.c"
    fields = [("gales_solver_params", "rel_res_tol"), ("gales_solver_params", "maxiters"),
              ("gales_solver_params", "precond"), ("gales_solver_result", "iterations"),
              ("gales_solver_result", "seconds"), ("gales_solver_result", "cycles"),
              ("gales_magma_desc", "melt_kappa"), ("gales_magma_desc", "gas_on_mu"),
              ("gales_magma_desc", "n_T"), ("gales_magma_desc", "p_table"), ("gales_magma_desc", "wf_l_co2")]
    body = " ".join(f'printf("%zu ", offsetof({t}, {f}));' for t, f in fields)
    body += ' printf("%zu %zu %zu' + chr(92) + 'n", sizeof(gales_solver_params), sizeof(gales_solver_result),' \
            ' sizeof(gales_magma_desc));'
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "{HEADER}"\nint main(){{{body} return 0;}}\n')
    exe = tmp_path / "sz2"
    subprocess.run([cc, str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    a = gm.abi
    types = {"gales_solver_params": a.SolverParams, "gales_solver_result": a.SolverResult,
             "gales_magma_desc": a.MagmaDesc}
    want = [getattr(types[t], f).offset for t, f in fields]
    want += [C.sizeof(a.SolverParams), C.sizeof(a.SolverResult), C.sizeof(a.MagmaDesc)]
    assert out == want


def test_c_constructors_match_python(lib, gm):
    a = gm.abi
    c = a.ChemicalDesc()
    lib.gales_chemical_ideal_gas(C.byref(c), 0.01802, 1.4)
    p = gm.ideal_gas(0.01802, 1.4)
    for f, _ in a.ChemicalDesc._fields_:
        assert getattr(c, f) == getattr(p, f), f
    lib.gales_chemical_custom(C.byref(c), 2400.0, 1e3, 1200.0, 1.5, 3e-5, 1e-10)
    p = gm.custom_chemical(2400.0, 1e3, 1200.0, 1.5, 3e-5, 1e-10)
    for f, _ in a.ChemicalDesc._fields_:
        assert getattr(c, f) == getattr(p, f), f
    s = a.SetupDesc()
    lib.gales_setup_default(C.byref(s), 2)
    ps = gm.Setup(2)
    assert s.tau == ps.desc.tau == 2019 and s.dc_2006 == 1 and s.dc_sharp == 2.0
    assert list(s.gravity) == list(ps.desc.gravity) == [0.0, -9.81, 0.0]
    assert s.p_ref == 70e6 and s.T_ref == 1300.0


def test_create_rejects_bad_input_before_device_work(lib, gm, syn):
    mesh = syn.channel_tri(4, 2)
    bad = gm.Mesh(mesh.coords, mesh.conn.copy(), mesh.node_flag, mesh.el_on_boundary, mesh.bd_sides)
    bad.conn[0, 0] = 10_000
    mat = syn.material_for(2)
    setup = syn.setup_for(2, 2)
    h = C.c_void_p()
    rc = lib.gales_asm_create(C.byref(bad.desc()), C.byref(mat.desc), C.byref(setup.desc), 0, C.byref(h))
    assert rc == gm.abi.ERR_BAD_INPUT and not h.value
    s2 = syn.setup_for(2, 2)
    s2.desc.tau = 1999
    rc = lib.gales_asm_create(C.byref(mesh.desc()), C.byref(mat.desc), C.byref(s2.desc), 0, C.byref(h))
    assert rc == gm.abi.ERR_BAD_INPUT
    m5 = gm.Material([gm.custom_chemical(1, 1, 1, 1, 0, 0)] * 4)
    m5.desc.nb_comp = 5
    rc = lib.gales_asm_create(C.byref(mesh.desc()), C.byref(m5.desc), C.byref(setup.desc), 0, C.byref(h))
    assert rc == gm.abi.ERR_UNSUPPORTED


def test_null_handle_calls_are_safe(lib):
    assert lib.gales_asm_assemble(None, None, None, 1e-3, 0, None, None, None) == 1
    assert lib.gales_asm_status(None, None) == 1
    assert lib.gales_asm_last_error(None) == b"null handle"


def test_solver_and_magma_entry_points_reject_bad_input(lib, gm):
    """Null handles and invalid descriptors return GALES_ERR_BAD_INPUT before any device
    work; the host-only ILU pattern checks its arguments."""
    a = gm.abi
    out = C.c_void_p()
    assert lib.gales_solver_create(None, None, C.byref(out)) == 1
    assert lib.gales_solver_solve(None, None, None, None, None, None) == 1
    assert lib.gales_solver_last_error(None) == b"null handle"
    lib.gales_solver_destroy(None)
    d = a.MagmaDesc()
    d.n_p = 1  # a table needs two pressures
    assert lib.gales_magma_create(C.byref(d), 1, C.byref(out)) == 1 and not out.value
    d.n_p = 3
    assert lib.gales_magma_create(C.byref(d), 1, C.byref(out)) == 1  # tables missing
    assert lib.gales_magma_create(C.byref(d), 0, C.byref(out)) == 1
    assert lib.gales_magma_properties(None, None, None, None, None, 0, None, None, None) == 1
    assert lib.gales_magma_last_error(None) == b"null handle"
    lib.gales_magma_destroy(None)
    rp = np.array([0, 1], dtype=np.int64)
    col = np.array([0], dtype=np.int32)
    nnz = C.c_int64()
    i64p, i32p = C.POINTER(C.c_int64), C.POINTER(C.c_int32)
    assert lib.gales_iluk_pattern(1, rp.ctypes.data_as(i64p), col.ctypes.data_as(i32p), -1, C.byref(nnz),
                                  None, None, None, None, None) == 1
    assert lib.gales_iluk_pattern(1, rp.ctypes.data_as(i64p), col.ctypes.data_as(i32p), 0, C.byref(nnz),
                                  None, None, None, None, None) == 0 and nnz.value == 1
