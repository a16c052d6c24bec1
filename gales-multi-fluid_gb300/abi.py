"""ctypes view of include/gales_asm.h (struct layouts, constants, prototypes).

The library is loaded from this directory; there is no CPU fallback: loading
raises if libgales_asm.so has not been built.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libgales_asm.so"

MAX_DIM = 3
MAX_COMP = 8
MAX_ND = 2 + MAX_DIM + MAX_COMP - 1
MAX_FLAGS = 32

OK = 0
ERR_BAD_INPUT = 1
ERR_NEG_JACOBIAN = 2
ERR_SINGULAR = 4
ERR_NONFINITE = 8
ERR_CUDA = 16
ERR_UNSUPPORTED = 32
ERR_NO_MEMORY = 64
ERR_MAGMA = 128
ERR_TIMEOUT = 256
NOALLOC_SCRATCH_BYTES = 8 << 20

FORM_FP64 = 0
FORM_MIXED = 1
CH_CUSTOM = 0
CH_IDEAL_GAS = 1
TAU_NONE = 0
MAGMA_LOOKUP_RANGE, MAGMA_VISCOSITY, MAGMA_PAL_ITER = 1, 2, 4  # gales_magma_status bits
SUBMIX_MAGMA, SUBMIX_CUSTOM, SUBMIX_CHEMICAL = 0, 1, 2
TAU_2001 = 2001
TAU_2019 = 2019
TAU_2007 = 2007
TAU_2014 = 2014
VJP_EXACT = 0
VJP_FROZEN = 1
SCATTER_ATOMIC = 0
SCATTER_COLOURED = 1

_p = C.POINTER


class MeshDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("nen", C.c_int32),
        ("n_nodes", C.c_int64), ("n_elements", C.c_int64),
        ("coords", _p(C.c_double)), ("conn", _p(C.c_int32)), ("node_flag", _p(C.c_int32)),
        ("el_on_boundary", _p(C.c_uint8)),
        ("n_bd_sides", C.c_int64),
        ("bd_side_el", _p(C.c_int32)), ("bd_side_local", _p(C.c_int32)), ("bd_side_flag", _p(C.c_int32)),
    ]


class ChemicalDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("reserved", C.c_int32),
        ("rho", C.c_double), ("mu", C.c_double), ("cp", C.c_double), ("cv", C.c_double),
        ("kappa", C.c_double), ("alpha", C.c_double), ("beta", C.c_double),
        ("R", C.c_double), ("gamma", C.c_double), ("chemical_diffusivity", C.c_double),
    ]


class MaterialDesc(C.Structure):
    _fields_ = [("nb_comp", C.c_int32), ("reserved", C.c_int32), ("comp", ChemicalDesc * MAX_COMP)]


class SideBC(C.Structure):
    _fields_ = [
        ("tau_mask", C.c_uint32), ("q_mask", C.c_uint32), ("J_mask", C.c_uint32), ("mass_flux_mask", C.c_uint32),
        ("tau", C.c_double * 9), ("q", C.c_double * 3), ("J", (C.c_double * 8) * 3), ("mass_flux", C.c_double * 3),
    ]


class SetupDesc(C.Structure):
    _fields_ = [
        ("tau", C.c_int32), ("dc_2006", C.c_int32), ("steady_state", C.c_int32), ("reserved", C.c_int32),
        ("dc_sharp", C.c_double), ("dc_scale_fact", C.c_double),
        ("gravity", C.c_double * 3),
        ("p_ref", C.c_double), ("T_ref", C.c_double), ("v_ref", C.c_double * 3),
        ("dirichlet_mask", C.c_uint32 * MAX_FLAGS),
        ("side_bc", SideBC * MAX_FLAGS),
    ]


class MagmaDesc(C.Structure):
    """gales_magma_desc (include/gales_asm.h)."""
    _fields_ = [("oxide_wf", C.c_double * 10), ("melt_kappa", C.c_double),
                ("h2o_wf", C.c_double), ("h2o_l_cp", C.c_double), ("h2o_l_kappa", C.c_double),
                ("co2_wf", C.c_double), ("co2_l_cp", C.c_double), ("co2_l_kappa", C.c_double),
                ("crystal_fraction", C.c_double), ("crystal_rho", C.c_double),
                ("gas_on_mu", C.c_int32), ("crystal_on_mu", C.c_int32), ("n_p", C.c_int32), ("n_T", C.c_int32),
                ("p_table", C.POINTER(C.c_double)), ("T_table", C.POINTER(C.c_double)),
                ("wf_l_h2o", C.POINTER(C.c_double)), ("wf_l_co2", C.POINTER(C.c_double)),
                ("kind", C.c_int32), ("reserved", C.c_int32), ("chemical", ChemicalDesc)]


class SolverParams(C.Structure):
    """gales_solver_params (include/gales_asm.h)."""
    _fields_ = [("rel_res_tol", C.c_double), ("maxsubspace", C.c_int32), ("maxrestarts", C.c_int32),
                ("maxiters", C.c_int64), ("fill", C.c_int32), ("precond", C.c_int32)]


class SolverResult(C.Structure):
    """gales_solver_result (include/gales_asm.h)."""
    _fields_ = [("iterations", C.c_int64), ("abs_res", C.c_double), ("rel_res", C.c_double),
                ("seconds", C.c_double), ("converged", C.c_int32), ("cycles", C.c_int32)]


_lib = None


def lib() -> C.CDLL:
    """Load libgales_asm.so (raises if it is missing: there is no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"GALES CUDA library not built: {LIB_PATH} is missing (run __graft_entry__.build())")
    L = C.CDLL(str(LIB_PATH))
    vp, dp, i32, i64 = C.c_void_p, _p(C.c_double), C.c_int32, C.c_int64
    L.gales_chemical_custom.argtypes = [_p(ChemicalDesc)] + [C.c_double] * 6
    L.gales_chemical_custom.restype = None
    L.gales_chemical_ideal_gas.argtypes = [_p(ChemicalDesc), C.c_double, C.c_double]
    L.gales_chemical_ideal_gas.restype = None
    L.gales_setup_default.argtypes = [_p(SetupDesc), i32]
    L.gales_setup_default.restype = None
    L.gales_asm_create.argtypes = [_p(MeshDesc), _p(MaterialDesc), _p(SetupDesc), C.c_int, _p(vp)]
    L.gales_asm_create.restype = C.c_int
    L.gales_asm_destroy.argtypes = [vp]
    L.gales_asm_destroy.restype = None
    L.gales_asm_pattern.argtypes = [vp, _p(i64), _p(i64), _p(_p(C.c_int64)), _p(_p(C.c_int32))]
    L.gales_asm_pattern.restype = C.c_int
    L.gales_asm_node_graph.argtypes = [vp, _p(i64), _p(i64), _p(_p(C.c_int64)), _p(_p(C.c_int32))]
    L.gales_asm_node_graph.restype = C.c_int
    L.gales_asm_colouring.argtypes = [vp, _p(i32), _p(_p(C.c_int32))]
    L.gales_asm_colouring.restype = C.c_int
    L.gales_asm_set_scatter.argtypes = [vp, i32]
    L.gales_asm_set_scatter.restype = C.c_int
    L.gales_asm_set_chunk.argtypes = [vp, C.c_int64]
    L.gales_asm_set_chunk.restype = C.c_int
    L.gales_asm_assemble.argtypes = [vp, vp, vp, C.c_double, i32, vp, vp, vp]
    L.gales_asm_assemble.restype = C.c_int
    L.gales_asm_assemble_noalloc.argtypes = [vp, vp, vp, C.c_double, i32, vp, vp, vp]
    L.gales_asm_assemble_noalloc.restype = C.c_int
    L.gales_asm_residual.argtypes = [vp, vp, vp, C.c_double, i32, vp, vp]
    L.gales_asm_residual.restype = C.c_int
    L.gales_asm_enqueue.argtypes = [vp, vp, vp, C.c_double, i32, vp, vp, vp]
    L.gales_asm_enqueue.restype = C.c_int
    L.gales_asm_sync.argtypes = [vp, vp]
    L.gales_asm_sync.restype = C.c_int
    L.gales_asm_vjp.argtypes = [vp, vp, vp, C.c_double, vp, i32, vp, vp, vp]
    L.gales_asm_vjp.restype = C.c_int
    L.gales_asm_element_blocks.argtypes = [vp, vp, vp, C.c_double, i32, i32, _p(C.c_int32), i64, vp, vp, vp]
    L.gales_asm_element_blocks.restype = C.c_int
    L.gales_asm_norm2.argtypes = [vp, vp, dp, vp]
    L.gales_asm_norm2.restype = C.c_int
    L.gales_asm_status.argtypes = [vp, _p(i64)]
    L.gales_asm_status.restype = C.c_int
    L.gales_asm_last_error.argtypes = [vp]
    L.gales_asm_last_error.restype = C.c_char_p
    L.gales_asm_last_ms.argtypes = [vp]
    L.gales_asm_last_ms.restype = C.c_double
    L.gales_asm_last_phase_ms.argtypes = [vp, i32]
    L.gales_asm_last_phase_ms.restype = C.c_double
    L.gales_asm_launch_count.argtypes = [vp]
    L.gales_asm_launch_count.restype = C.c_int64
    L.gales_asm_adaptive_dt.argtypes = [vp, vp, C.c_double, C.c_double, C.c_double, C.c_double, vp, _p(C.c_double), vp]
    L.gales_asm_adaptive_dt.restype = C.c_int
    L.gales_asm_secondary_dofs.argtypes = [vp, vp, vp, vp]
    L.gales_asm_secondary_dofs.restype = C.c_int
    L.gales_pressure_profile.argtypes = [_p(MaterialDesc), C.c_double, C.c_double, i32, dp, dp, dp, dp, dp]
    L.gales_pressure_profile.restype = C.c_int
    L.gales_pressure_interpolate.argtypes = [dp, dp, i32, dp, i64, dp]
    L.gales_pressure_interpolate.restype = C.c_int
    L.gales_dt_update.argtypes = [C.c_double] * 4
    L.gales_dt_update.restype = C.c_double
    L.gales_mesh_read.argtypes = [C.c_char_p, i32, _p(vp), C.c_char_p, i32]
    L.gales_mesh_read.restype = C.c_int
    L.gales_mesh_file_desc.argtypes = [vp, _p(MeshDesc), _p(_p(C.c_int64)), _p(_p(C.c_int64))]
    L.gales_mesh_file_desc.restype = C.c_int
    L.gales_mesh_file_free.argtypes = [vp]
    L.gales_mesh_file_free.restype = None
    sp_ = _p(SolverParams)
    L.gales_solver_default.argtypes = [sp_]
    L.gales_solver_default.restype = None
    L.gales_solver_create.argtypes = [vp, sp_, _p(vp)]
    L.gales_solver_create.restype = C.c_int
    L.gales_solver_solve.argtypes = [vp, vp, vp, vp, _p(SolverResult), vp]
    L.gales_solver_solve.restype = C.c_int
    L.gales_solver_factorize.argtypes = [vp, vp, vp]
    L.gales_solver_factorize.restype = C.c_int
    L.gales_solver_apply.argtypes = [vp, vp, vp, vp]
    L.gales_solver_apply.restype = C.c_int
    L.gales_solver_factor.argtypes = [vp, _p(i64), _p(i64), _p(_p(C.c_int64)), _p(_p(C.c_int32)), vp]
    L.gales_solver_factor.restype = C.c_int
    L.gales_solver_levels.argtypes = [vp, _p(i32), _p(i32)]
    L.gales_solver_levels.restype = C.c_int
    L.gales_solver_correct.argtypes = [vp, vp, vp, i32, i32, C.c_double, C.c_double, vp]
    L.gales_solver_correct.restype = C.c_int
    L.gales_solver_launches.argtypes = [vp]
    L.gales_solver_launches.restype = C.c_int64
    L.gales_solver_last_error.argtypes = [vp]
    L.gales_solver_last_error.restype = C.c_char_p
    L.gales_solver_destroy.argtypes = [vp]
    L.gales_solver_destroy.restype = None
    L.gales_iluk_pattern.argtypes = [i64, _p(C.c_int64), _p(C.c_int32), i32, _p(i64), _p(C.c_int64),
                                     _p(C.c_int32), _p(C.c_int32), _p(C.c_int32), _p(C.c_int32)]
    L.gales_iluk_pattern.restype = C.c_int
    L.gales_magma_create.argtypes = [_p(MagmaDesc), i32, _p(vp)]
    L.gales_magma_create.restype = C.c_int
    L.gales_magma_properties.argtypes = [vp, vp, vp, vp, vp, i64, vp, vp, vp]
    L.gales_magma_properties.restype = C.c_int
    L.gales_magma_status.argtypes = [vp]
    L.gales_magma_status.restype = C.c_int
    L.gales_magma_last_error.argtypes = [vp]
    L.gales_magma_last_error.restype = C.c_char_p
    L.gales_magma_destroy.argtypes = [vp]
    L.gales_magma_destroy.restype = None
    L.gales_asm_set_magma.argtypes = [vp, vp]
    L.gales_asm_set_magma.restype = C.c_int
    L.gales_asm_magma_fractions.argtypes = [vp, vp, vp, vp]
    L.gales_asm_magma_fractions.restype = C.c_int
    _lib = L
    return L


EXPORTED = [
    "gales_chemical_custom", "gales_chemical_ideal_gas", "gales_setup_default",
    "gales_asm_create", "gales_asm_destroy", "gales_asm_pattern", "gales_asm_node_graph",
    "gales_asm_colouring", "gales_asm_set_scatter", "gales_asm_set_chunk", "gales_asm_assemble", "gales_asm_assemble_noalloc",
    "gales_asm_residual", "gales_asm_enqueue", "gales_asm_sync",
    "gales_asm_vjp", "gales_asm_element_blocks", "gales_asm_norm2", "gales_asm_status", "gales_asm_last_error",
    "gales_asm_last_ms", "gales_asm_last_phase_ms", "gales_asm_launch_count",
    "gales_mesh_read", "gales_mesh_file_desc", "gales_mesh_file_free", "gales_asm_adaptive_dt", "gales_dt_update",
    "gales_asm_secondary_dofs", "gales_pressure_profile", "gales_pressure_interpolate",
    "gales_solver_default", "gales_solver_create", "gales_solver_solve", "gales_solver_factorize",
    "gales_solver_apply", "gales_solver_factor", "gales_solver_levels", "gales_solver_correct",
    "gales_solver_launches", "gales_solver_last_error", "gales_solver_destroy", "gales_iluk_pattern",
    "gales_magma_create", "gales_magma_properties", "gales_magma_status", "gales_magma_last_error",
    "gales_magma_destroy", "gales_asm_set_magma", "gales_asm_magma_fractions",
]
