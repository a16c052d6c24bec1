"""GB300 assembly of the fluid_mc equations of GALES-multi-fluid — Python host side.

This mirrors the reference's assembly-facing interface for the hot path:

  reference (C++, sim/fluid_mc/P0/main.cpp)          here
  ----------------------------------------------     ---------------------------------------------
  fluid_properties props  (props.txt mix_of_ch)      Material([custom_chemical(...), ideal_gas(...)])
  read_setup setup        (setup.txt flags)           Setup(dim, tau=2019, dc_2006=True, ...)
  fluid_ic_bc / fluid_dofs_ic_bc policies             Setup.dirichlet / Setup.neumann / Setup.mass_flux
  Mesh<dim>               (mesh file)                 Mesh(coords, conn, node_flag, ...)
  linear_system lp(model) (linear_system.hpp:40-66)   LinearSystem (pattern from FluidAssembly.pattern())
  fluid_assembly::execute() -> seconds                FluidAssembly.execute(I, P, dt, lp) -> seconds
  residual_check::execute (residual_check.hpp:42-80)  ResidualCheck.execute(b, it_count)

All arithmetic runs in the CUDA library libgales_asm.so through the C ABI of
include/gales_asm.h; nothing here computes the assembly on the CPU.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import abi
from .abi import (FORM_FP64, FORM_MIXED, SCATTER_ATOMIC, SCATTER_COLOURED, TAU_2001, TAU_2007,
                  TAU_2014, TAU_2019, TAU_NONE, VJP_EXACT, VJP_FROZEN)

R_UNIVERSAL = 8.314462  # chemicals.hpp:229


class GalesError(RuntimeError):
    def __init__(self, code: int, msg: str, first_bad: int = -1):
        super().__init__(f"GALES status {code:#x}: {msg}")
        self.code = code
        self.first_bad = first_bad


# ---------------------------------------------------------------------------
# Materials (src/fem/physical_props/fluid/chemicals.hpp, fluid_properties.hpp)

def custom_chemical(rho: float, mu: float, cp: float, kappa: float, alpha: float, beta: float,
                    chemical_diffusivity: float = 1.e-10) -> abi.ChemicalDesc:
    """custom_chemical(rho, mu, cp, kappa, alpha, beta) of chemicals.hpp:23-33."""
    c = abi.ChemicalDesc()
    c.kind = abi.CH_CUSTOM
    c.rho, c.mu, c.cp, c.kappa, c.alpha, c.beta = rho, mu, cp, kappa, alpha, beta
    c.cv = cp
    c.chemical_diffusivity = chemical_diffusivity
    return c


def ideal_gas(molar_mass: float, gamma: float = 1.4, chemical_diffusivity: float = 1.e-10) -> abi.ChemicalDesc:
    """ideal_gas(molar_mass, gamma) of chemicals.hpp:237-246 (mu = 1e-5, kappa = mu cp / 0.72)."""
    c = abi.ChemicalDesc()
    c.kind = abi.CH_IDEAL_GAS
    c.R = R_UNIVERSAL / molar_mass
    c.gamma = gamma
    c.cv = c.R / (gamma - 1.0)
    c.cp = gamma * c.cv
    c.mu = 1.e-5
    c.kappa = c.mu * c.cp / 0.72
    c.chemical_diffusivity = chemical_diffusivity
    return c


IDEAL_GAS_MOLAR_MASS = {"H2O": 0.01802, "CO2": 0.04401, "AIR": 0.02897, "HE": 0.004, "ARGON": 0.06}


def ideal_gas_named(name: str) -> abi.ChemicalDesc:
    """ideal_gas(std::string) of chemicals.hpp:201-234."""
    key = name.upper()
    gamma = 1.67 if key in ("HE", "ARGON") else 1.4
    return ideal_gas(IDEAL_GAS_MOLAR_MASS[key], gamma)


def ideal_gas_params(molar_mass: float, mu: float, cp: float, kappa: float,
                     chemical_diffusivity: float = 1.e-10) -> abi.ChemicalDesc:
    """Ideal gas parameterised by (M, mu, cp): R = R_u/M, cv = cp - R, gamma = cp/cv.

    This is the parameterisation in which the VJP reports d/d(theta) for a gas
    component; at the reference constructor's values it reproduces ideal_gas().
    """
    c = abi.ChemicalDesc()
    c.kind = abi.CH_IDEAL_GAS
    c.R = R_UNIVERSAL / molar_mass
    c.cp = cp
    c.cv = cp - c.R
    c.gamma = cp / c.cv
    c.mu = mu
    c.kappa = kappa
    c.chemical_diffusivity = chemical_diffusivity
    return c


class Material:
    """mix_of_ch mixture of 1..4 chemicals (fluid_properties.hpp:199-227)."""

    def __init__(self, chemicals: Sequence[abi.ChemicalDesc]):
        if not 1 <= len(chemicals) <= 4:
            raise ValueError("nb_comp must be 1..4")
        self.chemicals = list(chemicals)
        self.desc = abi.MaterialDesc()
        self.desc.nb_comp = len(chemicals)
        for i, c in enumerate(chemicals):
            self.desc.comp[i] = c

    @property
    def nb_comp(self) -> int:
        return self.desc.nb_comp


# ---------------------------------------------------------------------------
# Setup flags and boundary-condition policy as data

class Setup:
    """read_setup flags (setup.txt:24-31) plus the ic_bc policy of one case.

    dirichlet[flag] = list of constrained dof indices for nodes with that flag
    (fluid_dofs_ic_bc::dof_constraint); neumann/mass flux overrides per side flag
    (fluid_ic_bc::neumann_*, mass_flux*).
    """

    def __init__(self, dim: int, tau: int = TAU_2019, dc_2006: bool = True, dc_sharp: float = 2.0,
                 dc_scale_fact: float = 1.0, steady_state: bool = False,
                 gravity: Optional[Sequence[float]] = None, p_ref: float = 70.e6, T_ref: float = 1300.0,
                 v_ref: Sequence[float] = (0.0, 0.0, 0.0)):
        self.dim = dim
        d = abi.SetupDesc()
        d.tau = tau
        d.dc_2006 = int(dc_2006)
        d.steady_state = int(steady_state)
        d.dc_sharp = dc_sharp
        d.dc_scale_fact = dc_scale_fact
        g = gravity if gravity is not None else ((0.0, -9.81, 0.0) if dim == 2 else (0.0, 0.0, 0.0))
        for i in range(3):
            d.gravity[i] = g[i] if i < len(g) else 0.0
            d.v_ref[i] = v_ref[i] if i < len(v_ref) else 0.0
        d.p_ref = p_ref
        d.T_ref = T_ref
        self.desc = d

    def dirichlet(self, flag: int, dofs: Sequence[int]) -> "Setup":
        m = 0
        for k in dofs:
            m |= 1 << k
        self.desc.dirichlet_mask[flag] |= m
        return self

    def dirichlet_all_flags(self, dofs: Sequence[int]) -> "Setup":
        for f in range(abi.MAX_FLAGS):
            self.dirichlet(f, dofs)
        return self

    def neumann_tau(self, flag: int, k: int, j: int, value: float = 0.0) -> "Setup":
        lo, hi = min(k, j), max(k, j)
        bc = self.desc.side_bc[flag]
        bc.tau_mask |= 1 << (lo * 3 + hi)
        bc.tau[lo * 3 + hi] = value
        return self

    def neumann_q(self, flag: int, k: int, value: float = 0.0) -> "Setup":
        bc = self.desc.side_bc[flag]
        bc.q_mask |= 1 << k
        bc.q[k] = value
        return self

    def neumann_J(self, flag: int, k: int, comp: int, value: float = 0.0) -> "Setup":
        bc = self.desc.side_bc[flag]
        bc.J_mask |= 1 << (k * 8 + comp)
        bc.J[k][comp] = value
        return self

    def mass_flux(self, flag: int, k: int, value: float) -> "Setup":
        bc = self.desc.side_bc[flag]
        bc.mass_flux_mask |= 1 << k
        bc.mass_flux[k] = value
        return self


def p0_policy(setup: Setup, nb_comp: int, wall_flag: int = 5, dirichlet_T_everywhere: bool = True) -> Setup:
    """The shipped P0 case's boundary policy (fluid_ic_bc.hpp:84-194):
    no-slip velocity on nodes with flag 5, T Dirichlet on every node, and on side
    flag 5 zero heat flux and zero species-0 flux in every direction."""
    dim = setup.dim
    setup.dirichlet(wall_flag, list(range(1, 1 + dim)))
    if dirichlet_T_everywhere:
        setup.dirichlet_all_flags([dim + 1])
    for k in range(dim):
        setup.neumann_q(wall_flag, k, 0.0)
        if nb_comp > 1:
            setup.neumann_J(wall_flag, k, 0, 0.0)
    return setup


# ---------------------------------------------------------------------------
# Mesh

def _ptr(a: Optional[np.ndarray], ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


@dataclass
class Mesh:
    """One-rank mesh: node ids are 0..n_nodes-1 (= node gid).

    Element node order and local side numbering follow element.hpp; bd_sides is
    an (n, 3) array of (element, local side, side flag > 0).
    """
    coords: np.ndarray               # (n_nodes, dim) float64
    conn: np.ndarray                 # (n_el, nen) int32
    node_flag: np.ndarray            # (n_nodes,) int32
    el_on_boundary: np.ndarray       # (n_el,) uint8
    bd_sides: np.ndarray             # (n_bd, 3) int32
    name: str = ""
    _desc: Optional[abi.MeshDesc] = field(default=None, repr=False)

    def __post_init__(self):
        self.coords = np.ascontiguousarray(self.coords, dtype=np.float64)
        self.conn = np.ascontiguousarray(self.conn, dtype=np.int32)
        self.node_flag = np.ascontiguousarray(self.node_flag, dtype=np.int32)
        self.el_on_boundary = np.ascontiguousarray(self.el_on_boundary, dtype=np.uint8)
        bd = np.asarray(self.bd_sides, dtype=np.int32).reshape(-1, 3)
        self._bd_el = np.ascontiguousarray(bd[:, 0])
        self._bd_loc = np.ascontiguousarray(bd[:, 1])
        self._bd_flag = np.ascontiguousarray(bd[:, 2])
        self.bd_sides = bd

    @property
    def dim(self) -> int:
        return self.coords.shape[1]

    @property
    def nen(self) -> int:
        return self.conn.shape[1]

    @property
    def n_nodes(self) -> int:
        return self.coords.shape[0]

    @property
    def n_elements(self) -> int:
        return self.conn.shape[0]

    def desc(self) -> abi.MeshDesc:
        if self._desc is None:
            d = abi.MeshDesc()
            d.dim, d.nen = self.dim, self.nen
            d.n_nodes, d.n_elements = self.n_nodes, self.n_elements
            d.coords = _ptr(self.coords, C.c_double)
            d.conn = _ptr(self.conn, C.c_int32)
            d.node_flag = _ptr(self.node_flag, C.c_int32)
            d.el_on_boundary = _ptr(self.el_on_boundary, C.c_uint8)
            d.n_bd_sides = len(self._bd_el)
            d.bd_side_el = _ptr(self._bd_el, C.c_int32)
            d.bd_side_local = _ptr(self._bd_loc, C.c_int32)
            d.bd_side_flag = _ptr(self._bd_flag, C.c_int32)
            self._desc = d
        return self._desc


def nb_dofs(dim: int, nb_comp: int) -> int:
    """nb_dofs_f = 2 + dim + nb_comp - 1 (main.cpp:82)."""
    return 2 + dim + nb_comp - 1


# ---------------------------------------------------------------------------
# Linear system and assembly

def _addr(x) -> int:
    """Address of a numpy array or a torch tensor (host or device)."""
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("array must be C-contiguous")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return x.data_ptr()
    raise TypeError(f"unsupported buffer type {type(x)}")


class LinearSystem:
    """linear_system (linear_system.hpp:35-105): CSR matrix A and rhs b.

    row_ptr/col are the one-rank FECrsGraph (sorted global columns per row);
    vals and rhs are float64 numpy arrays or torch tensors (host or cuda).
    """

    def __init__(self, row_ptr: Optional[np.ndarray], col: Optional[np.ndarray], vals=None, rhs=None):
        self.row_ptr = row_ptr
        self.col = col
        if row_ptr is None and (vals is None or rhs is None):
            raise ValueError("without a pattern, vals and rhs must be given")
        self.vals = vals if vals is not None else np.zeros(int(row_ptr[-1]), dtype=np.float64)
        self.rhs = rhs if rhs is not None else np.zeros(len(row_ptr) - 1, dtype=np.float64)

    @property
    def n_rows(self) -> int:
        return len(self.rhs)

    def matrix_scipy(self):
        import scipy.sparse as sp
        vals = self.vals if isinstance(self.vals, np.ndarray) else self.vals.detach().cpu().numpy()
        return sp.csr_matrix((vals, self.col, self.row_ptr), shape=(self.n_rows, self.n_rows))

    def clear(self):
        """linear_system::clear (linear_system.hpp:90-94); execute() does this itself."""
        self.vals[...] = 0.0 if isinstance(self.vals, np.ndarray) else self.vals.zero_()
        self.rhs[...] = 0.0 if isinstance(self.rhs, np.ndarray) else self.rhs.zero_()


class FluidAssembly:
    """fluid_assembly<fluid<ic_bc,dim>, scatter<dofs_ic_bc>, dim> on one GPU.

    The constructor also does what linear_system's constructor (graph build) and
    the fluid integral's constructor (u_ref_inv) do in the reference.
    """

    def __init__(self, mesh: Mesh, material: Material, setup: Setup, device: int = 0):
        self.mesh, self.material, self.setup = mesh, material, setup
        self.dim = mesh.dim
        self.nb_comp = material.nb_comp
        self.nd = nb_dofs(self.dim, self.nb_comp)
        self.n_rows = mesh.n_nodes * self.nd
        L = abi.lib()
        h = C.c_void_p()
        rc = L.gales_asm_create(C.byref(mesh.desc()), C.byref(material.desc), C.byref(setup.desc), device,
                                C.byref(h))
        if rc != 0:
            raise GalesError(rc, "gales_asm_create failed (see stderr)")
        self._h = h
        self._L = L
        self.last_seconds = 0.0

    def close(self):
        if getattr(self, "_h", None):
            self._L.gales_asm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            fb = C.c_int64(-1)
            self._L.gales_asm_status(self._h, C.byref(fb))
            raise GalesError(rc, self._L.gales_asm_last_error(self._h).decode(), fb.value)

    # pattern / graph / colouring
    def pattern(self):
        n_rows, nnz = C.c_int64(), C.c_int64()
        rp, cl = C.POINTER(C.c_int64)(), C.POINTER(C.c_int32)()
        self._check(self._L.gales_asm_pattern(self._h, C.byref(n_rows), C.byref(nnz), C.byref(rp), C.byref(cl)))
        row_ptr = np.ctypeslib.as_array(rp, shape=(n_rows.value + 1,)).copy()
        col = np.ctypeslib.as_array(cl, shape=(nnz.value,)).copy() if nnz.value else np.zeros(0, np.int32)
        return row_ptr, col

    def nnz(self) -> int:
        n, nn = C.c_int64(), C.c_int64()
        self._check(self._L.gales_asm_node_graph(self._h, C.byref(n), C.byref(nn), None, None))
        return nn.value * self.nd * self.nd

    def node_graph(self):
        n, nn = C.c_int64(), C.c_int64()
        rp, cl = C.POINTER(C.c_int64)(), C.POINTER(C.c_int32)()
        self._check(self._L.gales_asm_node_graph(self._h, C.byref(n), C.byref(nn), C.byref(rp), C.byref(cl)))
        return (np.ctypeslib.as_array(rp, shape=(n.value + 1,)).copy(),
                np.ctypeslib.as_array(cl, shape=(nn.value,)).copy())

    def colouring(self):
        nc = C.c_int32()
        cp = C.POINTER(C.c_int32)()
        self._check(self._L.gales_asm_colouring(self._h, C.byref(nc), C.byref(cp)))
        return np.ctypeslib.as_array(cp, shape=(self.mesh.n_elements,)).copy(), nc.value

    def linear_system(self, device=None) -> LinearSystem:
        row_ptr, col = self.pattern()
        if device is None:
            return LinearSystem(row_ptr, col)
        import torch
        vals = torch.zeros(int(row_ptr[-1]), dtype=torch.float64, device=device)
        rhs = torch.zeros(len(row_ptr) - 1, dtype=torch.float64, device=device)
        return LinearSystem(row_ptr, col, vals, rhs)

    def nnz_from_graph(self) -> int:
        """nnz of the CSR pattern from the node graph (nd^2 entries per node pair)."""
        rp, _ = self.node_graph()
        return int(rp[-1]) * self.nd * self.nd

    def device_system(self, device) -> LinearSystem:
        """CSR values and rhs on the device without building the scalar pattern
        (row_ptr/col stay None): for meshes whose pattern would not fit the host."""
        import torch
        vals = torch.zeros(self.nnz_from_graph(), dtype=torch.float64, device=device)
        rhs = torch.zeros(self.n_rows, dtype=torch.float64, device=device)
        return LinearSystem(None, None, vals, rhs)

    def set_scatter(self, mode: int):
        self._check(self._L.gales_asm_set_scatter(self._h, mode))

    def set_chunk(self, elements: int = 0):
        """Elements per interior chunk (0: the default, as many as 3 GiB of records hold)."""
        self._check(self._L.gales_asm_set_chunk(self._h, int(elements)))

    # the hot path
    def execute(self, I, P, dt: float, lp: LinearSystem, form: int = FORM_FP64, stream: int = 0) -> float:
        """fluid_assembly::execute(): fill lp.vals and lp.rhs; returns wall seconds."""
        t0 = time.perf_counter()
        self._check(self._L.gales_asm_assemble(self._h, _addr(I), _addr(P), float(dt), form, _addr(lp.vals),
                                               _addr(lp.rhs), stream or None))
        self.last_seconds = time.perf_counter() - t0
        return self.last_seconds

    def execute_noalloc(self, I, P, dt: float, lp: LinearSystem, form: int = FORM_FP64, stream: int = 0) -> float:
        """Same as execute() but allocates nothing: for callers that must keep a fixed
        device-memory footprint.  All buffers must be CUDA tensors; calls share one
        library-wide scratch array, so calls that overlap on the GPU must be ordered."""
        t0 = time.perf_counter()
        self._check(self._L.gales_asm_assemble_noalloc(self._h, _addr(I), _addr(P), float(dt), form,
                                                       _addr(lp.vals), _addr(lp.rhs), stream or None))
        return time.perf_counter() - t0

    def residual(self, I, P, dt: float, rhs, form: int = FORM_FP64, stream: int = 0) -> float:
        t0 = time.perf_counter()
        self._check(self._L.gales_asm_residual(self._h, _addr(I), _addr(P), float(dt), form, _addr(rhs),
                                               stream or None))
        return time.perf_counter() - t0

    def enqueue(self, I, P, dt: float, lp: "LinearSystem", form: int = FORM_MIXED, stream: int = 0,
                want_matrix: bool = True):
        """Enqueue one assembly (device tensors only) without synchronising: capture-safe,
        so repeated calls can be recorded into a CUDA graph.  Check with sync()."""
        self._check(self._L.gales_asm_enqueue(self._h, _addr(I), _addr(P), float(dt), form,
                                              _addr(lp.vals) if want_matrix else None, _addr(lp.rhs),
                                              stream or None))

    def sync(self, stream: int = 0):
        """Wait for the stream and raise if any enqueued assembly reported an error."""
        self._check(self._L.gales_asm_sync(self._h, stream or None))

    def vjp(self, I, P, dt: float, lam, mode: int, g_state, g_params=None, stream: int = 0):
        self._check(self._L.gales_asm_vjp(self._h, _addr(I), _addr(P), float(dt), _addr(lam), mode,
                                          _addr(g_state), _addr(g_params) if g_params is not None else None,
                                          stream or None))

    def norm2(self, rhs) -> float:
        """||b||_2 on the device (residual_check.hpp:48-51)."""
        out = C.c_double()
        self._check(self._L.gales_asm_norm2(self._h, _addr(rhs), C.byref(out), None))
        return out.value

    def adaptive_dt(self, I, dt: float, cfl: float, dt_min: float, dt_max: float, dt_el=None,
                    stream: int = 0) -> float:
        """adaptive_time_criteria::f_mc + set_dt (adaptive_time_step.hpp:183-260, 380-393):
        the next time step from state I; dt_el (n_elements, host or device) optionally
        receives every element's smallest Gauss-point value."""
        out = C.c_double()
        self._check(self._L.gales_asm_adaptive_dt(self._h, _addr(I), float(dt), float(cfl), float(dt_min),
                                                  float(dt_max), _addr(dt_el) if dt_el is not None else None,
                                                  C.byref(out), stream or None))
        return out.value

    SECONDARY_FIELDS = ("rho", "mu", "cp", "cv", "alpha", "beta", "kappa", "sound_speed")

    @staticmethod
    def MAGMA_FRACTION_FIELDS(nb_comp: int):
        """Row names of magma_fractions (the names secondary_dofs.hpp:163-176 prints)."""
        per = [n for c in range(nb_comp) for n in (f"vf_g_comp_{c}", f"vf_comp_{c}")]
        return tuple(per) + ("vf_g_on_total", "vf_h2o_g_on_total", "vf_co2_g_on_total", "wf_g_on_total",
                             "wf_h2o_g_on_total", "wf_co2_g_on_total")

    def secondary_dofs(self, I, out=None, stream: int = 0):
        """secondary_dofs::execute (secondary_dofs.hpp:56-101): the mixture at every
        node, an (8, n_nodes) array (or the given host/device buffer) in the order of
        SECONDARY_FIELDS."""
        if out is None:
            out = np.zeros((8, self.mesh.n_nodes))
        self._check(self._L.gales_asm_secondary_dofs(self._h, _addr(I), _addr(out), stream or None))
        return out

    def set_magma(self, magma_material=None):
        """Attach magma mixtures (magma.MagmaMaterial, props.txt's mix_of_mix of
        magma_mix) as the material of every later call, or detach them (None).  The
        material must have this handle's number of components and outlive the
        attachment (the handle keeps a reference)."""
        h = None if magma_material is None else magma_material._h
        self._check(self._L.gales_asm_set_magma(self._h, h))
        self._magma = magma_material

    def magma_fractions(self, I, out=None, stream: int = 0):
        """The gas fractions of secondary_dofs::execute with pp_vf_g
        (secondary_dofs.hpp:56-131) at every node: a (2 nb_comp + 6, n_nodes) array (or
        the given buffer), rows MAGMA_FRACTION_FIELDS(nb_comp)."""
        if out is None:
            out = np.zeros((2 * self.nb_comp + 6, self.mesh.n_nodes))
        self._check(self._L.gales_asm_magma_fractions(self._h, _addr(I), _addr(out), stream or None))
        return out

    def element_blocks(self, I, P, dt: float, elements, which: int = 0, form: int = FORM_FP64,
                       want_matrix: bool = True):
        """Batched fluid::execute_i (which=0) / execute_b (which=1): local (m, r) per element."""
        el = np.ascontiguousarray(elements, dtype=np.int32)
        N = self.mesh.nen * self.nd
        m = np.zeros((len(el), N, N)) if want_matrix else None
        r = np.zeros((len(el), N))
        self._check(self._L.gales_asm_element_blocks(self._h, _addr(I), _addr(P), float(dt), form, which,
                                                     el.ctypes.data_as(C.POINTER(C.c_int32)), len(el),
                                                     _addr(m) if want_matrix else None, _addr(r), None))
        return m, r

    def device_ms(self) -> float:
        return self._L.gales_asm_last_ms(self._h)

    def phase_ms(self, phase: int) -> float:
        """0 = clear, 1 = interior kernel(s), 2 = boundary pass, 3 / 4 = point / matrix stage
        of the interior pass's first chunk (CUDA events, last call)."""
        return self._L.gales_asm_last_phase_ms(self._h, phase)

    def launch_count(self) -> int:
        return self._L.gales_asm_launch_count(self._h)


    def linear_solver(self, params: Optional["SolverParams"] = None) -> "LinearSolver":
        """belos_linear_solver for this handle's systems, on the GPU."""
        return LinearSolver(self, params)


PRECOND_NONE, PRECOND_ILU, PRECOND_ILU_FP32 = 0, 1, 2


@dataclass
class SolverParams:
    """The ls_* keys of setup.txt read by belos_linear_solver
    (belos_linear_solver_factory.hpp:77-86); defaults are the shipped P0 case's."""
    rel_res_tol: float = 1e-9
    maxsubspace: int = 200
    maxrestarts: int = 5
    maxiters: int = -1
    fill: int = 1
    precond: int = PRECOND_ILU

    def desc(self) -> abi.SolverParams:
        return abi.SolverParams(float(self.rel_res_tol), int(self.maxsubspace), int(self.maxrestarts),
                                int(self.maxiters), int(self.fill), int(self.precond))


class LinearSolver:
    """belos_linear_solver (belos_linear_solver_factory.hpp:69-274) on the GPU: flexible
    GMRES with a right ILU(fill) preconditioner on the assembled CSR values, which may
    stay in device memory.  solve() returns the execute() seconds and sets
    num_it / ARE / RRE like the reference's accessors."""

    def __init__(self, fa: "FluidAssembly", params: Optional[SolverParams] = None):
        self.params = params or SolverParams()
        self._L = fa._L
        self._fa = fa  # keeps the assembly handle alive
        h = C.c_void_p()
        rc = self._L.gales_solver_create(fa._h, C.byref(self.params.desc()), C.byref(h))
        if rc != 0:
            raise GalesError(rc, "gales_solver_create failed")
        self._h = h
        self.nd, self.n_rows = fa.nd, fa.n_rows
        self.result = abi.SolverResult()

    def close(self):
        if getattr(self, "_h", None):
            self._L.gales_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            raise GalesError(rc, self._L.gales_solver_last_error(self._h).decode())

    def solve(self, vals, rhs, x, stream: int = 0) -> float:
        """execute(): A x = rhs for the CSR values vals (host or device buffers)."""
        self._check(self._L.gales_solver_solve(self._h, _addr(vals), _addr(rhs), _addr(x), C.byref(self.result),
                                               stream or None))
        return self.result.seconds

    @property
    def num_it(self) -> int:
        return int(self.result.iterations)

    @property
    def ARE(self) -> float:
        return float(self.result.abs_res)

    @property
    def RRE(self) -> float:
        return float(self.result.rel_res)

    @property
    def converged(self) -> bool:
        return bool(self.result.converged)

    def factorize(self, vals, stream: int = 0):
        self._check(self._L.gales_solver_factorize(self._h, _addr(vals), stream or None))

    def apply(self, v, z, stream: int = 0):
        """z = M^-1 v with the current factor (device buffers)."""
        self._check(self._L.gales_solver_apply(self._h, _addr(v), _addr(z), stream or None))

    def factor(self):
        """The factor as node blocks: (row_ptr, col, blocks[nnz_blocks, nd, nd])."""
        nb, nnz = C.c_int64(), C.c_int64()
        rp, cl = C.POINTER(C.c_int64)(), C.POINTER(C.c_int32)()
        self._check(self._L.gales_solver_factor(self._h, C.byref(nb), C.byref(nnz), C.byref(rp), C.byref(cl), None))
        vals = np.zeros((nnz.value, self.nd, self.nd))
        self._check(self._L.gales_solver_factor(self._h, None, None, None, None, _addr(vals)))
        return (np.ctypeslib.as_array(rp, shape=(nb.value + 1,)).copy(),
                np.ctypeslib.as_array(cl, shape=(nnz.value,)).copy(), vals)

    def levels(self):
        f, b = C.c_int32(), C.c_int32()
        self._check(self._L.gales_solver_levels(self._h, C.byref(f), C.byref(b)))
        return f.value, b.value

    def correct(self, I, dx, trim=(-1, -1), lo: float = 0.0, hi: float = 1.0, stream: int = 0):
        """fluid_updater::corrector + model::dof_trimmer on the device: I += dx, then the
        dofs with index in [trim[0], trim[1]) clamped into [lo, hi]."""
        self._check(self._L.gales_solver_correct(self._h, _addr(I), _addr(dx), int(trim[0]), int(trim[1]),
                                                 float(lo), float(hi), stream or None))

    def launch_count(self) -> int:
        return self._L.gales_solver_launches(self._h)


def iluk_pattern(row_ptr, col, fill: int = 1):
    """Host-side node-level ILU(fill) pattern (no GPU): (f_row_ptr, f_col, level_fwd,
    level_bwd, (n_levels_fwd, n_levels_bwd))."""
    L = abi.lib()
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    n = len(row_ptr) - 1
    nnz = C.c_int64()
    i64p, i32p = C.POINTER(C.c_int64), C.POINTER(C.c_int32)
    rc = L.gales_iluk_pattern(n, row_ptr.ctypes.data_as(i64p), col.ctypes.data_as(i32p), int(fill), C.byref(nnz),
                              None, None, None, None, None)
    if rc:
        raise GalesError(rc, "gales_iluk_pattern failed")
    f_rp = np.zeros(n + 1, dtype=np.int64)
    f_col = np.zeros(nnz.value, dtype=np.int32)
    lf = np.zeros(n, dtype=np.int32)
    lb = np.zeros(n, dtype=np.int32)
    nl = np.zeros(2, dtype=np.int32)
    rc = L.gales_iluk_pattern(n, row_ptr.ctypes.data_as(i64p), col.ctypes.data_as(i32p), int(fill), C.byref(nnz),
                              f_rp.ctypes.data_as(i64p), f_col.ctypes.data_as(i32p), lf.ctypes.data_as(i32p),
                              lb.ctypes.data_as(i32p), nl.ctypes.data_as(i32p))
    if rc:
        raise GalesError(rc, "gales_iluk_pattern failed")
    return f_rp, f_col, lf, lb, (int(nl[0]), int(nl[1]))


class ResidualCheck:
    """residual_check (residual_check.hpp:42-80): ||b||_2 against iteration 0."""

    def __init__(self):
        self.res0 = 0.0

    def execute(self, b, it_count: int, norm: Optional[float] = None):
        """b is the rhs (host array) or None with norm = ||b||_2 computed elsewhere
        (FluidAssembly.norm2 on the device)."""
        if norm is not None:
            n = float(norm)
        else:
            n = float(np.linalg.norm(np.asarray(b if isinstance(b, np.ndarray) else b.detach().cpu().numpy())))
        if it_count == 0:
            self.res0 = n
            return False, n
        rel = n / self.res0 if self.res0 else math.inf
        return n <= max(1.e-8 * self.res0, 1.e-5), rel


from .meshio import read_mesh, write_mesh  # noqa: E402  (uses Mesh and GalesError above)

def pressure_profile(material: "Material", p0: float, h: float, T, T1, Y=None, Y1=None) -> np.ndarray:
    """Hydrostatic pressure column (pressure_profile.hpp:480-496, RK4 from p0 at the top
    with step h): T, Y at the n+1 column points and T1, Y1 at the points h/2 below them
    (Y, Y1: (n+1, nc-1) independent mass fractions).  Returns p at the column points."""
    T = np.ascontiguousarray(T, dtype=np.float64)
    T1 = np.ascontiguousarray(T1, dtype=np.float64)
    n = len(T) - 1
    nc = material.nb_comp
    Y = np.ascontiguousarray(np.zeros((n + 1, nc - 1)) if Y is None else Y, dtype=np.float64)
    Y1 = np.ascontiguousarray(np.zeros((n + 1, nc - 1)) if Y1 is None else Y1, dtype=np.float64)
    if len(T1) != n + 1 or Y.shape != (n + 1, nc - 1) or Y1.shape != (n + 1, nc - 1):
        raise ValueError("T, T1: n+1 values; Y, Y1: (n+1, nc-1)")
    p = np.zeros(n + 1)
    dp = C.POINTER(C.c_double)
    rc = abi.lib().gales_pressure_profile(C.byref(material.desc), float(p0), float(h), n, T.ctypes.data_as(dp),
                                          T1.ctypes.data_as(dp), Y.ctypes.data_as(dp), Y1.ctypes.data_as(dp),
                                          p.ctypes.data_as(dp))
    if rc:
        raise GalesError(rc, "gales_pressure_profile")
    return p


def pressure_interpolate(y_col, p_col, y) -> np.ndarray:
    """p_interpolation (pressure_profile.hpp:26-41) of a column at the heights y."""
    y_col = np.ascontiguousarray(y_col, dtype=np.float64)
    p_col = np.ascontiguousarray(p_col, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    out = np.zeros(len(y))
    dp = C.POINTER(C.c_double)
    rc = abi.lib().gales_pressure_interpolate(y_col.ctypes.data_as(dp), p_col.ctypes.data_as(dp), len(y_col),
                                              y.ctypes.data_as(dp), len(y), out.ctypes.data_as(dp))
    if rc:
        raise GalesError(rc, "gales_pressure_interpolate: a height outside the column")
    return out


def dt_update(dt_elem_min: float, dt: float, dt_min: float, dt_max: float) -> float:
    """set_dt (adaptive_time_step.hpp:380-393) through the library (host arithmetic)."""
    return abi.lib().gales_dt_update(float(dt_elem_min), float(dt), float(dt_min), float(dt_max))


__all__ = [
    "read_mesh", "write_mesh", "dt_update", "pressure_profile", "pressure_interpolate",
    "abi", "GalesError", "custom_chemical", "ideal_gas", "ideal_gas_named", "ideal_gas_params", "Material",
    "Setup", "p0_policy", "Mesh", "nb_dofs", "LinearSystem", "FluidAssembly", "ResidualCheck",
    "FORM_FP64", "FORM_MIXED", "TAU_NONE", "TAU_2001", "TAU_2019", "TAU_2007", "TAU_2014",
    "VJP_EXACT", "VJP_FROZEN", "SCATTER_ATOMIC", "SCATTER_COLOURED",
]
