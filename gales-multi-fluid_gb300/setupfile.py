"""setup.txt, as read_setup reads it (src/fem/base/read_setup.hpp:34-260), mapped onto
the library's Setup (the integral's flags), SolverParams (belos_linear_solver's ls_*
keys) and the time-loop settings of main.cpp.

Format: one "key value" per line, split on spaces; only the first value token counts
(read_setup.hpp:45-52, so "ls_solver Flexible GMRES" reads "Flexible" and falls back
to Flexible GMRES).  Booleans are T/True/TRUE/t/true.  Unlisted keys keep the
defaults of read_setup.hpp:114-191.
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path
from typing import Dict, Optional

_TRUE = ("T", "True", "TRUE", "t", "true")
# ls_solver names (read_setup.hpp:113-141); anything else is Flexible GMRES
_SOLVERS = {"GMRES": "GMRES", "Flexible_GMRES": "Flexible GMRES", "Block": "Block CG",
            "PseudoBlockCG": "PseudoBlockCG", "Recycling_GMRES": "Recycling GMRES", "Recycling_CG": "Recycling CG",
            "MINRES": "MINRES", "LSQR": "LSQR", "TFQMR": "TFQMR", "Pseudoblock": "Pseudoblock",
            "GmresPoly": "GmresPoly", "CGPoly": "CGPoly", "Klu": "Klu", "Lapack": "Lapack", "Umfpack": "Umfpack",
            "Pardiso": "Pardiso", "Taucs": "Taucs", "Superlu": "Superlu", "Superludist": "Superludist",
            "Mumps": "Mumps", "Dscpack": "Dscpack"}


@dataclass
class SetupFile:
    """The keys of setup.txt on the assembly / solve / time-step path, with
    read_setup's defaults."""
    fluid_mesh_file: str = ""
    delta_t: float = 0.002
    final_time: float = 100000.0
    restart: bool = False
    restart_time: float = 0.0
    n_max_it: int = 3
    print_freq: int = 10
    t_dependent_dirichlet_bc: bool = True
    ls_solver: str = "Flexible GMRES"
    ls_precond: str = "ILU"
    ls_rel_res_tol: float = 1.e-9
    ls_maxsubspace: int = 200
    ls_maxrestarts: int = 5
    ls_maxiters: int = 3000
    ls_fill: int = 1
    adaptive_time_step: bool = False
    dt_min: float = 0.002
    dt_max: float = 1.0
    N: int = 10
    CFL: float = 1.0
    steady_state: bool = False
    tau_diag_incomp_2007: bool = False
    tau_diag_2014: bool = False
    tau_non_diag_comp_2001: bool = False
    tau_non_diag_comp_2019: bool = False
    dc_2006: bool = False
    dc_sharp: float = 1.0
    dc_scale_fact: float = 1.0

    @property
    def tau(self) -> int:
        """The τ variant fluid::tau_matrix uses: 2001, else 2019, else 2007, else 2014
        (fluid_2d.hpp:895-994), none when no flag is set."""
        from . import abi
        if self.tau_non_diag_comp_2001:
            return abi.TAU_2001
        if self.tau_non_diag_comp_2019:
            return abi.TAU_2019
        if self.tau_diag_incomp_2007:
            return abi.TAU_2007
        if self.tau_diag_2014:
            return abi.TAU_2014
        return abi.TAU_NONE

    def setup(self, dim: int, **kw):
        """gm.Setup with this file's integral flags (the ic_bc policy is added by the caller)."""
        from . import Setup
        return Setup(dim, tau=self.tau, dc_2006=self.dc_2006, dc_sharp=self.dc_sharp,
                     dc_scale_fact=self.dc_scale_fact, steady_state=self.steady_state, **kw)

    def solver_params(self):
        """gm.SolverParams of belos_linear_solver's constructor (belos_linear_solver_factory.hpp:
        77-86).  The GPU solver provides Flexible GMRES with ILU; other choices raise."""
        from . import PRECOND_ILU, SolverParams
        if self.ls_solver != "Flexible GMRES":
            raise ValueError(f"ls_solver {self.ls_solver!r}: only Flexible GMRES is provided on the GPU")
        if self.ls_precond != "ILU":
            raise ValueError(f"ls_precond {self.ls_precond!r}: only ILU is provided on the GPU")
        return SolverParams(rel_res_tol=self.ls_rel_res_tol, maxsubspace=self.ls_maxsubspace,
                            maxrestarts=self.ls_maxrestarts, maxiters=self.ls_maxiters, fill=self.ls_fill,
                            precond=PRECOND_ILU)


def parse_setup(text: str) -> SetupFile:
    data: Dict[str, str] = {}
    for raw in text.splitlines():
        s = raw.strip()
        if not s:
            continue
        tok = [t for t in s.split(" ") if t]
        data[tok[0]] = tok[1] if len(tok) > 1 else ""
    out = SetupFile()
    for key, val in data.items():
        if key == "fluid_mesh_file":
            out.fluid_mesh_file = "input/" + val
        elif key == "final_time":
            out.final_time = float(val)
        elif key == "ls_solver":
            out.ls_solver = _SOLVERS.get(val, "Flexible GMRES")
        elif key in ("ls_precond",):
            out.ls_precond = val
        elif hasattr(out, key):
            cur = getattr(out, key)
            if isinstance(cur, bool):
                # read_setup.hpp sets a flag only to true (e.g. 104-105): a false
                # word leaves the default, so t_dependent_dirichlet_bc F stays true
                if val in _TRUE:
                    setattr(out, key, True)
            elif isinstance(cur, int):
                setattr(out, key, int(val))
            elif isinstance(cur, float):
                setattr(out, key, float(val))
    return out


def read_setup(path="setup.txt") -> SetupFile:
    return parse_setup(Path(path).read_text())
