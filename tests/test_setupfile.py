"""setup.txt as read_setup reads it (read_setup.hpp:34-260) and its mapping onto the
library's Setup and SolverParams."""
import importlib

import pytest

gm = importlib.import_module("gales-multi-fluid_gb300")
sf = importlib.import_module("gales-multi-fluid_gb300.setupfile")

# a setup.txt in the shipped case's layout (keys of sim/fluid_mc/P0/setup.txt)
TEXT = """fluid_mesh_file   mesh_8core.txt

delta_t           0.02
final_time        2.0
restart           F
n_max_it          4
t_dependent_dirichlet_bc  F

ls_solver         Flexible GMRES
ls_precond        ILU
ls_rel_res_tol    1.e-8
ls_maxsubspace    150
ls_maxrestarts    3
ls_maxiters      -1
ls_fill           2

adaptive_time_step    T
dt_min                0.001
dt_max                0.25
CFL                   0.4

steady_state                F
tau_non_diag_comp_2001      F
tau_non_diag_comp_2019      T
tau_diag_incomp_2007        F
dc_2006                     T
dc_sharp                    1.5
dc_scale_fact               0.5
"""


def test_parse_and_map():
    s = sf.parse_setup(TEXT)
    assert s.fluid_mesh_file == "input/mesh_8core.txt" and s.delta_t == 0.02 and s.final_time == 2.0
    assert s.n_max_it == 4 and not s.restart and s.adaptive_time_step and s.CFL == 0.4 and s.dt_max == 0.25
    # a flag is only ever set to true (read_setup.hpp:104-105); its default is true
    assert s.t_dependent_dirichlet_bc
    # "Flexible GMRES" splits to "Flexible", which falls back to Flexible GMRES
    assert s.ls_solver == "Flexible GMRES" and s.ls_precond == "ILU"
    p = s.solver_params()
    assert (p.rel_res_tol, p.maxsubspace, p.maxrestarts, p.maxiters, p.fill, p.precond) == \
        (1e-8, 150, 3, -1, 2, gm.PRECOND_ILU)
    st = s.setup(3)
    d = st.desc
    assert d.tau == gm.TAU_2019 and d.dc_2006 == 1 and d.dc_sharp == 1.5 and d.dc_scale_fact == 0.5
    assert d.steady_state == 0


def test_defaults_and_tau_precedence():
    s = sf.parse_setup("")
    assert (s.delta_t, s.n_max_it, s.ls_maxiters, s.ls_rel_res_tol, s.dc_sharp, s.CFL) == (0.002, 3, 3000, 1e-9, 1.0,
                                                                                             1.0)
    assert s.tau == gm.TAU_NONE and not s.dc_2006 and s.t_dependent_dirichlet_bc
    s = sf.parse_setup("tau_diag_2014 true\ntau_diag_incomp_2007 TRUE\n")
    assert s.tau == gm.TAU_2007
    s = sf.parse_setup("tau_non_diag_comp_2019 t\ntau_non_diag_comp_2001 True\n")
    assert s.tau == gm.TAU_2001


def test_unsupported_solver_choices_raise():
    with pytest.raises(ValueError):
        sf.parse_setup("ls_precond ML\n").solver_params()
    with pytest.raises(ValueError):
        sf.parse_setup("ls_solver GMRES\n").solver_params()


# the reference project's checkout, when one is present (GALES_REFERENCE_DIR)
REF_SETUP = __import__("pathlib").Path(__import__("os").environ.get("GALES_REFERENCE_DIR", "-"),
                                       "sim/fluid_mc/P0/setup.txt")


@pytest.mark.skipif(not REF_SETUP.exists(), reason="the reference's case files are not present")
def test_reads_the_reference_case_setup():
    """The shipped case's own setup.txt maps onto the library defaults: Flexible GMRES
    with ILU(1), 1e-9, 200 vectors, 5 restarts, maxiters -1; tau 2019, dc_2006, sharpness 2."""
    s = sf.read_setup(REF_SETUP)
    p = s.solver_params()
    d = gm.SolverParams()
    assert (p.rel_res_tol, p.maxsubspace, p.maxrestarts, p.maxiters, p.fill, p.precond) == \
        (d.rel_res_tol, d.maxsubspace, d.maxrestarts, d.maxiters, d.fill, d.precond)
    assert s.tau == gm.TAU_2019 and s.dc_2006 and s.dc_sharp == 2.0 and s.dc_scale_fact == 1.0
    assert not s.steady_state and s.n_max_it == 3 and s.delta_t == 0.01
    assert s.t_dependent_dirichlet_bc     # the file says F; the reader keeps the true default
