"""Hand-sized regression vectors (tests/golden/hand_meshes.npz, written by
tests/golden/make_golden.py).  They are SELF-GENERATED by the oracle, not reference
output (the reference ships none): they pin the oracle against regressions and give
the CUDA path fixed targets that do not need the oracle at run time."""
import importlib
from pathlib import Path

import numpy as np
import pytest

from cases import gm, syn, rel

GOLD = Path(__file__).with_name("golden") / "hand_meshes.npz"


def _load():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", Path(__file__).with_name("golden") / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod, np.load(GOLD)


@pytest.mark.parametrize("name", ["tri2", "tet1", "hex1"])
def test_oracle_reproduces_golden(name):
    mod, g = _load()
    mesh, nc, S = mod.cases()[name]
    d = mod.compute(name, mesh, nc, S)
    for k, v in d.items():
        assert rel(v, g[k]) <= 1e-14, k


@pytest.mark.parametrize("name", ["tri2", "tet1", "hex1"])
def test_golden_dirichlet_rows(name):
    """Rows of velocity dofs on wall nodes (flag 5): zero rhs, avg on the diagonal only."""
    mod, g = _load()
    mesh, nc, S = mod.cases()[name]
    nd = gm.nb_dofs(mesh.dim, nc)
    rp, cl, vals, rhs = g[f"{name}_row_ptr"], g[f"{name}_col"], g[f"{name}_vals"], g[f"{name}_rhs"]
    for node in np.nonzero(mesh.node_flag == 5)[0]:
        for k in range(1, 1 + mesh.dim):
            row = node * nd + k
            assert rhs[row] == 0.0
            seg = slice(rp[row], rp[row + 1])
            off = vals[seg][cl[seg] != row]
            assert np.all(off == 0.0) and vals[seg][cl[seg] == row][0] != 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tri2", "tet1", "hex1"])
def test_cuda_fp64_matches_golden(name, cuda_lib):
    mod, g = _load()
    mesh, nc, S = mod.cases()[name]
    mat = syn.material_for(nc, 0)
    setup = syn.setup_for(mesh.dim, nc)
    I, P = g[f"{name}_I"], g[f"{name}_P"]
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp = fa.linear_system()
    assert np.array_equal(lp.row_ptr, g[f"{name}_row_ptr"]) and np.array_equal(lp.col, g[f"{name}_col"])
    fa.execute(I, P, 1e-3, lp, form=gm.FORM_FP64)
    assert rel(lp.vals, g[f"{name}_vals"]) <= 1e-12
    assert rel(lp.rhs, g[f"{name}_rhs"]) <= 1e-12
    for which, tag in ((0, "interior"), (1, "boundary")):
        m, r = fa.element_blocks(I, P, 1e-3, [0], which=which, form=gm.FORM_FP64)
        assert rel(m[0], g[f"{name}_m_{tag}"]) <= 1e-12
        assert rel(r[0], g[f"{name}_r_{tag}"]) <= 1e-12
