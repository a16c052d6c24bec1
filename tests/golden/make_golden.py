"""Write tests/golden/hand_meshes.npz: regression vectors of hand-sized cases.

SELF-GENERATED by the oracle (the CPU restatement in oracle/), not reference
output: the reference ships no golden vectors and cannot be built here.  The cases
are written out in full below (coordinates, connectivity, states), small enough to
check by hand against the formulas the oracle cites:
  tri2  - the unit square split into 2 triangles, 2 components (melt + gas), 5 dofs
  tet1  - one tetrahedron, 3 components, 7 dofs
  hex1  - one (slightly skewed) hexahedron, 4 components, 8 dofs
For each: the element blocks of execute_i and execute_b (m, r = -r_) and the
assembled CSR values and rhs with the P0 wall policy (velocity Dirichlet on flag 5).

  python tests/golden/make_golden.py
"""
import importlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT, ROOT / "oracle"):
    sys.path.insert(0, str(p))
import oracle  # noqa: E402

gm = importlib.import_module("gales-multi-fluid_gb300")
syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")


def cases():
    out = {}
    # tri2: nodes 0(0,0) 1(1,0) 2(1,1) 3(0,1); walls at y = 0 (flag 5), open elsewhere
    coords = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    conn = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.int32)
    flag = np.array([5, 5, 2, 2], dtype=np.int32)
    bd = np.array([[0, 2, 5], [0, 0, 2], [1, 0, 2], [1, 1, 2]], dtype=np.int32)
    mesh = gm.Mesh(coords, conn, flag, np.array([1, 1], dtype=np.uint8), bd, name="tri2")
    S = np.array([[1.0e8, 0.0, 0.0, 1273.0, 0.6],
                  [1.0e8, 0.0, 0.0, 1280.0, 0.5],
                  [9.9e7, 0.05, -0.02, 1300.0, 0.4],
                  [9.9e7, -0.03, 0.01, 1290.0, 0.55]])
    out["tri2"] = (mesh, 2, S)
    # tet1
    coords = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [0.0, 0.5, 0.0], [0.0, 0.0, 0.5]])
    conn = np.array([[0, 1, 2, 3]], dtype=np.int32)
    flag = np.array([5, 0, 0, 2], dtype=np.int32)
    bd = np.array([[0, 3, 5], [0, 0, 2]], dtype=np.int32)
    mesh = gm.Mesh(coords, conn, flag, np.array([1], dtype=np.uint8), bd, name="tet1")
    S = np.array([[7.0e7, 0.0, 0.0, 0.0, 1300.0, 0.8, 0.15],
                  [7.01e7, 0.1, 0.0, -0.05, 1310.0, 0.7, 0.2],
                  [6.99e7, -0.04, 0.08, 0.0, 1290.0, 0.75, 0.1],
                  [6.98e7, 0.02, 0.03, 0.06, 1305.0, 0.85, 0.05]])
    out["tet1"] = (mesh, 3, S)
    # hex1: unit cube with one node pulled
    coords = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1.1, 1.05, 1.0], [0, 1, 1]],
                      dtype=np.float64)
    conn = np.array([[0, 1, 2, 3, 4, 5, 6, 7]], dtype=np.int32)
    flag = np.array([5, 5, 5, 5, 2, 2, 2, 2], dtype=np.int32)
    bd = np.array([[0, 0, 2], [0, 1, 5]], dtype=np.int32)
    mesh = gm.Mesh(coords, conn, flag, np.array([1], dtype=np.uint8), bd, name="hex1")
    rows = []
    for a in range(8):
        rows.append([7.0e7 - 1e4 * a, 0.01 * (a % 3), -0.02 * (a % 2), 0.015 * (a % 4) - 0.02, 1290.0 + 3 * a,
                     0.7 - 0.01 * a, 0.1 + 0.005 * a, 0.1])
    out["hex1"] = (mesh, 4, np.array(rows))
    return out


def compute(name, mesh, nc, S):
    mat = syn.material_for(nc, 0)
    setup = syn.setup_for(mesh.dim, nc)
    I = S.ravel().copy()
    P = (S * (1.0 + 1e-4 * np.cos(np.arange(S.size)).reshape(S.shape))).ravel()
    dt = 1e-3
    nd = gm.nb_dofs(mesh.dim, nc)
    m_i, r_i, s_i = oracle.element(mesh, mat, setup, I, P, dt, 0, which=0)
    m_b, r_b, s_b = oracle.element(mesh, mat, setup, I, P, dt, 0, which=1)
    nrp, ncol, rp, cl = oracle.pattern(mesh, nd)
    vals, rhs, s, fb = oracle.assemble(mesh, mat, setup, I, P, dt, rp, cl)
    assert s_i == 0 and s_b == 0 and s == 0
    return {f"{name}_I": I, f"{name}_P": P, f"{name}_m_interior": m_i, f"{name}_r_interior": r_i,
            f"{name}_m_boundary": m_b, f"{name}_r_boundary": r_b, f"{name}_row_ptr": rp, f"{name}_col": cl,
            f"{name}_vals": vals, f"{name}_rhs": rhs}


def main():
    data = {}
    for name, (mesh, nc, S) in cases().items():
        data.update(compute(name, mesh, nc, S))
    np.savez_compressed(Path(__file__).with_name("hand_meshes.npz"), **data)


if __name__ == "__main__":
    main()
