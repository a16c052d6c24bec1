"""Seeded synthetic meshes, materials and nodal states for the fluid_mc workloads.

The reference's case meshes and states are not available, so the workloads are
built here with the shapes, sizes and value distributions of the benchmark
configurations:

  channel_tri      2 m x 1 m channel, 64 x 32 quads split into 4096 CCW triangles
                   (2145 nodes), 2 components, 5 dofs
  box_tet_delaunay unit box, Delaunay tetrahedra of a jittered lattice
                   (n = 56 gives about 1.0M tets), 3 components, 7 dofs
  box_hex          structured hexahedra with seeded node jitter, 4 components, 8 dofs
  channel_quad     2D quadrilaterals (tests)

State: hydrostatic pressure 1e5..1e8 Pa with 1 % noise, velocity from 8 random
Fourier modes (0.1 m/s amplitude), T = 1273 +- 50 K, smooth mass fractions, and
P = I + a small seeded perturbation.  Everything is drawn from
numpy.random.default_rng(seed).
"""
from __future__ import annotations

import importlib

import numpy as np

from . import Material, Mesh, Setup, custom_chemical, ideal_gas, ideal_gas_named, nb_dofs, p0_policy

# local side tables of element.hpp:100-104, 145-149, 401-408, 455-460
SIDES = {
    (2, 3): [[1, 2], [2, 0], [0, 1]],
    (2, 4): [[0, 1], [1, 2], [2, 3], [3, 0]],
    (3, 4): [[1, 2, 3], [0, 3, 2], [0, 1, 3], [0, 2, 1]],
    (3, 8): [[4, 5, 6, 7], [0, 3, 2, 1], [0, 4, 7, 3], [1, 2, 6, 5], [2, 3, 7, 6], [1, 5, 4, 0]],
}

WALL = 5     # no-slip wall flag of the shipped policy (fluid_ic_bc.hpp:92,100,165)
OPEN = 2     # boundary without velocity Dirichlet


def boundary_sides(conn: np.ndarray, dim: int, coords: np.ndarray, face_flag) -> np.ndarray:
    """(element, local side, flag) of every side that belongs to one element only.

    face_flag(centroids) -> int flags (> 0) for the boundary faces.
    """
    nen = conn.shape[1]
    table = np.asarray(SIDES[(dim, nen)])
    ns, nsn = table.shape
    faces = conn[:, table]                         # (n_el, ns, nsn)
    key = np.sort(faces.reshape(-1, nsn), axis=1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    single = np.nonzero(cnt[inv.ravel()] == 1)[0]
    el = (single // ns).astype(np.int32)
    loc = (single % ns).astype(np.int32)
    cen = coords[faces.reshape(-1, nsn)[single]].mean(axis=1)
    flag = np.asarray(face_flag(cen), dtype=np.int32)
    keep = flag > 0
    return np.stack([el[keep], loc[keep], flag[keep]], axis=1)


def _finish(coords, conn, node_flag, face_flag, name) -> Mesh:
    dim = coords.shape[1]
    bd = boundary_sides(conn, dim, coords, face_flag)
    el_bd = np.zeros(conn.shape[0], dtype=np.uint8)
    el_bd[bd[:, 0]] = 1
    return Mesh(coords, conn, node_flag, el_bd, bd, name=name)


def _box_flags(x: np.ndarray, lo: np.ndarray, hi: np.ndarray, open_top: bool) -> np.ndarray:
    """Node flags: WALL on the box faces, OPEN on the top face (last axis, max) if open_top."""
    tol = 1e-9 * float(np.max(hi - lo))
    on = (np.abs(x - lo) < tol) | (np.abs(x - hi) < tol)
    flag = np.where(on.any(axis=1), WALL, 0).astype(np.int32)
    if open_top:
        top = np.abs(x[:, -1] - hi[-1]) < tol
        others = (on[:, :-1]).any(axis=1) | (np.abs(x[:, -1] - lo[-1]) < tol)
        flag[top & ~others] = OPEN
    return flag


def _face_flag_box(lo, hi, open_top):
    tol = 1e-9 * float(np.max(np.asarray(hi) - np.asarray(lo)))

    def f(c):
        flag = np.full(len(c), WALL, dtype=np.int32)
        if open_top:
            flag[np.abs(c[:, -1] - hi[-1]) < tol] = OPEN
        return flag
    return f


def channel_tri(nx: int = 64, ny: int = 32, Lx: float = 2.0, Ly: float = 1.0) -> Mesh:
    """Structured channel, each quad split into two counter-clockwise triangles.
    Walls (flag 5) at y = 0 and y = Ly; inflow/outflow ends (flag 2) at x = 0, Lx."""
    xs, ys = np.linspace(0.0, Lx, nx + 1), np.linspace(0.0, Ly, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    idx = np.arange((nx + 1) * (ny + 1)).reshape(ny + 1, nx + 1)
    n00, n10 = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel()
    n11, n01 = idx[1:, 1:].ravel(), idx[1:, :-1].ravel()
    t1 = np.stack([n00, n10, n11], axis=1)
    t2 = np.stack([n00, n11, n01], axis=1)
    conn = np.stack([t1, t2], axis=1).reshape(-1, 3).astype(np.int32)
    tol = 1e-12
    wall = (np.abs(coords[:, 1]) < tol) | (np.abs(coords[:, 1] - Ly) < tol)
    end = (np.abs(coords[:, 0]) < tol) | (np.abs(coords[:, 0] - Lx) < tol)
    node_flag = np.where(wall, WALL, np.where(end, OPEN, 0)).astype(np.int32)

    def ff(c):
        return np.where((np.abs(c[:, 1]) < tol) | (np.abs(c[:, 1] - Ly) < tol), WALL, OPEN)
    return _finish(coords, conn, node_flag, ff, f"channel_tri_{nx}x{ny}")


def channel_quad(nx: int = 16, ny: int = 8, Lx: float = 2.0, Ly: float = 1.0, jitter: float = 0.0,
                 seed: int = 0) -> Mesh:
    xs, ys = np.linspace(0.0, Lx, nx + 1), np.linspace(0.0, Ly, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    if jitter:
        rng = np.random.default_rng(seed)
        inner = (X.ravel() > 0) & (X.ravel() < Lx) & (Y.ravel() > 0) & (Y.ravel() < Ly)
        h = min(Lx / nx, Ly / ny)
        coords[inner] += rng.uniform(-jitter * h, jitter * h, size=(inner.sum(), 2))
    idx = np.arange((nx + 1) * (ny + 1)).reshape(ny + 1, nx + 1)
    conn = np.stack([idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel(), idx[1:, 1:].ravel(), idx[1:, :-1].ravel()],
                    axis=1).astype(np.int32)
    tol = 1e-12
    wall = (np.abs(coords[:, 1]) < tol) | (np.abs(coords[:, 1] - Ly) < tol)
    end = (np.abs(coords[:, 0]) < tol) | (np.abs(coords[:, 0] - Lx) < tol)
    node_flag = np.where(wall, WALL, np.where(end, OPEN, 0)).astype(np.int32)

    def ff(c):
        return np.where((np.abs(c[:, 1]) < tol) | (np.abs(c[:, 1] - Ly) < tol), WALL, OPEN)
    return _finish(coords, conn, node_flag, ff, f"channel_quad_{nx}x{ny}")


def _jittered_lattice(n, jitter, rng, dim):
    g = np.linspace(0.0, 1.0, n)
    grids = np.meshgrid(*([g] * dim), indexing="ij")
    pts = np.stack([x.ravel() for x in grids], axis=1)
    h = 1.0 / (n - 1)
    d = rng.uniform(-jitter * h, jitter * h, size=pts.shape)
    on_face = (pts < 1e-12) | (pts > 1 - 1e-12)
    d[on_face] = 0.0          # boundary points move only within their faces
    return pts + d


def box_tet_delaunay(n: int = 56, jitter: float = 0.3, seed: int = 1, min_quality: float = 1e-3) -> Mesh:
    """Delaunay tetrahedra of an n^3 jittered lattice in the unit box, oriented so
    that J > 0 (quad.hpp:549).  Near-flat tets (volume below min_quality * h^3 / 6)
    are dropped.  Walls (flag 5) everywhere except the open top z = 1 (flag 2)."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    pts = _jittered_lattice(n, jitter, rng, 3)
    tri = Delaunay(pts, qhull_options="Qbb Qc Qz Q12")
    conn = tri.simplices.astype(np.int64)
    x = pts[conn]
    vol = np.einsum("ij,ij->i", np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]), x[:, 3] - x[:, 0])
    flip = vol < 0
    conn[flip, 1], conn[flip, 2] = conn[flip, 2].copy(), conn[flip, 1].copy()
    h = 1.0 / (n - 1)
    keep = np.abs(vol) > min_quality * h ** 3
    conn = conn[keep]
    used = np.zeros(len(pts), dtype=bool)
    used[conn.ravel()] = True
    remap = -np.ones(len(pts), dtype=np.int64)
    remap[used] = np.arange(used.sum())
    pts = pts[used]
    conn = remap[conn].astype(np.int32)
    lo, hi = np.zeros(3), np.ones(3)
    node_flag = _box_flags(pts, lo, hi, open_top=True)
    return _finish(pts, conn, node_flag, _face_flag_box(lo, hi, True), f"box_tet_delaunay_n{n}")


def box_hex(nx: int, ny: int, nz: int, jitter: float = 0.1, seed: int = 4) -> Mesh:
    """Structured hexahedra of the unit box with interior-node jitter (fraction of h)."""
    rng = np.random.default_rng(seed)
    xs, ys, zs = np.linspace(0, 1, nx + 1), np.linspace(0, 1, ny + 1), np.linspace(0, 1, nz + 1)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    h = np.array([1.0 / nx, 1.0 / ny, 1.0 / nz])
    d = rng.uniform(-1.0, 1.0, size=pts.shape) * jitter * h
    d[(pts < 1e-12) | (pts > 1 - 1e-12)] = 0.0
    pts = pts + d
    idx = np.arange(pts.shape[0]).reshape(nx + 1, ny + 1, nz + 1)

    def c(i0, j0, k0):
        return idx[i0:i0 + nx, j0:j0 + ny, k0:k0 + nz].ravel()
    conn = np.stack([c(0, 0, 0), c(1, 0, 0), c(1, 1, 0), c(0, 1, 0),
                     c(0, 0, 1), c(1, 0, 1), c(1, 1, 1), c(0, 1, 1)], axis=1).astype(np.int32)
    lo, hi = np.zeros(3), np.ones(3)
    node_flag = _box_flags(pts, lo, hi, open_top=True)
    bd = box_hex_sides(nx, ny, nz, open_top=True)
    el_bd = np.zeros(conn.shape[0], dtype=np.uint8)
    el_bd[bd[:, 0]] = 1
    return Mesh(pts, conn, node_flag, el_bd, bd, name=f"box_hex_{nx}x{ny}x{nz}")


def box_hex_sides(nx: int, ny: int, nz: int, open_top: bool = True) -> np.ndarray:
    """Boundary sides of box_hex's structured grid without a face search (the same
    rows, in the same order, as boundary_sides): element (i, j, k) is i*ny*nz + j*nz + k;
    local sides of SIDES[(3, 8)] are 0: z+, 1: z-, 2: x-, 3: x+, 4: y+, 5: y-."""
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    e = (I * ny * nz + J * nz + K).ravel()
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    parts = []
    for side, mask in ((0, K == nz - 1), (1, K == 0), (2, I == 0), (3, I == nx - 1), (4, J == ny - 1), (5, J == 0)):
        flag = OPEN if (side == 0 and open_top) else WALL
        el = e[mask]
        parts.append(np.stack([el, np.full(el.shape, side), np.full(el.shape, flag)], axis=1))
    bd = np.concatenate(parts).astype(np.int64)
    bd = bd[np.lexsort((bd[:, 1], bd[:, 0]))]
    return bd.astype(np.int32)


# ---------------------------------------------------------------------------
# Materials

def melt(rng) -> "object":
    """Weakly compressible melt: rho 2400, bulk modulus 1e10 (beta 1e-10), viscosity
    log-uniform in [1e2, 1e4] (one seeded value), alpha 3e-5, cp 1200, kappa 1.5."""
    mu = float(10.0 ** rng.uniform(2.0, 4.0))
    return custom_chemical(rho=2400.0, mu=mu, cp=1200.0, kappa=1.5, alpha=3.0e-5, beta=1.0e-10)


def material_for(nb_comp: int, seed: int = 0) -> Material:
    rng = np.random.default_rng(seed)
    if nb_comp == 1:
        return Material([melt(rng)])
    if nb_comp == 2:
        return Material([melt(rng), ideal_gas(8.314462 / 461.0, 1.4)])
    if nb_comp == 3:
        return Material([melt(rng), ideal_gas_named("H2O"), ideal_gas_named("CO2")])
    return Material([melt(rng), ideal_gas_named("H2O"), ideal_gas_named("CO2"), ideal_gas_named("AIR")])


def setup_for(dim: int, nb_comp: int, dirichlet_T_everywhere: bool = False, **kw) -> Setup:
    """Shipped-case flags (tau 2019, dc_2006, dc_sharp 2) with the P0 wall policy.
    3D uses gravity (0, 0, -9.81)."""
    if dim == 3 and "gravity" not in kw:
        kw["gravity"] = (0.0, 0.0, -9.81)
    s = Setup(dim, **kw)
    return p0_policy(s, nb_comp, dirichlet_T_everywhere=dirichlet_T_everywhere)


# ---------------------------------------------------------------------------
# States

def _fourier(x: np.ndarray, rng, modes: int = 8, kmax: int = 3) -> np.ndarray:
    dim = x.shape[1]
    f = np.zeros(len(x))
    for _ in range(modes):
        k = rng.integers(-kmax, kmax + 1, size=dim)
        if not k.any():
            k[0] = 1
        phi = rng.uniform(0, 2 * np.pi)
        a = rng.normal()
        f += a * np.sin(2 * np.pi * (x @ k) + phi)
    m = np.max(np.abs(f))
    return f / m if m > 0 else f


def state_for(mesh: Mesh, nb_comp: int, seed: int = 0, perturb: float = 1e-4, no_slip_flag: int = WALL):
    """Seeded (I, P) nodal states, AoS float64 of shape (n_nodes*nd,)."""
    rng = np.random.default_rng(seed)
    x = mesh.coords
    dim = x.shape[1]
    nd = nb_dofs(dim, nb_comp)
    n = len(x)
    ext = x.max(axis=0) - x.min(axis=0)
    xn = (x - x.min(axis=0)) / np.where(ext > 0, ext, 1.0)
    height = xn[:, -1]
    S = np.zeros((n, nd))
    S[:, 0] = (1e5 + (1e8 - 1e5) * (1.0 - height)) * (1.0 + 0.01 * rng.normal(size=n))
    for k in range(dim):
        S[:, 1 + k] = 0.1 * _fourier(xn, rng)
    S[node_flag_mask(mesh, no_slip_flag), 1:1 + dim] = 0.0
    S[:, dim + 1] = 1273.0 + 50.0 * _fourier(xn, rng)
    if nb_comp == 2:
        S[:, dim + 2] = np.clip(0.5 + 0.7 * _fourier(xn, rng), 0.0, 1.0)
    elif nb_comp > 2:
        w = np.stack([np.exp(1.5 * _fourier(xn, rng)) for _ in range(nb_comp)], axis=1)
        w[:, 0] *= 6.0    # melt-dominated mixture
        Y = w / w.sum(axis=1, keepdims=True)
        S[:, dim + 2:] = Y[:, :nb_comp - 1]
    I = S.ravel().copy()
    P = I.copy()
    if perturb:
        scale = np.abs(S).max(axis=0)
        dP = perturb * rng.normal(size=S.shape) * scale
        dP[:, 1:1 + dim] *= 1.0
        P = (S + dP).ravel()
    return I, P


def state_near_rest(mesh: Mesh, nb_comp: int, seed: int = 0, p_top: float = 7.0e7, rho: float = 2400.0,
                    gravity: float = 9.81):
    """A state Newton can converge from: state_for's velocity and temperature fields,
    a hydrostatic pressure p_top + rho g (z_top - z) along the last axis, and mass
    fractions mapped into [0.25, 0.75] so that the mass-fraction clamp of the
    reference's driver (model.hpp:176-184) stays inactive.  I = P."""
    I, _ = state_for(mesh, nb_comp, seed, perturb=0.0)
    nd = nb_dofs(mesh.dim, nb_comp)
    S = I.reshape(-1, nd)
    z = mesh.coords[:, -1]
    S[:, 0] = p_top + rho * gravity * (z.max() - z)
    S[:, mesh.dim + 2:] = 0.25 + 0.5 * S[:, mesh.dim + 2:]
    I = S.ravel().copy()
    return I, I.copy()


def node_flag_mask(mesh: Mesh, flag: int) -> np.ndarray:
    return mesh.node_flag == flag


def workload(name: str, seed: int = 0):
    """(mesh, material, setup, I, P, dt) of a named workload."""
    if name == "c0_tri":
        mesh = channel_tri()
        nc = 2
    elif name == "c1_tet":
        mesh = box_tet_delaunay(56, seed=seed + 1)
        nc = 3
    elif name == "c3_tet":
        mesh = box_tet_delaunay(33, seed=seed + 3)
        nc = 3
    elif name == "c4_hex":
        mesh = box_hex(160, 160, 156, seed=seed + 4)
        nc = 4
    else:
        raise KeyError(name)
    mat = material_for(nc, seed)
    setup = setup_for(mesh.dim, nc)
    I, P = state_for(mesh, nc, seed)
    return mesh, mat, setup, I, P, 1e-3


# ---------------------------------------------------------------------------
# Magma mixtures (props.txt mix_of_mix of magma_mix): synthetic compositions and
# solubility tables in the input/lookuptable format.  The tables stand in for the
# reference's solwcad-generated files (not shipped with this project): the same
# pressure grid (60-300 MPa, 0.1 MPa steps), dissolved H2O growing as sqrt(p) and CO2
# linearly until all of the magma's volatile is dissolved.

TRACHYTE_LIKE = [0.600, 0.005, 0.180, 0.020, 0.030, 0.001, 0.010, 0.030, 0.060, 0.060]
BASALT_LIKE = [0.490, 0.015, 0.160, 0.020, 0.080, 0.002, 0.080, 0.110, 0.030, 0.013]


def magma_tables(h2o_wf: float, co2_wf: float, n_p: int = 2401, p_lo: float = 6.0e7, p_hi: float = 3.0e8,
                 n_T: int = 0, T_lo: float = 1100.0, T_hi: float = 1500.0):
    """(p_table, wf_l_h2o, wf_l_co2, T_table or None): dissolved weight fractions on the
    liquid, [n_T][n_p] when n_T > 0 (solubility falling slightly with T)."""
    p = np.linspace(p_lo, p_hi, n_p)
    h2o = np.minimum(h2o_wf, 0.8 * h2o_wf * np.sqrt(p / p_lo))
    co2 = np.minimum(co2_wf, 0.15 * co2_wf * (p / p_lo))
    if n_T <= 0:
        return p, h2o, co2, None
    T = np.linspace(T_lo, T_hi, n_T)
    f = 1.0 - 0.1 * (T - T_lo) / (T_hi - T_lo)
    return p, np.outer(f, h2o), np.outer(f, co2), T


def magma_pair(gas_on_mu: str = "Ishii_Zuber", crystal_on_mu: str = "none", crystal_fraction: float = 0.0,
               n_T: int = 0):
    """Two magma_mix components like the shipped P0 case's (a K-rich and a trachytic
    melt with a few wt% volatiles), with synthetic tables."""
    magma = importlib.import_module("gales-multi-fluid_gb300.magma")
    out = []
    for name, ox, h2o, co2 in (("basaltic", BASALT_LIKE, 0.02, 0.01), ("trachytic", TRACHYTE_LIKE, 0.01, 0.001)):
        m = magma.MagmaMix(name=name, oxide_wf=ox, h2o_wf=h2o, co2_wf=co2, gas_on_mu=gas_on_mu,
                           crystal_on_mu=crystal_on_mu, crystal_fraction=crystal_fraction,
                           crystal_rho=2700.0 if crystal_fraction else 0.0)
        p, a, b, T = magma_tables(h2o, co2, n_T=n_T)
        out.append(m.with_tables(p, a, b, T))
    return out
