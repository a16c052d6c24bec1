"""GALES mesh files: the native reader (gales_mesh_read) against the restatement of
the reference's reader (oracle/mesh_reader.py, mesh.hpp:147-456) on files written in
the format, whole meshes and MPI partitions, plus the reader's own edge cases."""
import importlib
import random
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
gm = importlib.import_module("gales-multi-fluid_gb300")
syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")
import mesh_reader  # noqa: E402  (oracle/mesh_reader.py)

MESHES = {
    "tri3": lambda: syn.channel_tri(8, 4),
    "quad4": lambda: syn.channel_quad(8, 4, jitter=0.1, seed=3),
    "tet4": lambda: syn.box_tet_delaunay(6, seed=2),
    "hex8": lambda: syn.box_hex(4, 3, 3, jitter=0.1, seed=5),
}


def _sorted_sides(a):
    a = np.asarray(a, dtype=np.int64).reshape(-1, 3)
    return a[np.lexsort(a.T[::-1])]


def _check_against_oracle(path, pid, dim):
    got = gm.read_mesh(path, pid=pid)
    ref = mesh_reader.read(str(path), pid, dim)
    assert np.array_equal(got.coords, np.asarray(ref["coords"], dtype=np.float64).reshape(-1, dim))
    assert np.array_equal(got.node_flag, np.asarray(ref["node_flag"], dtype=np.int32))
    assert np.array_equal(got.node_gid, np.asarray(ref["node_gid"], dtype=np.int64))
    assert np.array_equal(got.conn, np.asarray(ref["conn"], dtype=np.int32).reshape(got.conn.shape))
    assert np.array_equal(got.el_gid, np.asarray(ref["el_gid"], dtype=np.int64))
    assert np.array_equal(got.el_on_boundary, np.asarray(ref["el_on_boundary"], dtype=np.uint8))
    assert np.array_equal(_sorted_sides(got.bd_sides), _sorted_sides(ref["sides"]))
    return got


@pytest.mark.parametrize("kind", sorted(MESHES))
def test_whole_mesh_matches_oracle_and_round_trips(kind, tmp_path):
    m = MESHES[kind]()
    p = tmp_path / "mesh.txt"
    gm.write_mesh(m, p)
    got = _check_against_oracle(p, 0, m.dim)
    assert np.array_equal(got.coords, m.coords) and np.array_equal(got.conn, m.conn)
    assert np.array_equal(got.node_flag, m.node_flag)
    assert np.array_equal(_sorted_sides(got.bd_sides), _sorted_sides(m.bd_sides))
    every = gm.read_mesh(p, pid=-1)
    assert np.array_equal(every.conn, got.conn)


@pytest.mark.parametrize("kind", ["tri3", "tet4", "hex8"])
def test_partitions_match_oracle(kind, tmp_path):
    m = MESHES[kind]()
    rng = np.random.default_rng(7)
    # three partitions, contiguous in a random direction (as a graph partitioner's would be)
    c = m.coords[m.conn].mean(axis=1) @ rng.normal(size=m.dim)
    pid = np.searchsorted(np.quantile(c, [1 / 3, 2 / 3]), c)
    p = tmp_path / "mesh.txt"
    gm.write_mesh(m, p, el_pid=pid)
    seen = []
    for r in range(3):
        got = _check_against_oracle(p, r, m.dim)
        seen += list(got.el_gid)
        # local node ids are positions in the sorted gid list; gids address the file's nodes
        assert np.all(np.diff(got.node_gid) > 0)
        assert np.array_equal(got.coords, m.coords[got.node_gid])
        assert np.array_equal(got.node_gid[got.conn], m.conn[got.el_gid])
    assert sorted(seen) == list(range(m.n_elements))


@pytest.mark.parametrize("sep", [", ", "  ", ","])
def test_separators(sep, tmp_path):
    m = MESHES["tet4"]()
    a, b = tmp_path / "a.txt", tmp_path / "b.txt"
    gm.write_mesh(m, a)
    gm.write_mesh(m, b, sep=sep)
    ga = gm.read_mesh(a)
    gb = _check_against_oracle(b, 0, 3)
    assert np.array_equal(ga.coords, gb.coords) and np.array_equal(ga.conn, gb.conn)
    assert np.array_equal(_sorted_sides(ga.bd_sides), _sorted_sides(gb.bd_sides))


def test_side_flag_rules(tmp_path):
    """A Side line whose nodes are not all boundary nodes gives no flag; the last of
    several Side lines with one node set wins; Side lines of other pids are ignored."""
    m = MESHES["tet4"]()
    e, s, f = (int(x) for x in m.bd_sides[0])
    table = np.asarray(syn.SIDES[(3, 4)])
    nodes = [int(x) for x in m.conn[e, table[s]]]
    interior = int(np.nonzero(m.node_flag == 0)[0][0])
    extra = [(0, [nodes[0], nodes[1], interior], 7),        # an interior node: never matched
             (0, nodes[::-1], 9),                            # same set, later: wins
             (1, nodes, 11)]                                 # other pid: ignored for pid 0
    p = tmp_path / "mesh.txt"
    gm.write_mesh(m, p, extra_sides=extra)
    got = _check_against_oracle(p, 0, 3)
    row = got.bd_sides[(got.bd_sides[:, 0] == e) & (got.bd_sides[:, 1] == s)]
    assert row.shape == (1, 3) and row[0, 2] == 9


def test_sparse_gids(tmp_path):
    """Node gids far apart (a partition's extract of a large mesh) read as dense ones do."""
    m = MESHES["tet4"]()
    a, b = tmp_path / "a.txt", tmp_path / "b.txt"
    gm.write_mesh(m, a)
    remap = lambda g: str(int(g) * 1000003 + 17)  # noqa: E731
    out = []
    for line in a.read_text().splitlines():
        t = line.split(" ")
        if t[0] == "Node":
            t[1] = remap(t[1])
        elif t[0] in ("Element", "Side"):
            k = int(t[3])
            t[4:4 + k] = [remap(x) for x in t[4:4 + k]]
        out.append(" ".join(t))
    b.write_text("\n".join(out) + "\n")
    ga = gm.read_mesh(a)
    gb = _check_against_oracle(b, 0, 3)
    assert np.array_equal(gb.node_gid, np.arange(m.n_nodes) * 1000003 + 17)
    assert np.array_equal(ga.conn, gb.conn) and np.array_equal(ga.coords, gb.coords)
    assert np.array_equal(_sorted_sides(ga.bd_sides), _sorted_sides(gb.bd_sides))


def test_unsorted_node_lines(tmp_path):
    """Node lines in any order read the same (the reference needs them sorted)."""
    m = MESHES["hex8"]()
    a, b = tmp_path / "a.txt", tmp_path / "b.txt"
    gm.write_mesh(m, a)
    lines = a.read_text().splitlines()
    head, rest = lines[:4 + m.dim], lines[4 + m.dim:]
    nodes, others = rest[:m.n_nodes], rest[m.n_nodes:]
    random.Random(3).shuffle(nodes)
    b.write_text("\n".join(head + nodes + others) + "\n")
    ga, gb = gm.read_mesh(a), gm.read_mesh(b)
    assert np.array_equal(ga.coords, gb.coords) and np.array_equal(ga.node_flag, gb.node_flag)
    assert np.array_equal(ga.conn, gb.conn)
    assert np.array_equal(_sorted_sides(ga.bd_sides), _sorted_sides(gb.bd_sides))


@pytest.mark.parametrize("edit, msg", [
    (lambda L: L.__setitem__(6, L[6].replace("Node 0 ", "Node zero ")), "line 7"),
    (lambda L: L.__setitem__(0, "MESH! 4D"), "MESH! 2D"),
    (lambda L: L.__setitem__(1, "nodes"), "line 2"),
    (lambda L: L.pop(), "file ends"),
])
def test_malformed_files_report_the_line(edit, msg, tmp_path):
    m = MESHES["tri3"]()
    p = tmp_path / "mesh.txt"
    gm.write_mesh(m, p)
    lines = p.read_text().splitlines()
    edit(lines)
    p.write_text("\n".join(lines) + "\n")
    with pytest.raises(gm.GalesError) as ei:
        gm.read_mesh(p)
    assert msg in str(ei.value)


def test_missing_node_and_mixed_elements(tmp_path):
    m = MESHES["tri3"]()
    p = tmp_path / "mesh.txt"
    gm.write_mesh(m, p)
    lines = p.read_text().splitlines()
    q = tmp_path / "q.txt"
    q.write_text("\n".join(lines[:6] + ["Node 100000 0.0 0.0 0"] + lines[7:]) + "\n")
    with pytest.raises(gm.GalesError, match="has no Node line"):
        gm.read_mesh(q)
    k = next(i for i, s in enumerate(lines) if s.startswith("Element"))
    lines[k] = "Element 0 0 4 0 1 2 3 0"
    q.write_text("\n".join(lines) + "\n")
    with pytest.raises(gm.GalesError, match="different node counts"):
        gm.read_mesh(q)
    with pytest.raises(gm.GalesError, match="cannot open"):
        gm.read_mesh(tmp_path / "absent.txt")


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["tet", "hex"])
def test_mesh_from_file_assembles_like_the_in_memory_mesh(kind, tmp_path, cuda_lib):
    """The file path feeds the kernels: a mesh written and read back gives the same
    pattern, CSR values and rhs as the mesh it was written from."""
    import cases
    mesh, mat, setup, I, P, dt = cases.make(kind, 3)
    p = tmp_path / "mesh.txt"
    gm.write_mesh(mesh, p)
    back = gm.read_mesh(p)
    out = []
    for m in (mesh, back):
        fa = gm.FluidAssembly(m, mat, setup)
        lp = fa.linear_system()
        fa.execute(I, P, dt, lp, form=gm.FORM_FP64)
        out.append((lp.row_ptr.copy(), lp.col.copy(), np.asarray(lp.vals).copy(), np.asarray(lp.rhs).copy()))
    (rp0, c0, v0, b0), (rp1, c1, v1, b1) = out
    assert np.array_equal(rp0, rp1) and np.array_equal(c0, c1)
    assert cases.rel(v1, v0) <= 1e-13 and cases.rel(b1, b0) <= 1e-13
