"""GALES mesh files (the ``MESH!`` text format of src/fem/mesh/mesh.hpp).

``read_mesh`` parses a file with the library's native reader (``gales_mesh_read``,
host code, no GPU); ``write_mesh`` writes a ``Mesh`` in the same format, so that
synthetic meshes can be handed to the reference's own reader.

Format (mesh.hpp:147-456): ``MESH! 2D`` or ``MESH! 3D``, ``nodes N``, ``elements N``,
``sides N``, one bounds line per dimension (``X lo hi``), then N lines
``Node gid x y [z] flag``, N lines ``Element gid pid nnodes n_0 .. flag`` and N lines
``Side gid pid nsn n_0 .. flag``; tokens are separated by spaces or commas.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Optional

import numpy as np

from . import GalesError, Mesh, abi
from .synthetic import SIDES


def read_mesh(path, pid: int = -1, name: str = "") -> Mesh:
    """Mesh of one partition (pid >= 0: its elements and sides, as one MPI rank of the
    reference reads them) or of the whole file (pid < 0).  Node local ids are the
    positions of the sorted distinct node gids the elements use (mesh.hpp:239,
    303-331).  The result carries ``node_gid`` and ``el_gid``, the file's ids."""
    L = abi.lib()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    rc = L.gales_mesh_read(str(path).encode(), int(pid), C.byref(h), err, 512)
    if rc:
        raise GalesError(rc, f"gales_mesh_read({path}): {err.value.decode(errors='replace')}")
    try:
        d = abi.MeshDesc()
        ng, eg = C.POINTER(C.c_int64)(), C.POINTER(C.c_int64)()
        L.gales_mesh_file_desc(h, C.byref(d), C.byref(ng), C.byref(eg))
        nn, ne, nb, dim, nen = d.n_nodes, d.n_elements, d.n_bd_sides, d.dim, d.nen

        def take(ptr, shape, dtype):
            if int(np.prod(shape)) == 0:
                return np.zeros(shape, dtype)
            return np.ctypeslib.as_array(ptr, shape=shape).astype(dtype, copy=True)

        coords = take(d.coords, (nn, dim), np.float64)
        conn = take(d.conn, (ne, nen), np.int32)
        node_flag = take(d.node_flag, (nn,), np.int32)
        el_on_boundary = take(d.el_on_boundary, (ne,), np.uint8)
        bd = np.stack([take(d.bd_side_el, (nb,), np.int32), take(d.bd_side_local, (nb,), np.int32),
                       take(d.bd_side_flag, (nb,), np.int32)], axis=1) if nb else np.zeros((0, 3), np.int32)
        node_gid = take(ng, (nn,), np.int64)
        el_gid = take(eg, (ne,), np.int64)
    finally:
        L.gales_mesh_file_free(h)
    mesh = Mesh(coords, conn, node_flag, el_on_boundary, bd, name=name or Path(str(path)).name)
    mesh.node_gid = node_gid
    mesh.el_gid = el_gid
    return mesh


def write_mesh(mesh: Mesh, path, el_pid: Optional[np.ndarray] = None, sep: str = " ",
               extra_sides: Optional[list] = None) -> None:
    """Writes ``mesh`` in the GALES format.  Node gids are the node indices, element
    gids the element indices; ``el_pid`` gives each element's partition (default 0).
    An element is flagged 1 when it has a boundary side, and one Side line is written
    per boundary side (its nodes in the element's local side order, the pid of its
    element).  ``extra_sides`` appends (pid, node gids, flag) Side lines as given."""
    dim, nen = mesh.dim, mesh.nen
    pid = np.zeros(mesh.n_elements, np.int64) if el_pid is None else np.asarray(el_pid, np.int64)
    table = np.asarray(SIDES[(dim, nen)])
    bd = mesh.bd_sides
    sides = [(int(pid[e]), [int(x) for x in mesh.conn[e, table[s]]], int(f)) for e, s, f in bd]
    sides += list(extra_sides or [])
    el_flag = np.zeros(mesh.n_elements, np.int64)
    if len(bd):
        el_flag[bd[:, 0]] = 1
    el_flag = np.maximum(el_flag, mesh.el_on_boundary.astype(np.int64))
    lo, hi = mesh.coords.min(axis=0), mesh.coords.max(axis=0)
    lines = [f"MESH!{sep}{dim}D", f"nodes{sep}{mesh.n_nodes}", f"elements{sep}{mesh.n_elements}",
             f"sides{sep}{len(sides)}"]
    lines += [f"{'XYZ'[d]}{sep}{float(lo[d])!r}{sep}{float(hi[d])!r}" for d in range(dim)]
    for i in range(mesh.n_nodes):
        xyz = sep.join(repr(float(x)) for x in mesh.coords[i])
        lines.append(f"Node{sep}{i}{sep}{xyz}{sep}{int(mesh.node_flag[i])}")
    for e in range(mesh.n_elements):
        nodes = sep.join(str(int(x)) for x in mesh.conn[e])
        lines.append(f"Element{sep}{e}{sep}{int(pid[e])}{sep}{nen}{sep}{nodes}{sep}{int(el_flag[e])}")
    for k, (p, nodes, f) in enumerate(sides):
        lines.append(f"Side{sep}{k}{sep}{p}{sep}{len(nodes)}{sep}{sep.join(str(x) for x in nodes)}{sep}{f}")
    Path(path).write_text("\n".join(lines) + "\n")


def _main(argv) -> None:
    """python -m gales-multi-fluid_gb300.meshio FILE [PID]: time the native reader
    (median of three reads) and print one JSON line."""
    import json
    import statistics
    import time
    path, pid = argv[0], int(argv[1]) if len(argv) > 1 else -1
    times, m = [], None
    for _ in range(3):
        t0 = time.perf_counter()
        m = read_mesh(path, pid=pid)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    size = Path(path).stat().st_size
    print(json.dumps({"file": str(path), "bytes": size, "elements": int(m.n_elements), "nodes": int(m.n_nodes),
                      "boundary_sides": int(len(m.bd_sides)), "seconds": t, "MB_per_s": size / t / 1e6,
                      "elements_per_s": m.n_elements / t}))


if __name__ == "__main__":
    import sys
    _main(sys.argv[1:])
