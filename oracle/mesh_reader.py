"""TEST INFRASTRUCTURE — a plain-Python restatement of the reference's mesh reader,
used only by tests/ as the checker of the library's native reader (gales_mesh_read).

It follows src/fem/mesh/mesh.hpp step by step for one MPI rank `pid`:
  read_header (147-167): "MESH! nD", then "nodes N", "elements N", "sides N" (the
    second token of each), then one line per dimension;
  read_elements (184-242): skip the N Node lines; for each Element line of this pid
    keep gid, node gids (tokens 4..), flag (token 4+nnodes, on boundary when > 0);
    my_nodes = sorted distinct node gids of those elements;
  read_sides (253-277): for each Side line of this pid keep its node gids and flag;
  read_nodes (294-370): rewind; walk the lines, skipping those not starting with
    "Node"; a Node line whose gid equals the next entry of my_nodes becomes the next
    local node (x, y, [z], flag at token dim+2), so Node lines must be sorted by gid;
  set_element_node_links (383-399): an element node's local id is the position of its
    gid in my_nodes (a linear find);
  el_side_info (409-456): for each boundary element and local side (element.hpp side
    tables), if every side node is a boundary node, the flag of the last Side line with
    the same node set (are_equal sorts both, algorithm.hpp:183-189), else 0.
Tokens are split on spaces and commas with empty tokens compressed
(algorithm.hpp:219-225).  PARITY UNPINNED: the reference does not build here and no
case mesh ships, so this restatement is checked only against files written in the
format.  The linear searches are kept: use small meshes.
"""
from __future__ import annotations

import re

# local side tables (element.hpp:100-104, 145-149, 401-408, 455-460)
SIDE_TABLES = {
    (2, 3): [[1, 2], [2, 0], [0, 1]],
    (2, 4): [[0, 1], [1, 2], [2, 3], [3, 0]],
    (3, 4): [[1, 2, 3], [0, 3, 2], [0, 1, 3], [0, 2, 1]],
    (3, 8): [[4, 5, 6, 7], [0, 3, 2, 1], [0, 4, 7, 3], [1, 2, 6, 5], [2, 3, 7, 6], [1, 5, 4, 0]],
}


def _split(line: str) -> list:
    return [t for t in re.split(r"[ ,]+", line.strip()) if t != ""]


def read(path: str, pid: int, dim: int) -> dict:
    """Arrays of one rank's mesh: coords, node_flag, node_gid, conn (local ids),
    el_gid, el_on_boundary, and sides = list of (element index, local side, flag) for
    the sides with flag > 0."""
    with open(path) as f:
        lines = f.read().split("\n")
    pos = 0

    def next_tokens():
        nonlocal pos
        tok = _split(lines[pos])
        pos += 1
        return tok

    # read_header
    next_tokens()                                # MESH! nD
    tot_nodes = int(next_tokens()[1])
    tot_elements = int(next_tokens()[1])
    tot_sides = int(next_tokens()[1])
    for _ in range(dim):
        next_tokens()
    # read_elements
    pos += tot_nodes
    elements = []                                # (gid, node gids, flag)
    my_nodes = []
    for _ in range(tot_elements):
        r = next_tokens()
        if int(r[2]) == pid:
            nn = int(r[3])
            gids = [int(r[4 + j]) for j in range(nn)]
            my_nodes += gids
            elements.append((int(r[1]), gids, int(r[4 + nn])))
    my_nodes = sorted(set(my_nodes))
    # read_sides
    sides = []
    for _ in range(tot_sides):
        r = next_tokens()
        if int(r[2]) == pid:
            nsn = int(r[3])
            sides.append(([int(r[4 + j]) for j in range(nsn)], int(r[4 + nsn])))
    # read_nodes (rewind)
    coords, node_flag = [], []
    pos = 0
    k = 0
    while k < len(my_nodes):
        r = next_tokens()
        if not r or r[0] != "Node":
            continue
        if int(r[1]) == my_nodes[k]:
            coords.append([float(r[2 + d]) for d in range(dim)])
            node_flag.append(int(r[dim + 2]))
            k += 1
    # set_element_node_links
    conn = [[my_nodes.index(g) for g in gids] for _, gids, _ in elements]
    # el_side_info
    bd_sides = []
    for e, (_, gids, flag) in enumerate(elements):
        if flag <= 0:
            continue
        table = SIDE_TABLES[(dim, len(gids))]
        for s, loc in enumerate(table):
            side_nds = [gids[j] for j in loc]
            sd_flag = 0
            if all(node_flag[conn[e][j]] > 0 for j in loc):
                for nodes, f in sides:
                    if sorted(side_nds) == sorted(nodes):
                        sd_flag = f
            if sd_flag > 0:
                bd_sides.append((e, s, sd_flag))
    return {
        "coords": coords, "node_flag": node_flag, "node_gid": my_nodes, "conn": conn,
        "el_gid": [g for g, _, _ in elements], "el_on_boundary": [1 if f > 0 else 0 for _, _, f in elements],
        "sides": bd_sides,
    }
