"""Host-side logic of the Python mirror and the synthetic workloads (no GPU)."""
import numpy as np
import pytest


def test_setup_policy_masks(gm):
    s = gm.p0_policy(gm.Setup(2), nb_comp=2, dirichlet_T_everywhere=True)
    d = s.desc
    assert d.dirichlet_mask[5] == (1 << 1) | (1 << 2) | (1 << 3)      # vx, vy and T on walls
    assert d.dirichlet_mask[0] == 1 << 3                              # T on every node
    bc = d.side_bc[5]
    assert bc.q_mask == 0b11 and bc.J_mask == (1 << 0) | (1 << 8)     # q1,q2 and J1,J2 of comp 0
    s3 = gm.p0_policy(gm.Setup(3), nb_comp=3, dirichlet_T_everywhere=False)
    assert s3.desc.dirichlet_mask[5] == 0b1110 and s3.desc.dirichlet_mask[0] == 0
    s3.neumann_tau(2, 2, 0, 4.0)
    assert s3.desc.side_bc[2].tau_mask == 1 << 2 and s3.desc.side_bc[2].tau[2] == 4.0


def test_residual_check_semantics(gm):
    """residual_check.hpp:54-79: iteration 0 stores ||b||; later converged when
    ||b|| <= max(1e-8 ||b0||, 1e-5)."""
    rc = gm.ResidualCheck()
    conv, r0 = rc.execute(np.array([3.0, 4.0]), 0)
    assert not conv and r0 == 5.0
    conv, rel = rc.execute(np.array([1e-6, 0.0]), 1)
    assert conv and rel == pytest.approx(2e-7)
    conv, _ = rc.execute(np.array([1e-3, 0.0]), 2)
    assert not conv


def test_nb_dofs(gm):
    assert gm.nb_dofs(2, 2) == 5 and gm.nb_dofs(3, 3) == 7 and gm.nb_dofs(3, 4) == 8


def test_channel_workload_shape(syn, orc):
    m = syn.channel_tri()
    assert m.n_elements == 4096 and m.n_nodes == 2145
    assert set(np.unique(m.bd_sides[:, 2])) == {2, 5}
    assert len(m.bd_sides) == 2 * 64 + 2 * 32
    x = m.coords[m.conn]
    area = 0.5 * ((x[:, 1, 0] - x[:, 0, 0]) * (x[:, 2, 1] - x[:, 0, 1]) -
                  (x[:, 2, 0] - x[:, 0, 0]) * (x[:, 1, 1] - x[:, 0, 1]))
    assert np.all(area > 0) and area.sum() == pytest.approx(2.0)


@pytest.mark.parametrize("maker", ["tet", "hex"])
def test_3d_meshes_positive_and_closed(maker, syn):
    m = syn.box_tet_delaunay(7, seed=3) if maker == "tet" else syn.box_hex(4, 3, 5, jitter=0.1, seed=2)
    x = m.coords[m.conn]
    if maker == "tet":
        vol = np.einsum("ij,ij->i", np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]), x[:, 3] - x[:, 0]) / 6
        assert np.all(vol > 0) and vol.sum() == pytest.approx(1.0, rel=1e-9)
    # boundary faces tile the six box faces: flags 5 except the open top (2)
    assert set(np.unique(m.bd_sides[:, 2])) == {2, 5}
    assert np.all(m.el_on_boundary[m.bd_sides[:, 0]] == 1)


def test_state_generator_ranges(syn):
    m = syn.box_tet_delaunay(6, seed=1)
    I, P = syn.state_for(m, 3, seed=0)
    S = I.reshape(-1, 7)
    assert S[:, 0].min() > 5e4 and S[:, 0].max() < 1.1e8
    assert np.abs(S[:, 1:4]).max() <= 0.1 + 1e-12
    assert np.all(S[m.node_flag == 5, 1:4] == 0.0)
    assert S[:, 4].min() >= 1223.0 - 1e-9 and S[:, 4].max() <= 1323.0 + 1e-9
    Y = np.concatenate([S[:, 5:7], 1 - S[:, 5:7].sum(axis=1, keepdims=True)], axis=1)
    assert Y.min() > 0 and np.allclose(Y.sum(axis=1), 1.0)
    assert np.abs(P - I).max() > 0


def test_box_hex_sides_match_the_face_search(syn):
    """The structured shortcut for the hex workload's boundary equals the generic search."""
    import numpy as np
    m = syn.box_hex(5, 4, 3, jitter=0.1, seed=2)
    ref = syn.boundary_sides(m.conn, 3, m.coords, syn._face_flag_box(np.zeros(3), np.ones(3), True))
    assert np.array_equal(m.bd_sides, ref)
