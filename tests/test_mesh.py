"""Synthetic mesh generators: sizes of the benchmark configurations, the
reference's orientation conventions, level invariants, discrete divergence."""
import numpy as np

from fesom2_gb300 import mesh as M


def test_channel_configuration_1_sizes():
    m = M.config_mesh(1)
    c = m.counts()
    assert c["N2"] == 40000 and c["T2"] == 79800 and c["E2"] == 119800 and m.nl == 41
    assert c["N3"] == 40000 * 40


def test_elements_are_clockwise_and_edge_tri_left(sphere_small):
    m = sphere_small
    X = m.coord_nod2D
    t = m.elem2D_nodes
    b = X[t[:, 1]] - X[t[:, 0]]
    c = X[t[:, 2]] - X[t[:, 0]]
    b[:, 0] = M._trim(b[:, 0], m.cyclic_length)
    c[:, 0] = M._trim(c[:, 0], m.cyclic_length)
    assert np.all(b[:, 0] * c[:, 1] - b[:, 1] * c[:, 0] <= 0.0)
    cx, cy = M._elem_center(X, t[m.edge_tri[:, 0]], m.cyclic_length)
    xe0 = M._trim(X[m.edges[:, 1], 0] - X[m.edges[:, 0], 0], m.cyclic_length)
    xe1 = X[m.edges[:, 1], 1] - X[m.edges[:, 0], 1]
    xc0 = M._trim(cx - X[m.edges[:, 0], 0], m.cyclic_length)
    xc1 = cy - X[m.edges[:, 0], 1]
    assert np.all(xc0 * xe1 - xc1 * xe0 <= 0.0)
    # internal edges first
    inner = m.edge_tri[:, 1] >= 0
    assert inner[:m.edge2D_in].all() and not inner[m.edge2D_in:].any()


def test_levels(channel_seamount, sphere_small, basin_irregular):
    for m in (channel_seamount, sphere_small, basin_irregular):
        assert np.all(m.nlevels >= 5) and np.all(m.nlevels <= m.nl)
        assert np.all(m.nlevels_nod2D - m.ulevels_nod2D >= 4)
        # node levels are the max over the node's elements
        nmax = np.zeros(m.nod2D, int)
        np.maximum.at(nmax, m.elem2D_nodes.reshape(-1), np.repeat(m.nlevels, 3))
        assert np.array_equal(nmax, m.nlevels_nod2D)
        assert np.all(m.hnode[M.np.arange(m.nl - 1)[None, :] < (m.nlevels_nod2D - 1)[:, None]] > 0)


def test_rot_grad_velocity_is_divergence_free_on_flat_channel(channel_small):
    f = M.make_forcing(channel_small, "channel")
    assert np.abs(f.w).max() < 1e-13


def test_separable_w_matches_general_formula(sphere_small):
    f = M.make_forcing(sphere_small, "sphere")
    w2 = M.vert_vel(sphere_small, f.uv)
    assert np.allclose(f.w, w2, rtol=1e-10, atol=1e-18)


def test_tracers_are_seeded_and_positive(sphere_small):
    a = M.make_tracers(sphere_small, "sphere", ntr=4, seed=3)
    b = M.make_tracers(sphere_small, "sphere", ntr=4, seed=3)
    assert np.array_equal(a, b)
    lev = np.arange(sphere_small.nl - 1)[None, :]
    wet = lev < (sphere_small.nlevels_nod2D - 1)[:, None]
    assert a[2][wet].min() > 0 and a[3][wet].min() > 0


def test_irregular_basin_has_high_degree_nodes(basin_irregular):
    """The Delaunay basin carries nodes of more than 8 edges (the FP32 form's second
    launch) and its gyre has no flow through the walls: w vanishes on a flat bottom."""
    m = basin_irregular
    deg = np.bincount(m.edges.reshape(-1), minlength=m.nod2D)
    assert deg.max() > 8 and deg.min() >= 2
    flat = M.delaunay_mesh(400, zbar=M.stretched_zbar(30, 10.0, 200.0), seed=3)
    assert np.abs(M.make_forcing(flat, "basin").w).max() < 1e-12
