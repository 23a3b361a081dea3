"""The FESOM2 mesh-folder reader on the two meshes of the reference's test data (Soufflet
channel, PI): topology and levels as the files give them, geometry checks, and the
oracle's step on them (a constant tracer stays constant)."""
import os

import numpy as np
import pytest

from fesom2_gb300 import mesh as M
from fesom2_gb300 import meshio as MI
from oracle import oracle as O
from tests.conftest import GOLDEN, wet_mask

# the reference checkout, when one is at hand: FESOM2_REFERENCE=<checkout> enables the comparison
REF_MESHES = os.path.join(os.environ.get("FESOM2_REFERENCE", ""), "tests", "data", "MESHES")


@pytest.mark.parametrize("name", ["soufflet", "pi", "pi_cavity"])
def test_fixture_is_the_mesh_folder(name):
    """tests/golden/mesh_*.npz holds exactly the arrays of the reference's mesh folder."""
    folder = os.path.join(REF_MESHES, name)
    if not os.environ.get("FESOM2_REFERENCE") or not os.path.isdir(folder):
        pytest.skip("reference mesh folder not present")
    a = MI.read_files(folder)
    b = MI.load_files(os.path.join(GOLDEN, f"mesh_{name}.npz"))
    assert sorted(a) == sorted(b)
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


@pytest.mark.parametrize("meshname,E2,E2in,nl", [("soufflet_file_mesh", 8575, 8525, 41),
                                                 ("pi_file_mesh", 8986, 8531, 48),
                                                 ("pi_cavity_file_mesh", 19267, 18089, 48)])
def test_file_topology(meshname, E2, E2in, nl, request):
    """Edges in file order: internal ones first, the same set as the edges of the triangles,
    the first triangle left of n1 -> n2; node levels the deepest of their elements."""
    m = request.getfixturevalue(meshname)
    assert (m.edge2D, m.edge2D_in, m.nl) == (E2, E2in, nl)
    assert np.all(m.edge_tri[:E2in, 1] >= 0) and np.all(m.edge_tri[E2in:, 1] < 0)
    built, _, nin = M._build_edges(m.coord_nod2D, m.elem2D_nodes.astype(np.int64), m.cyclic_length)
    assert nin == E2in
    key = lambda e: set(map(tuple, np.sort(e, axis=1).tolist()))
    assert key(built) == key(m.edges)
    tri = m.elem2D_nodes.astype(np.int64)
    n1, n2, t1 = m.edges[:, 0], m.edges[:, 1], m.edge_tri[:, 0]
    # each edge's triangles hold both its nodes
    assert np.all((tri[t1] == n1[:, None]).any(1) & (tri[t1] == n2[:, None]).any(1))
    cx, cy = M._elem_center(m.coord_nod2D, tri[t1], m.cyclic_length)
    c = m.coord_nod2D
    xc0 = M._trim(cx - c[n1, 0], m.cyclic_length)
    xe0 = M._trim(c[n2, 0] - c[n1, 0], m.cyclic_length)
    assert np.all(xc0 * (c[n2, 1] - c[n1, 1]) - (cy - c[n1, 1]) * xe0 <= 0.0)
    deepest = np.zeros(m.nod2D, np.int32)
    np.maximum.at(deepest, tri.reshape(-1), np.repeat(m.nlevels, 3))
    assert np.array_equal(deepest, m.nlevels_nod2D)
    assert m.nlevels.min() >= 5 and m.nlevels.max() <= nl


def test_soufflet_geometry(soufflet_file_mesh):
    """Cartesian channel: element areas tile the 4.5-degree-wide strip exactly; equal
    triangles."""
    m = soufflet_file_mesh
    Lx = 4.5 * MI.RAD * M.R_EARTH
    y = m.coord_nod2D[:, 1]
    assert abs(m.elem_area.sum() / (Lx * (y.max() - y.min()) * M.R_EARTH) - 1.0) < 1e-12
    assert np.all(m.elem_cos == 1.0)
    assert m.elem_area.max() / m.elem_area.min() < 1.001


def test_pi_rotation(pi_file_mesh):
    """The Euler rotation is orthonormal and the rotated coordinates map back to the file's
    geographical ones; the wet elements cover two thirds of the sphere."""
    R = MI.euler_matrix(*MI.PI["rotation"])
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-15)
    m = pi_file_mesh
    lon, lat = m.coord_nod2D[:, 0], m.coord_nod2D[:, 1]
    # rotated -> geographical with the transposed matrix
    glon, glat = MI.geo_to_rot(lon, lat, R.T)
    r = MI.load_files(os.path.join(GOLDEN, "mesh_pi.npz"))
    g = r["xy_deg"] * MI.RAD
    dlon = np.angle(np.exp(1j * (glon - g[:, 0])))
    assert np.abs(dlon).max() < 1e-9 and np.abs(glat - g[:, 1]).max() < 1e-9
    frac = m.elem_area.sum() / (4.0 * np.pi * M.R_EARTH ** 2)
    assert 0.6 < frac < 0.75


@pytest.mark.parametrize("meshname,kind", [("soufflet_file_mesh", "channel"), ("pi_file_mesh", "sphere"),
                                           ("pi_cavity_file_mesh", "sphere")])
def test_oracle_keeps_a_constant_tracer(meshname, kind, request):
    """Constant-tracer preservation on the file meshes (the vertical velocity closes the
    discrete divergence of the horizontal flow)."""
    m = request.getfixturevalue(meshname)
    f = O.ensure_f64(M.make_forcing(m, kind, seed=3, dt=600.0))
    wet = wet_mask(m)
    T = np.ascontiguousarray(np.where(wet, 20.0, 0.0))
    old = T.copy()
    om = O.OracleMesh(m)
    for _ in range(2):
        om.tracer_step(f, O.cfg_struct(), T, np.zeros_like(T), old)
    assert np.abs(T[wet] - 20.0).max() < 1e-12


def test_reader_rejects_inconsistent_levels(tmp_path):
    r = MI.load_files(os.path.join(GOLDEN, "mesh_soufflet.npz"))
    r["nlvls"] = r["nlvls"].copy()
    r["nlvls"][0] -= 1
    with pytest.raises(ValueError):
        MI.mesh_from_files(r, **MI.SOUFFLET)
    r = MI.load_files(os.path.join(GOLDEN, "mesh_soufflet.npz"))
    r["elvls"] = r["elvls"][:-1]
    with pytest.raises(ValueError):
        MI.mesh_from_files(r, **MI.SOUFFLET)


def test_cavity_levels(pi_cavity_file_mesh):
    """Under the ice shelves the columns start below the surface: node first levels are the
    shallowest of their elements', the layers above have no thickness, and areasvol of a level
    with an element still under the shelf is the area of the level below."""
    m = pi_cavity_file_mesh
    assert (m.ulevels > 1).sum() == 170 and (m.ulevels_nod2D > 1).sum() == 95
    umin = np.full(m.nod2D, 99)
    np.minimum.at(umin, m.elem2D_nodes.reshape(-1), np.repeat(m.ulevels, 3))
    assert np.array_equal(umin, m.ulevels_nod2D)
    lev = np.arange(m.nl - 1)[None, :]
    above = lev < (m.ulevels_nod2D - 1)[:, None]
    assert np.all(m.hnode[above] == 0.0)
    wet = wet_mask(m)
    assert np.all(m.hnode[wet] > 0.0) and np.all(m.areasvol[:, :-1][wet] > 0.0)


@pytest.mark.parametrize("scheme", [("MUSCL", "QR4C", "FCT"), ("MFCT", "PPM", "NON"), ("UPW1", "CDIFF", "FCT")])
def test_cavity_step_matches_restatement(pi_cavity_file_mesh, scheme):
    """Both restatements agree bit for bit on columns that start below the surface."""
    from tests.conftest import perturbed_old
    from tests.refimpl import Ref
    m = pi_cavity_file_mesh
    f = O.ensure_f64(M.make_forcing(m, "sphere", seed=3, dt=600.0))
    T = np.ascontiguousarray(M.make_tracers(m, "sphere", ntr=1, seed=6)[0])
    Told = perturbed_old(T, np.random.default_rng(1))
    om = O.OracleMesh(m)
    To, Oo = T.copy(), Told.copy()
    om.tracer_step(f, O.cfg_struct(*scheme), To, np.zeros_like(To), Oo)
    Tr, _ = Ref(m).tracer_step(f, T, Told, om.work["edge_up_dn_tri"], om.work["nboundary_lay"], *scheme)
    assert np.array_equal(To, Tr)

