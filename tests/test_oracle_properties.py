"""Property checks of the oracle over many generated meshes (hypothesis; skipped where the
package is absent): on irregular Delaunay basins of random size, depth and seamounts, the
whole step of every scheme set equals the independent numpy restatement bit for bit, and every
FCT-limited value stays inside its bounds."""
import numpy as np
import pytest

hyp = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

from fesom2_gb300 import mesh as M  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.conftest import perturbed_old, wet_mask  # noqa: E402
from tests.refimpl import Ref  # noqa: E402

SCHEMES = [("MUSCL", "QR4C", "FCT"), ("MFCT", "QR4C", "FCT"), ("UPW1", "UPW1", "FCT"), ("MUSCL", "QR4C", "NON"),
           ("MFCT", "UPW1", "NON")]


@settings(max_examples=40, deadline=None)
@given(npts=st.integers(40, 160), nlev=st.integers(5, 25), seamounts=st.integers(0, 3), seed=st.integers(0, 10_000),
       scheme=st.sampled_from(SCHEMES), partial=st.booleans())
def test_random_basins_match_restatement(npts, nlev, seamounts, seed, scheme, partial):
    mesh = M.delaunay_mesh(npts, zbar=M.stretched_zbar(nlev, 10.0, 200.0), seamounts=seamounts, seed=seed,
                           partial_cells=partial)
    f = O.ensure_f64(M.make_forcing(mesh, "basin", seed=seed + 1, dt=600.0))
    T = np.ascontiguousarray(M.make_tracers(mesh, "basin", ntr=1, seed=seed + 2)[0])
    Told = perturbed_old(T, np.random.default_rng(seed))
    hor, ver, lim = scheme
    om = O.OracleMesh(mesh)
    To, Oo = T.copy(), Told.copy()
    om.tracer_step(f, O.cfg_struct(hor, ver, lim), To, np.zeros_like(To), Oo)
    Tr, Or = Ref(mesh).tracer_step(f, T, Told, om.work["edge_up_dn_tri"], om.work["nboundary_lay"], hor, ver, lim)
    assert np.array_equal(To, Tr)
    assert np.array_equal(Oo, Or)


@settings(max_examples=25, deadline=None)
@given(npts=st.integers(40, 160), nlev=st.integers(5, 25), seed=st.integers(0, 10_000))
def test_random_basins_fct_bounds(npts, nlev, seed):
    """do_oce_adv_tra with FCT: LO + the limited antidiffusive increments stays inside
    [bmin, bmax] of the FCT bounds (oce_adv_tra_fct.F90:124-248), up to round-off."""
    mesh = M.delaunay_mesh(npts, zbar=M.stretched_zbar(nlev, 10.0, 200.0), seamounts=2, seed=seed)
    f = O.ensure_f64(M.make_forcing(mesh, "basin", seed=seed + 1, dt=600.0))
    T = np.ascontiguousarray(M.make_tracers(mesh, "basin", ntr=1, seed=seed + 2)[0])
    om = O.OracleMesh(mesh)
    cfg = O.cfg_struct("MUSCL", "QR4C", "FCT")
    om.init_tracers_AB(cfg, T.copy(), np.zeros_like(T), T.copy())
    om.do_oce_adv_tra(f, cfg, T, T)
    wet = wet_mask(mesh)
    # T* of the advection alone: (T hnode + del_ttf) / hnode_new (oce_ale_tracer.F90:743-754)
    dttf = om.work["del_ttf_advhoriz"] + om.work["del_ttf_advvert"]
    with np.errstate(divide="ignore", invalid="ignore"):  # dry layers have no thickness
        Tstar = (T * mesh.hnode + dttf) / mesh.hnode_new
    LO = om.work["fct_LO"]
    hi = LO + om.work["fct_ttf_max"]
    lo = LO + om.work["fct_ttf_min"]
    scale = np.abs(T[wet]).max()
    assert (Tstar[wet] <= hi[wet] + 1e-11 * scale).all()
    assert (Tstar[wet] >= lo[wet] - 1e-11 * scale).all()
