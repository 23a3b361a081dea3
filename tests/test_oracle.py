"""The FP64 CPU oracle, pinned by known-answer properties and by an independent
numpy restatement of the same reference loops (tests/refimpl.py)."""
import numpy as np
import pytest

from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import perturbed_old, wet_mask
from tests.refimpl import Ref

SCHEMES = [("MUSCL", "QR4C", "FCT"), ("MFCT", "QR4C", "FCT"), ("UPW1", "UPW1", "FCT"),
           ("MUSCL", "QR4C", "NON"), ("UPW1", "QR4C", "NON")]


def _forcing(mesh, kind, **kw):
    return O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0, **kw))


@pytest.mark.parametrize("meshname,kind", [("channel_small", "channel"), ("channel_seamount", "channel"),
                                           ("sphere_small", "sphere")])
def test_gradients_match_restatement(meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    tr = M.make_tracers(mesh, kind, ntr=1, seed=4)
    T = np.ascontiguousarray(tr[0])
    om = O.OracleMesh(mesh)
    om.init_tracers_AB(O.cfg_struct(), T.copy(), np.zeros_like(T), T.copy())
    ref = Ref(mesh)
    trxy = ref.tr_xy(T)
    ewet = (ref.lev >= mesh.ulevels[:, None]) & (ref.lev <= mesh.nlevels[:, None] - 1)
    assert np.array_equal(trxy[ewet], om.work["tr_xy"][ewet])
    G = ref.fill_up_dn_grad(trxy, om.work["edge_up_dn_tri"])
    assert np.array_equal(G[ref.smask], om.work["edge_up_dn_grad"][ref.smask])


def trz_restatement(mesh, T, trz0):
    """tracer_gradient_z (src/oce_tracer_mod.F90:192-232) in numpy: tr_z(nz) = (T(nz-1) - T(nz)) /
    (0.5 (hnode(nz-1) + hnode(nz))) for nzmin < nz < nzmax, zero at nzmin and nzmax, other entries kept."""
    out = trz0.copy()
    for n in range(mesh.nod2D):
        lo, hi = int(mesh.ulevels_nod2D[n]), int(mesh.nlevels_nod2D[n])
        for nz in range(lo + 1, hi):
            dz = 0.5 * (mesh.hnode[n, nz - 2] + mesh.hnode[n, nz - 1])
            out[n, nz - 1] = (T[n, nz - 2] - T[n, nz - 1]) / dz
        out[n, lo - 1] = 0.0
        out[n, hi - 1] = 0.0
    return out


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("pi_cavity_file_mesh", "sphere")])
def test_vertical_gradient_matches_restatement(meshname, kind, request):
    """tr_z of the oracle (also filled by init_tracers_AB) against the loop restatement, on a mesh
    with partial cells and one with ice-shelf cavities (columns starting below the surface)."""
    mesh = request.getfixturevalue(meshname)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0])
    trz0 = np.full((mesh.nod2D, mesh.nl), 7.25)
    want = trz_restatement(mesh, T, trz0)
    om = O.OracleMesh(mesh)
    got = trz0.copy()
    om.tracer_gradient_z(T, got)
    assert np.array_equal(got, want)
    om.work["tr_z"][...] = trz0
    om.init_tracers_AB(O.cfg_struct(), T.copy(), np.zeros_like(T), T.copy())
    assert np.array_equal(om.work["tr_z"], want)


@pytest.mark.parametrize("scheme", SCHEMES, ids=["-".join(s) for s in SCHEMES])
@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("sphere_small", "sphere")])
def test_adv_tra_matches_restatement(scheme, meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    hor, ver, lim = scheme
    f = _forcing(mesh, kind)
    tr = M.make_tracers(mesh, kind, ntr=1, seed=4)
    T = np.ascontiguousarray(tr[0])
    rng = np.random.default_rng(5)
    TAB = np.ascontiguousarray(T * (1 + 1e-3 * rng.standard_normal(T.shape)))
    om = O.OracleMesh(mesh)
    ocfg = O.cfg_struct(hor, ver, lim)
    om.init_tracers_AB(ocfg, T.copy(), np.zeros_like(T), T.copy())
    G = om.work["edge_up_dn_grad"].copy()
    om.do_oce_adv_tra(f, ocfg, T, TAB)
    ref = Ref(mesh)
    dh, dv, aux = ref.adv_tra(f.dt, f.uv, f.w, f.w_e, T, TAB, hor, ver, lim, 0.0, 1.0, G, om.work["nboundary_lay"])
    wet = wet_mask(mesh)
    assert np.array_equal(dh[wet], om.work["del_ttf_advhoriz"][wet])
    assert np.array_equal(dv[wet], om.work["del_ttf_advvert"][wet])
    if lim == "FCT":
        assert np.array_equal(aux["LO"][wet], om.work["fct_LO"][wet])


@pytest.mark.parametrize("meshname,kind", [("channel_small", "channel"), ("sphere_small", "sphere")])
def test_vdiff_matches_restatement(meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    f = _forcing(mesh, kind)
    f.bc_surface = np.linspace(-2e-3, 1e-3, mesh.nod2D)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=2)[0])
    om = O.OracleMesh(mesh)
    To = T.copy()
    om.diff_ver_part_impl_ale(f, To)
    Tr = Ref(mesh).vdiff(f.dt, f.Kv, f.bc_surface, T)
    assert np.array_equal(To, Tr)


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("sphere_small", "sphere")])
def test_tracer_step_matches_restatement(meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    f = _forcing(mesh, kind)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=6)[0])
    Told = perturbed_old(T, np.random.default_rng(1))
    om = O.OracleMesh(mesh)
    To, Oo = T.copy(), Told.copy()
    om.tracer_step(f, O.cfg_struct(), To, np.zeros_like(To), Oo)
    Tr, Or = Ref(mesh).tracer_step(f, T, Told, om.work["edge_up_dn_tri"], om.work["nboundary_lay"])
    assert np.array_equal(To, Tr)
    assert np.array_equal(Oo, Or)


# ---- known-answer properties ----------------------------------------------------
@pytest.mark.parametrize("scheme", SCHEMES, ids=["-".join(s) for s in SCHEMES])
def test_constant_tracer_is_preserved(sphere_small, scheme):
    """With w from the discrete divergence, a constant tracer stays constant (LO = HO = c, AD = 0)."""
    mesh = sphere_small
    f = _forcing(mesh, "sphere")
    wet = wet_mask(mesh)
    T = np.where(wet, 7.25, 0.0)
    Told = T.copy()
    om = O.OracleMesh(mesh)
    cfg = O.cfg_struct(*scheme)
    for _ in range(3):
        om.tracer_step(f, cfg, T, np.zeros_like(T), Told)
    assert np.abs(T[wet] - 7.25).max() < 1e-12


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("sphere_small", "sphere")])
def test_content_conserved(meshname, kind, request):
    """Rigid lid (w(nzmin) = 0), linfs: sum T*hnode_new*areasvol conserved to 1e-12 relative."""
    mesh = request.getfixturevalue(meshname)
    f = _forcing(mesh, kind, surface_w_zero=True)
    wet = wet_mask(mesh)
    V = mesh.areasvol[:, :mesh.nl - 1]
    om = O.OracleMesh(mesh)
    for k, T in enumerate(M.make_tracers(mesh, kind, ntr=3, seed=8)):
        T = np.ascontiguousarray(T)
        Told = T.copy()
        c0 = np.sum(np.where(wet, T * mesh.hnode * V, 0.0))
        for _ in range(4):
            om.tracer_step(f, O.cfg_struct(), T, np.zeros_like(T), Told)
        c1 = np.sum(np.where(wet, T * mesh.hnode_new * V, 0.0))
        assert abs(c1 - c0) / abs(c0) < 1e-12, k


def test_fct_result_within_bounds(sphere_small):
    """After limited advection every value lies in [min, max] of max/min(LO, T) over the
    node's elements and the adjacent layers (the FCT bounds), up to round-off."""
    mesh = sphere_small
    f = _forcing(mesh, "sphere")
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    T = np.ascontiguousarray(M.make_tracers(mesh, "sphere", ntr=3, seed=12)[2])  # lognormal: sharp
    TAB = np.zeros_like(T)
    Told = T.copy()
    cfg = O.cfg_struct()
    om.init_tracers_AB(cfg, T, TAB, Told)
    om.do_oce_adv_tra(f, cfg, T, TAB)
    w = om.work
    Tadv = T + (w["del_ttf_advhoriz"] + w["del_ttf_advvert"] + T * (mesh.hnode - mesh.hnode_new)) / mesh.hnode_new
    tmax, tmin = w["tvert_max"], w["tvert_min"]
    up = np.concatenate([tmax[:, :1], tmax[:, :-1]], 1); dn = np.concatenate([tmax[:, 1:], tmax[:, -1:]], 1)
    upm = np.concatenate([tmin[:, :1], tmin[:, :-1]], 1); dnm = np.concatenate([tmin[:, 1:], tmin[:, -1:]], 1)
    lev = np.arange(1, mesh.nl)[None, :]
    inner = (lev >= mesh.ulevels_nod2D[:, None] + 1) & (lev <= mesh.nlevels_nod2D[:, None] - 2)
    hi = np.where(inner, np.maximum(np.maximum(up, tmax), dn), tmax)
    lo = np.where(inner, np.minimum(np.minimum(upm, tmin), dnm), tmin)
    tol = 1e-12 * np.abs(T).max()
    assert np.all(Tadv[wet] <= hi[wet] + tol)
    assert np.all(Tadv[wet] >= lo[wet] - tol)


def test_vertical_diffusion_solves_the_tridiagonal_system(channel_seamount):
    """The Thomas sweep equals a dense solve of the reference's tridiagonal system
    (coefficients rebuilt here from oce_ale_tracer.F90:1099-1229)."""
    mesh = channel_seamount
    f = _forcing(mesh, "channel")
    T = np.ascontiguousarray(M.make_tracers(mesh, "channel", ntr=1, seed=3)[0])
    om = O.OracleMesh(mesh)
    To = T.copy()
    om.diff_ver_part_impl_ale(f, To)
    dt = f.dt
    for n in [0, 7, mesh.nod2D // 2, mesh.nod2D - 1]:
        nzmin, nzmax = mesh.ulevels_nod2D[n], mesh.nlevels_nod2D[n]
        hn = mesh.hnode_new[n]
        z = np.zeros(mesh.nl + 1)
        zb = mesh.zbar_n_bot[n]
        z[nzmax - 1] = zb + hn[nzmax - 2] / 2
        for k in range(nzmax - 1, nzmin, -1):
            zb += hn[k - 1]
            z[k - 1] = zb + hn[k - 2] / 2
        K = np.arange(nzmin, nzmax)
        nlay = K.size
        A = np.zeros((nlay, nlay))
        for i, k in enumerate(K):
            ar, av, kv = mesh.area[n], mesh.areasvol[n], f.Kv[n]
            if k > nzmin:
                A[i, i - 1] = -kv[k - 1] * dt / (z[k - 1] - z[k]) * ar[k - 1] / av[k - 1]
            if k < nzmax - 1:
                A[i, i + 1] = -kv[k] * dt / (z[k] - z[k + 1]) * ar[k] / av[k - 1]
            A[i, i] = -A[i].sum() + hn[k - 1]
        rhs = hn[K - 1] * T[n, K - 1]
        sol = np.linalg.solve(A, rhs)
        assert np.allclose(To[n, K - 1], sol, rtol=1e-12, atol=1e-12)
        # column content conserved by the diffusion
        V = mesh.areasvol[n, K - 1] * hn[K - 1]
        assert abs(np.sum(V * To[n, K - 1]) - np.sum(V * T[n, K - 1])) <= 1e-12 * abs(np.sum(V * T[n, K - 1]))


def test_upwind_edge_flux_by_hand(channel_small):
    """One interior edge: F = -0.5*(T1*(v+|v|) + T2*(v-|v|)) with v the two-segment
    volume flux (oce_adv_tra_hor.F90:211-216), written out from the formula."""
    mesh = channel_small
    f = _forcing(mesh, "channel")
    T = np.ascontiguousarray(M.make_tracers(mesh, "channel", ntr=1, seed=3)[0])
    flux = np.zeros((mesh.edge2D, mesh.nl - 1))
    import ctypes as C
    O.lib().or_adv_tra_hor_upw1(C.byref(O.OracleMesh(mesh).s), O._ptr(f.uv), O._ptr(T), O._ptr(flux), 1)
    e = int(np.flatnonzero(mesh.edge_tri[:, 1] >= 0)[5])
    n1, n2 = mesh.edges[e]
    el1, el2 = mesh.edge_tri[e]
    dx1, dy1, dx2, dy2 = mesh.edge_cross_dxdy[e]
    for nz in range(3):
        u1, v1 = f.uv[el1, nz]
        u2, v2 = f.uv[el2, nz]
        vf = (-v1 * dx1 + u1 * dy1) * mesh.helem[el1, nz] + (v2 * dx2 - u2 * dy2) * mesh.helem[el2, nz]
        want = -0.5 * (T[n1, nz] * (vf + abs(vf)) + T[n2, nz] * (vf - abs(vf)))
        assert flux[e, nz] == want


def test_qr4c_interior_flux_by_hand(channel_seamount):
    """QR4C at an interior interface (oce_adv_tra_ver.F90:415-425), written out."""
    mesh = channel_seamount
    f = _forcing(mesh, "channel")
    n = 3
    rng = np.random.default_rng(0)
    T = np.ascontiguousarray(rng.uniform(1, 2, (mesh.nod2D, mesh.nl - 1)))
    W = np.ascontiguousarray(rng.uniform(-1e-4, 1e-4, (mesh.nod2D, mesh.nl)))
    flux = np.zeros((mesh.nod2D, mesh.nl))
    import ctypes as C
    pv = 0.7
    O.lib().or_adv_tra_ver_qr4c(C.byref(O.OracleMesh(mesh).s), O._ptr(W), O._ptr(T), C.c_double(pv), O._ptr(flux), 1)
    Z, zb = mesh.Z_3d_n[n], mesh.zbar_3d_n[n]
    nz = 5  # 1-based interface, interior
    t = lambda k: T[n, k - 1]
    zz = lambda k: Z[k - 1]
    qc = (t(nz - 1) - t(nz)) / (zz(nz - 1) - zz(nz))
    qu = (t(nz) - t(nz + 1)) / (zz(nz) - zz(nz + 1))
    qd = (t(nz - 2) - t(nz - 1)) / (zz(nz - 2) - zz(nz - 1))
    Tm1 = t(nz) + (2 * qc + qu) * (zb[nz - 1] - zz(nz)) / 3.0
    Tm2 = t(nz - 1) + (2 * qc + qd) * (zb[nz - 1] - zz(nz - 1)) / 3.0
    w = W[n, nz - 1]
    Tmean = (w + abs(w)) * Tm1 + (w - abs(w)) * Tm2
    want = (-0.5 * (1 - pv) * Tmean - pv * (0.5 * (Tm1 + Tm2)) * w) * mesh.area[n, nz - 1]
    assert flux[n, nz - 1] == want


def _tail_inputs(mesh, ntr, seed):
    rng = np.random.default_rng(seed)
    L1 = mesh.nl - 1
    vals = [np.ascontiguousarray(30.0 + 20.0 * rng.standard_normal((mesh.nod2D, L1))) for _ in range(ntr)]
    vals[-1][:] = 0.2 * rng.standard_normal((mesh.nod2D, L1))  # age tracer with negatives
    r2c = np.ascontiguousarray(rng.uniform(0.0, 1e-5, mesh.nod2D))
    Tclim = np.ascontiguousarray(10.0 + rng.standard_normal((mesh.nod2D, L1)))
    Sclim = np.ascontiguousarray(35.0 + rng.standard_normal((mesh.nod2D, L1)))
    ztem = np.ascontiguousarray(rng.standard_normal((12, L1)))
    return vals, r2c, Tclim, Sclim, ztem


def test_oracle_tail_matches_numpy(channel_small):
    """Decay, relax_to_clim and the clamps written out in numpy from the reference's formulas."""
    mesh = channel_small
    ids = [1, 2, 14, 39, 101]
    vals, r2c, Tclim, Sclim, ztem = _tail_inputs(mesh, len(ids), 3)
    dt = 600.0
    tc = O.tail_cfg(salt_index=1, age_index=4)
    got = [v.copy() for v in vals]
    O.tracer_tail(O.OracleMesh(mesh), ids, dt, tc, r2c, Tclim, Sclim, ztem, got)
    want = [v.copy() for v in vals]
    lev = np.arange(mesh.nl - 1)[None, :] + 1
    wet = (lev >= mesh.ulevels_nod2D[:, None]) & (lev <= mesh.nlevels_nod2D[:, None] - 1)
    want[2] = want[2] * np.exp(-3.8561e-12 * dt)
    want[3] = want[3] * np.exp(-8.1708e-11 * dt)
    for k, clim in ((0, Tclim), (1, Sclim)):
        upd = want[k] + r2c[:, None] * dt * (clim - want[k])
        want[k] = np.where(wet, upd, want[k])
    want[1] = np.where(wet, np.minimum(np.maximum(np.minimum(want[1], 45.0), 3.0), 45.0), want[1])
    want[4] = np.where(wet & (want[4] < 0.0), 0.0, want[4])
    for k in range(len(ids)):
        assert np.array_equal(got[k], want[k]), k


def test_oracle_tail_zonal_relax_repeats_per_tracer(channel_small):
    """relax_zonal_temp acts on tracer 1 once per tracer of the loop (the reference calls it
    inside the loop with tracers%data(1)): three tracers give three increments."""
    mesh = channel_small
    vals, r2c, Tclim, Sclim, ztem = _tail_inputs(mesh, 3, 4)
    y = mesh.coord_nod2D[:, 1]
    tc = O.tail_cfg(salt_index=-1, age_index=-1, zonal_relax=1, nbins=12, lat0=float(y.min()),
                    dy=float((y.max() - y.min()) / 12), tau_inv=1.0 / 86400.0)
    got = [v.copy() for v in vals]
    O.tracer_tail(O.OracleMesh(mesh), [1, 2, 101], 600.0, tc, r2c, Tclim, Sclim, ztem, got)
    assert np.array_equal(got[1], vals[1]) and np.array_equal(got[2], vals[2])
    one = [vals[0].copy()]
    O.tracer_tail(O.OracleMesh(mesh), [1], 600.0, tc, r2c, Tclim, Sclim, ztem, one)
    inc = one[0] - vals[0]
    assert np.allclose(got[0] - vals[0], 3 * inc, rtol=1e-12, atol=1e-12)
    assert np.abs(inc).max() > 0


def _ki(mesh, K_hor=10.0):
    """Ki = K_hor (resolution / 100 km)^2 (src/oce_setup_step.F90:968-972), resolution from the
    node's mean element area (a stand-in for mesh_resolution)."""
    ea = np.zeros(mesh.nod2D)
    np.add.at(ea, mesh.elem2D_nodes.reshape(-1), np.repeat(mesh.elem_area, 3) / 3.0)
    res = np.sqrt(ea)
    return np.ascontiguousarray(np.repeat((K_hor * (res / 100000.0) ** 2)[:, None], mesh.nl - 1, axis=1))


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("sphere_small", "sphere"),
                                           ("basin_irregular", "basin")])
def test_diffusion_parts_match_restatement(meshname, kind, request):
    """diff_part_hor_redi (Redi off) and diff_ver_part_expl_ale: oracle and numpy restatement
    agree bit for bit."""
    mesh = request.getfixturevalue(meshname)
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0])
    ref = Ref(mesh)
    om = O.OracleMesh(mesh)
    trxy = np.ascontiguousarray(ref.tr_xy(T))
    Ki = _ki(mesh)
    rng = np.random.default_rng(2)
    d0 = np.ascontiguousarray(rng.standard_normal(T.shape) * 1e-3)
    d = d0.copy()
    om.diff_part_hor_redi(600.0, Ki, trxy, d)
    assert np.array_equal(d, ref.diff_part_hor_redi(600.0, Ki, trxy, d0))
    assert np.abs(d - d0).max() > 0
    flux = np.ascontiguousarray(rng.standard_normal(mesh.nod2D) * 1e-4)
    d = d0.copy()
    om.diff_ver_part_expl_ale(600.0, f.Kv, flux, T, d)
    assert np.array_equal(d, ref.diff_ver_part_expl_ale(600.0, f.Kv, flux, T, d0))


def test_horizontal_diffusion_conserves_and_smooths(channel_seamount):
    """Edge fluxes cancel: sum del_ttf * areasvol is unchanged; a diffusion-only step lowers
    the variance of a noisy field."""
    mesh = channel_seamount
    rng = np.random.default_rng(5)
    T = np.ascontiguousarray(rng.standard_normal((mesh.nod2D, mesh.nl - 1)))
    wet = wet_mask(mesh)
    T = np.where(wet, T, 0.0)
    ref = Ref(mesh)
    trxy = np.ascontiguousarray(ref.tr_xy(T))
    d = np.zeros_like(T)
    O.OracleMesh(mesh).diff_part_hor_redi(600.0, _ki(mesh, 1e4), trxy, d)
    av = mesh.areasvol[:, :-1]
    assert abs(np.sum(d * av)) <= 1e-9 * np.sum(np.abs(d * av))
    Tn = T + d / np.where(wet, mesh.hnode_new, 1.0)
    assert np.var(Tn[wet]) < np.var(T[wet])


# ---- vertical schemes CDIFF and PPM, split vertical velocity ----------------------
from tests import refimpl as RI  # noqa: E402


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("basin_irregular", "basin")])
@pytest.mark.parametrize("scheme", ["CDIFF", "PPM"])
@pytest.mark.parametrize("wscale", [1.0, 400.0])
def test_vertical_schemes_match_restatement(meshname, kind, scheme, wscale, request):
    """adv_tra_ver_cdiff / adv_tra_vert_ppm: oracle and loop restatement agree bit for bit,
    from zero and from a given flux (the FCT form subtracts the LO flux); a large w makes
    the PPM sweep fraction reach its cap of 1."""
    mesh = request.getfixturevalue(meshname)
    f = _forcing(mesh, kind)
    W = np.ascontiguousarray(f.w * wscale)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0])
    om = O.OracleMesh(mesh)
    rng = np.random.default_rng(3)
    F0 = np.ascontiguousarray(rng.standard_normal((mesh.nod2D, mesh.nl)))
    for zero in (True, False):
        got = om.ver_flux(scheme, W, T, f.dt, flux=F0.copy(), init_zero=zero)
        start = np.zeros_like(F0) if zero else F0
        want = RI.ver_cdiff(mesh, W, T, start) if scheme == "CDIFF" else RI.ver_ppm(mesh, f.dt, W, T, start)
        assert np.array_equal(got, want), zero


def test_ppm_reconstruction_properties(channel_seamount):
    """PPM keeps a linear profile on uniform layers exactly away from the ends, and a
    constant one everywhere: the flux is then the upwind value times w area."""
    mesh = channel_seamount
    f = _forcing(mesh, "channel")
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    T = np.ascontiguousarray(np.where(wet, 3.5, 0.0))
    F = om.ver_flux("PPM", f.w, T, f.dt)
    Fu = om.ver_flux("UPW1", f.w, T, f.dt)
    assert np.allclose(F, Fu, rtol=1e-14, atol=1e-30)


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("basin_irregular", "basin")])
def test_vert_impl_and_wimpl_match_restatement(meshname, kind, request):
    """adv_tra_vert_impl and the w_i terms of diff_ver_part_impl_ale: oracle and loop
    restatement agree bit for bit; the implicit advection of a constant column changes it
    only by the column divergence of w_i."""
    mesh = request.getfixturevalue(meshname)
    f = M.split_vertical_velocity(mesh, _forcing(mesh, kind), maxcfl=0.01)
    assert np.abs(f.w_i).max() > 0
    f.bc_surface = np.linspace(-2e-3, 1e-3, mesh.nod2D)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=2)[0])
    om = O.OracleMesh(mesh)
    To = T.copy()
    om.adv_tra_vert_impl(f.w_i, To, f.dt)
    assert np.array_equal(To, RI.vert_impl(mesh, f.dt, f.w_i, T))
    assert np.abs(To - T).max() > 0
    To = T.copy()
    om.diff_ver_part_impl_ale(f, To, wimpl=True)
    assert np.array_equal(To, RI.vdiff_wimpl(mesh, f.dt, f.Kv, f.bc_surface, f.w_i, T))
    # without w_i terms the same routine is the plain implicit diffusion
    To = T.copy()
    om.diff_ver_part_impl_ale(f, To)
    assert np.array_equal(To, Ref(mesh).vdiff(f.dt, f.Kv, f.bc_surface, T))


NEW_SCHEMES = [("MUSCL", "CDIFF", "FCT", False), ("MFCT", "PPM", "FCT", False), ("UPW1", "PPM", "NON", False),
               ("MUSCL", "QR4C", "FCT", True), ("MFCT", "PPM", "FCT", True), ("MUSCL", "CDIFF", "NON", True)]


@pytest.mark.parametrize("scheme", NEW_SCHEMES, ids=["-".join(map(str, s)) for s in NEW_SCHEMES])
@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("basin_irregular", "basin")])
def test_new_vertical_options_match_restatement(scheme, meshname, kind, request):
    """do_oce_adv_tra and the whole step with CDIFF / PPM and with the split vertical
    velocity: oracle and restatement agree bit for bit."""
    hor, ver, lim, wsplit = scheme
    mesh = request.getfixturevalue(meshname)
    f = M.split_vertical_velocity(mesh, _forcing(mesh, kind), maxcfl=0.01) if wsplit else _forcing(mesh, kind)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0])
    rng = np.random.default_rng(5)
    TAB = np.ascontiguousarray(T * (1 + 1e-3 * rng.standard_normal(T.shape)))
    om = O.OracleMesh(mesh)
    ocfg = O.cfg_struct(hor, ver, lim, wsplit=wsplit)
    om.init_tracers_AB(ocfg, T.copy(), np.zeros_like(T), T.copy())
    G = om.work["edge_up_dn_grad"].copy()
    om.do_oce_adv_tra(f, ocfg, T, TAB)
    ref = Ref(mesh)
    dh, dv, aux = ref.adv_tra(f.dt, f.uv, f.w, f.w_e, T, TAB, hor, ver, lim, 0.0, 1.0, G, om.work["nboundary_lay"],
                              WI=f.w_i, wsplit=wsplit)
    wet = wet_mask(mesh)
    assert np.array_equal(dh[wet], om.work["del_ttf_advhoriz"][wet])
    assert np.array_equal(dv[wet], om.work["del_ttf_advvert"][wet])
    if lim == "FCT":
        assert np.array_equal(aux["LO"][wet], om.work["fct_LO"][wet])
    Told = perturbed_old(T, np.random.default_rng(1))
    To, Oo = T.copy(), Told.copy()
    om.tracer_step(f, ocfg, To, np.zeros_like(To), Oo)
    Tr, _ = ref.tracer_step(f, T, Told, om.work["edge_up_dn_tri"], om.work["nboundary_lay"], hor, ver, lim,
                            wsplit=wsplit)
    assert np.array_equal(To, Tr)


def test_wsplit_without_implicit_part_is_the_plain_step(channel_seamount):
    """With w_i = 0 the split path (implicit LO advection, LO flux of the full w) reduces to
    the plain one exactly; with w_i != 0 it does not."""
    mesh = channel_seamount
    f = _forcing(mesh, "channel")
    T = np.ascontiguousarray(M.make_tracers(mesh, "channel", ntr=1, seed=4)[0])
    om = O.OracleMesh(mesh)
    outs = []
    for ff, ws in ((f, False), (f, True), (M.split_vertical_velocity(mesh, f, maxcfl=0.01), True)):
        Tx, Ox = T.copy(), T.copy()
        om.tracer_step(ff, O.cfg_struct("MUSCL", "QR4C", "FCT", wsplit=ws), Tx, np.zeros_like(Tx), Ox)
        outs.append(Tx)
    assert np.array_equal(outs[0], outs[1])
    assert not np.array_equal(outs[0], outs[2])


@pytest.mark.parametrize("ver", ["CDIFF", "PPM"])
@pytest.mark.parametrize("lim", ["FCT", "NON"])
def test_constant_tracer_new_vertical_schemes(sphere_small, ver, lim):
    mesh = sphere_small
    f = _forcing(mesh, "sphere")
    wet = wet_mask(mesh)
    T = np.ascontiguousarray(np.where(wet, 7.25, 0.0))
    Told = T.copy()
    om = O.OracleMesh(mesh)
    om.tracer_step(f, O.cfg_struct("MUSCL", ver, lim), T, np.zeros_like(T), Told)
    assert np.abs(T[wet] - 7.25).max() < 1e-12


# ---- Redi = .true.: isoneutral diffusion with the tapered neutral slopes as input ----------
@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("basin_irregular", "basin"),
                                           ("sphere_small", "sphere")])
def test_redi_parts_match_restatement(meshname, kind, request):
    """The slope terms of diff_part_hor_redi, diff_ver_part_redi_expl and the K33 of the
    implicit solve: oracle and numpy restatement agree bit for bit, and each term is non-zero."""
    mesh = request.getfixturevalue(meshname)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0])
    ref = Ref(mesh)
    om = O.OracleMesh(mesh)
    trxy = np.ascontiguousarray(ref.tr_xy(T))
    trz = RI.tr_z(mesh, T)
    tz = np.zeros((mesh.nod2D, mesh.nl))
    om.tracer_gradient_z(T, tz)
    lev = np.arange(1, mesh.nl + 1)[None, :]
    col = (lev >= mesh.ulevels_nod2D[:, None]) & (lev <= mesh.nlevels_nod2D[:, None])
    assert np.array_equal(np.where(col, tz, 0.0), trz)
    slope = M.make_slopes(mesh)
    Ki = _ki(mesh, 1e3)
    rng = np.random.default_rng(2)
    d0 = np.ascontiguousarray(rng.standard_normal(T.shape) * 1e-3)
    d = d0.copy()
    om.diff_part_hor_redi(600.0, Ki, trxy, d, slope=slope, tr_z=trz)
    assert np.array_equal(d, ref.diff_part_hor_redi(600.0, Ki, trxy, d0, slope=slope, trz=trz))
    plain = d0.copy()
    om.diff_part_hor_redi(600.0, Ki, trxy, plain)
    assert np.abs(d - plain).max() > 0
    d = d0.copy()
    om.diff_ver_part_redi_expl(600.0, Ki, slope, trxy, d)
    assert np.array_equal(d, RI.redi_vexpl(mesh, 600.0, Ki, slope, trxy, d0))
    assert np.abs(d - d0).max() > 0
    Kv = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0)).Kv
    K33 = om.redi_k33(Kv, Ki, slope)
    assert np.array_equal(K33, RI.redi_k33(mesh, Kv, Ki, slope))
    assert (K33 >= Kv).all() and (K33 > Kv).any()


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("sphere_small", "sphere")])
def test_redi_step_properties(meshname, kind, request):
    """A whole step with Redi: zero slopes give the Redi-off step exactly; the isoneutral terms
    move tracer between columns and levels without changing the rigid-lid content beyond
    round-off; a constant tracer stays constant."""
    mesh = request.getfixturevalue(meshname)
    f = _forcing(mesh, kind)
    f0 = _forcing(mesh, kind, surface_w_zero=True)
    T0 = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0])
    om = O.OracleMesh(mesh)
    Ki = _ki(mesh, 1e3)
    slope = M.make_slopes(mesh, smax=5e-3, s_cr=4e-3)
    cfg = O.cfg_struct()

    def step(forcing, sl, T=T0):
        T = T.copy()
        old = T.copy()
        om.tracer_step_ex(forcing, cfg, T, np.zeros_like(T), old, Ki=Ki, slope=sl)
        return T

    off = step(f, None)
    assert np.array_equal(step(f, np.zeros_like(slope)), off)
    on = step(f, slope)
    assert np.abs(on - off).max() > 0
    wet = wet_mask(mesh)
    V = mesh.hnode_new * mesh.areasvol[:, :-1]
    c0 = np.sum(np.where(wet, T0 * mesh.hnode * mesh.areasvol[:, :-1], 0.0))
    c1 = np.sum(np.where(wet, step(f0, slope) * V, 0.0))
    assert abs(c1 - c0) <= 1e-12 * abs(c0)
    const = np.where(wet, 3.5, 0.0)
    got = step(f, slope, const)
    assert np.abs(got[wet] - 3.5).max() <= 1e-12 * 3.5
