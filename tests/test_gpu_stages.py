"""Stage-by-stage FP64 parity of the drop-in do_oce_adv_tra with the oracle's
individual routines: AB values, element gradients, LO edge fluxes, antidiffusive
edge and vertical fluxes, LO solution, R+/R-, advective increments."""
import ctypes as C

import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import wet_mask

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("meshname,kind", [("channel_small", "channel"), ("channel_seamount", "channel"),
                                           ("sphere_small", "sphere")])
def test_adv_tra_stages(meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0])
    rng = np.random.default_rng(5)
    TAB = np.ascontiguousarray(T * (1 + 1e-3 * rng.standard_normal(T.shape)))
    ctx = G.Context(mesh, G.PREC_FP64)
    dh, dv = ctx.adv_tra(f, G.tra_cfg(), T, TAB)
    om = O.OracleMesh(mesh)
    L = O.lib()
    s, w = C.byref(om.s), om.work
    cfg = O.cfg_struct()
    om.init_tracers_AB(cfg, T.copy(), np.zeros_like(T), T.copy())
    E, N2, L1, nl = mesh.edge2D, mesh.nod2D, mesh.nl - 1, mesh.nl
    wet = wet_mask(mesh)
    lev = np.arange(1, nl)[None, :]
    ewet = (lev >= mesh.ulevels[:, None]) & (lev <= mesh.nlevels[:, None] - 1)
    report = {}
    report["trxy"] = np.array_equal(ctx.debug_fetch("trxy")[ewet], w["tr_xy"][ewet])
    flo = np.zeros((E, L1))
    L.or_adv_tra_hor_upw1(s, O._ptr(f.uv), O._ptr(T), O._ptr(flo), 1)
    report["FLO"] = np.array_equal(ctx.debug_fetch("FLO"), flo)
    adh = flo.copy()
    L.or_adv_tra_hor_muscl(s, O._ptr(f.uv), O._ptr(TAB), C.c_double(0.0), O._ptr(adh),
                           O._ptr(w["edge_up_dn_grad"]), O._ptr(w["nboundary_lay"]), 0)
    report["ADh"] = np.array_equal(ctx.debug_fetch("ADh"), adh)
    fv = np.zeros((N2, nl))
    L.or_adv_tra_ver_upw1(s, O._ptr(f.w_e), O._ptr(T), O._ptr(fv), 1)
    adv = fv.copy()
    L.or_adv_tra_ver_qr4c(s, O._ptr(f.w), O._ptr(TAB), C.c_double(1.0), O._ptr(adv), 0)
    levI = np.arange(1, nl + 1)[None, :]
    wetI = (levI >= mesh.ulevels_nod2D[:, None]) & (levI <= mesh.nlevels_nod2D[:, None])
    report["ADv"] = np.array_equal(ctx.debug_fetch("ADv")[wetI], adv[wetI])
    om.do_oce_adv_tra(f, cfg, T, TAB)
    report["LO"] = np.array_equal(ctx.debug_fetch("LO")[wet], w["fct_LO"][wet])
    report["R+"] = np.array_equal(ctx.debug_fetch("bmax")[wet], w["fct_plus"][wet])
    report["R-"] = np.array_equal(ctx.debug_fetch("bmin")[wet], w["fct_minus"][wet])
    report["dttf_h"] = np.array_equal(dh[wet], w["del_ttf_advhoriz"][wet])
    report["dttf_v"] = np.array_equal(dv[wet], w["del_ttf_advvert"][wet])
    assert all(report.values()), report
