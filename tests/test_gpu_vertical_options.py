"""The vertical schemes CDIFF and PPM and the split vertical velocity (w = w_e + w_i, w_i
implicit) on the GPU, through the C ABI: FP64 bit for bit with the oracle (the routine
drop-ins and whole steps), FP32 within 1e-5 normwise of the FP64 oracle."""
import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import perturbed_old, wet_mask

pytestmark = pytest.mark.gpu

MESHES = [("channel_seamount", "channel"), ("sphere_small", "sphere"), ("basin_irregular", "basin")]
# (hor, ver, lim, wsplit)
OPTIONS = [("MUSCL", "CDIFF", "FCT", False), ("MFCT", "PPM", "FCT", False), ("UPW1", "PPM", "NON", False),
           ("MUSCL", "CDIFF", "NON", False), ("MUSCL", "QR4C", "FCT", True), ("MFCT", "PPM", "FCT", True),
           ("MUSCL", "CDIFF", "NON", True), ("UPW1", "UPW1", "NON", True)]
IDS = ["-".join(map(str, o)) for o in OPTIONS]


def _forcing(mesh, kind, wsplit):
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    return M.split_vertical_velocity(mesh, f, maxcfl=0.01) if wsplit else f


@pytest.mark.parametrize("opt", OPTIONS, ids=IDS)
@pytest.mark.parametrize("meshname,kind", MESHES)
def test_adv_tra_bitwise(opt, meshname, kind, request):
    hor, ver, lim, wsplit = opt
    mesh = request.getfixturevalue(meshname)
    f = _forcing(mesh, kind, wsplit)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0])
    rng = np.random.default_rng(11)
    TAB = np.ascontiguousarray(T * (1.0 + 1e-3 * rng.standard_normal(T.shape)))
    om = O.OracleMesh(mesh)
    ocfg = O.cfg_struct(hor, ver, lim, wsplit=wsplit)
    om.init_tracers_AB(ocfg, T.copy(), np.zeros_like(T), T.copy())
    om.do_oce_adv_tra(f, ocfg, T, TAB)
    ctx = G.Context(mesh, G.PREC_FP64)
    ctx.set_wsplit(wsplit)
    dh, dv = ctx.adv_tra(f, G.tra_cfg(hor, ver, lim), T, TAB)
    wet = wet_mask(mesh)
    assert np.array_equal(dh[wet], om.work["del_ttf_advhoriz"][wet])
    assert np.array_equal(dv[wet], om.work["del_ttf_advvert"][wet])


@pytest.mark.parametrize("meshname,kind", MESHES)
def test_vdiff_wimpl_bitwise(meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    f = _forcing(mesh, kind, True)
    f.bc_surface = np.linspace(-2e-3, 1e-3, mesh.nod2D)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=2)[0])
    om = O.OracleMesh(mesh)
    want = T.copy()
    om.diff_ver_part_impl_ale(f, want, wimpl=True)
    ctx = G.Context(mesh, G.PREC_FP64)
    got = T.copy()
    ctx.vdiff_impl(f, G.tra_cfg("MUSCL", "QR4C", "NON"), got, wimpl=True)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("opt", OPTIONS, ids=IDS)
@pytest.mark.parametrize("meshname,kind", MESHES)
def test_fp64_step_bitwise(opt, meshname, kind, request):
    """Three whole steps of two tracers (AB2 and AB3 contexts alike through the same path)."""
    hor, ver, lim, wsplit = opt
    mesh = request.getfixturevalue(meshname)
    f = _forcing(mesh, kind, wsplit)
    tr = M.make_tracers(mesh, kind, ntr=2, seed=4)
    om = O.OracleMesh(mesh)
    ocfg = O.cfg_struct(hor, ver, lim, wsplit=wsplit)
    gcfgs = [G.tra_cfg(hor, ver, lim, id=k + 1) for k in range(2)]
    ctx = G.Context(mesh, G.PREC_FP64, max_tracers=2)
    ctx.set_wsplit(wsplit)
    rng = np.random.default_rng(2)
    To = [np.array(t, copy=True) for t in tr]
    Oo = [perturbed_old(t, rng) for t in To]
    Tg = [t.copy() for t in To]
    Og = [o.copy() for o in Oo]
    for step in range(3):
        for k in range(2):
            om.tracer_step(f, ocfg, To[k], np.zeros_like(To[k]), Oo[k])
        ctx.tracer_step(f, gcfgs, Tg, Og)
        for k in range(2):
            assert np.array_equal(Tg[k], To[k]), f"step {step} tracer {k}"
    assert ctx.status() == 0


@pytest.mark.parametrize("meshname,kind", MESHES)
@pytest.mark.parametrize("wsplit", [False, True])
def test_fp32_step_vs_oracle(meshname, kind, wsplit, request):
    """All the options in one FP32 launch group (per-tracer switches), 3 steps."""
    mesh = request.getfixturevalue(meshname)
    f = _forcing(mesh, kind, wsplit)
    opts = [o for o in OPTIONS if o[3] == wsplit]
    ntr = len(opts)
    tr = M.make_tracers(mesh, kind, ntr=ntr, seed=4)
    cfgs = [G.tra_cfg(h, v, l, id=k + 1) for k, (h, v, l, _) in enumerate(opts)]
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=ntr)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f)
    ctx.set_wsplit(wsplit)
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    T64 = []
    for k in range(ntr):
        T = tr[k].astype(np.float32).astype(np.float64)
        ctx.tracer_upload(k, T, T)
        T64.append(T.copy())
    O64 = [t.copy() for t in T64]
    for step in range(3):
        ctx.run_steps(f.dt, 1, use_graph=(step > 0))
        for k, (h, v, l, ws) in enumerate(opts):
            om.tracer_step(f, O.cfg_struct(h, v, l, wsplit=ws), T64[k], np.zeros_like(T64[k]), O64[k])
    for k in range(ntr):
        v, _ = ctx.tracer_download(k)
        err = np.abs(v[wet] - T64[k][wet]).max() / np.abs(T64[k][wet]).max()
        assert err <= 1e-5, (opts[k], err)
    assert ctx.status() == 0


def test_split_velocity_changes_the_step(channel_seamount):
    """The split path is taken: with w_i != 0 the FP32 result moves well beyond round-off."""
    mesh = channel_seamount
    outs = []
    for ws in (False, True):
        f = _forcing(mesh, "channel", True)
        T = M.make_tracers(mesh, "channel", ntr=1, seed=4)[0].astype(np.float32)
        ctx = G.Context(mesh, G.PREC_FP32, max_tracers=1)
        ctx.state_setup([G.tra_cfg("MUSCL", "QR4C", "FCT")])
        ctx.forcing_upload(f)
        ctx.set_wsplit(ws)
        ctx.tracer_upload(0, T, T)
        ctx.run_steps(f.dt, 2, use_graph=False)
        outs.append(ctx.tracer_download(0)[0])
    wet = wet_mask(mesh)
    assert np.abs(outs[1][wet] - outs[0][wet]).max() > 1e-4 * np.abs(outs[0][wet]).max()


def test_batch_with_vertical_options_equals_alone(channel_seamount, sphere_small):
    """A batch of an instance with PPM and CDIFF tracers and an instance with the split
    vertical velocity steps as the instances do alone (FP32 rounding: the batch kernels are
    separate compilations)."""
    setups = [(channel_seamount, "channel", False, [("MFCT", "PPM", "FCT"), ("MUSCL", "CDIFF", "NON")]),
              (sphere_small, "sphere", True, [("MUSCL", "QR4C", "FCT"), ("UPW1", "PPM", "NON"),
                                              ("MUSCL", "CDIFF", "NON")])]
    runs = []
    for batched in (False, True):
        ctxs = []
        for mesh, kind, ws, opts in setups:
            f = _forcing(mesh, kind, ws)
            tr = M.make_tracers(mesh, kind, ntr=len(opts), seed=4)
            ctx = G.Context(mesh, G.PREC_FP32, max_tracers=len(opts))
            ctx.state_setup([G.tra_cfg(h, v, l, id=k + 1) for k, (h, v, l) in enumerate(opts)])
            ctx.forcing_upload(f)
            ctx.set_wsplit(ws)
            for k in range(len(opts)):
                t32 = tr[k].astype(np.float32)
                ctx.tracer_upload(k, t32, t32)
            ctxs.append(ctx)
        if batched:
            b = G.Batch(ctxs)
            b.run_steps(600.0, 3, use_graph=True)
            b.close()
        else:
            for c in ctxs:
                c.run_steps(600.0, 3, use_graph=True)
        runs.append([[c.tracer_download(k)[0] for k in range(c.ntr)] for c in ctxs])
        for c in ctxs:
            assert c.status() == 0
    for i in range(len(setups)):
        for k in range(len(runs[0][i])):
            a, b = runs[0][i][k], runs[1][i][k]
            assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max(), (i, k)
