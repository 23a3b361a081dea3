"""Redi (isoneutral) diffusion on the GPU, through the C ABI, against the oracle.

The tapered neutral slopes are an input (slope_tapered(3, nl-1, nod2D)).  The slope terms of
diff_part_hor_redi, diff_ver_part_redi_expl and the K33 of the implicit solve alone: FP64 bit
for bit.  Whole steps with Redi: FP64 bit for bit over several steps (implicit and explicit
vertical diffusion, Redi switched off again); FP32 normwise error <= 1e-5 against the FP64
oracle from the same FP32-rounded state; rigid-lid content of both forms.
"""
import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import perturbed_old, wet_mask
from tests.test_oracle import _ki

pytestmark = pytest.mark.gpu

MESHES = [("channel_seamount", "channel"), ("sphere_small", "sphere"), ("basin_irregular", "basin")]
KH = 2e5


def _slopes(mesh):
    return M.make_slopes(mesh, smax=5e-3, s_cr=4e-3)


@pytest.mark.parametrize("meshname,kind", MESHES)
def test_redi_routines_bitwise(meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0], dtype=np.float64)
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    om = O.OracleMesh(mesh)
    om.init_tracers_AB(O.cfg_struct(), T.copy(), np.zeros_like(T), T.copy())
    trxy = om.work["tr_xy"].copy()
    trz = np.zeros((mesh.nod2D, mesh.nl))
    om.tracer_gradient_z(T, trz)
    Ki, S = _ki(mesh, KH), _slopes(mesh)
    rng = np.random.default_rng(7)
    d0 = np.ascontiguousarray(rng.standard_normal(T.shape) * 1e-3)
    ctx = G.Context(mesh, G.PREC_FP64)
    want = d0.copy()
    om.diff_part_hor_redi(600.0, Ki, trxy, want, slope=S, tr_z=trz)
    got = d0.copy()
    ctx.diff_hor(600.0, Ki, T, got, slope=S)
    assert np.array_equal(got, want)
    plain = d0.copy()
    ctx.diff_hor(600.0, Ki, T, plain)
    assert np.abs(got - plain).max() > 0
    want = d0.copy()
    om.diff_ver_part_redi_expl(600.0, Ki, S, trxy, want)
    got = d0.copy()
    ctx.diff_ver_redi_expl(600.0, Ki, S, T, got)
    assert np.array_equal(got, want)
    assert np.abs(got - d0).max() > 0
    K33 = ctx.redi_k33(f.Kv, Ki, S)
    assert np.array_equal(K33, om.redi_k33(f.Kv, Ki, S))


@pytest.mark.parametrize("meshname,kind", MESHES)
def test_fp64_step_with_redi_bitwise(meshname, kind, request):
    """Three steps with Redi (tracer 1 implicit, tracer 2 explicit vertical diffusion, new
    slopes each step), then one with Redi off."""
    mesh = request.getfixturevalue(meshname)
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    tr = M.make_tracers(mesh, kind, ntr=2, seed=4)
    Ki = _ki(mesh, KH)
    om = O.OracleMesh(mesh)
    ivd = [1, 0]
    ocfgs = [O.cfg_struct("MUSCL", "QR4C", "FCT", 0.0, 1.0, i_vert_diff=v) for v in ivd]
    gcfgs = []
    for k in range(2):
        c = G.tra_cfg("MUSCL", "QR4C", "FCT", 0.0, 1.0, id=k + 1)
        c.i_vert_diff = ivd[k]
        gcfgs.append(c)
    ctx = G.Context(mesh, G.PREC_FP64, max_tracers=2)
    ctx.set_hdiff(Ki)
    rng = np.random.default_rng(2)
    To = [np.array(t, copy=True) for t in tr]
    Oo = [perturbed_old(t, rng) for t in To]
    Tg = [t.copy() for t in To]
    Og = [o.copy() for o in Oo]
    for step in range(4):
        S = M.make_slopes(mesh, seed=20 + step, smax=5e-3, s_cr=4e-3) if step < 3 else None
        ctx.set_redi(S)
        for k in range(2):
            om.tracer_step_ex(f, ocfgs[k], To[k], np.zeros_like(To[k]), Oo[k], Ki=Ki, slope=S)
        ctx.tracer_step(f, gcfgs, Tg, Og)
        for k in range(2):
            assert np.array_equal(Tg[k], To[k]), f"step {step} tracer {k}"
            assert np.array_equal(Og[k], Oo[k])


def test_redi_needs_the_horizontal_diffusivity(channel_small):
    mesh = channel_small
    for prec in (G.PREC_FP64, G.PREC_FP32):
        ctx = G.Context(mesh, prec)
        with pytest.raises(G.FesomGpuError):
            ctx.set_redi(_slopes(mesh))
        ctx.set_hdiff(_ki(mesh))
        ctx.set_redi(_slopes(mesh))
        ctx.set_redi(None)


def _fp32_ctx(mesh, kind, ivd, S):
    ntr = len(ivd)
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    tr = M.make_tracers(mesh, kind, ntr=ntr, seed=4)
    cfgs = []
    for k in range(ntr):
        c = G.tra_cfg("MUSCL", "QR4C", "FCT", 0.0, 1.0, id=k + 1)
        c.i_vert_diff = ivd[k]
        cfgs.append(c)
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=ntr)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f)
    ctx.set_hdiff(_ki(mesh, KH))
    if S is not None:
        ctx.set_redi(S)
    T64 = []
    for k in range(ntr):
        T = tr[k].astype(np.float32).astype(np.float64)
        ctx.tracer_upload(k, T, T)
        T64.append(T.copy())
    return f, ctx, T64


@pytest.mark.parametrize("meshname,kind", MESHES)
def test_fp32_step_with_redi_vs_oracle(meshname, kind, request):
    """Three FP32 steps with Redi against the FP64 oracle: normwise error <= 1e-5; and the Redi
    part alone (the step with Redi minus the step without, FP32 against FP64) within 5 % of its
    size plus the FP32 error of the two runs, so the isoneutral terms are neither dropped nor off
    by a factor."""
    mesh = request.getfixturevalue(meshname)
    ivd = [1, 0, 1, 0, 1]
    S = _slopes(mesh)
    Ki = _ki(mesh, KH)
    f, ctx, T64 = _fp32_ctx(mesh, kind, ivd, S)
    _, off, _ = _fp32_ctx(mesh, kind, ivd, None)
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    O64 = [t.copy() for t in T64]
    P64 = [t.copy() for t in T64]   # the oracle without Redi
    Q64 = [t.copy() for t in T64]
    ocfgs = [O.cfg_struct("MUSCL", "QR4C", "FCT", 0.0, 1.0, i_vert_diff=v) for v in ivd]
    for step in range(3):
        ctx.run_steps(f.dt, 1, use_graph=(step == 1))
        off.run_steps(f.dt, 1, use_graph=(step == 1))
        for k in range(len(ivd)):
            om.tracer_step_ex(f, ocfgs[k], T64[k], np.zeros_like(T64[k]), O64[k], Ki=Ki, slope=S)
            om.tracer_step_ex(f, ocfgs[k], P64[k], np.zeros_like(P64[k]), Q64[k], Ki=Ki)
    for k in range(len(ivd)):
        v = ctx.tracer_download(k)[0][wet]
        w = off.tracer_download(k)[0][wet]
        scale = np.abs(T64[k][wet]).max()
        err = np.abs(v - T64[k][wet]).max() / scale
        assert err <= 1e-5, (k, err)
        d64 = T64[k][wet] - P64[k][wet]
        d32 = v - w
        floor = np.abs(v - T64[k][wet]).max() + np.abs(w - P64[k][wet]).max()
        assert np.abs(d64).max() > 1e-6 * scale, k
        assert np.abs(d32 - d64).max() <= 0.05 * np.abs(d64).max() + floor, \
            (k, np.abs(d32 - d64).max(), np.abs(d64).max(), floor)
    assert ctx.status() == 0


@pytest.mark.parametrize("prec", [G.PREC_FP64, G.PREC_FP32])
def test_redi_rigid_lid_content(channel_seamount, prec):
    """Rigid lid, no surface flux: the isoneutral terms move tracer between nodes and levels
    only; the content drifts by round-off (FP64) or by the FP32 storage rounding (FP32)."""
    mesh = channel_seamount
    f = O.ensure_f64(M.make_forcing(mesh, "channel", seed=3, dt=600.0, surface_w_zero=True))
    tr = M.make_tracers(mesh, "channel", ntr=2, seed=4)
    cfgs = [G.tra_cfg("MUSCL", "QR4C", "FCT", 0.0, 1.0, id=k + 1) for k in range(2)]
    ctx = G.Context(mesh, prec, max_tracers=2)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f if prec == G.PREC_FP64 else f)
    ctx.set_hdiff(_ki(mesh, KH))
    ctx.set_redi(_slopes(mesh))
    for k in range(2):
        T = tr[k].astype(np.float32).astype(np.float64)
        ctx.tracer_upload(k, T, T)
    c0 = ctx.content()
    ctx.run_steps(f.dt, 5, use_graph=True)
    c1 = ctx.content()
    tol = 1e-13 if prec == G.PREC_FP64 else 1e-8
    for k in range(2):
        assert abs(c1[k] - c0[k]) <= tol * abs(c0[k]), (k, c1[k], c0[k])
    assert ctx.status() == 0
