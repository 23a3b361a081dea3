"""Diffusion of diff_tracers_ale on the GPU, through the C ABI, against the oracle.

diff_part_hor_redi (Redi off) and diff_ver_part_expl_ale alone: FP64, bit for bit.  Whole
steps with a horizontal diffusivity and with tracers on explicit vertical diffusion: FP64 bit
for bit over several steps; FP32 normwise error <= 1e-5 against the FP64 oracle started from
the same (FP32-rounded) state; the uneven-instance batch equal to the contexts stepped alone.
"""
import dataclasses

import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import perturbed_old, wet_mask
from tests.test_oracle import _ki

pytestmark = pytest.mark.gpu

MESHES = [("channel_seamount", "channel"), ("sphere_small", "sphere"), ("basin_irregular", "basin")]


def _setup(mesh, kind, ntr, seed=3):
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=seed, dt=600.0))
    tr = M.make_tracers(mesh, kind, ntr=ntr, seed=seed + 1)
    return f, tr


@pytest.mark.parametrize("meshname,kind", MESHES)
def test_diff_hor_bitwise(meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    f, tr = _setup(mesh, kind, 1)
    T = np.ascontiguousarray(tr[0], dtype=np.float64)
    om = O.OracleMesh(mesh)
    # the oracle's element gradients of T (init_tracers_AB computes them)
    om.init_tracers_AB(O.cfg_struct(), T.copy(), np.zeros_like(T), T.copy())
    trxy = om.work["tr_xy"].copy()
    Ki = _ki(mesh, 2e5)
    rng = np.random.default_rng(7)
    d0 = np.ascontiguousarray(rng.standard_normal(T.shape) * 1e-3)
    want = d0.copy()
    om.diff_part_hor_redi(600.0, Ki, trxy, want)
    ctx = G.Context(mesh, G.PREC_FP64)
    got = d0.copy()
    ctx.diff_hor(600.0, Ki, T, got)
    assert np.array_equal(got, want)
    assert np.abs(got - d0).max() > 0


@pytest.mark.parametrize("meshname,kind", MESHES)
def test_diff_ver_expl_bitwise(meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    f, tr = _setup(mesh, kind, 1)
    T = np.ascontiguousarray(tr[0], dtype=np.float64)
    rng = np.random.default_rng(8)
    flux = np.ascontiguousarray(rng.standard_normal(mesh.nod2D) * 1e-4)
    d0 = np.ascontiguousarray(rng.standard_normal(T.shape) * 1e-3)
    om = O.OracleMesh(mesh)
    ctx = G.Context(mesh, G.PREC_FP64)
    for fl in (flux, None):
        want = d0.copy()
        om.diff_ver_part_expl_ale(600.0, f.Kv, fl, T, want)
        got = d0.copy()
        ctx.diff_ver_expl(600.0, f.Kv, fl, T, got)
        assert np.array_equal(got, want), fl is None


def test_diff_entry_points_need_fp64(channel_small):
    mesh = channel_small
    ctx = G.Context(mesh, G.PREC_FP32)
    T = np.zeros((mesh.nod2D, mesh.nl - 1))
    with pytest.raises(G.FesomGpuError):
        ctx.diff_hor(600.0, _ki(mesh), T, T.copy())
    with pytest.raises(G.FesomGpuError):
        ctx.diff_ver_expl(600.0, np.zeros((mesh.nod2D, mesh.nl)), None, T, T.copy())


@pytest.mark.parametrize("meshname,kind", MESHES)
def test_fp64_step_with_diffusion_bitwise(meshname, kind, request):
    """Three whole steps: tracer 1 implicit, tracer 2 explicit vertical diffusion, both with
    horizontal diffusion; then horizontal diffusion switched off again."""
    mesh = request.getfixturevalue(meshname)
    f, tr = _setup(mesh, kind, 2)
    Ki = _ki(mesh, 2e5)
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
        ki = Ki if step < 3 else None
        if step == 3:
            ctx.set_hdiff(None)
        for k in range(2):
            om.tracer_step_ex(f, ocfgs[k], To[k], np.zeros_like(To[k]), Oo[k], Ki=ki)
        ctx.tracer_step(f, gcfgs, Tg, Og)
        for k in range(2):
            assert np.array_equal(Tg[k], To[k]), f"step {step} tracer {k}"
            assert np.array_equal(Og[k], Oo[k])


def _fp32_run(mesh, kind, ivd, Ki, steps, ab=2, seed=3):
    ntr = len(ivd)
    f, tr = _setup(mesh, kind, ntr, seed)
    cfgs = []
    for k in range(ntr):
        c = G.tra_cfg("MUSCL", "QR4C", "FCT", 0.0, 1.0, ab_order=ab, id=k + 1)
        c.i_vert_diff = ivd[k]
        cfgs.append(c)
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=ntr)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f)
    if Ki is not None:
        ctx.set_hdiff(Ki)
    T64 = []
    for k in range(ntr):
        T = tr[k].astype(np.float32).astype(np.float64)
        ctx.tracer_upload(k, T, np.repeat(T[..., None], ab - 1, axis=-1) if ab == 3 else T)
        T64.append(T.copy())
    return f, ctx, T64


@pytest.mark.parametrize("meshname,kind", MESHES)
@pytest.mark.parametrize("hdiff", [True, False])
def test_fp32_step_with_diffusion_vs_oracle(meshname, kind, hdiff, request):
    mesh = request.getfixturevalue(meshname)
    ivd = [1, 0, 1, 0]
    Ki = _ki(mesh, 2e5) if hdiff else None
    f, ctx, T64 = _fp32_run(mesh, kind, ivd, Ki, 3)
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    O64 = [t.copy() for t in T64]
    ocfgs = [O.cfg_struct("MUSCL", "QR4C", "FCT", 0.0, 1.0, i_vert_diff=v) for v in ivd]
    for step in range(3):
        ctx.run_steps(f.dt, 1, use_graph=(step == 1))
        for k in range(len(ivd)):
            om.tracer_step_ex(f, ocfgs[k], T64[k], np.zeros_like(T64[k]), O64[k], Ki=Ki)
    for k in range(len(ivd)):
        v, _ = ctx.tracer_download(k)
        err = np.abs(v[wet] - T64[k][wet]).max() / np.abs(T64[k][wet]).max()
        assert err <= 1e-5, (k, err)
    assert ctx.status() == 0


def test_fp32_horizontal_diffusion_changes_the_step(sphere_small):
    """A diffusion number of about 0.01 moves the FP32 result by far more than round-off:
    the term is not silently dropped."""
    mesh = sphere_small
    outs = []
    for Ki in (None, _ki(mesh, 2e5)):
        f, ctx, _ = _fp32_run(mesh, "sphere", [1, 1], Ki, 1)
        ctx.run_steps(f.dt, 1, use_graph=False)
        outs.append(ctx.tracer_download(0)[0])
    wet = wet_mask(mesh)
    d = np.abs(outs[1][wet] - outs[0][wet]).max() / np.abs(outs[0][wet]).max()
    assert d > 1e-4


def test_fp32_diffusion_content(channel_seamount):
    """Horizontal diffusion moves content between nodes only: with no flow, no surface flux
    and no vertical mixing, the layer contents stay put to FP32 round-off."""
    mesh = channel_seamount
    f, tr = _setup(mesh, "channel", 1)
    f0 = M.Forcing(uv=np.zeros_like(f.uv), w=np.zeros_like(f.w), w_e=np.zeros_like(f.w_e),
                   w_i=np.zeros_like(f.w_i), Kv=np.zeros_like(f.Kv), bc_surface=None, dt=f.dt)
    # thickness fixed in time, so that the content is sum T hnode areasvol before and after
    m = dataclasses.replace(mesh, hnode_new=mesh.hnode.copy())
    ctx = G.Context(m, G.PREC_FP32, max_tracers=1)
    ctx.state_setup([G.tra_cfg(id=1)])
    ctx.forcing_upload(f0)
    ctx.set_hdiff(_ki(m, 2e5))
    T = tr[0].astype(np.float32)
    ctx.tracer_upload(0, T, T)
    c0 = ctx.content()[0]
    ctx.run_steps(f.dt, 3, use_graph=True)
    c1 = ctx.content()[0]
    assert abs(c1 - c0) <= 1e-5 * abs(c0)
    v, _ = ctx.tracer_download(0)
    wet = wet_mask(m)
    assert np.abs(v[wet] - T[wet]).max() > 0


def test_batch_with_diffusion_equals_alone(channel_seamount, sphere_small):
    """Instances with horizontal diffusion and explicit vertical diffusion step in one batch
    as they do alone (FP32 round-off: the two builds contract products differently)."""
    runs = []
    for batched in (False, True):
        ctxs, f = [], []
        for mesh, kind, ivd, Ki in ((channel_seamount, "channel", [1, 0], _ki(channel_seamount, 2e5)),
                                    (sphere_small, "sphere", [0, 1, 1], None)):
            ff, ctx, _ = _fp32_run(mesh, kind, ivd, Ki, 1)
            ctxs.append(ctx)
            f.append(ff)
        if batched:
            b = G.Batch(ctxs)
            b.run_steps(600.0, 3, use_graph=True)
            b.close()
        else:
            for c in ctxs:
                c.run_steps(600.0, 3, use_graph=True)
        runs.append([[c.tracer_download(k)[0] for k in range(c.ntr)] for c in ctxs])
    for i in range(2):
        for k in range(len(runs[0][i])):
            a, b = runs[0][i][k], runs[1][i][k]
            assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max(), (i, k)
