"""Parity of the CUDA path (through the C ABI) with the FP64 CPU oracle.

FP64 plain form: bit-for-bit equality with the oracle (the kernels add every
sum in the reference's serial scatter order and are built without FMA
contraction).  FP32 form: max relative error per step <= 1e-5 against the
FP64 oracle started from the same state, content conserved, FCT bounds kept.
"""
import ctypes as C

import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import perturbed_old, wet_mask

pytestmark = pytest.mark.gpu

SCHEMES = [("MUSCL", "QR4C", "FCT"), ("MFCT", "QR4C", "FCT"), ("UPW1", "UPW1", "FCT"),
           ("MUSCL", "QR4C", "NON"), ("UPW1", "QR4C", "NON"), ("MFCT", "UPW1", "FCT")]


def _setup(mesh, kind, seed=3, ntr=2, surface_w_zero=False):
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=seed, dt=600.0, surface_w_zero=surface_w_zero))
    tr = M.make_tracers(mesh, kind, ntr=ntr, seed=seed + 1)
    return f, tr


@pytest.mark.parametrize("meshname", ["channel_small", "channel_seamount", "sphere_small", "basin_irregular"])
def test_muscl_init_matches_oracle(meshname, request):
    mesh = request.getfixturevalue(meshname)
    ctx = G.Context(mesh, G.PREC_FP64)
    om = O.OracleMesh(mesh)
    nbl, updn = ctx.muscl_init()
    assert np.array_equal(nbl, om.work["nboundary_lay"])
    assert np.array_equal(updn, om.work["edge_up_dn_tri"])


@pytest.mark.parametrize("meshname,kind", [("channel_small", "channel"), ("sphere_small", "sphere")])
@pytest.mark.parametrize("ab", [2, 3])
def test_init_tracers_ab_bitwise(meshname, kind, ab, request):
    mesh = request.getfixturevalue(meshname)
    f, tr = _setup(mesh, kind)
    rng = np.random.default_rng(7)
    T = np.ascontiguousarray(tr[0])
    old = np.ascontiguousarray(np.stack([perturbed_old(T, rng) for _ in range(ab - 1)], axis=-1))
    ocfg = O.cfg_struct(ab_order=ab)
    gcfg = G.tra_cfg(ab_order=ab)
    om = O.OracleMesh(mesh)
    o_old, o_ab = old.copy(), np.zeros_like(T)
    om.init_tracers_AB(ocfg, T.copy(), o_ab, o_old)
    ctx = G.Context(mesh, G.PREC_FP64)
    g_old, g_ab = old.copy(), np.zeros_like(T)
    ctx.init_tracers_ab(gcfg, T.copy(), g_ab, g_old)
    assert np.array_equal(g_ab, o_ab)
    assert np.array_equal(g_old, o_old)


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("sphere_small", "sphere"),
                                           ("pi_cavity_file_mesh", "sphere")])
def test_tracer_gradient_z_bitwise(meshname, kind, request):
    """fesom_gpu_tracer_gradient_z equals the oracle bit for bit, the interfaces outside each
    column (above a cavity's first wet level, below the bottom) keeping the caller's values."""
    mesh = request.getfixturevalue(meshname)
    _, tr = _setup(mesh, kind)
    T = np.ascontiguousarray(tr[0])
    trz0 = np.full((mesh.nod2D, mesh.nl), 7.25)
    want = trz0.copy()
    O.OracleMesh(mesh).tracer_gradient_z(T, want)
    ctx = G.Context(mesh, G.PREC_FP64)
    got = ctx.tracer_gradient_z(T, trz0.copy())
    assert np.array_equal(got, want)
    assert (want == 7.25).any()  # entries outside the columns exist and were kept


@pytest.mark.parametrize("scheme", SCHEMES, ids=["-".join(s) for s in SCHEMES])
@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("sphere_small", "sphere"),
                                           ("basin_irregular", "basin")])
def test_adv_tra_bitwise(scheme, meshname, kind, request):
    """do_oce_adv_tra: del_ttf_advhoriz / del_ttf_advvert equal the oracle's bit for bit."""
    mesh = request.getfixturevalue(meshname)
    hor, ver, lim = scheme
    f, tr = _setup(mesh, kind)
    rng = np.random.default_rng(11)
    T = np.ascontiguousarray(tr[0])
    TAB = np.ascontiguousarray(T * (1.0 + 1e-3 * rng.standard_normal(T.shape)))
    om = O.OracleMesh(mesh)
    ocfg = O.cfg_struct(hor, ver, lim, ph=0.0, pv=1.0)
    om.init_tracers_AB(ocfg, T.copy(), np.zeros_like(T), T.copy())  # zero del_ttf*, gradients of T
    om.do_oce_adv_tra(f, ocfg, T, TAB)
    ctx = G.Context(mesh, G.PREC_FP64)
    dh, dv = ctx.adv_tra(f, G.tra_cfg(hor, ver, lim, ph=0.0, pv=1.0), T, TAB)
    wet = wet_mask(mesh)
    assert np.array_equal(dh[wet], om.work["del_ttf_advhoriz"][wet])
    assert np.array_equal(dv[wet], om.work["del_ttf_advvert"][wet])


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("sphere_small", "sphere")])
def test_vdiff_bitwise(meshname, kind, request):
    mesh = request.getfixturevalue(meshname)
    f, tr = _setup(mesh, kind)
    f.bc_surface = np.linspace(-1e-3, 1e-3, mesh.nod2D)
    T = np.ascontiguousarray(tr[1])
    om = O.OracleMesh(mesh)
    To = T.copy()
    om.diff_ver_part_impl_ale(f, To)
    ctx = G.Context(mesh, G.PREC_FP64)
    Tg = T.copy()
    ctx.vdiff_impl(f, G.tra_cfg(), Tg)
    assert np.array_equal(Tg, To)


@pytest.mark.parametrize("meshname,kind", [("channel_small", "channel"), ("channel_seamount", "channel"),
                                           ("sphere_small", "sphere"), ("basin_irregular", "basin")])
def test_tracer_step_bitwise_multi_step(meshname, kind, request):
    """Whole per-tracer body (AB2, MUSCL+QR4C+FCT, T*, implicit diffusion), 3 steps, 2 tracers."""
    mesh = request.getfixturevalue(meshname)
    f, tr = _setup(mesh, kind)
    om = O.OracleMesh(mesh)
    ctx = G.Context(mesh, G.PREC_FP64, max_tracers=2)
    ocfg = O.cfg_struct("MUSCL", "QR4C", "FCT", 0.0, 1.0)
    gcfgs = [G.tra_cfg("MUSCL", "QR4C", "FCT", 0.0, 1.0, id=1), G.tra_cfg("MUSCL", "QR4C", "FCT", 0.0, 1.0, id=2)]
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
            assert np.array_equal(Og[k], Oo[k])


def test_device_resident_graph_matches_host_calls(channel_seamount):
    """run_steps (CUDA graph replay) equals the same steps through the host-array entry point."""
    mesh = channel_seamount
    f, tr = _setup(mesh, "channel")
    cfgs = [G.tra_cfg(id=1), G.tra_cfg(id=2)]
    a = G.Context(mesh, G.PREC_FP64, max_tracers=2)
    Ta = [np.array(t, copy=True) for t in tr]
    Oa = [t.copy() for t in Ta]
    for _ in range(4):
        a.tracer_step(f, cfgs, Ta, Oa)
    b = G.Context(mesh, G.PREC_FP64, max_tracers=2)
    b.state_setup(cfgs)
    b.forcing_upload(f)
    for k in range(2):
        b.tracer_upload(k, np.array(tr[k], copy=True), np.array(tr[k], copy=True))
    b.run_steps(f.dt, 4, use_graph=True)
    for k in range(2):
        v, o = b.tracer_download(k)
        assert np.array_equal(v, Ta[k])
        assert np.array_equal(o, Oa[k])


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("sphere_small", "sphere"),
                                           ("basin_irregular", "basin")])
def test_fp32_error_vs_fp64_oracle(meshname, kind, request):
    """FP32 form, one step from the same state: error against the FP64 oracle <= 1e-5,
    normwise (max |dT| / max |T|) for every tracer and pointwise relative for T and S.
    (Pointwise relative error of a lognormal tracer is ill-conditioned where a small
    value sits between large neighbours: inflow and outflow nearly cancel.)"""
    mesh = request.getfixturevalue(meshname)
    ntr = 4
    f, tr = _setup(mesh, kind, ntr=ntr)
    cfgs = [G.tra_cfg(id=k + 1) for k in range(ntr)]
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=ntr)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f)
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    ocfg = O.cfg_struct()
    for k in range(ntr):
        T32 = tr[k].astype(np.float32)
        ctx.tracer_upload(k, T32, T32)
    ctx.run_steps(f.dt, 1, use_graph=False)
    for k in range(ntr):
        T64 = tr[k].astype(np.float32).astype(np.float64)
        O64 = T64.copy()
        om.tracer_step(f, ocfg, T64, np.zeros_like(T64), O64)
        v, _ = ctx.tracer_download(k)
        err = np.abs(v[wet] - T64[wet])
        assert err.max() / np.abs(T64[wet]).max() <= 1e-5, (k, err.max())
        if k < 2:
            rel = err / np.maximum(np.abs(T64[wet]), 1e-30)
            assert rel.max() <= 1e-5, (k, rel.max())
    assert ctx.status() == 0


@pytest.mark.parametrize("prec,tol", [(G.PREC_FP64, 1e-12), (G.PREC_FP32, 3e-8)])
def test_content_conservation(channel_seamount, prec, tol):
    """Rigid lid (w = 0 at the surface), linfs: sum T*hnode_new*areasvol is conserved over 5
    steps, FP64 to round-off; FP32 to the rounding of FP32 storage (increments of the vertical
    diffusion below half an ulp of the stored value are lost, with the same sign over most
    columns: measured -6.2e-9 for T, -5.6e-10 for S; the bound leaves a factor 5)."""
    mesh = channel_seamount
    f, tr = _setup(mesh, "channel", surface_w_zero=True)
    cfgs = [G.tra_cfg(id=1), G.tra_cfg(id=2)]
    ctx = G.Context(mesh, prec, max_tracers=2)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f)
    for k in range(2):
        ctx.tracer_upload(k, np.ascontiguousarray(tr[k]), np.ascontiguousarray(tr[k]))
    c0 = ctx.content()
    ctx.run_steps(f.dt, 5)
    c1 = ctx.content()
    assert np.all(np.abs(c1 - c0) / np.abs(c0) <= tol), (c0, c1)


def test_lognormal_positivity_fp32(sphere_small):
    mesh = sphere_small
    ntr = 6
    f, tr = _setup(mesh, "sphere", ntr=ntr)
    cfgs = [G.tra_cfg(id=100 + k) for k in range(ntr)]
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=ntr)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f)
    for k in range(ntr):
        ctx.tracer_upload(k, tr[k].astype(np.float32), tr[k].astype(np.float32))
    ctx.run_steps(f.dt, 5)
    wet = wet_mask(mesh)
    for k in range(2, ntr):
        v, _ = ctx.tracer_download(k, dtype=np.float32)
        assert v[wet].min() >= 0.0


def test_errors_are_reported(channel_small):
    ctx = G.Context(channel_small, G.PREC_FP64)
    f, tr = _setup(channel_small, "channel")
    T = np.ascontiguousarray(tr[0])
    unknown = G.tra_cfg()
    unknown.adv_ver = 7
    with pytest.raises(G.FesomGpuError) as e:
        ctx.adv_tra(f, unknown, T, T)
    assert e.value.rc == 2
    bad = G.tra_cfg()
    bad.ab_order = 4
    with pytest.raises(G.FesomGpuError):
        ctx.adv_tra(f, bad, T, T)
    with pytest.raises(G.FesomGpuError) as e:
        ctx.run_steps(600.0, 1)
    assert e.value.rc == 8


FP32_SCHEMES = [("MUSCL", "QR4C", "FCT", 2), ("MFCT", "UPW1", "FCT", 3), ("UPW1", "QR4C", "NON", 2),
                ("MUSCL", "QR4C", "NON", 3)]


@pytest.mark.parametrize("scheme", FP32_SCHEMES, ids=["-".join(map(str, s)) for s in FP32_SCHEMES])
@pytest.mark.parametrize("meshname,kind", [("sphere_small", "sphere"), ("basin_irregular", "basin")])
def test_fp32_schemes_and_ab_orders_vs_oracle(meshname, kind, scheme, request):
    """FP32 batched form, 3 steps of every scheme family and AB order, against the
    FP64 oracle started from the same (FP32-rounded) state: normwise error <= 1e-5."""
    hor, ver, lim, ab = scheme
    mesh = request.getfixturevalue(meshname)
    f, tr = _setup(mesh, kind, ntr=3)
    rng = np.random.default_rng(4)
    cfgs = [G.tra_cfg(hor, ver, lim, 0.0, 1.0, ab_order=ab, id=k + 1) for k in range(3)]
    ocfg = O.cfg_struct(hor, ver, lim, 0.0, 1.0, ab_order=ab)
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=3)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f)
    T64, O64 = [], []
    for k in range(3):
        T = tr[k].astype(np.float32).astype(np.float64)
        old = np.stack([T * (1 + 1e-3 * rng.standard_normal(T.shape)) for _ in range(ab - 1)], axis=-1)
        old = np.ascontiguousarray(old.astype(np.float32).astype(np.float64))
        ctx.tracer_upload(k, T, old)
        T64.append(T.copy())
        O64.append(old.copy())
    for step in range(3):
        ctx.run_steps(f.dt, 1, use_graph=(step % 2 == 1))
        for k in range(3):
            om.tracer_step(f, ocfg, T64[k], np.zeros_like(T64[k]), O64[k])
    for k in range(3):
        v, o = ctx.tracer_download(k)
        err = np.abs(v[wet] - T64[k][wet]).max() / np.abs(T64[k][wet]).max()
        assert err <= 1e-5, (k, err)
        # the previous time levels come back in the caller's valuesold layout
        assert np.abs(o.reshape(-1)[:8] - O64[k].reshape(-1)[:8]).max() <= 1e-5 * np.abs(O64[k]).max()
    assert ctx.status() == 0


def test_fp32_graph_replay_equals_direct_launches(channel_seamount):
    mesh = channel_seamount
    f, tr = _setup(mesh, "channel", ntr=2)
    cfgs = [G.tra_cfg(id=1), G.tra_cfg(id=2)]
    out = []
    for use_graph in (False, True):
        ctx = G.Context(mesh, G.PREC_FP32, max_tracers=2)
        ctx.state_setup(cfgs)
        ctx.forcing_upload(f)
        for k in range(2):
            ctx.tracer_upload(k, tr[k].astype(np.float32), tr[k].astype(np.float32))
        ctx.run_steps(f.dt, 5, use_graph=use_graph)
        out.append([ctx.tracer_download(k, dtype=np.float32) for k in range(2)])
        ctx.close()
    for k in range(2):
        assert np.array_equal(out[0][k][0], out[1][k][0])
        assert np.array_equal(out[0][k][1], out[1][k][1])


def test_fp32_mixed_schemes_in_one_batch(basin_irregular):
    """Tracers of different schemes, limiters and vertical-diffusion switches share one
    FP32 launch per stage; each must match the oracle run with its own configuration."""
    mesh = basin_irregular
    f, tr = _setup(mesh, "basin", ntr=4)
    specs = [("MUSCL", "QR4C", "FCT", 1), ("UPW1", "UPW1", "NON", 1), ("MFCT", "QR4C", "FCT", 0),
             ("MUSCL", "UPW1", "NON", 0)]
    cfgs, ocfgs = [], []
    for k, (hor, ver, lim, ivd) in enumerate(specs):
        c = G.tra_cfg(hor, ver, lim, 0.0, 1.0, id=k + 1)
        c.i_vert_diff = ivd
        cfgs.append(c)
        ocfgs.append(O.cfg_struct(hor, ver, lim, 0.0, 1.0, i_vert_diff=ivd))
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=4)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f)
    T64, O64 = [], []
    for k in range(4):
        T = tr[k].astype(np.float32).astype(np.float64)
        ctx.tracer_upload(k, T, T)
        T64.append(T.copy())
        O64.append(T.copy())
    for step in range(2):
        ctx.run_steps(f.dt, 1, use_graph=(step == 1))
        for k in range(4):
            om.tracer_step(f, ocfgs[k], T64[k], np.zeros_like(T64[k]), O64[k])
    for k in range(4):
        v, _ = ctx.tracer_download(k)
        err = np.abs(v[wet] - T64[k][wet]).max() / np.abs(T64[k][wet]).max()
        assert err <= 1e-5, (specs[k], err)
    assert ctx.status() == 0


@pytest.mark.parametrize("meshname,kind", [("basin_irregular", "basin"), ("sphere_small", "sphere")])
def test_fp32_stage_passes_do_not_change_results(meshname, kind, request):
    """Tracers per launch of each node stage (fesom_gpu_set_stage_tracers), the grid of the
    stage kernels (fesom_gpu_set_launch_shape) and their variant (fesom_gpu_set_stage_variant:
    gathers in registers or staged in shared memory; the implicit vertical diffusion as the
    update's per-node epilogue or as its own kernel) are performance settings.  Splits, grids and
    the place of the diffusion run the same code and give the same bits; the register and staged
    variants of a stage are separate compilations whose products may contract differently, so
    they agree to FP32 round-off."""
    mesh = request.getfixturevalue(meshname)
    f, tr = _setup(mesh, kind, ntr=7)
    cfgs = [G.tra_cfg(["MUSCL", "MFCT", "UPW1"][k % 3], ["QR4C", "UPW1", "PPM", "CDIFF"][k % 4],
                      "FCT" if k % 3 else "NON", id=k + 1) for k in range(7)]
    combos = (([0, 0, 0, 0], [0, 0, 0, 0], [1, 0, 0, 0]), ([3, 2, 5, 1], [2, 3, 1, 2], [1, 0, 0, 0]),
              ([1, 7, 2, 4], [0, 0, 0, 0], [1, 0, 0, 0]), ([3, 2, 5, 1], [0, 0, 0, 0], [0, 1, 1, 1]),
              ([1, 7, 2, 4], [1, 2, 2, 1], [0, 1, 1, 1]), ([0, 0, 0, 0], [0, 0, 0, 0], [1, 0, 0, 2]),
              ([3, 2, 5, 1], [0, 0, 0, 0], [0, 1, 1, 3]), ([3, 2, 5, 1], [2, 3, 1, 2], [1, 0, 0, 2]))
    outs = []
    for split, shape, variant in combos:
        ctx = G.Context(mesh, G.PREC_FP32, max_tracers=7)
        ctx.state_setup(cfgs)
        ctx.forcing_upload(f)
        for st, v in enumerate(split):
            ctx.set_stage_tracers(st, v)
        for st, v in enumerate(shape):
            ctx.set_launch_shape(st, v)
        for st, v in enumerate(variant):
            ctx.set_stage_variant(st, v)
        for k in range(7):
            t32 = tr[k].astype(np.float32)
            ctx.tracer_upload(k, t32, t32)
        ctx.run_steps(f.dt, 3, use_graph=True)
        outs.append([ctx.tracer_download(k, dtype=np.float32)[0] for k in range(7)])
        assert ctx.status() == 0
        ctx.close()
    # same variant: bit for bit
    for i, ref in ((1, 0), (2, 0), (4, 3), (5, 0), (6, 3), (7, 0)):
        for k in range(7):
            assert np.array_equal(outs[i][k], outs[ref][k]), (i, k)
    # other variant: FP32 round-off
    for k in range(7):
        assert np.abs(outs[3][k] - outs[0][k]).max() <= 1e-6 * np.abs(outs[0][k]).max(), k


def test_device_pointers_give_the_host_results(channel_seamount):
    """Array arguments may live in device memory (an OpenACC caller's `host_data use_device`
    addresses): the copies inside each call take their direction from the pointer, and the
    results equal those of the same calls on host arrays bit for bit."""
    torch = pytest.importorskip("torch")
    mesh = channel_seamount
    f, tr = _setup(mesh, "channel")
    T = np.ascontiguousarray(tr[0])
    cfg = G.tra_cfg()
    ctx = G.Context(mesh, G.PREC_FP64)
    # host arrays
    want_z = ctx.tracer_gradient_z(T, np.full((mesh.nod2D, mesh.nl), 3.5))
    want_v = T.copy()
    ctx.vdiff_impl(f, cfg, want_v)
    # the same calls on device arrays
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to("cuda")
    T_d, z_d = dev(T), dev(np.full((mesh.nod2D, mesh.nl), 3.5))
    kv_d, v_d = dev(f.Kv), dev(T)
    bc_d = None if f.bc_surface is None else dev(np.asarray(f.bc_surface, dtype=np.float64))
    p = lambda t: None if t is None else G._P(t.data_ptr())
    assert ctx.L.fesom_gpu_tracer_gradient_z(ctx.h, p(T_d), p(z_d)) == 0
    assert ctx.L.fesom_gpu_vdiff_impl_wi(ctx.h, float(f.dt), C.byref(cfg), p(kv_d), p(bc_d), None, p(v_d)) == 0
    torch.cuda.synchronize()
    assert np.array_equal(z_d.cpu().numpy(), want_z)
    assert np.array_equal(v_d.cpu().numpy(), want_v)


def test_autotune_keeps_the_state_and_the_results(sphere_small):
    """fesom_gpu_autotune: the chosen settings are among the candidates, the tracer state after
    tuning is the state before it bit for bit, and steps under the chosen settings agree with
    steps under the defaults to FP32 round-off (the kernel variants are separate compilations)."""
    mesh = sphere_small
    f, tr = _setup(mesh, "sphere", ntr=12)
    cfgs = [G.tra_cfg(id=k + 1) for k in range(12)]
    ctxs = []
    for tune in (False, True):
        ctx = G.Context(mesh, G.PREC_FP32, max_tracers=12)
        ctx.state_setup(cfgs)
        ctx.forcing_upload(f)
        for k in range(12):
            ctx.tracer_upload(k, tr[k].astype(np.float32), tr[k].astype(np.float32))
        if tune:
            before = [ctx.tracer_download(k, dtype=np.float32) for k in range(12)]
            res = ctx.autotune(f.dt, steps=1)
            assert res["candidates"] >= 2 and res["tuned_ms"] <= res["default_ms"]
            assert all(b in (0, 2, 4) for b in res["blocks_per_sm"])
            assert all(t in (0, 8) for t in res["stage_tracers"])
            assert all(v in (0, 1) for v in res["variant"][:3]) and res["variant"][3] in (0, 1, 2, 3)
            for k in range(12):
                v, o = ctx.tracer_download(k, dtype=np.float32)
                assert np.array_equal(v, before[k][0]) and np.array_equal(o, before[k][1])
        ctx.run_steps(f.dt, 2)
        ctxs.append(ctx)
    wet = wet_mask(mesh)
    for k in range(12):
        a = ctxs[0].tracer_download(k)[0][wet]
        b = ctxs[1].tracer_download(k)[0][wet]
        assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max(), k
    assert ctxs[1].status() == 0
