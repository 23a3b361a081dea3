"""Edge cases on the GPU, through the C ABI: the shortest columns (2 and 3 layers) under every
vertical option, FP64 bit for bit and FP32 within 1e-5 of the oracle; more tracers than one
FP32 launch group holds (64), so that a step runs two groups."""
import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import perturbed_old, wet_mask
from tests.test_edge_cases import IDS, OPTIONS

pytestmark = pytest.mark.gpu


def _forcing(mesh, ws):
    f = O.ensure_f64(M.make_forcing(mesh, "channel", seed=3, dt=600.0))
    return M.split_vertical_velocity(mesh, f, maxcfl=0.001) if ws else f


@pytest.mark.parametrize("opt", OPTIONS, ids=IDS)
def test_short_columns_fp64_bitwise(shallow_channel, opt):
    hor, ver, lim, ws = opt
    mesh = shallow_channel
    f = _forcing(mesh, ws)
    tr = M.make_tracers(mesh, "channel", ntr=2, seed=4)
    om = O.OracleMesh(mesh)
    ocfg = O.cfg_struct(hor, ver, lim, wsplit=ws)
    ctx = G.Context(mesh, G.PREC_FP64, max_tracers=2)
    ctx.set_wsplit(ws)
    rng = np.random.default_rng(2)
    To = [np.array(t, copy=True) for t in tr]
    Oo = [perturbed_old(t, rng) for t in To]
    Tg = [t.copy() for t in To]
    Og = [o.copy() for o in Oo]
    for step in range(3):
        for k in range(2):
            om.tracer_step(f, ocfg, To[k], np.zeros_like(To[k]), Oo[k])
        ctx.tracer_step(f, [G.tra_cfg(hor, ver, lim, id=k + 1) for k in range(2)], Tg, Og)
        for k in range(2):
            assert np.array_equal(Tg[k], To[k]), f"step {step} tracer {k}"
    assert ctx.status() == 0


@pytest.mark.parametrize("ws", [False, True])
def test_short_columns_fp32_vs_oracle(shallow_channel, ws):
    mesh = shallow_channel
    f = _forcing(mesh, ws)
    opts = [o for o in OPTIONS if o[3] == ws]
    n = len(opts)
    tr = M.make_tracers(mesh, "channel", ntr=n, seed=4)
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=n)
    ctx.state_setup([G.tra_cfg(h, v, l, id=k + 1) for k, (h, v, l, _) in enumerate(opts)])
    ctx.forcing_upload(f)
    ctx.set_wsplit(ws)
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    T64 = []
    for k in range(n):
        T = tr[k].astype(np.float32).astype(np.float64)
        ctx.tracer_upload(k, T, T)
        T64.append(T.copy())
    O64 = [t.copy() for t in T64]
    for step in range(3):
        ctx.run_steps(f.dt, 1, use_graph=(step > 0))
        for k, (h, v, l, w) in enumerate(opts):
            om.tracer_step(f, O.cfg_struct(h, v, l, wsplit=w), T64[k], np.zeros_like(T64[k]), O64[k])
    for k in range(n):
        got, _ = ctx.tracer_download(k)
        err = np.abs(got[wet] - T64[k][wet]).max() / np.abs(T64[k][wet]).max()
        assert err <= 1e-5, (opts[k], err)
    assert ctx.status() == 0


def test_more_tracers_than_one_launch_group(channel_small):
    """70 tracers: the FP32 step runs a group of 64 and a group of 6; tracers on both sides of
    the split match the oracle, and the FP64 step matches it bit for bit."""
    mesh = channel_small
    ntr = 70
    f = O.ensure_f64(M.make_forcing(mesh, "channel", seed=3, dt=600.0))
    tr = M.make_tracers(mesh, "channel", ntr=ntr, seed=4)
    cfgs = [G.tra_cfg("MUSCL" if k % 3 else "UPW1", "QR4C" if k % 2 else "PPM", "FCT" if k % 4 else "NON",
                      id=k + 1) for k in range(ntr)]
    ocfgs = [O.cfg_struct("MUSCL" if k % 3 else "UPW1", "QR4C" if k % 2 else "PPM", "FCT" if k % 4 else "NON")
             for k in range(ntr)]
    c32 = G.Context(mesh, G.PREC_FP32, max_tracers=ntr)
    c32.state_setup(cfgs)
    c32.forcing_upload(f)
    for k in range(ntr):
        t32 = tr[k].astype(np.float32)
        c32.tracer_upload(k, t32, t32)
    assert c32.launches_per_step() > 0
    c32.run_steps(f.dt, 2, use_graph=True)
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    check = [0, 1, 62, 63, 64, 65, 69]
    for k in check:
        T = tr[k].astype(np.float32).astype(np.float64)
        Oo = T.copy()
        for _ in range(2):
            om.tracer_step(f, ocfgs[k], T, np.zeros_like(T), Oo)
        got, _ = c32.tracer_download(k)
        err = np.abs(got[wet] - T[wet]).max() / np.abs(T[wet]).max()
        assert err <= 1e-5, (k, err)
    assert c32.status() == 0
    c64 = G.Context(mesh, G.PREC_FP64, max_tracers=ntr)
    Tg = [np.array(t, copy=True) for t in tr]
    Og = [t.copy() for t in Tg]
    c64.tracer_step(f, cfgs, Tg, Og)
    for k in (0, 63, 64, 69):
        T = np.array(tr[k], copy=True)
        Oo = T.copy()
        om.tracer_step(f, ocfgs[k], T, np.zeros_like(T), Oo)
        assert np.array_equal(Tg[k], T), k
