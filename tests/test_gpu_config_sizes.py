"""Parity at the benchmark configurations' full sizes (channel 100 x 400 / 40 levels, channel
400 x 1600 / 60 levels with seamounts, sphere of 7 subdivisions / 48 levels): the FP64 GPU
form equals the single-threaded oracle bit for bit where the oracle finishes in seconds to a
minute (configuration 1 over its 100 steps, configuration 3 over a step); the FP32 form is
checked against the FP64 GPU form step by step over the runs of configurations 2 (50 steps)
and 3 (20 steps), and through size-independent properties (a constant tracer, clean
status)."""
import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import perturbed_old, wet_mask

pytestmark = pytest.mark.gpu


def _fp64_vs_oracle(mesh, kind, scheme, steps):
    O.set_threads(1)  # the serial scatter order of the reference
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    tr = M.make_tracers(mesh, kind, ntr=2, seed=4)
    om = O.OracleMesh(mesh)
    ocfg = O.cfg_struct(*scheme)
    ctx = G.Context(mesh, G.PREC_FP64, max_tracers=2)
    rng = np.random.default_rng(2)
    To = [np.array(t, copy=True) for t in tr]
    Oo = [perturbed_old(t, rng) for t in To]
    Tg = [t.copy() for t in To]
    Og = [o.copy() for o in Oo]
    for step in range(steps):
        for k in range(2):
            om.tracer_step(f, ocfg, To[k], np.zeros_like(To[k]), Oo[k])
        ctx.tracer_step(f, [G.tra_cfg(*scheme, id=k + 1) for k in range(2)], Tg, Og)
        for k in range(2):
            assert np.array_equal(Tg[k], To[k]), (scheme, step, k)
    assert ctx.status() == 0


@pytest.mark.parametrize("scheme", [("MUSCL", "QR4C", "FCT"), ("MFCT", "QR4C", "FCT")])
def test_configuration_1_fp64_bitwise(scheme):
    mesh = M.config_mesh(1)
    assert mesh.nod2D == 40000 and mesh.nl == 41
    _fp64_vs_oracle(mesh, "channel", scheme, steps=2)


def test_configuration_1_fp64_bitwise_100_steps():
    """The configuration's own run: T and S, MUSCL + QR4C + FCT, AB2, implicit vertical
    diffusion, 100 steps of 600 s; the FP64 GPU form equals the oracle after every step."""
    mesh = M.config_mesh(1)
    _fp64_vs_oracle(mesh, "channel", ("MUSCL", "QR4C", "FCT"), steps=100)


def test_configuration_3_fp32_per_step_20_steps():
    """The configuration's run: FP32 against FP64 over 20 steps, each step within 1e-5."""
    _fp32_per_step(M.config_mesh(3), "sphere", 20)


def test_configuration_3_fp64_bitwise_and_fp32():
    mesh = M.config_mesh(3)
    _fp64_vs_oracle(mesh, "sphere", ("MUSCL", "QR4C", "FCT"), steps=1)
    # FP32 form, one step against the oracle from the same FP32-rounded state
    f = O.ensure_f64(M.make_forcing(mesh, "sphere", seed=3, dt=600.0))
    tr = M.make_tracers(mesh, "sphere", ntr=2, seed=4)
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=2)
    ctx.state_setup([G.tra_cfg(id=1), G.tra_cfg(id=2)])
    ctx.forcing_upload(f)
    T64 = []
    for k in range(2):
        t32 = tr[k].astype(np.float32)
        ctx.tracer_upload(k, t32, t32)
        T64.append(t32.astype(np.float64))
    ctx.run_steps(f.dt, 1, use_graph=True)
    om = O.OracleMesh(mesh)
    wet = wet_mask(mesh)
    for k in range(2):
        Oo = T64[k].copy()
        om.tracer_step(f, O.cfg_struct(), T64[k], np.zeros_like(T64[k]), Oo)
        got, _ = ctx.tracer_download(k)
        err = np.abs(got[wet] - T64[k][wet]).max() / np.abs(T64[k][wet]).max()
        assert err <= 1e-5, (k, err)
    assert ctx.status() == 0


def _fp32_per_step(mesh, kind, steps):
    """FP32 form against the FP64 GPU form (the form checked bit for bit against the oracle
    above), step by step over the configuration's run: both start every step from the FP32
    state, so each step's error is measured alone."""
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    tr = M.make_tracers(mesh, kind, ntr=2, seed=4)
    wet = wet_mask(mesh)
    cfgs = [G.tra_cfg(id=1), G.tra_cfg(id=2)]
    c64 = G.Context(mesh, G.PREC_FP64, max_tracers=2)
    c64.state_setup(cfgs)
    c64.forcing_upload(f)
    c32 = G.Context(mesh, G.PREC_FP32, max_tracers=2)
    c32.state_setup(cfgs)
    c32.forcing_upload(f)
    for k in range(2):
        t32 = tr[k].astype(np.float32)
        c64.tracer_upload(k, t32.astype(np.float64), t32.astype(np.float64))
        c32.tracer_upload(k, t32, t32)
    worst = 0.0
    for step in range(steps):
        c64.run_steps(f.dt, 1, use_graph=True)
        c32.run_steps(f.dt, 1, use_graph=True)
        for k in range(2):
            a = c64.tracer_download(k)[0]
            b, bold = c32.tracer_download(k)
            err = np.abs(b[wet] - a[wet]).max() / np.abs(a[wet]).max()
            worst = max(worst, err)
            assert err <= 1e-5, (step, k, err)
            c64.tracer_upload(k, b.astype(np.float64), bold.astype(np.float64))
    assert c32.status() == 0 and c64.status() == 0
    return f, c32, wet, worst


def test_configuration_2_fp32_against_fp64_and_properties():
    mesh = M.config_mesh(2)
    assert mesh.nod2D == 640000
    # the configuration's run: T and S, 50 steps
    f, c32, wet, worst = _fp32_per_step(mesh, "channel", 50)
    # a constant tracer stays constant in the FP32 form at this size
    cst = np.where(wet, 12.5, 0.0).astype(np.float32)
    c32.tracer_upload(0, cst, cst)
    c32.run_steps(f.dt, 2, use_graph=True)
    got = c32.tracer_download(0)[0]
    assert np.abs(got[wet] - 12.5).max() <= 12.5 * 1e-6
