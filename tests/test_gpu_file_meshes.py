"""The GPU step on the meshes of the reference's test data (Soufflet channel, PI, PI with
ice-shelf cavities),
through the C ABI: FP64 bit for bit with the oracle over several steps (with the
Soufflet namelist's horizontal diffusion, K_hor = 10), FP32 within 1e-5 normwise."""
import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import perturbed_old, wet_mask
from tests.test_oracle import _ki

pytestmark = pytest.mark.gpu

CASES = [("soufflet_file_mesh", "channel", 10.0), ("pi_file_mesh", "sphere", None),
         ("pi_cavity_file_mesh", "sphere", None)]


@pytest.mark.parametrize("meshname,kind,khor", CASES)
@pytest.mark.parametrize("scheme", [("MUSCL", "QR4C", "FCT"), ("MFCT", "QR4C", "FCT"), ("UPW1", "UPW1", "NON")])
def test_fp64_bitwise_on_file_mesh(meshname, kind, khor, scheme, request):
    mesh = request.getfixturevalue(meshname)
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    tr = M.make_tracers(mesh, kind, ntr=2, seed=4)
    Ki = None if khor is None else _ki(mesh, khor)
    om = O.OracleMesh(mesh)
    ocfg = O.cfg_struct(*scheme, 0.0, 1.0)
    gcfgs = [G.tra_cfg(*scheme, 0.0, 1.0, id=k + 1) for k in range(2)]
    ctx = G.Context(mesh, G.PREC_FP64, max_tracers=2)
    if Ki is not None:
        ctx.set_hdiff(Ki)
    rng = np.random.default_rng(2)
    To = [np.array(t, copy=True) for t in tr]
    Oo = [perturbed_old(t, rng) for t in To]
    Tg = [t.copy() for t in To]
    Og = [o.copy() for o in Oo]
    for step in range(3):
        for k in range(2):
            om.tracer_step_ex(f, ocfg, To[k], np.zeros_like(To[k]), Oo[k], Ki=Ki)
        ctx.tracer_step(f, gcfgs, Tg, Og)
        for k in range(2):
            assert np.array_equal(Tg[k], To[k]), f"step {step} tracer {k}"
    assert ctx.status() == 0


@pytest.mark.parametrize("meshname,kind,khor", CASES)
def test_fp32_on_file_mesh(meshname, kind, khor, request):
    mesh = request.getfixturevalue(meshname)
    ntr = 4
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    tr = M.make_tracers(mesh, kind, ntr=ntr, seed=4)
    Ki = None if khor is None else _ki(mesh, khor)
    cfgs = [G.tra_cfg(id=k + 1) for k in range(ntr)]
    ctx = G.Context(mesh, G.PREC_FP32, max_tracers=ntr)
    ctx.state_setup(cfgs)
    ctx.forcing_upload(f)
    if Ki is not None:
        ctx.set_hdiff(Ki)
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
        for k in range(ntr):
            om.tracer_step_ex(f, O.cfg_struct(), T64[k], np.zeros_like(T64[k]), O64[k], Ki=Ki)
    for k in range(ntr):
        v, _ = ctx.tracer_download(k)
        err = np.abs(v[wet] - T64[k][wet]).max() / np.abs(T64[k][wet]).max()
        assert err <= 1e-5, (k, err)
    assert ctx.status() == 0
