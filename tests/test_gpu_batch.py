"""Multi-instance batch of the FP32 form: independent meshes of different sizes, level
counts, tracer counts and schemes stepped together (one launch per stage over all of
them) give the values of each context stepped alone, to FP32 rounding (the multi-instance
kernels are separate compilations of the same code, so the compiler may contract a few
multiply-adds differently), and stay within 1e-5 of the FP64 oracle."""
import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import wet_mask

pytestmark = pytest.mark.gpu

SPECS = [("MUSCL", "QR4C", "FCT", 1), ("UPW1", "UPW1", "NON", 1), ("MFCT", "QR4C", "FCT", 0),
         ("MUSCL", "UPW1", "NON", 0)]


def _instances(request):
    out = []
    for name, kind, ntr in [("channel_seamount", "channel", 2), ("sphere_small", "sphere", 3),
                            ("basin_irregular", "basin", 4)]:
        mesh = request.getfixturevalue(name)
        f = O.ensure_f64(M.make_forcing(mesh, kind, seed=7, dt=600.0))
        tr = M.make_tracers(mesh, kind, ntr=ntr, seed=8)
        cfgs = []
        for k in range(ntr):
            hor, ver, lim, ivd = SPECS[k % len(SPECS)]
            c = G.tra_cfg(hor, ver, lim, 0.0, 1.0, id=k + 1)
            c.i_vert_diff = ivd
            cfgs.append(c)
        out.append((mesh, f, tr, cfgs))
    return out


def _contexts(inst):
    ctxs = []
    for mesh, f, tr, cfgs in inst:
        c = G.Context(mesh, G.PREC_FP32, max_tracers=len(cfgs))
        c.state_setup(cfgs)
        c.forcing_upload(f)
        for k in range(len(cfgs)):
            T = tr[k].astype(np.float32)
            c.tracer_upload(k, T, T)
        ctxs.append(c)
    return ctxs


def test_batch_equals_contexts_stepped_alone(request):
    inst = _instances(request)
    alone = _contexts(inst)
    for c in alone:
        c.run_steps(600.0, 1, use_graph=False)
        c.run_steps(600.0, 3, use_graph=True)
    together = _contexts(inst)
    b = G.Batch(together)
    assert b.launches_per_step() >= 6
    b.run_steps(600.0, 1, use_graph=False)
    b.run_steps(600.0, 3, use_graph=True)
    for ca, cb, (mesh, f, tr, cfgs) in zip(alone, together, inst):
        for k in range(len(cfgs)):
            va, oa = ca.tracer_download(k, dtype=np.float32)
            vb, ob = cb.tracer_download(k, dtype=np.float32)
            scale = float(np.abs(va).max())
            assert np.abs(va - vb).max() <= 1e-6 * scale, (mesh.name, k)
            assert np.abs(oa - ob).max() <= 1e-6 * scale, (mesh.name, k)
        assert cb.status() == 0
    b.close()


def test_batch_error_vs_fp64_oracle(request):
    """One batched step: every instance and tracer within 1e-5 (normwise) of the FP64 oracle."""
    inst = _instances(request)
    ctxs = _contexts(inst)
    b = G.Batch(ctxs)
    b.run_steps(600.0, 1, use_graph=True)
    for c, (mesh, f, tr, cfgs) in zip(ctxs, inst):
        om = O.OracleMesh(mesh)
        wet = wet_mask(mesh)
        for k, cfg in enumerate(cfgs):
            hor, ver, lim, ivd = SPECS[k % len(SPECS)]
            T64 = tr[k].astype(np.float32).astype(np.float64)
            O64 = T64.copy()
            om.tracer_step(f, O.cfg_struct(hor, ver, lim, 0.0, 1.0, i_vert_diff=ivd), T64, np.zeros_like(T64), O64)
            v, _ = c.tracer_download(k)
            err = np.abs(v[wet] - T64[wet]).max() / np.abs(T64[wet]).max()
            assert err <= 1e-5, (mesh.name, k, err)
    b.close()


def test_batch_rejects_mixed_precision_and_unset_state(channel_small):
    a = G.Context(channel_small, G.PREC_FP64)
    with pytest.raises(G.FesomGpuError):
        G.Batch([a])
    c = G.Context(channel_small, G.PREC_FP32)
    with pytest.raises(G.FesomGpuError):
        G.Batch([c])
