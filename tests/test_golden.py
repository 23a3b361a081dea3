"""Committed golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py):
the oracle (CPU) and the FP64 CUDA path (GPU, through the C ABI) reproduce the
stored results of three tracer steps bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.golden.make_golden import CASES, load, options

NAMES = sorted(CASES)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    mesh, f, d = load(name)
    om = O.OracleMesh(mesh)
    assert np.array_equal(om.work["nboundary_lay"], d["muscl_nbl"])
    assert np.array_equal(om.work["edge_up_dn_tri"], d["muscl_updn"])
    hor, ver, lim = [str(x) for x in d["scheme"]]
    ws, Ki, ivd = options(d)
    for k in range(2):
        cfg = O.cfg_struct(hor, ver, lim, ph=0.0, pv=1.0, ab_order=int(d["ab"]), i_vert_diff=bool(ivd[k]), wsplit=ws)
        T, old = d[f"T0_{k}"].copy(), d[f"old0_{k}"].copy()
        for s in range(3):
            om.tracer_step_ex(f, cfg, T, np.zeros_like(T), old, Ki=Ki)
            assert np.array_equal(T, d[f"T{s + 1}_{k}"]), (name, k, s)
            assert np.array_equal(old, d[f"old{s + 1}_{k}"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_fp64_reproduces_golden(name):
    from fesom2_gb300 import gpu as G
    mesh, f, d = load(name)
    hor, ver, lim = [str(x) for x in d["scheme"]]
    ab = int(d["ab"])
    ws, Ki, ivd = options(d)
    cfgs = [G.tra_cfg(hor, ver, lim, 0.0, 1.0, ab_order=ab, i_vert_diff=bool(ivd[k]), id=k + 1) for k in range(2)]
    # the fixture carries the MUSCL init arrays it was made with (as FESOM passes its own
    # tracers%work arrays): the up/down-triangle search uses atan2, whose last bit may
    # differ between the C libraries of two machines
    ctx = G.Context(mesh, G.PREC_FP64, max_tracers=2, pass_muscl_init=(d["muscl_nbl"], d["muscl_updn"]))
    ctx.set_wsplit(ws)
    if Ki is not None:
        ctx.set_hdiff(Ki)
    T = [d[f"T0_{k}"].copy() for k in range(2)]
    old = [np.ascontiguousarray(d[f"old0_{k}"]).copy() for k in range(2)]
    for s in range(3):
        ctx.tracer_step(f, cfgs, T, old)
        for k in range(2):
            assert np.array_equal(T[k], d[f"T{s + 1}_{k}"]), (name, k, s)
            assert np.array_equal(old[k].reshape(-1), d[f"old{s + 1}_{k}"].reshape(-1))
