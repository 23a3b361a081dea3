"""fesom_gpu_step_host_f32: one FP32 step from and to host arrays with the transfers
overlapped with the compute (tracer groups in flight on three streams) gives the same
values and previous levels, bit for bit, as the device-resident steps."""
import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SPECS = [("MUSCL", "QR4C", "FCT", 1), ("UPW1", "UPW1", "NON", 1), ("MFCT", "QR4C", "FCT", 0),
         ("MUSCL", "UPW1", "NON", 0), ("MUSCL", "QR4C", "FCT", 1)]


def _setup(mesh, kind, ab):
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    f32 = M.Forcing(uv=np.ascontiguousarray(f.uv, dtype=np.float32), w=np.ascontiguousarray(f.w, dtype=np.float32),
                    w_e=np.ascontiguousarray(f.w_e, dtype=np.float32), w_i=None,
                    Kv=np.ascontiguousarray(f.Kv, dtype=np.float32), bc_surface=None, dt=600.0)
    tr = M.make_tracers(mesh, kind, ntr=len(SPECS), seed=4, dtype=np.float32)
    cfgs = []
    for k, (hor, ver, lim, ivd) in enumerate(SPECS):
        c = G.tra_cfg(hor, ver, lim, 0.0, 1.0, ab_order=ab, id=k + 1)
        c.i_vert_diff = ivd
        cfgs.append(c)
    return f32, tr, cfgs


@pytest.mark.parametrize("ab", [2, 3])
def test_host_step_equals_device_resident_steps(channel_seamount, ab):
    mesh = channel_seamount
    f32, tr, cfgs = _setup(mesh, "channel", ab)
    n = len(cfgs)
    rng = np.random.default_rng(5)
    old0 = [np.ascontiguousarray(np.repeat((tr[k] * (1 + 1e-3 * rng.standard_normal(tr[k].shape)))[..., None],
                                           ab - 1, axis=-1).astype(np.float32)) for k in range(n)]
    if ab == 2:
        old0 = [np.ascontiguousarray(o[..., 0]) for o in old0]
    a = G.Context(mesh, G.PREC_FP32, max_tracers=n)
    a.state_setup(cfgs)
    a.set_tracers_per_launch(2)
    a.forcing_upload(f32)
    for k in range(n):
        a.tracer_upload(k, np.array(tr[k], copy=True), np.array(old0[k], copy=True))
    a.run_steps(600.0, 3, use_graph=True)
    want = [a.tracer_download(k, dtype=np.float32) for k in range(n)]
    b = G.Context(mesh, G.PREC_FP32, max_tracers=n)
    b.state_setup(cfgs)
    b.set_tracers_per_launch(2)
    vals = [np.array(tr[k], copy=True) for k in range(n)]
    olds = [np.array(old0[k], copy=True) for k in range(n)]
    for _ in range(3):
        b.step_host_f32(f32, vals, olds, vals, olds)
    for k in range(n):
        assert np.array_equal(vals[k], want[k][0]), k
        assert np.array_equal(olds[k].reshape(-1), want[k][1].reshape(-1)), k
    assert b.status() == 0


def test_host_step_with_swapped_time_levels(channel_seamount):
    """Two host time levels that swap roles (new values written over the consumed previous
    level, no previous level copied back) give the device-resident steps' values."""
    mesh = channel_seamount
    f32, tr, cfgs = _setup(mesh, "channel", 2)
    n = len(cfgs)
    a = G.Context(mesh, G.PREC_FP32, max_tracers=n)
    a.state_setup(cfgs)
    a.set_tracers_per_launch(3)
    a.forcing_upload(f32)
    for k in range(n):
        a.tracer_upload(k, np.array(tr[k], copy=True), np.array(tr[k], copy=True))
    a.run_steps(600.0, 4, use_graph=True)
    want = [a.tracer_download(k, dtype=np.float32) for k in range(n)]
    b = G.Context(mesh, G.PREC_FP32, max_tracers=n)
    b.state_setup(cfgs)
    b.set_tracers_per_launch(3)
    levels = [[np.array(tr[k], copy=True) for k in range(n)], [np.array(tr[k], copy=True) for k in range(n)]]
    for _ in range(4):
        cur, old = levels
        b.step_host_f32(f32, cur, old, old, None)
        levels.reverse()
    for k in range(n):
        assert np.array_equal(levels[0][k], want[k][0]), k
        assert np.array_equal(levels[1][k], want[k][1]), k
    assert b.status() == 0


def test_host_step_with_explicit_groups(channel_seamount):
    """Pipeline stages set by fesom_gpu_set_host_groups (in tracer groups) give the same values
    as the default ramp; orders that miss or repeat a group, or exceed the groups per launch,
    are rejected.  The five tracers of four schemes sit in four groups of two slots."""
    mesh = channel_seamount
    f32, tr, cfgs = _setup(mesh, "channel", 2)
    n = len(cfgs)
    results = []
    for sizes in ((), (2, 2), (1, 1, 1, 1), (1, 2, 1)):
        b = G.Context(mesh, G.PREC_FP32, max_tracers=n)
        b.state_setup(cfgs)
        ngr, width, grp, slot = b.tracer_groups()
        assert (ngr, width) == (4, 2)
        assert list(grp) == [0, 1, 2, 3, 0] and list(slot) == [0, 0, 0, 0, 1]
        b.set_tracers_per_launch(3)  # two groups per launch
        b.set_host_groups(sizes)
        levels = [[np.array(tr[k], copy=True) for k in range(n)], [np.array(tr[k], copy=True) for k in range(n)]]
        for _ in range(2):
            cur, old = levels
            b.step_host_f32(f32, cur, old, old, None)
            levels.reverse()
        results.append(levels[0])
        assert b.status() == 0
        for bad in ((3, 1), (2, 1), (2, 2, 1), (0, 2, 2)):
            with pytest.raises(G.FesomGpuError):
                b.set_host_groups(bad)
        b.close()
    for r in results[1:]:
        for k in range(n):
            assert np.array_equal(r[k], results[0][k]), k


def test_host_step_from_library_pinned_arrays(channel_seamount):
    """Host arrays in the library's page-locked memory (fesom_gpu_host_alloc) give the same
    step as ordinary host arrays, bit for bit; dropping them gives the memory back."""
    mesh = channel_seamount
    f32, tr, cfgs = _setup(mesh, "channel", 2)
    n = len(cfgs)
    outs = []
    for pinned in (False, True):
        c = G.Context(mesh, G.PREC_FP32, max_tracers=n)
        c.state_setup(cfgs)
        mk = (lambda a: (lambda h: (h.__setitem__(Ellipsis, a), h)[1])(G.host_array(a.shape, np.float32))) if pinned \
            else (lambda a: np.array(a, copy=True))
        fe = M.Forcing(uv=mk(f32.uv), w=mk(f32.w), w_e=mk(f32.w_e), w_i=None, Kv=mk(f32.Kv), bc_surface=None,
                       dt=600.0)
        vals = [mk(tr[k]) for k in range(n)]
        olds = [mk(tr[k]) for k in range(n)]
        for _ in range(2):
            c.step_host_f32(fe, vals, olds, vals, olds)
        outs.append([np.array(v, copy=True) for v in vals])
        assert c.status() == 0
        c.close()
        del fe, vals, olds
    for k in range(n):
        assert np.array_equal(outs[0][k], outs[1][k]), k
