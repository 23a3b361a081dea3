"""The allocation-free vertical diffusion entry point (fesom_gpu_vdiff_impl_noalloc).

It exists for callers that cannot call cudaMalloc -- FESOM2's OpenACC build,
whose data regions own every device array and pass device addresses to native
code, and codes held to a fixed device-memory budget.  Here the test plays such
a caller: it owns the device arrays (made with torch, outside the library),
calls the entry point through the C ABI twice in a row, and checks each result
against the regular entry point (fesom_gpu_vdiff_impl) applied the same number
of times: equal bit for bit, the tolerance of the other FP64 tests.

The level arrays are the caller's and the entry point cannot check them on the
host; a column with bad level bounds is skipped on the device and the call
returns FESOM_ERR_MESH, which the last test checks on a values array with a
sentinel tail inside its own allocation.

This file is collected last, so a run that stops at the first failure has run
every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M

pytestmark = pytest.mark.gpu

_P = C.c_void_p


def _entry():
    fn = G.load().fesom_gpu_vdiff_impl_noalloc
    fn.argtypes = [C.c_int32, C.c_int32, _P, _P, _P, _P, _P, _P, _P, _P, C.c_double, _P, _P, C.c_char_p, C.c_int32]
    fn.restype = C.c_int
    return fn


def _case():
    mesh = M.channel_mesh(16, 24, 5000.0, M.stretched_zbar(60, 10.0, 200.0), seamounts=3, seed=4,
                          partial_cells=True)
    f = M.make_forcing(mesh, "channel", seed=3, dt=600.0)
    f.bc_surface = np.linspace(-1e-3, 1e-3, mesh.nod2D)
    T0 = np.array(M.make_tracers(mesh, "channel", ntr=1, seed=4)[0], dtype=np.float64, copy=True)
    return mesh, f, T0


def test_noalloc_vdiff_equals_regular_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    mesh, f, T0 = _case()
    ctx = G.Context(mesh, G.PREC_FP64)
    expected = []
    cur = T0.copy()
    for _ in range(2):
        ctx.vdiff_impl(f, G.tra_cfg(), cur)
        expected.append(cur.copy())
    ctx.close()

    dev = torch.device("cuda:0")

    def on_device(a, dtype):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(dev)

    nlev = on_device(mesh.nlevels_nod2D, np.int32)
    ulev = on_device(mesh.ulevels_nod2D, np.int32)
    zbot = on_device(mesh.zbar_n_bot, np.float64)
    hnew = on_device(mesh.hnode_new, np.float64)
    area = on_device(mesh.area, np.float64)
    asvol = on_device(mesh.areasvol, np.float64)
    kv = on_device(f.Kv, np.float64)
    bc = on_device(f.bc_surface, np.float64)
    values = on_device(T0, np.float64)
    torch.cuda.synchronize()
    fn = _entry()
    err = C.create_string_buffer(256)
    for want in expected:
        rc = fn(mesh.nod2D, mesh.nl, nlev.data_ptr(), ulev.data_ptr(), zbot.data_ptr(), hnew.data_ptr(),
                area.data_ptr(), asvol.data_ptr(), kv.data_ptr(), bc.data_ptr(), float(f.dt), values.data_ptr(),
                None, err, 256)
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        got = values.cpu().numpy()
        assert np.array_equal(got, want)


def test_noalloc_vdiff_rejects_meshes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    one = torch.zeros(8, dtype=torch.float64, device=dev)
    ione = torch.zeros(8, dtype=torch.int32, device=dev)
    err = C.create_string_buffer(256)
    # 3 * nl * nod2D above the fixed scratch: refused on the host before any launch
    rc = _entry()(10_000_000, 71, ione.data_ptr(), ione.data_ptr(), one.data_ptr(), one.data_ptr(), one.data_ptr(),
                  one.data_ptr(), one.data_ptr(), None, 600.0, one.data_ptr(), None, err, 256)
    assert rc == 1
    assert b"too large" in err.value


def test_noalloc_vdiff_skips_columns_with_bad_level_bounds():
    """A one-layer column, a bottom level past nl and a top level below 1 are skipped and
    reported as FESOM_ERR_MESH; the other columns equal the regular entry point's result,
    the skipped ones and a sentinel tail behind the values are unchanged."""
    torch = pytest.importorskip("torch")
    mesh, f, T0 = _case()
    ctx = G.Context(mesh, G.PREC_FP64)
    want = T0.copy()
    ctx.vdiff_impl(f, G.tra_cfg(), want)
    ctx.close()

    nlev = np.array(mesh.nlevels_nod2D, dtype=np.int32, copy=True)
    ulev = np.array(mesh.ulevels_nod2D, dtype=np.int32, copy=True)
    last = mesh.nod2D - 1
    bad = {last: "one layer", 3: "below nl", 7: "top"}
    nlev[last] = ulev[last] + 1          # one wet layer: the solve would read past the column
    nlev[3] = mesh.nl + 1                # bottom level past nl
    ulev[7] = 0                          # top level below 1
    L1 = mesh.nl - 1
    sentinel = 12345.5
    tail = 4 * L1
    vals = np.concatenate([np.ravel(T0), np.full(tail, sentinel)])  # T0[n, :] is column n

    dev = torch.device("cuda:0")

    def on_device(a, dtype):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(dev)

    dv = on_device(vals, np.float64)
    args = [on_device(nlev, np.int32), on_device(ulev, np.int32), on_device(mesh.zbar_n_bot, np.float64),
            on_device(mesh.hnode_new, np.float64), on_device(mesh.area, np.float64),
            on_device(mesh.areasvol, np.float64), on_device(f.Kv, np.float64), on_device(f.bc_surface, np.float64)]
    torch.cuda.synchronize()
    err = C.create_string_buffer(256)
    rc = _entry()(mesh.nod2D, mesh.nl, *[a.data_ptr() for a in args], float(f.dt), dv.data_ptr(), None, err, 256)
    assert rc == 3, (rc, err.value)
    assert b"skipped" in err.value
    got = dv.cpu().numpy()
    assert np.all(got[-tail:] == sentinel)
    got = got[:-tail].reshape(np.shape(T0))
    for n in range(mesh.nod2D):
        if n in bad:
            assert np.array_equal(got[n], T0[n]), bad[n]
        else:
            assert np.array_equal(got[n], want[n])
