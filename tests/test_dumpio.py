"""The reader of the reference's unformatted tracer dump (READ_T_TRACER layout): a dump
written in that record layout reads back field for field, subrecords of long records are
joined, damaged files are refused, and the state it holds steps in the oracle."""
import io
import struct

import numpy as np
import pytest

from fesom2_gb300 import dumpio as D
from fesom2_gb300 import mesh as M
from oracle import oracle as O


def _dump(mesh, ntr=3, ab=(2, 3, 2), seed=1):
    rng = np.random.default_rng(seed)
    tr = M.make_tracers(mesh, "channel", ntr=ntr, seed=seed)
    L1, N2 = mesh.nl - 1, mesh.nod2D
    data = []
    schemes = [("MUSCL", "QR4C", "FCT"), ("MFCT", "PPM", "FCT"), ("UPW1", "CDIFF", "none")]
    for k in range(ntr):
        T = np.ascontiguousarray(tr[k])
        old = np.ascontiguousarray(np.stack([T * (1 + 1e-3 * rng.standard_normal(T.shape))
                                             for _ in range(ab[k] - 1)], axis=-1))
        h, v, l = schemes[k % 3]
        data.append(D.TracerData(T, old, T * 1.01, False, 0.0, 0.0025, 0.0, k != 2, h, v, l, 0.0, 1.0,
                                 [1, 2, 101][k % 3]))
    work = {}
    for name, dt, rank in D.WORK_FIELDS:
        if name in ("dvd_trflx_hor", "dvd_trflx_ver"):
            work[name] = None  # unallocated (ldiag_DVD off)
        elif name == "nboundary_lay":
            work[name] = rng.integers(0, 10, N2).astype(np.int32)
        elif name == "edge_up_dn_tri":
            work[name] = rng.integers(-1, mesh.elem2D, (mesh.edge2D, 2)).astype(np.int32)
        elif name == "edge_up_dn_grad":
            work[name] = rng.standard_normal((mesh.edge2D, L1, 4))
        elif name in ("adv_flux_hor",):
            work[name] = rng.standard_normal((mesh.edge2D, L1))
        elif name in ("adv_flux_ver",):
            work[name] = rng.standard_normal((N2, mesh.nl))
        else:
            work[name] = rng.standard_normal((N2, L1))
    return D.Tracers(data, work)


def test_round_trip(tmp_path, channel_small):
    tr = _dump(channel_small)
    p = tmp_path / "t_tracer.bin"
    D.write_tracers(str(p), tr)
    back = D.read_tracers(str(p))
    assert len(back.data) == 3
    for a, b in zip(tr.data, back.data):
        for f in ("values", "valuesold", "valuesAB"):
            assert np.array_equal(getattr(a, f), getattr(b, f))
        for f in ("smooth_bh_tra", "gamma0_tra", "gamma1_tra", "gamma2_tra", "i_vert_diff", "tra_adv_ph",
                  "tra_adv_pv", "ID"):
            assert getattr(a, f) == getattr(b, f)
        assert (a.tra_adv_hor, a.tra_adv_ver, a.tra_adv_lim) == (b.tra_adv_hor, b.tra_adv_ver, b.tra_adv_lim)
        assert b.ab_order == a.valuesold.shape[-1] + 1
    for name, _, _ in D.WORK_FIELDS:
        x, y = tr.work[name], back.work[name]
        assert (x is None and y is None) or np.array_equal(x, y), name


def test_record_layout_is_fortran_sequential(tmp_path):
    """First records: num_tracers, then the extents (column-major order) of values."""
    mesh = M.channel_mesh(6, 8, 5000.0, -np.arange(6) * 50.0)
    tr = _dump(mesh, ntr=1, ab=(2,))
    p = tmp_path / "d.bin"
    D.write_tracers(str(p), tr)
    b = p.read_bytes()
    assert struct.unpack("<iii", b[:12]) == (4, 1, 4)
    n, s1, s2, n2 = struct.unpack("<iiii", b[12:28])
    assert (n, s1, s2, n2) == (8, mesh.nl - 1, mesh.nod2D, 8)


def test_subrecords_are_joined(monkeypatch):
    monkeypatch.setattr(D, "_MAX_SUB", 40)
    buf = io.BytesIO()
    a = np.arange(50, dtype=np.float64)
    D.RecordWriter(buf).array(a, "f8", 1)
    buf.seek(0)
    assert np.array_equal(D.RecordReader(buf).array("f8", 1), a)


def test_damaged_dumps_are_refused(tmp_path, channel_small):
    tr = _dump(channel_small)
    p = tmp_path / "t.bin"
    D.write_tracers(str(p), tr)
    b = bytearray(p.read_bytes())
    (tmp_path / "short.bin").write_bytes(bytes(b[:-10]))
    with pytest.raises((EOFError, ValueError, struct.error)):
        D.read_tracers(str(tmp_path / "short.bin"))
    b2 = bytearray(b)
    b2[16:20] = struct.pack("<i", 999999)  # an extent that does not match its data record
    (tmp_path / "bad.bin").write_bytes(bytes(b2))
    with pytest.raises(ValueError):
        D.read_tracers(str(tmp_path / "bad.bin"))
    (tmp_path / "long.bin").write_bytes(bytes(b) + b"\0")
    with pytest.raises(ValueError):
        D.read_tracers(str(tmp_path / "long.bin"))


def test_dump_state_steps_in_the_oracle(tmp_path, channel_small):
    """The state of a dump (values, valuesold, schemes) feeds the step as it is."""
    mesh = channel_small
    tr = _dump(mesh)
    p = tmp_path / "t.bin"
    D.write_tracers(str(p), tr)
    cfgs, vals, olds = D.step_inputs(D.read_tracers(str(p)))
    assert [c.adv_ver for c in cfgs] == [0, 3, 2] and [c.adv_lim for c in cfgs] == [1, 1, 0]
    assert [c.ab_order for c in cfgs] == [2, 3, 2] and [c.i_vert_diff for c in cfgs] == [1, 1, 0]
    f = O.ensure_f64(M.make_forcing(mesh, "channel", seed=3, dt=600.0))
    om = O.OracleMesh(mesh)
    for k, c in enumerate(cfgs):
        oc = O.cfg_struct(["MUSCL", "MFCT", "UPW1"][c.adv_hor], ["QR4C", "UPW1", "CDIFF", "PPM"][c.adv_ver],
                          "FCT" if c.adv_lim else "NON", ab_order=c.ab_order, i_vert_diff=bool(c.i_vert_diff))
        T, old = vals[k].copy(), np.ascontiguousarray(olds[k]).copy()
        om.tracer_step(f, oc, T, np.zeros_like(T), old)
        assert np.isfinite(T).all() and np.abs(T - vals[k]).max() > 0
