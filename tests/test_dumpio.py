"""The readers of the reference's derived-type binary restarts (t_tracer, t_mesh, t_dynamics,
t_partit): dumps written in their layout -- one record per file, the fields of the
defined-I/O procedures one after another -- read back field for field, gfortran subrecords are
joined, damaged files are refused, and the state they hold steps in the oracle as the mesh and
tracers it came from do."""
import math
import os
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


def test_dump_is_one_record(tmp_path):
    """The defined-I/O write of the derived type is one record: its fields one after another
    (num_tracers, the extents of values in column-major order, the values ...) between the two
    length markers of the whole record."""
    mesh = M.channel_mesh(6, 8, 5000.0, -np.arange(6) * 50.0)
    tr = _dump(mesh, ntr=1, ab=(2,))
    p = tmp_path / "d.bin"
    D.write_tracers(str(p), tr)
    b = p.read_bytes()
    L = struct.unpack("<i", b[:4])[0]
    assert L == len(b) - 8 and struct.unpack("<i", b[-4:])[0] == L
    n, s1, s2 = struct.unpack("<iii", b[4:16])
    assert (n, s1, s2) == (1, mesh.nl - 1, mesh.nod2D)
    v = np.frombuffer(b[16:16 + 8 * s1 * s2], dtype="<f8").reshape(s2, s1)
    assert np.array_equal(v, tr.data[0].values)
    # valuesold(1, nl-1, nod2D) follows: three extents
    assert struct.unpack("<iii", b[16 + 8 * s1 * s2:28 + 8 * s1 * s2]) == (1, mesh.nl - 1, mesh.nod2D)


def test_subrecords_are_joined(tmp_path, monkeypatch, channel_small):
    """A record above the subrecord limit is split as gfortran splits it: the leading marker of
    every subrecord but the last is negative, the trailing marker of every one but the first."""
    monkeypatch.setattr(D, "_MAX_SUB", 1000)
    tr = _dump(channel_small)
    p = tmp_path / "d.bin"
    D.write_tracers(str(p), tr)
    b = p.read_bytes()
    heads, tails, pos = [], [], 0
    while pos < len(b):
        h = struct.unpack("<i", b[pos:pos + 4])[0]
        t = struct.unpack("<i", b[pos + 4 + abs(h):pos + 8 + abs(h)])[0]
        heads.append(h)
        tails.append(t)
        pos += abs(h) + 8
    assert len(heads) > 3
    assert all(h < 0 for h in heads[:-1]) and heads[-1] > 0
    assert tails[0] > 0 and all(t < 0 for t in tails[1:])
    back = D.read_tracers(str(p))
    assert np.array_equal(back.data[1].valuesold, tr.data[1].valuesold)


def test_damaged_dumps_are_refused(tmp_path, channel_small):
    tr = _dump(channel_small)
    p = tmp_path / "t.bin"
    D.write_tracers(str(p), tr)
    b = bytearray(p.read_bytes())
    (tmp_path / "short.bin").write_bytes(bytes(b[:-10]))
    with pytest.raises((EOFError, ValueError)):
        D.read_tracers(str(tmp_path / "short.bin"))
    b2 = bytearray(b)
    b2[8:12] = struct.pack("<i", 999999)  # an extent the record cannot hold
    (tmp_path / "bad.bin").write_bytes(bytes(b2))
    with pytest.raises(ValueError):
        D.read_tracers(str(tmp_path / "bad.bin"))
    (tmp_path / "long.bin").write_bytes(bytes(b) + b"\0")
    with pytest.raises((EOFError, ValueError)):
        D.read_tracers(str(tmp_path / "long.bin"))
    b3 = bytearray(b)
    b3[-4:] = struct.pack("<i", -struct.unpack("<i", bytes(b[-4:]))[0])  # a trailing marker of a continuation
    (tmp_path / "marker.bin").write_bytes(bytes(b3))
    with pytest.raises(ValueError):
        D.read_tracers(str(tmp_path / "marker.bin"))


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


def _mesh_fields_equal(a, b):
    for f in ("elem2D_nodes", "edges", "edge_tri", "nod_in_elem2D_ptr", "nod_in_elem2D", "nlevels", "ulevels",
              "nlevels_nod2D", "ulevels_nod2D", "nlevels_nod2D_min", "ulevels_nod2D_max", "elem_area", "elem_cos",
              "edge_dxdy", "edge_cross_dxdy", "gradient_sca", "area", "areasvol", "hnode", "hnode_new", "helem",
              "zbar", "Z", "zbar_3d_n", "Z_3d_n", "zbar_n_bot"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert (a.nl, a.nod2D, a.elem2D, a.edge2D, a.edge2D_in) == (b.nl, b.nod2D, b.elem2D, b.edge2D, b.edge2D_in)


@pytest.mark.parametrize("meshname,kind", [("channel_seamount", "channel"), ("pi_cavity_file_mesh", "sphere")])
def test_mesh_dump_steps_as_its_mesh(tmp_path, meshname, kind, request):
    """A t_mesh dump of a mesh gives back every field the step reads, and the oracle steps on it
    -- with the MUSCL set-up of the tracer dump's work arrays, as the dump holds no coordinates --
    bit for bit as on the mesh itself."""
    mesh = request.getfixturevalue(meshname)
    p = str(tmp_path / "t_mesh.0")
    D.write_mesh_dump(p, D.dump_from_mesh(mesh))
    tm = D.read_mesh_dump(p)
    assert tm["metric_factor"] is None and tm["ssh_stiff_dim"] == 0  # fields the step does not read
    m2 = D.mesh_from_dump(tm, cyclic_length=mesh.cyclic_length, cartesian=mesh.cartesian)
    _mesh_fields_equal(mesh, m2)
    om = O.OracleMesh(mesh)
    work = {name: None for name, _, _ in D.WORK_FIELDS}
    work["nboundary_lay"] = om.work["nboundary_lay"]
    work["edge_up_dn_tri"] = np.where(om.work["edge_up_dn_tri"] >= 0, om.work["edge_up_dn_tri"] + 1, 0)
    nbl, updn = D.muscl_init_from_dump(D.Tracers([], work))
    om2 = O.OracleMesh(m2)
    om2.work["nboundary_lay"][...] = nbl
    om2.work["edge_up_dn_tri"][...] = updn
    f = O.ensure_f64(M.make_forcing(mesh, kind, seed=3, dt=600.0))
    T = np.ascontiguousarray(M.make_tracers(mesh, kind, ntr=1, seed=4)[0])
    a, ao, b, bo = T.copy(), T.copy(), T.copy(), T.copy()
    for _ in range(2):
        om.tracer_step(f, O.cfg_struct(), a, np.zeros_like(a), ao)
        om2.tracer_step(f, O.cfg_struct(), b, np.zeros_like(b), bo)
    assert np.array_equal(a, b)


def _dyn_fields(rng, T2=5, N2=7, nl=4, se=False):
    d = {name: (0 if kind in ("i4", "f8") else False) if isinstance(kind, str) else None for name, kind in D.DYN_HEAD}
    d.update(opt_visc=5, visc_gamma0=0.03, use_ivertvisc=True, momadv_opt=2, use_wsplit=False, wsplit_maxcfl=1.0,
             use_ssh_se_subcycl=se, solver_ident=1, solver_maxiter=2000, solver_soltol=1e-5,
             solver_rr=rng.standard_normal(N2))
    d["uv"] = rng.standard_normal((T2, nl - 1, 2))
    d["uv_rhsAB"] = rng.standard_normal((1, T2, nl - 1, 2))
    for k in ("w", "w_e", "w_i", "cfl_z"):
        d[k] = rng.standard_normal((N2, nl))
    d["fer_w"] = rng.standard_normal((N2, nl))
    d["fer_uv"] = rng.standard_normal((T2, nl - 1, 2))
    d["se_uvBT"] = rng.standard_normal((T2, 2))
    d["se_uvBT_stab_bdrag"] = rng.standard_normal(T2)
    return d


@pytest.mark.parametrize("fer_gm,se", [(False, False), (True, False), (False, True), (True, True)])
def test_dyn_dump_round_trip(tmp_path, fer_gm, se):
    rng = np.random.default_rng(5)
    d = _dyn_fields(rng, se=se)
    p = str(tmp_path / "t_dynamics.0")
    D.write_dyn_dump(p, d, fer_gm=fer_gm)
    for detect in (None, fer_gm):
        back = D.read_dyn_dump(p, fer_gm=detect)
        for k in ("uv", "uv_rhsAB", "w", "w_e", "w_i", "cfl_z", "solver_rr"):
            assert np.array_equal(back[k], d[k]), k
        assert back["opt_visc"] == 5 and back["use_ivertvisc"] is True and back["use_ssh_se_subcycl"] is se
        assert ("fer_w" in back) == fer_gm and (not fer_gm or np.array_equal(back["fer_uv"], d["fer_uv"]))
        assert ("se_uvBT" in back) == se
    f = D.dyn_forcing(back, 600.0)
    assert f.uv.shape == (5, 3, 2) and f.w_i.shape == (7, 4) and f.dt == 600.0


def test_partit_dump_and_the_whole_mesh_rule(tmp_path, channel_small):
    mesh = channel_small
    com = {"rPEnum": 0, "rPE": np.zeros(32, np.int32), "rptr": np.zeros(33, np.int32), "rlist": None,
           "sPEnum": 0, "sPE": np.zeros(32, np.int32), "sptr": np.zeros(32, np.int32), "slist": None, "nreq": 0}
    part = {c: com for c in D.COM_NAMES}
    part.update(npes=1, mype=0, maxPEnum=100, part=np.array([0, mesh.nod2D], np.int32), myDim_nod2D=mesh.nod2D,
                eDim_nod2D=0, myList_nod2D=np.arange(1, mesh.nod2D + 1, dtype=np.int32), myDim_elem2D=mesh.elem2D,
                eDim_elem2D=0, eXDim_elem2D=0, myList_elem2D=np.arange(1, mesh.elem2D + 1, dtype=np.int32),
                myDim_edge2D=mesh.edge2D, eDim_edge2D=0, myList_edge2D=np.arange(1, mesh.edge2D + 1, dtype=np.int32),
                pe_status=0)
    d = tmp_path / "fesom_bin_restart" / "np1"
    d.mkdir(parents=True)
    D.write_partit_dump(str(d / "t_partit.0"), part)
    D.write_mesh_dump(str(d / "t_mesh.0"), D.dump_from_mesh(mesh))
    D.write_tracers(str(d / "t_tracer.0"), _dump(mesh))
    r = D.read_restart(str(d))
    assert set(r) == {"mesh", "partit", "tracers"}
    assert r["partit"]["myDim_nod2D"] == mesh.nod2D and np.array_equal(r["partit"]["com_nod2D"]["rptr"], com["rptr"])
    _mesh_fields_equal(mesh, D.mesh_from_dump(r["mesh"], r["partit"], mesh.cyclic_length, mesh.cartesian))
    with pytest.raises(ValueError):
        D.mesh_from_dump(r["mesh"], dict(r["partit"], npes=2, eDim_nod2D=5))
    assert D.rank_suffix(3, 1) == "3" and D.rank_suffix(3, 8) == "3" and D.rank_suffix(3, 16) == "03"


def test_payload_round_trip_random_fields(tmp_path, monkeypatch):
    """Random field sequences (scalars, logicals, characters, arrays of rank 1-4 with zero and
    unallocated extents) read back as written, with records split into subrecords."""
    hyp = pytest.importorskip("hypothesis")
    from hypothesis import given, settings, strategies as st

    monkeypatch.setattr(D, "_MAX_SUB", 64)
    kinds = st.sampled_from(["i4", "f8", "L4", "c", ("i4", 1), ("f8", 2), ("i4", 3), ("f8", 4)])

    @settings(max_examples=60, deadline=None)
    @given(st.lists(st.tuples(kinds, st.integers(0, 2 ** 31 - 1)), min_size=1, max_size=12))
    def check(spec):
        rng = np.random.default_rng(spec[0][1])
        w = D.PayloadWriter()
        want = []
        for kind, seed in spec:
            r = np.random.default_rng(seed)
            if kind == "c":
                v = "".join(r.choice(list("ABCDEFGH"), size=int(r.integers(0, 20))))
                w.chars(v, 20)
            elif isinstance(kind, str):
                v = {"i4": int(r.integers(-2 ** 31, 2 ** 31)), "f8": float(r.standard_normal()),
                     "L4": bool(r.integers(0, 2))}[kind]
                w.scalar(kind, v)
            else:
                dt, rank = kind
                if r.random() < 0.2:
                    v = None
                else:
                    shape = tuple(int(x) for x in r.integers(0, 4, rank))
                    v = (r.integers(-9, 9, shape).astype(np.int32) if dt == "i4" else r.standard_normal(shape))
                    if v.size == 0 and all(d == 0 for d in shape):
                        v = None
                w.array(v, dt, rank)
            want.append((kind, v))
        p = str(tmp_path / f"rand{rng.integers(1 << 30)}.bin")
        w.write(p)
        rd = D.read_dump(p)
        for kind, v in want:
            if kind == "c":
                assert rd.chars(20) == v.rstrip()
            elif isinstance(kind, str):
                assert rd.scalar(kind) == v
            else:
                got = rd.array(*kind)
                assert (got is None and v is None) or np.array_equal(got, v)
        rd.done()

    check()
