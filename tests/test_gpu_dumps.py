"""The dwarf harness's flow on this library (dwarf_ini/fesom.F90:64-128): the state is read
from derived-type dumps -- t_mesh, t_dynamics, t_tracer -- and do_oce_adv_tra runs on it.
Dumps written from the PI mesh and a seeded state give, through the C ABI on the GPU, the
oracle's results on the mesh and state they came from, bit for bit.

The dwarf passes the dump's edge_up_dn_grad to do_oce_adv_tra; the library forms the
gradients from the values, as init_tracers_AB does before every advection in the model, so the
dumps here hold the gradients of their own values and the comparison is of the first call."""
import numpy as np
import pytest

from fesom2_gb300 import dumpio as D
from fesom2_gb300 import gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import wet_mask

pytestmark = pytest.mark.gpu


def _write_dumps(path, mesh, f, T, old, om):
    D.write_mesh_dump(str(path / "t_mesh.0"), D.dump_from_mesh(mesh))
    dyn = {name: (False if kind == "L4" else 0) if isinstance(kind, str) else None for name, kind in D.DYN_HEAD}
    dyn.update(uv=f.uv, w=f.w, w_e=f.w_e, w_i=f.w_i)
    D.write_dyn_dump(str(path / "t_dynamics.0"), dyn)
    work = {name: None for name, _, _ in D.WORK_FIELDS}
    work["nboundary_lay"] = om.work["nboundary_lay"]
    work["edge_up_dn_tri"] = np.where(om.work["edge_up_dn_tri"] >= 0, om.work["edge_up_dn_tri"] + 1, 0)
    work["edge_up_dn_grad"] = om.work["edge_up_dn_grad"]
    data = [D.TracerData(T, old[..., None], T, False, 0.0, 0.0, 0.0, True, "MUSCL", "QR4C", "FCT", 0.0, 1.0, 1)]
    D.write_tracers(str(path / "t_tracer.0"), D.Tracers(data, work))


def test_dwarf_adv_tra_from_dumps(tmp_path, pi_file_mesh):
    mesh = pi_file_mesh
    f = O.ensure_f64(M.make_forcing(mesh, "sphere", seed=3, dt=600.0))
    T = np.ascontiguousarray(M.make_tracers(mesh, "sphere", ntr=1, seed=4)[0])
    old = T * (1.0 + 1e-3 * np.random.default_rng(2).standard_normal(T.shape))
    om = O.OracleMesh(mesh)
    ocfg = O.cfg_struct("MUSCL", "QR4C", "FCT", ph=0.0, pv=1.0)
    om.init_tracers_AB(ocfg, T.copy(), np.zeros_like(T), old.copy()[..., None].copy())
    _write_dumps(tmp_path, mesh, f, T, old, om)
    # the dwarf's state, from the files
    r = D.read_restart(str(tmp_path))
    m2 = D.mesh_from_dump(r["mesh"], cyclic_length=mesh.cyclic_length, cartesian=mesh.cartesian)
    f2 = D.dyn_forcing(r["dynamics"], 1.0e-3)
    cfgs, vals, _ = D.step_inputs(r["tracers"])
    TAB = np.ascontiguousarray(r["tracers"].data[0].valuesAB)
    ctx = G.Context(m2, G.PREC_FP64, pass_muscl_init=D.muscl_init_from_dump(r["tracers"]))
    # the oracle on the mesh and state the dumps came from, with the dwarf's dt
    f1 = O.ensure_f64(M.Forcing(uv=f.uv, w=f.w, w_e=f.w_e, w_i=f.w_i, Kv=f.Kv, bc_surface=None, dt=1.0e-3))
    wet = wet_mask(mesh)
    om.do_oce_adv_tra(f1, ocfg, T, TAB)
    dh, dv = ctx.adv_tra(f2, cfgs[0], vals[0], TAB)
    assert np.array_equal(dh[wet], om.work["del_ttf_advhoriz"][wet])
    assert np.array_equal(dv[wet], om.work["del_ttf_advvert"][wet])
    # the dwarf repeats the call on the same state; the library forms the gradients again at
    # every call and gives the same bits.  (The reference's FCT limiter uses edge_up_dn_grad as
    # its scratch array AUX, src/oce_adv_tra_fct.F90:96, so a repeat without init_tracers_AB
    # there runs on the element bounds of the first call in place of the gradients.)
    for _ in range(2):
        dh2, dv2 = ctx.adv_tra(f2, cfgs[0], vals[0], TAB)
        assert np.array_equal(dh2, dh) and np.array_equal(dv2, dv)


def test_tracer_step_from_dumps(tmp_path, pi_file_mesh):
    """The whole FP64 step from the dumped state (Kv from the forcing: it is not in t_dyn)."""
    mesh = pi_file_mesh
    f = O.ensure_f64(M.make_forcing(mesh, "sphere", seed=3, dt=600.0))
    T = np.ascontiguousarray(M.make_tracers(mesh, "sphere", ntr=1, seed=4)[0])
    old = np.ascontiguousarray(T * (1.0 + 1e-3 * np.random.default_rng(2).standard_normal(T.shape)))
    om = O.OracleMesh(mesh)
    _write_dumps(tmp_path, mesh, f, T, old, om)
    r = D.read_restart(str(tmp_path))
    m2 = D.mesh_from_dump(r["mesh"], cyclic_length=mesh.cyclic_length, cartesian=mesh.cartesian)
    fd = D.dyn_forcing(r["dynamics"], 600.0)
    f2 = M.Forcing(uv=fd.uv, w=fd.w, w_e=fd.w_e, w_i=fd.w_i, Kv=f.Kv, bc_surface=f.bc_surface, dt=600.0)
    cfgs, vals, olds = D.step_inputs(r["tracers"])
    ctx = G.Context(m2, G.PREC_FP64, max_tracers=1, pass_muscl_init=D.muscl_init_from_dump(r["tracers"]))
    Tg, Og = [vals[0].copy()], [olds[0].copy()]
    To, Oo = T.copy(), old.copy()
    for _ in range(2):
        ctx.tracer_step(f2, cfgs, Tg, Og)
        om.tracer_step(f, O.cfg_struct(), To, np.zeros_like(To), Oo)
        assert np.array_equal(Tg[0], To)
