"""ctypes front end of the FP64 CPU oracle (test infrastructure only).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module; it is the checker of the CUDA path, never
part of it.  The restatement itself lives in ``tracer_oracle.c`` with
file:line citations of the reference routines it follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

HOR = {"MUSCL": 0, "MFCT": 1, "UPW1": 2}
VER = {"QR4C": 0, "UPW1": 1, "CDIFF": 2, "PPM": 3}

_P = C.c_void_p


class _OrMesh(C.Structure):
    _fields_ = [("nod2D", C.c_int), ("elem2D", C.c_int), ("edge2D", C.c_int), ("nl", C.c_int)] + \
        [(n, _P) for n in ("elem2D_nodes", "edges", "edge_tri", "nod_in_elem2D_ptr", "nod_in_elem2D",
                           "nlevels", "ulevels", "nlevels_nod2D", "ulevels_nod2D", "nlevels_nod2D_min",
                           "ulevels_nod2D_max", "coord_nod2D", "elem_area", "elem_cos", "edge_dxdy",
                           "edge_cross_dxdy", "gradient_sca", "area", "areasvol", "hnode", "hnode_new",
                           "helem", "Z_3d_n", "zbar_3d_n", "zbar_n_bot")] + \
        [("cyclic_length", C.c_double)]


class _OrCfg(C.Structure):
    _fields_ = [("hor", C.c_int), ("ver", C.c_int), ("lim_fct", C.c_int), ("ph", C.c_double),
                ("pv", C.c_double), ("ab_order", C.c_int), ("i_vert_diff", C.c_int), ("wsplit", C.c_int)]


class _OrWork(C.Structure):
    _fields_ = [(n, _P) for n in ("nboundary_lay", "edge_up_dn_tri", "edge_up_dn_grad", "tr_xy", "tr_z",
                                  "fct_LO", "adv_flux_hor", "adv_flux_ver", "fct_ttf_max", "fct_ttf_min",
                                  "fct_plus", "fct_minus", "tvert_max", "tvert_min", "del_ttf",
                                  "del_ttf_advhoriz", "del_ttf_advvert")]


_lib: Optional[C.CDLL] = None


def build() -> str:
    """Compile the oracle with its Makefile (gcc only, seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        for name in ("or_muscl_adv_init", "or_init_tracers_AB", "or_tracer_gradient_elements",
                     "or_fill_up_dn_grad", "or_adv_tra_hor_upw1", "or_adv_tra_hor_muscl", "or_adv_tra_hor_mfct",
                     "or_adv_tra_ver_upw1", "or_adv_tra_ver_qr4c", "or_oce_tra_adv_fct",
                     "or_oce_tra_adv_flux2dtracer", "or_do_oce_adv_tra", "or_diff_ver_part_impl_ale",
                     "or_tracer_step", "or_set_threads", "or_get_threads", "or_tracer_tail",
                     "or_diff_part_hor_redi", "or_diff_ver_part_expl_ale", "or_tracer_step_ex",
                     "or_tracer_gradient_z", "or_tracer_step_redi", "or_diff_part_hor_redi_s",
                     "or_diff_ver_part_redi_expl", "or_redi_k33"):
            getattr(L, name)
        L.or_tracer_step.restype = C.c_int
        L.or_tracer_step_ex.restype = C.c_int
        L.or_tracer_step_redi.restype = C.c_int
        L.or_do_oce_adv_tra.restype = C.c_int
        L.or_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_P)


def cfg_struct(hor="MUSCL", ver="QR4C", lim="FCT", ph=0.0, pv=1.0, ab_order=2, i_vert_diff=True,
               wsplit=False) -> _OrCfg:
    return _OrCfg(HOR[hor], VER[ver], 1 if lim == "FCT" else 0, float(ph), float(pv), int(ab_order),
                  1 if i_vert_diff else 0, 1 if wsplit else 0)


class OracleMesh:
    """Holds contiguous copies of the mesh arrays and the C struct that points at them."""

    def __init__(self, mesh):
        self.mesh = mesh
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self._keep = {
            "elem2D_nodes": i32(mesh.elem2D_nodes), "edges": i32(mesh.edges), "edge_tri": i32(mesh.edge_tri),
            "nod_in_elem2D_ptr": i32(mesh.nod_in_elem2D_ptr), "nod_in_elem2D": i32(mesh.nod_in_elem2D),
            "nlevels": i32(mesh.nlevels), "ulevels": i32(mesh.ulevels), "nlevels_nod2D": i32(mesh.nlevels_nod2D),
            "ulevels_nod2D": i32(mesh.ulevels_nod2D), "nlevels_nod2D_min": i32(mesh.nlevels_nod2D_min),
            "ulevels_nod2D_max": i32(mesh.ulevels_nod2D_max), "coord_nod2D": f64(mesh.coord_nod2D),
            "elem_area": f64(mesh.elem_area), "elem_cos": f64(mesh.elem_cos), "edge_dxdy": f64(mesh.edge_dxdy),
            "edge_cross_dxdy": f64(mesh.edge_cross_dxdy), "gradient_sca": f64(mesh.gradient_sca),
            "area": f64(mesh.area), "areasvol": f64(mesh.areasvol), "hnode": f64(mesh.hnode),
            "hnode_new": f64(mesh.hnode_new), "helem": f64(mesh.helem), "Z_3d_n": f64(mesh.Z_3d_n),
            "zbar_3d_n": f64(mesh.zbar_3d_n), "zbar_n_bot": f64(mesh.zbar_n_bot),
        }
        s = _OrMesh()
        s.nod2D, s.elem2D, s.edge2D, s.nl = mesh.nod2D, mesh.elem2D, mesh.edge2D, mesh.nl
        for k, v in self._keep.items():
            setattr(s, k, v.ctypes.data_as(_P))
        s.cyclic_length = float(mesh.cyclic_length)
        self.s = s
        N2, E2, T2, nl = mesh.nod2D, mesh.edge2D, mesh.elem2D, mesh.nl
        L1 = nl - 1
        z = lambda *shape: np.zeros(shape, dtype=np.float64)
        self.work = {
            "nboundary_lay": np.zeros(N2, np.int32), "edge_up_dn_tri": np.zeros((E2, 2), np.int32),
            "edge_up_dn_grad": z(E2, L1, 4), "tr_xy": z(T2, L1, 2), "tr_z": z(N2, nl),
            "fct_LO": z(N2, L1), "adv_flux_hor": z(E2, L1), "adv_flux_ver": z(N2, nl),
            "fct_ttf_max": z(N2, L1), "fct_ttf_min": z(N2, L1), "fct_plus": z(N2, L1), "fct_minus": z(N2, L1),
            "tvert_max": z(N2, L1), "tvert_min": z(N2, L1), "del_ttf": z(N2, L1),
            "del_ttf_advhoriz": z(N2, L1), "del_ttf_advvert": z(N2, L1),
        }
        w = _OrWork()
        for k, v in self.work.items():
            setattr(w, k, v.ctypes.data_as(_P))
        self.w = w
        lib().or_muscl_adv_init(C.byref(self.s), C.byref(self.w))

    # ---- whole tracer step -------------------------------------------------
    def tracer_step(self, forcing, cfg: _OrCfg, values, valuesAB, valuesold, dt=None) -> None:
        """One per-tracer body of solve_tracers_ale, in place on ``values``/``valuesold``."""
        for a in (values, valuesAB, valuesold):
            assert a.flags.c_contiguous and a.dtype == np.float64
        rc = lib().or_tracer_step(C.byref(self.s), C.byref(cfg), C.c_double(forcing.dt if dt is None else dt),
                                  _ptr(forcing.uv), _ptr(forcing.w), _ptr(forcing.w_i), _ptr(forcing.w_e),
                                  _ptr(forcing.Kv), _ptr(forcing.bc_surface), _ptr(values), _ptr(valuesAB),
                                  _ptr(valuesold), C.byref(self.w))
        if rc != 0:
            raise RuntimeError(f"oracle tracer step failed with status {rc}")

    def tracer_gradient_z(self, values, tr_z) -> None:
        """tracer_gradient_z (src/oce_tracer_mod.F90:192-232) of values into tr_z (nod2D, nl), in place."""
        for a in (values, tr_z):
            assert a.flags.c_contiguous and a.dtype == np.float64
        lib().or_tracer_gradient_z(C.byref(self.s), _ptr(values), _ptr(tr_z))

    def init_tracers_AB(self, cfg, values, valuesAB, valuesold) -> None:
        lib().or_init_tracers_AB(C.byref(self.s), C.byref(cfg), _ptr(values), _ptr(valuesAB), _ptr(valuesold),
                                 C.byref(self.w))

    def do_oce_adv_tra(self, forcing, cfg, values, valuesAB, dt=None) -> None:
        rc = lib().or_do_oce_adv_tra(C.byref(self.s), C.c_double(forcing.dt if dt is None else dt),
                                     _ptr(forcing.uv), _ptr(forcing.w), _ptr(forcing.w_i), _ptr(forcing.w_e),
                                     C.byref(cfg), _ptr(values), _ptr(valuesAB), C.byref(self.w))
        if rc != 0:
            raise RuntimeError(f"oracle do_oce_adv_tra failed with status {rc}")

    def tracer_step_ex(self, forcing, cfg: _OrCfg, values, valuesAB, valuesold, Ki=None, dt=None,
                       slope=None) -> None:
        """tracer_step with the horizontal diffusion of Ki (None: K_hor = 0) and, with the tapered
        neutral slopes ``slope`` (nod2D, nl-1, 3), the Redi terms (Redi = .true.)."""
        for a in (values, valuesAB, valuesold):
            assert a.flags.c_contiguous and a.dtype == np.float64
        ki = None if Ki is None else np.ascontiguousarray(Ki, dtype=np.float64)
        sl = None if slope is None else np.ascontiguousarray(slope, dtype=np.float64)
        rc = lib().or_tracer_step_redi(C.byref(self.s), C.byref(cfg), C.c_double(forcing.dt if dt is None else dt),
                                       _ptr(forcing.uv), _ptr(forcing.w), _ptr(forcing.w_i), _ptr(forcing.w_e),
                                       _ptr(forcing.Kv), _ptr(forcing.bc_surface), _ptr(ki), _ptr(sl),
                                       _ptr(values), _ptr(valuesAB), _ptr(valuesold), C.byref(self.w))
        if rc != 0:
            raise RuntimeError(f"oracle tracer step failed with status {rc}")

    def diff_part_hor_redi(self, dt, Ki, tr_xy, del_ttf, slope=None, tr_z=None) -> None:
        ki = np.ascontiguousarray(Ki, dtype=np.float64)
        sl = None if slope is None else np.ascontiguousarray(slope, dtype=np.float64)
        lib().or_diff_part_hor_redi_s(C.byref(self.s), C.c_double(dt), _ptr(ki), _ptr(sl), _ptr(tr_xy),
                                      _ptr(tr_z), _ptr(del_ttf))

    def diff_ver_part_redi_expl(self, dt, Ki, slope, tr_xy, del_ttf) -> None:
        """diff_ver_part_redi_expl: del_ttf (nod2D, nl-1) += the vertical projection of the
        isoneutral flux, from the element gradients tr_xy (elem2D, nl-1, 2)."""
        ki = np.ascontiguousarray(Ki, dtype=np.float64)
        sl = np.ascontiguousarray(slope, dtype=np.float64)
        lib().or_diff_ver_part_redi_expl(C.byref(self.s), C.c_double(dt), _ptr(ki), _ptr(sl), _ptr(tr_xy),
                                         _ptr(del_ttf))

    def redi_k33(self, Kv, Ki, slope) -> np.ndarray:
        """Kv + Kd s^2 of the implicit solve with Redi, (nod2D, nl)."""
        out = np.empty((self.mesh.nod2D, self.mesh.nl))
        lib().or_redi_k33(C.byref(self.s), _ptr(np.ascontiguousarray(Kv, dtype=np.float64)),
                          _ptr(np.ascontiguousarray(Ki, dtype=np.float64)),
                          _ptr(np.ascontiguousarray(slope, dtype=np.float64)), _ptr(out))
        return out

    def diff_ver_part_expl_ale(self, dt, Kv, flux, values, del_ttf) -> None:
        lib().or_diff_ver_part_expl_ale(C.byref(self.s), C.c_double(dt), _ptr(Kv), _ptr(flux), _ptr(values),
                                        _ptr(del_ttf))

    def diff_ver_part_impl_ale(self, forcing, values, dt=None, wimpl=False) -> None:
        """In place on ``values``; ``wimpl``: with the implicit advection by forcing.w_i."""
        lib().or_diff_ver_part_impl_ale_w(C.byref(self.s), C.c_double(forcing.dt if dt is None else dt),
                                          _ptr(forcing.Kv), _ptr(forcing.bc_surface),
                                          _ptr(forcing.w_i) if wimpl else None, 1 if wimpl else 0, _ptr(values))

    def adv_tra_vert_impl(self, W, values, dt) -> None:
        """adv_tra_vert_impl in place on ``values``."""
        lib().or_adv_tra_vert_impl(C.byref(self.s), C.c_double(dt), _ptr(W), _ptr(values))

    def ver_flux(self, scheme, W, values, dt, flux=None, init_zero=True) -> np.ndarray:
        """One vertical flux routine (UPW1, QR4C with pv = 1, CDIFF, PPM) into flux(nod2D, nl)."""
        m = self.mesh
        out = np.zeros((m.nod2D, m.nl)) if flux is None else flux
        z = 1 if init_zero else 0
        if scheme == "UPW1":
            lib().or_adv_tra_ver_upw1(C.byref(self.s), _ptr(W), _ptr(values), _ptr(out), z)
        elif scheme == "QR4C":
            lib().or_adv_tra_ver_qr4c(C.byref(self.s), _ptr(W), _ptr(values), C.c_double(1.0), _ptr(out), z)
        elif scheme == "CDIFF":
            lib().or_adv_tra_ver_cdiff(C.byref(self.s), _ptr(W), _ptr(values), _ptr(out), z)
        elif scheme == "PPM":
            lib().or_adv_tra_vert_ppm(C.byref(self.s), C.c_double(dt), _ptr(W), _ptr(values), _ptr(out), z)
        else:
            raise ValueError(scheme)
        return out


class TailCfg(C.Structure):
    """or_tail_cfg: the tail of solve_tracers_ale (decay, climatology relaxation, clamps)."""
    _fields_ = [("clim_relax", C.c_double), ("salt_index", C.c_int), ("age_index", C.c_int),
                ("zonal_relax", C.c_int), ("nbins", C.c_int), ("lat0", C.c_double), ("dy", C.c_double),
                ("tau_inv", C.c_double)]


def tail_cfg(clim_relax=1.0 / (10 * 3600.0 * 24), salt_index=1, age_index=-1, zonal_relax=0, nbins=100,
             lat0=0.0, dy=1.0, tau_inv=0.0) -> TailCfg:
    return TailCfg(float(clim_relax), int(salt_index), int(age_index), int(zonal_relax), int(nbins), float(lat0),
                   float(dy), float(tau_inv))


def tracer_tail(om, ids, dt, tc: TailCfg, relax2clim, Tclim, Sclim, ztem, values) -> None:
    """The tail of solve_tracers_ale on the list ``values`` (in place)."""
    for a in values:
        assert a.flags.c_contiguous and a.dtype == np.float64
    n = len(values)
    arr = (_P * n)(*[a.ctypes.data_as(_P) for a in values])
    idv = np.ascontiguousarray(ids, dtype=np.int32)
    lib().or_tracer_tail(C.byref(om.s), C.c_int(n), idv.ctypes.data_as(_P), C.c_double(dt), C.byref(tc),
                         _ptr(relax2clim), _ptr(Tclim), _ptr(Sclim), _ptr(ztem), arr)


def ensure_f64(forcing):
    for k in ("uv", "w", "w_e", "w_i", "Kv", "bc_surface"):
        setattr(forcing, k, np.ascontiguousarray(getattr(forcing, k), dtype=np.float64))
    return forcing
