"""ctypes binding of libfesom_gpu.so (the C ABI in include/fesom_gpu.h).

This module is the Python face of the library: it fills a
``fesom_mesh_desc`` from a :class:`fesom2_gb300.mesh.Mesh` and exposes each
entry point.  There is no CPU fallback: if the shared library cannot be
loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from . import build as _build

_P = C.c_void_p
# the in-tree build, or another build of the same sources named by FESOM_GPU_LIB
LIB_PATH = os.path.abspath(os.environ["FESOM_GPU_LIB"]) if os.environ.get("FESOM_GPU_LIB") else _build.LIB

PREC_FP64, PREC_FP32 = 0, 1
HOR = {"MUSCL": 0, "MFCT": 1, "UPW1": 2}
VER = {"QR4C": 0, "UPW1": 1, "CDIFF": 2, "PPM": 3}
LIM = {"NON": 0, "FCT": 1}
ERRORS = {1: "ARG", 2: "SCHEME", 3: "MESH", 4: "CUDA", 5: "NOMEM", 6: "TIMEOUT", 7: "NUMERIC", 8: "STATE"}
STATUS_NAN, STATUS_FCT_BOUND, STATUS_INDEX = 1, 2, 4
STAGES = ["ab", "trxy", "edge_flux", "node_lo", "bounds", "rpm", "update", "vdiff", "vflux", "vfactors", "lo_ad"]
STAGES_N = len(STAGES)


class TraCfg(C.Structure):
    _fields_ = [("adv_hor", C.c_int32), ("adv_ver", C.c_int32), ("adv_lim", C.c_int32), ("ab_order", C.c_int32),
                ("adv_ph", C.c_double), ("adv_pv", C.c_double), ("i_vert_diff", C.c_int32), ("id", C.c_int32)]


def tra_cfg(hor="MUSCL", ver="QR4C", lim="FCT", ph=0.0, pv=1.0, ab_order=2, i_vert_diff=True, id=1) -> TraCfg:
    """One nml_tracer_list row of namelist.tra (plus AB_order and i_vert_diff)."""
    return TraCfg(HOR[hor], VER[ver], LIM[lim.strip()], int(ab_order), float(ph), float(pv),
                  1 if i_vert_diff else 0, int(id))


class MeshDesc(C.Structure):
    _fields_ = [("nod2D", C.c_int32), ("elem2D", C.c_int32), ("edge2D", C.c_int32), ("nl", C.c_int32),
                ("index_base", C.c_int32), ("ld_nie", C.c_int32)] + \
        [(n, _P) for n in ("elem2D_nodes", "edges", "edge_tri", "nod_in_elem2D_num", "nod_in_elem2D",
                           "nlevels", "ulevels", "nlevels_nod2D", "ulevels_nod2D", "nlevels_nod2D_min",
                           "ulevels_nod2D_max", "coord_nod2D", "elem_area", "elem_cos", "edge_dxdy",
                           "edge_cross_dxdy", "gradient_sca", "area", "areasvol", "hnode", "hnode_new", "helem",
                           "Z_3d_n", "zbar_3d_n", "zbar_n_bot")] + \
        [("cyclic_length", C.c_double), ("nboundary_lay", _P), ("edge_up_dn_tri", _P)]


class TuneResult(C.Structure):
    """``fesom_tune_result``: the FP32 launch settings chosen by ``fesom_gpu_autotune``."""
    _fields_ = [("default_ms", C.c_float), ("tuned_ms", C.c_float), ("candidates", C.c_int32),
                ("stage_tracers", C.c_int32 * 4), ("blocks_per_sm", C.c_int32 * 4), ("variant", C.c_int32 * 4)]


class FesomGpuError(RuntimeError):
    def __init__(self, rc: int, msg: str):
        super().__init__(f"FESOM_ERR_{ERRORS.get(rc, rc)}: {msg}")
        self.rc = rc


_lib: Optional[C.CDLL] = None

_SIGS = {
    "fesom_gpu_abi_version": ([], C.c_int),
    "fesom_gpu_host_alloc": ([C.c_size_t, C.POINTER(_P)], C.c_int),
    "fesom_gpu_host_free": ([_P], C.c_int),
    "fesom_gpu_last_error": ([_P], C.c_char_p),
    "fesom_gpu_init": ([C.POINTER(MeshDesc), C.c_int32, C.c_int32, C.POINTER(_P)], C.c_int),
    "fesom_gpu_finalize": ([_P], C.c_int),
    "fesom_gpu_mesh_check": ([C.POINTER(MeshDesc), _P, _P, C.c_char_p, C.c_int32], C.c_int),
    "fesom_gpu_set_stream": ([_P, _P], C.c_int),
    "fesom_gpu_get_muscl_init": ([_P, _P, _P], C.c_int),
    "fesom_gpu_status": ([_P, C.POINTER(C.c_uint32), C.c_int32], C.c_int),
    "fesom_gpu_update_thickness": ([_P, _P, _P, _P, _P, _P], C.c_int),
    "fesom_gpu_init_tracers_ab": ([_P, C.POINTER(TraCfg), _P, _P, _P], C.c_int),
    "fesom_gpu_adv_tra": ([_P, C.c_double, _P, _P, _P, _P, C.POINTER(TraCfg), _P, _P, _P, _P], C.c_int),
    "fesom_gpu_vdiff_impl": ([_P, C.c_double, C.POINTER(TraCfg), _P, _P, _P], C.c_int),
    "fesom_gpu_tracer_step": ([_P, C.c_int32, C.POINTER(TraCfg), C.c_double, _P, _P, _P, _P, _P, _P,
                               C.POINTER(_P), C.POINTER(_P)], C.c_int),
    "fesom_gpu_state_setup": ([_P, C.c_int32, C.POINTER(TraCfg)], C.c_int),
    "fesom_gpu_forcing_upload": ([_P, _P, _P, _P, _P, _P, _P], C.c_int),
    "fesom_gpu_forcing_upload_f32": ([_P, _P, _P, _P, _P, _P, _P], C.c_int),
    "fesom_gpu_tracer_upload": ([_P, C.c_int32, _P, _P], C.c_int),
    "fesom_gpu_tracer_download": ([_P, C.c_int32, _P, _P], C.c_int),
    "fesom_gpu_tracer_upload_f32": ([_P, C.c_int32, _P, _P], C.c_int),
    "fesom_gpu_tracer_download_f32": ([_P, C.c_int32, _P, _P], C.c_int),
    "fesom_gpu_run_steps": ([_P, C.c_double, C.c_int32, C.c_int32], C.c_int),
    "fesom_gpu_tracer_content": ([_P, _P], C.c_int),
    "fesom_gpu_set_tracers_per_launch": ([_P, C.c_int32], C.c_int),
    "fesom_gpu_set_host_groups": ([_P, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "fesom_gpu_set_tracer_width": ([_P, C.c_int32], C.c_int),
    "fesom_gpu_tracer_groups": ([_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P, _P], C.c_int),
    "fesom_gpu_tracer_gradient_z": ([_P, _P, _P], C.c_int),
    "fesom_gpu_profile_step": ([_P, C.c_double, _P, _P], C.c_int),
    "fesom_gpu_launches_per_step": ([_P, C.POINTER(C.c_int32)], C.c_int),
    "fesom_gpu_debug_fetch": ([_P, C.c_char_p, C.c_int32, _P, C.c_size_t], C.c_int),
    "fesom_gpu_tracer_device_ptr": ([_P, C.c_int32, C.POINTER(_P), C.POINTER(_P)], C.c_int),
    "fesom_gpu_tracer_tail": ([_P, C.c_int32, _P, C.c_double, _P, _P, _P, _P, _P, C.POINTER(_P)], C.c_int),
    "fesom_gpu_set_hdiff": ([_P, _P], C.c_int),
    "fesom_gpu_set_wsplit": ([_P, C.c_int32], C.c_int),
    "fesom_gpu_set_stage_tracers": ([_P, C.c_int32, C.c_int32], C.c_int),
    "fesom_gpu_set_launch_shape": ([_P, C.c_int32, C.c_int32], C.c_int),
    "fesom_gpu_set_stage_variant": ([_P, C.c_int32, C.c_int32], C.c_int),
    "fesom_gpu_autotune": ([_P, C.c_double, C.c_int32, C.POINTER(TuneResult)], C.c_int),
    "fesom_gpu_vdiff_impl_wi": ([_P, C.c_double, C.POINTER(TraCfg), _P, _P, _P, _P], C.c_int),
    "fesom_gpu_diff_hor": ([_P, C.c_double, _P, _P, _P], C.c_int),
    "fesom_gpu_set_redi": ([_P, _P], C.c_int),
    "fesom_gpu_diff_hor_redi": ([_P, C.c_double, _P, _P, _P, _P], C.c_int),
    "fesom_gpu_diff_ver_redi_expl": ([_P, C.c_double, _P, _P, _P, _P], C.c_int),
    "fesom_gpu_redi_k33": ([_P, _P, _P, _P, _P], C.c_int),
    "fesom_gpu_diff_ver_expl": ([_P, C.c_double, _P, _P, _P, _P], C.c_int),
    "fesom_gpu_step_host_f32": ([_P, C.c_double, _P, _P, _P, _P, _P, _P, C.POINTER(_P), C.POINTER(_P),
                                 C.POINTER(_P), C.POINTER(_P)], C.c_int),
    "fesom_gpu_batch_create": ([C.POINTER(_P), C.c_int32, C.POINTER(_P)], C.c_int),
    "fesom_gpu_batch_set_stream": ([_P, _P], C.c_int),
    "fesom_gpu_batch_run_steps": ([_P, C.c_double, C.c_int32, C.c_int32], C.c_int),
    "fesom_gpu_batch_launches_per_step": ([_P, C.POINTER(C.c_int32)], C.c_int),
    "fesom_gpu_batch_last_error": ([_P], C.c_char_p),
    "fesom_gpu_batch_destroy": ([_P], C.c_int),
}


def load(path: Optional[str] = None) -> C.CDLL:
    """Load the shared library (raises if it is missing; no fallback)."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise FileNotFoundError(f"{p} is missing: build it with `python -m fesom2_gb300.build`")
        L = C.CDLL(p)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray]):
    if a is None:
        return None
    return C.c_void_p(a.ctypes.data)


def host_array(shape, dtype=np.float32) -> np.ndarray:
    """A numpy array in page-locked host memory (fesom_gpu_host_alloc), freed when the array and
    every view of it are gone: the host arrays of the host-array steps."""
    import weakref
    L = load()
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    p = _P()
    rc = L.fesom_gpu_host_alloc(max(n, 1), C.byref(p))
    if rc != 0:
        raise FesomGpuError(rc, f"fesom_gpu_host_alloc of {n} bytes failed")
    buf = (C.c_char * max(n, 1)).from_address(p.value)
    weakref.finalize(buf, L.fesom_gpu_host_free, C.c_void_p(p.value))
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)


def _c64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _bc_all(forcing, bc, ntr):
    """Surface term of every tracer, (ntr, nod2D): bc as given, else forcing.bc_surface
    (one term per node) applied to every tracer, else None (zero)."""
    if bc is not None:
        return bc
    b = getattr(forcing, "bc_surface", None)
    if b is None:
        return None
    return np.ascontiguousarray(np.broadcast_to(np.asarray(b), (ntr, np.asarray(b).shape[-1])))


def mesh_desc(mesh, pass_muscl_init=None):
    """Build a ``fesom_mesh_desc`` (and the arrays it points to) for a Mesh."""
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    nie_num = mesh.nod_in_elem2D_num()
    ld = int(nie_num.max())
    nie2 = np.zeros((mesh.nod2D, ld), dtype=np.int32)
    rows = np.repeat(np.arange(mesh.nod2D), nie_num)
    cols = np.arange(mesh.nod_in_elem2D.size) - np.repeat(mesh.nod_in_elem2D_ptr[:-1], nie_num)
    nie2[rows, cols] = mesh.nod_in_elem2D
    keep = dict(
            elem2D_nodes=i32(mesh.elem2D_nodes), edges=i32(mesh.edges), edge_tri=i32(mesh.edge_tri),
            nod_in_elem2D_num=i32(nie_num), nod_in_elem2D=nie2, nlevels=i32(mesh.nlevels),
            ulevels=i32(mesh.ulevels), nlevels_nod2D=i32(mesh.nlevels_nod2D), ulevels_nod2D=i32(mesh.ulevels_nod2D),
            nlevels_nod2D_min=i32(mesh.nlevels_nod2D_min), ulevels_nod2D_max=i32(mesh.ulevels_nod2D_max),
            coord_nod2D=f64(mesh.coord_nod2D), elem_area=f64(mesh.elem_area), elem_cos=f64(mesh.elem_cos),
            edge_dxdy=f64(mesh.edge_dxdy), edge_cross_dxdy=f64(mesh.edge_cross_dxdy),
            gradient_sca=f64(mesh.gradient_sca), area=f64(mesh.area), areasvol=f64(mesh.areasvol),
            hnode=f64(mesh.hnode), hnode_new=f64(mesh.hnode_new), helem=f64(mesh.helem), Z_3d_n=f64(mesh.Z_3d_n),
            zbar_3d_n=f64(mesh.zbar_3d_n), zbar_n_bot=f64(mesh.zbar_n_bot))
    d = MeshDesc()
    d.nod2D, d.elem2D, d.edge2D, d.nl = mesh.nod2D, mesh.elem2D, mesh.edge2D, mesh.nl
    d.index_base = 0
    d.ld_nie = ld
    for k, v in keep.items():
        setattr(d, k, v.ctypes.data)
    d.cyclic_length = float(mesh.cyclic_length)
    if pass_muscl_init is not None:
        nbl, updn = pass_muscl_init
        keep["nbl"] = i32(nbl)
        keep["updn"] = i32(updn)
        d.nboundary_lay = keep["nbl"].ctypes.data
        d.edge_up_dn_tri = keep["updn"].ctypes.data
    return d, keep


def mesh_check(mesh, pass_muscl_init=None):
    """Host-only validation; returns (nboundary_lay, edge_up_dn_tri) 0-based (-1 = none)."""
    L = load()
    d, keep = mesh_desc(mesh, pass_muscl_init)
    nbl = np.zeros(mesh.nod2D, np.int32)
    updn = np.zeros((mesh.edge2D, 2), np.int32)
    buf = C.create_string_buffer(512)
    rc = L.fesom_gpu_mesh_check(C.byref(d), _p(nbl), _p(updn), buf, 512)
    if rc != 0:
        raise FesomGpuError(rc, buf.value.decode())
    return nbl, updn


class Context:
    """One ``fesom_gpu_ctx``: a mesh on the current CUDA device."""

    def __init__(self, mesh, precision: int = PREC_FP64, max_tracers: int = 1, pass_muscl_init=None):
        L = load()
        self.mesh = mesh
        self.prec = precision
        d, self._keep = mesh_desc(mesh, pass_muscl_init)
        self.desc = d
        h = _P()
        rc = L.fesom_gpu_init(C.byref(d), int(precision), int(max_tracers), C.byref(h))
        self.h = h
        if rc != 0:
            msg = L.fesom_gpu_last_error(h).decode() if h.value else "init failed"
            L.fesom_gpu_finalize(h)
            self.h = _P()
            raise FesomGpuError(rc, msg)
        self.L = L

    # -- plumbing -------------------------------------------------------------
    def _chk(self, rc: int):
        if rc != 0:
            raise FesomGpuError(rc, self.L.fesom_gpu_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.fesom_gpu_finalize(self.h)
            self.h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int):
        self._chk(self.L.fesom_gpu_set_stream(self.h, C.c_void_p(stream_handle)))

    def muscl_init(self):
        nbl = np.zeros(self.mesh.nod2D, np.int32)
        updn = np.zeros((self.mesh.edge2D, 2), np.int32)
        self._chk(self.L.fesom_gpu_get_muscl_init(self.h, _p(nbl), _p(updn)))
        return nbl, updn

    def status(self, timeout_ms: int = 60000) -> int:
        s = C.c_uint32(0)
        self._chk(self.L.fesom_gpu_status(self.h, C.byref(s), int(timeout_ms)))
        return int(s.value)

    # -- per-routine drop-ins (FP64) ---------------------------------------------
    def init_tracers_ab(self, cfg: TraCfg, values, valuesAB, valuesold):
        self._chk(self.L.fesom_gpu_init_tracers_ab(self.h, C.byref(cfg), _p(values), _p(valuesAB), _p(valuesold)))

    def tracer_gradient_z(self, values, tr_z=None):
        """tracer_gradient_z of values (nod2D, nl-1) (``fesom_gpu_tracer_gradient_z``); tr_z
        (nod2D, nl) is updated in place (a new zero array when None) and returned."""
        N2, nl = self.mesh.nod2D, self.mesh.nl
        out = np.zeros((N2, nl)) if tr_z is None else tr_z
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.shape != (N2, nl):
            raise ValueError("tr_z must be a C-contiguous float64 (nod2D, nl) array")
        v = _c64(values)
        self._chk(self.L.fesom_gpu_tracer_gradient_z(self.h, _p(v), _p(out)))
        return out

    def adv_tra(self, forcing, cfg: TraCfg, ttf, ttfAB, dt=None):
        N2, L1 = self.mesh.nod2D, self.mesh.nl - 1
        dh = np.zeros((N2, L1))
        dv = np.zeros((N2, L1))
        uv, w, wi, we = _c64(forcing.uv), _c64(forcing.w), _c64(forcing.w_i), _c64(forcing.w_e)
        t64, tab64 = _c64(ttf), _c64(ttfAB)  # alive through the call
        self._chk(self.L.fesom_gpu_adv_tra(self.h, float(forcing.dt if dt is None else dt), _p(uv), _p(w), _p(wi),
                                           _p(we), C.byref(cfg), _p(t64), _p(tab64), _p(dh), _p(dv)))
        return dh, dv

    def vdiff_impl(self, forcing, cfg: TraCfg, values, dt=None, bc=None, wimpl=False):
        """diff_ver_part_impl_ale on ``values`` in place; ``wimpl``: with the w_i terms of a split
        vertical velocity (forcing.w_i)."""
        Kv = _c64(forcing.Kv)
        bcs = _c64(forcing.bc_surface if bc is None else bc)
        wi = _c64(forcing.w_i) if wimpl else None
        self._chk(self.L.fesom_gpu_vdiff_impl_wi(self.h, float(forcing.dt if dt is None else dt), C.byref(cfg),
                                                 _p(Kv), _p(bcs), _p(wi), _p(values)))

    def set_tracer_width(self, width: int):
        """FP32 form: slots per tracer group for the next ``state_setup`` (0: automatic, 2, 4)."""
        self._chk(self.L.fesom_gpu_set_tracer_width(self.h, int(width)))

    def tracer_groups(self):
        """FP32 form: (group count, width, group of each tracer, slot of each tracer)."""
        ng, w = C.c_int32(0), C.c_int32(0)
        g = np.zeros(self.ntr, np.int32)
        c = np.zeros(self.ntr, np.int32)
        self._chk(self.L.fesom_gpu_tracer_groups(self.h, C.byref(ng), C.byref(w), _p(g), _p(c)))
        return int(ng.value), int(w.value), g, c

    def set_stage_tracers(self, stage: int, tracers: int):
        """FP32 form: tracers per launch of stage 0 lo_ad, 1 ho, 2 bounds, 3 update (0: all)."""
        self._chk(self.L.fesom_gpu_set_stage_tracers(self.h, int(stage), int(tracers)))

    def set_launch_shape(self, stage: int, blocks_per_sm: int):
        """FP32 form: at most blocks_per_sm x 152 blocks for stage 0 lo_ad, 1 ho, 2 bounds, 3 update
        (0: one warp per node or edge)."""
        self._chk(self.L.fesom_gpu_set_launch_shape(self.h, int(stage), int(blocks_per_sm)))

    def set_stage_variant(self, stage: int, variant: int):
        """FP32 form: kernel variant of stage 0 lo_ad, 1 ho, 2 bounds, 3 update (bit 0 clear: gathers
        in registers, set: staged in shared memory; stage 3, bit 1: the implicit vertical diffusion
        as its own kernel instead of the update's per-node epilogue)."""
        self._chk(self.L.fesom_gpu_set_stage_variant(self.h, int(stage), int(variant)))

    def autotune(self, dt: float, steps: int = 2) -> dict:
        """FP32 form: time the step under candidate launch settings, keep the fastest
        (fesom_gpu_autotune); the tracer state is left as it was.  Returns the choice and the
        ms per step under the defaults and under the choice."""
        r = TuneResult()
        self._chk(self.L.fesom_gpu_autotune(self.h, float(dt), int(steps), C.byref(r)))
        return {"default_ms": float(r.default_ms), "tuned_ms": float(r.tuned_ms), "candidates": int(r.candidates),
                "stage_tracers": list(r.stage_tracers), "blocks_per_sm": list(r.blocks_per_sm),
                "variant": list(r.variant)}

    def set_wsplit(self, on: bool):
        """dynamics%use_wsplit for every later step (fesom_gpu_set_wsplit)."""
        self._chk(self.L.fesom_gpu_set_wsplit(self.h, 1 if on else 0))

    # -- whole step ------------------------------------------------------------
    def tracer_step(self, forcing, cfgs: Sequence[TraCfg], values: Sequence[np.ndarray],
                    valuesold: Sequence[np.ndarray], dt=None, bc=None):
        n = len(cfgs)
        arr = (TraCfg * n)(*cfgs)
        vp = (_P * n)(*[C.c_void_p(v.ctypes.data) for v in values])
        op = (_P * n)(*[C.c_void_p(v.ctypes.data) for v in valuesold])
        for v in list(values) + list(valuesold):
            assert v.dtype == np.float64 and v.flags.c_contiguous
        uv, w, wi, we, Kv = (_c64(forcing.uv), _c64(forcing.w), _c64(forcing.w_i), _c64(forcing.w_e),
                             _c64(forcing.Kv))
        bcs = _c64(_bc_all(forcing, bc, n))
        self._chk(self.L.fesom_gpu_tracer_step(self.h, n, arr, float(forcing.dt if dt is None else dt), _p(uv),
                                               _p(w), _p(wi), _p(we), _p(Kv), _p(bcs), vp, op))

    # -- device-resident stepping --------------------------------------------------
    def state_setup(self, cfgs: Sequence[TraCfg]):
        n = len(cfgs)
        self._cfgs = (TraCfg * n)(*cfgs)
        self._chk(self.L.fesom_gpu_state_setup(self.h, n, self._cfgs))
        self.ntr = n

    def forcing_upload(self, forcing, bc=None):
        bc = _bc_all(forcing, bc, getattr(self, "ntr", 1))
        if self.prec == PREC_FP32 and forcing.uv.dtype == np.float32:
            f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)
            self._fk = [f(forcing.uv), f(forcing.w), f(forcing.w_i), f(forcing.w_e), f(forcing.Kv), f(bc)]
            self._chk(self.L.fesom_gpu_forcing_upload_f32(self.h, *[_p(a) for a in self._fk]))
        else:
            self._fk = [_c64(forcing.uv), _c64(forcing.w), _c64(forcing.w_i), _c64(forcing.w_e), _c64(forcing.Kv),
                        _c64(bc)]
            self._chk(self.L.fesom_gpu_forcing_upload(self.h, *[_p(a) for a in self._fk]))

    def tracer_upload(self, tr: int, values, valuesold):
        ab = int(self._cfgs[0].ab_order) if getattr(self, "_cfgs", None) else 2
        N2, L1 = self.mesh.nod2D, self.mesh.nl - 1
        if values.size != N2 * L1 or valuesold.size != N2 * L1 * (ab - 1):
            raise ValueError("values must hold (nod2D, nl-1) and valuesold (ab_order-1)*(nod2D, nl-1) entries")
        if values.dtype == np.float32:
            self._chk(self.L.fesom_gpu_tracer_upload_f32(self.h, tr, _p(values), _p(valuesold)))
        else:
            v64, o64 = _c64(values), _c64(valuesold)  # alive through the call
            self._chk(self.L.fesom_gpu_tracer_upload(self.h, tr, _p(v64), _p(o64)))

    def tracer_download(self, tr: int, dtype=np.float64):
        """values (nod2D, nl-1) and valuesold in the reference's layout: (nod2D, nl-1)
        for AB2, (nod2D, nl-1, 2) for AB3 (valuesold(1:2, nz, n))."""
        N2, L1 = self.mesh.nod2D, self.mesh.nl - 1
        ab = int(self._cfgs[0].ab_order) if getattr(self, "_cfgs", None) else 2
        v = np.zeros((N2, L1), dtype=dtype)
        o = np.zeros((N2, L1) if ab == 2 else (N2, L1, ab - 1), dtype=dtype)
        if dtype == np.float32:
            self._chk(self.L.fesom_gpu_tracer_download_f32(self.h, tr, _p(v), _p(o)))
            self.status()
        else:
            self._chk(self.L.fesom_gpu_tracer_download(self.h, tr, _p(v), _p(o)))
        return v, o

    def run_steps(self, dt: float, nsteps: int, use_graph: bool = True):
        self._chk(self.L.fesom_gpu_run_steps(self.h, float(dt), int(nsteps), 1 if use_graph else 0))

    def set_tracers_per_launch(self, n: int):
        self._chk(self.L.fesom_gpu_set_tracers_per_launch(self.h, int(n)))

    def set_host_groups(self, sizes=()):
        """Pipeline stages of ``step_host_f32`` in order, in tracer groups
        (``fesom_gpu_set_host_groups``); an empty sequence restores the default ramp."""
        a = (C.c_int32 * max(1, len(sizes)))(*[int(x) for x in sizes])
        self._chk(self.L.fesom_gpu_set_host_groups(self.h, len(sizes), a))

    def step_host_f32(self, forcing, values_in, valuesold_in, values_out=None, valuesold_out=None):
        """One FP32 step from and to host float32 arrays with the transfers overlapped with the
        compute (``fesom_gpu_step_host_f32``); the outputs default to the inputs (in place)."""
        f = forcing
        for a in (f.uv, f.w, f.w_e, f.Kv):
            if a.dtype != np.float32 or not a.flags.c_contiguous:
                raise ValueError("forcing arrays must be C-contiguous float32")
        n = len(values_in)
        values_out = values_in if values_out is None else values_out
        arrs = [values_in, valuesold_in, values_out] + ([valuesold_out] if valuesold_out is not None else [])
        for lst in arrs:
            for a in lst:
                if a.dtype != np.float32 or not a.flags.c_contiguous:
                    raise ValueError("tracer arrays must be C-contiguous float32")
        mk = lambda lst: (_P * n)(*[a.ctypes.data for a in lst])
        self._chk(self.L.fesom_gpu_step_host_f32(
            self.h, float(f.dt), _p(f.uv), _p(f.w), _p(getattr(f, "w_i", None)), _p(f.w_e), _p(f.Kv),
            _p(f.bc_surface), mk(values_in), mk(valuesold_in), mk(values_out),
            mk(valuesold_out) if valuesold_out is not None else None))

    def tracer_tail(self, cfgs, dt, tc: "TailCfg", relax2clim, Tclim, Sclim, ztem, values):
        """Tail of the tracer loop (``fesom_gpu_tracer_tail``) on the FP64 arrays ``values`` in place."""
        for a in values:
            if a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("tracer arrays must be C-contiguous float64")
        n = len(values)
        arr = (TraCfg * n)(*cfgs)
        vp = (_P * n)(*[a.ctypes.data for a in values])
        keep = [_c64(relax2clim), _c64(Tclim), _c64(Sclim), _c64(ztem)]  # alive through the call
        self._chk(self.L.fesom_gpu_tracer_tail(self.h, n, C.cast(arr, _P), float(dt), C.cast(C.pointer(tc), _P),
                                               *[_p(a) for a in keep], vp))

    def set_hdiff(self, Ki):
        """Horizontal diffusivity Ki(nod2D, nl-1) for every later step (``None``: no horizontal
        diffusion)."""
        self._Ki = None if Ki is None else _c64(Ki)
        self._chk(self.L.fesom_gpu_set_hdiff(self.h, None if self._Ki is None else _p(self._Ki)))

    def set_redi(self, slope):
        """Redi = .true. with the tapered neutral slopes ``slope`` (nod2D, nl-1, 3) for every later
        step (``None``: Redi off); needs set_hdiff first."""
        self._slope = None if slope is None else _c64(slope)
        self._chk(self.L.fesom_gpu_set_redi(self.h, None if self._slope is None else _p(self._slope)))

    def diff_hor(self, dt, Ki, values, del_ttf, slope=None):
        """diff_part_hor_redi alone (FP64): ``del_ttf`` (float64, in place) += the horizontal
        diffusion of ``values`` (with the Redi slope terms when ``slope`` is given)."""
        if del_ttf.dtype != np.float64 or not del_ttf.flags.c_contiguous:
            raise ValueError("del_ttf must be C-contiguous float64")
        keep = [_c64(Ki), _c64(values)]
        if slope is None:
            self._chk(self.L.fesom_gpu_diff_hor(self.h, float(dt), _p(keep[0]), _p(keep[1]), _p(del_ttf)))
        else:
            sl = _c64(slope)
            self._chk(self.L.fesom_gpu_diff_hor_redi(self.h, float(dt), _p(keep[0]), _p(sl), _p(keep[1]),
                                                     _p(del_ttf)))

    def diff_ver_redi_expl(self, dt, Ki, slope, values, del_ttf):
        """diff_ver_part_redi_expl alone (FP64): ``del_ttf`` (float64, in place) += the vertical
        projection of the isoneutral flux of ``values``."""
        if del_ttf.dtype != np.float64 or not del_ttf.flags.c_contiguous:
            raise ValueError("del_ttf must be C-contiguous float64")
        keep = [_c64(Ki), _c64(slope), _c64(values)]
        self._chk(self.L.fesom_gpu_diff_ver_redi_expl(self.h, float(dt), *[_p(a) for a in keep], _p(del_ttf)))

    def redi_k33(self, Kv, Ki, slope):
        """K33 = Kv + Kd s^2 of the implicit solve with Redi (FP64), (nod2D, nl)."""
        out = np.empty(np.shape(Kv), np.float64)
        keep = [_c64(Kv), _c64(Ki), _c64(slope)]
        self._chk(self.L.fesom_gpu_redi_k33(self.h, *[_p(a) for a in keep], _p(out)))
        return out

    def diff_ver_expl(self, dt, Kv, flux_surf, values, del_ttf):
        """diff_ver_part_expl_ale alone (FP64): ``del_ttf`` (float64, in place) += the explicit
        vertical diffusion of ``values``."""
        if del_ttf.dtype != np.float64 or not del_ttf.flags.c_contiguous:
            raise ValueError("del_ttf must be C-contiguous float64")
        keep = [_c64(Kv), _c64(flux_surf), _c64(values)]
        self._chk(self.L.fesom_gpu_diff_ver_expl(self.h, float(dt), *[_p(a) for a in keep], _p(del_ttf)))

    def launches_per_step(self) -> int:
        n = C.c_int32(0)
        self._chk(self.L.fesom_gpu_launches_per_step(self.h, C.byref(n)))
        return int(n.value)

    def profile_step(self, dt: float):
        """One non-graph step with events around each stage: {stage: (ms, launches)}."""
        ms = np.zeros(STAGES_N, np.float32)
        nl = np.zeros(STAGES_N, np.int32)
        self._chk(self.L.fesom_gpu_profile_step(self.h, float(dt), _p(ms), _p(nl)))
        return {STAGES[i]: (float(ms[i]), int(nl[i])) for i in range(STAGES_N)}

    def debug_fetch(self, name: str, tr: int = 0) -> np.ndarray:
        """Internal work array of a tracer slot (FP64 contexts; testing aid)."""
        m = self.mesh
        L1, nl = m.nl - 1, m.nl
        shapes = {"T": (m.nod2D, L1), "Told": (m.nod2D, L1, -1), "TAB": (m.nod2D, L1), "trxy": (m.elem2D, L1, 2),
                  "FLO": (m.edge2D, L1), "ADh": (m.edge2D, L1), "LO": (m.nod2D, L1), "ADv": (m.nod2D, nl),
                  "bmax": (m.nod2D, L1), "bmin": (m.nod2D, L1), "dttf_h": (m.nod2D, L1), "dttf_v": (m.nod2D, L1)}
        n = int(np.prod([abs(x) for x in shapes[name]])) * (3 if name == "Told" else 1)
        out = np.zeros(n)
        self._chk(self.L.fesom_gpu_debug_fetch(self.h, name.encode(), int(tr), _p(out), n))
        if name == "Told":
            return out
        return out.reshape(shapes[name])

    def content(self) -> np.ndarray:
        out = np.zeros(self.ntr)
        self._chk(self.L.fesom_gpu_tracer_content(self.h, _p(out)))
        return out


class TailCfg(C.Structure):
    """``fesom_tail_cfg``: decay, climatology relaxation and clamps after the tracer loop."""
    _fields_ = [("clim_relax", C.c_double), ("salt_index", C.c_int32), ("age_index", C.c_int32),
                ("zonal_relax", C.c_int32), ("nbins", C.c_int32), ("lat0", C.c_double), ("dy", C.c_double),
                ("tau_inv", C.c_double)]


def tail_cfg(clim_relax=1.0 / (10 * 3600.0 * 24), salt_index=1, age_index=-1, zonal_relax=0, nbins=100,
             lat0=0.0, dy=1.0, tau_inv=0.0) -> TailCfg:
    return TailCfg(float(clim_relax), int(salt_index), int(age_index), int(zonal_relax), int(nbins), float(lat0),
                   float(dy), float(tau_inv))


class Batch:
    """``fesom_gpu_batch``: FP32 contexts stepped together, one launch per stage over all of
    them (each context set up with ``state_setup`` and ``forcing_upload`` first)."""

    def __init__(self, contexts):
        L = load()
        self.L = L
        self.contexts = list(contexts)  # the batch points into them: keep them alive
        arr = (_P * len(self.contexts))(*[c.h for c in self.contexts])
        h = _P()
        rc = L.fesom_gpu_batch_create(arr, len(self.contexts), C.byref(h))
        self.h = h
        if rc != 0:
            msg = L.fesom_gpu_batch_last_error(h).decode() if h.value else "batch create failed"
            L.fesom_gpu_batch_destroy(h)
            self.h = _P()
            raise FesomGpuError(rc, msg)

    def _chk(self, rc: int):
        if rc != 0:
            raise FesomGpuError(rc, self.L.fesom_gpu_batch_last_error(self.h).decode())

    def set_stream(self, stream: int):
        self._chk(self.L.fesom_gpu_batch_set_stream(self.h, _P(stream)))

    def run_steps(self, dt: float, nsteps: int, use_graph: bool = True):
        self._chk(self.L.fesom_gpu_batch_run_steps(self.h, float(dt), int(nsteps), 1 if use_graph else 0))

    def launches_per_step(self) -> int:
        n = C.c_int32(0)
        self._chk(self.L.fesom_gpu_batch_launches_per_step(self.h, C.byref(n)))
        return int(n.value)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.fesom_gpu_batch_destroy(self.h)
            self.h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

