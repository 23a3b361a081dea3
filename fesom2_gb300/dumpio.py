"""Reader (and writer) of the reference's derived-type binary restarts -- the files the dwarf
harness reads its state from (dwarf_ini/fesom.F90:64; src/io_restart_derivedtype.F90):
``t_mesh.<rank>``, ``t_partit.<rank>``, ``t_dynamics.<rank>`` and ``t_tracer.<rank>`` in
``<resultpath>/fesom_bin_restart/np<npes>/``.

Each file is written by ONE unformatted sequential ``write(unit) <derived type>`` whose
defined-I/O procedure (``generic :: write(unformatted)``) issues the field writes as child
data transfer statements.  Child statements do not start records, so the whole dump is a
single Fortran record: the fields one after another with no inner markers, framed by the
4-byte little-endian length markers of a sequential file (a record above 2 GiB - 9 bytes is
split into subrecords, as gfortran writes them: the leading marker of every subrecord but
the last is negative, and so is the trailing marker of every subrecord but the first).
Arrays go through ``write_bin_array`` (src/MOD_WRITE_BINARY_ARRAYS.F90): the extents (int32
each), then the elements in column-major order; an unallocated array writes zero extents
and no elements.

Layouts (field order of the writers):
  * ``WRITE_T_TRACER`` (src/MOD_TRACER.F90:211-230): num_tracers; per tracer values(nl-1,
    nod2D), valuesold(AB_order-1, nl-1, nod2D), valuesAB, smooth_bh_tra (logical),
    gamma0/1/2_tra, i_vert_diff (logical), tra_adv_hor/ver/lim (character(20)), tra_adv_ph,
    tra_adv_pv, ID; then the work arrays (``WORK_FIELDS``).
  * ``write_t_mesh`` (src/MOD_MESH.F90:180-274): ``MESH_FIELDS``.
  * ``WRITE_T_DYN`` (src/MOD_DYN.F90:290-346): ``DYN_HEAD``, the solver info, the work
    arrays, uv ... cfl_z, then fer_w/fer_uv when Fer_GM is on and the split-explicit arrays
    when use_ssh_se_subcycl is.
  * ``WRITE_T_PARTIT`` (src/MOD_PARTIT.F90:165-195): three communication structures, then
    npes, mype, maxPEnum, part, and the owned/halo sizes and lists.

Arrays come back in this package's (row-major) layout: a Fortran array a(level, node) is
returned as a numpy array of shape (node, level), the same memory.
"""
from __future__ import annotations

import dataclasses
import math
import os
import struct
from typing import BinaryIO, Dict, List, Optional

import numpy as np

_MAX_SUB = 2 ** 31 - 9  # largest subrecord gfortran writes

# ---------------------------------------------------------------------------
# field tables: (name, kind) with kind "i4" / "f8" / "L4" (a scalar) or ("i4" | "f8", rank)
# ---------------------------------------------------------------------------
WORK_FIELDS = [("del_ttf", "f8", 2), ("del_ttf_advhoriz", "f8", 2), ("del_ttf_advvert", "f8", 2),
               ("dvd_trflx_hor", "f8", 3), ("dvd_trflx_ver", "f8", 3), ("fct_LO", "f8", 2),
               ("adv_flux_hor", "f8", 2), ("adv_flux_ver", "f8", 2), ("fct_ttf_max", "f8", 2),
               ("fct_ttf_min", "f8", 2), ("fct_plus", "f8", 2), ("fct_minus", "f8", 2),
               ("nboundary_lay", "i4", 1), ("edge_up_dn_tri", "i4", 2), ("edge_up_dn_grad", "f8", 3)]

MESH_FIELDS = [
    ("nod2D", "i4"), ("ocean_area", "f8"), ("ocean_areawithcav", "f8"), ("edge2D", "i4"), ("edge2D_in", "i4"),
    ("elem2D", "i4"), ("elem2D_nodes", ("i4", 2)), ("edges", ("i4", 2)), ("edge_tri", ("i4", 2)),
    ("elem_edges", ("i4", 2)), ("elem_area", ("f8", 1)), ("edge_dxdy", ("f8", 2)), ("edge_cross_dxdy", ("f8", 2)),
    ("elem_cos", ("f8", 1)), ("metric_factor", ("f8", 1)), ("elem_neighbors", ("i4", 2)),
    ("nod_in_elem2D", ("i4", 2)), ("x_corners", ("f8", 2)), ("y_corners", ("f8", 2)),
    ("nod_in_elem2D_num", ("i4", 1)), ("depth", ("f8", 1)), ("gradient_vec", ("f8", 2)),
    ("gradient_sca", ("f8", 2)), ("bc_index_nod2D", ("i4", 1)), ("nl", "i4"), ("zbar", ("f8", 1)),
    ("Z", ("f8", 1)), ("elem_depth", ("f8", 1)), ("ulevels", ("i4", 1)), ("ulevels_nod2D", ("i4", 1)),
    ("ulevels_nod2D_max", ("i4", 1)), ("nlevels", ("i4", 1)), ("nlevels_nod2D", ("i4", 1)),
    ("nlevels_nod2D_min", ("i4", 1)), ("area", ("f8", 2)), ("area_inv", ("f8", 2)), ("areasvol", ("f8", 2)),
    ("areasvol_inv", ("f8", 2)), ("mesh_resolution", ("f8", 1)), ("cavity_flag_n", ("i4", 1)),
    ("cavity_flag_e", ("i4", 1)), ("cavity_depth", ("f8", 1)), ("cavity_nrst_cavlpnt_xyz", ("f8", 2)),
    ("ssh_stiff_dim", "i4"), ("ssh_stiff_nza", "i4"), ("ssh_stiff_rowptr", ("i4", 1)),
    ("ssh_stiff_colind", ("i4", 1)), ("ssh_stiff_values", ("f8", 1)), ("ssh_stiff_colind_loc", ("i4", 1)),
    ("ssh_stiff_rowptr_loc", ("i4", 1)), ("lump2d_south", ("f8", 1)), ("lump2d_north", ("f8", 1)),
    ("ind_south", ("i4", 1)), ("ind_north", ("i4", 1)), ("nn_size", "i4"), ("nn_num", ("i4", 1)),
    ("nn_pos", ("i4", 2)), ("hnode", ("f8", 2)), ("hnode_new", ("f8", 2)), ("zbar_3d_n", ("f8", 2)),
    ("Z_3d_n", ("f8", 2)), ("Z_3d_n_ib", ("f8", 2)), ("helem", ("f8", 2)), ("bottom_elem_thickness", ("f8", 1)),
    ("bottom_node_thickness", ("f8", 1)), ("dhe", ("f8", 1)), ("hbar", ("f8", 1)), ("hbar_old", ("f8", 1)),
    ("zbar_n_bot", ("f8", 1)), ("zbar_e_bot", ("f8", 1)), ("zbar_n_srf", ("f8", 1)), ("zbar_e_srf", ("f8", 1)),
    ("coriolis", ("f8", 1)), ("coriolis_node", ("f8", 1)),
]

DYN_HEAD = [("opt_visc", "i4"), ("visc_gamma0", "f8"), ("visc_gamma1", "f8"), ("visc_gamma2", "f8"),
            ("visc_easybsreturn", "f8"), ("use_ivertvisc", "L4"), ("momadv_opt", "i4"), ("use_freeslip", "L4"),
            ("use_wsplit", "L4"), ("wsplit_maxcfl", "f8"), ("use_ssh_se_subcycl", "L4"),
            # T_SOLVERINFO (src/MOD_DYN.F90:212-230)
            ("solver_ident", "i4"), ("solver_maxiter", "i4"), ("solver_restart", "i4"), ("solver_fillin", "i4"),
            ("solver_lutype", "i4"), ("solver_droptol", "f8"), ("solver_soltol", "f8"), ("solver_rr", ("f8", 1)),
            ("solver_zz", ("f8", 1)), ("solver_pp", ("f8", 1)), ("solver_App", ("f8", 1)),
            # T_DYN_WORK (src/MOD_DYN.F90:260-271)
            ("work_uvnode_rhs", ("f8", 3)), ("work_u_c", ("f8", 2)), ("work_v_c", ("f8", 2)),
            ("work_u_b", ("f8", 2)), ("work_v_b", ("f8", 2)),
            ("uv", ("f8", 3)), ("uv_rhs", ("f8", 3)), ("uv_rhsAB", ("f8", 4)), ("uvnode", ("f8", 3)),
            ("w", ("f8", 2)), ("w_e", ("f8", 2)), ("w_i", ("f8", 2)), ("cfl_z", ("f8", 2))]
DYN_FER = [("fer_w", ("f8", 2)), ("fer_uv", ("f8", 3))]
DYN_SE = [("se_uvh", ("f8", 3)), ("se_uvBT_rhs", ("f8", 2)), ("se_uvBT_4AB", ("f8", 2)), ("se_uvBT", ("f8", 2)),
          ("se_uvBT_theta", ("f8", 2)), ("se_uvBT_mean", ("f8", 2)), ("se_uvBT_12", ("f8", 2)),
          ("se_uvBT_stab_hvisc", ("f8", 2)), ("se_uvBT_stab_bdrag", ("f8", 1))]

# COM_STRUCT (src/MOD_PARTIT.F90:124-142); rPE / rptr / sPE / sptr are static arrays written
# with their size like a rank-1 array
COM_FIELDS = [("rPEnum", "i4"), ("rPE", ("i4", 1)), ("rptr", ("i4", 1)), ("rlist", ("i4", 1)), ("sPEnum", "i4"),
              ("sPE", ("i4", 1)), ("sptr", ("i4", 1)), ("slist", ("i4", 1)), ("nreq", "i4")]
PARTIT_FIELDS = [("npes", "i4"), ("mype", "i4"), ("maxPEnum", "i4"), ("part", ("i4", 1)), ("myDim_nod2D", "i4"),
                 ("eDim_nod2D", "i4"), ("myList_nod2D", ("i4", 1)), ("myDim_elem2D", "i4"), ("eDim_elem2D", "i4"),
                 ("eXDim_elem2D", "i4"), ("myList_elem2D", ("i4", 1)), ("myDim_edge2D", "i4"),
                 ("eDim_edge2D", "i4"), ("myList_edge2D", ("i4", 1)), ("pe_status", "i4")]
COM_NAMES = ("com_nod2D", "com_elem2D", "com_elem2D_full")


# ---------------------------------------------------------------------------
# one sequential record, and a cursor over its payload
# ---------------------------------------------------------------------------
def read_record(f: BinaryIO) -> bytes:
    """The payload of the next record, its subrecords joined."""
    out = []
    first = True
    while True:
        head = f.read(4)
        if len(head) < 4:
            raise EOFError("end of file inside a record")
        n = struct.unpack("<i", head)[0]
        body = f.read(abs(n))
        t = f.read(4)
        if len(body) != abs(n) or len(t) < 4:
            raise EOFError("end of file inside a record")
        tail = struct.unpack("<i", t)[0]
        # the trailing marker is negative exactly for the subrecords after the first
        if abs(tail) != abs(n) or (tail < 0) == first:
            raise ValueError("corrupt record markers")
        out.append(body)
        first = False
        if n >= 0:
            return b"".join(out)


def write_record(f: BinaryIO, b: bytes) -> None:
    """One record; above the subrecord limit in gfortran's subrecords."""
    if len(b) <= _MAX_SUB:
        f.write(struct.pack("<i", len(b)) + b + struct.pack("<i", len(b)))
        return
    pos, first = 0, True
    while pos < len(b):
        chunk = b[pos:pos + _MAX_SUB]
        last = pos + len(chunk) >= len(b)
        f.write(struct.pack("<i", len(chunk) if last else -len(chunk)) + chunk +
                struct.pack("<i", len(chunk) if first else -len(chunk)))
        pos += len(chunk)
        first = False


class Payload:
    """Cursor over the fields of a dump record, read in the writer's order."""

    def __init__(self, b: bytes):
        self.b = b
        self.pos = 0

    def take(self, n: int) -> bytes:
        if n < 0 or self.pos + n > len(self.b):
            raise ValueError(f"field of {n} bytes past the end of the record ({len(self.b) - self.pos} left)")
        out = self.b[self.pos:self.pos + n]
        self.pos += n
        return out

    def left(self) -> int:
        return len(self.b) - self.pos

    def scalar(self, kind: str):
        if kind == "L4":
            return struct.unpack("<i", self.take(4))[0] != 0
        fmt = {"i4": "<i", "f8": "<d"}[kind]
        return struct.unpack(fmt, self.take(struct.calcsize(fmt)))[0]

    def chars(self, n: int) -> str:
        return self.take(n).decode("ascii").rstrip()

    def array(self, dtype: str, rank: int) -> Optional[np.ndarray]:
        dims = struct.unpack(f"<{rank}i", self.take(4 * rank))
        if any(d < 0 for d in dims):
            raise ValueError(f"negative extent {dims}")
        if all(d == 0 for d in dims):
            return None
        n = int(np.prod(dims))
        data = np.frombuffer(self.take(n * np.dtype(dtype).itemsize), dtype="<" + dtype)
        # Fortran a(d1, ..., dk) column-major == row-major shape (dk, ..., d1)
        return data.reshape(tuple(reversed(dims))).copy()

    def field(self, kind):
        return self.scalar(kind) if isinstance(kind, str) else self.array(*kind)

    def fields(self, table) -> Dict[str, object]:
        return {name: self.field(kind) for name, kind in table}

    def done(self) -> None:
        if self.left():
            raise ValueError(f"{self.left()} bytes left in the record after the last field")


class PayloadWriter:
    """The writer's side of ``Payload``: fields appended in order, one record at the end."""

    def __init__(self):
        self.parts: List[bytes] = []

    def scalar(self, kind: str, v) -> None:
        if kind == "L4":
            self.parts.append(struct.pack("<i", 1 if v else 0))
        else:
            self.parts.append(struct.pack({"i4": "<i", "f8": "<d"}[kind], v))

    def chars(self, s: str, n: int) -> None:
        self.parts.append(s.ljust(n)[:n].encode("ascii"))

    def array(self, a: Optional[np.ndarray], dtype: str, rank: int) -> None:
        if a is None:
            self.parts.append(struct.pack(f"<{rank}i", *([0] * rank)))
            return
        a = np.ascontiguousarray(a, dtype="<" + dtype)
        if a.ndim != rank:
            raise ValueError(f"rank-{rank} array expected, got shape {a.shape}")
        self.parts.append(struct.pack(f"<{rank}i", *reversed(a.shape)))
        self.parts.append(a.tobytes())

    def field(self, kind, v) -> None:
        if isinstance(kind, str):
            self.scalar(kind, v)
        else:
            self.array(v, *kind)

    def fields(self, table, values: Dict[str, object]) -> None:
        for name, kind in table:
            self.field(kind, values.get(name, None if not isinstance(kind, str) else 0))

    def write(self, path: str) -> None:
        with open(path, "wb") as f:
            write_record(f, b"".join(self.parts))


def read_dump(path: str) -> Payload:
    """The single record of a derived-type dump."""
    with open(path, "rb") as f:
        b = read_record(f)
        if f.read(1):
            raise ValueError("bytes left after the dump's record")
    return Payload(b)


# ---------------------------------------------------------------------------
# t_tracer
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class TracerData:
    values: np.ndarray            # (nod2D, nl-1)
    valuesold: np.ndarray         # (nod2D, nl-1, AB_order-1)
    valuesAB: Optional[np.ndarray]
    smooth_bh_tra: bool
    gamma0_tra: float
    gamma1_tra: float
    gamma2_tra: float
    i_vert_diff: bool
    tra_adv_hor: str
    tra_adv_ver: str
    tra_adv_lim: str
    tra_adv_ph: float
    tra_adv_pv: float
    ID: int

    @property
    def ab_order(self) -> int:
        return self.valuesold.shape[-1] + 1


@dataclasses.dataclass
class Tracers:
    data: List[TracerData]
    work: Dict[str, Optional[np.ndarray]]


def read_tracers(path: str) -> Tracers:
    """READ_T_TRACER (src/MOD_TRACER.F90:233-254)."""
    p = read_dump(path)
    n = p.scalar("i4")
    if n < 0:
        raise ValueError("negative tracer count")
    data = []
    for _ in range(n):
        values = p.array("f8", 2)
        valuesold = p.array("f8", 3)
        valuesAB = p.array("f8", 2)
        smooth = p.scalar("L4")
        g0, g1, g2 = p.scalar("f8"), p.scalar("f8"), p.scalar("f8")
        ivd = p.scalar("L4")
        hor, ver, lim = p.chars(20), p.chars(20), p.chars(20)
        ph, pv = p.scalar("f8"), p.scalar("f8")
        tid = p.scalar("i4")
        data.append(TracerData(values, valuesold, valuesAB, smooth, g0, g1, g2, ivd, hor, ver, lim, ph, pv, tid))
    work = {name: p.array(dt, rank) for name, dt, rank in WORK_FIELDS}
    p.done()
    return Tracers(data, work)


def write_tracers(path: str, tr: Tracers) -> None:
    """WRITE_T_TRACER (src/MOD_TRACER.F90:211-230): the layout ``read_tracers`` reads."""
    w = PayloadWriter()
    w.scalar("i4", len(tr.data))
    for d in tr.data:
        w.array(d.values, "f8", 2)
        w.array(d.valuesold, "f8", 3)
        w.array(d.valuesAB, "f8", 2)
        w.scalar("L4", d.smooth_bh_tra)
        for g in (d.gamma0_tra, d.gamma1_tra, d.gamma2_tra):
            w.scalar("f8", g)
        w.scalar("L4", d.i_vert_diff)
        for s in (d.tra_adv_hor, d.tra_adv_ver, d.tra_adv_lim):
            w.chars(s, 20)
        w.scalar("f8", d.tra_adv_ph)
        w.scalar("f8", d.tra_adv_pv)
        w.scalar("i4", d.ID)
    for name, dt, rank in WORK_FIELDS:
        w.array(tr.work.get(name), dt, rank)
    w.write(path)


def step_inputs(tr: Tracers):
    """The tracer configurations and state of a dump in the form the step entry points take:
    (tra_cfg list, values list (nod2D, nl-1), valuesold list (nod2D, nl-1[, AB_order-1]))."""
    from . import gpu as G
    cfgs, vals, olds = [], [], []
    for d in tr.data:
        # any limiter string but 'FCT' means no limiter (oce_adv_tra_driver.F90:111)
        lim = "FCT" if d.tra_adv_lim.strip() == "FCT" else "NON"
        c = G.tra_cfg(d.tra_adv_hor.strip(), d.tra_adv_ver.strip(), lim, d.tra_adv_ph, d.tra_adv_pv,
                      ab_order=d.ab_order, i_vert_diff=d.i_vert_diff, id=d.ID)
        cfgs.append(c)
        vals.append(np.ascontiguousarray(d.values))
        o = d.valuesold
        olds.append(np.ascontiguousarray(o[..., 0] if o.shape[-1] == 1 else o))
    return cfgs, vals, olds


# ---------------------------------------------------------------------------
# t_mesh, t_dynamics, t_partit
# ---------------------------------------------------------------------------
def read_mesh_dump(path: str) -> Dict[str, object]:
    """read_t_mesh (src/MOD_MESH.F90:277-371): every field by its name in ``MESH_FIELDS``."""
    p = read_dump(path)
    out = p.fields(MESH_FIELDS)
    p.done()
    return out


def write_mesh_dump(path: str, fields: Dict[str, object]) -> None:
    w = PayloadWriter()
    w.fields(MESH_FIELDS, fields)
    w.write(path)


def read_dyn_dump(path: str, fer_gm: Optional[bool] = None) -> Dict[str, object]:
    """READ_T_DYN (src/MOD_DYN.F90:348-403).  Whether the GM arrays follow cfl_z is a namelist
    switch (Fer_GM) the dump does not hold: None takes them when bytes remain for them."""
    p = read_dump(path)
    out = p.fields(DYN_HEAD)
    se = bool(out["use_ssh_se_subcycl"])
    if fer_gm is None:
        fer_gm = p.left() > 0 and not se
        if se and p.left() > 0:
            # with the split-explicit arrays also present: take the GM pair when it parses
            # and leaves exactly the split-explicit arrays
            save = p.pos
            try:
                p.fields(DYN_FER)
                p.fields(DYN_SE)
                fer_gm = p.left() == 0
            except ValueError:
                fer_gm = False
            p.pos = save
    if fer_gm:
        out.update(p.fields(DYN_FER))
    if se:
        out.update(p.fields(DYN_SE))
    p.done()
    return out


def write_dyn_dump(path: str, fields: Dict[str, object], fer_gm: bool = False) -> None:
    w = PayloadWriter()
    w.fields(DYN_HEAD, fields)
    if fer_gm:
        w.fields(DYN_FER, fields)
    if fields.get("use_ssh_se_subcycl"):
        w.fields(DYN_SE, fields)
    w.write(path)


def read_partit_dump(path: str) -> Dict[str, object]:
    """READ_T_PARTIT (src/MOD_PARTIT.F90:197-227)."""
    p = read_dump(path)
    out: Dict[str, object] = {c: p.fields(COM_FIELDS) for c in COM_NAMES}
    out.update(p.fields(PARTIT_FIELDS))
    p.done()
    return out


def write_partit_dump(path: str, fields: Dict[str, object]) -> None:
    w = PayloadWriter()
    for c in COM_NAMES:
        w.fields(COM_FIELDS, fields.get(c, {}))
    w.fields(PARTIT_FIELDS, fields)
    w.write(path)


def rank_suffix(rank: int, npes: int) -> str:
    """mpirank_to_txt (src/fortran_utils.F90:45-56): the rank zero-padded to the digits of npes."""
    return str(rank).zfill(int(math.log10(npes)) + 1)


def read_restart(path: str, npes: int = 1, rank: int = 0) -> Dict[str, object]:
    """The derived-type dumps of one rank in ``path`` (``.../fesom_bin_restart/np<npes>``):
    whichever of t_mesh, t_partit, t_dynamics and t_tracer are present."""
    sfx = rank_suffix(rank, npes)
    out: Dict[str, object] = {}
    for key, name, fn in (("mesh", "t_mesh", read_mesh_dump), ("partit", "t_partit", read_partit_dump),
                          ("dynamics", "t_dynamics", read_dyn_dump), ("tracers", "t_tracer", read_tracers)):
        f = os.path.join(path, f"{name}.{sfx}")
        if os.path.exists(f):
            out[key] = fn(f)
    return out


# ---------------------------------------------------------------------------
# the dumps as the step's inputs
# ---------------------------------------------------------------------------
def mesh_from_dump(tm: Dict[str, object], partit: Optional[Dict[str, object]] = None,
                   cyclic_length: float = 2.0 * math.pi, cartesian: bool = False, name: str = "dump"):
    """A ``Mesh`` from the fields of a t_mesh dump.  The path runs on the whole mesh, so the dump
    must be that of one rank owning everything (npes = 1, no halo).  The dump holds no node
    coordinates: the mesh's coordinates are zero, and the MUSCL set-up (nboundary_lay,
    edge_up_dn_tri) comes from the tracer dump's work arrays (``muscl_init_from_dump``)."""
    from . import mesh as M
    if partit is not None and (partit["npes"] != 1 or partit["eDim_nod2D"] != 0):
        raise ValueError("a partitioned dump: the tracer step runs on the whole mesh (npes = 1)")
    N2, T2, E2, nl = int(tm["nod2D"]), int(tm["elem2D"]), int(tm["edge2D"]), int(tm["nl"])
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    need = ("elem2D_nodes", "edges", "edge_tri", "nod_in_elem2D", "nod_in_elem2D_num", "elem_area", "elem_cos",
            "edge_dxdy", "edge_cross_dxdy", "gradient_sca", "area", "areasvol", "hnode", "hnode_new", "helem",
            "zbar", "Z", "zbar_3d_n", "Z_3d_n", "zbar_n_bot", "nlevels", "ulevels", "nlevels_nod2D",
            "ulevels_nod2D", "nlevels_nod2D_min", "ulevels_nod2D_max")
    missing = [k for k in need if tm.get(k) is None]
    if missing:
        raise ValueError(f"t_mesh dump without {', '.join(missing)}")
    tri = i32(tm["elem2D_nodes"])[:T2, :3] - 1
    edges = i32(tm["edges"])[:E2, :2] - 1
    etri = i32(tm["edge_tri"])[:E2, :2]
    etri = np.where(etri <= 0, -1, etri - 1).astype(np.int32)
    num = i32(tm["nod_in_elem2D_num"])[:N2]
    nie = i32(tm["nod_in_elem2D"])  # (nod2D, maxK) row-major view of nod_in_elem2D(maxK, nod2D)
    ptr = np.zeros(N2 + 1, np.int32)
    ptr[1:] = np.cumsum(num)
    # the first num(n) entries of every column nod_in_elem2D(:, n), in order
    lists = nie[:N2][np.arange(nie.shape[1])[None, :] < num[:, None]] - 1
    return M.Mesh(
        nl=nl, coord_nod2D=np.zeros((N2, 2)), elem2D_nodes=i32(tri), edges=i32(edges), edge_tri=etri,
        edge2D_in=int(tm["edge2D_in"]), nod_in_elem2D_ptr=ptr, nod_in_elem2D=i32(lists),
        nlevels=i32(tm["nlevels"])[:T2], ulevels=i32(tm["ulevels"])[:T2],
        nlevels_nod2D=i32(tm["nlevels_nod2D"])[:N2], ulevels_nod2D=i32(tm["ulevels_nod2D"])[:N2],
        nlevels_nod2D_min=i32(tm["nlevels_nod2D_min"])[:N2], ulevels_nod2D_max=i32(tm["ulevels_nod2D_max"])[:N2],
        elem_area=f64(tm["elem_area"])[:T2], elem_cos=f64(tm["elem_cos"])[:T2],
        edge_dxdy=f64(tm["edge_dxdy"])[:E2], edge_cross_dxdy=f64(tm["edge_cross_dxdy"])[:E2],
        gradient_sca=f64(tm["gradient_sca"])[:T2], area=f64(tm["area"])[:N2], areasvol=f64(tm["areasvol"])[:N2],
        hnode=f64(tm["hnode"])[:N2], hnode_new=f64(tm["hnode_new"])[:N2], helem=f64(tm["helem"])[:T2],
        zbar=f64(tm["zbar"]), Z=f64(tm["Z"]), zbar_3d_n=f64(tm["zbar_3d_n"])[:N2], Z_3d_n=f64(tm["Z_3d_n"])[:N2],
        zbar_n_bot=f64(tm["zbar_n_bot"])[:N2], cyclic_length=float(cyclic_length), cartesian=bool(cartesian),
        name=name)


def dump_from_mesh(mesh) -> Dict[str, object]:
    """The t_mesh dump fields a ``Mesh`` holds (1-based indices, the reference's layouts); the
    fields the tracer step does not read are left unallocated."""
    N2, T2, E2 = mesh.nod2D, mesh.elem2D, mesh.edge2D
    num = mesh.nod_in_elem2D_num()
    maxk = int(num.max()) if N2 else 0
    nie = np.zeros((N2, maxk), np.int32)
    nie[np.arange(maxk)[None, :] < num[:, None]] = mesh.nod_in_elem2D + 1
    etri = np.where(mesh.edge_tri < 0, 0, mesh.edge_tri + 1).astype(np.int32)
    out: Dict[str, object] = {
        "nod2D": N2, "ocean_area": float(np.sum(mesh.area[:, 0])), "ocean_areawithcav": float(np.sum(mesh.area[:, 0])),
        "edge2D": E2, "edge2D_in": int(mesh.edge2D_in), "elem2D": T2,
        "elem2D_nodes": mesh.elem2D_nodes + 1, "edges": mesh.edges + 1, "edge_tri": etri,
        "elem_area": mesh.elem_area, "edge_dxdy": mesh.edge_dxdy, "edge_cross_dxdy": mesh.edge_cross_dxdy,
        "elem_cos": mesh.elem_cos, "nod_in_elem2D": nie, "nod_in_elem2D_num": num, "gradient_sca": mesh.gradient_sca,
        "nl": int(mesh.nl), "zbar": mesh.zbar, "Z": mesh.Z, "ulevels": mesh.ulevels,
        "ulevels_nod2D": mesh.ulevels_nod2D, "ulevels_nod2D_max": mesh.ulevels_nod2D_max, "nlevels": mesh.nlevels,
        "nlevels_nod2D": mesh.nlevels_nod2D, "nlevels_nod2D_min": mesh.nlevels_nod2D_min, "area": mesh.area,
        "areasvol": mesh.areasvol, "hnode": mesh.hnode, "hnode_new": mesh.hnode_new, "zbar_3d_n": mesh.zbar_3d_n,
        "Z_3d_n": mesh.Z_3d_n, "helem": mesh.helem, "zbar_n_bot": mesh.zbar_n_bot,
    }
    return out


def muscl_init_from_dump(tr: Tracers):
    """(nboundary_lay, edge_up_dn_tri) of a tracer dump's work arrays in the form
    ``gpu.Context(pass_muscl_init=...)`` takes: level counts as they are, triangle indices
    0-based with -1 for none (the dump's are 1-based, <= 0 for none)."""
    nbl, updn = tr.work.get("nboundary_lay"), tr.work.get("edge_up_dn_tri")
    if nbl is None or updn is None:
        raise ValueError("the tracer dump holds no MUSCL work arrays")
    updn = np.asarray(updn, dtype=np.int32)
    return (np.ascontiguousarray(nbl, dtype=np.int32),
            np.ascontiguousarray(np.where(updn > 0, updn - 1, -1), dtype=np.int32))


def dyn_forcing(dyn: Dict[str, object], dt: float):
    """The velocities of a t_dynamics dump as the step's forcing (uv, w, w_e, w_i); Kv and the
    surface fluxes are not part of t_dyn."""
    from . import mesh as M
    f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
    return M.Forcing(uv=f64(dyn["uv"]), w=f64(dyn["w"]), w_e=f64(dyn["w_e"]), w_i=f64(dyn["w_i"]), Kv=None,
                     bc_surface=None, dt=float(dt))
