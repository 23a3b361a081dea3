"""Reader (and writer) of the reference's unformatted derived-type dump of the tracers
(``T_TRACER``, src/MOD_TRACER.F90:113-254), as the dwarf harness reads its saved state
(dwarf_ini/fesom.F90:64).

The dump is a Fortran sequential unformatted file: every ``write`` statement is one record
framed by 4-byte little-endian length markers (a record above 2 GiB - 9 bytes is split into
subrecords whose leading marker is negative, as gfortran writes them).  Arrays go through
``write_bin_array`` (src/MOD_WRITE_BINARY_ARRAYS.F90): a record with the extents (int32 each),
then, when the extents are not all zero, a record with the elements in column-major order.

Order of ``WRITE_T_TRACER``: num_tracers; per tracer ``WRITE_T_TRACER_DATA`` -- values(nl-1,
nod2D), valuesold(AB_order-1, nl-1, nod2D), valuesAB(nl-1, nod2D), smooth_bh_tra (logical),
gamma0_tra, gamma1_tra, gamma2_tra, i_vert_diff (logical), tra_adv_hor, tra_adv_ver,
tra_adv_lim (character(20)), tra_adv_ph, tra_adv_pv, ID -- each scalar its own record; then
``WRITE_T_TRACER_WORK``: del_ttf, del_ttf_advhoriz, del_ttf_advvert, dvd_trflx_hor,
dvd_trflx_ver, fct_LO, adv_flux_hor, adv_flux_ver, fct_ttf_max, fct_ttf_min, fct_plus,
fct_minus, nboundary_lay, edge_up_dn_tri, edge_up_dn_grad.

Arrays come back in this package's (row-major) layout: a Fortran array a(level, node) is
returned as a numpy array of shape (node, level), the same memory.
"""
from __future__ import annotations

import dataclasses
import struct
from typing import BinaryIO, Dict, List, Optional

import numpy as np

_MAX_SUB = 2 ** 31 - 9  # largest subrecord gfortran writes

WORK_FIELDS = [("del_ttf", "f8", 2), ("del_ttf_advhoriz", "f8", 2), ("del_ttf_advvert", "f8", 2),
               ("dvd_trflx_hor", "f8", 3), ("dvd_trflx_ver", "f8", 3), ("fct_LO", "f8", 2),
               ("adv_flux_hor", "f8", 2), ("adv_flux_ver", "f8", 2), ("fct_ttf_max", "f8", 2),
               ("fct_ttf_min", "f8", 2), ("fct_plus", "f8", 2), ("fct_minus", "f8", 2),
               ("nboundary_lay", "i4", 1), ("edge_up_dn_tri", "i4", 2), ("edge_up_dn_grad", "f8", 3)]


class RecordReader:
    def __init__(self, f: BinaryIO):
        self.f = f

    def record(self) -> bytes:
        out = []
        while True:
            head = self.f.read(4)
            if len(head) < 4:
                raise EOFError("end of the dump inside a record")
            n = struct.unpack("<i", head)[0]
            body = self.f.read(abs(n))
            tail = struct.unpack("<i", self.f.read(4))[0]
            if len(body) != abs(n) or abs(tail) != abs(n):
                raise ValueError("corrupt record markers")
            out.append(body)
            if n >= 0:  # the last (or only) subrecord
                return b"".join(out)

    def scalar(self, fmt: str):
        b = self.record()
        if len(b) != struct.calcsize(fmt):
            raise ValueError(f"record of {len(b)} bytes where {fmt} was expected")
        return struct.unpack(fmt, b)[0]

    def chars(self, n: int) -> str:
        b = self.record()
        if len(b) != n:
            raise ValueError(f"character record of {len(b)} bytes where {n} were expected")
        return b.decode("ascii").rstrip()

    def array(self, dtype: str, rank: int) -> Optional[np.ndarray]:
        ext = self.record()
        if len(ext) != 4 * rank:
            raise ValueError(f"extent record of {len(ext)} bytes for a rank-{rank} array")
        dims = struct.unpack(f"<{rank}i", ext)
        if all(d == 0 for d in dims):
            return None
        data = np.frombuffer(self.record(), dtype="<" + dtype)
        if data.size != int(np.prod(dims)):
            raise ValueError(f"array record of {data.size} elements for extents {dims}")
        # Fortran a(d1, ..., dk) column-major == row-major shape (dk, ..., d1)
        return data.reshape(tuple(reversed(dims))).copy()


class RecordWriter:
    def __init__(self, f: BinaryIO):
        self.f = f

    def record(self, b: bytes) -> None:
        if len(b) <= _MAX_SUB:
            self.f.write(struct.pack("<i", len(b)) + b + struct.pack("<i", len(b)))
            return
        pos = 0
        while pos < len(b):
            chunk = b[pos:pos + _MAX_SUB]
            last = pos + len(chunk) >= len(b)
            n = len(chunk) if last else -len(chunk)
            self.f.write(struct.pack("<i", n) + chunk + struct.pack("<i", n))
            pos += len(chunk)

    def scalar(self, fmt: str, v) -> None:
        self.record(struct.pack(fmt, v))

    def chars(self, s: str, n: int) -> None:
        self.record(s.ljust(n)[:n].encode("ascii"))

    def array(self, a: Optional[np.ndarray], dtype: str, rank: int) -> None:
        if a is None:
            self.record(struct.pack(f"<{rank}i", *([0] * rank)))
            return
        a = np.ascontiguousarray(a, dtype="<" + dtype)
        if a.ndim != rank:
            raise ValueError(f"rank-{rank} array expected")
        self.record(struct.pack(f"<{rank}i", *reversed(a.shape)))
        self.record(a.tobytes())


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
    with open(path, "rb") as f:
        r = RecordReader(f)
        n = r.scalar("<i")
        if n < 0:
            raise ValueError("negative tracer count")
        data = []
        for _ in range(n):
            values = r.array("f8", 2)
            valuesold = r.array("f8", 3)
            valuesAB = r.array("f8", 2)
            smooth = bool(r.scalar("<i"))
            g0, g1, g2 = r.scalar("<d"), r.scalar("<d"), r.scalar("<d")
            ivd = bool(r.scalar("<i"))
            hor, ver, lim = r.chars(20), r.chars(20), r.chars(20)
            ph, pv = r.scalar("<d"), r.scalar("<d")
            tid = r.scalar("<i")
            data.append(TracerData(values, valuesold, valuesAB, smooth, g0, g1, g2, ivd, hor, ver, lim, ph, pv, tid))
        work = {name: r.array(dt, rank) for name, dt, rank in WORK_FIELDS}
        if f.read(1):
            raise ValueError("bytes left after the tracer dump")
    return Tracers(data, work)


def write_tracers(path: str, tr: Tracers) -> None:
    """WRITE_T_TRACER (src/MOD_TRACER.F90:211-230): the layout ``read_tracers`` reads."""
    with open(path, "wb") as f:
        w = RecordWriter(f)
        w.scalar("<i", len(tr.data))
        for d in tr.data:
            w.array(d.values, "f8", 2)
            w.array(d.valuesold, "f8", 3)
            w.array(d.valuesAB, "f8", 2)
            w.scalar("<i", int(d.smooth_bh_tra))
            for g in (d.gamma0_tra, d.gamma1_tra, d.gamma2_tra):
                w.scalar("<d", g)
            w.scalar("<i", int(d.i_vert_diff))
            for s in (d.tra_adv_hor, d.tra_adv_ver, d.tra_adv_lim):
                w.chars(s, 20)
            w.scalar("<d", d.tra_adv_ph)
            w.scalar("<d", d.tra_adv_pv)
            w.scalar("<i", d.ID)
        for name, dt, rank in WORK_FIELDS:
            w.array(tr.work.get(name), dt, rank)


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
