"""Reader of FESOM2 mesh folders: the text files the reference's partitioner leaves beside
the mesh (``nod2d.out``, ``elem2d.out``, ``aux3d.out``, ``elvls.out``, ``nlvls.out``,
``edges.out``, ``edge_tri.out``, ``edgenum.out``).

What the reference does on load, and this reader with it (src/oce_mesh.F90):
  * node coordinates in degrees -> radians, optionally rotated from geographical to model
    coordinates by the Euler angles (alpha, beta, gamma) (``read_mesh`` :431-440;
    ``set_mesh_transform_matrix`` / ``g2r``, src/gen_modules_rotate_grid.F90:30-116);
  * ``aux3d.out``: the level count, the level depths (made negative when the second one is
    positive, :596-599) and the depth of every node (made negative and cut at
    zbar(thers_zbar_lev = 5), :717-722);
  * element and node level counts from ``elvls.out`` / ``nlvls.out`` (:938-1110);
  * edges and their triangles from ``edges.out`` / ``edge_tri.out`` in file order, a
    triangle index <= 0 marking a boundary edge (:1791-1930);
  * triangle orientation made clockwise (``test_tri``, :1721-1742), then the derived
    geometry as for the generated meshes.
Cavities: ``cavity_elvls.out`` gives each element's first wet level (ulevels) and
``cavity_nlvls.out`` each node's, the smallest of its elements' (checked); without them every
column starts at level 1.  The top cell under an ice shelf is a full cell.
"""
from __future__ import annotations

import math
import os
from typing import Optional, Tuple

import numpy as np

from . import mesh as M

RAD = math.pi / 180.0


def _tokens(path: str) -> np.ndarray:
    with open(path) as f:
        return np.array(f.read().split())


def _ints(path: str, ncol: int) -> np.ndarray:
    t = _tokens(path).astype(np.int64)
    if t.size % ncol:
        raise ValueError(f"{path}: {t.size} integers, not a multiple of {ncol}")
    return t.reshape(-1, ncol)


def euler_matrix(alpha_deg: float, beta_deg: float, gamma_deg: float) -> np.ndarray:
    """Rotation matrix of the Euler angles: a rotation by alpha about z, then by beta about
    the new x axis, then by gamma about the new z axis (rows: rotated axes in geographical
    Cartesian coordinates)."""
    al, be, ga = alpha_deg * RAD, beta_deg * RAD, gamma_deg * RAD
    ca, sa, cb, sb, cg, sg = math.cos(al), math.sin(al), math.cos(be), math.sin(be), math.cos(ga), math.sin(ga)
    return np.array([[cg * ca - sg * cb * sa, cg * sa + sg * cb * ca, sg * sb],
                     [-sg * ca - cg * cb * sa, -sg * sa + cg * cb * ca, cg * sb],
                     [sb * sa, -sb * ca, cb]])


def geo_to_rot(lon: np.ndarray, lat: np.ndarray, R: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Geographical lon/lat (radians) to rotated model coordinates (radians)."""
    xg = np.cos(lat) * np.cos(lon)
    yg = np.cos(lat) * np.sin(lon)
    zg = np.sin(lat)
    xr = R[0, 0] * xg + R[0, 1] * yg + R[0, 2] * zg
    yr = R[1, 0] * xg + R[1, 1] * yg + R[1, 2] * zg
    zr = R[2, 0] * xg + R[2, 1] * yg + R[2, 2] * zg
    rlat = np.arcsin(np.clip(zr, -1.0, 1.0))
    pole = (xr == 0.0) & (yr == 0.0)
    rlon = np.where(pole, 0.0, np.arctan2(yr, xr))
    return rlon, rlat


def read_files(path: str) -> dict:
    """The raw arrays of a mesh folder (0-based indices, file order)."""
    f = lambda n: os.path.join(path, n)
    nod = _tokens(f("nod2d.out"))
    N2 = int(nod[0])
    rows = nod[1:].reshape(N2, 4)
    ids = rows[:, 0].astype(np.int64)
    if not np.array_equal(ids, np.arange(1, N2 + 1)):
        raise ValueError("nod2d.out: node numbers must run 1..nod2D in order")
    xy = rows[:, 1:3].astype(np.float64)
    flag = rows[:, 3].astype(np.int32)
    el = _tokens(f("elem2d.out")).astype(np.int64)
    T2 = int(el[0])
    tri = el[1:].reshape(T2, 3) - 1
    aux = _tokens(f("aux3d.out")).astype(np.float64)
    nl = int(aux[0])
    if nl < 3:
        raise ValueError("aux3d.out: fewer than 3 levels")
    zbar = aux[1:1 + nl].copy()
    depth = aux[1 + nl:].copy()
    out = {"xy_deg": xy, "flag": flag, "tri": tri, "zbar": zbar, "depth": depth, "N2": N2, "T2": T2}
    for name, key in (("elvls.out", "elvls"), ("nlvls.out", "nlvls"), ("cavity_elvls.out", "cavity_elvls"),
                      ("cavity_nlvls.out", "cavity_nlvls")):
        if os.path.exists(f(name)):
            out[key] = _tokens(f(name)).astype(np.int32)
    if os.path.exists(f("edges.out")):
        edges = _ints(f("edges.out"), 2) - 1
        etri = _ints(f("edge_tri.out"), 2)
        etri = np.where(etri <= 0, -1, etri - 1)
        num = _tokens(f("edgenum.out")).astype(np.int64)
        if edges.shape[0] != num[0] or etri.shape[0] != num[0]:
            raise ValueError("edges.out / edge_tri.out do not hold edgenum.out's edge count")
        out.update(edges=edges, edge_tri=etri, edge2D_in=int(num[1]))
    return out


def read_mesh(path: str, cartesian: bool = False, cyclic_length_deg: float = 360.0,
              rotation: Optional[Tuple[float, float, float]] = None, partial_cells: bool = False,
              name: Optional[str] = None, thers_zbar_lev: int = 5) -> M.Mesh:
    """A ``Mesh`` from a FESOM2 mesh folder.

    ``cartesian``, ``cyclic_length_deg`` and ``rotation`` (Euler angles in degrees; None: no
    rotation, as ``force_rotation = .false.``) are the namelist.config switches of the
    mesh.  Levels come from elvls.out when present, else from the node depths; edges from
    edges.out / edge_tri.out when present, else they are built."""
    return mesh_from_files(read_files(path), cartesian, cyclic_length_deg, rotation, partial_cells,
                           name or os.path.basename(os.path.normpath(path)), thers_zbar_lev)


def mesh_from_files(r: dict, cartesian: bool = False, cyclic_length_deg: float = 360.0,
                    rotation: Optional[Tuple[float, float, float]] = None, partial_cells: bool = False,
                    name: str = "mesh", thers_zbar_lev: int = 5) -> M.Mesh:
    """``read_mesh`` on the arrays of ``read_files`` (or a saved copy of them)."""
    lon = r["xy_deg"][:, 0] * RAD
    lat = r["xy_deg"][:, 1] * RAD
    if rotation is not None:
        lon, lat = geo_to_rot(lon, lat, euler_matrix(*rotation))
    coord = np.ascontiguousarray(np.stack([lon, lat], axis=1))
    zbar = r["zbar"]
    if zbar[1] > 0:
        zbar = -zbar
    N2, T2 = int(r["N2"]), int(r["T2"])
    depth = r["depth"]
    if depth.size == T2 and T2 != N2:
        if partial_cells:
            raise ValueError("aux3d.out holds element depths: partial cells need node depths")
        # only partial cells read the depth once the levels are known
        depth_el = -np.abs(depth)
        depth = np.full(N2, 0.0)
        np.minimum.at(depth, r["tri"].reshape(-1), np.repeat(depth_el, 3))
    elif depth.size != N2:
        raise ValueError(f"aux3d.out: {depth.size} depths for {N2} nodes and {T2} elements")
    depth = np.where(depth > 0, -depth, depth)
    depth = np.minimum(depth, zbar[thers_zbar_lev - 1])
    nlevels = r.get("elvls")
    if nlevels is not None and nlevels.size != T2:
        raise ValueError("elvls.out does not hold one level count per element")
    edge_set = (r["edges"], r["edge_tri"], int(r["edge2D_in"])) if "edges" in r else None
    ulevels = r.get("cavity_elvls")
    if ulevels is not None and ulevels.size != T2:
        raise ValueError("cavity_elvls.out does not hold one level per element")
    mesh = M._finish_mesh(coord, r["tri"], cyclic_length_deg * RAD, cartesian, zbar, depth, partial_cells,
                          name, nlevels=nlevels, edge_set=edge_set, ulevels=ulevels)
    if "cavity_nlvls" in r and not np.array_equal(np.asarray(r["cavity_nlvls"]), mesh.ulevels_nod2D):
        raise ValueError("cavity_nlvls.out disagrees with the shallowest element level around each node")
    if "nlvls" in r and not np.array_equal(np.asarray(r["nlvls"]), mesh.nlevels_nod2D):
        raise ValueError("nlvls.out disagrees with the deepest element level around each node")
    return mesh


# the namelist.config switches of the two meshes the reference's tests carry
SOUFFLET = dict(cartesian=True, cyclic_length_deg=4.5, rotation=None)
PI = dict(cartesian=False, cyclic_length_deg=360.0, rotation=(50.0, 15.0, -90.0))
# the PI mesh with cavities: the default namelist.config switches, as for PI
PI_CAVITY = dict(PI)


def save_files(r: dict, path: str) -> None:
    """The arrays of ``read_files`` as one compressed ``.npz`` (indices as int32)."""
    out = {}
    for k, v in r.items():
        a = np.asarray(v)
        out[k] = a.astype(np.int32) if a.dtype.kind == "i" else a
    np.savez_compressed(path, **out)


def load_files(path: str) -> dict:
    with np.load(path) as d:
        r = {k: d[k] for k in d.files}
    for k in ("tri", "edges", "edge_tri"):
        if k in r:
            r[k] = r[k].astype(np.int64)
    return r
