"""Synthetic FESOM2 meshes and tracer-step inputs.

Builds the mesh arrays that the tracer-transport step reads from FESOM2's
``t_mesh`` / ``t_tracer`` / ``t_dyn`` derived types, for two seeded
generators:

* a Soufflet-like periodic zonal channel (staggered rows, cyclic in x, walls
  on the first and last row), and
* a quasi-uniform sphere from a subdivided icosahedron, land-masked by a
  seeded smooth random field.

Every array keeps the reference's memory layout: a Fortran array
``a(level, entity)`` is stored here as a C-contiguous numpy array of shape
``(entity, level)``, i.e. level-contiguous per column.  Indices are 0-based;
"no element" in ``edge_tri[:, 1]`` is ``-1`` (the reference stores ``-999``).

Geometry follows the reference formulas:

* element orientation (clockwise) -- ``src/oce_mesh.F90:1699-1742`` (test_tri)
* edges, ``edge_tri`` ordering (internal edges first, el(1) left of n1->n2)
  -- ``src/fvom_init.F90:490-607``
* ``elem_area``, ``area``, ``areasvol`` -- ``src/oce_mesh.F90:2227-2340``
* ``elem_cos``, ``edge_dxdy``, ``edge_cross_dxdy``, ``gradient_sca``
  -- ``src/oce_mesh.F90:2533-2666``; ``elem_center``/``edge_center``
  -- ``src/oce_mesh.F90:2140-2180``
* element levels from depth -- ``src/fvom_init.F90:855-946``; node levels as
  the max over elements -- ``src/fvom_init.F90:978-985``
* ``nlevels_nod2D_min`` / ``ulevels_nod2D_max`` -- ``src/oce_mesh.F90:1656-1694``
* partial bottom cells -- ``src/oce_ale.F90:381-621``; linfs thicknesses
  -- ``src/oce_ale.F90:795-812``
* vertical velocity from the discrete divergence -- ``src/oce_ale.F90:2107-2306``
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Optional

import numpy as np

R_EARTH = 6367500.0  # src/oce_modules.F90:29


# ---------------------------------------------------------------------------
# containers
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Mesh:
    """Mirror of the ``t_mesh`` fields the tracer step reads (0-based)."""

    nl: int                      # number of levels (interfaces); layers = nl-1
    coord_nod2D: np.ndarray      # (N2, 2) rotated lon/lat in radians (channel: x/R, y/R)
    elem2D_nodes: np.ndarray     # (T2, 3) int32
    edges: np.ndarray            # (E2, 2) int32
    edge_tri: np.ndarray         # (E2, 2) int32, -1 = none
    edge2D_in: int
    nod_in_elem2D_ptr: np.ndarray  # (N2+1,) int32 CSR over ascending element index
    nod_in_elem2D: np.ndarray      # (nnz,) int32
    nlevels: np.ndarray          # (T2,) int32 (1-based level counts, as in the reference)
    ulevels: np.ndarray          # (T2,)
    nlevels_nod2D: np.ndarray    # (N2,)
    ulevels_nod2D: np.ndarray    # (N2,)
    nlevels_nod2D_min: np.ndarray
    ulevels_nod2D_max: np.ndarray
    elem_area: np.ndarray        # (T2,)
    elem_cos: np.ndarray         # (T2,)
    edge_dxdy: np.ndarray        # (E2, 2)
    edge_cross_dxdy: np.ndarray  # (E2, 4)
    gradient_sca: np.ndarray     # (T2, 6)
    area: np.ndarray             # (N2, nl)
    areasvol: np.ndarray         # (N2, nl)
    hnode: np.ndarray            # (N2, nl-1)
    hnode_new: np.ndarray        # (N2, nl-1)
    helem: np.ndarray            # (T2, nl-1)
    zbar: np.ndarray             # (nl,)
    Z: np.ndarray                # (nl-1,)
    zbar_3d_n: np.ndarray        # (N2, nl)
    Z_3d_n: np.ndarray           # (N2, nl-1)
    zbar_n_bot: np.ndarray       # (N2,)
    cyclic_length: float
    cartesian: bool
    name: str = "mesh"

    @property
    def nod2D(self) -> int:
        return int(self.coord_nod2D.shape[0])

    @property
    def elem2D(self) -> int:
        return int(self.elem2D_nodes.shape[0])

    @property
    def edge2D(self) -> int:
        return int(self.edges.shape[0])

    def nod_in_elem2D_num(self) -> np.ndarray:
        return np.diff(self.nod_in_elem2D_ptr).astype(np.int32)

    def counts(self) -> dict:
        """Wet node-, edge- and element-layer counts (N3, E3, T3)."""
        N3 = int(np.sum(self.nlevels_nod2D - self.ulevels_nod2D))
        el1 = self.edge_tri[:, 0]
        el2 = self.edge_tri[:, 1]
        nl1 = self.nlevels[el1] - 1
        nu1 = self.ulevels[el1]
        has2 = el2 >= 0
        nl2 = np.where(has2, self.nlevels[np.maximum(el2, 0)] - 1, 0)
        nu2 = np.where(has2, self.ulevels[np.maximum(el2, 0)], 0)
        nl12 = np.maximum(nl1, nl2)
        nu12 = np.where(nu2 > 0, np.minimum(nu1, nu2), nu1)
        E3 = int(np.sum(nl12 - nu12 + 1))
        T3 = int(np.sum(self.nlevels - self.ulevels))
        return {"N2": self.nod2D, "E2": self.edge2D, "T2": self.elem2D,
                "N3": N3, "E3": E3, "T3": T3, "nl": self.nl}


@dataclasses.dataclass
class Forcing:
    """Mirror of the ``t_dyn`` velocities plus the vertical-diffusion inputs."""

    uv: np.ndarray      # (T2, nl-1, 2)  uv(1:2, nz, elem)
    w: np.ndarray       # (N2, nl)
    w_e: np.ndarray     # (N2, nl)
    w_i: np.ndarray     # (N2, nl)
    Kv: np.ndarray      # (N2, nl)
    bc_surface: np.ndarray  # (N2,) per-node surface boundary term, added at nzmin
    dt: float


# ---------------------------------------------------------------------------
# seeded smooth random fields
# ---------------------------------------------------------------------------
def _smooth_field_3d(xyz: np.ndarray, rng: np.random.Generator, nmodes: int = 24,
                     kmin: float = 1.0, kmax: float = 6.0) -> np.ndarray:
    """Sum of random plane waves on the unit sphere, normalised to unit RMS."""
    dirs = rng.normal(size=(nmodes, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    ks = rng.uniform(kmin, kmax, size=nmodes)
    ph = rng.uniform(0, 2 * np.pi, size=nmodes)
    amp = rng.normal(size=nmodes) / ks
    f = np.zeros(xyz.shape[0])
    for j in range(nmodes):
        f += amp[j] * np.cos(ks[j] * (xyz @ dirs[j]) + ph[j])
    f -= f.mean()
    f /= (f.std() + 1e-300)
    return f


# ---------------------------------------------------------------------------
# topology helpers
# ---------------------------------------------------------------------------
def _trim(a: np.ndarray, cyc: float) -> np.ndarray:
    """trim_cyclic, src/gen_modules_rotate_grid.F90:204-211 (vectorised)."""
    a = np.where(a > cyc / 2.0, a - cyc, a)
    a = np.where(a < -cyc / 2.0, a + cyc, a)
    return a


def _elem_center(coord: np.ndarray, tri: np.ndarray, cyc: float):
    """elem_center, src/oce_mesh.F90:2160-2180 (vectorised)."""
    ax = coord[tri, 0].copy()
    amin = ax.min(axis=1, keepdims=True)
    ax = np.where(ax - amin >= cyc / 2.0, ax - cyc, ax)
    ax = np.where(ax - amin < -cyc / 2.0, ax + cyc, ax)
    x = (ax[:, 0] + ax[:, 1] + ax[:, 2]) / 3.0
    y = (coord[tri[:, 0], 1] + coord[tri[:, 1], 1] + coord[tri[:, 2], 1]) / 3.0
    return x, y


def _orient_clockwise(coord: np.ndarray, tri: np.ndarray, cyc: float) -> np.ndarray:
    """test_tri, src/oce_mesh.F90:1721-1742: swap nodes 2/3 when b x c > 0."""
    a = coord[tri[:, 0]]
    b = coord[tri[:, 1]] - a
    c = coord[tri[:, 2]] - a
    b[:, 0] = _trim(b[:, 0], cyc)
    c[:, 0] = _trim(c[:, 0], cyc)
    r = b[:, 0] * c[:, 1] - b[:, 1] * c[:, 0]
    out = tri.copy()
    sw = r > 0.0
    out[sw, 1] = tri[sw, 2]
    out[sw, 2] = tri[sw, 1]
    return out


def _build_edges(coord: np.ndarray, tri: np.ndarray, cyc: float):
    """Edges and edge_tri as src/fvom_init.F90:490-607 lays them out.

    Internal edges come first (ordered by their lower node, then upper node),
    boundary edges after; edge_tri(1) is the element left of n1 -> n2.
    """
    T2 = tri.shape[0]
    he = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]], axis=0)
    hel = np.concatenate([np.arange(T2)] * 3)
    lo = np.minimum(he[:, 0], he[:, 1]).astype(np.int64)
    hi = np.maximum(he[:, 0], he[:, 1]).astype(np.int64)
    key = lo * (coord.shape[0] + 1) + hi
    order = np.argsort(key, kind="stable")
    key_s = key[order]
    starts = np.flatnonzero(np.r_[True, key_s[1:] != key_s[:-1]])
    cnt = np.diff(np.r_[starts, key_s.size])
    if np.any(cnt > 2):
        raise ValueError("non-manifold mesh: an edge has more than two triangles")
    first = order[starts]
    e_lo = lo[first]
    e_hi = hi[first]
    t1 = hel[first]
    t2 = np.full(first.size, -1, dtype=np.int64)
    two = cnt == 2
    t2[two] = hel[order[starts[two] + 1]]
    # internal first, then boundary (stable keeps (lo, hi) order inside groups)
    grp = np.argsort(~two, kind="stable")
    e_lo, e_hi, t1, t2 = e_lo[grp], e_hi[grp], t1[grp], t2[grp]
    edge2D_in = int(two.sum())
    n1 = e_lo.copy()
    n2 = e_hi.copy()
    # el(1) must lie left of n1 -> n2 (fvom_init.F90:579-607)
    cx, cy = _elem_center(coord, tri[t1], cyc)
    xc0 = cx - coord[n1, 0]
    xc1 = cy - coord[n1, 1]
    xe0 = _trim(coord[n2, 0] - coord[n1, 0], cyc)
    xe1 = coord[n2, 1] - coord[n1, 1]
    xc0 = _trim(xc0, cyc)
    right = (xc0 * xe1 - xc1 * xe0) > 0.0
    sw_tri = right & (t2 >= 0)
    sw_nod = right & (t2 < 0)
    t1n = np.where(sw_tri, t2, t1)
    t2n = np.where(sw_tri, t1, t2)
    n1n = np.where(sw_nod, n2, n1)
    n2n = np.where(sw_nod, n1, n2)
    edges = np.stack([n1n, n2n], axis=1).astype(np.int32)
    edge_tri = np.stack([t1n, t2n], axis=1).astype(np.int32)
    return edges, edge_tri, edge2D_in


def _nod_in_elem(tri: np.ndarray, N2: int):
    """Node -> element CSR; each list in ascending element order (as the
    reference fills nod_in_elem2D by a loop over elements, oce_mesh.F90:2054-2062)."""
    T2 = tri.shape[0]
    nodes = tri.reshape(-1).astype(np.int64)
    elems = np.repeat(np.arange(T2, dtype=np.int64), 3)
    order = np.lexsort((elems, nodes))
    ptr = np.zeros(N2 + 1, dtype=np.int64)
    np.add.at(ptr, nodes + 1, 1)
    ptr = np.cumsum(ptr)
    return ptr.astype(np.int32), elems[order].astype(np.int32)


def _compact(coord: np.ndarray, tri: np.ndarray, keep_node: np.ndarray, order_key: Optional[np.ndarray]):
    """Keep triangles whose nodes are all kept, drop orphans, renumber nodes
    (optionally sorted by ``order_key``) and sort elements by their first node."""
    keep_tri = keep_node[tri].all(axis=1)
    tri = tri[keep_tri]
    used = np.zeros(coord.shape[0], dtype=bool)
    used[tri.reshape(-1)] = True
    old = np.flatnonzero(used)
    if order_key is not None:
        old = old[np.argsort(order_key[old], kind="stable")]
    new_of_old = np.full(coord.shape[0], -1, dtype=np.int64)
    new_of_old[old] = np.arange(old.size)
    tri = new_of_old[tri]
    # element order: by (min node, centroid-ish) for locality
    tkey = np.sort(tri, axis=1)
    torder = np.lexsort((tkey[:, 2], tkey[:, 1], tkey[:, 0]))
    tri = tri[torder]
    return coord[old], tri, old


def _morton_key(xyz: np.ndarray, bits: int = 20) -> np.ndarray:
    """Morton (Z-order) key of points in [-1, 1]^3."""
    q = np.clip(((xyz + 1.0) * 0.5 * ((1 << bits) - 1)).astype(np.int64), 0, (1 << bits) - 1)

    def spread(v):
        v = v & 0x1FFFFF
        v = (v | (v << 32)) & 0x1F00000000FFFF
        v = (v | (v << 16)) & 0x1F0000FF0000FF
        v = (v | (v << 8)) & 0x100F00F00F00F00F
        v = (v | (v << 4)) & 0x10C30C30C30C30C3
        v = (v | (v << 2)) & 0x1249249249249249
        return v

    return spread(q[:, 0]) | (spread(q[:, 1]) << 1) | (spread(q[:, 2]) << 2)


# ---------------------------------------------------------------------------
# vertical grid, levels, geometry
# ---------------------------------------------------------------------------
def _levels_from_depth(tri: np.ndarray, depth_nod: np.ndarray, zbar: np.ndarray, Z: np.ndarray,
                       thers_zbar_lev: int = 5) -> np.ndarray:
    """Element nlevels from the mean node depth (src/fvom_init.F90:855-883) and the
    open-neighbour cleanup (src/fvom_init.F90:897-946, vectorised per level)."""
    nl = zbar.size
    T2 = tri.shape[0]
    dmean = depth_nod[tri].mean(axis=1)  # negative below the surface
    # first nz with Z(nz) < dmean  (1-based)
    below = Z[None, :] < dmean[:, None]
    has = below.any(axis=1)
    first = np.argmax(below, axis=1) + 1
    nlev = np.where(has, first, nl).astype(np.int64)
    nlev = np.where(dmean >= 0, thers_zbar_lev, nlev)
    nlev = np.maximum(nlev, thers_zbar_lev)
    # element neighbours through shared edges
    he = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]], axis=0)
    hel = np.concatenate([np.arange(T2)] * 3)
    lo = np.minimum(he[:, 0], he[:, 1]).astype(np.int64)
    hi = np.maximum(he[:, 0], he[:, 1]).astype(np.int64)
    key = lo * (tri.max() + 2) + hi
    order = np.argsort(key, kind="stable")
    ks = key[order]
    same = np.r_[ks[1:] == ks[:-1], False]
    a = hel[order][:-1][same[:-1]]
    b = hel[order][1:][same[:-1]]
    u = np.concatenate([a, b])
    v = np.concatenate([b, a])
    o = np.argsort(u, kind="stable")
    u, v = u[o], v[o]
    st = np.r_[0, np.flatnonzero(u[1:] != u[:-1]) + 1]
    rank = np.arange(u.size) - np.repeat(st, np.diff(np.r_[st, u.size]))
    nbr = np.full((T2, 3), -1, dtype=np.int64)
    nbr[u, rank] = v
    for nz in range(thers_zbar_lev + 1, nl + 1):
        # only elements open at nz with a closed (or missing) neighbour can fail the test
        nb_lev = np.where(nbr >= 0, nlev[np.maximum(nbr, 0)], -1)
        cand = np.flatnonzero((nlev >= nz) & (nb_lev < nz).any(axis=1))
        for _ in range(1000):
            if cand.size == 0:
                break
            nbc = nbr[cand]
            openn = np.where(nbc >= 0, nlev[np.maximum(nbc, 0)] >= nz, False).sum(axis=1)
            bad = cand[(nlev[cand] >= nz) & (openn < 2)]
            if bad.size == 0:
                break
            if nz - 1 < thers_zbar_lev:
                idx = nbr[bad].reshape(-1)
                idx = idx[idx >= 0]
                nlev[idx] = np.maximum(nlev[idx], nz)
                cand = np.unique(np.concatenate([idx, bad]))
            else:
                nlev[bad] = nz - 1
                nb = nbr[bad].reshape(-1)
                cand = np.unique(nb[nb >= 0])
    return nlev.astype(np.int32)


def _finish_mesh(coord: np.ndarray, tri: np.ndarray, cyc: float, cartesian: bool,
                 zbar: np.ndarray, depth_nod: np.ndarray, partial_cells: bool,
                 name: str, nlevels: Optional[np.ndarray] = None, edge_set=None,
                 ulevels: Optional[np.ndarray] = None) -> Mesh:
    """Derived arrays of a mesh from node coordinates (radians), triangles (0-based), levels
    and node depths.  ``nlevels`` (element level counts) and ``edge_set`` = (edges, edge_tri,
    edge2D_in), 0-based with -1 for a missing triangle, are taken as given when passed (as
    the reference takes them from the partitioner's files), else built here.  ``ulevels``
    (element first wet levels, cavities under ice shelves) defaults to 1 everywhere."""
    nl = zbar.size
    Z = 0.5 * (zbar[:-1] + zbar[1:])
    tri = _orient_clockwise(coord, tri.astype(np.int64), cyc)
    N2 = coord.shape[0]
    T2 = tri.shape[0]
    if edge_set is None:
        edges, edge_tri, edge2D_in = _build_edges(coord, tri, cyc)
    else:
        edges, edge_tri, edge2D_in = edge_set
        edges = np.ascontiguousarray(edges, dtype=np.int32)
        edge_tri = np.ascontiguousarray(edge_tri, dtype=np.int32)
    ptr, nie = _nod_in_elem(tri, N2)
    nie_node = np.repeat(np.arange(N2), np.diff(ptr))

    # --- levels --------------------------------------------------------------
    if nlevels is None:
        nlevels = _levels_from_depth(tri, depth_nod, zbar, Z)
    nlevels = np.ascontiguousarray(nlevels, dtype=np.int32)
    ulevels = np.ones(T2, dtype=np.int32) if ulevels is None else np.ascontiguousarray(ulevels, dtype=np.int32)
    cavity = bool((ulevels > 1).any())
    nlevels_nod2D = np.zeros(N2, dtype=np.int32)
    np.maximum.at(nlevels_nod2D, tri.reshape(-1), np.repeat(nlevels, 3))
    ulevels_nod2D = np.full(N2, nl + 1, dtype=np.int32)
    np.minimum.at(ulevels_nod2D, nie_node, ulevels[nie])
    nlevels_nod2D_min = np.full(N2, nl + 1, dtype=np.int32)
    np.minimum.at(nlevels_nod2D_min, nie_node, nlevels[nie])
    ulevels_nod2D_max = np.zeros(N2, dtype=np.int32)
    np.maximum.at(ulevels_nod2D_max, nie_node, ulevels[nie])

    # --- horizontal geometry (oce_mesh.F90:2227-2240, 2533-2666) -------------
    ay = coord[tri, 1].sum(axis=1) / 3.0
    ay = np.cos(ay)
    if cartesian:
        ay = np.ones_like(ay)
    a = coord[tri[:, 1]] - coord[tri[:, 0]]
    b = coord[tri[:, 2]] - coord[tri[:, 0]]
    a[:, 0] = _trim(a[:, 0], cyc) * ay
    b[:, 0] = _trim(b[:, 0], cyc) * ay
    elem_area_rad = 0.5 * np.abs(a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1])

    cx, cy = _elem_center(coord, tri, cyc)
    elem_cos = np.cos(cy)
    if cartesian:
        elem_cos = np.ones(T2)

    ed = edges.astype(np.int64)
    edge_dxdy = coord[ed[:, 1]] - coord[ed[:, 0]]
    edge_dxdy[:, 0] = _trim(edge_dxdy[:, 0], cyc)

    # edge_center (oce_mesh.F90:2140-2157)
    pa = coord[ed[:, 0]].copy()
    pb = coord[ed[:, 1]].copy()
    d = pa[:, 0] - pb[:, 0]
    pa[:, 0] = np.where(d > cyc / 2.0, pa[:, 0] - cyc, pa[:, 0])
    pb[:, 0] = np.where(d < -cyc / 2.0, pb[:, 0] - cyc, pb[:, 0])
    ecx = 0.5 * (pa[:, 0] + pb[:, 0])
    ecy = 0.5 * (pa[:, 1] + pb[:, 1])
    el1 = edge_tri[:, 0].astype(np.int64)
    el2 = edge_tri[:, 1].astype(np.int64)
    has2 = el2 >= 0
    ecd = np.zeros((edges.shape[0], 4))
    bx = _trim(cx[el1] - ecx, cyc) * elem_cos[el1]
    by = cy[el1] - ecy
    ecd[:, 0] = bx * R_EARTH
    ecd[:, 1] = by * R_EARTH
    e2 = np.maximum(el2, 0)
    bx2 = _trim(cx[e2] - ecx, cyc) * elem_cos[e2]
    by2 = cy[e2] - ecy
    ecd[:, 2] = np.where(has2, bx2 * R_EARTH, 0.0)
    ecd[:, 3] = np.where(has2, by2 * R_EARTH, 0.0)

    elem_area = elem_area_rad * R_EARTH * R_EARTH
    dX31 = elem_cos * _trim(coord[tri[:, 2], 0] - coord[tri[:, 0], 0], cyc)
    dX21 = elem_cos * _trim(coord[tri[:, 1], 0] - coord[tri[:, 0], 0], cyc)
    dY31 = coord[tri[:, 2], 1] - coord[tri[:, 0], 1]
    dY21 = coord[tri[:, 1], 1] - coord[tri[:, 0], 1]
    dfac = -0.5 * R_EARTH / elem_area
    gs = np.stack([(-dY31 + dY21) * dfac, dY31 * dfac, -dY21 * dfac,
                   (dX31 - dX21) * dfac, -dX31 * dfac, dX21 * dfac], axis=1)

    # --- vertical: partial cells (oce_ale.F90:381-560) ------------------------
    dd_e = depth_nod[tri].mean(axis=1)
    nle = nlevels.astype(np.int64)
    zb_nle = zbar[nle - 1]          # zbar(nle)
    zb_nle1 = zbar[nle - 2]         # zbar(nle-1)
    if partial_cells:
        zeb = np.where(dd_e < zb_nle,
                       np.where(nle == nl, np.maximum(dd_e, zb_nle + (zb_nle - Z[np.minimum(nle - 2, nl - 2)])),
                                np.maximum(Z[np.minimum(nle - 1, nl - 2)], dd_e)),
                       np.minimum(Z[nle - 2], dd_e))
    else:
        zeb = zb_nle
    bottom_elem_thickness = zb_nle1 - zeb
    zbar_e_bot = zeb
    zbar_n_bot = np.full(N2, np.inf)
    np.minimum.at(zbar_n_bot, nie_node, zbar_e_bot[nie])
    nln = nlevels_nod2D.astype(np.int64)
    bottom_node_thickness = zbar[nln - 2] - zbar_n_bot

    zbar_3d_n = np.broadcast_to(zbar, (N2, nl)).copy()
    zbar_3d_n[np.arange(N2), nln - 1] = zbar_n_bot
    Z_3d_n = np.broadcast_to(Z, (N2, nl - 1)).copy()
    Z_3d_n[np.arange(N2), nln - 2] = 0.5 * (zbar[nln - 2] + zbar_n_bot)

    Lh = np.arange(nl - 1)[None, :]
    dz = (zbar[:-1] - zbar[1:])[None, :]
    uln = ulevels_nod2D.astype(np.int64)
    ule = ulevels.astype(np.int64)
    # layers above the first wet level (under an ice shelf) have no thickness
    hnode = np.where((Lh < (nln - 2)[:, None]) & (Lh >= (uln - 1)[:, None]), dz, 0.0)
    hnode[np.arange(N2), nln - 2] = bottom_node_thickness
    helem = np.where((Lh < (nle - 2)[:, None]) & (Lh >= (ule - 1)[:, None]), dz, 0.0)
    helem[np.arange(T2), nle - 2] = bottom_elem_thickness

    # area / areasvol (oce_mesh.F90:2277-2340)
    # area(nz, n) = sum over the node's elements wet at layer nz of elem_area/3: every
    # element contributes to layers 1..nlevels-1, so accumulate at the layer where it
    # stops and take a reverse cumulative sum over levels
    a3 = (elem_area_rad / 3.0)[nie]
    stop = nle[nie] - 2                     # last wet layer (0-based)
    if not cavity:
        D = np.bincount(nie_node.astype(np.int64) * nl + stop, weights=a3, minlength=N2 * nl).reshape(N2, nl)
        area = np.flip(np.cumsum(np.flip(D, axis=1), axis=1), axis=1) * (R_EARTH * R_EARTH)
        wet_n = np.arange(nl)[None, :] < (nln - 1)[:, None]
        areasvol = np.where(wet_n, area, 0.0)
    else:
        # an element counts at levels ulevels..nlevels-1 only; areasvol of a level with an
        # element still under the shelf takes the area of the level below
        # (oce_mesh.F90:2277-2330, use_cavity)
        start = ule[nie] - 1
        area = np.zeros((N2, nl))
        cav = np.zeros((N2, nl), dtype=np.int64)
        nn = nie_node.astype(np.int64)
        for k in range(nl):
            on = (start <= k) & (k <= stop)
            area[:, k] = np.bincount(nn, weights=np.where(on, a3, 0.0), minlength=N2)
            cav[:, k] = np.bincount(nn, weights=(k < start).astype(np.float64), minlength=N2).astype(np.int64)
        lev = np.arange(nl)[None, :]
        wet_n = (lev >= (uln - 1)[:, None]) & (lev < (nln - 1)[:, None])
        below = np.minimum(lev + 1, (nln - 2)[:, None])
        area_below = np.take_along_axis(area, np.broadcast_to(below, area.shape), axis=1)
        areasvol = np.where(wet_n, np.where(cav > 0, area_below, area), 0.0) * (R_EARTH * R_EARTH)
        area = area * (R_EARTH * R_EARTH)

    return Mesh(
        nl=nl, coord_nod2D=np.ascontiguousarray(coord), elem2D_nodes=tri.astype(np.int32),
        edges=edges, edge_tri=edge_tri, edge2D_in=edge2D_in,
        nod_in_elem2D_ptr=ptr, nod_in_elem2D=nie,
        nlevels=nlevels, ulevels=ulevels, nlevels_nod2D=nlevels_nod2D, ulevels_nod2D=ulevels_nod2D,
        nlevels_nod2D_min=nlevels_nod2D_min, ulevels_nod2D_max=ulevels_nod2D_max,
        elem_area=elem_area, elem_cos=elem_cos, edge_dxdy=np.ascontiguousarray(edge_dxdy),
        edge_cross_dxdy=ecd, gradient_sca=np.ascontiguousarray(gs),
        area=area, areasvol=areasvol, hnode=np.ascontiguousarray(hnode),
        hnode_new=np.ascontiguousarray(hnode.copy()), helem=np.ascontiguousarray(helem),
        zbar=zbar, Z=Z, zbar_3d_n=zbar_3d_n, Z_3d_n=Z_3d_n, zbar_n_bot=zbar_n_bot,
        cyclic_length=float(cyc), cartesian=cartesian, name=name)


def stretched_zbar(nlayers: int, dz_top: float, dz_bot: float) -> np.ndarray:
    """Interfaces 0 > zbar(2) > ... with layer thickness growing geometrically."""
    if nlayers == 1 or dz_top == dz_bot:
        dz = np.full(nlayers, float(dz_top))
    else:
        r = (dz_bot / dz_top) ** (1.0 / (nlayers - 1))
        dz = dz_top * r ** np.arange(nlayers)
    return -np.concatenate([[0.0], np.cumsum(dz)])


# ---------------------------------------------------------------------------
# generators
# ---------------------------------------------------------------------------
def channel_mesh(nx: int = 100, ny: int = 400, dx: float = 5000.0, zbar: Optional[np.ndarray] = None,
                 seamounts: int = 0, seed: int = 1, partial_cells: bool = False,
                 min_layers_target: Optional[int] = None) -> Mesh:
    """Periodic zonal channel with staggered rows (the mesh2d_soufflet.m layout):
    ``nx`` cyclic columns by ``ny`` rows, spacing ``dx`` metres, walls on the
    first and last rows, cartesian metric (coordinates are metres / r_earth)."""
    if zbar is None:
        zbar = -np.arange(41) * 100.0
    dy = dx * math.sqrt(3.0) / 2.0
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    x = (i + 0.5 * (j % 2)) * dx
    y = j * dy
    coord = np.stack([x.reshape(-1) / R_EARTH, y.reshape(-1) / R_EARTH], axis=1)
    cyc = nx * dx / R_EARTH

    def nid(ii, jj):
        return jj * nx + (ii % nx)

    tris = []
    for jj in range(ny - 1):
        ii = np.arange(nx)
        if jj % 2 == 0:
            tris.append(np.stack([nid(ii, jj), nid(ii + 1, jj), nid(ii, jj + 1)], axis=1))
            tris.append(np.stack([nid(ii + 1, jj), nid(ii + 1, jj + 1), nid(ii, jj + 1)], axis=1))
        else:
            tris.append(np.stack([nid(ii, jj), nid(ii + 1, jj + 1), nid(ii, jj + 1)], axis=1))
            tris.append(np.stack([nid(ii, jj), nid(ii + 1, jj), nid(ii + 1, jj + 1)], axis=1))
    tri = np.concatenate(tris, axis=0)
    depth = _seamount_depth(x.reshape(-1), y.reshape(-1), nx * dx, ny * dy, -zbar[-1], seamounts, seed, True)
    m = _finish_mesh(coord, tri, cyc, True, zbar, depth, partial_cells, name=f"channel_{nx}x{ny}")
    return m


def _seamount_depth(x, y, Lx, Ly, H, seamounts, seed, periodic):
    """Node depth (negative, metres): flat bottom at H minus seeded Gaussian seamounts."""
    depth = np.full(x.shape[0], -H)
    if seamounts > 0:
        rng = np.random.default_rng(seed + 7)
        cxs = rng.uniform(0, Lx, seamounts)
        cys = rng.uniform(0.1 * Ly, 0.9 * Ly, seamounts)
        rad = rng.uniform(0.04, 0.12, seamounts) * Ly
        amp = rng.uniform(0.5, 0.82, seamounts) * H
        bump = np.zeros_like(x)
        for k in range(seamounts):
            ddx = np.abs(x - cxs[k])
            if periodic:
                ddx = np.minimum(ddx, Lx - ddx)
            bump = np.maximum(bump, amp[k] * np.exp(-(ddx ** 2 + (y - cys[k]) ** 2) / (2 * rad[k] ** 2)))
        depth = -(H - bump) - 1e-3
    return depth


def delaunay_mesh(npts: int = 400, Lx: float = 100e3, Ly: float = 80e3, zbar: Optional[np.ndarray] = None,
                  seamounts: int = 0, seed: int = 1, partial_cells: bool = False) -> Mesh:
    """Closed rectangular basin meshed by the Delaunay triangulation of seeded random
    points (plus points along the walls): an irregular mesh whose node degrees spread
    from 3 to 10 and more, unlike the regular channel and icosahedral meshes.
    Cartesian metric, not periodic."""
    from scipy.spatial import Delaunay
    if zbar is None:
        zbar = -np.arange(41) * 100.0
    rng = np.random.default_rng(seed)
    nb = max(4, int(round(math.sqrt(npts))))
    side = np.linspace(0.0, 1.0, nb, endpoint=False)
    wall = np.concatenate([np.stack([side * Lx, np.zeros(nb)], 1), np.stack([np.full(nb, Lx), side * Ly], 1),
                           np.stack([Lx - side * Lx, np.full(nb, Ly)], 1), np.stack([np.zeros(nb), Ly - side * Ly], 1)])
    inner = np.stack([rng.uniform(0.02, 0.98, npts) * Lx, rng.uniform(0.02, 0.98, npts) * Ly], 1)
    pts = np.concatenate([wall, inner])
    tri = Delaunay(pts).simplices
    # drop slivers along the walls (three wall points in a row)
    a, b, c = pts[tri[:, 0]], pts[tri[:, 1]], pts[tri[:, 2]]
    area2 = np.abs((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))
    tri = tri[area2 > 1e-6 * Lx * Ly / npts]
    used = np.zeros(pts.shape[0], bool)
    used[tri.reshape(-1)] = True
    remap = np.cumsum(used) - 1
    pts = pts[used]
    tri = remap[tri]
    order = np.argsort(_morton_key(np.stack([2 * pts[:, 0] / Lx - 1, 2 * pts[:, 1] / Ly - 1, np.zeros(len(pts))], 1)),
                       kind="stable")
    inv = np.empty_like(order)
    inv[order] = np.arange(order.size)
    pts = pts[order]
    tri = inv[tri]
    coord = pts / R_EARTH
    cyc = 1e3 * max(Lx, Ly) / R_EARTH  # never reached: no cyclic wrap
    depth = _seamount_depth(pts[:, 0], pts[:, 1], Lx, Ly, -zbar[-1], seamounts, seed, False)
    return _finish_mesh(coord, tri, cyc, True, zbar, depth, partial_cells, name=f"delaunay_{npts}")


def _icosphere(nsub: int):
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=float)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(nsub):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        lo = np.minimum(e[:, 0], e[:, 1])
        hi = np.maximum(e[:, 0], e[:, 1])
        key = lo * nv + hi
        uk, inv = np.unique(key, return_inverse=True)
        mid = 0.5 * (v[uk // nv] + v[uk % nv])
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1).T + nv  # midpoints of (01, 12, 20)
        v = np.concatenate([v, mid], axis=0)
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1),
                            np.stack([c, m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=0)
    return v, f


def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def sphere_mesh(nsub: int = 7, zbar: Optional[np.ndarray] = None, land_fraction: float = 0.3,
                seed: int = 3, partial_cells: bool = True, polar_cap_deg: float = 12.0) -> Mesh:
    """Icosahedral sphere, ``nsub`` subdivisions, rotated by a seeded rotation,
    land-masked by a seeded smooth field (``land_fraction`` of nodes, plus polar
    caps so that no element straddles a pole of the lon/lat grid), with depth
    from a second smooth field mapped onto 1..nl-1 layers (levels are clamped to
    >= 4 layers as the reference's ``thers_zbar_lev = 5`` requires)."""
    if zbar is None:
        zbar = stretched_zbar(48, 5.0, 250.0)
    rng = np.random.default_rng(seed)
    v, f = _icosphere(nsub)
    v = v @ _random_rotation(rng).T
    lon = np.arctan2(v[:, 1], v[:, 0])
    lat = np.arcsin(np.clip(v[:, 2], -1.0, 1.0))
    land_f = _smooth_field_3d(v, rng, kmin=1.0, kmax=5.0)
    depth_f = _smooth_field_3d(v, rng, kmin=1.5, kmax=7.0)
    thr = np.quantile(land_f, land_fraction)
    wet = (land_f > thr) & (np.abs(lat) < np.deg2rad(90.0 - polar_cap_deg))
    # depth: smooth field -> [~4 layers, full depth], negative downward
    H = -zbar[-1]
    s = 0.5 * (1.0 + np.tanh(depth_f))
    dmin = -zbar[5] * 0.9
    depth = -(dmin + (H - dmin) * s)
    coord = np.stack([lon, lat], axis=1)
    key = _morton_key(v)
    coord, tri, old = _compact(coord, f, wet, key)
    depth = depth[old]
    m = _finish_mesh(coord, tri, 2.0 * np.pi, False, zbar, depth, partial_cells, name=f"sphere_{nsub}")
    m._xyz = v[old]  # type: ignore[attr-defined]
    return m


# ---------------------------------------------------------------------------
# velocities, w, Kv, tracers
# ---------------------------------------------------------------------------
def _coast_taper(mesh: Mesh, hops: int = 3) -> np.ndarray:
    """1 in the interior, 0 on nodes of boundary edges, linear over ``hops`` edges."""
    N2 = mesh.nod2D
    dist = np.full(N2, hops, dtype=np.int64)
    bnd = mesh.edge_tri[:, 1] < 0
    cur = np.zeros(N2, dtype=bool)
    cur[mesh.edges[bnd].reshape(-1)] = True
    dist[cur] = 0
    e = mesh.edges.astype(np.int64)
    for h in range(1, hops):
        nxt = cur.copy()
        nxt[e[cur[e[:, 0]], 1]] = True
        nxt[e[cur[e[:, 1]], 0]] = True
        newly = nxt & ~cur
        dist[newly] = h
        cur = nxt
    return np.minimum(dist, hops) / float(hops)


def _rot_grad(mesh: Mesh, psi_nod: np.ndarray) -> np.ndarray:
    """Element velocity (u, v) = (-dpsi/dy, dpsi/dx) with the reference's
    gradient_sca coefficients (one value per element)."""
    tri = mesh.elem2D_nodes.astype(np.int64)
    gs = mesh.gradient_sca
    px = gs[:, 0] * psi_nod[tri[:, 0]] + gs[:, 1] * psi_nod[tri[:, 1]] + gs[:, 2] * psi_nod[tri[:, 2]]
    py = gs[:, 3] * psi_nod[tri[:, 0]] + gs[:, 4] * psi_nod[tri[:, 1]] + gs[:, 5] * psi_nod[tri[:, 2]]
    return np.stack([-py, px], axis=1)


def vert_vel(mesh: Mesh, uv: np.ndarray) -> np.ndarray:
    """w from the discrete divergence, as src/oce_ale.F90:2165-2306 (linfs):
    edge scatter of helem-weighted segment fluxes, bottom-up cumulative sum,
    divided by area."""
    nl = mesh.nl
    N2 = mesh.nod2D
    W = np.zeros((N2, nl))
    e = mesh.edges.astype(np.int64)
    el1 = mesh.edge_tri[:, 0].astype(np.int64)
    el2 = mesh.edge_tri[:, 1].astype(np.int64)
    ecd = mesh.edge_cross_dxdy
    lev = np.arange(nl - 1)[None, :]
    wet1 = (lev >= (mesh.ulevels[el1] - 1)[:, None]) & (lev < (mesh.nlevels[el1] - 1)[:, None])
    c1 = (uv[el1, :, 1] * ecd[:, 0:1] - uv[el1, :, 0] * ecd[:, 1:2]) * mesh.helem[el1]
    c1 = np.where(wet1, c1, 0.0)
    has2 = el2 >= 0
    e2 = np.maximum(el2, 0)
    wet2 = (lev >= (mesh.ulevels[e2] - 1)[:, None]) & (lev < (mesh.nlevels[e2] - 1)[:, None]) & has2[:, None]
    c2 = -(uv[e2, :, 1] * ecd[:, 2:3] - uv[e2, :, 0] * ecd[:, 3:4]) * mesh.helem[e2]
    c2 = np.where(wet2, c2, 0.0)
    # edge scatter (+ to edges(1,e), - to edges(2,e)) as a segmented sum over
    # edges sorted by node
    c = c1 + c2
    del c1, c2
    nodes = np.concatenate([e[:, 0], e[:, 1]])
    sign = np.concatenate([np.ones(e.shape[0]), -np.ones(e.shape[0])])
    order = np.argsort(nodes, kind="stable")
    rows = np.where(order < e.shape[0], order, order - e.shape[0])
    vals = c[rows] * sign[order][:, None]
    starts = np.flatnonzero(np.r_[True, nodes[order][1:] != nodes[order][:-1]])
    acc = np.zeros((N2, nl - 1))
    acc[nodes[order][starts]] = np.add.reduceat(vals, starts, axis=0)
    del vals
    W[:, :nl - 1] = acc
    # bottom-up cumulative sum over wet levels
    nln = mesh.nlevels_nod2D.astype(np.int64)
    wetn = np.arange(nl)[None, :] < (nln - 1)[:, None]
    W = np.where(wetn, W, 0.0)
    W = np.flip(np.cumsum(np.flip(W, axis=1), axis=1), axis=1)
    W = np.where(wetn, W, 0.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        W = np.where(wetn, W / np.where(mesh.area > 0, mesh.area, 1.0), 0.0)
    return W


def vert_vel_separable(mesh: Mesh, base: np.ndarray, prof: np.ndarray) -> np.ndarray:
    """vert_vel for uv(:, nz, el) = base(:, el) * prof(nz) on wet layers: the
    edge-segment fluxes factor into per-(node, element) coefficients times
    prof*helem, so the node divergence is one sparse product."""
    import scipy.sparse as sp
    nl, N2, T2 = mesh.nl, mesh.nod2D, mesh.elem2D
    e = mesh.edges.astype(np.int64)
    el1 = mesh.edge_tri[:, 0].astype(np.int64)
    el2 = mesh.edge_tri[:, 1].astype(np.int64)
    ecd = mesh.edge_cross_dxdy
    s1 = base[el1, 1] * ecd[:, 0] - base[el1, 0] * ecd[:, 1]
    has2 = el2 >= 0
    e2 = np.maximum(el2, 0)
    s2 = np.where(has2, -(base[e2, 1] * ecd[:, 2] - base[e2, 0] * ecd[:, 3]), 0.0)
    rows = np.concatenate([e[:, 0], e[:, 1], e[:, 0], e[:, 1]])
    cols = np.concatenate([el1, el1, e2, e2])
    vals = np.concatenate([s1, -s1, s2, -s2])
    A = sp.csr_matrix((vals, (rows, cols)), shape=(N2, T2))
    q = mesh.helem * prof[None, :]          # helem is 0 below each element's bottom
    acc = np.asarray(A @ q)
    W = np.zeros((N2, nl))
    W[:, :nl - 1] = acc
    nln = mesh.nlevels_nod2D.astype(np.int64)
    wetn = np.arange(nl)[None, :] < (nln - 1)[:, None]
    W *= wetn
    W = np.flip(np.cumsum(np.flip(W, axis=1), axis=1), axis=1)
    W *= wetn
    with np.errstate(divide="ignore", invalid="ignore"):
        W = np.where(wetn, W / np.where(mesh.area > 0, mesh.area, 1.0), 0.0)
    return W


def make_forcing(mesh: Mesh, kind: str, seed: int = 11, dt: float = 600.0,
                 U0: float = 0.5, Lj: float = 100e3, rms: float = 0.2,
                 kv_profile: str = "surface", surface_w_zero: bool = False) -> Forcing:
    """Seeded velocity / Kv for a mesh.

    ``kind='channel'``: psi = U0*L*tanh(y'/L) + 0.05*U0*L*(Fourier modes k<=8),
    multiplied by a vertical profile; ``kind='basin'``: a closed gyre, psi zero on the walls; ``kind='sphere'``: smooth random psi scaled
    to ``rms`` m/s, tapered to zero on coasts.  Element velocity is the discrete
    rot-grad of psi (divergence-free in the edge-flux form where the dual cell is
    closed), w comes from the discrete divergence.  ``surface_w_zero`` sets
    w(nzmin) = 0 (rigid lid: the total tracer content is then conserved exactly).
    """
    rng = np.random.default_rng(seed)
    nl = mesh.nl
    Zm = mesh.Z
    if kind == "channel":
        x = mesh.coord_nod2D[:, 0] * R_EARTH
        y = mesh.coord_nod2D[:, 1] * R_EARTH
        Lx = mesh.cyclic_length * R_EARTH
        Ly = y.max() - y.min()
        yp = y - (y.min() + 0.5 * Ly)
        psi = U0 * Lj * np.tanh(yp / Lj)
        modes = np.zeros_like(x)
        for k in range(1, 9):
            a, ph, mm = rng.normal(), rng.uniform(0, 2 * np.pi), rng.integers(1, 5)
            modes += a / k * np.sin(2 * np.pi * k * x / Lx + ph) * np.sin(np.pi * mm * (y - y.min()) / Ly)
        psi = psi + 0.05 * U0 * Lj * modes
        prof = 0.3 + 0.7 * np.exp(Zm / 1000.0)
        base = _rot_grad(mesh, psi)
    elif kind == "basin":
        # closed basin: psi vanishes on every wall, a gyre plus seeded modes
        x = mesh.coord_nod2D[:, 0] * R_EARTH
        y = mesh.coord_nod2D[:, 1] * R_EARTH
        Lx, Ly = x.max() - x.min(), y.max() - y.min()
        xs, ys = (x - x.min()) / Lx, (y - y.min()) / Ly
        psi = np.sin(np.pi * xs) * np.sin(np.pi * ys)
        for k in range(1, 5):
            a, mm = rng.normal(), rng.integers(1, 4)
            psi = psi + 0.2 * a / k * np.sin(np.pi * (k + 1) * xs) * np.sin(np.pi * mm * ys)
        psi *= U0 * min(Lx, Ly) / np.pi
        prof = 0.3 + 0.7 * np.exp(Zm / 1000.0)
        base = _rot_grad(mesh, psi)
    else:
        xyz = getattr(mesh, "_xyz", None)
        if xyz is None:
            lon, lat = mesh.coord_nod2D[:, 0], mesh.coord_nod2D[:, 1]
            xyz = np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], 1)
        psi = _smooth_field_3d(xyz, rng, kmin=2.0, kmax=10.0) * _coast_taper(mesh)
        base = _rot_grad(mesh, psi)
        s = np.sqrt(np.mean(np.sum(base ** 2, axis=1)))
        base *= rms / max(s, 1e-300)
        prof = 0.4 + 0.6 * np.exp(Zm / 800.0)
    lev = np.arange(nl - 1)[None, :]
    wet = (lev >= (mesh.ulevels - 1)[:, None]) & (lev < (mesh.nlevels - 1)[:, None])
    uv = np.empty((mesh.elem2D, nl - 1, 2))
    np.multiply(base[:, None, :], prof[None, :, None], out=uv)
    uv *= wet[:, :, None]
    W = vert_vel_separable(mesh, base, prof)
    if surface_w_zero:
        W[np.arange(mesh.nod2D), mesh.ulevels_nod2D - 1] = 0.0
    if kv_profile == "const":
        Kv = np.full((mesh.nod2D, nl), 1e-5)
    else:
        d = -mesh.zbar
        Kv = np.broadcast_to(1e-5 + (1e-2 - 1e-5) * np.exp(-d / 50.0), (mesh.nod2D, nl)).copy()
    return Forcing(uv=uv, w=W, w_e=W.copy(), w_i=np.zeros_like(W), Kv=Kv,
                   bc_surface=np.zeros(mesh.nod2D), dt=float(dt))


def split_vertical_velocity(mesh: Mesh, forcing: Forcing, maxcfl: float) -> Forcing:
    """The forcing with w split into an explicit part w_e and an implicit part w_i as
    compute_Wvel_split does (src/oce_ale.F90:3034-3047): where the vertical Courant number
    exceeds maxcfl, dd = (CFL - maxcfl) / maxcfl, w_e = w / (1 + dd), w_i = dd w / (1 + dd).
    The Courant number of an interface here is |w| dt over the thinner adjacent layer (a
    stand-in for the model's CFL_z diagnostic)."""
    W = forcing.w
    N2, nl = W.shape
    h = np.where(mesh.hnode > 0, mesh.hnode, np.inf)
    up = np.concatenate([np.full((N2, 1), np.inf), h], axis=1)      # layer above interface k
    dn = np.concatenate([h, np.full((N2, 1), np.inf)], axis=1)      # layer below interface k
    hmin = np.minimum(up, dn)
    cfl = np.where(np.isfinite(hmin), np.abs(W) * forcing.dt / hmin, 0.0)
    dd = np.maximum(cfl - maxcfl, 0.0) / max(maxcfl, 1e-12)
    split = cfl > maxcfl
    we = np.where(split, (1.0 / (1.0 + dd)) * W, W)
    wi = np.where(split, (dd / (1.0 + dd)) * W, 0.0)
    return dataclasses.replace(forcing, w_e=np.ascontiguousarray(we), w_i=np.ascontiguousarray(wi))


def node_depth_mid(mesh: Mesh) -> np.ndarray:
    """Layer mid-depth (positive down, metres) per node-layer."""
    return -mesh.Z_3d_n


def make_tracers(mesh: Mesh, kind: str, ntr: int = 2, seed: int = 5, Lj: float = 100e3,
                 noise: Optional[float] = None, dtype=np.float64) -> np.ndarray:
    """Initial tracer values, shape (ntr, N2, nl-1); dry levels are 0.

    Tracer 0 is temperature, 1 salinity, the rest lognormal(0, 1) passive
    tracers (strictly positive).  Each tracer draws from its own seeded stream
    (seed, k), so the values do not depend on the thread that makes them."""
    import concurrent.futures as cf
    N2, nl = mesh.nod2D, mesh.nl
    d = node_depth_mid(mesh)
    out = np.zeros((ntr, N2, nl - 1), dtype=dtype)
    lev = np.arange(nl - 1)[None, :]
    wet = (lev >= (mesh.ulevels_nod2D - 1)[:, None]) & (lev < (mesh.nlevels_nod2D - 1)[:, None])

    def one(k):
        rng = np.random.default_rng([seed, k])
        if k == 0:
            if kind in ("channel", "basin"):
                y = mesh.coord_nod2D[:, 1] * R_EARTH
                yp = y - 0.5 * (y.min() + y.max())
                sig = 0.01 if noise is None else noise
                v = 20.0 - 0.005 * d + 2.0 * np.tanh(yp / Lj)[:, None] + rng.normal(0, sig, d.shape)
            else:
                lat = mesh.coord_nod2D[:, 1]
                sig = 0.1 if noise is None else noise
                v = 2.0 + 26.0 * (np.cos(lat) ** 2)[:, None] * np.exp(-d / 1000.0) + rng.normal(0, sig, d.shape)
        elif k == 1:
            sig = (0.01 if kind in ("channel", "basin") else 0.1) if noise is None else noise
            if kind in ("channel", "basin"):
                v = 35.0 + rng.normal(0, sig, d.shape)
            else:
                lat = mesh.coord_nod2D[:, 1]
                v = 34.0 + 1.5 * np.cos(2 * lat)[:, None] + rng.normal(0, sig, d.shape)
        else:
            z = rng.standard_normal(d.shape, dtype=np.float32)
            v = np.exp(z, out=z)
        np.copyto(out[k], np.where(wet, v, 0.0).astype(dtype, copy=False))

    with cf.ThreadPoolExecutor(max_workers=min(ntr, os.cpu_count() or 4)) as ex:
        list(ex.map(one, range(ntr)))
    return out


def make_slopes(mesh: Mesh, seed: int = 13, smax: float = 2e-3, s_cr: float = 1e-3, s_d: float = 1e-3,
                dtype=np.float64) -> np.ndarray:
    """Tapered neutral slopes slope_tapered(3, nl-1, nod2D) as (N2, nl-1, 3); dry levels 0.

    Components 1, 2 are smooth random horizontal slopes of magnitude ~smax, component 3 their
    norm; all three carry the hyperbolic-tangent taper c = (1 + tanh((s_cr - |S|) / s_d)) / 2 of
    compute_neutral_slope (src/oce_ale_pressure_bv.F90:3039-3157, ODM95 tapering)."""
    rng = np.random.default_rng(seed)
    N2, L1 = mesh.nod2D, mesh.nl - 1
    lat, lon = mesh.coord_nod2D[:, 1], mesh.coord_nod2D[:, 0]
    xyz = np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], axis=1)
    sx = _smooth_field_3d(xyz, rng)[:, None]
    sy = _smooth_field_3d(xyz, rng)[:, None]
    prof = np.exp(-node_depth_mid(mesh) / 1500.0) * (0.5 + rng.uniform(0, 1, (1, L1)))
    S = np.stack([smax * sx * prof, smax * sy * prof], axis=2)
    s3 = np.sqrt(S[:, :, 0] ** 2 + S[:, :, 1] ** 2)
    c = 0.5 * (1.0 + np.tanh((s_cr - s3) / s_d))
    out = np.concatenate([S, s3[:, :, None]], axis=2) * c[:, :, None]
    lev = np.arange(L1)[None, :]
    wet = (lev >= (mesh.ulevels_nod2D - 1)[:, None]) & (lev < (mesh.nlevels_nod2D - 1)[:, None])
    return np.ascontiguousarray(np.where(wet[:, :, None], out, 0.0).astype(dtype))


# ---------------------------------------------------------------------------
# named configurations
# ---------------------------------------------------------------------------
def config_mesh(cfg: int, scale: float = 1.0, seed: int = 1) -> Mesh:
    """Meshes of the benchmark configurations (``scale`` < 1 shrinks them for tests).

    1: channel 100x400, 40 x 100 m levels, flat.
    2: channel 400x1600, 60 levels 10 -> 200 m, Gaussian seamounts, partial cells.
    3: sphere, 7 subdivisions, 48 levels 5 -> 250 m, 30% land, partial cells.
    4: sphere, 9 subdivisions, 70 levels 5 -> 250 m, 30% land, partial cells.
    """
    if cfg == 1:
        nx, ny = max(4, int(round(100 * scale))), max(6, int(round(400 * scale)))
        return channel_mesh(nx, ny, 5000.0, -np.arange(41) * 100.0, seed=seed)
    if cfg == 2:
        nx, ny = max(4, int(round(400 * scale))), max(6, int(round(1600 * scale)))
        return channel_mesh(nx, ny, 5000.0 * (1.0 if scale >= 1 else 1.0), stretched_zbar(60, 10.0, 200.0),
                            seamounts=12, seed=seed, partial_cells=True)
    if cfg == 3:
        nsub = 7 if scale >= 1 else max(3, 7 + int(math.floor(math.log2(max(scale, 1e-6)) / 2)))
        return sphere_mesh(nsub, stretched_zbar(48, 5.0, 250.0), seed=seed + 2)
    if cfg == 4:
        nsub = 9 if scale >= 1 else max(3, 9 + int(math.floor(math.log2(max(scale, 1e-6)) / 2)))
        return sphere_mesh(nsub, stretched_zbar(70, 5.0, 250.0), seed=seed + 3)
    raise ValueError(f"unknown configuration {cfg}")
