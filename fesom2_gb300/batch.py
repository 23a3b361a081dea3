"""Uneven-instance batch (the fifth benchmark configuration) and its partition over ranks.

Sixteen independent meshes, channel or sphere by a seeded coin, with node counts drawn
log-uniform in [20k, 800k], 20..80 layers and 2..24 tracers each, every one with its own
seeded velocity, Kv profile and tracers.  All instances step together through
``fesom2_gb300.gpu.Batch`` (one launch per stage over all of them).

Before batching, each instance's node order is chosen by timing: the generators' Morton
order, reverse Cuthill-McKee on the node graph, or a Hilbert curve through the node positions.  With several ranks the instances are
split by greedy longest-processing-time packing of their work (tracer-DOF per step); the
instances are independent, so ranks exchange no data, only timings and per-instance metrics.
"""
from __future__ import annotations

import dataclasses
import math
import time
from typing import List, Optional, Sequence

import numpy as np

from . import mesh as M


@dataclasses.dataclass
class InstanceSpec:
    index: int
    kind: str            # "channel" | "sphere"
    nodes_target: int
    layers: int
    tracers: int
    seed: int


def instance_specs(n: int = 16, seed: int = 2024, nodes_lo: int = 20_000, nodes_hi: int = 800_000,
                   layers=(20, 80), tracers=(2, 24)) -> List[InstanceSpec]:
    """The seeded draw of the batch: kind, node count, layers and tracers of each instance."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        kind = "channel" if rng.random() < 0.5 else "sphere"
        nodes = int(round(math.exp(rng.uniform(math.log(nodes_lo), math.log(nodes_hi)))))
        nlay = int(rng.integers(layers[0], layers[1] + 1))
        ntr = int(rng.integers(tracers[0], tracers[1] + 1))
        out.append(InstanceSpec(i, kind, nodes, nlay, ntr, int(rng.integers(1, 1 << 30))))
    return out


def make_instance(spec: InstanceSpec, node_scale: float = 1.0):
    """Mesh, forcing, tracers and scheme configurations of one instance.

    ``node_scale`` < 1 shrinks the node count (tests); channels take ny = 4 nx rows, spheres
    the subdivision whose masked node count is closest to the target."""
    target = max(400, int(spec.nodes_target * node_scale))
    if spec.kind == "channel":
        nx = max(6, int(round(math.sqrt(target / 4.0))))
        zbar = M.stretched_zbar(spec.layers, 10.0, 200.0)
        mesh = M.channel_mesh(nx, 4 * nx, 5000.0, zbar, seamounts=max(1, nx // 40), seed=spec.seed % 100000,
                              partial_cells=True)
        kind = "channel"
    else:
        # masked node count of each subdivision (about 65% of the icosphere's vertices)
        sizes = {k: 0.65 * (10 * 4 ** k + 2) for k in range(3, 9)}
        nsub = min(sizes, key=lambda k: abs(math.log(sizes[k] / target)))
        zbar = M.stretched_zbar(spec.layers, 5.0, 250.0)
        mesh = M.sphere_mesh(nsub, zbar, seed=spec.seed % 100000)
        kind = "sphere"
    forcing = M.make_forcing(mesh, kind, seed=spec.seed % 99991, dt=600.0)
    tracers = M.make_tracers(mesh, kind, ntr=spec.tracers, seed=spec.seed % 99989, dtype=np.float32)
    return mesh, kind, forcing, tracers


# ---------------------------------------------------------------------------
# node reordering
# ---------------------------------------------------------------------------
def rcm_order(mesh: M.Mesh) -> np.ndarray:
    """Reverse Cuthill-McKee order of the node graph (new position -> old node)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import reverse_cuthill_mckee
    e = mesh.edges.astype(np.int64)
    N = mesh.nod2D
    A = coo_matrix((np.ones(2 * len(e)), (np.r_[e[:, 0], e[:, 1]], np.r_[e[:, 1], e[:, 0]])), shape=(N, N)).tocsr()
    return np.asarray(reverse_cuthill_mckee(A, symmetric_mode=True), dtype=np.int64)


def hilbert_key(q: np.ndarray, bits: int) -> np.ndarray:
    """Position along the Hilbert curve of the integer points q (N, n) in [0, 2^bits)^n
    (n * bits <= 63): J. Skilling's transpose method ("Programming the Hilbert curve", AIP Conf.
    Proc. 707, 381 (2004)) — the coordinates are turned into the curve's transposed index by
    inverting and exchanging low bits from the top bit down, Gray-decoded, and the index bits are
    read out interleaved (coordinate 0 most significant within each bit level)."""
    q = np.asarray(q, dtype=np.int64)
    n = q.shape[1]
    X = [q[:, i].copy() for i in range(n)]
    top = np.int64(1) << (bits - 1)
    Q = top
    while Q > 1:
        P = Q - 1
        for i in range(n):
            hit = (X[i] & Q) != 0
            X[0] = np.where(hit, X[0] ^ P, X[0])            # invert the low bits of X[0]
            t = np.where(hit, 0, (X[0] ^ X[i]) & P)         # or exchange them with X[i]'s
            X[0] ^= t
            X[i] ^= t
        Q >>= 1
    for i in range(1, n):
        X[i] ^= X[i - 1]
    t = np.zeros_like(X[0])
    Q = top
    while Q > 1:
        t = np.where((X[n - 1] & Q) != 0, t ^ (Q - 1), t)
        Q >>= 1
    for i in range(n):
        X[i] ^= t
    key = np.zeros_like(X[0])
    for b in range(bits - 1, -1, -1):
        for i in range(n):
            key = (key << 1) | ((X[i] >> b) & 1)
    return key


def hilbert_order(mesh: M.Mesh, bits: int = 20) -> np.ndarray:
    """Nodes along a Hilbert curve through their positions (new position -> old node): the 3-D
    curve through the unit-sphere points of the nodes' lon/lat on a spherical mesh, the 2-D curve
    through x/y on a cartesian one.  Unlike the Morton order it has no jumps between far-apart
    cells, so consecutive nodes (and the blocks of warps that take them) stay neighbours."""
    lon, lat = mesh.coord_nod2D[:, 0], mesh.coord_nod2D[:, 1]
    if mesh.cartesian:
        p = np.stack([lon, lat], 1)
    else:
        p = np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], 1)
    lo, hi = p.min(0), p.max(0)
    q = np.clip(((p - lo) / np.maximum(hi - lo, 1e-300) * ((1 << bits) - 1)).astype(np.int64), 0, (1 << bits) - 1)
    return np.argsort(hilbert_key(q, bits), kind="stable").astype(np.int64)


def permute_nodes(mesh: M.Mesh, order: np.ndarray) -> M.Mesh:
    """The same mesh with its nodes renumbered (``order[new] = old``): node arrays permuted,
    element and edge node indices remapped, edges re-sorted (internal first, then by their
    lower and upper new node, as the generators lay them out), node-to-element lists rebuilt."""
    N = mesh.nod2D
    inv = np.empty(N, dtype=np.int64)
    inv[order] = np.arange(N)
    tri = inv[mesh.elem2D_nodes].astype(np.int32)
    ed = inv[mesh.edges]
    internal = mesh.edge_tri[:, 1] >= 0
    key = np.minimum(ed[:, 0], ed[:, 1]) * (N + 1) + np.maximum(ed[:, 0], ed[:, 1])
    eorder = np.lexsort((key, ~internal))
    ptr, nie = M._nod_in_elem(tri.astype(np.int64), N)
    out = dataclasses.replace(
        mesh,
        coord_nod2D=np.ascontiguousarray(mesh.coord_nod2D[order]), elem2D_nodes=tri,
        edges=np.ascontiguousarray(ed[eorder].astype(np.int32)),
        edge_tri=np.ascontiguousarray(mesh.edge_tri[eorder]),
        nod_in_elem2D_ptr=ptr, nod_in_elem2D=nie,
        nlevels_nod2D=mesh.nlevels_nod2D[order], ulevels_nod2D=mesh.ulevels_nod2D[order],
        nlevels_nod2D_min=mesh.nlevels_nod2D_min[order], ulevels_nod2D_max=mesh.ulevels_nod2D_max[order],
        edge_dxdy=np.ascontiguousarray(mesh.edge_dxdy[eorder]),
        edge_cross_dxdy=np.ascontiguousarray(mesh.edge_cross_dxdy[eorder]),
        area=mesh.area[order], areasvol=mesh.areasvol[order], hnode=mesh.hnode[order],
        hnode_new=mesh.hnode_new[order], zbar_3d_n=mesh.zbar_3d_n[order], Z_3d_n=mesh.Z_3d_n[order],
        zbar_n_bot=mesh.zbar_n_bot[order], name=mesh.name + "_perm")
    return out


def permute_forcing(f: M.Forcing, order: np.ndarray) -> M.Forcing:
    return M.Forcing(uv=f.uv, w=f.w[order], w_e=f.w_e[order], w_i=f.w_i[order], Kv=f.Kv[order],
                     bc_surface=None if f.bc_surface is None else f.bc_surface[order], dt=f.dt)


def orderings(mesh: M.Mesh) -> dict:
    """Candidate node orders: as generated (Morton), reverse Cuthill-McKee, Hilbert curve."""
    return {"morton": np.arange(mesh.nod2D), "rcm": rcm_order(mesh), "hilbert": hilbert_order(mesh)}


def autotune_order(mesh, forcing, tracers, cfgs, steps: int = 2, stream=None):
    """Time the FP32 step of one instance under each candidate node order and return
    (name, order, {name: ms per step}).  Needs a GPU."""
    import torch

    from . import gpu as G
    f32 = M.Forcing(uv=forcing.uv.astype(np.float32), w=forcing.w.astype(np.float32),
                    w_e=forcing.w_e.astype(np.float32), w_i=forcing.w_i.astype(np.float32),
                    Kv=forcing.Kv.astype(np.float32), bc_surface=None, dt=forcing.dt)
    times = {}
    best = None
    cands = orderings(mesh)
    for name, order in cands.items():
        m = mesh if name == "morton" else permute_nodes(mesh, order)
        f = f32 if name == "morton" else permute_forcing(f32, order)
        ctx = G.Context(m, G.PREC_FP32, max_tracers=len(cfgs))
        if stream is not None:
            ctx.set_stream(stream.cuda_stream)
        ctx.state_setup(cfgs)
        ctx.forcing_upload(f)
        for k in range(len(cfgs)):
            T = tracers[k] if name == "morton" else tracers[k][order]
            ctx.tracer_upload(k, T, T)
        ctx.run_steps(forcing.dt, 1, use_graph=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.run_steps(forcing.dt, steps, use_graph=True)
        torch.cuda.synchronize()
        times[name] = (time.perf_counter() - t0) * 1e3 / steps
        ctx.close()
        if best is None or times[name] < times[best]:
            best = name
    return best, cands[best], times


# ---------------------------------------------------------------------------
# partition over ranks
# ---------------------------------------------------------------------------
def partition(weights: Sequence[float], nranks: int) -> List[List[int]]:
    """Greedy longest-processing-time packing: instances in decreasing weight, each to the
    rank with the least work so far (ties to the lower rank).  Every instance goes to
    exactly one rank; the result is deterministic."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    load = [0.0] * nranks
    parts: List[List[int]] = [[] for _ in range(nranks)]
    for i in order:
        r = min(range(nranks), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += weights[i]
    return [sorted(p) for p in parts]


def work(mesh: M.Mesh, ntr: int) -> int:
    """Tracer-DOF of one step of an instance (the partition weight and the metric's units)."""
    return int(ntr * np.sum(mesh.nlevels_nod2D - mesh.ulevels_nod2D))


def scheme_configs(ntr: int, cfg_factory, seed: int) -> list:
    """Per-tracer schemes of an instance: T and S (ids 1, 2) and passive tracers (ids 100+),
    MUSCL + QR4C + FCT with implicit vertical diffusion, as the reference's defaults."""
    return [cfg_factory("MUSCL", "QR4C", "FCT", 0.0, 1.0, id=(k + 1 if k < 2 else 100 + k)) for k in range(ntr)]
