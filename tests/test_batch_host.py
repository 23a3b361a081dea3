"""Host logic of the uneven-instance batch: the seeded draw, node reordering (checked
against the oracle) and the partition of instances over ranks, including a two-rank
gloo run of the sharded step with the oracle as the worker (no GPU)."""
import os

import numpy as np
import pytest

from fesom2_gb300 import batch as Bt
from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests.conftest import wet_mask


def test_instance_specs_are_seeded_and_in_range():
    a = Bt.instance_specs()
    b = Bt.instance_specs()
    assert a == b and len(a) == 16
    for s in a:
        assert s.kind in ("channel", "sphere")
        assert 20_000 <= s.nodes_target <= 800_000
        assert 20 <= s.layers <= 80 and 2 <= s.tracers <= 24
    assert {s.kind for s in a} == {"channel", "sphere"}


def test_partition_covers_every_instance_once_and_balances():
    rng = np.random.default_rng(1)
    w = list(rng.lognormal(0, 1, 16))
    for n in (1, 2, 3, 4, 8):
        parts = Bt.partition(w, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(16))
        loads = [sum(w[i] for i in p) for p in parts]
        assert max(loads) <= sum(w) / n + max(w) + 1e-12
        assert parts == Bt.partition(w, n)
    assert Bt.partition([1.0, 1.0], 4)[2:] == [[], []]


def test_permuted_mesh_gives_the_permuted_step(basin_irregular):
    """Renumbering nodes (reverse Cuthill-McKee) leaves the step unchanged up to the order of
    the FP64 sums: the oracle on the permuted mesh equals the permuted oracle result."""
    mesh = basin_irregular
    f = O.ensure_f64(M.make_forcing(mesh, "basin", seed=5, dt=600.0))
    T = M.make_tracers(mesh, "basin", ntr=1, seed=6)[0]
    order = Bt.rcm_order(mesh)
    assert sorted(order.tolist()) == list(range(mesh.nod2D))
    pm = Bt.permute_nodes(mesh, order)
    pf = O.ensure_f64(Bt.permute_forcing(f, order))
    cfg = O.cfg_struct()
    a = T.copy()
    O.OracleMesh(mesh).tracer_step(f, cfg, a, np.zeros_like(a), a.copy())
    b = np.ascontiguousarray(T[order])
    O.OracleMesh(pm).tracer_step(pf, cfg, b, np.zeros_like(b), b.copy())
    wet = wet_mask(mesh)
    assert np.abs(a[order][wet[order]] - b[wet[order]]).max() <= 1e-12 * np.abs(a[wet]).max()


def test_hilbert_key_walks_the_grid_in_unit_steps():
    """The Hilbert index of every point of a full 2^b grid (2-D and 3-D) is a bijection onto
    0..N-1, and points with consecutive indices are one grid step apart."""
    for n, bits in ((2, 5), (3, 3), (3, 4)):
        g = np.stack(np.meshgrid(*[np.arange(1 << bits)] * n, indexing="ij"), -1).reshape(-1, n)
        k = Bt.hilbert_key(g, bits)
        assert np.array_equal(np.sort(k), np.arange(len(g)))
        walk = g[np.argsort(k)]
        assert np.all(np.abs(np.diff(walk, axis=0)).sum(1) == 1)


@pytest.mark.parametrize("meshname", ["basin_irregular", "sphere_small"])
def test_hilbert_order_is_a_local_permutation(meshname, request):
    """hilbert_order is a permutation of the nodes, and along it consecutive nodes lie closer
    together than along a random order (a locality check, on a cartesian and a spherical mesh)."""
    mesh = request.getfixturevalue(meshname)
    order = Bt.hilbert_order(mesh)
    assert np.array_equal(np.sort(order), np.arange(mesh.nod2D))
    lon, lat = mesh.coord_nod2D[:, 0], mesh.coord_nod2D[:, 1]
    p = np.stack([lon, lat], 1) if mesh.cartesian else \
        np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], 1)
    step = lambda o: np.median(np.linalg.norm(np.diff(p[o], axis=0), axis=1))
    rnd = np.random.default_rng(0).permutation(mesh.nod2D)
    assert step(order) < 0.2 * step(rnd)


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    specs = Bt.instance_specs(n=4, seed=77, nodes_lo=400, nodes_hi=1200, layers=(8, 12), tracers=(1, 3))
    weights = [s.nodes_target * s.layers * s.tracers for s in specs]
    mine = Bt.partition(weights, world)[rank]
    result = {}
    for i in mine:
        mesh, kind, forcing, tracers = Bt.make_instance(specs[i])
        f = O.ensure_f64(forcing)
        om = O.OracleMesh(mesh)
        sums = []
        for k in range(specs[i].tracers):
            T = tracers[k].astype(np.float64)
            om.tracer_step(f, O.cfg_struct(), T, np.zeros_like(T), T.copy())
            sums.append(float(np.sum(T)))
        result[i] = sums
    gathered = [None] * world
    dist.all_gather_object(gathered, result)
    if rank == 0:
        merged = {}
        for g in gathered:
            merged.update(g)
        np.save(os.path.join(out_dir, "merged.npy"), np.array([merged], dtype=object), allow_pickle=True)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_step_matches_one_rank(tmp_path):
    """Two gloo ranks each step their share of a small uneven batch (oracle as the worker) and
    gather per-instance checksums; the merge covers every instance once and equals the
    checksums of one process stepping all instances."""
    import torch.multiprocessing as mp
    port = 29500 + (os.getpid() % 2000)
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    merged = np.load(tmp_path / "merged.npy", allow_pickle=True)[0]
    specs = Bt.instance_specs(n=4, seed=77, nodes_lo=400, nodes_hi=1200, layers=(8, 12), tracers=(1, 3))
    assert sorted(merged) == list(range(4))
    for i, s in enumerate(specs):
        mesh, kind, forcing, tracers = Bt.make_instance(s)
        f = O.ensure_f64(forcing)
        om = O.OracleMesh(mesh)
        for k in range(s.tracers):
            T = tracers[k].astype(np.float64)
            om.tracer_step(f, O.cfg_struct(), T, np.zeros_like(T), T.copy())
            assert float(np.sum(T)) == merged[i][k]
