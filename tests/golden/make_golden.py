"""Generate tests/golden/*.npz: small self-contained cases (mesh arrays, forcing,
initial tracers) and the FP64 oracle's results after each of 3 tracer steps.

The fixtures hold every input, so the checks do not depend on the mesh
generator or on numpy's random streams on the machine that runs them.
Run from the repository root:  python tests/golden/make_golden.py
"""
import dataclasses
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fesom2_gb300 import mesh as M  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = {
    "channel_seamount_fct": dict(make=lambda: M.channel_mesh(8, 10, 5000.0, M.stretched_zbar(20, 10.0, 150.0),
                                                             seamounts=2, seed=6, partial_cells=True),
                                 kind="channel", scheme=("MUSCL", "QR4C", "FCT"), ab=2),
    "sphere_mfct_ab3": dict(make=lambda: M.sphere_mesh(3, M.stretched_zbar(10, 10.0, 200.0), seed=5),
                            kind="sphere", scheme=("MFCT", "QR4C", "FCT"), ab=3),
    "channel_upw1_nolim": dict(make=lambda: M.channel_mesh(6, 8, 5000.0, -np.arange(13) * 50.0),
                               kind="channel", scheme=("UPW1", "UPW1", "NON"), ab=2),
}
MESH_FIELDS = [f.name for f in dataclasses.fields(M.Mesh)]


def make(name, spec):
    mesh = spec["make"]()
    f = O.ensure_f64(M.make_forcing(mesh, spec["kind"], seed=3, dt=600.0))
    f.bc_surface = np.linspace(-1e-4, 1e-4, mesh.nod2D)
    tr = M.make_tracers(mesh, spec["kind"], ntr=2, seed=7)
    rng = np.random.default_rng(11)
    ab = spec["ab"]
    om = O.OracleMesh(mesh)
    cfg = O.cfg_struct(*spec["scheme"], ph=0.0, pv=1.0, ab_order=ab)
    out = {}
    for k in range(2):
        T = np.array(tr[k], copy=True)
        old = np.stack([T * (1 + 1e-3 * rng.standard_normal(T.shape)) for _ in range(ab - 1)], axis=-1)
        old = np.ascontiguousarray(old)
        out[f"T0_{k}"] = T.copy()
        out[f"old0_{k}"] = old.copy()
        for s in range(3):
            om.tracer_step(f, cfg, T, np.zeros_like(T), old)
            out[f"T{s + 1}_{k}"] = T.copy()
            out[f"old{s + 1}_{k}"] = old.copy()
    arrays = {f"mesh_{k}": getattr(mesh, k) for k in MESH_FIELDS if isinstance(getattr(mesh, k), np.ndarray)}
    scalars = {f"meshs_{k}": np.array(getattr(mesh, k)) for k in MESH_FIELDS if not isinstance(getattr(mesh, k), np.ndarray)}
    forc = {f"forcing_{k}": getattr(f, k) for k in ("uv", "w", "w_e", "w_i", "Kv", "bc_surface")}
    meta = {"scheme": np.array(spec["scheme"]), "ab": np.array(ab), "dt": np.array(f.dt),
            "muscl_nbl": om.work["nboundary_lay"], "muscl_updn": om.work["edge_up_dn_tri"]}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), f"{name}.npz")
    np.savez_compressed(path, **arrays, **scalars, **forc, **out, **meta)
    print(path, os.path.getsize(path))


def load(name):
    """Rebuild (mesh, forcing, data) from a fixture."""
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), f"{name}.npz"))
    kw = {}
    for k in MESH_FIELDS:
        if f"mesh_{k}" in d:
            kw[k] = d[f"mesh_{k}"]
        elif f"meshs_{k}" in d:
            v = d[f"meshs_{k}"]
            kw[k] = v.item() if v.shape == () else v
    kw["nl"] = int(kw["nl"])
    kw["edge2D_in"] = int(kw["edge2D_in"])
    kw["cyclic_length"] = float(kw["cyclic_length"])
    kw["cartesian"] = bool(kw["cartesian"])
    kw["name"] = str(kw["name"])
    mesh = M.Mesh(**kw)
    f = M.Forcing(**{k: d[f"forcing_{k}"] for k in ("uv", "w", "w_e", "w_i", "Kv", "bc_surface")}, dt=float(d["dt"]))
    return mesh, f, d


if __name__ == "__main__":
    for name, spec in CASES.items():
        make(name, spec)
