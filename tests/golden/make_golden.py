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
    # the later rows: PPM with the split vertical velocity; CDIFF without the limiter, with
    # horizontal diffusion and one tracer on explicit vertical diffusion
    "basin_ppm_wsplit": dict(make=lambda: M.delaunay_mesh(150, zbar=M.stretched_zbar(16, 10.0, 150.0), seamounts=1,
                                                          seed=8, partial_cells=True),
                             kind="basin", scheme=("MFCT", "PPM", "FCT"), ab=2, wsplit=0.01),
    "channel_cdiff_hdiff": dict(make=lambda: M.channel_mesh(8, 10, 5000.0, M.stretched_zbar(14, 10.0, 150.0),
                                                            seamounts=1, seed=3, partial_cells=True),
                                kind="channel", scheme=("MUSCL", "CDIFF", "NON"), ab=3, khor=2e5, ivd=(1, 0)),
}
MESH_FIELDS = [f.name for f in dataclasses.fields(M.Mesh)]


def ki_field(mesh, K_hor):
    """Ki = K_hor (resolution / 100 km)^2 (src/oce_setup_step.F90:968-972), the resolution
    from the node's mean element area."""
    ea = np.zeros(mesh.nod2D)
    np.add.at(ea, mesh.elem2D_nodes.reshape(-1), np.repeat(mesh.elem_area, 3) / 3.0)
    res = np.sqrt(ea)
    return np.ascontiguousarray(np.repeat((K_hor * (res / 100000.0) ** 2)[:, None], mesh.nl - 1, axis=1))


def make(name, spec):
    mesh = spec["make"]()
    f = O.ensure_f64(M.make_forcing(mesh, spec["kind"], seed=3, dt=600.0))
    if spec.get("wsplit"):
        f = M.split_vertical_velocity(mesh, f, maxcfl=spec["wsplit"])
    f.bc_surface = np.linspace(-1e-4, 1e-4, mesh.nod2D)
    Ki = ki_field(mesh, spec["khor"]) if spec.get("khor") else None
    ivd = spec.get("ivd", (1, 1))
    tr = M.make_tracers(mesh, spec["kind"], ntr=2, seed=7)
    rng = np.random.default_rng(11)
    ab = spec["ab"]
    om = O.OracleMesh(mesh)
    out = {}
    for k in range(2):
        cfg = O.cfg_struct(*spec["scheme"], ph=0.0, pv=1.0, ab_order=ab, i_vert_diff=bool(ivd[k]),
                           wsplit=bool(spec.get("wsplit")))
        T = np.array(tr[k], copy=True)
        old = np.stack([T * (1 + 1e-3 * rng.standard_normal(T.shape)) for _ in range(ab - 1)], axis=-1)
        old = np.ascontiguousarray(old)
        out[f"T0_{k}"] = T.copy()
        out[f"old0_{k}"] = old.copy()
        for s in range(3):
            om.tracer_step_ex(f, cfg, T, np.zeros_like(T), old, Ki=Ki)
            out[f"T{s + 1}_{k}"] = T.copy()
            out[f"old{s + 1}_{k}"] = old.copy()
    arrays = {f"mesh_{k}": getattr(mesh, k) for k in MESH_FIELDS if isinstance(getattr(mesh, k), np.ndarray)}
    scalars = {f"meshs_{k}": np.array(getattr(mesh, k)) for k in MESH_FIELDS if not isinstance(getattr(mesh, k), np.ndarray)}
    forc = {f"forcing_{k}": getattr(f, k) for k in ("uv", "w", "w_e", "w_i", "Kv", "bc_surface")}
    meta = {"scheme": np.array(spec["scheme"]), "ab": np.array(ab), "dt": np.array(f.dt),
            "muscl_nbl": om.work["nboundary_lay"], "muscl_updn": om.work["edge_up_dn_tri"],
            "wsplit": np.array(bool(spec.get("wsplit"))), "ivd": np.array(ivd, dtype=np.int32)}
    if Ki is not None:
        meta["Ki"] = Ki
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


def options(d):
    """(wsplit, Ki or None, i_vert_diff per tracer) of a fixture (defaults for the first ones)."""
    ws = bool(d["wsplit"]) if "wsplit" in d else False
    Ki = d["Ki"] if "Ki" in d else None
    ivd = tuple(int(x) for x in d["ivd"]) if "ivd" in d else (1, 1)
    return ws, Ki, ivd


if __name__ == "__main__":
    # python tests/golden/make_golden.py [case ...]: the named cases, else every case
    for name, spec in CASES.items():
        if len(sys.argv) == 1 or name in sys.argv[1:]:
            make(name, spec)
