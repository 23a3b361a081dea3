"""Shared fixtures: small seeded meshes and forcings; the `gpu` marker."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from fesom2_gb300 import mesh as M  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available() -> bool:
    """True when the CUDA driver reports a device (checked through libcuda, no torch import)."""
    import ctypes
    try:
        cu = ctypes.CDLL("libcuda.so.1")
        if cu.cuInit(0) != 0:
            return False
        n = ctypes.c_int(0)
        return cu.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def channel_small():
    """12 x 16 channel, 40 x 100 m levels, flat (configuration 1 layout, shrunk)."""
    return M.channel_mesh(12, 16, 5000.0, -np.arange(41) * 100.0)


@pytest.fixture(scope="session")
def channel_seamount():
    """16 x 24 channel, 60 stretched levels, seamounts and partial cells (configuration 2 layout, shrunk)."""
    return M.channel_mesh(16, 24, 5000.0, M.stretched_zbar(60, 10.0, 200.0), seamounts=3, seed=4,
                          partial_cells=True)


@pytest.fixture(scope="session")
def sphere_small():
    """Icosahedral sphere, 4 subdivisions, 30% land, 48 levels, partial cells (configuration 3 layout, shrunk)."""
    return M.sphere_mesh(4, M.stretched_zbar(48, 5.0, 250.0), seed=9)


@pytest.fixture(scope="session")
def basin_irregular():
    """Closed basin, Delaunay triangulation of 400 random points (node degrees 2 to 10),
    30 stretched levels, seamounts and partial cells."""
    return M.delaunay_mesh(400, zbar=M.stretched_zbar(30, 10.0, 200.0), seamounts=2, seed=3, partial_cells=True)


def wet_mask(mesh):
    lev = np.arange(mesh.nl - 1)[None, :]
    return (lev >= (mesh.ulevels_nod2D - 1)[:, None]) & (lev < (mesh.nlevels_nod2D - 1)[:, None])


def perturbed_old(T, rng, scale=1e-3):
    """valuesold for the first AB step: T plus a small seeded perturbation."""
    return np.ascontiguousarray(T * (1.0 + scale * rng.standard_normal(T.shape)))


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="session")
def soufflet_file_mesh():
    """The Soufflet channel of the reference's test data (2875 nodes, 41 levels, Cartesian,
    cyclic over 4.5 degrees), built from the copy of its .out files in tests/golden."""
    from fesom2_gb300 import meshio as MI
    return MI.mesh_from_files(MI.load_files(os.path.join(GOLDEN, "mesh_soufflet.npz")), name="soufflet",
                              **MI.SOUFFLET)


@pytest.fixture(scope="session")
def pi_file_mesh():
    """The PI mesh of the reference's test data (3140 nodes, 48 levels, global, rotated by
    the Euler angles 50, 15, -90), built from the copy of its .out files in tests/golden."""
    from fesom2_gb300 import meshio as MI
    return MI.mesh_from_files(MI.load_files(os.path.join(GOLDEN, "mesh_pi.npz")), name="pi", **MI.PI)


@pytest.fixture(scope="session")
def pi_cavity_file_mesh():
    """The PI mesh with ice-shelf cavities of the reference's test data (6808 nodes, 48 levels,
    170 elements whose columns start below the surface), from the copy in tests/golden."""
    from fesom2_gb300 import meshio as MI
    return MI.mesh_from_files(MI.load_files(os.path.join(GOLDEN, "mesh_pi_cavity.npz")), name="pi_cavity",
                              **MI.PI_CAVITY)


def shallow_mesh(nl: int = 5, seed: int = 7):
    """A 10 x 12 channel whose element columns hold 2 to nl-1 layers at random (2-layer,
    3-layer and deeper columns side by side): the shortest columns the path accepts."""
    base = M.channel_mesh(10, 12, 5000.0, -np.arange(nl) * 40.0)
    rng = np.random.default_rng(seed)
    p = np.r_[0.7, np.full(nl - 3, 0.3 / (nl - 3))]
    nlev = rng.choice(np.arange(3, nl + 1), size=base.elem2D, p=p).astype(np.int32)
    depth = np.full(base.nod2D, -40.0 * (nl - 1))
    return M._finish_mesh(base.coord_nod2D, base.elem2D_nodes.astype(np.int64), base.cyclic_length, True,
                          base.zbar, depth, False, "shallow", nlevels=nlev)


@pytest.fixture(scope="session")
def shallow_channel():
    return shallow_mesh()

