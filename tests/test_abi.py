"""The C-ABI library: loads without a GPU, exports every entry point declared in
include/fesom_gpu.h, and its host-side mesh preparation (validation, MUSCL
init arrays) agrees with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from fesom2_gb300 import build, gpu as G
from fesom2_gb300 import mesh as M
from oracle import oracle as O

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "fesom_gpu.h")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(G.LIB_PATH):
        build.build()
    return G.load()


def declared_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(fesom_gpu_\w+)\s*\(", txt, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("fesom_gpu_init", "fesom_gpu_adv_tra", "fesom_gpu_vdiff_impl", "fesom_gpu_tracer_step",
                 "fesom_gpu_init_tracers_ab", "fesom_gpu_run_steps", "fesom_gpu_finalize"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.fesom_gpu_abi_version() == 1


def test_nm_shows_symbols_as_text(lib):
    import subprocess
    out = subprocess.run(["nm", "-D", G.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fesom_gpu_\w+)", out))
    assert set(declared_functions()) <= exported


@pytest.mark.parametrize("meshname", ["channel_small", "channel_seamount", "sphere_small", "basin_irregular"])
def test_mesh_check_matches_oracle_muscl_init(lib, meshname, request):
    mesh = request.getfixturevalue(meshname)
    nbl, updn = G.mesh_check(mesh)
    om = O.OracleMesh(mesh)
    assert np.array_equal(nbl, om.work["nboundary_lay"])
    assert np.array_equal(updn, om.work["edge_up_dn_tri"])


def test_mesh_check_passes_given_muscl_arrays(lib, channel_small):
    nbl, updn = G.mesh_check(channel_small)
    nbl2, updn2 = G.mesh_check(channel_small, pass_muscl_init=(nbl, updn))
    assert np.array_equal(nbl, nbl2) and np.array_equal(updn, updn2)


def test_mesh_check_rejects_bad_meshes(lib, channel_small):
    import copy
    m = copy.deepcopy(channel_small)
    m.edges = m.edges.copy()
    m.edges[3, 0] = m.nod2D + 5
    with pytest.raises(G.FesomGpuError) as e:
        G.mesh_check(m)
    assert e.value.rc == 3 and "edges" in str(e.value)
    m = copy.deepcopy(channel_small)
    m.nlevels_nod2D = m.nlevels_nod2D.copy()
    m.nlevels_nod2D[0] = 2          # one layer only
    with pytest.raises(G.FesomGpuError) as e:
        G.mesh_check(m)
    assert e.value.rc == 3


def test_missing_library_fails_loudly(tmp_path):
    import importlib
    G2 = importlib.reload(G)
    G2._lib = None
    with pytest.raises(FileNotFoundError):
        G2.load(str(tmp_path / "nope.so"))
    importlib.reload(G)


@pytest.mark.parametrize("field,index,value", [("elem2D_nodes", (0, 1), -1), ("elem2D_nodes", (5, 2), 10 ** 6),
                                               ("edge_tri", (0, 0), 10 ** 6), ("nlevels", (2,), 99),
                                               ("ulevels_nod2D", (0,), 40), ("edges", (1, 1), -3)])
def test_mesh_check_rejects_out_of_range_entries(lib, channel_small, field, index, value):
    """Index and level validation on the host, before any device work: every out-of-range
    entry is a FESOM_ERR_MESH with a message."""
    import copy
    m = copy.deepcopy(channel_small)
    a = getattr(m, field).copy()
    a[index] = value
    setattr(m, field, a)
    with pytest.raises(G.FesomGpuError) as e:
        G.mesh_check(m)
    assert e.value.rc == 3 and len(str(e.value)) > 20
