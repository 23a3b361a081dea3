"""Edge cases of the oracle on the shortest columns the path accepts (2 and 3 layers next to
deeper ones): both restatements agree bit for bit, a constant tracer stays constant."""
import numpy as np
import pytest

from fesom2_gb300 import mesh as M
from oracle import oracle as O
from tests import refimpl as RI
from tests.conftest import perturbed_old, wet_mask
from tests.refimpl import Ref

OPTIONS = [("MUSCL", "QR4C", "FCT", False), ("UPW1", "UPW1", "NON", False), ("MFCT", "CDIFF", "FCT", False),
           ("MUSCL", "PPM", "FCT", False), ("UPW1", "PPM", "NON", False), ("MUSCL", "QR4C", "FCT", True),
           ("MFCT", "CDIFF", "NON", True)]
IDS = ["-".join(map(str, o)) for o in OPTIONS]


def test_shallow_mesh_has_two_layer_columns(shallow_channel):
    lay = shallow_channel.nlevels_nod2D - shallow_channel.ulevels_nod2D
    assert lay.min() == 2 and (lay == 2).sum() >= 5 and (lay == 3).sum() >= 5


@pytest.mark.parametrize("opt", OPTIONS, ids=IDS)
def test_short_columns_match_restatement(shallow_channel, opt):
    hor, ver, lim, ws = opt
    mesh = shallow_channel
    f = O.ensure_f64(M.make_forcing(mesh, "channel", seed=3, dt=600.0))
    if ws:
        f = M.split_vertical_velocity(mesh, f, maxcfl=0.001)
    T = np.ascontiguousarray(M.make_tracers(mesh, "channel", ntr=1, seed=4)[0])
    Told = perturbed_old(T, np.random.default_rng(1))
    om = O.OracleMesh(mesh)
    To, Oo = T.copy(), Told.copy()
    om.tracer_step(f, O.cfg_struct(hor, ver, lim, wsplit=ws), To, np.zeros_like(To), Oo)
    Tr, Or = Ref(mesh).tracer_step(f, T, Told, om.work["edge_up_dn_tri"], om.work["nboundary_lay"], hor, ver, lim,
                                   wsplit=ws)
    assert np.array_equal(To, Tr)
    assert np.array_equal(Oo, Or)


@pytest.mark.parametrize("opt", OPTIONS, ids=IDS)
def test_short_columns_keep_a_constant(shallow_channel, opt):
    hor, ver, lim, ws = opt
    if ws:
        pytest.skip("the split velocity's implicit LO step keeps a constant only to the column divergence of w_i")
    mesh = shallow_channel
    f = O.ensure_f64(M.make_forcing(mesh, "channel", seed=3, dt=600.0))
    wet = wet_mask(mesh)
    T = np.ascontiguousarray(np.where(wet, 4.5, 0.0))
    Told = T.copy()
    O.OracleMesh(mesh).tracer_step(f, O.cfg_struct(hor, ver, lim), T, np.zeros_like(T), Told)
    assert np.abs(T[wet] - 4.5).max() < 1e-12
