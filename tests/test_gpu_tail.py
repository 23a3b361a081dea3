"""fesom_gpu_tracer_tail (decay, climatology relaxation, salinity and age clamps) equals the
oracle bit for bit, through the C ABI."""
import numpy as np
import pytest

from fesom2_gb300 import gpu as G
from oracle import oracle as O
from tests.test_oracle import _tail_inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("zonal", [0, 1])
def test_tail_bitwise(channel_seamount, zonal):
    mesh = channel_seamount
    ids = [1, 2, 14, 39, 101]
    vals, r2c, Tclim, Sclim, ztem = _tail_inputs(mesh, len(ids), 9)
    y = mesh.coord_nod2D[:, 1]
    kw = dict(salt_index=1, age_index=4, zonal_relax=zonal, nbins=12, lat0=float(y.min()),
              dy=float((y.max() - y.min()) / 12), tau_inv=1.0 / 86400.0)
    want = [v.copy() for v in vals]
    O.tracer_tail(O.OracleMesh(mesh), ids, 600.0, O.tail_cfg(**kw), r2c, Tclim, Sclim, ztem, want)
    ctx = G.Context(mesh, G.PREC_FP64)
    got = [v.copy() for v in vals]
    ctx.tracer_tail([G.tra_cfg(id=i) for i in ids], 600.0, G.tail_cfg(**kw), r2c, Tclim, Sclim, ztem, got)
    for k in range(len(ids)):
        assert np.array_equal(got[k], want[k]), (zonal, k)


def test_tail_needs_fp64_and_inputs(channel_small):
    ctx = G.Context(channel_small, G.PREC_FP32)
    v = [np.zeros((channel_small.nod2D, channel_small.nl - 1))]
    with pytest.raises(G.FesomGpuError):
        ctx.tracer_tail([G.tra_cfg(id=1)], 600.0, G.tail_cfg(), None, None, None, None, v)
    c64 = G.Context(channel_small, G.PREC_FP64)
    with pytest.raises(G.FesomGpuError):
        c64.tracer_tail([G.tra_cfg(id=1)], 600.0, G.tail_cfg(), None, None, None, None, v)
