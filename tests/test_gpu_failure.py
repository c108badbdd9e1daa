"""The failure path of the tensor-core pipelines on the GPU, without a GPU
fault: every mbarrier wait is bounded; a wait that gives up records
XC_ERR_TIMEOUT, its kernel unwinds (TMEM released, nothing in flight) and
the call returns XC_ERR_TIMEOUT with the CUDA context still usable.
xc_grid_wait_probe makes such a wait run out (a barrier nothing arrives on,
a budget of milliseconds); the builds before and after it must agree."""
import numpy as np
import pytest

import chinium_gb300 as cg
from chinium_gb300 import molecules as M
from chinium_gb300._lib import lib
from conftest import model_density

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_the_grid_stays_usable(h2o_oracle):
    Z, xyz, ob, og = h2o_oracle
    b = cg.Basis(Z, xyz, "def2-svp")
    g = cg.Grid(b, "SG-1")
    xc = cg.ExchangeCorrelation().Read("PBE")
    g.setType(xc.type)
    g.getAO(0)
    D = model_density(og, 5)
    E64, V64 = g.build(xc, [D])
    E1, V1 = g.build(xc, [D], precision=cg.PRECISION_MIXED)
    for budget_ms in (2.0, 20.0):
        with pytest.raises(cg.XCError) as e:
            g.wait_probe(budget_ms)
        assert e.value.code == -8  # XC_ERR_TIMEOUT
    # the context and the grid are intact: the same mixed and FP64 results
    E2, V2 = g.build(xc, [D], precision=cg.PRECISION_MIXED)
    assert E2 == E1 and np.abs(V2[0] - V1[0]).max() < 1e-14
    E3, V3 = g.build(xc, [D])
    assert abs(E3 - E64) < 1e-13 and np.abs(V3[0] - V64[0]).max() < 1e-13
