"""The launch-shape autotuner: it leaves the bound state as it was, picks a
block height per tunable kernel among 4, 2, 1, and the hot path with the chosen
shapes still matches the oracle."""
import numpy as np
import pytest

from harness import Pair, relerr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TUNABLE = ("fct_a", "fct_b", "fct_c", "iso_flux", "zdf_imp", "spg_cor", "spg_p1a", "spg_p1b", "spg_p3")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_autotune_keeps_state_and_parity(prec):
    p = Pair(nn=2, prec=prec, seed=41, nmem=2)
    p.bind_hotpath()
    names = ("TSA", "UN", "VN", "UA", "VA", "SSHA", "UA_B", "UN_ADV", "AH_WSLP2")
    before = {n: p.dev[n].clone() for n in names}
    torch.cuda.synchronize()
    p.ctx.autotune(5, nrep=2)
    p.ctx.synchronize()
    for n in names:
        assert torch.equal(before[n], p.dev[n]), n
    shape = p.ctx.launch_shape()
    assert all(shape[k] in (1, 2, 4) for k in TUNABLE)
    for kt in (5, 6):
        for o in p.ora:
            o.stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
    p.ctx.synchronize()
    tol = 1e-12 if prec == "fp64" else 5e-6
    p.compare("TSA", p.s4, tol)
    p.compare("UN", p.s3, 1e-12 if prec == "fp64" else 2e-3)
