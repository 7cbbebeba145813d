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


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_launch_shapes_give_the_same_bits(prec):
    """Race hazards at tile boundaries: the hot path from the same state under every
    block height of the tunable kernels (32 x 4, 32 x 2, 32 x 1) gives bit-identical
    fields, two steps each (a leapfrog step and a graph replay)."""
    names = ("TSA", "UN", "VN", "UA", "VA", "SSHA", "UA_B", "VA_B", "UN_ADV", "VN_ADV", "AH_WSLP2")
    res = {}
    for h in (4, 2, 1):
        p = Pair(nn=2, prec=prec, seed=29, nmem=2)
        p.bind_hotpath()
        p.ctx.set_launch_shape({k: h for k in TUNABLE})
        assert all(v == h for k, v in p.ctx.launch_shape().items() if k in TUNABLE)
        for kt in (5, 6):
            p.ctx.stp_hotpath(kt)
        p.ctx.synchronize()
        res[h] = {n: p.dev[n].detach().cpu().clone() for n in names}
    for h in (2, 1):
        for n in names:
            assert torch.equal(res[4][n], res[h][n]), f"{n}: block height {h} differs from 4"


def test_launch_shape_rejects_untunable_heights():
    from nemo_gpu.api import NemoError
    p = Pair(nn=1, prec="mixed", seed=1)
    with pytest.raises(NemoError):
        p.ctx.set_launch_shape({"spg_p2": 2})
    with pytest.raises(NemoError):
        p.ctx.set_launch_shape({"fct_a": 3})
