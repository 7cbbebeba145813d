"""GPU run control (stp_ctl) and conservation budgets (dia_hsb) through the C ABI
against the oracle: the extrema of each member, the blow-up test on values injected
on the host (NEMO_ERR_BLOWUP at the next synchronize, the positions of the offending
values, and a usable context afterwards), and the budget terms of forced model steps
including ten model days. No GPU fault is involved: the failures are values."""
import numpy as np
import pytest

from harness import Pair
from nemo_gpu import gyre

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SBC_FIELDS = ("QNS", "QSR", "SFX", "SBC_TSC", "SBC_TSC_B", "QSR_HC", "QSR_HC_B", "FRAQSR_1LEV", "GDEPW_N")


@pytest.fixture(autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def forced_pair(prec, nn=2, nmem=2, seed=41):
    p = Pair(nn=nn, prec=prec, seed=seed, nmem=nmem, neuler=0)
    for m, st in enumerate(p.states):
        st.update(gyre.sbc_inputs(p.dom, p.nam, st, kt=1 + m))
    p.bind_hotpath()
    for name in SBC_FIELDS:
        p.bind(name)
    return p


def put(p, name, shape):
    """upload the oracles' (host) copies of field NAME to the GPU"""
    torch.cuda.synchronize()   # after the context's work (its own stream)
    p.dev[name].copy_(p.to_dev([p.host[m][name] for m in range(p.nmem)], fp64=p.dev[name].dtype == torch.float64))
    torch.cuda.synchronize()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_stp_ctl(prec):
    p = forced_pair(prec)
    p.ctx.stp_ctl(5)
    p.ctx.synchronize()
    z, loc, kindic = p.ctx.stp_ctl_result()
    for m, o in enumerate(p.ora):
        rz, rloc, rk = o.stp_ctl(5)
        if prec == "fp64":
            np.testing.assert_array_equal(z[m], rz)
        else:
            np.testing.assert_allclose(z[m], rz, rtol=1e-6)
        assert kindic[m] == rk == 0 and not loc[m].any()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_stp_ctl_blowup_is_reported(prec):
    """Member 0 gets a negative salinity at a wet point, member 1 a NaN velocity:
    both fire, with the oracle's positions; once the values are repaired the same
    context checks clean."""
    from nemo_gpu.api import NemoError
    p = forced_pair(prec)
    i, j, k = 7, 9, 3
    assert p.dom["k_bot"][i, j] > k
    p.host[0]["TSN"][i, j, k, 1] = -1.0
    p.host[1]["UN"][5, 6, 2] = np.nan
    put(p, "TSN", p.s4)
    put(p, "UN", p.s3)
    p.ctx.stp_ctl(5)
    with pytest.raises(NemoError, match="status 8"):
        p.ctx.synchronize()
    z, loc, kindic = p.ctx.stp_ctl_result()
    assert list(kindic) == [-3, -3]
    for m, o in enumerate(p.ora):
        rz, rloc, rk = o.stp_ctl(5)
        assert rk == -3
        if prec == "fp64":  # FP32 rounding may reorder near-equal extrema elsewhere
            np.testing.assert_array_equal(loc[m], rloc)
    assert tuple(loc[0][5:8]) == (i + 1, j + 1, k + 1) and tuple(loc[1][2:5]) == (6, 7, 3)
    assert np.isnan(z[1][1])
    p.host[0]["TSN"][i, j, k, 1] = 35.0
    p.host[1]["UN"][5, 6, 2] = 0.0
    put(p, "TSN", p.s4)
    put(p, "UN", p.s3)
    p.ctx.stp_ctl(6)
    p.ctx.synchronize()
    assert not p.ctx.stp_ctl_result()[2].any()


def hsb_close(got, ref, prec):
    """budget terms agree to a fraction of the content they are differences of"""
    vol = ref[13]
    scale = np.array([vol * 1e-3, 40 * vol, 40 * vol, 40 * vol, 40 * vol, vol * 1e-3, vol, 40 * vol, 40 * vol,
                      40 * vol, 40 * vol, 40 * vol, 40 * vol, vol, ref[14], 1.0])
    tol = 1e-14 if prec == "fp64" else 1e-6
    bad = np.abs(got - ref) > tol * scale
    assert not bad.any(), (np.nonzero(bad), got[bad], ref[bad])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_dia_hsb_model_steps(prec):
    """dia_hsb of the model step (step.F90:282) over four forced steps from an Euler
    start, two members, against the oracle's after every step."""
    p = forced_pair(prec)
    p.ctx.dia_hsb_init()
    for o in p.ora:
        o.dia_hsb_init()
    for kt in (1, 2, 3, 4):
        for o in p.ora:
            o.stp_model(kt)
        p.ctx.stp_model(kt)
        got = p.ctx.dia_hsb_result()
        for m, o in enumerate(p.ora):
            hsb_close(got[m], o.dia_hsb_last(), prec)
    p.ctx.synchronize()


def test_gpu_ten_day_budgets():
    """120 forced model steps (ten days) of GYRE nn_GYRE=1 in FP64: the budget terms
    against the oracle's, and the budgets close: after the Euler step the heat drift
    moves by less than 1e-3 of the heat forcing and the volume drift stays at rounding
    level; stp_ctl stays quiet."""
    p = forced_pair("fp64", nn=1, nmem=1, seed=43)
    p.ctx.dia_hsb_init()
    p.ora[0].dia_hsb_init()
    first = None
    for kt in range(1, 121):
        p.ora[0].stp_model(kt)
        p.ctx.stp_model(kt)
        if kt == 1:
            first = p.ctx.dia_hsb_result()[0]
    p.ctx.synchronize()
    h = p.ctx.dia_hsb_result()[0]
    hsb_close(h, p.ora[0].dia_hsb_last(), "fp64")
    assert abs(h[7] - first[7]) <= 1e-3 * abs(h[1])
    assert abs(h[5]) <= 1e-12 * h[13]
    z, loc, kindic = p.ctx.stp_ctl_result()
    assert kindic[0] == 0
    np.testing.assert_array_equal(z[0], p.ora[0].stp_ctl_last()[0])
