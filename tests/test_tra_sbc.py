"""tra_sbc and tra_qsr (the surface forcing of the tracers): known answers of the
oracle on the CPU, and the GPU through the C ABI against the oracle, routine by
routine and inside the model step."""
import math

import numpy as np
import pytest

from nemo_gpu import gyre
from harness import Pair

R1_RAU0_RCP = 1.0 / (gyre.RAU0 * gyre.RCP)


def oracle_case(nn=1, **over):
    from oracle import ora
    dom = gyre.domain(nn)
    nam = gyre.namelist(**over)
    st = gyre.state(dom, nam, seed=5)
    st.update(gyre.sbc_inputs(dom, nam, st))
    o = ora.Oracle(dom, nam)
    arrs = {}
    for name, key in (("TSN", "tsn"), ("EMP", "emp"), ("QNS", "qns"), ("QSR", "qsr"), ("SFX", "sfx"),
                      ("SBC_TSC", "sbc_tsc"), ("SBC_TSC_B", "sbc_tsc_b"), ("QSR_HC", "qsr_hc"),
                      ("QSR_HC_B", "qsr_hc_b"), ("FRAQSR_1LEV", "fraqsr_1lev"), ("GDEPW_N", "gdepw_n")):
        arrs[name] = np.array(st[key], dtype=np.float64, order="F", copy=True)
        o.bind(name, arrs[name])
    arrs["TSA"] = np.zeros(st["tsn"].shape, order="F")
    o.bind("TSA", arrs["TSA"])
    return dom, nam, o, arrs


def test_nksr_is_the_extinction_level():
    """trc_oce_ext_lev for the two bands: the last level whose bottom lies above
    rn_si1 * (15 ln 10 + ln 100) in a flat-bottom basin."""
    dom, nam, o, _ = oracle_case(ln_traqsr=1)
    zhext = 23.0 * (math.log(10.0) * 15.0 + math.log(100.0))
    e3t = dom["e3t_0"][1, 1, :]
    gdepw = np.concatenate([[0.0], np.cumsum(e3t)])          # gdepw_0(1..jpk+1)
    jpk = dom["jpk"]
    want = jpk - 1
    for jk in range(jpk - 1, 0, -1):
        if gdepw[jk] >= zhext:                                # gdepw_0(jk+1), 1-based
            want = jk
    assert o.nksr() == want
    assert 1 <= want < jpk - 1


def test_tra_sbc_heat_flux_known_answer():
    """Uniform qns, no E-P and no salt flux: an Euler first step adds
    qns / (rau0 rcp e3t) to the first level of T on jj = 2..jpj, ji = 2..jpi-1, the
    next step the mean of the before and now trends."""
    dom, nam, o, a = oracle_case(neuler=0, ln_traqsr=1)
    a["QNS"][...] = 150.0
    a["EMP"][...] = 0.0
    o.tra_sbc(1)
    e3 = dom["e3t_0"][:, :, 0]
    want = 150.0 * R1_RAU0_RCP / e3
    got = a["TSA"][:, :, 0, 0]
    assert np.allclose(got[1:-1, 1:], want[1:-1, 1:], rtol=1e-14, atol=0)
    assert np.all(got[0, :] == 0) and np.all(got[-1, :] == 0) and np.all(got[:, 0] == 0)
    assert np.all(a["TSA"][:, :, 0, 1] == 0) and np.all(a["TSA"][:, :, 1:, :] == 0)
    assert np.all(a["SBC_TSC_B"] == 0)
    a["TSA"][...] = 0.0
    a["QNS"][...] = 50.0
    o.tra_sbc(2)
    want = 0.5 * (150.0 + 50.0) * R1_RAU0_RCP / e3
    assert np.allclose(a["TSA"][1:-1, 1:, 0, 0], want[1:-1, 1:], rtol=1e-14, atol=0)


def test_tra_sbc_moves_qsr_without_penetration():
    dom, nam, o, a = oracle_case(neuler=0, ln_traqsr=0)
    qsum = a["QNS"] + a["QSR"]
    o.tra_sbc(1)
    assert np.array_equal(a["QNS"], qsum)
    assert np.all(a["QSR"] == 0)


def test_tra_qsr_column_budget():
    """The absorbed heat of each wet interior column telescopes: levels 1..nksr take
    qsr (1 - zc(nksr+1)) / (rau0 rcp), zc the two-band attenuation at the bottom of
    level nksr; fraqsr_1lev is the first level's share, 0 on the edge."""
    dom, nam, o, a = oracle_case(neuler=0, ln_traqsr=1)
    o.tra_qsr(1)
    n = o.nksr()
    g = a["GDEPW_N"][:, :, n]                                 # 0-based level n = 1-based nksr+1
    zc = 0.58 * np.exp(-g / 0.35) + 0.42 * np.exp(-g / 23.0)
    tm = gyre.masks(dom)[0]
    inner = (slice(1, -1), slice(1, -1))
    wet = tm[:, :, n][inner] > 0
    col = a["QSR_HC"][:, :, :n].sum(axis=2)
    want = a["QSR"] * R1_RAU0_RCP * (1.0 - zc)
    assert np.allclose(col[inner][wet], want[inner][wet], rtol=1e-12, atol=1e-30)
    assert np.all(a["QSR_HC"][:, :, n:] == 0)
    zc1 = 0.58 * np.exp(-a["GDEPW_N"][:, :, 1] / 0.35) + 0.42 * np.exp(-a["GDEPW_N"][:, :, 1] / 23.0)
    assert np.allclose(a["FRAQSR_1LEV"][inner], (1.0 - zc1)[inner], rtol=1e-12)
    f = a["FRAQSR_1LEV"]
    assert np.all(f[0, :] == 0) and np.all(f[-1, :] == 0) and np.all(f[:, 0] == 0) and np.all(f[:, -1] == 0)
    t = a["TSA"][:, :, :n, 0]
    e3 = dom["e3t_0"][:, :, :n]
    assert np.allclose(t[inner], (a["QSR_HC"][:, :, :n] / e3)[inner], rtol=1e-14, atol=0)


# ------------------------------------------------------------------------- GPU
SBC_FIELDS = ("QNS", "QSR", "SFX", "SBC_TSC", "SBC_TSC_B", "QSR_HC", "QSR_HC_B", "FRAQSR_1LEV", "GDEPW_N")


def sbc_pair(prec, nmem=2, **over):
    pytest.importorskip("torch")
    p = Pair(nn=2, prec=prec, seed=41, nmem=nmem, **over)
    for m, st in enumerate(p.states):
        st.update(gyre.sbc_inputs(p.dom, p.nam, st, kt=1 + m))
    p.bind_hotpath()
    for name in SBC_FIELDS:
        p.bind(name)
    return p


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_tra_sbc_qsr(prec):
    """An Euler first step, then a swapping step, two members."""
    p = sbc_pair(prec, neuler=0)
    for kt in (1, 2):
        for o in p.ora:
            o.tra_sbc(kt)
            o.tra_qsr(kt)
        p.ctx.tra_sbc(kt)
        p.ctx.tra_qsr(kt)
    p.ctx.synchronize()
    t = 1e-12 if prec == "fp64" else 5e-6
    p.compare("TSA", p.s4, t)
    for name in ("QNS", "QSR", "FRAQSR_1LEV"):
        p.compare(name, p.s2, t)
    for name in ("SBC_TSC", "SBC_TSC_B"):
        p.compare(name, (p.s2[0], p.s2[1], 2), t)
    for name in ("QSR_HC", "QSR_HC_B"):
        p.compare(name, p.s3, t)


@pytest.mark.gpu
def test_gpu_tra_sbc_without_penetration():
    p = sbc_pair("fp64", nmem=1, neuler=0, ln_traqsr=0)
    for kt in (1, 2):
        p.ora[0].tra_sbc(kt)
        p.ctx.tra_sbc(kt)
    p.ctx.synchronize()
    for name in ("QNS", "QSR"):
        p.compare(name, p.s2, 0.0)
    p.compare("TSA", p.s4, 1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_stp_model_with_surface_forcing(prec):
    """The model step with tra_sbc and tra_qsr bound: steps 1 (Euler), 2, 3 (graph
    capture) and 4 (replay)."""
    p = sbc_pair(prec, neuler=0)
    for kt in (1, 2, 3, 4):
        for o in p.ora:
            o.stp_model(kt)
        p.ctx.stp_model(kt)
    p.ctx.synchronize()
    tt = 1e-12 if prec == "fp64" else 2e-5
    p.compare("TSN", p.s4, tt)
    p.compare("TSB", p.s4, tt)
    for name in ("QSR_HC", "QSR_HC_B"):
        p.compare(name, p.s3, 1e-12 if prec == "fp64" else 5e-6)
