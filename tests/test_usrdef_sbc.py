"""GYRE's analytic surface forcing formed every model step: usrdef_sbc_oce
(usrdef_sbc.F90:62-190) with sbc's swap of the before fields (sbcmod.F90:389-394).

On the CPU: the shared FP64 sine and cosine (nemo_sin.h) against the host's; the
oracle against an independent numpy restatement of the reference's formulas at
several time steps of the seasonal cycle; E-P has zero domain mean; the restoring
heat flux responds to the SST; the before fields are swapped. On the GPU:
nemo_gpu_usrdef_sbc through the C ABI against the oracle, FP64 and mixed, two
members, at the first step and a later one."""
import math

import numpy as np
import pytest

from harness import Pair
from nemo_gpu import gyre

OUT2 = ("QSR", "QNS", "EMP", "SFX", "UTAU", "VTAU", "TAUM")


def test_shared_sin_cos_within_two_ulps_of_the_host():
    from oracle import ora
    L = ora.lib()
    x = np.concatenate([np.linspace(-2000.0, 2000.0, 40001), np.random.default_rng(5).uniform(-1e5, 1e5, 20000),
                        [0.0, np.pi / 4, np.pi / 2, np.pi, 1e-300]])
    for f, ref in ((L.ora_sin, np.sin), (L.ora_cos, np.cos)):
        got = np.array([f(float(v)) for v in x])
        want = ref(x)
        ulp = np.abs(got - want) / np.spacing(np.maximum(np.abs(want), 1e-300))
        assert ulp.max() <= 2.0, (f.__name__, ulp.max(), x[ulp.argmax()])


def usrdef_numpy(dom, nam, tsb1, tsn1, kt, tmask_i):
    """usrdef_sbc.F90:90-186 in numpy (the library's own sine and cosine)"""
    rpi = math.pi
    ztime = kt * nam["rn_rdt"] / 3600.0
    tmax1 = (5 * 30 + 21) * 24.0
    tmin1 = tmax1 + 24.0 * 360 / 2
    tmax2 = (6 * 30 + 21) * 24.0
    tmin2 = tmax2 - 24.0 * 360 / 2
    c1 = math.cos((ztime - tmax1) / (tmin1 - tmax1) * rpi)
    c2 = math.cos((ztime - tmax2) / (tmax2 - tmin2) * rpi)
    g = dom["gphit"]
    t_star = 28.3 * (1.0 + c2 / 50.0) * np.cos(rpi * (g - 5.0) / (53.5 * (1 + 11 / 53.5 * c2) * 2.0))
    qsr = 230.0 * np.cos(3.1415 * (g - 23.5 * c1) / (0.9 * 180))
    qns = -40.0 * (tsb1 - t_star) - qsr
    emp = np.where((g >= 14.845) & (g <= 37.2),
                   0.7 * 3.16e-5 * np.sin(rpi / 2 * (g - 37.2) / (24.6 - 37.2)) * (1 - 0.1 / 0.7 * c1),
                   -0.8 * 3.16e-5 * np.sin(rpi / 2 * (g - 37.2) / (46.8 - 37.2)) * (1 - 0.1 / 0.8 * c1))
    tm1 = (dom["k_bot"] > 0).astype(float)
    tm1[0], tm1[-1], tm1[:, 0], tm1[:, -1] = 0, 0, 0, 0
    zsum = (emp * tmask_i).sum() / (tm1 * tmask_i).sum()
    emp = emp - zsum * tm1
    qns = qns - emp * tsn1 * (nam.get("rcp") or 3991.86795711963)
    ztaun = 0.105 / math.sqrt(2.0) - 0.015 * math.cos((ztime - tmax1) / (tmin1 - tmax1) * rpi)
    utau = -ztaun * np.sin(rpi * (dom["gphiu"] - 15.0) / 14.0)
    vtau = ztaun * np.sin(rpi * (dom["gphiv"] - 15.0) / 14.0)
    taum = np.zeros_like(utau)
    ztx = utau[:-2, 1:-1] + utau[1:-1, 1:-1]
    zty = vtau[1:-1, :-2] + vtau[1:-1, 1:-1]
    taum[1:-1, 1:-1] = 0.5 * np.sqrt(ztx * ztx + zty * zty)
    return dict(QSR=qsr, QNS=qns, EMP=emp, SFX=np.zeros_like(qsr), UTAU=utau, VTAU=vtau, TAUM=taum)


def oracle_case(nn=1, seed=7):
    from oracle import ora
    dom = gyre.domain(nn)
    nam = gyre.namelist(ln_usr=1)
    st = gyre.state(dom, nam, seed=seed)
    o = ora.Oracle(dom, nam)
    f = {"TSB": np.array(st["tsb"], order="F"), "TSN": np.array(st["tsn"], order="F")}
    for n in ("GPHIT", "GPHIU", "GPHIV"):
        f[n] = np.array(dom[n.lower()], order="F", copy=True)
    for n in OUT2 + ("UTAU_B", "VTAU_B", "EMP_B"):
        f[n] = np.zeros((dom["jpi"], dom["jpj"]), order="F")
    for n, a in f.items():
        o.bind(n, a)
    return dom, nam, o, f


@pytest.mark.parametrize("kt", [1, 1500, 3000])
def test_oracle_matches_the_formulas(kt):
    dom, nam, o, f = oracle_case()
    o.usrdef_sbc(kt)
    want = usrdef_numpy(dom, nam, f["TSB"][:, :, 0, 0], f["TSN"][:, :, 0, 0], kt, o.array("tmask_i"))
    for n in OUT2:
        scale = max(np.abs(want[n]).max(), 1e-30)
        np.testing.assert_allclose(f[n], want[n], rtol=0, atol=1e-13 * scale, err_msg=n)


def test_forcing_properties_and_swap():
    dom, nam, o, f = oracle_case()
    tmi = o.array("tmask_i")
    o.usrdef_sbc(1)
    assert abs((f["EMP"] * tmi).sum()) <= 1e-15 * np.abs(f["EMP"]).sum()   # zero domain mean
    assert not f["TAUM"][0].any() and not f["TAUM"][:, 0].any() and (f["TAUM"][1:-1, 1:-1] > 0).all()
    assert not f["UTAU_B"].any()                       # no swap at nit000
    u1, q1 = f["UTAU"].copy(), f["QNS"].copy()
    f["TSB"][:, :, 0, 0] += 1.0                        # a warmer before SST: 40 W/m2 more loss
    o.usrdef_sbc(2)
    np.testing.assert_array_equal(f["UTAU_B"], u1)     # the before fields of step 2
    wet = tmi > 0
    d = (f["QNS"] - q1)[wet]
    assert np.all(np.abs(d + 40.0) < 1.0), (d.min(), d.max())


# ------------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_usrdef_sbc(prec):
    pytest.importorskip("torch")
    p = Pair(nn=2, prec=prec, seed=17, nmem=2, ln_usr=1)
    for st in p.states:
        for n in ("gphit", "gphiu", "gphiv"):
            st[n] = np.asfortranarray(p.dom[n])
        for n in ("qsr", "qns", "sfx", "taum", "utau_b", "vtau_b", "emp_b"):
            st[n] = np.zeros(p.s2, order="F")
    for n in ("TSB", "TSN", "GPHIT", "GPHIU", "GPHIV", "UTAU", "VTAU", "EMP") + ("QSR", "QNS", "SFX", "TAUM",
                                                                                 "UTAU_B", "VTAU_B", "EMP_B"):
        p.bind(n)
    tol = 1e-12 if prec == "fp64" else 2e-5
    for kt in (1, 2, 1500):
        for o in p.ora:
            o.usrdef_sbc(kt)
        p.ctx.usrdef_sbc(kt)
        p.ctx.synchronize()
        for n in OUT2 + ("UTAU_B", "EMP_B"):
            # E-P is a difference of values close to its mean: its FP32 error is
            # relative to the raw flux, about 2e-5 of the field's range
            p.compare(n, p.s2, tol if (prec == "fp64" or n != "EMP") else 1e-4)
