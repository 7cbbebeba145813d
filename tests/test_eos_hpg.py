"""The equations of state (eos_insitu, eos_insitu_pot, rab_3d: the simplified one
and the polynomial EOS-80), bn2 and hpg_zco: known answers of the oracle on the CPU
(including the reference's EOS-80 check value, eosbn2.F90:208), and the GPU through
the C ABI against the oracle, routine by routine and inside the model step."""
import numpy as np
import pytest

from nemo_gpu import gyre
from harness import Pair, relerr

LINEAR = dict(rn_lambda1=0.0, rn_lambda2=0.0, rn_mu1=0.0, rn_mu2=0.0, rn_nu=0.0)


def oracle_case(nn=1, **over):
    from oracle import ora
    dom = gyre.domain(nn)
    nam = gyre.namelist(ln_seos=1, **over)
    st = gyre.state(dom, nam, seed=9)
    sl = gyre.slope_inputs(dom, nam, st)
    o = ora.Oracle(dom, nam)
    gdept = np.array(sl["gdept_n"], order="F")
    gdepw = np.array(sl["gdepw_n"], order="F")
    o.bind("GDEPT_N", gdept)
    o.bind("GDEPW_N", gdepw)
    return dom, nam, st, o, gdept, gdepw


def test_eos_reference_state_and_linear_case():
    dom, nam, st, o, gdept, _ = oracle_case()
    tm = gyre.masks(dom)[0]
    ts = np.zeros(st["tsn"].shape, order="F")
    ts[..., 0], ts[..., 1] = 10.0, 35.0
    prd, rhop = np.ones(tm.shape, order="F"), np.ones(tm.shape, order="F")
    o.eos_insitu_pot(ts, prd, rhop, gdept)
    assert np.all(prd[:, :, :-1] == 0.0)
    assert np.all(rhop[:, :, :-1] == gyre.RAU0 * tm[:, :, :-1])
    assert np.all(prd[:, :, -1] == 1.0)                       # level jpk is not written
    dom, nam, st, o, gdept, _ = oracle_case(**LINEAR)
    ts = np.asfortranarray(st["tsn"])
    o.eos_insitu(ts, prd, gdept)
    want = (-nam["rn_a0"] * (ts[..., 0] - 10.0) + nam["rn_b0"] * (ts[..., 1] - 35.0)) / gyre.RAU0 * tm
    assert relerr(want[:, :, :-1], prd[:, :, :-1]) < 1e-14
    pab = np.zeros(ts.shape, order="F")
    o.rab_3d(ts, pab)
    assert np.allclose(pab[:, :, :-1, 0], nam["rn_a0"] / gyre.RAU0 * tm[:, :, :-1], rtol=1e-15, atol=0)
    assert np.allclose(pab[:, :, :-1, 1], nam["rn_b0"] / gyre.RAU0 * tm[:, :, :-1], rtol=1e-15, atol=0)


def test_bn2_of_a_linear_eos():
    """With constant expansion ratios N^2 = g (alpha dT - beta dS) / e3w between levels."""
    dom, nam, st, o, gdept, _ = oracle_case(**LINEAR)
    ts = np.asfortranarray(st["tsn"])
    pab = np.zeros(ts.shape, order="F")
    o.rab_3d(ts, pab)
    pn2 = np.zeros(ts.shape[:3], order="F")
    o.bn2(ts, pab, pn2)
    wm = gyre.masks(dom)[3]
    al, be = nam["rn_a0"] / gyre.RAU0, nam["rn_b0"] / gyre.RAU0
    dt = ts[:, :, :-1, 0] - ts[:, :, 1:, 0]
    ds = ts[:, :, :-1, 1] - ts[:, :, 1:, 1]
    want = nam["grav"] * (al * dt - be * ds) / dom["e3w_0"][:, :, 1:] * wm[:, :, 1:]
    tm = gyre.masks(dom)[0]
    both = (tm[:, :, :-1] * tm[:, :, 1:])[:, :, :-1] > 0       # levels 2..jpk-1 between wet T-points
    assert relerr(want[:, :, :-1][both], pn2[:, :, 1:-1][both]) < 1e-13
    assert np.all(pn2[:, :, 0] == 0) and np.all(pn2[:, :, -1] == 0)


def test_hpg_zco_known_answers():
    """A horizontally uniform density gives no trend; a density growing linearly in i
    gives, at the surface level, -g/2 e3w(1) d(rhd) / e1u, and below, the sum over the
    levels above of the same with the level pair's two densities."""
    from oracle import ora
    dom = gyre.domain(1)
    nam = gyre.namelist(ln_seos=1)
    o = ora.Oracle(dom, nam)
    s3 = (dom["jpi"], dom["jpj"], dom["jpk"])
    rhd = np.asfortranarray(np.broadcast_to(np.linspace(0, 1e-3, s3[2]), s3).copy())
    ua, va = np.zeros(s3, order="F"), np.zeros(s3, order="F")
    for name, a in (("RHD", rhd), ("UA", ua), ("VA", va)):
        o.bind(name, a)
    o.dyn_hpg(1)
    assert np.all(ua == 0) and np.all(va == 0)
    rhd[...] = (1e-5 * np.arange(s3[0]))[:, None, None]
    o.dyn_hpg(1)
    e1u = dom["e1u"]
    e3w = dom["e3w_0"]
    want1 = -nam["grav"] * 0.5 * e3w[:, :, 0] * 1e-5 / e1u
    assert np.allclose(ua[1:-1, 1:-1, 0], want1[1:-1, 1:-1], rtol=1e-13, atol=0)
    want = np.cumsum(-nam["grav"] * 0.5 * e3w * np.where(np.arange(s3[2]) == 0, 1e-5, 2e-5) / e1u[:, :, None], axis=2)
    assert np.allclose(ua[1:-1, 1:-1, :-1], want[1:-1, 1:-1, :-1], rtol=1e-12, atol=0)
    assert np.all(va == 0) and np.all(ua[:, :, -1] == 0)


def eos80_case(nn=1):
    from oracle import ora
    dom = gyre.domain(nn)
    nam = gyre.namelist(ln_eos80=1)
    return dom, nam, ora.Oracle(dom, nam)


def test_eos80_check_value():
    """eosbn2.F90:208: rho = 1028.35011066567 kg/m3 at 3000 m, pt = 3 degC, sp = 35.5 psu."""
    dom, nam, o = eos80_case()
    s3 = (dom["jpi"], dom["jpj"], dom["jpk"])
    ts = np.zeros(s3 + (2,), order="F")
    ts[..., 0], ts[..., 1] = 3.0, 35.5
    dep = np.full(s3, 3000.0, order="F")
    prd, rhop = np.zeros(s3, order="F"), np.zeros(s3, order="F")
    o.eos_insitu(ts, prd, dep)
    tm = gyre.masks(dom)[0]
    rho = (prd[:, :, :-1][tm[:, :, :-1] > 0] + 1.0) * nam["rau0"]
    assert np.allclose(rho, 1028.35011066567, rtol=0, atol=1e-10)
    o.eos_insitu_pot(ts, prd, rhop, dep)
    assert np.allclose((prd[:, :, :-1][tm[:, :, :-1] > 0] + 1.0) * nam["rau0"], 1028.35011066567, rtol=0, atol=1e-10)


def test_eos80_expansion_coefficients_are_the_derivatives():
    """rab_3d's alpha and beta tables against central differences of the density
    polynomial: alpha = -1/rau0 drho/dT, beta = 1/rau0 drho/dS (eosbn2.F90:588-642)."""
    dom, nam, o = eos80_case()
    s3 = (dom["jpi"], dom["jpj"], dom["jpk"])
    rng = np.random.default_rng(3)
    ts = np.zeros(s3 + (2,), order="F")
    ts[..., 0] = rng.uniform(-1.5, 28.0, s3)
    ts[..., 1] = rng.uniform(33.0, 37.5, s3)
    dep = np.asfortranarray(rng.uniform(0.0, 4000.0, s3))
    o.bind("GDEPT_N", dep)
    pab = np.zeros(s3 + (2,), order="F")
    o.rab_3d(ts, pab)
    h = 1e-3
    rho = {}
    for key, (n, d) in {"t+": (0, h), "t-": (0, -h), "s+": (1, h), "s-": (1, -h)}.items():
        t2 = ts.copy(order="F")
        t2[..., n] += d
        prd = np.zeros(s3, order="F")
        o.eos_insitu(t2, prd, dep)
        rho[key] = prd
    tm = gyre.masks(dom)[0][:, :, :-1] > 0
    alpha = -(rho["t+"] - rho["t-"]) / (2 * h)
    beta = (rho["s+"] - rho["s-"]) / (2 * h)
    assert np.allclose(pab[:, :, :-1, 0][tm], alpha[:, :, :-1][tm], rtol=2e-6, atol=0)
    assert np.allclose(pab[:, :, :-1, 1][tm], beta[:, :, :-1][tm], rtol=2e-6, atol=0)


def test_eos_needs_the_simplified_eos():
    from oracle import ora
    dom = gyre.domain(1)
    o = ora.Oracle(dom, gyre.namelist(ln_seos=0))
    a = np.zeros((dom["jpi"], dom["jpj"], dom["jpk"], 2), order="F")
    with pytest.raises(RuntimeError):
        o.eos_insitu(a, a[..., 0].copy(order="F"), a[..., 0].copy(order="F"))


# ------------------------------------------------------------------------- GPU
EOS = {"seos": dict(ln_seos=1), "eos80": dict(ln_eos80=1)}


def eos_pair(prec, nmem=2, eos="seos", **over):
    pytest.importorskip("torch")
    p = Pair(nn=2, prec=prec, seed=43, nmem=nmem, **EOS[eos], **over)
    for st in p.states:
        sl = gyre.slope_inputs(p.dom, p.nam, st)
        st.update(gdept_n=sl["gdept_n"], gdepw_n=sl["gdepw_n"], rhd=np.zeros(p.s3), rhop=np.zeros(p.s3))
    p.bind_hotpath()
    for name in ("GDEPT_N", "GDEPW_N"):
        p.bind(name)
    return p


@pytest.mark.gpu
@pytest.mark.parametrize("eos", ["seos", "eos80"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_eos_bn2_hpg(prec, eos):
    p = eos_pair(prec, eos=eos)
    nm = p.nmem
    z3 = [np.zeros(p.s3, order="F") for _ in range(nm)]
    z4 = [np.zeros(p.s4, order="F") for _ in range(nm)]
    host = {k: [a.copy(order="F") for a in (z4 if k == "pab" else z3)] for k in ("prd", "rhop", "pab", "pn2", "prd0")}
    dev = {k: p.to_dev(v) for k, v in host.items()}
    for m, o in enumerate(p.ora):
        ts, gt = p.host[m]["TSN"], p.host[m]["GDEPT_N"]
        o.eos_insitu(ts, host["prd0"][m], gt)
        o.eos_insitu_pot(ts, host["prd"][m], host["rhop"][m], gt)
        o.rab_3d(ts, host["pab"][m])
        o.bn2(ts, host["pab"][m], host["pn2"][m])
        o.bind("RHD", host["prd"][m])
        o.dyn_hpg(3)
    c = p.ctx
    c.eos_insitu(p.dev["TSN"], dev["prd0"], p.dev["GDEPT_N"])
    c.eos_insitu_pot(p.dev["TSN"], dev["prd"], dev["rhop"], p.dev["GDEPT_N"])
    c.rab_3d(p.dev["TSN"], dev["pab"])
    c.bn2(p.dev["TSN"], dev["pab"], dev["pn2"])
    c.bind("RHD", dev["prd"])
    c.dyn_hpg(3)
    c.synchronize()
    tol = {"fp64": dict(prd=1e-12, rhop=1e-12, pab=1e-12, pn2=1e-12, u=1e-12),
           "mixed": dict(prd=2e-5, rhop=1e-6, pab=1e-6, pn2=5e-4, u=5e-5)}[prec]
    for k in ("prd0", "prd", "rhop", "pab", "pn2"):
        got = p.per_member(dev[k], p.s4 if k == "pab" else p.s3)
        for m in range(nm):
            e = relerr(host[k][m], got[m])
            assert e <= tol[k.rstrip("0")], (k, m, e)
    p.compare("UA", p.s3, tol["u"])
    p.compare("VA", p.s3, tol["u"])


@pytest.mark.gpu
@pytest.mark.parametrize("eos", ["seos", "eos80"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_stp_model_with_hpg(prec, eos):
    """The model step with eos and dyn_hpg: steps 1 (Euler), 2, 3 (graph capture) and
    4 (replay)."""
    p = eos_pair(prec, eos=eos, neuler=0)
    for name in ("RHD", "RHOP"):
        p.bind(name)
    for kt in (1, 2, 3, 4):
        for o in p.ora:
            o.stp_model(kt)
        p.ctx.stp_model(kt)
    p.ctx.synchronize()
    tt = 1e-12 if prec == "fp64" else 2e-5
    tu = 1e-12 if prec == "fp64" else 2e-3
    p.compare("TSN", p.s4, tt)
    for name in ("UN", "VN", "UB", "VB"):
        p.compare(name, p.s3, tu)
    p.compare("RHD", p.s3, 1e-12 if prec == "fp64" else 2e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("eos", ["seos", "eos80"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_stp_model_with_slopes_from_the_tracers(prec, eos):
    """The model step forming its iso-neutral slopes from the before tracers
    (rab_3d, bn2, zdf_mxl, eos_insitu, ldf_slp) before the path, with eos and dyn_hpg
    of the now tracers: steps 1 (Euler), 2, 3 (graph capture) and 4 (replay)."""
    torch = pytest.importorskip("torch")
    p = eos_pair(prec, eos=eos, neuler=0)
    for st in p.states:
        st.update(rn2b=np.zeros(p.s3), hmlp=np.zeros(p.s2), hmlpt=np.zeros(p.s2))
    for name in ("RHD", "RHOP", "RN2B", "HMLP", "HMLPT"):
        p.bind(name)
    nm = [np.zeros(p.s2, dtype=np.int32, order="F") for _ in range(p.nmem)]
    for m, o in enumerate(p.ora):
        o.bind("NMLN", nm[m])
    p.ctx.bind("NMLN", torch.zeros(p.nmem * nm[0].size, dtype=torch.int32, device="cuda"))
    for kt in (1, 2, 3, 4):
        for o in p.ora:
            o.stp_model(kt)
        p.ctx.stp_model(kt)
    p.ctx.synchronize()
    if prec == "fp64":
        got = p.ctx.bound["NMLN"].cpu().numpy()
        assert np.array_equal(got, np.concatenate([a.ravel(order="F") for a in nm]))
        for name in ("USLP", "VSLP", "WSLPI", "WSLPJ", "RN2B"):
            p.compare(name, p.s3, 1e-12)
        p.compare("TSN", p.s4, 1e-12)
    else:
        # The slopes divide the horizontal density gradient by N^2 from FP32 tracer
        # differences: where the water is nearly unstratified they are ill-conditioned
        # (the FP64 form above matches the oracle to 1e-12), so the mixed form is held
        # to the tracers it produces and to agreement of the slopes at almost all points.
        p.compare("TSN", p.s4, 1e-4)
        for name in ("USLP", "VSLP", "WSLPI", "WSLPJ"):
            got = p.per_member(p.dev[name], p.s3)
            for m in range(p.nmem):
                ref = p.host[m][name]
                off = np.abs(got[m] - ref) > 1e-3 * np.abs(ref).max()
                assert off.mean() < 0.01, (name, m, off.mean())
