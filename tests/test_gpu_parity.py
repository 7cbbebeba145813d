"""GPU parity: every entry point of the C ABI against the oracle on the same seeded
inputs, through the ctypes binding of libnemo_gpu.so.

Tolerances (normwise relative error max|gpu - oracle| / max|oracle| per field):
* FP64 plain form: 1e-12, the bar of the reference's FP64 CPU build (the kernels
  are compiled without FMA contraction and keep the reference's operation order,
  so most fields match bit for bit; the fraction of identical values is reported);
* mixed precision (FP32 bulk): TOL32_TREND for tendencies (differences of FP32
  fluxes), TOL32_FIELD for after-tracers and velocities, TOL32_SPG for the
  barotropic fields integrated over the sub-steps.
"""
import numpy as np
import pytest

from harness import ACC_2D, Pair, relerr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32_TREND = 2e-4
TOL32_FIELD = 5e-6
TOL32_SPG = 2e-3
PRECS = ["fp64", "mixed"]


def tol(prec, kind):
    if prec == "fp64":
        return TOL64
    return {"trend": TOL32_TREND, "field": TOL32_FIELD, "spg": TOL32_SPG}[kind]


@pytest.fixture(autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("prec", PRECS)
def test_adv_trp(prec):
    p = Pair(nn=2, prec=prec, seed=1)
    st = p.states[0]
    zun, zvn, zwn = p.ora[0].tra_adv_trp(st["un"], st["vn"], st["wn"])
    u, v, w = (p.to_dev([st[n]]) for n in ("un", "vn", "wn"))
    out = [torch.empty_like(u) for _ in range(3)]
    p.ctx.tra_adv_trp(u, v, w, *out)
    p.ctx.synchronize()
    for ref, t in zip((zun, zvn, zwn), out):
        assert relerr(ref, p.ctx.to_host(t, p.s3)) <= tol(prec, "field")


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("kh,kv", [(2, 2), (4, 4), (2, 4), (4, 2)])
def test_tra_adv_fct(prec, kh, kv):
    p = Pair(nn=2, prec=prec, seed=2)
    st = p.states[0]
    zun, zvn, zwn = p.ora[0].tra_adv_trp(st["un"], st["vn"], st["wn"])
    ta = np.asfortranarray(1e-7 * np.random.default_rng(0).standard_normal(p.s4))
    ta_dev = p.to_dev([ta])
    p.ora[0].tra_adv_fct(5, 1, "TRA", 14400.0, zun, zvn, zwn, st["tsb"], st["tsn"], ta, 2, kh, kv)
    p.ctx.tra_adv_fct(5, 1, "TRA", 14400.0, p.to_dev([zun]), p.to_dev([zvn]), p.to_dev([zwn]),
                      p.to_dev([st["tsb"]]), p.to_dev([st["tsn"]]), ta_dev, 2, kh, kv)
    p.ctx.synchronize()
    assert relerr(ta, p.ctx.to_host(ta_dev, p.s4)) <= tol(prec, "trend")


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("kh,kv", [(2, 2), (4, 4)])
def test_tra_adv_fct_shelf(prec, kh, kv):
    """FCT over a bathymetry: interior columns with land below their bottom cell, where
    the limiter's masked extrema (+-zbig) are all the stencil holds; z* scale factors."""
    from nemo_gpu import shelf
    dom = shelf.domain(40, 36, 56, seed=5)
    nam = shelf.namelist()
    st = shelf.state(dom, nam, seed=6)
    p = Pair(prec=prec, dom=dom, nam=nam, states=[st])
    for n in ("E3T_B", "E3T_N", "E3T_A", "E3U_N", "E3V_N", "E3W_N"):
        p.bind(n)
    zun, zvn, zwn = p.ora[0].tra_adv_trp(st["un"], st["vn"], st["wn"])
    ta = np.zeros(p.s4, order="F")
    ta_dev = p.to_dev([ta])
    p.ora[0].tra_adv_fct(5, 1, "TRA", 600.0, zun, zvn, zwn, st["tsb"], st["tsn"], ta, 2, kh, kv)
    p.ctx.tra_adv_fct(5, 1, "TRA", 600.0, p.to_dev([zun]), p.to_dev([zvn]), p.to_dev([zwn]),
                      p.to_dev([st["tsb"]]), p.to_dev([st["tsn"]]), ta_dev, 2, kh, kv)
    p.ctx.synchronize()
    assert relerr(ta, p.ctx.to_host(ta_dev, p.s4)) <= tol(prec, "trend")


def test_tra_adv_fct_passive_tracers():
    """cdtype = TRC with kjpt = 3 (trcadv.F90:127 calls the same routine)."""
    p = Pair(nn=1, prec="fp64", seed=3)
    st = p.states[0]
    zun, zvn, zwn = p.ora[0].tra_adv_trp(st["un"], st["vn"], st["wn"])
    rng = np.random.default_rng(1)
    shape = p.s3 + (3,)
    tb = np.asfortranarray(np.abs(rng.standard_normal(shape)) * 5)
    tn = np.asfortranarray(tb + 0.01 * rng.standard_normal(shape))
    ta = np.zeros(shape, order="F")
    ta_dev = p.to_dev([ta])
    p.ora[0].tra_adv_fct(5, 1, "TRC", 14400.0, zun, zvn, zwn, tb, tn, ta, 3, 2, 2)
    p.ctx.tra_adv_fct(5, 1, "TRC", 14400.0, p.to_dev([zun]), p.to_dev([zvn]), p.to_dev([zwn]),
                      p.to_dev([tb]), p.to_dev([tn]), ta_dev, 3, 2, 2)
    p.ctx.synchronize()
    assert relerr(ta, p.ctx.to_host(ta_dev, shape)) <= TOL64


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("kpass", [1, 2])
def test_tra_ldf_lap(prec, kpass):
    p = Pair(nn=2, prec=prec, seed=4)
    st = p.states[0]
    ta = np.asfortranarray(1e-7 * np.random.default_rng(0).standard_normal(p.s4))
    ta_dev = p.to_dev([ta])
    p.ora[0].tra_ldf_lap(5, 1, "TRA", None, None, None, None, None, None, st["tsb"], ta, 2, kpass)
    p.ctx.tra_ldf_lap(5, 1, "TRA", None, None, None, None, None, None, p.to_dev([st["tsb"]]), ta_dev, 2, kpass)
    p.ctx.synchronize()
    assert relerr(ta, p.ctx.to_host(ta_dev, p.s4)) <= tol(prec, "trend")


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("msc", [0, 1])
def test_tra_ldf_iso(prec, msc):
    p = Pair(nn=2, prec=prec, seed=5, ln_traldf_msc=msc)
    st = p.states[0]
    p.bind_iso()
    ta = np.asfortranarray(1e-7 * np.random.default_rng(0).standard_normal(p.s4))
    ta_dev = p.to_dev([ta])
    # kt = kit000 exercises the zeroing of ah_wslp2 / akz
    p.ora[0].tra_ldf_iso(1, 1, "TRA", None, None, None, None, None, None, st["tsb"], st["tsb"], ta, 2, 1)
    tb = p.to_dev([st["tsb"]])
    p.ctx.tra_ldf_iso(1, 1, "TRA", None, None, None, None, None, None, tb, tb, ta_dev, 2, 1)
    p.ctx.synchronize()
    assert relerr(ta, p.ctx.to_host(ta_dev, p.s4)) <= tol(prec, "trend")
    p.compare("AH_WSLP2", p.s3, tol(prec, "field"))
    p.compare("AKZ", p.s3, tol(prec, "field"))


def test_tra_ldf_iso_bilaplacian_second_pass():
    """kpass = 2 with ln_traldf_blp (tra_ldf_blp, traldf_lap_blp.F90:226)."""
    p = Pair(nn=1, prec="fp64", seed=6, ln_traldf_lap=0, ln_traldf_blp=1, rn_aht_0=1.e11)
    st = p.states[0]
    p.bind_iso()
    zlap = np.zeros(p.s4, order="F")
    p.ora[0].tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, st["tsb"], st["tsb"], zlap, 2, 1)
    tb = p.to_dev([st["tsb"]])
    zlap_dev = p.to_dev([np.zeros(p.s4, order="F")])
    p.ctx.tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, tb, tb, zlap_dev, 2, 1)
    p.ctx.synchronize()
    assert relerr(zlap, p.ctx.to_host(zlap_dev, p.s4)) <= TOL64
    ta = np.zeros(p.s4, order="F")
    ta_dev = p.to_dev([ta])
    p.ora[0].tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, zlap, st["tsb"], ta, 2, 2)
    p.ctx.tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, zlap_dev, tb, ta_dev, 2, 2)
    p.ctx.synchronize()
    assert relerr(ta, p.ctx.to_host(ta_dev, p.s4)) <= TOL64


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("iso", [0, 1])
def test_tra_zdf_imp(prec, iso):
    p = Pair(nn=2, prec=prec, seed=7, ln_traldf_iso=iso)
    st = p.states[0]
    p.bind("AVT")
    if iso:
        p.bind_iso()
        scratch = np.zeros(p.s4, order="F")
        p.ora[0].tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, st["tsb"], st["tsb"], scratch, 2, 1)
        tb = p.to_dev([st["tsb"]])
        p.ctx.tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, tb, tb, p.to_dev([scratch * 0]), 2, 1)
    ta = np.asfortranarray(1e-6 * np.random.default_rng(0).standard_normal(p.s4))
    ta_dev = p.to_dev([ta])
    p.ora[0].tra_zdf_imp(5, 1, "TRA", 14400.0, st["tsb"], ta, 2)
    p.ctx.tra_zdf_imp(5, 1, "TRA", 14400.0, p.to_dev([st["tsb"]]), ta_dev, 2)
    p.ctx.synchronize()
    assert relerr(ta, p.ctx.to_host(ta_dev, p.s4)) <= tol(prec, "field")


def test_tra_zdf_salinity_clamp():
    """tra_zdf: after the solve, negative salinities become 0.1 (trazdf.F90:83)."""
    p = Pair(nn=1, prec="fp64", seed=8)
    st = p.states[0]
    st["tsb"][5:9, 5:9, :4, 1] = -2.0
    p.bind("AVT")
    p.bind_iso()
    p.bind("TSB", key="tsb")
    ta = np.zeros(p.s4, order="F")
    ta[10:12, 3:5, :, 1] = -3.0          # also on points the solve does not touch
    st["ta0"] = ta
    p.bind("TSA", key="ta0")
    p.ora[0].tra_zdf(5)
    p.ctx.tra_zdf(5)
    p.ctx.synchronize()
    p.compare("TSA", p.s4, TOL64)
    assert (p.host[0]["TSA"][..., 1] == 0.1).any()


SPG_CASES = [
    dict(),
    dict(nvor_scheme=0),
    dict(nvor_scheme=2),
    dict(nvor_scheme=3),
    dict(nvor_scheme=4, nn_een_e3f=1),
    dict(nvor_scheme=5),
    dict(nn_bt_flt=0),
    dict(nn_bt_flt=2),
    dict(ln_bt_fw=0),
    dict(ln_bt_av=0, rn_bt_alpha=0.1),
    dict(ln_apr_dyn=1),
]


def _spg_pair(prec, case, seed=9, nn=2, nmem=1):
    p = Pair(nn=nn, prec=prec, seed=seed, nmem=nmem, **case)
    for m in range(nmem):
        st = p.states[m]
        st["utau_b"], st["vtau_b"], st["emp_b"] = 0.9 * st["utau"], 0.9 * st["vtau"], 0.8 * st["emp"]
        st["ssh_ib"] = np.asfortranarray(0.05 * np.sin(np.arange(p.s2[0])[:, None] / 5.0) * np.ones(p.s2))
        st["ssh_ibb"] = np.asfortranarray(0.9 * st["ssh_ib"])
    p.bind_spg()
    for n in ("UTAU_B", "VTAU_B", "EMP_B", "SSH_IB", "SSH_IBB"):
        p.bind(n)
    return p


def _spg_compare(p, prec, report=None):
    t3, t2 = tol(prec, "spg"), tol(prec, "spg")
    for n in ("UA", "VA", "UN", "VN"):
        p.compare(n, p.s3, t3, report=report)
    for n in ACC_2D:
        p.compare(n, p.s2, t2, report=report)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", range(len(SPG_CASES)))
def test_dyn_spg_ts(prec, case):
    p = _spg_pair(prec, SPG_CASES[case])
    for kt in (5, 6):                       # two calls: the restart fields carry over
        for o in p.ora:
            o.dyn_spg_ts(kt)
        p.ctx.dyn_spg_ts(kt)
        p.ctx.synchronize()
    _spg_compare(p, prec)


# variable-volume free surface (ln_linssh = 0): vector- and flux-form momentum,
# forward and centred integration, every vorticity scheme
VVL_CASES = [
    dict(),
    dict(ln_dynadv_vec=0),
    dict(ln_dynadv_vec=0, ln_bt_fw=0),
    dict(ln_bt_fw=0, nvor_scheme=0),
    dict(nvor_scheme=2),
    dict(ln_dynadv_vec=0, nvor_scheme=2),
    dict(nvor_scheme=3),
    dict(ln_dynadv_vec=0, nvor_scheme=4, nn_een_e3f=1),
    dict(nvor_scheme=4),
    dict(nvor_scheme=5, ln_apr_dyn=1),
    dict(ln_dynadv_vec=0, ln_bt_av=0, rn_bt_alpha=0.1),
]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", range(len(VVL_CASES)))
def test_dyn_spg_ts_variable_volume(prec, case):
    p = _spg_pair(prec, dict(ln_linssh=0, **VVL_CASES[case]))
    for kt in (5, 6):
        for o in p.ora:
            o.dyn_spg_ts(kt)
        p.ctx.dyn_spg_ts(kt)
        p.ctx.synchronize()
    _spg_compare(p, prec)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("flux", [0, 1])
def test_stp_hotpath_variable_volume(prec, flux):
    """The full path with z* scale factors and depths, two members, from nit000."""
    p = Pair(nn=2, prec=prec, seed=15, neuler=0, nmem=2, ln_linssh=0, ln_dynadv_vec=1 - flux)
    p.bind_hotpath()
    for kt in (1, 2, 3):
        for o in p.ora:
            o.stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
        p.ctx.synchronize()
    p.compare("TSA", p.s4, tol(prec, "field"))
    p.compare("AH_WSLP2", p.s3, tol(prec, "field"))
    _spg_compare(p, prec)


@pytest.mark.parametrize("prec", PRECS)
def test_stp_hotpath_shelf(prec):
    """The shelf configuration at reduced horizontal size (56 levels): z* variable
    volume, partial bottom cells with their bottom gradients, FCT 4/4 through the
    compact vertical interpolation, iso-neutral diffusion, EEN vorticity, flux-form
    momentum and atmospheric pressure, nn_baro = 30, two members."""
    from nemo_gpu import shelf
    dom = shelf.domain(72, 56, 56, seed=3)
    nam = shelf.namelist(neuler=0)
    states = [shelf.state(dom, nam, seed=4, member=m) for m in range(2)]
    p = Pair(prec=prec, nmem=2, dom=dom, nam=nam, states=states)
    p.bind_hotpath()
    for n in ("GTSU", "GTSV", "SSH_IB"):
        p.bind(n)
    for kt in (1, 2, 3):
        for o in p.ora:
            o.stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
        p.ctx.synchronize()
    p.compare("TSA", p.s4, tol(prec, "field"))
    p.compare("AH_WSLP2", p.s3, tol(prec, "field"))
    _spg_compare(p, prec)


def test_variable_volume_requires_depths():
    p = Pair(nn=1, prec="fp64", seed=16, ln_linssh=0)
    p.bind_spg()
    p.ctx.bind("HU_N", None)
    with pytest.raises(RuntimeError):
        p.ctx.dyn_spg_ts(5)


@pytest.mark.parametrize("neuler", [0, 1])
def test_dyn_spg_ts_first_steps(neuler):
    """kt = nit000 (Euler start or restart), then nit000 + 1."""
    p = _spg_pair("fp64", dict(neuler=neuler))
    for kt in (1, 2, 3):
        for o in p.ora:
            o.dyn_spg_ts(kt)
        p.ctx.dyn_spg_ts(kt)
        p.ctx.synchronize()
    _spg_compare(p, "fp64")


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("nat", ["T", "U", "V", "W", "F"])
def test_lbc_lnk(prec, nat):
    p = Pair(nn=1, prec=prec, seed=10)
    rng = np.random.default_rng(2)
    a = np.asfortranarray(rng.standard_normal(p.s3))
    t = p.to_dev([a])
    p.ora[0].lbc_lnk(a, nat, pval=0.5)
    p.ctx.lbc_lnk(t, p.s3[2], nat, pval=0.5)
    p.ctx.synchronize()
    assert relerr(a, p.ctx.to_host(t, p.s3)) <= tol(prec, "field")


@pytest.mark.parametrize("prec", PRECS)
def test_glob_sum(prec):
    p = Pair(nn=2, prec=prec, seed=11)
    st = p.states[0]
    x = np.asfortranarray(st["tsb"][..., 0] * p.dom["e3t_0"] * 1e10)
    ref = p.ora[0].glob_sum(x)
    got = p.ctx.glob_sum(p.to_dev([x], fp64=True), p.s3[2])[0]
    assert abs(got - ref) <= 4 * np.spacing(abs(ref))
    if prec == "mixed":
        x32 = x.astype(np.float32).astype(np.float64)
        ref32 = p.ora[0].glob_sum(np.asfortranarray(x32))
        got32 = p.ctx.glob_sum(p.to_dev([x32]), p.s3[2])[0]
        assert abs(got32 - ref32) <= 4 * np.spacing(abs(ref32))


@pytest.mark.parametrize("prec", PRECS)
def test_stp_hotpath(prec):
    """Three timesteps of the full path (spg, adv, iso, zdf) from nit000, graph replay included."""
    p = Pair(nn=2, prec=prec, seed=12, neuler=0)
    p.bind_hotpath()
    for kt in (1, 2, 3, 4):
        for o in p.ora:
            o.stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
        p.ctx.synchronize()
    p.compare("TSA", p.s4, tol(prec, "field"))
    p.compare("AH_WSLP2", p.s3, tol(prec, "field"))
    _spg_compare(p, prec)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("jpk", [20, 46])
def test_stp_hotpath_other_level_counts(prec, jpk):
    """The hot path with jpk other than GYRE's 31: the general FP32 column kernels (the
    register ones are compiled for 31 levels) and level chunks that split unevenly."""
    p = Pair(nn=1, prec=prec, seed=14, jpk=jpk)
    p.bind_hotpath()
    for kt in (5, 6, 7):
        for o in p.ora:
            o.stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
        p.ctx.synchronize()
    p.compare("TSA", p.s4, tol(prec, "field"))
    p.compare("AH_WSLP2", p.s3, tol(prec, "field"))
    _spg_compare(p, prec)


@pytest.mark.parametrize("prec", PRECS)
def test_ensemble_members(prec):
    """Three members in one context, member index outermost; each against its own oracle."""
    p = Pair(nn=1, prec=prec, seed=13, nmem=3)
    p.bind_hotpath()
    for kt in (5, 6):
        for o in p.ora:
            o.stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
        p.ctx.synchronize()
    p.compare("TSA", p.s4, tol(prec, "field"))
    _spg_compare(p, prec)


def test_barrier_timeout_is_reported():
    """A grid barrier that can never complete gives NEMO_ERR_TIMEOUT, and the context stays usable."""
    from nemo_gpu.api import NemoError
    p = _spg_pair("fp64", {})
    p.ctx.set_barrier_limit(20000, extra_arrivals=1)
    p.ctx.dyn_spg_ts(5)
    with pytest.raises(NemoError, match="status 5"):
        p.ctx.synchronize()
    p.ctx.set_barrier_limit(4000000, 0)
    # a clean call afterwards still matches the oracle
    q = _spg_pair("fp64", {})
    q.ora[0].dyn_spg_ts(5)
    q.ctx.dyn_spg_ts(5)
    q.ctx.synchronize()
    _spg_compare(q, "fp64")
    p.ctx.dyn_spg_ts(6)
    p.ctx.synchronize()


@pytest.mark.parametrize("case", [dict(), dict(nvor_scheme=5), dict(ln_bt_fw=0), dict(nn_bt_flt=2)])
def test_spg_specialised_kernel(case):
    """The mixed form's specialised sub-step kernel (linear free surface, ENE/MIX)
    against the oracle and against the general kernel on the same inputs: both
    within the mixed tolerance of the oracle, and within FP32 rounding of each
    other (the constants are combined in another order, so they are not identical)."""
    res = {}
    for spec in (1, 0):
        p = _spg_pair("mixed", case, nn=5)
        p.ctx.set_spg_specialised(spec)
        for kt in (5, 6):
            for o in p.ora:
                o.dyn_spg_ts(kt)
            p.ctx.dyn_spg_ts(kt)
            p.ctx.synchronize()
        _spg_compare(p, "mixed")
        res[spec] = {n: np.asarray(p.ctx.to_host(p.dev[n], p.s2)) for n in ACC_2D}
        res[spec].update({n: np.asarray(p.ctx.to_host(p.dev[n], p.s3)) for n in ("UA", "VA", "UN", "VN")})
    for n in res[1]:
        assert relerr(res[0][n], res[1][n]) <= 2e-5, n
    assert any(not np.array_equal(res[0][n], res[1][n]) for n in res[1])  # two different kernels ran


def test_tma_wait_timeout_is_reported():
    """A TMA-staged tracer kernel whose waits on its tensor copies give up at once
    (poll limit 0) records the failure, drains its copies and returns:
    NEMO_ERR_TIMEOUT at the next synchronize, and the context stays usable."""
    from nemo_gpu.api import NemoError
    p = Pair(nn=3, prec="mixed", seed=23)
    p.bind_hotpath()
    p.ctx.set_tma_poll_limit(0)
    p.ctx.stp_hotpath(5)
    with pytest.raises(NemoError, match="tensor copy"):
        p.ctx.synchronize()
    p.ctx.set_tma_poll_limit(1 << 16)
    p.ctx.stp_hotpath(6)  # the context steps again without error
    p.ctx.synchronize()
    # and a clean step in this process still matches the oracle
    q = Pair(nn=3, prec="mixed", seed=23)
    q.bind_hotpath()
    q.ora[0].stp_hotpath(5)
    q.ctx.stp_hotpath(5)
    q.ctx.synchronize()
    q.compare("TSA", q.s4, TOL32_FIELD)


def test_gyre25_one_step_fp64():
    """One full hot-path step at the benchmark size (752 x 502 x 31) against the oracle."""
    p = Pair(nn=25, prec="fp64", seed=14)
    p.bind_hotpath()
    p.ora[0].stp_hotpath(5)
    p.ctx.stp_hotpath(5)
    p.ctx.synchronize()
    rep = {}
    p.compare("TSA", p.s4, TOL64, report=rep)
    _spg_compare(p, "fp64", report=rep)
    print({k: (f"{v[0]:.2e}", f"{v[1]:.4f}") for k, v in rep.items()})


@pytest.mark.parametrize("msc", [0, 1])
def test_fused_tracer_kernel_matches_per_routine_kernels(msc):
    """The fused FCT + iso-neutral kernel of the mixed form against the per-routine
    FP32 kernels and against the oracle, over three steps."""
    res = {}
    for fusion in (1, 0):
        p = Pair(nn=3, prec="mixed", seed=15, ln_traldf_msc=msc)
        p.ctx.set_fusion(fusion)
        p.bind_hotpath()
        for kt in (5, 6, 7):
            for o in p.ora:
                o.stp_hotpath(kt)
            p.ctx.stp_hotpath(kt)
            p.ctx.synchronize()
        p.compare("TSA", p.s4, TOL32_FIELD)
        p.compare("AH_WSLP2", p.s3, TOL32_FIELD)
        p.compare("AKZ", p.s3, TOL32_FIELD)
        res[fusion] = {n: p.ctx.to_host(p.dev[n], s) for n, s in (("TSA", p.s4), ("AH_WSLP2", p.s3), ("AKZ", p.s3))}
    for n in res[1]:
        assert relerr(res[0][n], res[1][n]) <= TOL32_FIELD, n


# kernel with TMA -> the kernels it replaces
TMA_KERNELS = {"iso_flux_tma": ("iso_flux",), "fct_a_tma": ("fct_a",), "fct_b_tma": ("fct_b",)}


@pytest.mark.parametrize("nmem", [1, 2])
def test_tma_kernels_match_plain_kernels(nmem):
    """The FP32 hot-path kernels with TMA-staged planes (jpi = 92, a multiple of 4)
    against the same kernels reading global memory: identical results (same
    arithmetic; the iso-neutral vertical term left out is exactly 0), and both against
    the oracle, over three steps with two level chunks per column."""
    res = {}
    for tma in (1, 0):
        p = Pair(nn=3, prec="mixed", seed=17, nmem=nmem)
        p.ctx.set_tma(tma)
        p.bind_hotpath()
        p.ctx.set_timing(True)  # per-kernel launch counts show which kernel ran
        for kt in (5, 6, 7):
            for o in p.ora:
                o.stp_hotpath(kt)
            p.ctx.stp_hotpath(kt)
            p.ctx.synchronize()
        ran = p.ctx.get_kernel_timing()
        for k, plain in TMA_KERNELS.items():
            assert (k in ran) == bool(tma), ran
            assert all((x in ran) != bool(tma) for x in plain), ran
        p.compare("TSA", p.s4, TOL32_FIELD)
        p.compare("AH_WSLP2", p.s3, TOL32_FIELD)
        p.compare("AKZ", p.s3, TOL32_FIELD)
        res[tma] = {n: p.ctx.to_host(p.dev[n], s) for n, s in (("TSA", p.s4), ("AH_WSLP2", p.s3), ("AKZ", p.s3))}
    for n in res[1]:
        a, b = np.asarray(res[0][n]), np.asarray(res[1][n])
        assert np.array_equal(a, b), f"{n}: TMA and plain kernels differ (max {np.abs(a - b).max():.3e})"


def test_fct_fused_kernel_matches_three_kernels():
    """The one-kernel FCT (intermediates in shared memory, halos recomputed) against
    the three-kernel FCT: identical results, and against the oracle, with jpk = 20
    (level chunks of the three-kernel form split unevenly) and two members."""
    res = {}
    for fused in (1, 0):
        p = Pair(nn=1, prec="mixed", seed=19, nmem=2, jpk=20)
        p.ctx.set_fct_fused(fused)
        p.bind_hotpath()
        p.ctx.set_timing(True)
        for kt in (5, 6, 7):
            for o in p.ora:
                o.stp_hotpath(kt)
            p.ctx.stp_hotpath(kt)
            p.ctx.synchronize()
        ran = p.ctx.get_kernel_timing()
        assert ("fct_fused" in ran) == bool(fused), ran
        p.compare("TSA", p.s4, TOL32_FIELD)
        res[fused] = p.ctx.to_host(p.dev["TSA"], p.s4)
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(np.asarray(a), np.asarray(b))
