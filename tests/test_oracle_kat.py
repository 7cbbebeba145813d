"""Known-answer tests that pin the oracle (the CPU FP64 restatement of the reference).

The reference ships no golden vectors or unit tests for these routines and cannot
be built here, so the oracle is pinned by analytic properties of the reference
algorithms (CPU only, no GPU):

* ts_wgt weights and sub-step count (dynspg_ts.F90:1313-1388, :1491);
* FCT advection of a constant tracer in a non-divergent flow leaves it unchanged,
  the limiter keeps the after field within the before field's range, and the
  domain-integrated trend equals the surface flux (traadv_fct.F90);
* laplacian / iso-neutral diffusion of a constant field is zero, and the
  iso-neutral operator with zero slopes equals the iso-level laplacian;
* the implicit vertical diffusion conserves each column's tracer content;
* the barotropic sub-stepping keeps a fluid at rest at rest and conserves volume;
* lbc_lnk closed-boundary values; glob_sum against an exact sum;
* no routine reads a point the reference leaves undefined (NaN poisoning).
"""
import math

import numpy as np
import pytest

from nemo_gpu import gyre
from oracle import ora


def make(nn=1, seed=3, **nam_over):
    dom = gyre.domain(nn)
    nam = gyre.namelist(**nam_over)
    st = gyre.state(dom, nam, seed=seed)
    return dom, nam, st, ora.Oracle(dom, nam)


def interior(a):
    return a[1:-1, 1:-1]


def test_ts_wgt_boxcar():
    dom, nam, st, o = make()
    icycle, nn_baro, rdtbt = o.spg_info()
    assert nn_baro == 25 and icycle == 37          # rdt=7200, e1=106 km, depth 4 km, cmax 0.8
    assert rdtbt == 7200.0 / 25
    w1, w2 = o.array("wgtbtp1"), o.array("wgtbtp2")
    nz = np.nonzero(w1)[0] + 1
    assert nz[0] == 13 and nz[-1] == 37            # |jn - nn_baro| / nn_baro < 0.5
    np.testing.assert_allclose(w1[12:37], 1.0 / 25, rtol=0, atol=1e-17)
    assert abs(w1.sum() - 1.0) < 1e-15 and abs(w2.sum() - 1.0) < 1e-15
    # secondary weights: cumulative sums of the primary ones from jn to icycle
    raw = np.array([max(0, min(37, 37) - max(jn, 13) + 1) for jn in range(1, 38)], dtype=float)
    np.testing.assert_allclose(w2[:37], raw / raw.sum(), rtol=1e-14)


@pytest.mark.parametrize("flt,expect", [(0, 25), (2, 49)])
def test_ts_wgt_other_filters(flt, expect):
    dom, nam, st, o = make(nn_bt_flt=flt)
    icycle, nn_baro, _ = o.spg_info()
    assert icycle == expect
    assert abs(o.array("wgtbtp1").sum() - 1.0) < 1e-15


def _nondivergent(dom, st):
    """Transports of the state's flow with the surface w from continuity."""
    return st["un"], st["vn"], st["wn"]


@pytest.mark.parametrize("kh,kv", [(2, 2), (4, 4)])
def test_fct_constant_tracer(kh, kv):
    dom, nam, st, o = make()
    tm, um, vm, wm = gyre.masks(dom)
    zun, zvn, zwn = o.tra_adv_trp(*_nondivergent(dom, st))
    tb = np.zeros(st["tsb"].shape, order="F")
    tb[..., 0] = 15.0 * tm
    tb[..., 1] = 35.0 * tm
    ta = np.zeros_like(tb, order="F")
    o.tra_adv_fct(5, 1, "TRA", 14400.0, zun, zvn, zwn, tb, tb.copy(order="F"), ta, 2, kh, kv)
    # a constant tracer in a flow that satisfies continuity has no trend
    scale = 35.0 * np.abs(st["un"]).max() / dom["e1t"][0, 0]
    assert np.abs(ta).max() < 1e-11 * scale


def test_fct_monotone_and_conservative():
    dom, nam, st, o = make(seed=11)
    tm = gyre.masks(dom)[0]
    zun, zvn, zwn = o.tra_adv_trp(st["un"], st["vn"], st["wn"])
    # a sharp front: the limiter must not create new extrema
    tb = np.zeros(st["tsb"].shape, order="F")
    ii = np.arange(dom["jpi"])[:, None, None]
    tb[..., 0] = np.where(ii < dom["jpi"] // 2, 20.0, 5.0) * tm
    tb[..., 1] = (35.0 + 0.5 * np.sin(ii / 3.0)) * tm
    ta = np.zeros_like(tb, order="F")
    p2dt = 14400.0
    o.tra_adv_fct(5, 1, "TRA", p2dt, zun, zvn, zwn, tb, tb.copy(order="F"), ta, 2, 2, 2)
    after = tb + p2dt * ta
    wet = np.broadcast_to(tm[..., None] > 0, tb.shape)
    for n in range(2):
        lo, hi = tb[..., n][wet[..., n]].min(), tb[..., n][wet[..., n]].max()
        a = after[..., n][wet[..., n]]
        assert a.min() >= lo - 1e-9 and a.max() <= hi + 1e-9
    # the domain integral of the trend is the surface (upstream) flux only
    e1e2t = dom["e1t"] * dom["e2t"]
    vol = e1e2t[:, :, None] * dom["e3t_0"]
    for n in range(2):
        total = math.fsum((vol * ta[..., n] * tm).ravel())
        surf = -math.fsum((zwn[:, :, 0] * tb[:, :, 0, n] * tm[:, :, 0])[1:-1, 1:-1].ravel())
        assert abs(total - surf) <= 1e-10 * max(1.0, abs(surf))


def test_diffusion_of_constant_is_zero():
    dom, nam, st, o = make()
    tm = gyre.masks(dom)[0]
    tb = np.zeros(st["tsb"].shape, order="F")
    tb[..., 0] = 12.0 * tm
    tb[..., 1] = 34.5 * tm
    for n in ("USLP", "VSLP", "WSLPI", "WSLPJ"):
        o.bind(n, st[n.lower()])
    ah = np.zeros(st["avt"].shape, order="F")
    akz = np.zeros_like(ah, order="F")
    o.bind("AH_WSLP2", ah)
    o.bind("AKZ", akz)
    ta = np.zeros_like(tb, order="F")
    o.tra_ldf_lap(5, 1, "TRA", None, None, None, None, None, None, tb, ta, 2, 1)
    assert np.abs(ta).max() == 0.0
    # land values are zero, so only the iso-neutral coupling across the coast can act
    o.tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, tb, tb, ta, 2, 1)
    assert np.abs(interior(ta)[:, :, 1:-1]).max() < 1e-18


def test_iso_with_zero_slopes_is_laplacian():
    dom, nam, st, o = make(seed=5)
    z = np.zeros(st["avt"].shape, order="F")
    for n in ("USLP", "VSLP", "WSLPI", "WSLPJ"):
        o.bind(n, z)
    ah = np.zeros_like(z, order="F")
    akz = np.zeros_like(z, order="F")
    o.bind("AH_WSLP2", ah)
    o.bind("AKZ", akz)
    ta_iso = np.zeros(st["tsb"].shape, order="F")
    ta_lap = np.zeros(st["tsb"].shape, order="F")
    o.tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, st["tsb"], st["tsb"], ta_iso, 2, 1)
    o.tra_ldf_lap(5, 1, "TRA", None, None, None, None, None, None, st["tsb"], ta_lap, 2, 1)
    np.testing.assert_allclose(ta_iso, ta_lap, rtol=0, atol=1e-13 * np.abs(ta_lap).max())
    assert np.abs(ah).max() == 0.0


def test_zdf_conserves_column_content():
    dom, nam, st, o = make(seed=7)
    tm = gyre.masks(dom)[0]
    o.bind("AVT", st["avt"])
    for n in ("USLP", "VSLP", "WSLPI", "WSLPJ"):
        o.bind(n, st[n.lower()])
    ah = np.zeros(st["avt"].shape, order="F")
    o.bind("AH_WSLP2", ah)
    o.bind("AKZ", np.zeros_like(ah, order="F"))
    o.tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, st["tsb"], st["tsb"],
                  np.zeros(st["tsb"].shape, order="F"), 2, 1)
    ta_in = 1e-6 * np.random.default_rng(0).standard_normal(st["tsb"].shape) * tm[..., None]
    ta = np.asfortranarray(ta_in)
    p2dt = 14400.0
    o.tra_zdf_imp(5, 1, "TRA", p2dt, st["tsb"], ta, 2)
    e3 = dom["e3t_0"]
    before = ((e3[..., None] * st["tsb"] + p2dt * e3[..., None] * ta_in) * tm[..., None]).sum(axis=2)
    after = (e3[..., None] * ta * tm[..., None]).sum(axis=2)
    np.testing.assert_allclose(interior(after), interior(before), rtol=1e-13)
    # diffusion smooths: the after column range lies within the forced column range
    assert np.isfinite(ta).all()


def _bind_spg(o, dom, st, zero_flow=False):
    keep = {}
    n2 = (dom["jpi"], dom["jpj"])
    for n in ("ua", "va", "un", "vn", "ub", "vb", "sshn", "sshb", "un_b", "vn_b", "ub_b", "vb_b", "utau", "vtau", "emp"):
        a = np.zeros_like(st[n], order="F") if zero_flow else st[n].copy(order="F")
        keep[n] = a
        o.bind(n.upper(), a)
    keep["rcdu"] = st["rcdu_bot"].copy(order="F")
    o.bind("RCDU_BOT", keep["rcdu"])
    for n in ("SSHA", "UA_B", "VA_B", "UN_ADV", "VN_ADV", "UB2_B", "VB2_B", "UN_BF", "VN_BF"):
        keep[n] = np.zeros(n2, order="F")
        o.bind(n, keep[n])
    return keep


def test_spg_rest_stays_at_rest():
    dom, nam, st, o = make()
    f = _bind_spg(o, dom, st, zero_flow=True)
    o.dyn_spg_ts(5)
    for n in ("SSHA", "UA_B", "VA_B", "UN_ADV", "VN_ADV"):
        assert np.abs(f[n]).max() == 0.0
    assert np.abs(f["ua"]).max() == 0.0 and np.abs(f["un"]).max() == 0.0


def test_spg_conserves_volume():
    dom, nam, st, o = make(seed=9)
    f = _bind_spg(o, dom, st)
    f["emp"][:] = 0.0
    o.dyn_spg_ts(5)
    e1e2t = dom["e1t"] * dom["e2t"]
    v0 = math.fsum((e1e2t * st["sshn"]).ravel())
    v1 = math.fsum((e1e2t * f["SSHA"]).ravel())
    assert abs(v1 - v0) <= 1e-12 * math.fsum(np.abs(e1e2t * st["sshn"]).ravel())
    assert np.abs(f["SSHA"]).max() > 0


ZSTAR_FIELDS = ("HT_N", "HU_N", "HV_N", "R1_HU_N", "R1_HV_N", "HU_B", "HV_B", "R1_HU_B", "R1_HV_B", "E3F_N",
                "E3T_B", "E3T_N", "E3T_A", "E3U_N", "E3V_N", "E3W_N")


def _bind_zstar(o, dom, st, keep):
    """Bind the z* scale factors and depths of the state (variable volume)."""
    z = gyre.zstar(dom, st)
    for n in ZSTAR_FIELDS:
        keep[n] = z[n.lower()]
        o.bind(n, keep[n])
    return keep


VVL_CASES = [dict(ln_dynadv_vec=1, ln_bt_fw=1), dict(ln_dynadv_vec=0, ln_bt_fw=1),
             dict(ln_dynadv_vec=0, ln_bt_fw=0, nvor_scheme=4), dict(ln_dynadv_vec=1, ln_bt_fw=1, nvor_scheme=2)]


@pytest.mark.parametrize("case", VVL_CASES, ids=["vec", "flux", "flux-centred-een", "vec-ent"])
def test_spg_vvl_rest_stays_at_rest(case):
    dom, nam, st, o = make(ln_linssh=0, **case)
    f = _bind_spg(o, dom, st, zero_flow=True)
    _bind_zstar(o, dom, {k: np.zeros_like(v) if k.startswith("ssh") else v for k, v in st.items()}, f)
    for n in ("UTAU_B", "VTAU_B", "EMP_B"):
        f[n] = np.zeros((dom["jpi"], dom["jpj"]), order="F")
        o.bind(n, f[n])
    o.dyn_spg_ts(5)
    for n in ("SSHA", "UA_B", "VA_B", "UN_ADV", "VN_ADV"):
        assert np.abs(f[n]).max() == 0.0, n
    assert np.abs(f["ua"]).max() == 0.0 and np.abs(f["un"]).max() == 0.0


@pytest.mark.parametrize("case", VVL_CASES, ids=["vec", "flux", "flux-centred-een", "vec-ent"])
def test_spg_vvl_conserves_volume(case):
    """The time-averaged ssh of the sub-steps keeps the volume of the now ssh when
    there is no surface water flux (flux-form divergence, closed basin)."""
    dom, nam, st, o = make(seed=9, ln_linssh=0, **case)
    f = _bind_spg(o, dom, st)
    _bind_zstar(o, dom, st, f)
    for n, k in (("UTAU_B", "utau"), ("VTAU_B", "vtau"), ("EMP_B", "emp")):
        f[n] = st[k].copy(order="F")
        o.bind(n, f[n])
    f["emp"][:] = 0.0
    f["EMP_B"][:] = 0.0
    o.dyn_spg_ts(5)
    e1e2t = dom["e1t"] * dom["e2t"]
    ssh0 = st["sshn"] if case["ln_bt_fw"] else st["sshb"]
    v0 = math.fsum((e1e2t * ssh0).ravel())
    v1 = math.fsum((e1e2t * f["SSHA"]).ravel())
    assert abs(v1 - v0) <= 1e-12 * math.fsum(np.abs(e1e2t * ssh0).ravel())
    assert np.abs(f["SSHA"]).max() > 0
    assert np.isfinite(f["ua"]).all() and np.isfinite(f["UA_B"]).all()


def test_spg_vvl_requires_depths():
    dom, nam, st, o = make(ln_linssh=0)
    _bind_spg(o, dom, st)
    with pytest.raises(RuntimeError):
        o.dyn_spg_ts(5)


def test_lbc_closed():
    dom, nam, st, o = make()
    a = np.asfortranarray(np.random.default_rng(1).standard_normal((dom["jpi"], dom["jpj"], 3)))
    b = a.copy(order="F")
    o.lbc_lnk(a, "T", pval=7.0)
    assert (a[0] == 7).all() and (a[-1] == 7).all() and (a[:, 0] == 7).all() and (a[:, -1] == 7).all()
    np.testing.assert_array_equal(a[1:-1, 1:-1], b[1:-1, 1:-1])
    c = b.copy(order="F")
    o.lbc_lnk(c, "F", pval=0.0)
    np.testing.assert_array_equal(c[0, 1:-1], b[0, 1:-1])   # F-points keep column 1
    np.testing.assert_array_equal(c[1:-1, 0], b[1:-1, 0])   # and row 1
    assert (c[-1] == 0).all() and (c[:, -1] == 0).all()


def test_glob_sum_is_compensated():
    dom, nam, st, o = make()
    rng = np.random.default_rng(4)
    x = np.asfortranarray(rng.standard_normal((dom["jpi"], dom["jpj"], dom["jpk"])) * 10.0 ** rng.integers(-8, 9, (dom["jpi"], dom["jpj"], dom["jpk"])))
    tmi = o.array("tmask_i")
    exact = math.fsum((x * tmi[:, :, None]).ravel())
    got = o.glob_sum(x)
    assert abs(got - exact) <= 2 * np.spacing(abs(exact))


def test_no_undefined_reads():
    """Every routine gives the same result when its automatic work arrays start as NaN."""
    def run(poison):
        ora.set_poison(poison)
        try:
            dom, nam, st, o = make(seed=13)
            out = {}
            zun, zvn, zwn = o.tra_adv_trp(st["un"], st["vn"], st["wn"])
            for kh, kv in ((2, 2), (4, 4)):
                ta = np.zeros(st["tsb"].shape, order="F")
                o.tra_adv_fct(5, 1, "TRA", 14400.0, zun, zvn, zwn, st["tsb"], st["tsn"], ta, 2, kh, kv)
                out[f"fct{kh}{kv}"] = ta
            for n in ("USLP", "VSLP", "WSLPI", "WSLPJ"):
                o.bind(n, st[n.lower()])
            ah = np.zeros(st["avt"].shape, order="F")
            akz = np.zeros_like(ah, order="F")
            o.bind("AH_WSLP2", ah)
            o.bind("AKZ", akz)
            o.bind("AVT", st["avt"])
            ta = np.zeros(st["tsb"].shape, order="F")
            o.tra_ldf_iso(5, 1, "TRA", None, None, None, None, None, None, st["tsb"], st["tsb"], ta, 2, 1)
            o.tra_ldf_lap(5, 1, "TRA", None, None, None, None, None, None, st["tsb"], ta, 2, 1)
            o.tra_zdf_imp(5, 1, "TRA", 14400.0, st["tsb"], ta, 2)
            out["tra"] = ta
            f = _bind_spg(o, dom, st)
            o.dyn_spg_ts(5)
            for n in ("SSHA", "UA_B", "UN_ADV", "ua", "un"):
                out[n] = f[n].copy()
            for vec in (1, 0):  # variable volume, vector and flux form
                dom, nam, st, o = make(seed=13, ln_linssh=0, ln_dynadv_vec=vec)
                f = _bind_spg(o, dom, st)
                _bind_zstar(o, dom, st, f)
                o.dyn_spg_ts(5)
                for n in ("SSHA", "UA_B", "UN_ADV", "ua", "un"):
                    out[f"vvl{vec}_{n}"] = f[n].copy()
            return out
        finally:
            ora.set_poison(0)
    a, b = run(0), run(1)
    for k in a:
        assert np.isfinite(b[k]).all(), k
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_shelf_domain_partial_cells():
    """The synthetic shelf: partial bottom cells no thicker than their level, u/v
    thicknesses the minima of their T-neighbours, column depths equal to the
    bathymetry within the partial-cell rule, and a finite oracle hot-path step."""
    from nemo_gpu import shelf
    dom = shelf.domain(28, 24, 56, seed=1)
    tm, um, vm, _ = gyre.masks(dom)
    e3t1 = dom["e3t_0"][0, 0, :]
    kb = dom["k_bot"]
    wet = kb > 0
    assert wet.sum() > 0.3 * wet.size
    ii, jj = np.nonzero(wet)
    ik = kb[ii, jj] - 1
    part = dom["e3t_0"][ii, jj, ik]
    assert (part > 0).all() and (part <= e3t1[ik] + 1e-12).all()
    e3t = dom["e3t_0"]
    np.testing.assert_array_equal(dom["e3u_0"][:-1, :-1], np.minimum(e3t[:-1, :-1], e3t[1:, :-1]))
    np.testing.assert_array_equal(dom["e3v_0"][:-1, :-1], np.minimum(e3t[:-1, :-1], e3t[:-1, 1:]))
    assert (np.diff(tm, axis=2) <= 0).all()          # wet levels are contiguous from the top
    nam = shelf.namelist(neuler=0)
    st = shelf.state(dom, nam, seed=2)
    o = ora.Oracle(dom, nam)
    keep = _bind_spg(o, dom, st)
    for n in ("TSB", "TSN", "WN", "AVT", "USLP", "VSLP", "WSLPI", "WSLPJ", "GTSU", "GTSV", "SSH_IB"):
        keep[n] = st[n.lower()].copy(order="F")
        o.bind(n, keep[n])
    _bind_zstar(o, dom, st, keep)
    for n, shape in (("TSA", st["tsb"].shape), ("AH_WSLP2", st["avt"].shape), ("AKZ", st["avt"].shape)):
        keep[n] = np.zeros(shape, order="F")
        o.bind(n, keep[n])
    for kt in (1, 2):
        o.stp_hotpath(kt)
    assert np.isfinite(keep["TSA"]).all() and np.isfinite(keep["ua"]).all() and np.abs(keep["SSHA"]).max() > 0
    icycle, nn_baro, _ = o.spg_info()
    assert nn_baro == 30 and icycle == 44
