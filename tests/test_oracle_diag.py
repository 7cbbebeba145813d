"""Known answers of the oracle's run control (stp_ctl, stpctl.F90:44-194) and
conservation budgets (dia_hsb, diahsb.F90:60-239): the extrema against numpy, the
blow-up test and its positions on values injected on the host, the identities of a
first call, and the closure of the heat, salt and volume budgets over a forced run."""
import numpy as np

from nemo_gpu import gyre
from oracle import ora

S2_FIELDS = ("sshn", "sshb", "un_b", "vn_b", "ub_b", "vb_b", "utau", "vtau", "emp", "qsr", "qns", "sfx",
             "fraqsr_1lev")
S3_FIELDS = ("tsb", "tsn", "un", "vn", "wn", "ub", "vb", "ua", "va", "avt", "uslp", "vslp", "wslpi", "wslpj",
             "sbc_tsc", "sbc_tsc_b", "qsr_hc", "qsr_hc_b", "gdepw_n")
ACC = ("SSHA", "UA_B", "VA_B", "UN_ADV", "VN_ADV", "UB2_B", "VB2_B", "UN_BF", "VN_BF")


def forced_oracle(nn=1, seed=41, **over):
    """An oracle holding a GYRE state with the analytic surface forcing bound."""
    dom = gyre.domain(nn)
    nam = gyre.namelist(neuler=0, **over)
    st = gyre.state(dom, nam, seed=seed)
    st.update(gyre.sbc_inputs(dom, nam, st, kt=1))
    o = ora.Oracle(dom, nam)
    keep = {}
    for n in S2_FIELDS + S3_FIELDS:
        keep[n] = np.array(st[n], order="F", copy=True)
        o.bind(n.upper(), keep[n])
    keep["rcdu_bot"] = np.array(st["rcdu_bot"], order="F", copy=True)
    o.bind("RCDU_BOT", keep["rcdu_bot"])
    for n, shape in (("TSA", st["tsb"].shape), ("AH_WSLP2", st["avt"].shape), ("AKZ", st["avt"].shape)):
        keep[n] = np.zeros(shape, order="F")
        o.bind(n, keep[n])
    for n in ACC:
        keep[n] = np.zeros(st["sshn"].shape, order="F")
        o.bind(n, keep[n])
    return dom, nam, o, keep


def test_stp_ctl_extrema():
    dom, nam, o, f = forced_oracle()
    zmax, loc, kindic = o.stp_ctl(5)
    tm = np.arange(1, dom["jpk"] + 1)[None, None, :] <= dom["k_bot"][:, :, None]
    t, s = f["tsn"][..., 0], f["tsn"][..., 1]
    ref = [np.abs(f["sshn"]).max(), np.abs(f["un"]).max(), (-s[tm]).max(), s[tm].max(), (-t[tm]).max(), t[tm].max()]
    np.testing.assert_array_equal(zmax, ref)
    assert kindic == 0 and not loc.any()


def test_stp_ctl_blowup_and_positions():
    """Each condition of stpctl.F90:149-157 on a value injected on the host: the
    test fires (kindic = -3) and the position of the offending value is reported."""
    dom, nam, o, f = forced_oracle()
    jpi, jpj = dom["jpi"], dom["jpj"]
    i, j, k = 7, 9, 3                                   # a wet interior point (0-based)
    assert dom["k_bot"][i, j] > k
    s0 = f["tsn"][i, j, k, 1]
    f["tsn"][i, j, k, 1] = -1.0                         # S <= 0
    zmax, loc, kindic = o.stp_ctl(5)
    assert kindic == -3 and zmax[2] == 1.0
    assert tuple(loc[5:8]) == (i + 1, j + 1, k + 1)    # MINLOC(S)
    f["tsn"][i, j, k, 1] = 120.0                        # S >= 100
    zmax, loc, kindic = o.stp_ctl(5)
    assert kindic == -3 and zmax[3] == 120.0 and tuple(loc[8:11]) == (i + 1, j + 1, k + 1)
    f["tsn"][i, j, k, 1] = s0
    f["sshn"][3, 4] = -25.0                             # |ssh| > 20 m
    zmax, loc, kindic = o.stp_ctl(5)
    assert kindic == -3 and zmax[0] == 25.0 and tuple(loc[0:2]) == (4, 5)
    f["sshn"][3, 4] = 0.0
    f["un"][5, 6, 2] = np.nan                           # NaN
    zmax, loc, kindic = o.stp_ctl(5)
    assert kindic == -3 and np.isnan(zmax[1]) and tuple(loc[2:5]) == (6, 7, 3)
    f["un"][5, 6, 2] = 0.0
    assert o.stp_ctl(5)[2] == 0
    assert jpi > 8 and jpj > 10


def test_dia_hsb_first_call():
    """Right after dia_hsb_init, with the state unchanged, the content variations are
    zero: the drifts are minus the forcing of one step."""
    dom, nam, o, f = forced_oracle()
    o.dia_hsb_init()
    # tra_sbc forms sbc_tsc; here it is set directly
    f["sbc_tsc"][..., 0] = 1e-5
    f["sbc_tsc"][..., 1] = 2e-6
    h = o.dia_hsb(5)
    frc_v, frc_t, frc_s = h[0], h[1], h[2]
    assert frc_t > 0 and frc_s > 0
    np.testing.assert_allclose(h[5], -frc_v, rtol=0, atol=1e-9 * abs(frc_v) + 1e-30)
    # the content is summed as (surf e3t) T against the initial surf (T e3t): rounding
    # of the two products, ~1e-16 of the content
    content = 40.0 * h[13]
    assert abs(h[7] + frc_t) <= 1e-15 * content and abs(h[8] + frc_s) <= 1e-15 * content
    assert h[6] == 0.0 and h[11] == -h[3] and h[12] == -h[4]
    tm = np.arange(1, dom["jpk"] + 1)[None, None, :] <= dom["k_bot"][:, :, None]
    surf = dom["e1t"] * dom["e2t"]
    inner = np.zeros(surf.shape, bool)
    inner[1:-1, 1:-1] = True
    vol = (surf[:, :, None] * dom["e3t_0"] * tm)[:, :, :-1][inner].sum()
    np.testing.assert_allclose(h[13], vol, rtol=1e-13)


def test_dia_hsb_budget_closes_over_a_forced_run():
    """Thirty model steps with the analytic surface forcing: after the first (Euler)
    step the heat drift changes by less than 1e-3 of the accumulated heat forcing, the
    salt drift by less than 1e-8 of the salt content, and the volume drift stays at
    rounding level."""
    dom, nam, o, f = forced_oracle()
    o.dia_hsb_init()
    first = None
    for kt in range(1, 31):
        o.stp_model(kt)
        if kt == 1:
            first = o.dia_hsb_last()
    h = o.dia_hsb_last()
    salt = 35.0 * h[13]
    assert abs(h[7] - first[7]) <= 1e-3 * abs(h[1])
    assert abs(h[8] - first[8]) <= 1e-8 * salt
    assert abs(h[5]) <= 1e-12 * h[13]
    z, loc, kindic = o.stp_ctl_last()
    assert kindic == 0 and z[3] < 100 and z[2] < 0
