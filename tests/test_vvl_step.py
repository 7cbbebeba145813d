"""z* time stepping of a variable-volume model: dom_vvl_sf_nxt (domvvl.F90:268-562),
tra_nxt_vvl (tranxt.F90:240-380), dyn_nxt's filter of the before scale factors and
velocities (dynnxt.F90:217-343), ssh_swp with the forcing removed (sshwzv.F90:254-258)
and dom_vvl_sf_swp (domvvl.F90:565-675).

On the CPU, known answers of the oracle on a partial-step shelf: the after scale
factors of an ssh increment are the z* scale factors of the after ssh; the swap
copies the after fields and its depths are the running sums of the scale factors;
a uniform tracer stays uniform under the thickness-weighted filter and a fixed volume
gives the fixed-volume filter; after dyn_nxt and ssh_swp the filtered before column
thickness equals ht_0 + the filtered before ssh (the forcing removed from both). On
the GPU: each routine through the C ABI against the oracle over a few steps of a
host-driven cycle, FP64 to 1e-12 and the mixed form, vector- and flux-form momentum,
with and without runoff and penetrating light."""
import numpy as np
import pytest

from harness import Pair
from nemo_gpu import gyre, shelf

F = np.asfortranarray


def w_rest(dom):
    """e3uw_0, e3vw_0 of a z-coordinate with partial steps: the MIN of the
    neighbouring e3w_0 (the domain file's fields; closed last row/column: e3w_0)."""
    e3w = dom["e3w_0"]
    uw, vw = e3w.copy(), e3w.copy()
    uw[:-1] = np.minimum(e3w[:-1], e3w[1:])
    vw[:, :-1] = np.minimum(e3w[:, :-1], e3w[:, 1:])
    return F(uw), F(vw)


def vvl_state(dom, nam, seed=0, member=0, rnf=False):
    """A shelf state with every field of the z* time stepping: z*-consistent before,
    now and after scale factors for sshb, sshn and an after ssh; after tracers and
    velocities near the now ones; surface forcing and penetrating-light trends."""
    st = shelf.state(dom, nam, seed=seed, member=member)
    rng = np.random.default_rng([seed, member, 9])
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    tm, um, vm, _ = gyre.masks(dom)
    ssm = tm.max(axis=2)
    noise = lambda *s: rng.standard_normal(s)
    st["ssha"] = F((2.0 * st["sshn"] - st["sshb"] + 1e-3 * noise(jpi, jpj)) * ssm)
    za = gyre.zstar(dom, dict(st, sshb=st["sshn"], sshn=st["ssha"]))
    for n in ("e3t", "e3u", "e3v"):
        st[n + "_a"] = za[n + "_n"]
    for n in ("hu", "hv", "r1_hu", "r1_hv"):
        st[n + "_a"] = za[n + "_n"]
    zb = gyre.zstar(dom, dict(st, sshn=st["sshb"]))
    st["e3u_b"], st["e3v_b"], st["e3w_b"] = zb["e3u_n"], zb["e3v_n"], zb["e3w_n"]
    st["e3uw_0"], st["e3vw_0"] = w_rest(dom)
    for n in ("e3uw_n", "e3vw_n"):
        st[n] = st[n[:3] + "w_0"].copy(order="F")
    st["e3uw_b"], st["e3vw_b"] = st["e3uw_0"].copy(order="F"), st["e3vw_0"].copy(order="F")
    st.update(shelf.depths(st))
    st["gde3w_n"] = F(st["gdept_n"] - st["sshn"][:, :, None])
    st["gdept_b"], st["gdepw_b"] = st["gdept_n"].copy(order="F"), st["gdepw_n"].copy(order="F")
    st["emp"] = F(2e-4 * noise(jpi, jpj) * ssm)
    st["emp_b"] = F(st["emp"] + 5e-5 * noise(jpi, jpj) * ssm)
    if rnf:
        st["rnf"] = F(1e-4 * np.abs(noise(jpi, jpj)) * ssm)
        st["rnf_b"] = F(0.8 * st["rnf"])
    st["tsa"] = F(st["tsn"] + 0.02 * noise(jpi, jpj, jpk, 2) * tm[..., None])
    st["ua"] = F(st["un"] + 0.003 * noise(jpi, jpj, jpk) * um)
    st["va"] = F(st["vn"] + 0.003 * noise(jpi, jpj, jpk) * vm)
    st["ua_b"] = F(st["un_b"] + 1e-3 * noise(jpi, jpj) * um.max(axis=2))
    st["va_b"] = F(st["vn_b"] + 1e-3 * noise(jpi, jpj) * vm.max(axis=2))
    st["sbc_tsc"] = F(1e-5 * noise(jpi, jpj, 2) * ssm[..., None])
    st["sbc_tsc_b"] = F(1e-5 * noise(jpi, jpj, 2) * ssm[..., None])
    st["qsr_hc"] = F(1e-6 * np.abs(noise(jpi, jpj, jpk)) * tm)
    st["qsr_hc_b"] = F(1e-6 * np.abs(noise(jpi, jpj, jpk)) * tm)
    return st


SMALL = dict(jpi=30, jpj=26, jpk=18)
OUT3 = ("E3T_A", "E3U_A", "E3V_A", "E3U_B", "E3V_B", "E3W_B", "E3UW_N", "E3VW_N", "E3UW_B", "E3VW_B",
        "E3T_B", "E3T_N", "E3U_N", "E3V_N", "E3W_N", "E3F_N", "GDEPT_N", "GDEPW_N", "GDE3W_N", "GDEPT_B",
        "GDEPW_B", "UN", "VN", "UB", "VB", "UA", "VA")
OUT2 = ("HU_A", "HV_A", "R1_HU_A", "R1_HV_A", "HU_N", "HV_N", "R1_HU_N", "R1_HV_N", "HT_N", "HU_B", "HV_B",
        "R1_HU_B", "R1_HV_B", "SSHB", "SSHN", "UN_B", "VN_B", "UB_B", "VB_B")
IN3 = ("E3UW_0", "E3VW_0", "QSR_HC", "QSR_HC_B")
IN2 = ("SSHA", "EMP", "EMP_B", "UA_B", "VA_B")


def oracle_case(nam_over=None, rnf=False, seed=4):
    from oracle import ora
    dom = shelf.domain(seed=seed, **SMALL)
    nam = shelf.namelist(**(nam_over or {}))
    st = vvl_state(dom, nam, seed=seed, rnf=rnf)
    o = ora.Oracle(dom, nam)
    f = {}
    names = OUT3 + OUT2 + IN3 + IN2 + ("TSB", "TSN", "TSA", "SBC_TSC", "SBC_TSC_B")
    if rnf:
        names += ("RNF", "RNF_B")
    for n in names:
        f[n] = np.array(st[n.lower()], dtype=np.float64, order="F", copy=True)
        o.bind(n, f[n])
    return dom, nam, o, f


def test_oracle_sf_nxt_is_the_zstar_of_the_after_ssh():
    dom, nam, o, f = oracle_case()
    want = {n: f[n].copy() for n in ("E3T_A", "E3U_A", "E3V_A", "HU_A", "R1_HU_A", "HV_A")}
    for n in want:
        f[n][...] = 0.0
    o.dom_vvl_sf_nxt(2)
    jpk = dom["jpk"]
    for n, w in want.items():
        g = f[n][:, :, :jpk - 1] if n == "E3T_A" else f[n]
        ww = w[:, :, :jpk - 1] if n == "E3T_A" else w
        np.testing.assert_allclose(g, ww, rtol=2e-14, atol=2e-14 * np.abs(ww).max(), err_msg=n)


def test_oracle_sf_swp_copies_and_depths():
    dom, nam, o, f = oracle_case()
    o.dom_vvl_sf_nxt(2)
    f["SSHN"][...] = f["SSHA"]                       # ssh_swp ran before the swap
    o.dom_vvl_sf_swp(2)
    tm, um, _, _ = gyre.masks(dom)
    for a, b in (("E3T_N", "E3T_A"), ("E3U_N", "E3U_A"), ("E3V_N", "E3V_A"), ("HU_N", "HU_A"),
                 ("R1_HV_N", "R1_HV_A")):
        np.testing.assert_array_equal(f[a], f[b], err_msg=a)
    e3t = f["E3T_N"]
    gw = np.zeros_like(e3t)
    gw[:, :, 1:] = np.cumsum(e3t[:, :, :-1], axis=2)
    np.testing.assert_allclose(f["GDEPW_N"], gw, rtol=1e-13, atol=1e-12)
    gt = 0.5 * f["E3W_N"][:, :, :1] + np.concatenate(
        [np.zeros_like(e3t[:, :, :1]), np.cumsum(f["E3W_N"][:, :, 1:], axis=2)], axis=2)
    np.testing.assert_allclose(f["GDEPT_N"], gt, rtol=1e-13, atol=1e-12)
    np.testing.assert_allclose(f["GDE3W_N"], gt - f["SSHN"][:, :, None], rtol=1e-13, atol=1e-12)
    ht_0 = (dom["e3t_0"] * tm)[:, :, :-1].sum(axis=2)
    np.testing.assert_allclose(f["HT_N"], ht_0 + f["SSHN"] * tm.max(axis=2), rtol=0, atol=1e-11)
    z = gyre.zstar(dom, {"sshb": f["SSHA"], "sshn": f["SSHA"]})
    for n in ("E3W_N", "E3F_N"):
        np.testing.assert_allclose(f[n], z[n.lower()], rtol=1e-13, atol=1e-13, err_msg=n)
    # uw: the rest state plus the mean of the u-level changes around the w-level
    d = f["E3U_N"] - dom["e3u_0"]
    uw = f["E3UW_0"].copy()
    uw[:, :, 0] += d[:, :, 0]
    uw[:, :, 1:] += (1.0 - 0.5 * um[:, :, 1:]) * d[:, :, :-1] + 0.5 * um[:, :, 1:] * d[:, :, 1:]
    np.testing.assert_allclose(f["E3UW_N"], uw, rtol=1e-14, atol=1e-14)


def test_oracle_tra_nxt_vvl_uniform_tracer_and_fixed_volume():
    dom, nam, o, f = oracle_case(dict(ln_traqsr=0))
    tm = gyre.masks(dom)[0]
    for n in ("SBC_TSC", "SBC_TSC_B"):
        f[n][...] = 0.0
    f["EMP_B"][...] = f["EMP"]
    for n in ("TSB", "TSN", "TSA"):
        f[n][..., 0] = 7.5
        f[n][..., 1] = 34.25
    o.tra_nxt(2)
    inner = (slice(1, -1), slice(1, -1), slice(0, dom["jpk"] - 1))
    np.testing.assert_allclose(f["TSB"][inner][..., 0], 7.5, rtol=4e-15)
    np.testing.assert_allclose(f["TSB"][inner][..., 1], 34.25, rtol=4e-15)
    # a fixed volume: the fixed-volume filter
    dom, nam, o, f = oracle_case(dict(ln_traqsr=0), seed=5)
    for n in ("E3T_B", "E3T_A"):
        f[n][...] = f["E3T_N"]
    for n in ("SBC_TSC", "SBC_TSC_B"):
        f[n][...] = 0.0
    f["EMP_B"][...] = f["EMP"]
    tb, tn, ta = f["TSB"].copy(), f["TSN"].copy(), f["TSA"].copy()
    o.tra_nxt(2)
    want = tn + nam["rn_atfp"] * (tb - 2.0 * tn + ta)
    np.testing.assert_allclose(f["TSB"][inner], want[inner], rtol=1e-13, atol=1e-13)
    np.testing.assert_array_equal(f["TSN"][inner], ta[inner])
    assert not f["TSB"][0].any() and not f["TSN"][:, -1].any()      # lbc of the closed edges


def test_oracle_tra_nxt_vvl_forcing_terms():
    """The first-level and light terms against a numpy restatement (:293-341)."""
    dom, nam, o, f = oracle_case(dict(ln_traqsr=1), rnf=True)
    nksr = o.nksr()
    atfp, rdt, rau0 = nam["rn_atfp"], nam["rn_rdt"], nam["rau0"]
    tb, tn, ta = f["TSB"].copy(), f["TSN"].copy(), f["TSA"].copy()
    e3b, e3n, e3a = (f[n][..., None] for n in ("E3T_B", "E3T_N", "E3T_A"))
    o.tra_nxt(2)
    z1, z2 = atfp * rdt, atfp * rdt / rau0
    e3f = e3n + atfp * (e3a - 2 * e3n + e3b)
    tcf = tn * e3n + atfp * (ta * e3a - 2 * tn * e3n + tb * e3b)
    e3f[:, :, 0] -= (z2 * (f["EMP_B"] - f["EMP"]) - z2 * (f["RNF_B"] - f["RNF"]))[..., None]
    tcf[:, :, 0] -= z1 * (f["SBC_TSC"] - f["SBC_TSC_B"])
    tcf[:, :, :nksr, 0] -= z1 * (f["QSR_HC"] - f["QSR_HC_B"])[:, :, :nksr]
    want = tcf / e3f
    inner = (slice(1, -1), slice(1, -1), slice(0, dom["jpk"] - 1))
    np.testing.assert_allclose(f["TSB"][inner], want[inner], rtol=1e-13)


@pytest.mark.parametrize("vec", [1, 0])
def test_oracle_dyn_nxt_and_ssh_swp_keep_the_column_volume(vec):
    """e3t_b and sshb are filtered alike with the same forcing removed, so the
    filtered before column thickness is ht_0 + the filtered before ssh."""
    dom, nam, o, f = oracle_case(dict(ln_dynadv_vec=vec))
    tm = gyre.masks(dom)[0]
    ht_0 = (dom["e3t_0"] * tm)[:, :, :-1].sum(axis=2)
    o.dom_vvl_sf_nxt(2)
    o.dyn_nxt(2)
    o.ssh_swp(2)
    h = (f["E3T_B"] * tm)[:, :, :-1].sum(axis=2)
    np.testing.assert_allclose(h, ht_0 + f["SSHB"] * tm.max(axis=2), rtol=0, atol=2e-11)
    np.testing.assert_array_equal(f["SSHN"], f["SSHA"])
    # the before velocity carries the time-split barotropic velocity un_b of the step
    um = gyre.masks(dom)[1]
    hu_b = (f["E3U_B"] * um)[:, :, :-1].sum(axis=2)
    np.testing.assert_allclose(f["HU_B"], hu_b, rtol=1e-14, atol=1e-12)


# ------------------------------------------------------------------------- GPU
def gpu_pair(prec, nmem=2, rnf=False, **over):
    pytest.importorskip("torch")
    dom = shelf.domain(seed=6, **SMALL)
    nam = shelf.namelist(**over)
    states = [vvl_state(dom, nam, seed=6, member=m, rnf=rnf) for m in range(nmem)]
    p = Pair(dom=dom, nam=nam, prec=prec, states=states)
    names = OUT3 + OUT2 + IN3 + IN2 + ("TSB", "TSN", "TSA", "SBC_TSC", "SBC_TSC_B")
    if rnf:
        names += ("RNF", "RNF_B")
    for n in names:
        p.bind(n)
    return p


def refresh(p, kt):
    """New after fields for the next step, the same on both sides: ssha, tsa, ua, va,
    ua_b, va_b from the oracle's now fields and a seeded perturbation."""
    rng = np.random.default_rng([kt, 99])
    tm, um, vm, _ = gyre.masks(p.dom)
    ssm = tm.max(axis=2)
    new = {n: [] for n in ("SSHA", "TSA", "UA", "VA", "UA_B", "VA_B")}
    for m in range(p.nmem):
        h = p.host[m]
        jpi, jpj, jpk = p.s3
        new["SSHA"].append(F((h["SSHN"] + 0.3 * (h["SSHN"] - h["SSHB"]) + 2e-4 * rng.standard_normal((jpi, jpj)))
                             * ssm))
        new["TSA"].append(F(h["TSN"] + 0.01 * rng.standard_normal(p.s4) * tm[..., None]))
        new["UA"].append(F(h["UN"] + 0.002 * rng.standard_normal(p.s3) * um))
        new["VA"].append(F(h["VN"] + 0.002 * rng.standard_normal(p.s3) * vm))
        new["UA_B"].append(F(h["UN_B"] + 5e-4 * rng.standard_normal((jpi, jpj)) * um.max(axis=2)))
        new["VA_B"].append(F(h["VN_B"] + 5e-4 * rng.standard_normal((jpi, jpj)) * vm.max(axis=2)))
    for n, arrs in new.items():
        p.set(n, arrs)


def cycle(p, steps, tol3, tol2):
    for kt in range(1, steps + 1):
        if kt > 1:
            refresh(p, kt)
        for o in p.ora:
            o.dom_vvl_sf_nxt(kt)
        p.ctx.dom_vvl_sf_nxt(kt)
        for n in ("E3T_A", "E3U_A", "E3V_A"):
            p.compare(n, p.s3, tol3)
        for n in ("HU_A", "R1_HV_A"):
            p.compare(n, p.s2, tol2)
        for o in p.ora:
            o.tra_nxt(kt)
            o.dyn_nxt(kt)
            o.ssh_swp(kt)
        p.ctx.tra_nxt(kt)
        p.ctx.dyn_nxt(kt)
        p.ctx.ssh_swp(kt)
        p.compare("TSB", p.s4, tol3)
        p.compare("TSN", p.s4, tol3)
        for n in ("E3T_B", "E3U_B", "E3V_B", "UB", "VB", "UN", "VN", "UA"):
            p.compare(n, p.s3, tol3)
        for n in ("SSHB", "SSHN", "UN_B", "UB_B", "VB_B", "HU_B", "R1_HV_B"):
            p.compare(n, p.s2, tol2)
        for o in p.ora:
            o.dom_vvl_sf_swp(kt)
        p.ctx.dom_vvl_sf_swp(kt)
        for n in ("E3T_N", "E3U_N", "E3W_N", "E3F_N", "E3UW_N", "E3VW_N", "E3W_B", "E3UW_B", "E3VW_B",
                  "GDEPT_N", "GDEPW_N", "GDE3W_N", "GDEPT_B"):
            p.compare(n, p.s3, tol3)
        for n in ("HT_N", "HU_N", "R1_HV_N"):
            p.compare(n, p.s2, tol2)
    p.ctx.synchronize()


@pytest.mark.gpu
@pytest.mark.parametrize("vec", [0, 1])
def test_gpu_vvl_cycle_fp64(vec):
    """Euler first step, then leap-frog steps; flux-form (the shelf's) and vector-form
    momentum; runoff and penetrating light in the flux-form case."""
    p = gpu_pair("fp64", rnf=not vec, neuler=0, ln_dynadv_vec=vec, ln_traqsr=1 - vec)
    cycle(p, 4, 1e-12, 1e-12)


@pytest.mark.gpu
def test_gpu_vvl_cycle_mixed():
    """The mixed form: FP32 fields, the time laplacians from differences; against the
    FP64 oracle the scale factors and depths hold to FP32 rounding of their values,
    the filtered velocities and tracers to the rounding of the differences."""
    p = gpu_pair("mixed", neuler=0, ln_dynadv_vec=0, ln_traqsr=1)
    cycle(p, 3, 2e-5, 2e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_zstar_hotpath_and_time_stepping_cycle(prec):
    """The variable-volume hot path (FCT 4/4, iso-neutral diffusion with partial-step
    gradients, zdf, dyn_spg_ts with EEN and flux-form momentum) chained with the z*
    time stepping for four steps from an Euler start, on both sides: wzv, stp_hotpath,
    the flux-form time step of dyn_zdf, dom_vvl_sf_nxt of the time-split ssha,
    tra_nxt_vvl, dyn_nxt, ssh_swp, dom_vvl_sf_swp -- each step reads the scale factors,
    depths and velocities the previous one formed; the other momentum trends are held
    fixed. (Chain parity; NEMO forms e3t_a before the tracer trends, here the hot path
    reads the previous step's.)"""
    pytest.importorskip("torch")
    dom = shelf.domain(seed=6, **SMALL)
    nam = shelf.namelist(neuler=0, ln_traqsr=0)
    states = []
    for m in range(2):
        st = vvl_state(dom, nam, seed=6, member=m)
        base = shelf.state(dom, nam, seed=6, member=m)
        st["ua"], st["va"] = base["ua"], base["va"]   # the hot path's ua, va are trends
        states.append(st)
    p = Pair(dom=dom, nam=nam, prec=prec, states=states)
    p.bind_hotpath()
    for n in OUT3 + OUT2 + IN3 + IN2 + ("SBC_TSC", "SBC_TSC_B", "GTSU", "GTSV", "SSH_IB"):
        if n not in ("UN", "VN", "UB", "VB", "UA", "VA", "SSHB", "SSHN", "UN_B", "VN_B", "UB_B", "VB_B"):
            p.bind(n)
    tol3 = 1e-12 if prec == "fp64" else 2e-4
    trend = [(F(st["ua"]), F(st["va"])) for st in states]
    for kt in range(1, 5):
        if kt > 1:  # the momentum trend of the other routines, held fixed
            for n, i in (("UA", 0), ("VA", 1)):
                p.set(n, [trend[m][i] for m in range(2)])
        for o in p.ora:
            o.wzv(kt)
            o.stp_hotpath(kt)
            o.dyn_zdf_step(kt)
            o.dom_vvl_sf_nxt(kt)
            o.tra_nxt(kt)
            o.dyn_nxt(kt)
            o.ssh_swp(kt)
            o.dom_vvl_sf_swp(kt)
        p.ctx.wzv(kt)
        p.ctx.stp_hotpath(kt)
        p.ctx.dyn_zdf_step(kt)
        p.ctx.dom_vvl_sf_nxt(kt)
        p.ctx.tra_nxt(kt)
        p.ctx.dyn_nxt(kt)
        p.ctx.ssh_swp(kt)
        p.ctx.dom_vvl_sf_swp(kt)
    p.ctx.synchronize()
    p.compare("TSN", p.s4, tol3)
    p.compare("TSB", p.s4, tol3)
    for n in ("UN", "VN", "UB", "E3T_N", "E3T_B", "E3U_N", "E3W_N", "GDEPT_N"):
        p.compare(n, p.s3, tol3)
    for n in ("SSHN", "SSHB", "HT_N", "UN_B"):
        p.compare(n, p.s2, tol3)


def test_oracle_dyn_zdf_flux_form_time_step():
    """dyn_zdf's flux-form time step with a variable volume (dynzdf.F90:115-120):
    (e3u_b ub + r2dt e3u_n ua) / e3u_a, which is the vector form when the three
    scale factors are equal."""
    from oracle import ora
    dom = shelf.domain(seed=4, **SMALL)
    nam = shelf.namelist(neuler=1, ln_dynadv_vec=0)
    st = vvl_state(dom, nam, seed=4)
    um = gyre.masks(dom)[1]
    r2dt = 2.0 * nam["rn_rdt"]
    for equal in (False, True):
        o = ora.Oracle(dom, nam)
        f = {n: np.array(st[n.lower()], order="F", copy=True) for n in ("UA", "VA", "UB", "VB", "E3U_B", "E3V_B",
                                                                         "E3U_N", "E3V_N", "E3U_A", "E3V_A")}
        if equal:
            for n in ("E3U_B", "E3U_A"):
                f[n][...] = f["E3U_N"]
        for n, a in f.items():
            o.bind(n, a)
        ua0, ub = f["UA"].copy(), f["UB"]
        o.dyn_zdf_step(3)
        k = slice(0, dom["jpk"] - 1)
        if equal:
            want = (ub + r2dt * ua0) * um
        else:
            want = (st["e3u_b"] * ub + r2dt * st["e3u_n"] * ua0) / st["e3u_a"] * um
        np.testing.assert_allclose(f["UA"][:, :, k], want[:, :, k], rtol=1e-14, atol=1e-14 * np.abs(want).max())
