"""The triad (Griffies) iso-neutral operator: ldf_slp_triad (ldfslp.F90:377-617) and
tra_ldf_triad (traldf_triad.F90:50-429).

On the CPU, known answers of the oracle: a uniformly tilted stratification gives
every triad below the mixed layer the slope -a/b of its isopycnals, the switching
scheme keeps the two triads aligned with the tilt (weight 2) and drops the others,
and inside the mixed layer the slope tapers linearly with depth from its value
below the base; over isopycnals flat in the levels the operator with bottom mixing
is the laplacian; the operator conserves the tracer content. On the GPU: the slopes,
wslp2, ah_wslp2, akz and the trend through the C ABI against the oracle on GYRE and
on the partial-step z* shelf, FP64 to 1e-12 and the mixed form; the bilaplacian's
second pass; tra_zdf_imp with the triad's ah_wslp2."""
import numpy as np
import pytest

from nemo_gpu import gyre, shelf

F = np.asfortranarray
TRIADS = ("TRIADI_G", "TRIADJ_G", "TRIADI", "TRIADJ")


def rab_of(o, tsb):
    pab = np.zeros_like(tsb, order="F")
    o.rab_3d(tsb, pab)
    return pab


def oracle_case(dom=None, seed=3, **over):
    from oracle import ora
    dom = dom or gyre.domain(1)
    nam = gyre.namelist(ln_traldf_iso=0, ln_traldf_triad=1, ln_seos=1, **over)
    st = gyre.state(dom, nam, seed=seed)
    inp = gyre.slope_inputs(dom, nam, st)
    o = ora.Oracle(dom, nam)
    s3 = (dom["jpi"], dom["jpj"], dom["jpk"])
    f = {n: np.zeros(s3 + (2, 2), order="F") for n in TRIADS}
    f["WSLP2"] = np.zeros(s3, order="F")
    f["AH_WSLP2"] = np.zeros(s3, order="F")
    f["AKZ"] = np.zeros(s3, order="F")
    f["TSB"] = F(st["tsb"].copy())
    for n in ("GDEPT_N", "GDEPW_N", "NMLN"):
        f[n] = inp[n.lower()]
    for n, a in f.items():
        o.bind(n, a)
    return dom, nam, st, o, f


def tilted(dom, o, f, a=2e-6, b=1e-2):
    """T = 20 + a x - b D with D the running sum of e3w (so T(k-1) - T(k) = b e3w(k)),
    S uniform, constant expansion ratios; the isopycnal slope is a / b."""
    tm = gyre.masks(dom)[0]
    x = np.cumsum(dom["e1t"], axis=0)[:, :, None]
    D = np.cumsum(dom["e3w_0"], axis=2)
    f["TSB"][..., 0] = (20.0 + a * x - b * D) * tm
    f["TSB"][..., 1] = 35.0 * tm
    rab = np.zeros_like(f["TSB"])
    rab[..., 0], rab[..., 1] = 2e-4, 7.7e-4
    return F(rab * tm[..., None])


def test_oracle_tilted_stratification_slopes_and_switching():
    dom, nam, st, o, f = oracle_case()
    a, b = 2e-6, 1e-2
    rab = tilted(dom, o, f, a, b)
    f["NMLN"][...] = 3
    o.ldf_slp_triad(1, rab)
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    kb = dom["k_bot"]
    # deep interior T-points whose columns and i-neighbours are wet to below level 12
    ii, jj = np.nonzero(kb[1:-2, 1:-1] >= 14)
    ii, jj = ii + 1, jj + 1
    ok = (kb[ii + 1, jj] >= 14) & (kb[ii - 1, jj] >= 14)
    ii, jj = ii[ok], jj[ok]
    ks = np.arange(5, 12)                        # 0-based levels 5..11: below the mixed layer
    g = f["TRIADI_G"][ii[:, None], jj[:, None], ks[None, :]]
    np.testing.assert_allclose(g, -a / b, rtol=1e-12)
    t = f["TRIADI"][ii[:, None], jj[:, None], ks[None, :]]
    # dx(rho) < 0: the triads (a, kp) = (1, 0) and (0, 1) carry weight 2, the others 0
    np.testing.assert_allclose(t[..., 1, 0], -2 * a / b, rtol=1e-12)
    np.testing.assert_allclose(t[..., 0, 1], -2 * a / b, rtol=1e-12)
    assert not t[..., 0, 0].any() and not t[..., 1, 1].any()
    # inside the mixed layer (levels 1..nmln - 1 for kp = 0): linear taper in depth
    gdepw = f["GDEPW_N"]
    i0, j0 = ii[0], jj[0]
    k = 1                                         # 1-based level 2, kp = 0: gdepw(2) / gdepw(4)
    want = (-a / b) * gdepw[i0, j0, k] / gdepw[i0, j0, 3]
    np.testing.assert_allclose(f["TRIADI_G"][i0, j0, k, 1, 0], want, rtol=1e-12)
    assert not f["TRIADI_G"][:, :, 0, :, 0].any()  # the surface triads of level 1
    assert (f["WSLP2"] >= 0).all() and not f["WSLP2"][:, :, 0].any()


def test_oracle_flat_isopycnals_with_bottom_mixing_is_the_laplacian():
    dom, nam, st, o, f = oracle_case(ln_botmix_triad=1)
    tm = gyre.masks(dom)[0]
    d1 = np.linspace(20.0, 5.0, dom["jpk"])[None, None, :]
    f["TSB"][..., 0] = d1 * tm
    f["TSB"][..., 1] = 35.0 * tm
    rab = np.zeros_like(f["TSB"])
    rab[..., 0], rab[..., 1] = 2e-4, 7.7e-4
    o.ldf_slp_triad(1, F(rab * tm[..., None]))
    ptb = F(st["tsb"])                            # a tracer with horizontal structure
    ta = np.zeros_like(ptb, order="F")
    o.tra_ldf_triad(1, 1, "TRA", None, None, None, None, None, None, ptb, ptb, ta, 2, 1)
    tl = np.zeros_like(ptb, order="F")
    o.tra_ldf_lap(1, 1, "TRA", None, None, None, None, None, None, ptb, tl, 2, 1)
    assert np.abs(tl).max() > 0
    np.testing.assert_allclose(ta, tl, rtol=0, atol=1e-12 * np.abs(tl).max())
    np.testing.assert_array_equal(f["AKZ"], f["AH_WSLP2"])


@pytest.mark.parametrize("msc", [0, 1])
def test_oracle_triad_conserves_the_tracer_content(msc):
    dom, nam, st, o, f = oracle_case(ln_traldf_msc=msc)
    rab = rab_of(o, f["TSB"])
    o.ldf_slp_triad(1, rab)
    ptb = F(st["tsb"])
    ta = np.zeros_like(ptb, order="F")
    o.tra_ldf_triad(1, 1, "TRA", None, None, None, None, None, None, ptb, ptb, ta, 2, 1)
    vol = (dom["e1t"] * dom["e2t"])[:, :, None] * dom["e3t_0"] * gyre.masks(dom)[0]
    for n in range(2):
        x = vol * ta[..., n]
        assert abs(x.sum()) <= 1e-13 * np.abs(x).sum(), (n, x.sum(), np.abs(x).sum())
    assert (f["AH_WSLP2"] >= 0).all() and np.abs(ta).max() > 0


# ------------------------------------------------------------------------- GPU
def gpu_case(prec, where, nmem=2, **over):
    pytest.importorskip("torch")
    import torch
    from harness import Pair
    if where == "shelf":
        dom = shelf.domain(seed=8, jpi=30, jpj=26, jpk=18)
        nam = shelf.namelist(ln_traldf_iso=0, ln_traldf_triad=1, ln_seos=1, **over)
        states = [shelf.state(dom, nam, seed=8, member=m) for m in range(nmem)]
        for st in states:
            st.update(shelf.depths(st))
    else:
        dom = gyre.domain(1)
        nam = gyre.namelist(ln_traldf_iso=0, ln_traldf_triad=1, ln_seos=1, **over)
        states = [gyre.state(dom, nam, seed=9, member=m) for m in range(nmem)]
    for st in states:
        inp = gyre.slope_inputs(dom, nam, st)
        st.setdefault("gdept_n", inp["gdept_n"])
        st.setdefault("gdepw_n", inp["gdepw_n"])
        st["nmln"] = inp["nmln"]
        if prec == "mixed":  # the oracle sees the FP32 values the GPU holds
            for n in ("tsb", "gdept_n", "gdepw_n"):
                st[n] = F(st[n].astype(np.float32).astype(np.float64))
    p = Pair(dom=dom, nam=nam, prec=prec, states=states)
    from oracle import ora
    o0 = ora.Oracle(dom, nam)
    rabs = []
    for st in states:
        o0.bind("GDEPT_N", st["gdept_n"])          # eos_rab at the now depths
        rabs.append(rab_of(o0, st["tsb"]))
    if prec == "mixed":
        rabs = [F(r.astype(np.float32).astype(np.float64)) for r in rabs]
    s3 = p.s3
    for n in TRIADS:
        p.bind(n, zero=True, shape=s3 + (2, 2))
    for n in ("WSLP2", "AH_WSLP2", "AKZ"):
        p.bind(n, zero=True, shape=s3)
    for n in ("TSB", "GDEPT_N", "GDEPW_N"):
        p.bind(n)
    if p.vvl:
        p.bind_zstar()
    nm = [F(st["nmln"]) for st in states]
    for i, o in enumerate(p.ora):
        o.bind("NMLN", nm[p.sample[i]])
    p.ctx.bind("NMLN", torch.from_numpy(np.concatenate([a.ravel(order="F") for a in nm])).cuda())
    p.rab_d = p.to_dev(rabs)
    p.rabs = rabs
    return p


@pytest.mark.gpu
@pytest.mark.parametrize("where", ["gyre", "shelf"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_triad_slopes_and_operator(prec, where):
    p = gpu_case(prec, where)
    tol = 1e-12 if prec == "fp64" else 2e-4
    for i, o in enumerate(p.ora):
        o.ldf_slp_triad(1, p.rabs[p.sample[i]])
    p.ctx.ldf_slp_triad(1, p.rab_d)
    for n in TRIADS:
        p.compare(n, p.s3 + (2, 2), tol)
    p.compare("WSLP2", p.s3, tol)
    # pass 1 of the laplacian on T and S
    ta = [np.zeros(p.s4, order="F") for _ in range(p.nmem)]
    ta_d = p.to_dev(ta)
    tb_d = p.dev["TSB"]
    for i, o in enumerate(p.ora):
        o.tra_ldf_triad(1, 1, "TRA", None, None, None, None, None, None, p.host[i]["TSB"], p.host[i]["TSB"], ta[i],
                        2, 1)
    p.ctx.tra_ldf_triad(1, 1, "TRA", None, None, None, None, None, None, tb_d, tb_d, ta_d, 2, 1)
    p.ctx.synchronize()
    got = p.per_member(ta_d, p.s4)
    from harness import relerr
    for i, m in enumerate(p.sample):
        e = relerr(ta[i], got[m], name="TA")
        assert e <= (1e-12 if prec == "fp64" else 2e-3), e
    p.compare("AH_WSLP2", p.s3, tol)
    p.compare("AKZ", p.s3, tol)
    # tra_zdf_imp adds the triad's ah_wslp2 to avt (l_ldfslp without msc)
    p.bind("AVT")
    p2dt = 2.0 * p.nam["rn_rdt"]
    for i, o in enumerate(p.ora):
        o.tra_zdf_imp(1, 1, "TRA", p2dt, p.host[i]["TSB"], ta[i], 2)
    p.ctx.tra_zdf_imp(1, 1, "TRA", p2dt, tb_d, ta_d, 2)
    p.ctx.synchronize()
    got = p.per_member(ta_d, p.s4)
    for i, m in enumerate(p.sample):
        e = relerr(ta[i], got[m], name="TA_ZDF")
        assert e <= (1e-12 if prec == "fp64" else 2e-5), e


@pytest.mark.gpu
def test_gpu_triad_bilaplacian_second_pass():
    """kpass = 2 of the bilaplacian (sign -1, akz on ptbb) on the laplacian of pass 1
    after its lbc_lnk, with the stabilising akz of ln_traldf_msc."""
    p = gpu_case("fp64", "gyre", ln_traldf_blp=1, ln_traldf_lap=0, ln_traldf_msc=1)
    for i, o in enumerate(p.ora):
        o.ldf_slp_triad(1, p.rabs[p.sample[i]])
    p.ctx.ldf_slp_triad(1, p.rab_d)
    lap = [np.zeros(p.s4, order="F") for _ in range(p.nmem)]
    out = [np.zeros(p.s4, order="F") for _ in range(p.nmem)]
    lap_d, out_d = p.to_dev(lap), p.to_dev(out)
    tb_d = p.dev["TSB"]
    for i, o in enumerate(p.ora):
        tb = p.host[i]["TSB"]
        o.tra_ldf_triad(1, 1, "TRA", None, None, None, None, None, None, tb, tb, lap[i], 2, 1)
        o.lbc_lnk(lap[i], "T")
        o.tra_ldf_triad(1, 1, "TRA", None, None, None, None, None, None, lap[i], tb, out[i], 2, 2)
    p.ctx.tra_ldf_triad(1, 1, "TRA", None, None, None, None, None, None, tb_d, tb_d, lap_d, 2, 1)
    p.ctx.lbc_lnk(lap_d, p.dom["jpk"], "T", nl=2)
    p.ctx.tra_ldf_triad(1, 1, "TRA", None, None, None, None, None, None, lap_d, tb_d, out_d, 2, 2)
    p.ctx.synchronize()
    from harness import relerr
    g = p.per_member(out_d, p.s4)
    for i, m in enumerate(p.sample):
        assert relerr(out[i], g[m], name="TA2") <= 1e-12
    p.compare("AKZ", p.s3, 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("blp", [0, 1])
def test_stp_hotpath_with_the_triad_operator(prec, blp):
    """nemo_gpu_stp_hotpath with ln_traldf_triad: the laplacian (np_lap_it) or the
    bilaplacian (np_blp_it, kldf = 22) in place of the standard iso-neutral operator,
    the triad slopes of the oracle bound on both sides, three steps from an Euler
    start."""
    pytest.importorskip("torch")
    import torch
    from harness import Pair
    from oracle import ora
    over = dict(ln_traldf_lap=0, ln_traldf_blp=1, rn_aht_0=1.e11) if blp else {}
    p = Pair(nn=2, prec=prec, seed=75, neuler=0, ln_traldf_iso=0, ln_traldf_triad=1, ln_seos=1, **over)
    st = p.states[0]
    inp = gyre.slope_inputs(p.dom, p.nam, st)
    st["gdept_n"], st["gdepw_n"] = inp["gdept_n"], inp["gdepw_n"]
    p.bind_hotpath()
    p.bind("GDEPT_N")
    p.bind("GDEPW_N")
    o = p.ora[0]
    nm = F(inp["nmln"])
    o.bind("NMLN", nm)
    p.ctx.bind("NMLN", torch.from_numpy(nm.ravel(order="F").copy()).cuda())
    tri = {n: np.zeros(p.s3 + (2, 2), order="F") for n in TRIADS}
    for n, a in tri.items():
        o.bind(n, a)
    o.ldf_slp_triad(1, rab_of(o, p.host[0]["TSB"]))
    for n, a in tri.items():                       # the same slopes on the device
        st[n.lower()] = a
        t = p.to_dev([a])
        p.dev[n] = t
        p.ctx.bind(n, t)
    for kt in (1, 2, 3):
        o.stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
    p.ctx.synchronize()
    p.compare("TSA", p.s4, 1e-12 if prec == "fp64" else 5e-6)
