"""GPU adjoint kernels against the oracle: the same adjoint (to 1e-12), and the
dot-product test <TL x, y> = <x, ADJ y> with the oracle's FP64 tangent-linear on
the left and the GPU adjoint on the right (to 1e-12). FCT uses the limiter
multipliers the GPU forward recorded, which match the oracle's."""
import numpy as np
import pytest

from adj_cases import Case, GpuCase, dot_test

pytestmark = pytest.mark.gpu
TOL = 1e-12


def relerr(ref, got):
    ref, got = np.asarray(ref), np.asarray(got)
    s = np.abs(ref).max()
    return np.abs(got - ref).max() / (s if s > 0 else 1.0)


@pytest.fixture(scope="module", params=["gyre", "shelf"])
def cases(request):
    c = Case(request.param, seed=11)
    return c, GpuCase(c)


@pytest.mark.parametrize("kh,kv", [(2, 2), (4, 4), (4, 2), (2, 4)])
def test_fct_tape_matches_oracle_and_adjoint(cases, kh, kv):
    """FCT 2/2 and, with the 4th-order centred horizontal fluxes and the compact
    vertical interpolation, FCT 4/4 (the shelf's configuration) and the mixed orders."""
    c, g = cases
    tape_o, ta_o = c.fct_record(kh=kh, kv=kv)
    tape_d = g.dev(np.zeros(3 * 2 * c.n3))
    g.ctx.bind("FCT_TAPE", tape_d)
    ta_d = g.dev(np.zeros(c.s4, order="F"))
    kt = c.kit + 2
    g.ctx.tra_adv_fct(kt, c.kit, "TRA", c.p2dt, g.zun, g.zvn, g.zwn, g.dev(c.tsb()), g.dev(c.tsn()), ta_d, 2, kh, kv)
    assert relerr(ta_o, g.host(ta_d, c.s4)[0]) <= TOL
    g.ctx.synchronize()
    tape_g = tape_d.cpu().numpy()
    assert np.abs(tape_g - tape_o).max() <= 1e-12
    assert (tape_g == tape_o).mean() > 0.999
    # the GPU adjoint against the oracle adjoint with the GPU's tape
    lam = c.rand4(masked=False)
    dtb, dtn = c.rand4(), c.rand4()
    tb_ad, tn_ad = g.dev(np.zeros(c.s4, order="F")), g.dev(np.zeros(c.s4, order="F"))
    lam_d = g.dev(lam)
    g.ctx.tra_adv_fct_adj(kt, c.kit, "TRA", c.p2dt, g.zun, g.zvn, g.zwn, tb_ad, tn_ad, lam_d, 2, kh, kv)
    g.ctx.synchronize()
    assert np.array_equal(g.host(lam_d, c.s4)[0], lam)   # pta_ad is left unchanged
    rtb, rtn = c.fct_adj(tape_g.copy(), lam, kh=kh, kv=kv)
    gtb, gtn = g.host(tb_ad, c.s4)[0], g.host(tn_ad, c.s4)[0]
    assert relerr(rtb, gtb) <= TOL and relerr(rtn, gtn) <= TOL, (relerr(rtb, gtb), relerr(rtn, gtn))
    # dot-product test: oracle tangent-linear with the same tape, GPU adjoint
    y = c.fct_tl(tape_g.copy(), dtb, dtn, kh=kh, kv=kv)
    err, lhs, _ = dot_test([(y, lam)], [(dtb, gtb), (dtn, gtn)])
    assert lhs != 0 and err <= TOL, err
    g.ctx.bind("FCT_TAPE", None)


def test_ldf_lap_adjoint(cases):
    c, g = cases
    for kpass in (1, 2):
        lam, dtb = c.rand4(masked=False), c.rand4()
        rtb = np.zeros(c.s4, order="F")
        c.o.tra_ldf_lap_adj(c.kit + 2, c.kit, "TRA", None, None, c.gtsu, c.gtsv, None, None, rtb, lam, 2, kpass)
        tb_ad = g.dev(np.zeros(c.s4, order="F"))
        g.ctx.tra_ldf_lap_adj(c.kit + 2, c.kit, "TRA", None, None, g.gtsu, g.gtsv, None, None, tb_ad, g.dev(lam), 2,
                              kpass)
        gtb = g.host(tb_ad, c.s4)[0]
        assert relerr(rtb, gtb) <= TOL
        y = np.zeros(c.s4, order="F")
        c.o.tra_ldf_lap(c.kit + 2, c.kit, "TRA", None, None, c.zero2, c.zero2, None, None, dtb, y, 2, kpass)
        err, lhs, _ = dot_test([(y, lam)], [(dtb, gtb)])
        assert lhs != 0 and err <= TOL, err


def test_ldf_iso_adjoint(cases):
    c, g = cases
    c.iso_coefficients()
    g.iso_coefficients()
    lam, dtb = c.rand4(masked=False), c.rand4()
    rtb = np.zeros(c.s4, order="F")
    c.o.tra_ldf_iso_adj(c.kit + 2, c.kit, "TRA", None, None, c.gtsu, c.gtsv, None, None, rtb, None, lam, 2, 1)
    tb_ad = g.dev(np.zeros(c.s4, order="F"))
    g.ctx.tra_ldf_iso_adj(c.kit + 2, c.kit, "TRA", None, None, g.gtsu, g.gtsv, None, None, tb_ad, None, g.dev(lam),
                          2, 1)
    gtb = g.host(tb_ad, c.s4)[0]
    assert relerr(rtb, gtb) <= TOL
    y = np.zeros(c.s4, order="F")
    c.o.tra_ldf_iso(c.kit + 2, c.kit, "TRA", None, None, c.zero2, c.zero2, None, None, dtb, dtb, y, 2, 1)
    err, lhs, _ = dot_test([(y, lam)], [(dtb, gtb)])
    assert lhs != 0 and err <= TOL, err


def test_ldf_iso_bilaplacian_second_pass_adjoint():
    c = Case("gyre", seed=12, ln_traldf_lap=0, ln_traldf_blp=1, rn_aht_0=1.e11)
    g = GpuCase(c)
    c.iso_coefficients()
    g.iso_coefficients()
    lam = c.rand4(masked=False)
    rtb, rtbb = np.zeros(c.s4, order="F"), np.zeros(c.s4, order="F")
    c.o.tra_ldf_iso_adj(c.kit + 2, c.kit, "TRA", None, None, c.zero2, c.zero2, None, None, rtb, rtbb, lam, 2, 2)
    tb_ad, tbb_ad = g.dev(np.zeros(c.s4, order="F")), g.dev(np.zeros(c.s4, order="F"))
    g.ctx.tra_ldf_iso_adj(c.kit + 2, c.kit, "TRA", None, None, g.gtsu, g.gtsv, None, None, tb_ad, tbb_ad,
                          g.dev(lam), 2, 2)
    assert relerr(rtb, g.host(tb_ad, c.s4)[0]) <= TOL
    assert relerr(rtbb, g.host(tbb_ad, c.s4)[0]) <= TOL


def test_zdf_imp_adjoint(cases):
    c, g = cases
    c.iso_coefficients()
    g.iso_coefficients()
    lam, dtb, dta = c.rand4(masked=False), c.rand4(), c.rand4(masked=False)
    rtb, rta = np.zeros(c.s4, order="F"), lam.copy(order="F")
    c.o.tra_zdf_imp_adj(c.kit + 2, c.kit, "TRA", c.p2dt, rtb, rta, 2)
    tb_ad, ta_ad = g.dev(np.zeros(c.s4, order="F")), g.dev(lam)
    g.ctx.tra_zdf_imp_adj(c.kit + 2, c.kit, "TRA", c.p2dt, tb_ad, ta_ad, 2)
    gtb, gta = g.host(tb_ad, c.s4)[0], g.host(ta_ad, c.s4)[0]
    assert relerr(rtb, gtb) <= TOL and relerr(rta, gta) <= TOL
    y = dta.copy(order="F")
    c.o.tra_zdf_imp(c.kit + 2, c.kit, "TRA", c.p2dt, dtb, y, 2)
    err, lhs, _ = dot_test([(y, lam)], [(dtb, gtb), (dta, gta)])
    assert lhs != 0 and err <= TOL, err


@pytest.mark.parametrize("euler", [True, False])
def test_tra_nxt_and_adjoint(euler):
    c = Case("gyre", seed=13, neuler=0 if euler else 1)
    g = GpuCase(c)
    kt = c.kit if euler else c.kit + 3
    xs = [c.rand4(False) for _ in range(3)]
    hs = [x.copy(order="F") for x in xs]
    for n, a in zip(("TSB", "TSN", "TSA"), hs):
        c.bind(n, a)
    c.o.tra_nxt(kt)
    ds = [g.bind(n, x) for n, x in zip(("TSB", "TSN", "TSA"), xs)]
    g.ctx.tra_nxt(kt)
    for h, dd in zip(hs, ds):
        assert np.array_equal(h, g.host(dd, c.s4)[0])
    lams = [c.rand4(False) for _ in range(3)]
    rs = [lam.copy(order="F") for lam in lams]
    c.o.tra_nxt_adj(kt, *rs)
    gs = [g.dev(lam) for lam in lams]
    g.ctx.tra_nxt_adj(kt, *gs)
    for r, dd in zip(rs, gs):
        assert relerr(r, g.host(dd, c.s4)[0]) <= 1e-15


def test_adjoints_of_two_members():
    """Member-outermost layout: each member's adjoint is that of its own fields."""
    c = Case("gyre", seed=14)
    g = GpuCase(c, nmem=2)
    tape_o, _ = c.fct_record()
    tape_d = g.dev(None, members=[tape_o, tape_o])
    g.ctx.bind("FCT_TAPE", tape_d)
    lams = [c.rand4(masked=False), c.rand4(masked=False)]
    tb_ad, tn_ad = g.dev(np.zeros(c.s4, order="F")), g.dev(np.zeros(c.s4, order="F"))
    g.ctx.tra_adv_fct_adj(c.kit + 2, c.kit, "TRA", c.p2dt, g.zun, g.zvn, g.zwn, tb_ad, tn_ad,
                          g.dev(None, members=lams), 2, 2, 2)
    gtb, gtn = g.host(tb_ad, c.s4), g.host(tn_ad, c.s4)
    for m in range(2):
        rtb, rtn = c.fct_adj(tape_o, lams[m])
        assert relerr(rtb, gtb[m]) <= TOL and relerr(rtn, gtn[m]) <= TOL
    g.ctx.bind("FCT_TAPE", None)


def test_adjoint_refuses_mixed_precision():
    from nemo_gpu import api
    c = Case("gyre", seed=15)
    ctx = api.Context(c.dom, c.nam, nmembers=1, prec="mixed")
    z = ctx.to_device(np.zeros(c.s4, order="F"))
    with pytest.raises(api.NemoError, match="FP64"):
        ctx.tra_zdf_imp_adj(c.kit + 2, c.kit, "TRA", c.p2dt, z, z, 2)
