"""The oracle's adjoints against its tangent-linears (dot-product test, FP64, to
1e-12) and the tangent-linears against finite differences of the forward
routines (away from limiter switches for FCT). These pin the host tangent-linear
and adjoint that the GPU adjoint kernels are checked against."""
import numpy as np
import pytest

from adj_cases import Case, dot_test

DOT_TOL = 1e-12


@pytest.fixture(scope="module")
def gyre_case():
    return Case("gyre", seed=3)


@pytest.fixture(scope="module")
def shelf_case():
    return Case("shelf", seed=4)


def test_fct_records_multipliers_in_0_1(gyre_case):
    c = gyre_case
    tape, ta = c.fct_record()
    assert np.all(tape >= 0.0) and np.all(tape <= 1.0)
    assert (tape == 1.0).mean() > 0.3 and (tape < 1.0).any()
    # replaying the tape on the state itself reproduces the forward trend exactly
    ta2 = c.fct_tl(tape, c.tsb(), c.tsn())
    assert np.array_equal(ta, ta2)


@pytest.mark.parametrize("kind", ["gyre", "shelf"])
def test_fct_dot_product(kind, gyre_case, shelf_case):
    c = gyre_case if kind == "gyre" else shelf_case
    tape, _ = c.fct_record()
    dtb, dtn, lam = c.rand4(), c.rand4(), c.rand4(masked=False)
    y = c.fct_tl(tape, dtb, dtn)
    tb_ad, tn_ad = c.fct_adj(tape, lam)
    err, lhs, _ = dot_test([(y, lam)], [(dtb, tb_ad), (dtn, tn_ad)])
    assert abs(lhs) > 0
    assert err < DOT_TOL, err


@pytest.mark.parametrize("kh,kv", [(4, 4), (4, 2), (2, 4)])
@pytest.mark.parametrize("kind", ["gyre", "shelf"])
def test_fct_fourth_order_dot_product(kind, kh, kv, gyre_case, shelf_case):
    """FCT with the 4th-order centred horizontal fluxes (traadv_fct.F90:191-227)
    and/or the compact 4th-order vertical interpolation (:517-616)."""
    c = gyre_case if kind == "gyre" else shelf_case
    tape, _ = c.fct_record(kh=kh, kv=kv)
    dtb, dtn, lam = c.rand4(), c.rand4(), c.rand4(masked=False)
    y = c.fct_tl(tape, dtb, dtn, kh=kh, kv=kv)
    tb_ad, tn_ad = c.fct_adj(tape, lam, kh=kh, kv=kv)
    err, lhs, _ = dot_test([(y, lam)], [(dtb, tb_ad), (dtn, tn_ad)])
    assert abs(lhs) > 0
    assert err < DOT_TOL, err


def test_interp_4th_cpt_dot_product(shelf_case):
    """<interp(dt), v> = <dt, interp^T v> on the interior columns, levels 2..jpk-1."""
    c = shelf_case
    rng = np.random.default_rng(7)
    jpi, jpj, jpk = c.s4[:3]
    dt = np.asfortranarray(rng.standard_normal((jpi, jpj, jpk)))
    v = np.zeros((jpi, jpj, jpk), order="F")
    v[1:-1, 1:-1, 1:-1] = rng.standard_normal((jpi - 2, jpj - 2, jpk - 2))
    y = c.o.interp_4th_cpt(dt)
    ad = np.zeros((jpi, jpj, jpk), order="F")
    c.o.interp_4th_cpt_adj(v, ad)
    lhs = (y[1:-1, 1:-1, 1:-1] * v[1:-1, 1:-1, 1:-1]).sum()
    rhs = (dt * ad).sum()
    assert abs(lhs - rhs) <= 1e-12 * (np.abs(y[1:-1, 1:-1, 1:-1] * v[1:-1, 1:-1, 1:-1]).sum()), (lhs, rhs)


def test_fct_tangent_linear_matches_finite_differences_away_from_limiter(gyre_case):
    """Perturb one wet point whose neighbourhood (3 points each way) has every
    limiter multiplier at 1: the forward is linear there, so the central
    difference equals the frozen-limiter tangent-linear. With the limiter
    inactive the upstream flux of tb cancels against the antidiffusive flux, so
    the response to tb is zero and that to tn is the centred scheme's."""
    c = gyre_case
    tape, _ = c.fct_record()
    t3 = tape.reshape((2, 3) + c.s3[::-1]).transpose(0, 1, 4, 3, 2)   # (n, face, i, j, k)
    ones = np.all(t3[0] == 1.0, axis=0)
    cand = None
    for i in range(5, c.jpi - 5):
        for j in range(5, c.jpj - 5):
            for k in range(4, c.jpk - 5):
                if c.tmask[i, j, k] and ones[i - 3:i + 4, j - 3:j + 4, k - 3:k + 4].all():
                    cand = (i, j, k)
                    break
            if cand:
                break
        if cand:
            break
    assert cand is not None, "no point with an inactive limiter neighbourhood"
    d = np.zeros(c.s4, order="F")
    d[cand + (0,)] = 1.0
    zero = np.zeros(c.s4, order="F")
    eps = 1e-4
    tb, tn = c.tsb(), c.tsn()
    scale = None
    for which in ("tn", "tb"):
        tl = c.fct_tl(tape, d if which == "tb" else zero, zero if which == "tb" else d)
        db = eps * d if which == "tb" else zero
        dn = eps * d if which == "tn" else zero
        tp, fp = c.fct_record(tb + db, tn + dn)
        tm, fm = c.fct_record(tb - db, tn - dn)
        near = (slice(cand[0] - 3, cand[0] + 4), slice(cand[1] - 3, cand[1] + 4), slice(cand[2] - 3, cand[2] + 4))
        for tt in (tp, tm):
            assert np.all(tt.reshape((2, 3) + c.s3[::-1]).transpose(0, 1, 4, 3, 2)[0][(slice(None),) + near] == 1.0)
        fd = (fp - fm) / (2 * eps)
        if which == "tn":
            scale = np.abs(tl).max()
            assert scale > 0
        else:
            assert np.abs(tl).max() <= 1e-12 * scale
        assert np.abs(fd - tl).max() <= 1e-7 * scale, (which, np.abs(fd - tl).max() / scale)


@pytest.mark.parametrize("kind", ["gyre", "shelf"])
def test_ldf_lap_dot_product(kind, gyre_case, shelf_case):
    c = gyre_case if kind == "gyre" else shelf_case
    for kpass in (1, 2):
        dtb, lam = c.rand4(), c.rand4(masked=False)
        y = np.zeros(c.s4, order="F")
        c.o.tra_ldf_lap(c.kit + 2, c.kit, "TRA", None, None, c.zero2, c.zero2, None, None, dtb, y, 2, kpass)
        tb_ad = np.zeros(c.s4, order="F")
        c.o.tra_ldf_lap_adj(c.kit + 2, c.kit, "TRA", None, None, c.gtsu, c.gtsv, None, None, tb_ad, lam, 2, kpass)
        err, lhs, _ = dot_test([(y, lam)], [(dtb, tb_ad)])
        assert abs(lhs) > 0
        assert err < DOT_TOL, (kpass, err)


@pytest.mark.parametrize("kind", ["gyre", "shelf"])
def test_ldf_iso_dot_product(kind, gyre_case, shelf_case):
    c = gyre_case if kind == "gyre" else shelf_case
    c.iso_coefficients()
    dtb, lam = c.rand4(), c.rand4(masked=False)
    y = np.zeros(c.s4, order="F")
    c.o.tra_ldf_iso(c.kit + 2, c.kit, "TRA", None, None, c.zero2, c.zero2, None, None, dtb, dtb, y, 2, 1)
    tb_ad = np.zeros(c.s4, order="F")
    c.o.tra_ldf_iso_adj(c.kit + 2, c.kit, "TRA", None, None, c.gtsu, c.gtsv, None, None, tb_ad, None, lam, 2, 1)
    err, lhs, _ = dot_test([(y, lam)], [(dtb, tb_ad)])
    assert abs(lhs) > 0
    assert err < DOT_TOL, err


def test_ldf_iso_bilaplacian_second_pass_dot_product():
    """kpass = 2 without ln_traldf_lap also reads ptbb (traldf_iso.F90:343-356)."""
    c = Case("gyre", seed=5, ln_traldf_lap=0, ln_traldf_blp=1, rn_aht_0=1.e11)
    c.iso_coefficients()
    dtb, dtbb, lam = c.rand4(), c.rand4(), c.rand4(masked=False)
    y = np.zeros(c.s4, order="F")
    c.o.tra_ldf_iso(c.kit + 2, c.kit, "TRA", None, None, c.zero2, c.zero2, None, None, dtb, dtbb, y, 2, 2)
    tb_ad = np.zeros(c.s4, order="F")
    tbb_ad = np.zeros(c.s4, order="F")
    c.o.tra_ldf_iso_adj(c.kit + 2, c.kit, "TRA", None, None, c.zero2, c.zero2, None, None, tb_ad, tbb_ad, lam, 2, 2)
    err, lhs, _ = dot_test([(y, lam)], [(dtb, tb_ad), (dtbb, tbb_ad)])
    assert abs(lhs) > 0 and np.abs(tbb_ad).max() > 0
    assert err < DOT_TOL, err


@pytest.mark.parametrize("kind", ["gyre", "shelf"])
def test_zdf_imp_dot_product(kind, gyre_case, shelf_case):
    c = gyre_case if kind == "gyre" else shelf_case
    c.iso_coefficients()
    dtb, dta, lam = c.rand4(), c.rand4(masked=False), c.rand4(masked=False)
    y = dta.copy(order="F")
    c.o.tra_zdf_imp(c.kit + 2, c.kit, "TRA", c.p2dt, dtb, y, 2)
    tb_ad = np.zeros(c.s4, order="F")
    ta_ad = lam.copy(order="F")
    c.o.tra_zdf_imp_adj(c.kit + 2, c.kit, "TRA", c.p2dt, tb_ad, ta_ad, 2)
    err, lhs, _ = dot_test([(y, lam)], [(dtb, tb_ad), (dta, ta_ad)])
    assert abs(lhs) > 0
    assert err < DOT_TOL, err


@pytest.mark.parametrize("euler", [True, False])
def test_tra_nxt_dot_product(euler):
    c = Case("gyre", seed=6, neuler=0 if euler else 1)
    kt = c.kit if euler else c.kit + 3
    xb, xn, xa = c.rand4(False), c.rand4(False), c.rand4(False)
    yb, yn, ya = xb.copy(order="F"), xn.copy(order="F"), xa.copy(order="F")
    c.bind("TSB", yb)
    c.bind("TSN", yn)
    c.bind("TSA", ya)
    c.o.tra_nxt(kt)
    lb, ln, la = c.rand4(False), c.rand4(False), c.rand4(False)
    ab, an, aa = lb.copy(order="F"), ln.copy(order="F"), la.copy(order="F")
    c.o.tra_nxt_adj(kt, ab, an, aa)
    err, lhs, _ = dot_test([(yb, lb), (yn, ln), (ya, la)], [(xb, ab), (xn, an), (xa, aa)])
    assert abs(lhs) > 0
    assert err < DOT_TOL, err


def test_tra_nxt_leapfrog_known_answer():
    """Interior: tb <- tn + atfp (ta - 2 tn + tb), tn <- ta; edges zeroed."""
    c = Case("gyre", seed=7)
    tb, tn, ta = c.rand4(False), c.rand4(False), c.rand4(False)
    b, n, a = tb.copy(order="F"), tn.copy(order="F"), ta.copy(order="F")
    c.bind("TSB", b)
    c.bind("TSN", n)
    c.bind("TSA", a)
    c.o.tra_nxt(c.kit + 3)
    atfp = c.nam["rn_atfp"]
    I = (slice(1, -1), slice(1, -1), slice(0, -1))
    assert np.array_equal(n[I], ta[I])
    exp = tn[I] + atfp * (ta[I] - 2.0 * tn[I] + tb[I])
    assert np.abs(b[I] - exp).max() <= 1e-15 * np.abs(exp).max()
    assert not b[0].any() and not n[:, -1].any() and not a[-1].any()
