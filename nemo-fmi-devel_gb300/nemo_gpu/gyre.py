"""Synthetic GYRE inputs: the analytic GYRE configuration of the reference plus
seeded noise, standing in for a model state (the reference ships no data files).

Formulas restated from the reference's user-defined GYRE configuration:
grid and Coriolis parameter from src/OCE/USR/usrdef_hgr.F90:85-165, vertical levels
from usrdef_zgr.F90:94-176 with DOM/depth_e3.F90 (depth_to_e3 / e3_to_depth), the
closed flat-bottom basin from usrdef_zgr.F90:179-210, initial T/S from
usrdef_istate.F90:64-78, wind stress and E-P from usrdef_sbc.F90:90-188, the
constant eddy diffusivity aht0 = 1/2 Ud Ld from LDF/ldftra.F90:296-299 and the
non-linear bottom drag from ZDF/zdfdrg.F90:126-136. Namelist values follow
cfgs/GYRE_PISCES/EXPREF/namelist_cfg on top of cfgs/SHARED/namelist_ref.

Velocities, slopes, vertical diffusivity and the momentum trend are synthetic:
a surface-intensified double-gyre from a streamfunction plus seeded noise, with w
from continuity, so that the flow is realistic in size and structure.

All arrays are numpy float64 in Fortran order (jpi,jpj[,jpk][,2]); an ensemble
stacks members along a trailing axis (member outermost in memory).
"""
import math

import numpy as np

RA, RAD, OMEGA, GRAV, RAU0 = 6371229.0, math.pi / 180.0, 7.292116e-05, 9.80665, 1026.0
RCP = 3991.86795711963   # specific heat of sea water (eosbn2.F90:1245)


def namelist(**over):
    """Namelist subset for GYRE (namelist_cfg over namelist_ref)."""
    nam = dict(
        rn_rdt=7200.0, rn_atfp=0.1, nit000=1, neuler=1, ln_linssh=1, ln_zps=0, ln_isfcav=0,
        ln_traldf_lap=1, ln_traldf_blp=0, ln_traldf_iso=1, ln_traldf_msc=0,
        rn_aht_0=(0.5 * 0.02) * 100.0e3, ln_zdfddm=0, ln_zad_Aimp=0,
        ln_bt_fw=1, ln_bt_av=1, nn_bt_flt=1, ln_bt_auto=1, nn_baro=30, rn_bt_cmax=0.8, rn_bt_alpha=0.0,
        nvor_scheme=1, nn_een_e3f=0, ln_dynadv_vec=1, ln_sco=0, ln_apr_dyn=0, rn_scal_load=0.0,
        grav=GRAV, rau0=RAU0, nn_fct_h=2, nn_fct_v=2, rn_slpmax=0.01,
        ln_traqsr=1, rn_abs=0.58, rn_si0=0.35, rn_si1=23.0, rcp=RCP,
        # GYRE's namelist_cfg selects EOS-80 (ln_eos80 = 1 below for a GYRE run); the
        # simplified eos of namelist_ref &nameos is the alternative
        ln_seos=0, rn_a0=1.6550e-1, rn_b0=7.6554e-1, rn_lambda1=5.9520e-2, rn_lambda2=7.4914e-4,
        rn_mu1=1.4970e-4, rn_mu2=1.1090e-5, rn_nu=2.4341e-3, ln_eos80=0)
    nam.update(over)
    return nam


def zgr_z(jpk):
    """1-D GYRE levels (usrdef_zgr.F90:134-165 and depth_e3.F90)."""
    zsur, za0, za1, zkth, zacr = -2033.194295283385, 155.8325369664153, 146.3615918601890, 17.28520372419791, 5.0
    k = np.arange(1, jpk + 1, dtype=np.float64)
    depw = zsur + za0 * k + za1 * zacr * np.log(np.cosh((k - zkth) / zacr))
    dept = zsur + za0 * (k + 0.5) + za1 * zacr * np.log(np.cosh((k + 0.5 - zkth) / zacr))
    e3w = np.empty(jpk)
    e3t = np.empty(jpk)
    e3w[0] = 2.0 * (dept[0] - depw[0])
    e3w[1:] = dept[1:] - dept[:-1]
    e3t[:-1] = depw[1:] - depw[:-1]
    e3t[-1] = 2.0 * (dept[-1] - depw[-1])
    depw2 = np.empty(jpk)
    dept2 = np.empty(jpk)
    depw2[0] = 0.0
    dept2[0] = 0.5 * e3w[0]
    for j in range(1, jpk):
        depw2[j] = depw2[j - 1] + e3t[j - 1]
        dept2[j] = dept2[j - 1] + e3w[j]
    return dept2, depw2, e3t, e3w


def domain(nn_gyre, jpk=31, ln_bench=True):
    """GYRE domain: jpi = 30 nn_GYRE + 2, jpj = 20 nn_GYRE + 2 (usrdef_nam.F90:76-77)."""
    jpi, jpj = 30 * nn_gyre + 2, 20 * nn_gyre + 2
    ze1 = 106000.0 / nn_gyre
    zsin, zcos = -math.sqrt(2.0) * 0.5, math.sqrt(2.0) * 0.5
    ze1deg = ze1 / (RA * RAD)
    zlam1, zphi1 = -85.0, 29.0
    zphi0 = zphi1 + zsin * ze1deg * (jpj - 2)
    if ln_bench:
        ze1 = 106000.0
    ii = np.arange(1, jpi + 1, dtype=np.float64)[:, None]
    jj = np.arange(1, jpj + 1, dtype=np.float64)[None, :]
    gphit = zphi0 - (ii - 1.5) * ze1deg * zsin + (jj - 1.5) * ze1deg * zcos
    gphiu = zphi0 - (ii - 1.0) * ze1deg * zsin + (jj - 1.5) * ze1deg * zcos
    gphiv = zphi0 - (ii - 1.5) * ze1deg * zsin + (jj - 1.0) * ze1deg * zcos
    gphif = zphi0 - (ii - 1.0) * ze1deg * zsin + (jj - 1.0) * ze1deg * zcos
    zbeta = 2.0 * OMEGA * math.cos(RAD * zphi1) / RA
    zf0 = 2.0 * OMEGA * math.sin(RAD * 15.0)
    ff_f = zf0 + zbeta * np.abs(gphif - 15.0) * RAD * RA
    ff_t = zf0 + zbeta * np.abs(gphit - 15.0) * RAD * RA
    e1 = np.full((jpi, jpj), ze1, order="F")
    dept, depw, e3t1, e3w1 = zgr_z(jpk)
    def lev(p):
        return np.asfortranarray(np.broadcast_to(p[None, None, :], (jpi, jpj, jpk)).copy())
    kb = np.full((jpi, jpj), jpk - 1, dtype=np.int32)
    kb[0, :] = kb[-1, :] = 0
    kb[:, 0] = kb[:, -1] = 0
    kt = np.minimum(1, kb).astype(np.int32)
    dom = dict(jpi=jpi, jpj=jpj, jpk=jpk, jperio=0,
               e1t=e1, e2t=e1.copy(order="F"), e1u=e1.copy(order="F"), e2u=e1.copy(order="F"),
               e1v=e1.copy(order="F"), e2v=e1.copy(order="F"), e1f=e1.copy(order="F"), e2f=e1.copy(order="F"),
               ff_f=np.asfortranarray(ff_f), ff_t=np.asfortranarray(ff_t),
               k_top=np.asfortranarray(kt), k_bot=np.asfortranarray(kb),
               e3t_0=lev(e3t1), e3u_0=lev(e3t1), e3v_0=lev(e3t1), e3w_0=lev(e3w1), e3f_0=lev(e3t1),
               gdept_1d=dept, gphit=gphit, gphiu=gphiu, gphiv=gphiv)
    return dom


def masks(dom):
    """tmask, umask, vmask, wmask (float64, Fortran order) as dommsk.F90 builds them."""
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    k = np.arange(1, jpk + 1)[None, None, :]
    kt, kb = dom["k_top"][:, :, None], dom["k_bot"][:, :, None]
    t = ((kt != 0) & (k >= kt) & (k <= kb)).astype(np.float64)
    t[0], t[-1], t[:, 0], t[:, -1] = 0, 0, 0, 0
    u = np.zeros_like(t)
    v = np.zeros_like(t)
    u[:-1, :-1] = t[:-1, :-1] * t[1:, :-1]
    v[:-1, :-1] = t[:-1, :-1] * t[:-1, 1:]
    u[0], u[:, 0], v[0], v[:, 0] = 0, 0, 0, 0
    w = t.copy()
    w[:, :, 1:] = t[:, :, 1:] * t[:, :, :-1]
    f = lambda a: np.asfortranarray(a)
    return f(t), f(u), f(v), f(w)


def _istate(dept):
    """Analytic T and S profiles (usrdef_istate.F90:64-78)."""
    d = dept
    t = ((16. - 12. * np.tanh((d - 400) / 700)) * (-np.tanh((500. - d) / 150.) + 1.) / 2.
         + (15. * (1. - np.tanh((d - 50.) / 1500.)) - 1.4 * np.tanh((d - 100.) / 100.)
            + 7. * (1500. - d) / 1500.) * (-np.tanh((d - 500.) / 150.) + 1.) / 2.)
    s = ((36.25 - 1.13 * np.tanh((d - 305) / 460)) * (-np.tanh((500. - d) / 150.) + 1.) / 2
         + (35.55 + 1.25 * (5000. - d) / 5000. - 1.62 * np.tanh((d - 60.) / 650.)
            + 0.2 * np.tanh((d - 35.) / 100.) + 0.2 * np.tanh((d - 1000.) / 5000.))
         * (-np.tanh((d - 500.) / 150.) + 1.) / 2)
    return t, s


def _smooth(rng, shape, passes=2):
    a = rng.standard_normal(shape)
    for _ in range(passes):
        a[1:-1, 1:-1] = 0.25 * (a[2:, 1:-1] + a[:-2, 1:-1] + a[1:-1, 2:] + a[1:-1, :-2])
    return a


def state(dom, nam, seed=0, noise_t=0.05, noise_s=0.01, u0=0.5, member=0, noise_u=0.03):
    """Seeded synthetic state (one member) on a GYRE domain."""
    rng = np.random.default_rng([seed, member])
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    tm, um, vm, wm = masks(dom)
    e3t = dom["e3t_0"]
    e1, e2 = dom["e1u"], dom["e2v"]
    t1, s1 = _istate(dom["gdept_1d"])
    ts = np.zeros((jpi, jpj, jpk, 2), order="F")
    ts[..., 0] = (t1[None, None, :] + noise_t * rng.standard_normal((jpi, jpj, jpk))) * tm
    ts[..., 1] = (s1[None, None, :] + noise_s * rng.standard_normal((jpi, jpj, jpk))) * tm
    tsn = ts.copy(order="F")
    tsn[..., 0] += 0.01 * rng.standard_normal((jpi, jpj, jpk)) * tm
    tsn[..., 1] += 0.002 * rng.standard_normal((jpi, jpj, jpk)) * tm
    # double gyre streamfunction at f-points, zero on the closed boundary
    x = (np.arange(1, jpi + 1) - 1.0) / (jpi - 2)
    y = (np.arange(1, jpj + 1) - 1.0) / (jpj - 2)
    psi = np.sin(np.pi * np.clip(x, 0, 1))[:, None] * np.sin(2 * np.pi * np.clip(y, 0, 1))[None, :]
    psi[-1, :] = 0
    psi[:, -1] = 0
    psi = psi * u0 * e1.mean() * (jpj - 2) / (2 * np.pi)
    ubt = np.zeros((jpi, jpj))
    vbt = np.zeros((jpi, jpj))
    ubt[:, 1:] = -(psi[:, 1:] - psi[:, :-1]) / e2[:, 1:]
    vbt[1:, :] = (psi[1:, :] - psi[:-1, :]) / e1[1:, :]
    prof = np.exp(-dom["gdept_1d"] / 600.0)
    un = ubt[:, :, None] * prof[None, None, :] + noise_u * rng.standard_normal((jpi, jpj, jpk))
    vn = vbt[:, :, None] * prof[None, None, :] + noise_u * rng.standard_normal((jpi, jpj, jpk))
    un, vn = np.asfortranarray(un * um), np.asfortranarray(vn * vm)
    # w from continuity (sshwzv.F90 wzv, linear free surface)
    e2u, e1v, e1e2t = dom["e2u"], dom["e1v"], dom["e1t"] * dom["e2t"]
    fu = e2u[:, :, None] * dom["e3u_0"] * un
    fv = e1v[:, :, None] * dom["e3v_0"] * vn
    hdiv = np.zeros((jpi, jpj, jpk))
    hdiv[1:-1, 1:-1, :] = (fu[1:-1, 1:-1] - fu[:-2, 1:-1] + fv[1:-1, 1:-1] - fv[1:-1, :-2]) / (
        e1e2t[1:-1, 1:-1, None] * e3t[1:-1, 1:-1])
    wn = np.zeros((jpi, jpj, jpk), order="F")
    for k in range(jpk - 2, -1, -1):
        wn[:, :, k] = wn[:, :, k + 1] - e3t[:, :, k] * hdiv[:, :, k] * tm[:, :, k]
    ub = np.asfortranarray((un + 0.01 * rng.standard_normal(un.shape)) * um)
    vb = np.asfortranarray((vn + 0.01 * rng.standard_normal(vn.shape)) * vm)
    ua = np.asfortranarray(1.0e-6 * rng.standard_normal(un.shape) * um)
    va = np.asfortranarray(1.0e-6 * rng.standard_normal(vn.shape) * vm)
    hu = (dom["e3u_0"] * um).sum(axis=2)
    hv = (dom["e3v_0"] * vm).sum(axis=2)
    r1hu = np.where(hu > 0, 1.0 / np.where(hu > 0, hu, 1.0), 0.0)
    r1hv = np.where(hv > 0, 1.0 / np.where(hv > 0, hv, 1.0), 0.0)
    def bt(u, e3, m, r1h):
        return np.asfortranarray((e3 * u * m).sum(axis=2) * r1h)
    un_b, vn_b = bt(un, dom["e3u_0"], um, r1hu), bt(vn, dom["e3v_0"], vm, r1hv)
    ub_b, vb_b = bt(ub, dom["e3u_0"], um, r1hu), bt(vb, dom["e3v_0"], vm, r1hv)
    sshn = np.asfortranarray(0.3 * _smooth(rng, (jpi, jpj), 4) * tm[:, :, 0])
    sshb = np.asfortranarray((sshn + 0.01 * rng.standard_normal((jpi, jpj))) * tm[:, :, 0])
    # wind stress (usrdef_sbc.F90:160-172 at the first day) and E-P (:107-139)
    ztau = 0.105 / math.sqrt(2.0)
    ztaun = ztau - 0.015 * math.cos((1.0 * nam["rn_rdt"] / 3600.0 - 171 * 24) / (180 * 24) * math.pi)
    utau = np.asfortranarray(-ztaun * np.sin(math.pi * (dom["gphiu"] - 15.) / (29. - 15.)))
    vtau = np.asfortranarray(ztaun * np.sin(math.pi * (dom["gphiv"] - 15.) / (29. - 15.)))
    g = dom["gphit"]
    emp = np.where((g >= 14.845) & (g <= 37.2),
                   0.7 * 3.16e-5 * np.sin(math.pi / 2 * (g - 37.2) / (24.6 - 37.2)),
                   -0.8 * 3.16e-5 * np.sin(math.pi / 2 * (g - 37.2) / (46.8 - 37.2))) * tm[:, :, 0]
    wet = tm[:, :, 0] > 0
    emp = np.asfortranarray(emp - emp[wet].mean() * tm[:, :, 0])
    # bottom drag coefficient * |U| at t-points, negative (zdfdrg.F90:126-136)
    kbot = np.maximum(dom["k_bot"], 1) - 1
    ubot = np.take_along_axis(ub, kbot[:, :, None], axis=2)[:, :, 0]
    vbot = np.take_along_axis(vb, kbot[:, :, None], axis=2)[:, :, 0]
    zut = ubot + np.roll(ubot, 1, axis=0)
    zvt = vbot + np.roll(vbot, 1, axis=1)
    rcdu = np.asfortranarray(-1.e-3 * np.sqrt(0.25 * (zut * zut + zvt * zvt) + 2.5e-3) * tm[:, :, 0])
    # vertical diffusivity: background 1.2e-5 + mixed layer + a few convective columns
    avt = 1.2e-5 + 1e-3 * np.exp(-dom["gdept_1d"] / 50.0)[None, None, :] * (1 + rng.random((jpi, jpj, jpk)))
    conv = rng.random((jpi, jpj)) < 0.02
    avt = avt + np.where(conv[:, :, None], 10.0, 0.0) * (dom["gdept_1d"] < 300)[None, None, :]
    avt = avt * wm
    avt[:, :, 0] = 0.0
    avt[:, :, -1] = 0.0
    avt = np.asfortranarray(avt)
    # iso-neutral slopes, |slope| <= rn_slpmax = 0.01
    def slope(m):
        a = 0.004 * rng.standard_normal((jpi, jpj, jpk))
        return np.asfortranarray(np.clip(a, -0.01, 0.01) * m)
    uslp, vslp, wslpi, wslpj = slope(um), slope(vm), slope(wm), slope(wm)
    # ldf_slp writes levels 2..jpk-1 only: the surface slopes stay at their initial 0
    # (ldf_slp_init), and a model step that forms the slopes keeps them there
    for a in (uslp, vslp, wslpi, wslpj):
        a[:, :, 0] = 0.0
    # restart fields of a run in progress (dynspg_ts.F90:1214-1227): the half-step
    # transports of the previous step, close to the now barotropic transports
    ub2_b, vb2_b = np.asfortranarray(un_b * hu), np.asfortranarray(vn_b * hv)
    return dict(tsb=ts, tsn=tsn, un=un, vn=vn, wn=wn, ub=ub, vb=vb, ua=ua, va=va,
                un_b=un_b, vn_b=vn_b, ub_b=ub_b, vb_b=vb_b, sshn=sshn, sshb=sshb, ub2_b=ub2_b, vb2_b=vb2_b,
                utau=utau, vtau=vtau, emp=emp, rcdu_bot=rcdu, avt=avt,
                uslp=uslp, vslp=vslp, wslpi=wslpi, wslpj=wslpj)


def zstar(dom, st, ssha=None):
    """Variable-volume (z*) scale factors and depths of a state: the fields
    domvvl.F90 maintains when ln_linssh = .false. -- e3t = e3t_0 (ht_0 + ssh) /
    (ht_0 + 1 - ssmask) on wet levels (:849-851), e3u/e3v/e3f/e3w interpolated from
    the e3t changes as dom_vvl_interpol does, column depths and their masked
    inverses (:183-196). Before / now / after levels use sshb, sshn and ssha (by
    default the linear extrapolation sshn + (sshn - sshb))."""
    tm, um, vm, wm = masks(dom)
    e1e2t = dom["e1t"] * dom["e2t"]
    e1e2u = dom["e1u"] * dom["e2u"]
    e1e2f = dom["e1f"] * dom["e2f"]
    ssmask = tm.max(axis=2)
    ssumask = um.max(axis=2)
    ssvmask = vm.max(axis=2)
    ht_0 = (dom["e3t_0"] * tm).sum(axis=2)
    f = np.asfortranarray

    def e3t_of(ssh):
        s = (ht_0 + ssh) / (ht_0 + 1.0 - ssmask)
        return f(dom["e3t_0"] * s[:, :, None] * tm + dom["e3t_0"] * (1.0 - tm))

    def to_u(e3t):
        d = e1e2t[:, :, None] * (e3t - dom["e3t_0"])
        out = dom["e3u_0"].copy()
        out[:-1] += um[:-1] * 0.5 * (d[:-1] + d[1:]) / e1e2u[:-1, :, None]
        return f(out)

    def to_v(e3t):
        d = e1e2t[:, :, None] * (e3t - dom["e3t_0"])
        e1e2v = dom["e1v"] * dom["e2v"]
        out = dom["e3v_0"].copy()
        out[:, :-1] += vm[:, :-1] * 0.5 * (d[:, :-1] + d[:, 1:]) / e1e2v[:, :-1, None]
        return f(out)

    def to_f(e3u):
        d = e1e2u[:, :, None] * (e3u - dom["e3u_0"])
        out = dom["e3f_0"].copy()
        out[:, :-1] += um[:, :-1] * um[:, 1:] * 0.5 * (d[:, :-1] + d[:, 1:]) / e1e2f[:, :-1, None]
        return f(out)

    def to_w(e3t):
        d = e3t - dom["e3t_0"]
        out = dom["e3w_0"].copy()
        out[:, :, 0] += d[:, :, 0]
        out[:, :, 1:] += (1.0 - 0.5 * tm[:, :, 1:]) * d[:, :, :-1] + 0.5 * tm[:, :, 1:] * d[:, :, 1:]
        return f(out)

    def inv(h, m):
        return f(m / (h + 1.0 - m))

    if ssha is None:
        ssha = (st["sshn"] + (st["sshn"] - st["sshb"])) * ssmask
    e3t_b, e3t_n, e3t_a = e3t_of(st["sshb"]), e3t_of(st["sshn"]), e3t_of(ssha)
    e3u_b, e3u_n, e3v_b, e3v_n = to_u(e3t_b), to_u(e3t_n), to_v(e3t_b), to_v(e3t_n)
    hu_b, hu_n = f((e3u_b * um)[:, :, :-1].sum(axis=2)), f((e3u_n * um)[:, :, :-1].sum(axis=2))
    hv_b, hv_n = f((e3v_b * vm)[:, :, :-1].sum(axis=2)), f((e3v_n * vm)[:, :, :-1].sum(axis=2))
    return dict(e3t_b=e3t_b, e3t_n=e3t_n, e3t_a=e3t_a, e3u_n=e3u_n, e3v_n=e3v_n, e3w_n=to_w(e3t_n),
                e3f_n=to_f(e3u_n), ht_n=f((e3t_n * tm)[:, :, :-1].sum(axis=2)),
                hu_n=hu_n, hv_n=hv_n, r1_hu_n=inv(hu_n, ssumask), r1_hv_n=inv(hv_n, ssvmask),
                hu_b=hu_b, hv_b=hv_b, r1_hu_b=inv(hu_b, ssumask), r1_hv_b=inv(hv_b, ssvmask))


def slope_inputs(dom, nam, st, rho_c=0.01):
    """Inputs of ldf_slp from a state: the in situ density anomaly of a linear
    equation of state (rn_a0 = 1.655e-1, rn_b0 = 7.6554e-1 of eosbn2's linear case),
    N^2 from it, the mixed layer of zdf_mxl (zdfmxl.F90:92-122, rho_c = 0.01) and the
    rest-state depths of the T- and W-points."""
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    tm, _, _, wm = masks(dom)
    ts = st["tsn"]
    rhd = (-1.655e-1 * (ts[..., 0] - 10.0) + 7.6554e-1 * (ts[..., 1] - 35.0)) / nam["rau0"] * tm
    e3t, e3w = dom["e3t_0"], dom["e3w_0"]
    rn2 = np.zeros_like(rhd)
    rn2[:, :, 1:-1] = nam["grav"] * (rhd[:, :, 1:-1] - rhd[:, :, :-2]) / e3w[:, :, 1:-1] * wm[:, :, 1:-1]
    gdepw = np.zeros_like(e3t)
    gdepw[:, :, 1:] = np.cumsum(e3t[:, :, :-1], axis=2)
    gdept = gdepw + 0.5 * e3t if "gdept_1d" not in dom else np.broadcast_to(dom["gdept_1d"], e3t.shape).copy()
    n2c = nam["grav"] * rho_c / nam["rau0"]
    nlb10 = 1 + int((gdepw[1, 1, :] < 10.0).sum())          # 1-based level below 10 m
    mbkt = dom["k_bot"]
    nmln = np.full((jpi, jpj), nlb10, dtype=np.int32)
    h = np.zeros((jpi, jpj))
    for jk in range(nlb10, jpk):                            # 1-based jk = nlb10 .. jpk-1
        h += np.maximum(rn2[:, :, jk - 1], 0.0) * e3w[:, :, jk - 1]
        nmln = np.where(h < n2c, np.minimum(jk, mbkt) + 1, nmln).astype(np.int32)
    ssm = tm.max(axis=2)
    ii, jj = np.meshgrid(np.arange(jpi), np.arange(jpj), indexing="ij")
    hmlp = gdepw[ii, jj, nmln - 1] * ssm
    hmlpt = gdept[ii, jj, np.maximum(nmln - 2, 0)] * ssm
    f = np.asfortranarray
    return dict(rhd=f(rhd), rn2b=f(rn2), nmln=f(nmln.astype(np.int32)), hmlp=f(hmlp), hmlpt=f(hmlpt),
                gdept_n=f(gdept), gdepw_n=f(gdepw))


def sbc_inputs(dom, nam, st, kt=1):
    """Surface heat and salt forcing of tra_sbc / tra_qsr at time step kt, from the
    GYRE analytic fluxes (usrdef_sbc.F90:90-151, year 1 starting on January 1st, 360-day
    year): qsr, and qns with the -40 W/m2/K restoring to the seasonal T* computed from
    the before SST and the sensible heat of E-P at the SST (sst_m = the now SST); sfx
    = 0. Also the rest-state depths of the W-points (gdepw_n) that tra_qsr reads, and
    zeroed restart fields sbc_tsc, sbc_tsc_b (jpi,jpj,2), qsr_hc, qsr_hc_b."""
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    g = dom["gphit"]
    ztime = kt * nam["rn_rdt"] / 3600.0                       # hours since January 1st
    tmax1 = (5 * 30 + 21) * 24.0
    tmin1 = tmax1 + 24.0 * 360 / 2
    tmax2 = (6 * 30 + 21) * 24.0
    tmin2 = tmax2 - 24.0 * 360 / 2
    c1 = math.cos((ztime - tmax1) / (tmin1 - tmax1) * math.pi)
    c2 = math.cos((ztime - tmax2) / (tmax2 - tmin2) * math.pi)
    t_star = 28.3 * (1.0 + c2 / 50.0) * np.cos(math.pi * (g - 5.0) / (53.5 * (1 + 11 / 53.5 * c2) * 2.0))
    qsr = 230.0 * np.cos(3.1415 * (g - 23.5 * c1) / (0.9 * 180))
    qns = -40.0 * (st["tsb"][:, :, 0, 0] - t_star) - qsr
    qns = qns - st["emp"] * st["tsn"][:, :, 0, 0] * RCP
    e3t = dom["e3t_0"]
    gdepw = np.zeros_like(e3t)
    gdepw[:, :, 1:] = np.cumsum(e3t[:, :, :-1], axis=2)         # e3_to_depth (depth_e3.F90)
    f = np.asfortranarray
    return dict(qsr=f(qsr * 1.0), qns=f(qns), sfx=f(np.zeros((jpi, jpj))), gdepw_n=f(gdepw),
                sbc_tsc=f(np.zeros((jpi, jpj, 2))), sbc_tsc_b=f(np.zeros((jpi, jpj, 2))),
                qsr_hc=f(np.zeros((jpi, jpj, jpk))), qsr_hc_b=f(np.zeros((jpi, jpj, jpk))),
                fraqsr_1lev=f(np.ones((jpi, jpj))))


def vphys_inputs(dom, nam, st):
    """Inputs of zdf_phy with the TKE closure for a state: the wind-stress modulus at
    T-points from the state's utau, vtau (usrdef_sbc.F90:176-186, interior points,
    zero on the closed edges) and the cold start of the closure (zdf_phy_init and
    tke_rst, zdftke.F90:778-783): en = rn_emin wmask, dissl = 1e-12, avm_k = rn_avm0
    wmask, avt_k = rn_avt0 wmask, avm = avs = 0; rn2 is formed by the step (zeros)."""
    from ._ffi import NAMELIST_DEFAULTS
    nam = {**NAMELIST_DEFAULTS, **nam}
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    wm = masks(dom)[3]
    ut, vt = st["utau"], st["vtau"]
    taum = np.zeros((jpi, jpj))
    ztx = ut[:-2, 1:-1] + ut[1:-1, 1:-1]
    zty = vt[1:-1, :-2] + vt[1:-1, 1:-1]
    taum[1:-1, 1:-1] = 0.5 * np.sqrt(ztx * ztx + zty * zty)
    f = np.asfortranarray
    z3 = lambda: f(np.zeros((jpi, jpj, jpk)))
    return dict(taum=f(taum), en=f(nam["rn_emin"] * wm), dissl=f(np.full((jpi, jpj, jpk), 1.e-12)),
                avm_k=f(nam["rn_avm0"] * wm), avt_k=f(nam["rn_avt0"] * wm), avm=z3(), avs=z3(), rn2=z3())


def viscosity(dom, ahm0=1.0e5):
    """The lateral eddy viscosity of GYRE's &namdyn_ldf (laplacian, iso-level,
    nn_ahm_ijk_t = 0: 1/2 rn_Uv rn_Lv = 1/2 x 2 m/s x 100 km = 1e5 m2/s, ldfdyn.F90:
    248-259): ahmt = ahm0 tmask, ahmf = ahm0 fmask, fmask of the free-slip coast
    (rn_shlat = 0) from the four surrounding T-points; level jpk is 0."""
    tm = masks(dom)[0]
    fm = np.zeros_like(tm)
    fm[:-1, :-1] = tm[:-1, :-1] * tm[1:, :-1] * tm[:-1, 1:] * tm[1:, 1:]
    ahmt, ahmf = ahm0 * tm, ahm0 * fm
    ahmt[:, :, -1] = 0.0
    ahmf[:, :, -1] = 0.0
    return np.asfortranarray(ahmt), np.asfortranarray(ahmf)


# GYRE's physics (cfgs/GYRE_PISCES/EXPREF/namelist_cfg): the analytic surface forcing
# formed every step, EOS-80, the TKE closure with enhanced vertical diffusion, the
# penetrating solar flux
FULL_NAMELIST = dict(ln_usr=1, ln_eos80=1, ln_seos=0, ln_zdftke=1, ln_zdfevd=1, ln_traqsr=1)
# the fields of the full step besides the hot path's (3-D, then 2-D; nmln is int32)
FULL_3D = ("en", "dissl", "avm_k", "avt_k", "avm", "avs", "rn2", "rn2b", "rhd", "rhop", "gdept_n", "gdepw_n",
           "qsr_hc", "qsr_hc_b", "ahmt", "ahmf")
FULL_2D = ("taum", "qsr", "qns", "sfx", "fraqsr_1lev", "hmlp", "hmlpt", "sbc_tsc", "sbc_tsc_b", "gphit", "gphiu",
           "gphiv", "utau_b", "vtau_b")


def full_physics(dom, nam, st):
    """The namelist and the state of the full GYRE step from a state of state(): the
    latitudes the analytic forcing reads (the step forms the forcing itself;
    sbc_inputs gives the first values and the restart fields of tra_sbc / tra_qsr),
    the cold start of the TKE closure (vphys_inputs), the rest-state depths, the
    lateral viscosity, and zeroed rn2b, rhd, rhop, mixed-layer fields (the step forms
    them)."""
    nam = dict(nam, **FULL_NAMELIST)
    ahmt, ahmf = viscosity(dom)
    st = dict(st)
    st.update(sbc_inputs(dom, nam, st, kt=1))
    st.update(vphys_inputs(dom, nam, st))
    sl = slope_inputs(dom, nam, st)
    z3, z2 = np.zeros_like(st["avt"]), np.zeros_like(st["sshn"])
    st.update(gdept_n=sl["gdept_n"], rn2b=z3, rhd=z3.copy(), rhop=z3.copy(), ahmt=ahmt, ahmf=ahmf, hmlp=z2,
              hmlpt=z2.copy(), nmln=np.zeros(z2.shape, dtype=np.int32, order="F"),
              gphit=np.asfortranarray(dom["gphit"]), gphiu=np.asfortranarray(dom["gphiu"]),
              gphiv=np.asfortranarray(dom["gphiv"]), utau_b=np.array(st["utau"], order="F"),
              vtau_b=np.array(st["vtau"], order="F"))
    return nam, st
