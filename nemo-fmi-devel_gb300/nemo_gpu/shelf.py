"""Synthetic shelf configuration: a regional z* model on a shallow shelf, standing
in for a configuration whose input files do not exist here.

* Bathymetry: lognormal depths between 10 and 400 m, smoothed by a 5-cell box
  filter; land where the depth is below 10 m and on the closed frame.
* Vertical grid: jpk = 56 levels over 0-420 m, 2.3 m at the surface growing to
  9.8 m at depth, with
  partial bottom cells (ln_zps) built as the reference's zgr_zps does
  (tools/DOMAINcfg/src/domzgr.f90:1040-1100): the bottom cell's e3t / e3w scale with
  the part of the level above the bathymetry, and e3u / e3v / e3f are the minima of
  the neighbouring e3t / e3u.
* Horizontal grid: 1 km cells on a beta-plane from 45 N; Coriolis from the latitude.
* Namelist: z* variable volume, FCT 4/4 (compact vertical interpolation), laplacian
  iso-neutral diffusion with partial-step bottom gradients, EEN vorticity, flux-form
  momentum, atmospheric pressure forcing, rdt = 300 s, nn_baro = 30 fixed.

The domain dict has the keys of gyre.domain(), so gyre.state() and gyre.zstar()
build states on it unchanged.
"""
import math

import numpy as np

from . import gyre


def namelist(**over):
    nam = gyre.namelist(rn_rdt=300.0, ln_linssh=0, ln_zps=1, ln_traldf_lap=1, ln_traldf_iso=1,
                        rn_aht_0=100.0, ln_bt_auto=0, nn_baro=30, nvor_scheme=4, nn_een_e3f=1,
                        ln_dynadv_vec=0, ln_apr_dyn=1, nn_fct_h=4, nn_fct_v=4)
    nam.update(over)
    return nam


def _levels(jpk, hmax=420.0, stretch=1.3):
    """1-D depths of the w- and t-levels and the level thicknesses."""
    k = np.arange(1, jpk + 1, dtype=np.float64)
    depw = hmax * ((k - 1.0) / (jpk - 1.0)) ** stretch
    dept = hmax * ((k - 0.5) / (jpk - 1.0)) ** stretch
    e3t = np.empty(jpk)
    e3t[:-1] = depw[1:] - depw[:-1]
    e3t[-1] = e3t[-2]
    e3w = np.empty(jpk)
    e3w[0] = 2.0 * (dept[0] - depw[0])
    e3w[1:] = dept[1:] - dept[:-1]
    return dept, depw, e3t, e3w


def domain(jpi=1000, jpj=1200, jpk=56, seed=0, e1=1000.0):
    rng = np.random.default_rng([seed, 77])
    # bathymetry: lognormal, 5-cell box smoothing, clipped to 10-400 m
    z = rng.standard_normal((jpi, jpj))
    bathy = np.exp(math.log(60.0) + 0.9 * z)
    pad = np.pad(bathy, 2, mode="edge")
    sm = np.zeros_like(bathy)
    for di in range(5):
        for dj in range(5):
            sm += pad[di:di + jpi, dj:dj + jpj]
    bathy = np.clip(sm / 25.0, 0.0, 400.0)
    dept, depw, e3t1, e3w1 = _levels(jpk)
    land = bathy < 10.0
    land[0, :] = land[-1, :] = True
    land[:, 0] = land[:, -1] = True
    # bottom level: depw(kb) < bathy <= depw(kb + 1), keeping a partial cell of at
    # least a tenth of its level (the zps minimum thickness)
    kb = np.searchsorted(depw, bathy, side="left")  # first depw >= bathy -> kb = index of that level (1-based)
    kb = np.clip(kb, 1, jpk - 1)
    thin = bathy - depw[kb - 1] < 0.1 * e3t1[kb - 1]
    bathy = np.where(thin, depw[kb - 1] + 0.1 * e3t1[kb - 1], bathy)
    kb = np.where(land, 0, kb).astype(np.int32)
    kt = np.minimum(1, kb).astype(np.int32)
    e3t = np.broadcast_to(e3t1, (jpi, jpj, jpk)).copy()
    e3w = np.broadcast_to(e3w1, (jpi, jpj, jpk)).copy()
    ii, jj = np.nonzero(kb > 0)
    ik = kb[ii, jj] - 1                              # 0-based bottom level
    frac = (bathy[ii, jj] - depw[ik]) / (depw[ik + 1] - depw[ik])
    e3t[ii, jj, ik] = e3t1[ik] * frac
    e3w[ii, jj, ik] = 0.5 * (bathy[ii, jj] + depw[ik + 1] - 2.0 * depw[ik]) * (e3w1[ik] / (depw[ik + 1] - depw[ik]))
    below = ik + 1 <= jpk - 1
    e3w[ii[below], jj[below], ik[below] + 1] = e3t[ii[below], jj[below], ik[below]]
    e3t[ii[below], jj[below], ik[below] + 1] = e3t[ii[below], jj[below], ik[below]]
    e3u = np.broadcast_to(e3t1, (jpi, jpj, jpk)).copy()
    e3v = e3u.copy()
    e3u[:-1, :-1] = np.minimum(e3t[:-1, :-1], e3t[1:, :-1])
    e3v[:-1, :-1] = np.minimum(e3t[:-1, :-1], e3t[:-1, 1:])
    e3f = e3u.copy()
    e3f[:-1, :-1] = np.minimum(e3v[:-1, :-1], e3v[1:, :-1])
    # beta-plane grid from 45 N
    deg = e1 / (gyre.RA * gyre.RAD)
    i1 = np.arange(1, jpi + 1, dtype=np.float64)[:, None]
    j1 = np.arange(1, jpj + 1, dtype=np.float64)[None, :]
    gphit = 45.0 + (j1 - 1.5) * deg + 0.0 * i1
    gphiu = gphit.copy()
    gphiv = 45.0 + (j1 - 1.0) * deg + 0.0 * i1
    gphif = gphiv.copy()
    f = np.asfortranarray
    ee = np.full((jpi, jpj), e1, order="F")
    return dict(jpi=jpi, jpj=jpj, jpk=jpk, jperio=0,
                e1t=ee, e2t=ee.copy(order="F"), e1u=ee.copy(order="F"), e2u=ee.copy(order="F"),
                e1v=ee.copy(order="F"), e2v=ee.copy(order="F"), e1f=ee.copy(order="F"), e2f=ee.copy(order="F"),
                ff_f=f(2.0 * gyre.OMEGA * np.sin(gyre.RAD * gphif)), ff_t=f(2.0 * gyre.OMEGA * np.sin(gyre.RAD * gphit)),
                k_top=f(kt), k_bot=f(kb), e3t_0=f(e3t), e3u_0=f(e3u), e3v_0=f(e3v), e3w_0=f(e3w), e3f_0=f(e3f),
                gdept_1d=dept, gphit=f(gphit), gphiu=f(gphiu), gphiv=f(gphiv))


def state(dom, nam, seed=0, member=0):
    """gyre.state() on the shelf, plus the z* fields, partial-step bottom gradients
    of T and S (zpshde) and an inverse-barometer ssh. The gyre is weak (3 cm/s) and
    the level-to-level noise small: the flow across the bathymetry steps then implies
    vertical velocities that, with 2.3 m surface cells and rdt = 300 s, stay within
    the advective stability limit of FCT (|w| 2 rdt / e3t < 1)."""
    st = gyre.state(dom, nam, seed=seed, member=member, u0=0.03, noise_u=0.003)
    rng = np.random.default_rng([seed, member, 5])
    jpi, jpj = dom["jpi"], dom["jpj"]
    _, um, vm, _ = gyre.masks(dom)
    # a basin-scale sea level (near balance, unlike GYRE's grid-scale noise, which on
    # 1 km cells would drive barotropic adjustments of ~0.1 m/s within one step)
    ssm = gyre.masks(dom)[0].max(axis=2)
    xs = np.linspace(0.0, 1.0, jpi)[:, None]
    ys = np.linspace(0.0, 1.0, jpj)[None, :]
    sshn = 0.05 * np.sin(np.pi * xs) * np.sin(2 * np.pi * ys) + 0.002 * rng.standard_normal((jpi, jpj))
    st["sshn"] = np.asfortranarray(sshn * ssm)
    st["sshb"] = np.asfortranarray((0.999 * sshn + 0.0005 * rng.standard_normal((jpi, jpj))) * ssm)
    # z* continuity (sshwzv.F90 ssh_nxt :99-121 and wzv :183-184): the after ssh
    # from the column divergence of the now transports, then w from the bottom up
    # with the thickness change, so w vanishes at the surface
    tm = gyre.masks(dom)[0]
    z = gyre.zstar(dom, st)
    e1e2t = dom["e1t"] * dom["e2t"]
    fu = dom["e2u"][:, :, None] * z["e3u_n"] * st["un"]
    fv = dom["e1v"][:, :, None] * z["e3v_n"] * st["vn"]
    div = np.zeros_like(fu)                                  # e3t_n * hdivn
    div[1:-1, 1:-1] = (fu[1:-1, 1:-1] - fu[:-2, 1:-1] + fv[1:-1, 1:-1] - fv[1:-1, :-2]) / e1e2t[1:-1, 1:-1, None]
    div = div * tm
    r2dt = 2.0 * nam["rn_rdt"]
    ssha = (st["sshb"] - r2dt * div[:, :, :-1].sum(axis=2)) * tm.max(axis=2)
    z = gyre.zstar(dom, st, ssha=ssha)
    wn = np.zeros_like(div)
    for k in range(dom["jpk"] - 2, -1, -1):
        wn[:, :, k] = wn[:, :, k + 1] - (div[:, :, k] + (z["e3t_a"][:, :, k] - z["e3t_b"][:, :, k]) / r2dt) * tm[:, :, k]
    st["wn"] = np.asfortranarray(wn)
    st.update(z)
    g = lambda m: np.asfortranarray(1e-3 * rng.standard_normal((jpi, jpj, 2)) * m.max(axis=2)[:, :, None])
    st["gtsu"], st["gtsv"] = g(um), g(vm)
    x = np.arange(jpi)[:, None] / max(jpi - 1, 1)
    st["ssh_ib"] = np.asfortranarray(0.02 * np.sin(2 * math.pi * (x + 0.3 * np.arange(jpj)[None, :] / jpj)))
    st["ssh_ibb"] = np.asfortranarray(0.9 * st["ssh_ib"])
    return st


def depths(st):
    """The now depths of a state's z* levels (domvvl.F90:641-652, no cavities): gdepw_n = 0 at the
    surface and the running sum of e3t_n below; gdept_n = e3w_n / 2 at the surface and
    the running sum of e3w_n below."""
    e3t, e3w = st["e3t_n"], st["e3w_n"]
    gdepw = np.zeros_like(e3t)
    gdept = np.zeros_like(e3t)
    gdept[:, :, 0] = 0.5 * e3w[:, :, 0]
    for k in range(1, e3t.shape[2]):
        gdepw[:, :, k] = gdepw[:, :, k - 1] + e3t[:, :, k - 1]
        gdept[:, :, k] = gdept[:, :, k - 1] + e3w[:, :, k]
    return dict(gdept_n=np.asfortranarray(gdept), gdepw_n=np.asfortranarray(gdepw))
