"""Known answers of the oracle's rest-of-step routines (wzv, the dyn_zdf time step,
dyn_nxt, ssh_swp) that close the path into a model step."""
import numpy as np

from nemo_gpu import gyre
from oracle import ora


def setup(seed=0, **over):
    dom = gyre.domain(1)
    nam = gyre.namelist(**over)
    st = gyre.state(dom, nam, seed=seed)
    o = ora.Oracle(dom, nam)
    keep = {}
    for n in ("un", "vn", "wn", "ub", "vb", "ua", "va", "sshb", "sshn", "un_b", "vn_b", "ub_b", "vb_b"):
        keep[n] = np.array(st[n], dtype=np.float64, order="F")
        o.bind(n.upper(), keep[n])
    return dom, nam, st, o, keep


def test_wzv_integrates_the_divergence():
    dom, nam, st, o, f = setup(1)
    rng = np.random.default_rng(3)
    tm, um, vm, _ = gyre.masks(dom)
    f["un"][...] = rng.standard_normal(f["un"].shape) * um
    f["vn"][...] = rng.standard_normal(f["vn"].shape) * vm
    o.wzv(5)
    e3t, e3u, e3v = dom["e3t_0"], dom["e3u_0"], dom["e3v_0"]
    fu = dom["e2u"][:, :, None] * e3u * f["un"]
    fv = dom["e1v"][:, :, None] * e3v * f["vn"]
    hd = np.zeros_like(fu)
    r1 = 1.0 / (dom["e1t"] * dom["e2t"])
    hd[1:-1, 1:-1] = (fu[1:-1, 1:-1] - fu[:-2, 1:-1] + fv[1:-1, 1:-1] - fv[1:-1, :-2]) * r1[1:-1, 1:-1, None] / e3t[1:-1, 1:-1]
    hd[:, :, -1] = 0.0
    w = -np.cumsum((e3t * hd * tm)[:, :, ::-1], axis=2)[:, :, ::-1]
    assert np.all(f["wn"][:, :, -1] == 0.0)
    assert np.abs(f["wn"] - w).max() <= 1e-12 * np.abs(w).max()
    # a horizontally non-divergent flow (from a streamfunction) has w = 0 (to rounding)
    psi = rng.standard_normal((dom["jpi"], dom["jpj"]))
    # f-points on the closed faces (the first and last wet faces, and beyond): 0
    psi[[0, -2, -1], :] = 0.0
    psi[:, [0, -2, -1]] = 0.0
    u = np.zeros_like(f["un"])
    v = np.zeros_like(f["vn"])
    u[:, 1:, :] = (-(psi[:, 1:] - psi[:, :-1]) / dom["e2u"][:, 1:])[:, :, None] / e3u[:, 1:]
    v[1:, :, :] = ((psi[1:, :] - psi[:-1, :]) / dom["e1v"][1:, :])[:, :, None] / e3v[1:]
    f["un"][...] = u * um
    f["vn"][...] = v * vm
    o.wzv(5)
    assert np.abs(f["wn"]).max() <= 1e-12 * np.abs(u).max()


def test_dyn_zdf_step_and_dyn_nxt_euler_swap():
    dom, nam, st, o, f = setup(2, neuler=0)
    jpi, jpj = dom["jpi"], dom["jpj"]
    rng = np.random.default_rng(4)
    ua_b = np.asfortranarray(0.1 * rng.standard_normal((jpi, jpj)) * gyre.masks(dom)[1].max(axis=2))
    va_b = np.asfortranarray(0.1 * rng.standard_normal((jpi, jpj)) * gyre.masks(dom)[2].max(axis=2))
    o.bind("UA_B", ua_b)
    o.bind("VA_B", va_b)
    ub0 = f["ub"].copy()
    ua0 = f["ua"].copy()
    o.dyn_zdf_step(1)
    um = gyre.masks(dom)[1]
    assert np.allclose(f["ua"][:, :, :-1], ((ub0 + nam["rn_rdt"] * ua0) * um)[:, :, :-1], rtol=0, atol=1e-13)
    o.dyn_nxt(1)
    # Euler: un = ua with the barotropic part of the sub-steps, so un_b = ua_b where wet
    wet = um.max(axis=2) > 0
    wet[0, :] = wet[-1, :] = wet[:, 0] = wet[:, -1] = False
    assert np.abs(f["un_b"][wet] - ua_b[wet]).max() <= 1e-12 * np.abs(ua_b).max()
    assert np.all(f["un"][0] == 0.0) and np.all(f["un"][:, -1] == 0.0)


def test_ssh_swp_leapfrog_and_euler():
    dom, nam, st, o, f = setup(3)
    ssha = np.asfortranarray(np.random.default_rng(5).standard_normal((dom["jpi"], dom["jpj"])))
    o.bind("SSHA", ssha)
    b, n = f["sshb"].copy(), f["sshn"].copy()
    o.ssh_swp(5)
    assert np.array_equal(f["sshn"], ssha)
    exp = n + nam["rn_atfp"] * (b - 2 * n + ssha)
    assert np.abs(f["sshb"] - exp).max() <= 1e-15 * np.abs(exp).max()
    dom, nam, st, o, f = setup(3, neuler=0)
    o.bind("SSHA", ssha)
    b = f["sshb"].copy()
    o.ssh_swp(1)
    assert np.array_equal(f["sshn"], ssha) and np.array_equal(f["sshb"], b)
