"""dyn_ldf_lap (the iso-level laplacian viscosity of the momentum): known answers of
the oracle on the CPU and the GPU through the C ABI against the oracle."""
import numpy as np
import pytest

from nemo_gpu import gyre
from harness import Pair


def viscosity(dom, ahm0=1.0e5):
    return gyre.viscosity(dom, ahm0)


def oracle_case(nn=2):
    from oracle import ora
    dom = gyre.domain(nn)
    nam = gyre.namelist()
    o = ora.Oracle(dom, nam)
    ahmt, ahmf = viscosity(dom)
    o.bind("AHMT", ahmt)
    o.bind("AHMF", ahmf)
    return dom, o, (ahmt, ahmf)


def test_uniform_flow_has_no_interior_trend_and_passes_flip_sign():
    dom, o, keep = oracle_case()
    s3 = (dom["jpi"], dom["jpj"], dom["jpk"])
    _, um, vm, _ = gyre.masks(dom)
    ub = np.asfortranarray(0.3 * um)
    vb = np.asfortranarray(-0.2 * vm)
    ua, va = np.zeros(s3, order="F"), np.zeros(s3, order="F")
    o.dyn_ldf_lap(1, ub, vb, ua, va, 1)
    inner = (slice(3, -3), slice(3, -3), slice(0, -1))
    scale = 1e5 * 0.3 / dom["e1u"].min() ** 2
    assert np.abs(ua[inner]).max() < 1e-12 * scale and np.abs(va[inner]).max() < 1e-12 * scale
    assert np.abs(ua).max() > 1e-6 * scale            # the walls do act
    rng = np.random.default_rng(3)
    ub = np.asfortranarray(rng.standard_normal(s3) * um)
    vb = np.asfortranarray(rng.standard_normal(s3) * vm)
    a1, b1 = np.zeros(s3, order="F"), np.zeros(s3, order="F")
    a2, b2 = np.zeros(s3, order="F"), np.zeros(s3, order="F")
    o.dyn_ldf_lap(1, ub, vb, a1, b1, 1)
    o.dyn_ldf_lap(1, ub, vb, a2, b2, 2)
    assert np.array_equal(a1, -a2) and np.array_equal(b1, -b2)
    a3, b3 = np.zeros(s3, order="F"), np.zeros(s3, order="F")
    o.dyn_ldf_lap(1, np.asfortranarray(2 * ub), np.asfortranarray(2 * vb), a3, b3, 1)
    assert np.array_equal(a3, 2 * a1) and np.array_equal(b3, 2 * b1)   # exact: scaling by 2


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_dyn_ldf_lap(prec):
    pytest.importorskip("torch")
    p = Pair(nn=2, prec=prec, seed=47, nmem=2)
    for st in p.states:
        st["ahmt"], st["ahmf"] = viscosity(p.dom)
    p.bind_spg()
    p.bind("AHMT")
    p.bind("AHMF")
    for kpass, (u, v) in ((1, ("UB", "VB")), (2, ("UN", "VN"))):   # the second pass on other velocities
        for m, o in enumerate(p.ora):
            h = p.host[m]
            o.dyn_ldf_lap(3, h[u], h[v], h["UA"], h["VA"], kpass)
        p.ctx.dyn_ldf_lap(3, p.dev[u], p.dev[v], p.dev["UA"], p.dev["VA"], kpass)
    p.ctx.synchronize()
    t = 1e-12 if prec == "fp64" else 5e-5
    p.compare("UA", p.s3, t)
    p.compare("VA", p.s3, t)


@pytest.mark.parametrize("kvor", [1, 2, 4])
def test_vor_ene_does_no_work(kvor):
    """The energy-conserving scheme: for any vorticity the trend is normal to the
    flow, sum(e1e2u u ua) + sum(e1e2v v va) = 0 on each level of a closed basin."""
    from oracle import ora
    dom = gyre.domain(2)
    o = ora.Oracle(dom, gyre.namelist())
    s3 = (dom["jpi"], dom["jpj"], dom["jpk"])
    _, um, vm, _ = gyre.masks(dom)
    rng = np.random.default_rng(kvor)
    un = np.asfortranarray(rng.standard_normal(s3) * um)
    vn = np.asfortranarray(rng.standard_normal(s3) * vm)
    ua, va = np.zeros(s3, order="F"), np.zeros(s3, order="F")
    o.vor_ene(1, kvor, un, vn, ua, va)
    wu = (dom["e1u"] * dom["e2u"])[:, :, None] * un * ua
    wv = (dom["e1v"] * dom["e2v"])[:, :, None] * vn * va
    work = (wu + wv).sum(axis=(0, 1))
    size = (np.abs(wu) + np.abs(wv)).sum(axis=(0, 1))
    assert np.all(np.abs(work[:-1]) <= 1e-12 * size[:-1])
    assert np.all(size[:-1] > 0)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_vor_ene(prec):
    pytest.importorskip("torch")
    p = Pair(nn=2, prec=prec, seed=49, nmem=2)
    p.bind_spg()
    for kvor, (u, v) in ((4, ("UN", "VN")), (1, ("UB", "VB")), (2, ("UN", "VN"))):
        for m, o in enumerate(p.ora):
            h = p.host[m]
            o.vor_ene(3, kvor, h[u], h[v], h["UA"], h["VA"])
        p.ctx.vor_ene(3, kvor, p.dev[u], p.dev[v], p.dev["UA"], p.dev["VA"])
    p.ctx.synchronize()
    t = 1e-12 if prec == "fp64" else 5e-5
    p.compare("UA", p.s3, t)
    p.compare("VA", p.s3, t)


def test_keg_and_zad_known_answers():
    """Uniform horizontal flow: no kinetic-energy gradient in the interior; a trend
    quadratic in the velocity (x2 -> x4, exactly); no vertical advection without w or
    with a depth-independent flow."""
    from oracle import ora
    dom = gyre.domain(2)
    o = ora.Oracle(dom, gyre.namelist())
    s3 = (dom["jpi"], dom["jpj"], dom["jpk"])
    _, um, vm, wm = gyre.masks(dom)
    a = {k: np.zeros(s3, order="F") for k in ("UN", "VN", "WN", "UA", "VA")}
    for k, v in a.items():
        o.bind(k, v)
    a["UN"][...] = 0.2 * um
    a["VN"][...] = -0.1 * vm
    o.dyn_keg(1)
    inner = (slice(3, -3), slice(3, -3), slice(0, -1))
    assert np.all(a["UA"][inner] == 0) and np.all(a["VA"][inner] == 0)
    rng = np.random.default_rng(5)
    a["UN"][...] = rng.standard_normal(s3) * um
    a["VN"][...] = rng.standard_normal(s3) * vm
    a["UA"][...] = 0.0
    a["VA"][...] = 0.0
    o.dyn_keg(1)
    t1 = a["UA"].copy(), a["VA"].copy()
    a["UN"][...] *= 2
    a["VN"][...] *= 2
    a["UA"][...] = 0.0
    a["VA"][...] = 0.0
    o.dyn_keg(1)
    assert np.array_equal(a["UA"], 4 * t1[0]) and np.array_equal(a["VA"], 4 * t1[1])
    a["UA"][...] = 0.0
    a["VA"][...] = 0.0
    o.dyn_zad(1)                                            # w = 0
    assert np.all(a["UA"] == 0) and np.all(a["VA"] == 0)
    a["WN"][...] = rng.standard_normal(s3) * wm
    a["UN"][...] = np.broadcast_to(a["UN"][:, :, :1], s3)   # depth-independent
    a["VN"][...] = np.broadcast_to(a["VN"][:, :, :1], s3)
    o.dyn_zad(1)
    assert np.all(a["UA"] == 0) and np.all(a["VA"] == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_keg_zad(prec):
    pytest.importorskip("torch")
    p = Pair(nn=2, prec=prec, seed=51, nmem=2)
    p.bind_spg()
    p.bind("WN")
    for o in p.ora:
        o.dyn_keg(3)
        o.dyn_zad(3)
    p.ctx.dyn_keg(3)
    p.ctx.dyn_zad(3)
    p.ctx.synchronize()
    t = 1e-12 if prec == "fp64" else 5e-5
    p.compare("UA", p.s3, t)
    p.compare("VA", p.s3, t)
