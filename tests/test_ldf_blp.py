"""tra_ldf_blp (bilaplacian, two passes of the laplacian): the oracle's known
answers, the GPU driver against the oracle, and the hot path with a bilaplacian
namelist (np_blp and np_blp_i)."""
import numpy as np
import pytest

from harness import Pair, relerr
from nemo_gpu import gyre
from oracle import ora


def test_bilaplacian_of_a_constant_is_zero_and_composes():
    dom = gyre.domain(1)
    nam = gyre.namelist(ln_traldf_lap=0, ln_traldf_blp=1, ln_traldf_iso=0, rn_aht_0=1.e11)
    o = ora.Oracle(dom, nam)
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    tm = gyre.masks(dom)[0]
    tb = np.asfortranarray(np.stack([7.0 * tm, 35.0 * tm], axis=3))
    ta = np.zeros_like(tb, order="F")
    o.tra_ldf_blp(5, 1, "TRA", None, None, None, None, None, None, tb, ta, 2, 20)
    assert np.abs(ta).max() < 1e-12 * 35
    st = gyre.state(dom, nam, seed=71)
    tb = np.asfortranarray(st["tsb"])
    ta = np.zeros_like(tb, order="F")
    o.tra_ldf_blp(5, 1, "TRA", None, None, None, None, None, None, tb, ta, 2, 20)
    zl = np.zeros_like(tb, order="F")
    o.tra_ldf_lap(5, 1, "TRA", None, None, None, None, None, None, tb, zl, 2, 1)
    o.lbc_lnk(zl, "T")
    ta2 = np.zeros_like(tb, order="F")
    o.tra_ldf_lap(5, 1, "TRA", None, None, None, None, None, None, zl, ta2, 2, 2)
    assert np.array_equal(ta, ta2) and np.abs(ta).max() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("kldf", [20, 21])
def test_tra_ldf_blp_gpu(prec, kldf):
    p = Pair(nn=2, prec=prec, seed=72, ln_traldf_lap=0, ln_traldf_blp=1, ln_traldf_iso=int(kldf == 21),
             rn_aht_0=1.e11)
    if kldf == 21:
        p.bind_iso()
    st = p.states[0]
    ta = np.zeros(p.s4, order="F")
    ta_dev = p.to_dev([ta])
    p.ora[0].tra_ldf_blp(1, 1, "TRA", None, None, None, None, None, None, st["tsb"], ta, 2, kldf)
    p.ctx.tra_ldf_blp(1, 1, "TRA", None, None, None, None, None, None, p.to_dev([st["tsb"]]), ta_dev, 2, kldf)
    p.ctx.synchronize()
    tol = 1e-12 if prec == "fp64" else 2e-4
    assert relerr(ta, p.ctx.to_host(ta_dev, p.s4)) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("iso", [0, 1])
def test_stp_hotpath_bilaplacian(prec, iso):
    p = Pair(nn=2, prec=prec, seed=73, neuler=0, ln_traldf_lap=0, ln_traldf_blp=1, ln_traldf_iso=iso,
             rn_aht_0=1.e11)
    p.bind_hotpath()
    for kt in (1, 2, 3):
        p.ora[0].stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
    p.ctx.synchronize()
    p.compare("TSA", p.s4, 1e-12 if prec == "fp64" else 5e-6)


def test_zps_hde_flat_bottom_is_the_plain_difference():
    dom = gyre.domain(1)
    nam = gyre.namelist()
    o = ora.Oracle(dom, nam)
    st = gyre.state(dom, nam, seed=74)
    t = np.asfortranarray(st["tsb"])
    gu, gv = o.zps_hde(5, 2, t)
    ku = o.iarray("mbku")
    i, j = 5, 7
    k = ku[i, j] - 1
    assert gu[i, j, 0] == t[i + 1, j, k, 0] - t[i, j, k, 0]
    assert not gu[0].any() and not gv[:, -1].any()


def shelf_pair(prec, seed, **over):
    from nemo_gpu import shelf
    dom = shelf.domain(40, 36, 21, seed=seed)
    nam = shelf.namelist(**over)
    st = shelf.state(dom, nam, seed=seed + 1)
    p = Pair(prec=prec, dom=dom, nam=nam, states=[st])
    for n in ("E3T_B", "E3T_N", "E3T_A", "E3U_N", "E3V_N", "E3W_N"):
        p.bind(n)
    return p, st


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_zps_hde_gpu_shelf(prec):
    import torch
    p, st = shelf_pair(prec, 75)
    gu, gv = p.ora[0].zps_hde(5, 2, st["tsb"])
    du = p.to_dev([np.zeros_like(gu)])
    dv = p.to_dev([np.zeros_like(gv)])
    p.ctx.zps_hde(5, 2, p.to_dev([st["tsb"]]), du, dv)
    p.ctx.synchronize()
    tol = 1e-12 if prec == "fp64" else 2e-4
    assert np.abs(gu).max() > 0
    assert relerr(gu, p.ctx.to_host(du, gu.shape)) <= tol
    assert relerr(gv, p.ctx.to_host(dv, gv.shape)) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("kldf", [20, 21])
def test_tra_ldf_blp_partial_steps(prec, kldf):
    p, st = shelf_pair(prec, 76, ln_traldf_lap=0, ln_traldf_blp=1, ln_traldf_iso=int(kldf == 21),
                       rn_aht_0=1.e9)
    if kldf == 21:
        p.bind_iso()
    ta = np.zeros(p.s4, order="F")
    ta_dev = p.to_dev([ta])
    p.ora[0].tra_ldf_blp(1, 1, "TRA", None, None, st["gtsu"], st["gtsv"], None, None, st["tsb"], ta, 2, kldf)
    p.ctx.tra_ldf_blp(1, 1, "TRA", None, None, p.to_dev([st["gtsu"]]), p.to_dev([st["gtsv"]]), None, None,
                      p.to_dev([st["tsb"]]), ta_dev, 2, kldf)
    p.ctx.synchronize()
    tol = 1e-12 if prec == "fp64" else 5e-4
    assert np.abs(ta).max() > 0
    assert relerr(ta, p.ctx.to_host(ta_dev, p.s4)) <= tol
