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
