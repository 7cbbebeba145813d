"""zdf_mxl (the mixed layer of the density criterion and the turbocline): known
answers and a restatement check of the oracle on the CPU, and the GPU through the C
ABI against the oracle."""
import numpy as np
import pytest

from nemo_gpu import gyre


def case(seed=11):
    from oracle import ora
    dom = gyre.domain(1)
    nam = gyre.namelist()
    st = gyre.state(dom, nam, seed=seed)
    sl = gyre.slope_inputs(dom, nam, st)
    o = ora.Oracle(dom, nam)
    s2 = (dom["jpi"], dom["jpj"])
    a = dict(RN2B=np.array(sl["rn2b"], order="F"), AVT=np.array(st["avt"], order="F"),
             GDEPT_N=np.array(sl["gdept_n"], order="F"), GDEPW_N=np.array(sl["gdepw_n"], order="F"),
             NMLN=np.zeros(s2, dtype=np.int32, order="F"), HMLP=np.zeros(s2, order="F"),
             HMLPT=np.zeros(s2, order="F"), HMLD=np.zeros(s2, order="F"))
    for k, v in a.items():
        o.bind(k, v)
    return dom, nam, o, a


def restated(dom, nam, a, nlb10):
    """zdfmxl.F90:93-130 in numpy, column-wise."""
    jpk = dom["jpk"]
    mbkt = np.maximum(dom["k_bot"], 1)
    e3w = dom["e3w_0"]
    wm = gyre.masks(dom)[3]
    ssm = gyre.masks(dom)[0].max(axis=2)
    zn2c = nam["grav"] * 0.01 * (1.0 / nam["rau0"])
    h = np.zeros(mbkt.shape)
    nmln = np.full(mbkt.shape, nlb10)
    for jk in range(nlb10, jpk):
        h = h + np.maximum(a["RN2B"][:, :, jk - 1], 0.0) * e3w[:, :, jk - 1]
        nmln = np.where(h < zn2c, np.minimum(jk, mbkt) + 1, nmln)
    imld = mbkt + 1
    for jk in range(jpk - 1, nlb10 - 1, -1):
        imld = np.where(a["AVT"][:, :, jk - 1] < 5.e-4 * wm[:, :, jk - 1], jk, imld)
    ii, jj = np.meshgrid(np.arange(dom["jpi"]), np.arange(dom["jpj"]), indexing="ij")
    return (nmln, a["GDEPW_N"][ii, jj, nmln - 1] * ssm, a["GDEPT_N"][ii, jj, nmln - 2] * ssm,
            a["GDEPW_N"][ii, jj, imld - 1] * ssm)


def test_nlb10_is_the_first_w_level_below_10m():
    dom, nam, o, a = case()
    gdepw = np.concatenate([[0.0], np.cumsum(dom["e3t_0"][1, 1, :])])
    zref = 10.0 - 0.1 * dom["e3w_0"][1, 1, :].min()
    assert o.nlb10() == 1 + int(np.argmax(gdepw > zref))


def test_zdf_mxl_against_a_restatement_and_limits():
    dom, nam, o, a = case()
    o.zdf_mxl(1)
    nmln, hmlp, hmlpt, hmld = restated(dom, nam, a, o.nlb10())
    assert np.array_equal(a["NMLN"], nmln)
    assert np.array_equal(a["HMLP"], hmlp) and np.array_equal(a["HMLPT"], hmlpt)
    assert np.array_equal(a["HMLD"], hmld)
    # no stratification: the mixed layer reaches the bottom W-level of each column
    a["RN2B"][...] = 0.0
    o.zdf_mxl(2)
    mbkt = np.maximum(dom["k_bot"], 1)
    assert np.array_equal(a["NMLN"], np.minimum(dom["jpk"] - 1, mbkt) + 1)
    # strong stratification: it stops at nlb10
    a["RN2B"][...] = 1.0
    o.zdf_mxl(3)
    assert np.all(a["NMLN"] == o.nlb10())


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_zdf_mxl(prec):
    torch = pytest.importorskip("torch")
    from nemo_gpu import api
    dom, nam, o, a = case(seed=12)
    if prec == "mixed":      # the oracle sees the FP32 inputs the GPU holds
        for k in ("RN2B", "AVT", "GDEPT_N", "GDEPW_N"):
            a[k][...] = a[k].astype(np.float32)
    o.zdf_mxl(4)
    ctx = api.Context(dom, nam, nmembers=1, prec=prec)
    dev = {}
    for k, v in a.items():
        if k == "NMLN":
            dev[k] = torch.zeros(v.size, dtype=torch.int32, device="cuda")
        else:
            dev[k] = ctx.to_device(np.zeros_like(v) if k.startswith("HML") else v)
        ctx.bind(k, dev[k])
    ctx.zdf_mxl(4)
    ctx.synchronize()
    got_n = dev["NMLN"].cpu().numpy().reshape(a["NMLN"].shape, order="F")
    assert np.array_equal(got_n, a["NMLN"]) or (prec == "mixed" and np.mean(got_n != a["NMLN"]) < 1e-3
                                                and np.abs(got_n - a["NMLN"]).max() <= 1)
    same = got_n == a["NMLN"]
    for k in ("HMLP", "HMLPT", "HMLD"):
        g = ctx.to_host(dev[k], a[k].shape)
        msk = same if k != "HMLD" else np.ones_like(same)
        assert np.allclose(g[msk], a[k][msk], rtol=1e-7 if prec == "mixed" else 0, atol=0), k
