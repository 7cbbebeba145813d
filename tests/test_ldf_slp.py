"""ldf_slp (iso-neutral slopes): the oracle's known answers, and the GPU against the
oracle on the slopes of a seeded GYRE state."""
import numpy as np
import pytest

from nemo_gpu import gyre
from oracle import ora

SLOPES = ("USLP", "VSLP", "WSLPI", "WSLPJ")


def oracle_case(seed=61, **over):
    dom = gyre.domain(1)
    nam = gyre.namelist(**over)
    st = gyre.state(dom, nam, seed=seed)
    inp = gyre.slope_inputs(dom, nam, st)
    o = ora.Oracle(dom, nam)
    out = {n: np.zeros((dom["jpi"], dom["jpj"], dom["jpk"]), order="F") for n in SLOPES}
    for n, a in out.items():
        o.bind(n, a)
    for n in ("GDEPT_N", "GDEPW_N", "NMLN", "HMLP", "HMLPT"):
        o.bind(n, inp[n.lower()])
    return dom, nam, inp, o, out


def test_flat_isopycnals_have_zero_slopes():
    dom, nam, inp, o, out = oracle_case()
    prd = np.asfortranarray(np.broadcast_to(np.linspace(0.0, 2e-3, dom["jpk"]), inp["rhd"].shape).copy())
    pn2 = np.asfortranarray(np.full_like(prd, 1e-5))
    o.ldf_slp(5, prd, pn2)
    for n in SLOPES:
        assert not np.any(out[n]), n


def test_uniform_tilt_below_the_mixed_layer():
    """prd = a i - b k with constant N^2: away from coasts and below the mixed layer
    the u-slope is zgru / e1u / zdzr (the filter keeps a uniform field)."""
    dom, nam, inp, o, out = oracle_case()
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    tm = gyre.masks(dom)[0]
    i = np.arange(jpi)[:, None, None]
    k = np.arange(jpk)[None, None, :]
    prd = np.asfortranarray(np.broadcast_to(1e-7 * i + 1e-4 * k, (jpi, jpj, jpk)) * tm)
    n0 = 1e-5
    pn2 = np.asfortranarray(np.full_like(prd, n0))
    inp["nmln"][...] = 2
    o.ldf_slp(5, prd, pn2)
    g = nam["grav"]
    zau = 1e-7 / dom["e1u"][:, :, None]
    # mean of zdzr = -(prd + 1) / g * 2 N0 * (1 - 0.5) at i and i+1
    zbu = -1.0 / g * ((prd[:-1] + 1.0) + (prd[1:] + 1.0)) * 0.5 * (2.0 * n0) * 0.5
    exp = zau[:-1] / zbu
    sel = (slice(4, jpi - 5), slice(4, jpj - 5), slice(3, jpk - 4))
    got = out["USLP"][sel]
    ref = exp[sel]
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_ldf_slp_refuses_partial_steps():
    dom, nam, inp, o, out = oracle_case(ln_zps=1)
    with pytest.raises(RuntimeError):
        o.ldf_slp(5, inp["rhd"], inp["rn2b"])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_ldf_slp_gpu_matches_oracle(prec):
    import torch
    from harness import relerr
    from nemo_gpu import api
    dom, nam, inp, o, out = oracle_case(seed=62)
    if prec == "mixed":
        # the FP32 inputs: the horizontal density differences (~1e-6 of a 1e-3
        # anomaly) lose ~1e-4 of their value to the rounding of prd itself, so the
        # oracle is given the same rounded inputs and the check is of the arithmetic
        for n in ("rhd", "rn2b", "gdept_n", "gdepw_n", "hmlp", "hmlpt"):
            inp[n] = np.asfortranarray(inp[n].astype(np.float32).astype(np.float64))
        for n in ("GDEPT_N", "GDEPW_N", "HMLP", "HMLPT"):
            o.bind(n, inp[n.lower()])
    o.ldf_slp(5, inp["rhd"], inp["rn2b"])
    ctx = api.Context(dom, nam, nmembers=2, prec=prec)
    dev = {}
    for n in SLOPES:
        dev[n] = ctx.to_device([np.zeros_like(out[n])] * 2)
        ctx.bind(n, dev[n])
    for n in ("GDEPT_N", "GDEPW_N", "HMLP", "HMLPT"):
        dev[n] = ctx.to_device([inp[n.lower()]] * 2)
        ctx.bind(n, dev[n])
    dev["NMLN"] = torch.from_numpy(np.concatenate([inp["nmln"].ravel(order="F")] * 2)).cuda()
    ctx.bind("NMLN", dev["NMLN"])
    prd, pn2 = ctx.to_device([inp["rhd"]] * 2), ctx.to_device([inp["rn2b"]] * 2)
    torch.cuda.synchronize()
    ctx.ldf_slp(5, prd, pn2)
    ctx.synchronize()
    tol = 1e-12 if prec == "fp64" else 2e-5
    for n in SLOPES:
        got = ctx.to_host(dev[n], out[n].shape)
        assert np.abs(out[n]).max() > 0, n
        for m in range(2):
            assert relerr(out[n], got[m]) <= tol, (n, m, relerr(out[n], got[m]))
