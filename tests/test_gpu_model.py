"""The model step (the hot path closed by wzv, the dyn_zdf time step, tra_nxt,
dyn_nxt and ssh_swp) against the oracle: the routines one by one, a few steps from
an Euler start through the captured graph, and ten model days (120 steps of
rdt = 7200 s) in FP64 and in the mixed form."""
import numpy as np
import pytest

from harness import Pair, relerr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

PRECS = ["fp64", "mixed"]
TOL = {"fp64": 1e-12, "mixed": 5e-6}


@pytest.mark.parametrize("prec", PRECS)
def test_rest_of_step_routines(prec):
    p = Pair(nn=2, prec=prec, seed=31, nmem=2)
    p.bind_hotpath()
    rng = np.random.default_rng(7)
    s2 = p.s2
    for name in ("UA_B", "VA_B", "SSHA"):
        arrs = [np.asfortranarray(0.05 * rng.standard_normal(s2)) for _ in range(2)]
        for m in range(2):
            p.host[m][name][...] = arrs[m]
        p.dev[name].copy_(p.to_dev(arrs, fp64=True))
    torch.cuda.synchronize()   # the context runs on its own stream
    for o in p.ora:
        o.wzv(5)
        o.dyn_zdf_step(5)
        o.dyn_nxt(5)
        o.ssh_swp(5)
    for f in (p.ctx.wzv, p.ctx.dyn_zdf_step, p.ctx.dyn_nxt, p.ctx.ssh_swp):
        f(5)
    p.ctx.synchronize()
    t = TOL[prec]
    for name in ("WN", "UA", "VA", "UN", "VN", "UB", "VB"):
        p.compare(name, p.s3, t)
    for name in ("UN_B", "VN_B", "UB_B", "VB_B", "SSHB", "SSHN"):
        p.compare(name, s2, t)


@pytest.mark.parametrize("prec", PRECS)
def test_stp_model_from_an_euler_start(prec):
    """Steps 1 (Euler), 2, 3 (graph capture), 4 (graph replay), two members."""
    p = Pair(nn=2, prec=prec, seed=32, nmem=2, neuler=0)
    p.bind_hotpath()
    for kt in (1, 2, 3, 4):
        for o in p.ora:
            o.stp_model(kt)
        p.ctx.stp_model(kt)
    p.ctx.synchronize()
    tt = 1e-12 if prec == "fp64" else 2e-5
    tu = 1e-12 if prec == "fp64" else 2e-3
    p.compare("TSN", p.s4, tt)
    p.compare("TSB", p.s4, tt)
    for name in ("UN", "VN", "UB", "VB", "WN"):
        p.compare(name, p.s3, tu)
    for name in ("SSHN", "SSHB", "UN_B", "VN_B"):
        p.compare(name, p.s2, tu)


def divergence(a, b, mask):
    d = (np.asarray(a) - np.asarray(b))[mask]
    return float(np.sqrt(np.mean(d * d))), float(np.abs(d).max())


def test_ten_days():
    """120 steps of rdt = 7200 s on GYRE nn_GYRE=1 from an Euler start: the FP64 GPU
    run against the oracle, and the mixed form against the FP64 GPU run."""
    runs = {}
    for prec in ("fp64", "mixed"):
        p = Pair(nn=1, prec=prec, seed=33, neuler=0)
        p.bind_hotpath()
        for kt in range(1, 121):
            if prec == "fp64":
                p.ora[0].stp_model(kt)
            p.ctx.stp_model(kt)
        p.ctx.synchronize()
        runs[prec] = p
    p64, pmx = runs["fp64"], runs["mixed"]
    tm = p64.ora[0].array("tmask", 3) > 0
    got = {n: p64.per_member(p64.dev[n], p64.s4 if n == "TSN" else (p64.s3 if n in ("UN", "VN") else p64.s2))[0]
           for n in ("TSN", "UN", "VN", "SSHN")}
    mix = {n: pmx.per_member(pmx.dev[n], pmx.s4 if n == "TSN" else (pmx.s3 if n in ("UN", "VN") else pmx.s2))[0]
           for n in ("TSN", "UN", "VN", "SSHN")}
    ref = {n: p64.host[0][n] for n in ("TSN", "UN", "VN", "SSHN")}
    assert np.isfinite(ref["TSN"]).all() and np.abs(ref["TSN"][..., 0][tm]).max() < 40.0
    # FP64 GPU against the oracle: relative to each field's range
    for n in ("TSN", "UN", "VN", "SSHN"):
        assert relerr(ref[n], got[n]) <= 1e-10, (n, relerr(ref[n], got[n]))
    # mixed against FP64 after ten days: SST and SSS (the surface level)
    sst = divergence(mix["TSN"][:, :, 0, 0], got["TSN"][:, :, 0, 0], tm[:, :, 0])
    sss = divergence(mix["TSN"][:, :, 0, 1], got["TSN"][:, :, 0, 1], tm[:, :, 0])
    assert sst[1] <= 1e-3, sst
    assert sss[1] <= 1e-4, sss
