"""Iso-neutral slopes over partial-step bottoms: zps_hde's density part
(zpshde.F90:150-184) and ldf_slp with its bottom-level correction
(ldfslp.F90:144-151).

On the CPU, known answers of the oracle: a density that depends on depth only (T and
S uniform) has zero partial-step gradients, though the bottom cells of neighbouring
columns sit at different depths; over a flat bottom the partial-step form gives the
plain gradients, so the slopes are bit-identical with and without ln_zps. On the
GPU, both routines through the C ABI against the oracle on a slice of the synthetic
shelf (z*, partial steps), FP64 and mixed, with the simplified eos and EOS-80."""
import numpy as np
import pytest

from nemo_gpu import gyre, shelf

SLOPES = ("USLP", "VSLP", "WSLPI", "WSLPJ")
EOS = {"seos": dict(ln_seos=1, ln_eos80=0), "eos80": dict(ln_eos80=1, ln_seos=0)}


def shelf_case(nx=60, ny=70, nz=30, eos="seos", seed=3):
    """an oracle on a shelf slice with the slope inputs formed by the oracle itself:
    prd = eos_insitu(tsb), N^2 = bn2(tsb), the mixed layer of zdf_mxl"""
    from oracle import ora
    dom = shelf.domain(nx, ny, nz, seed=seed)
    nam = shelf.namelist(**EOS[eos])
    st = shelf.state(dom, nam, seed=seed + 1)
    st.update(shelf.depths(st))
    o = ora.Oracle(dom, nam)
    f = {}
    for n in ("E3T_N", "E3U_N", "E3V_N", "E3W_N", "E3T_B", "E3T_A", "GDEPT_N", "GDEPW_N", "AVT"):
        f[n] = np.array(st[n.lower()], order="F", copy=True)
        o.bind(n, f[n])
    s3 = f["AVT"].shape
    ts = np.array(st["tsb"], order="F", copy=True)
    prd, pn2 = np.zeros(s3, order="F"), np.zeros(s3, order="F")
    pab = np.zeros(ts.shape, order="F")
    o.eos_insitu(ts, prd, f["GDEPT_N"])
    o.rab_3d(ts, pab)
    o.bn2(ts, pab, pn2)
    f["RN2B"] = pn2
    f["NMLN"] = np.zeros(s3[:2], dtype=np.int32, order="F")
    for n in ("HMLP", "HMLPT"):
        f[n] = np.zeros(s3[:2], order="F")
    for n in ("RN2B", "NMLN", "HMLP", "HMLPT"):
        o.bind(n, f[n])
    o.zdf_mxl(5)
    for n in SLOPES:
        f[n] = np.zeros(s3, order="F")
        o.bind(n, f[n])
    return dom, nam, st, o, f, ts, prd, pn2


def test_depth_only_density_has_zero_partial_step_gradients():
    dom, nam, st, o, f, ts, prd, pn2 = shelf_case()
    ts[..., 0] = 12.0
    ts[..., 1] = 34.5
    o.eos_insitu(ts, prd, f["GDEPT_N"])
    gru, grv = o.zps_hde_rd(5, ts, prd)
    assert not gru.any() and not grv.any()
    # the plain difference at the bottom level of a u-point is not zero: the two
    # bottom cells lie at different depths
    mbku = o.iarray("mbku")
    um = o.array("umask", ndim=3)
    jpi, jpj = dom["jpi"], dom["jpj"]
    plain = [prd[i + 1, j, mbku[i, j] - 1] - prd[i, j, mbku[i, j] - 1]
             for i in range(1, jpi - 2) for j in range(1, jpj - 1) if um[i, j, 0] > 0]
    assert np.abs(plain).max() > 0


def test_flat_bottom_gives_the_plain_slopes():
    from oracle import ora
    dom = gyre.domain(1)
    out = {}
    for zps in (0, 1):
        nam = gyre.namelist(ln_zps=zps, ln_seos=1)
        st = gyre.state(dom, nam, seed=63)
        inp = gyre.slope_inputs(dom, nam, st)
        o = ora.Oracle(dom, nam)
        f = {n: np.zeros(st["avt"].shape, order="F") for n in SLOPES}
        for n in SLOPES:
            o.bind(n, f[n])
        for n in ("GDEPT_N", "GDEPW_N", "NMLN", "HMLP", "HMLPT"):
            o.bind(n, inp[n.lower()])
        prd = np.zeros(st["avt"].shape, order="F")
        o.eos_insitu(st["tsb"], prd, inp["gdept_n"])
        if zps:
            gru, grv = o.zps_hde_rd(5, st["tsb"], prd)
            o.bind("GRU", gru)
            o.bind("GRV", grv)
        o.ldf_slp(5, prd, inp["rn2b"])
        out[zps] = f
    for n in SLOPES:
        assert np.abs(out[0][n]).max() > 0
        np.testing.assert_array_equal(out[1][n], out[0][n], err_msg=n)


# ------------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("eos", ["seos", "eos80"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_zps_gradients_and_slopes(prec, eos):
    import torch
    from harness import relerr
    from nemo_gpu import api
    dom, nam, st, o, f, ts, prd, pn2 = shelf_case(eos=eos)
    if prec == "mixed":  # the oracle on the FP32-rounded inputs: the check is of the arithmetic
        r = lambda a: np.asfortranarray(a.astype(np.float32).astype(np.float64))
        ts, prd, pn2 = r(ts), r(prd), r(pn2)
        for n in ("E3T_N", "E3U_N", "E3V_N", "E3W_N", "E3T_B", "E3T_A", "GDEPT_N", "GDEPW_N", "HMLP", "HMLPT"):
            f[n] = r(f[n])
            o.bind(n, f[n])
    gru, grv = o.zps_hde_rd(5, ts, prd)
    o.bind("GRU", gru)
    o.bind("GRV", grv)
    o.ldf_slp(5, prd, pn2)
    ctx = api.Context(dom, nam, nmembers=1, prec=prec)
    dev = {}
    for n in ("E3T_N", "E3U_N", "E3V_N", "E3W_N", "E3T_B", "E3T_A", "GDEPT_N", "GDEPW_N", "HMLP", "HMLPT"):
        dev[n] = ctx.to_device([f[n]])
        ctx.bind(n, dev[n])
    for n in SLOPES:
        dev[n] = ctx.to_device([np.zeros_like(f[n])])
        ctx.bind(n, dev[n])
    dev["NMLN"] = torch.from_numpy(np.ascontiguousarray(f["NMLN"].ravel(order="F"))).cuda()
    ctx.bind("NMLN", dev["NMLN"])
    dts, dprd, dpn2 = ctx.to_device([ts]), ctx.to_device([prd]), ctx.to_device([pn2])
    dgu, dgv = ctx.to_device([np.zeros_like(gru)]), ctx.to_device([np.zeros_like(grv)])
    ctx.zps_hde_rd(5, dts, dprd, dgu, dgv)
    ctx.bind("GRU", dgu)
    ctx.bind("GRV", dgv)
    ctx.ldf_slp(5, dprd, dpn2)
    ctx.synchronize()
    tol = 1e-12 if prec == "fp64" else 2e-5
    for n, ref, t in (("gru", gru, dgu), ("grv", grv, dgv)):
        got = ctx.to_host(t, ref.shape)
        assert np.abs(ref).max() > 0, n
        assert relerr(ref, got) <= (tol if prec == "fp64" else 1e-4), (n, relerr(ref, got))
    for n in SLOPES:
        got = ctx.to_host(dev[n], f[n].shape)
        assert np.abs(f[n]).max() > 0, n
        if prec == "fp64":
            assert relerr(f[n], got) <= tol, (n, relerr(f[n], got))
        else:  # slopes of nearly unstratified water are ill-conditioned in FP32
            off = np.abs(got - f[n]) > 1e-3 * np.abs(f[n]).max()
            assert off.mean() < 0.01, (n, off.mean())
