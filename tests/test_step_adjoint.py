"""Adjoints of the time stepping of the model step, linear free surface: wzv
(sshwzv.F90:129-213), dyn_nxt (dynnxt.F90:66-377, ln_bt_fw) and ssh_swp
(sshwzv.F90:216-267). Each forward is linear in its state, so it is its own
tangent-linear. On the CPU: the oracle adjoints by the dot-product test against the
oracle forward, Euler first step and leap-frog. On the GPU: the adjoints through the
C ABI against the oracle adjoints (1e-12) and the same dot-product test, two members."""
import numpy as np
import pytest

from nemo_gpu import _ffi, gyre

F = np.asfortranarray


def case(neuler=1, seed=5):
    from oracle import ora
    dom = gyre.domain(1)
    nam = gyre.namelist(neuler=neuler)
    return dom, nam, ora.Oracle(dom, nam), np.random.default_rng(seed)


def rnd3(dom, rng, msk=None):
    a = rng.standard_normal((dom["jpi"], dom["jpj"], dom["jpk"]))
    return F(a * msk if msk is not None else a)


def rnd2(dom, rng, msk=None):
    a = rng.standard_normal((dom["jpi"], dom["jpj"]))
    return F(a * msk if msk is not None else a)


# ------------------------------------------------------------------------ wzv
def wzv_forward(o, dom, un, vn):
    wn = np.zeros_like(un)
    for n, a in (("UN", un), ("VN", vn), ("WN", wn)):
        o.bind(n, a)
    o.wzv(3)
    return wn


@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_wzv_adjoint_dot_product(seed):
    dom, nam, o, rng = case(seed=seed)
    _, um, vm, _ = gyre.masks(dom)
    du, dv = rnd3(dom, rng, um), rnd3(dom, rng, vm)
    dw = wzv_forward(o, dom, du.copy(order="F"), dv.copy(order="F"))
    lam = rnd3(dom, rng)
    ua, va, wa = np.zeros_like(du), np.zeros_like(dv), lam.copy(order="F")
    o.wzv_adj(3, ua, va, wa)
    lhs, rhs = float((dw * lam).sum()), float((du * ua).sum() + (dv * va).sum())
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs), (lhs, rhs)
    assert not wa.any()


# -------------------------------------------------------------------- dyn_nxt
NX3 = ("ua", "va", "un", "vn", "ub", "vb")
NX2 = ("un_b", "vn_b", "ub_b", "vb_b", "ua_b", "va_b")


def nxt_inputs(dom, rng):
    _, um, vm, _ = gyre.masks(dom)
    d = {}
    d["ua"], d["un"], d["ub"] = rnd3(dom, rng, um), rnd3(dom, rng, um), rnd3(dom, rng, um)
    d["va"], d["vn"], d["vb"] = rnd3(dom, rng, vm), rnd3(dom, rng, vm), rnd3(dom, rng, vm)
    for n in NX2:
        d[n] = rnd2(dom, rng, (um if "u" in n[:2] else vm).max(axis=2))
    return d


def nxt_forward(o, dx, kt):
    f = {n: dx[n].copy(order="F") for n in NX3 + NX2}
    for n, a in f.items():
        o.bind(n.upper(), a)
    o.dyn_nxt(kt)
    return f


@pytest.mark.parametrize("neuler,kt", [(0, 1), (1, 3)])
def test_oracle_dyn_nxt_adjoint_dot_product(neuler, kt):
    dom, nam, o, rng = case(neuler=neuler)
    dx = nxt_inputs(dom, rng)
    dx["ub_b"][...] = 0.0
    dx["vb_b"][...] = 0.0          # an output only: its input value is not read
    dy = nxt_forward(o, dx, kt)
    lam = {n: (rnd3 if n in NX3 else rnd2)(dom, rng) for n in NX3 + NX2}
    lam["ua_b"][...] = 0.0
    lam["va_b"][...] = 0.0         # an input only
    adj = {n: lam[n].copy(order="F") for n in NX3 + NX2}
    o.dyn_nxt_adj(kt, adj)
    lhs = sum(float((dy[n] * lam[n]).sum()) for n in NX3 + ("un_b", "vn_b", "ub_b", "vb_b"))
    rhs = sum(float((dx[n] * adj[n]).sum()) for n in NX3 + ("un_b", "vn_b", "ua_b", "va_b"))
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs), (lhs, rhs)
    assert not adj["ub_b"].any() and not adj["vb_b"].any()


# -------------------------------------------------------------------- ssh_swp
@pytest.mark.parametrize("neuler,kt", [(0, 1), (1, 3)])
def test_oracle_ssh_swp_adjoint_dot_product(neuler, kt):
    dom, nam, o, rng = case(neuler=neuler)
    dx = {n: rnd2(dom, rng) for n in ("sshb", "sshn", "ssha")}
    f = {n: dx[n].copy(order="F") for n in dx}
    for n, a in f.items():
        o.bind(n.upper(), a)
    o.ssh_swp(kt)
    lam = {n: rnd2(dom, rng) for n in ("sshb", "sshn", "ssha")}
    adj = {n: lam[n].copy(order="F") for n in lam}
    o.ssh_swp_adj(kt, adj["sshb"], adj["sshn"], adj["ssha"])
    lhs = sum(float((f[n] * lam[n]).sum()) for n in f)
    rhs = sum(float((dx[n] * adj[n]).sum()) for n in dx)
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs), (lhs, rhs)


# ------------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("neuler,kt", [(0, 1), (1, 3)])
def test_gpu_step_adjoints(neuler, kt):
    pytest.importorskip("torch")
    from harness import relerr
    from nemo_gpu import api
    dom, nam, o, rng = case(neuler=neuler, seed=9)
    nmem = 2
    ctx = api.Context(dom, nam, nmembers=nmem, prec="fp64")
    dev = lambda arrs: ctx.to_device(arrs, dtype=ctx.torch.float64)
    host = lambda t, shape: ctx.to_host(t, shape)
    _, um, vm, _ = gyre.masks(dom)
    s3, s2 = um.shape, um.shape[:2]
    # wzv
    lam = [rnd3(dom, rng) for _ in range(nmem)]
    ref_u, ref_v = [], []
    for m in range(nmem):
        ua, va, wa = np.zeros(s3, order="F"), np.zeros(s3, order="F"), lam[m].copy(order="F")
        o.wzv_adj(kt, ua, va, wa)
        ref_u.append(ua); ref_v.append(va)
    gu, gv, gw = dev([np.zeros(s3)] * nmem), dev([np.zeros(s3)] * nmem), dev(lam)
    ctx.wzv_adj(kt, gu, gv, gw)
    ctx.synchronize()
    for m in range(nmem):
        assert relerr(ref_u[m], host(gu, s3)[m], name="UN_AD") <= 1e-12
        assert relerr(ref_v[m], host(gv, s3)[m], name="VN_AD") <= 1e-12
    assert not host(gw, s3)[0].any()
    # dyn_nxt
    lams = [{n: (rnd3 if n in NX3 else rnd2)(dom, rng) for n in _ffi.NXT_ADJ} for _ in range(nmem)]
    refs = []
    for m in range(nmem):
        a = {n: lams[m][n].copy(order="F") for n in _ffi.NXT_ADJ}
        o.dyn_nxt_adj(kt, a)
        refs.append(a)
    g = {n: dev([lams[m][n] for m in range(nmem)]) for n in _ffi.NXT_ADJ}
    ctx.dyn_nxt_adj(kt, g)
    ctx.synchronize()
    for n in _ffi.NXT_ADJ:
        shape = s3 if n in NX3 else s2
        got = host(g[n], shape)
        for m in range(nmem):
            assert relerr(refs[m][n], got[m], name=n) <= 1e-12, n
    # ssh_swp
    lam = [{n: rnd2(dom, rng) for n in ("sshb", "sshn", "ssha")} for _ in range(nmem)]
    refs = []
    for m in range(nmem):
        a = {n: lam[m][n].copy(order="F") for n in lam[m]}
        o.ssh_swp_adj(kt, a["sshb"], a["sshn"], a["ssha"])
        refs.append(a)
    g = {n: dev([lam[m][n] for m in range(nmem)]) for n in ("sshb", "sshn", "ssha")}
    ctx.ssh_swp_adj(kt, g["sshb"], g["sshn"], g["ssha"])
    ctx.synchronize()
    for n in g:
        got = host(g[n], s2)
        for m in range(nmem):
            assert relerr(refs[m][n], got[m], name=n) <= 1e-12, n
