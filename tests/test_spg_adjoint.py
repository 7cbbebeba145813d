"""Adjoint of the split-explicit free surface, dyn_spg_ts (dynspg_ts.F90:121-1310),
for the linear free surface with ln_bt_fw and ln_bt_av.

The forward is affine in the state (the forcing is the constant part), so the
tangent-linear is the forward itself with the forcing set to zero. On the CPU: the
oracle adjoint against that tangent-linear by the dot-product test <M dx, l> =
<dx, M^T l> over every input and output of the call, for the ENE, ENS, EEN and MIX
schemes, at an Euler first step and a leap-frog step. On the GPU: the adjoint
through the C ABI against the oracle adjoint (1e-12) and the same dot-product test
with the oracle's tangent-linear, one and two members."""
import numpy as np
import pytest

from nemo_gpu import _ffi, gyre

F = np.asfortranarray
IN3 = ("ua", "va", "un", "vn")
INOUT2 = ("ub2_b", "vb2_b", "un_bf", "vn_bf")
IN2 = ("sshn", "un_b", "vn_b", "ub_b", "vb_b")
OUT2 = ("ssha", "ua_b", "va_b", "un_adv", "vn_adv")
FORCING = ("UTAU", "VTAU", "EMP")


def tl_oracle(dom, nam):
    """An oracle whose bound fields hold a perturbation; forcing zero, drag fixed."""
    from oracle import ora
    o = ora.Oracle(dom, nam)
    st = gyre.state(dom, nam, seed=11)
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    f = {}
    for n in IN3 + ("ub", "vb"):
        f[n.upper()] = np.zeros((jpi, jpj, jpk), order="F")
    for n in INOUT2 + IN2 + OUT2 + ("sshb",):
        f[n.upper()] = np.zeros((jpi, jpj), order="F")
    for n in FORCING:
        f[n] = np.zeros((jpi, jpj), order="F")
    f["RCDU_BOT"] = F(st["rcdu_bot"])
    for n, a in f.items():
        o.bind(n, a)
    return o, f


def perturbation(dom, rng):
    tm, um, vm, _ = gyre.masks(dom)
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    d = {}
    d["ua"], d["va"] = F(1e-6 * rng.standard_normal(um.shape) * um), F(1e-6 * rng.standard_normal(vm.shape) * vm)
    d["un"], d["vn"] = F(0.1 * rng.standard_normal(um.shape) * um), F(0.1 * rng.standard_normal(vm.shape) * vm)
    ssm = tm.max(axis=2)
    d["sshn"] = F(0.1 * rng.standard_normal((jpi, jpj)) * ssm)
    for n in ("un_b", "ub_b", "ub2_b", "un_bf"):
        d[n] = F(0.05 * rng.standard_normal((jpi, jpj)) * um.max(axis=2))
    for n in ("vn_b", "vb_b", "vb2_b", "vn_bf"):
        d[n] = F(0.05 * rng.standard_normal((jpi, jpj)) * vm.max(axis=2))
    for n in ("ub2_b", "un_bf"):
        d[n] = F(d[n] * 100.0)                  # transports: velocity x depth
    for n in ("vb2_b", "vn_bf"):
        d[n] = F(d[n] * 100.0)
    return d


def tangent_linear(o, f, dx, kt):
    for n in IN3 + INOUT2 + IN2:
        f[n.upper()][...] = dx[n]
    for n in OUT2:
        f[n.upper()][...] = 0.0
    o.dyn_spg_ts(kt)
    return {n: f[n.upper()].copy() for n in IN3 + INOUT2 + OUT2}


def cotangent(dom, rng):
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    lam = {n: F(rng.standard_normal((jpi, jpj, jpk))) for n in IN3}
    lam.update({n: F(rng.standard_normal((jpi, jpj))) for n in INOUT2 + OUT2})
    return lam


def adjoint_arrays(dom, lam):
    jpi, jpj = dom["jpi"], dom["jpj"]
    a = {n: F(lam[n].copy()) for n in IN3 + INOUT2 + OUT2}
    a.update({n: np.zeros((jpi, jpj), order="F") for n in IN2})
    return a


def dot_sides(dx, dy, lam, adj):
    lhs = sum(float((dy[n] * lam[n]).sum()) for n in dy)
    rhs = sum(float((dx[n] * adj[n]).sum()) for n in IN3 + INOUT2 + IN2)
    return lhs, rhs


@pytest.mark.parametrize("sc", [1, 0, 4, 5])
@pytest.mark.parametrize("euler", [True, False])
def test_oracle_spg_adjoint_dot_product(sc, euler):
    dom = gyre.domain(1)
    nam = gyre.namelist(nvor_scheme=sc, neuler=0 if euler else 1)
    o, f = tl_oracle(dom, nam)
    rng = np.random.default_rng([sc, int(euler)])
    if not euler:
        tangent_linear(o, f, perturbation(dom, rng), 1)   # the weights of nit000
    kt = 1 if euler else 3
    dx = perturbation(dom, rng)
    dy = tangent_linear(o, f, dx, kt)
    lam = cotangent(dom, rng)
    adj = adjoint_arrays(dom, lam)
    o.dyn_spg_ts_adj(kt, adj)
    lhs, rhs = dot_sides(dx, dy, lam, adj)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    for n in OUT2:
        assert not adj[n].any()


@pytest.mark.parametrize("sc", [1, 4])
def test_oracle_spg_adjoint_of_the_sub_steps_alone(sc):
    """Only the barotropic path: dx in sshn, un_b, vn_b and l on ssha, ua_b, va_b,
    un_adv, vn_adv, so no identity term of the 3-D fields hides the sub-steps."""
    dom = gyre.domain(1)
    nam = gyre.namelist(nvor_scheme=sc, neuler=1)
    o, f = tl_oracle(dom, nam)
    rng = np.random.default_rng([sc, 7])
    tangent_linear(o, f, perturbation(dom, rng), 1)
    dx = {n: np.zeros_like(a) for n, a in perturbation(dom, rng).items()}
    full = perturbation(dom, rng)
    for n in ("sshn", "un_b", "vn_b"):
        dx[n] = full[n]
    dy = tangent_linear(o, f, dx, 3)
    lam = {n: np.zeros_like(a) for n, a in cotangent(dom, rng).items()}
    full = cotangent(dom, rng)
    for n in OUT2:
        lam[n] = full[n]
    adj = adjoint_arrays(dom, lam)
    o.dyn_spg_ts_adj(3, adj)
    lhs, rhs = dot_sides(dx, dy, lam, adj)
    assert abs(lhs) > 0 and abs(lhs - rhs) <= 1e-13 * abs(lhs), (lhs, rhs)


def test_oracle_spg_adjoint_refuses_what_it_does_not_cover():
    from oracle import ora
    dom = gyre.domain(1)
    for over in (dict(nvor_scheme=2), dict(ln_bt_av=0), dict(ln_bt_fw=0)):
        nam = gyre.namelist(**over)
        o, f = tl_oracle(dom, nam)
        adj = adjoint_arrays(dom, cotangent(dom, np.random.default_rng(1)))
        with pytest.raises(RuntimeError):
            o.dyn_spg_ts_adj(1, adj)


# ------------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("sc,nmem,euler", [(1, 1, True), (1, 2, False), (4, 2, False), (0, 1, False)])
def test_gpu_spg_adjoint(sc, nmem, euler):
    pytest.importorskip("torch")
    from harness import Pair, relerr
    dom = gyre.domain(2)
    nam = gyre.namelist(nvor_scheme=sc, neuler=0 if euler else 1)
    kt = 1 if euler else 3
    # the GPU context, with its forward run at nit000 (and kt) for the weights
    p = Pair(dom=dom, nam=nam, prec="fp64", nmem=nmem, seed=21)
    p.bind_spg()
    p.ctx.dyn_spg_ts(1)
    if kt != 1:
        p.ctx.dyn_spg_ts(kt)
    o, f = tl_oracle(dom, nam)
    p.set("RCDU_BOT", [f["RCDU_BOT"]] * nmem)   # one drag coefficient for both
    rng = np.random.default_rng([sc, nmem])
    if not euler:
        tangent_linear(o, f, perturbation(dom, rng), 1)
    dxs, dys, lams, ora_adj = [], [], [], []
    for m in range(nmem):
        dx = perturbation(dom, rng)
        dys.append(tangent_linear(o, f, dx, kt))
        dxs.append(dx)
        lam = cotangent(dom, rng)
        lams.append(lam)
        a = adjoint_arrays(dom, lam)
        o.dyn_spg_ts_adj(kt, a)
        ora_adj.append(a)
    gadj = {}
    for n in _ffi.SPG_ADJ:
        arrs = [adjoint_arrays(dom, lams[m])[n] for m in range(nmem)]
        gadj[n] = p.to_dev(arrs, fp64=True)
    p.ctx.dyn_spg_ts_adj(kt, gadj)
    p.ctx.synchronize()
    for n in _ffi.SPG_ADJ:
        shape = ora_adj[0][n].shape
        got = p.per_member(gadj[n], shape)
        for m in range(nmem):
            assert relerr(ora_adj[m][n], got[m], name=n) <= 1e-12, n
    for m in range(nmem):
        got = {n: p.per_member(gadj[n], ora_adj[0][n].shape)[m] for n in _ffi.SPG_ADJ}
        lhs, rhs = dot_sides(dxs[m], dys[m], lams[m], got)
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)
