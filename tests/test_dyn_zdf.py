"""dyn_zdf (dynzdf.F90:47-499) with the implicit vertical viscosity, and the shared
sine of the TKE closure's Langmuir source.

On the CPU, known answers of the oracle: with no viscosity, drag or wind the solve
returns its right-hand side (the time step less the barotropic after velocity);
with viscosity and wind but no drag, the implicit diffusion conserves the column's
momentum, sum(e3u ua), up to the wind input r2dt (utau_b + utau) / (2 rau0); with
drag alone the bottom level is divided by 1 + the implicit drag. On the GPU, nemo_gpu_dyn_zdf_step
through the C ABI against the oracle, FP64 and mixed, two members."""
import numpy as np
import pytest

from harness import Pair
from nemo_gpu import gyre


def test_shared_sine_is_within_two_ulps_of_the_host_sine():
    from oracle import ora
    f = ora.lib().ora_sin_0pi
    x = np.concatenate([np.linspace(0.0, np.pi, 20001), np.pi * np.random.default_rng(3).random(20000),
                        [np.pi / 2, np.nextafter(np.pi / 2, 0), np.nextafter(np.pi / 2, 4), 3.141592653589793,
                         1e-300, 1e-8]])
    got = np.array([f(float(v)) for v in x])
    ref = np.sin(x)
    ulp = np.abs(got - ref) / np.spacing(np.maximum(np.abs(ref), 1e-300))
    assert ulp.max() <= 2.0, (ulp.max(), x[ulp.argmax()])
    assert got[0] == 0.0 and got[len(x) - 6] == 1.0


def zdf_case(seed=3, avm=1e-2, wind=1.0, drag=0.0, **over):
    """an oracle with a GYRE state, random trends ua, va, a barotropic after velocity,
    the ocean avm (avm * wmask on levels 2..jpk-1), wind and drag as asked"""
    from oracle import ora
    dom = gyre.domain(1)
    nam = gyre.namelist(**over)
    st = gyre.state(dom, nam, seed=seed)
    rng = np.random.default_rng(seed)
    tm, um, vm, wm = gyre.masks(dom)
    f = {}
    f["UB"], f["VB"] = st["ub"].copy(order="F"), st["vb"].copy(order="F")
    f["UA"] = np.asfortranarray(1e-6 * rng.standard_normal(um.shape) * um)
    f["VA"] = np.asfortranarray(1e-6 * rng.standard_normal(vm.shape) * vm)
    f["UA_B"] = np.asfortranarray(0.05 * rng.standard_normal(um.shape[:2]) * um[:, :, 0])
    f["VA_B"] = np.asfortranarray(0.05 * rng.standard_normal(vm.shape[:2]) * vm[:, :, 0])
    a = avm * (1.0 + rng.random(wm.shape)) * wm
    a[:, :, 0] = 0.0
    a[:, :, -1] = 0.0
    f["AVM"] = np.asfortranarray(a)
    f["UTAU"], f["VTAU"] = np.asfortranarray(st["utau"] * wind), np.asfortranarray(st["vtau"] * wind)
    f["RCDU_BOT"] = np.asfortranarray(drag * st["rcdu_bot"])
    o = ora.Oracle(dom, nam)
    for n, v in f.items():
        o.bind(n, v)
    return dom, nam, o, f


def rhs(dom, nam, f0, r2dt, comp="u"):
    """the time step less the barotropic after velocity, as the solve sees it"""
    tm, um, vm, wm = gyre.masks(dom)
    m = um if comp == "u" else vm
    b, a, ab = (f0["UB"], f0["UA"], f0["UA_B"]) if comp == "u" else (f0["VB"], f0["VA"], f0["VA_B"])
    x = (b + r2dt * a) * m
    x[:, :, -1] = 0.0
    x = (x - ab[:, :, None]) * m
    x[:, :, -1] = 0.0
    return x


def test_no_viscosity_returns_the_right_hand_side():
    dom, nam, o, f = zdf_case(avm=0.0, wind=0.0, drag=0.0)
    f0 = {k: v.copy() for k, v in f.items()}
    o.dyn_zdf_step(5)
    r2dt = 2 * nam["rn_rdt"]
    inner = np.zeros(f["UA"].shape, bool)
    inner[1:-1, 1:-1, :-1] = True
    for comp, n in (("u", "UA"), ("v", "VA")):
        np.testing.assert_array_equal(f[n][inner], rhs(dom, nam, f0, r2dt, comp)[inner])


@pytest.mark.parametrize("comp", ["u", "v"])
def test_viscosity_conserves_column_momentum_up_to_the_wind(comp):
    dom, nam, o, f = zdf_case(avm=5e-2, wind=1.0, drag=0.0)
    f0 = {k: v.copy() for k, v in f.items()}
    o.dyn_zdf_step(5)
    r2dt = 2 * nam["rn_rdt"]
    tm, um, vm, wm = gyre.masks(dom)
    m = um if comp == "u" else vm
    e3 = dom["e3u_0"] if comp == "u" else dom["e3v_0"]
    n, tau = ("UA", "UTAU") if comp == "u" else ("VA", "VTAU")
    before = (e3 * rhs(dom, nam, f0, r2dt, comp)).sum(axis=2)
    after = (e3 * f[n]).sum(axis=2)
    wind = r2dt * 0.5 * (2 * f0[tau]) / nam["rau0"] * m[:, :, 0]
    inner = np.zeros(before.shape, bool)
    inner[1:-1, 1:-1] = True
    scale = np.abs(e3 * rhs(dom, nam, f0, r2dt, comp)).sum(axis=2).max()
    np.testing.assert_allclose(after[inner], (before + wind)[inner], rtol=0, atol=1e-13 * scale)
    # viscosity mixes: the column's vertical spread shrinks where there is water
    assert np.abs(np.diff(f[n], axis=2))[inner].sum() < np.abs(np.diff(rhs(dom, nam, f0, r2dt, comp), axis=2))[inner].sum()


def test_implicit_drag_on_the_bottom_level():
    """Without viscosity the system is diagonal: the bottom level holds its right-hand
    side plus the explicit stress of the barotropic part, divided by 1 + the implicit
    drag (rCdU_bot < 0), every other level its right-hand side."""
    dom, nam, o, f = zdf_case(avm=0.0, wind=0.0, drag=1.0)
    f0 = {k: v.copy() for k, v in f.items()}
    o.dyn_zdf_step(5)
    r2dt = 2 * nam["rn_rdt"]
    tm, um, vm, wm = gyre.masks(dom)
    kt = dom["k_bot"]
    for comp, n, ab in (("u", "UA", "UA_B"), ("v", "VA", "VA_B")):
        x = rhs(dom, nam, f0, r2dt, comp)
        e3 = dom["e3u_0"] if comp == "u" else dom["e3v_0"]
        rc0 = f0["RCDU_BOT"]
        for i in range(1, dom["jpi"] - 1):
            for j in range(1, dom["jpj"] - 1):
                ni, nj = (i + 1, j) if comp == "u" else (i, j + 1)
                kb = max(min(kt[i, j], kt[ni, nj]), 1) - 1 if min(kt[i, j], kt[ni, nj]) > 0 else 0
                rc = rc0[ni, nj] + rc0[i, j]
                want = x[i, j].copy()
                want[kb] = want[kb] + r2dt * 0.5 * rc * f0[ab][i, j] / e3[i, j, kb]
                want[kb] = want[kb] / (1.0 - r2dt * 0.5 * rc / e3[i, j, kb])
                np.testing.assert_array_equal(f[n][i, j, :-1], want[:-1])
                if um[i, j, 0] > 0 and comp == "u":
                    assert abs(f[n][i, j, kb]) <= abs(x[i, j, kb] + r2dt * 0.5 * rc * f0[ab][i, j] / e3[i, j, kb])


# ------------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_dyn_zdf_implicit(prec):
    """nemo_gpu_dyn_zdf_step with the ocean viscosity bound, kt = 5 (leap-frog) and
    kt = 1 of an Euler start, two members."""
    pytest.importorskip("torch")
    for kt, neuler in ((5, 1), (1, 0)):
        p = Pair(nn=2, prec=prec, seed=21, nmem=2, neuler=neuler)
        tm, um, vm, wm = gyre.masks(p.dom)
        for m, st in enumerate(p.states):
            rng = np.random.default_rng(100 + m)
            a = 2e-2 * (1.0 + rng.random(wm.shape)) * wm
            a[:, :, 0] = 0.0
            a[:, :, -1] = 0.0
            st["avm"] = np.asfortranarray(a)
            st["ua"] = np.asfortranarray(1e-6 * rng.standard_normal(um.shape) * um)
            st["va"] = np.asfortranarray(1e-6 * rng.standard_normal(vm.shape) * vm)
            st["ua_b"] = np.asfortranarray(0.05 * rng.standard_normal(um.shape[:2]) * um[:, :, 0])
            st["va_b"] = np.asfortranarray(0.05 * rng.standard_normal(vm.shape[:2]) * vm[:, :, 0])
        for n in ("UA", "VA", "UB", "VB", "AVM", "UA_B", "VA_B", "UTAU", "VTAU"):
            p.bind(n)
        p.bind("RCDU_BOT", key="rcdu_bot")
        for o in p.ora:
            o.dyn_zdf_step(kt)
        p.ctx.dyn_zdf_step(kt)
        p.ctx.synchronize()
        tol = 1e-12 if prec == "fp64" else 2e-5
        p.compare("UA", p.s3, tol)
        p.compare("VA", p.s3, tol)
