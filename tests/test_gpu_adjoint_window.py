"""The checkpointed adjoint of a GPU tracer window: the gradient of the SST cost
through torch.autograd against the oracle's FP64 tangent-linear of the same window
(with the limiter multipliers the GPU forward recorded), the checkpointing against
storing every step, and finite differences on a window without advection (where
the cost is quadratic and the frozen limiter plays no part)."""
import numpy as np
import pytest

from adj_cases import Case, GpuCase

pytestmark = pytest.mark.gpu


def make(nsteps, every, seed=21, advect=True):
    from nemo_gpu import adjoint
    c = Case("gyre", seed=seed, neuler=0)
    if not advect:
        for a in (c.zun, c.zvn, c.zwn):
            a[...] = 0.0
    g = GpuCase(c)
    torch = g.torch
    z4 = np.zeros(c.s4, order="F")
    for n in ("TSB", "TSN", "TSA"):
        g.bind(n, z4)
    win = adjoint.TracerWindow(g.ctx, g.zun, g.zvn, g.zwn, nsteps, every=every)
    t0 = g.dev(c.tsn())
    rng = np.random.default_rng([seed, 3])
    tm = c.tmask[:, :, 0]
    target = np.asfortranarray((c.tsn()[:, :, 0, 0] + 0.1 * rng.standard_normal(tm.shape)) * tm)
    target_d = torch.from_numpy(np.ascontiguousarray(target.T)).cuda()[None]
    tm_d = torch.from_numpy(np.ascontiguousarray(tm.T)).cuda()
    shape = (c.jpi, c.jpj, c.jpk)
    return c, g, win, t0, target, target_d, tm_d, shape


def host_tl_window(c, tapes, d0):
    """The oracle's tangent-linear of the window from dtb = dtn = d0."""
    dtb, dtn = d0.copy(order="F"), d0.copy(order="F")
    dta = np.zeros(c.s4, order="F")
    c.bind("TSB", dtb)
    c.bind("TSN", dtn)
    c.bind("TSA", dta)
    nam = c.nam
    for s, tape in enumerate(tapes):
        kt = c.kit + s
        p2dt = nam["rn_rdt"] if (nam["neuler"] == 0 and kt == c.kit) else 2.0 * nam["rn_rdt"]
        dta[...] = 0.0
        c.o.set_fct_tape(tape, 2)
        c.o.tra_adv_fct(kt, c.kit, "TRA", p2dt, c.zun, c.zvn, c.zwn, dtb, dtn, dta, 2, 2, 2)
        c.o.set_fct_tape(None, 0)
        c.o.tra_ldf_iso(kt, c.kit, "TRA", None, None, c.zero2, c.zero2, None, None, dtb, dtb, dta, 2, 1)
        c.o.tra_zdf_imp(kt, c.kit, "TRA", p2dt, dtb, dta, 2)
        c.o.tra_nxt(kt)
    return dtn


def test_window_gradient_against_host_tangent_linear():
    import torch
    from adj_autograd import WindowCost
    c, g, win, t0, target, target_d, tm_d, shape = make(12, every=4)
    # tapes of the forward, for the host tangent-linear
    tapes = []
    win.forward(t0, t0, tapes=tapes)
    g.ctx.synchronize()
    tapes_h = [t.cpu().numpy().copy() for t in tapes]
    x = t0.clone().requires_grad_(True)
    J = WindowCost.apply(x, win, target_d, tm_d, shape)
    J.backward()
    grad = x.grad.cpu().numpy()
    assert np.isfinite(grad).all() and np.abs(grad).max() > 0
    # directional derivative by the host tangent-linear
    rng = np.random.default_rng(5)
    d0 = np.asfortranarray(rng.standard_normal(c.s4) * c.tmask[..., None])
    dtn = host_tl_window(c, tapes_h, d0)
    _, tsn_final = win.forward(t0, t0)
    g.ctx.synchronize()
    sst = g.host(tsn_final, c.s4)[0][:, :, 0, 0]
    tm = c.tmask[:, :, 0]
    dJ = float(np.sum(2.0 * (sst - target) * tm * dtn[:, :, 0, 0]))
    gd = float(np.dot(np.ravel(d0, order="F"), grad))
    assert dJ != 0
    assert abs(gd - dJ) <= 1e-12 * abs(dJ), (gd, dJ)


def test_checkpointing_matches_storing_every_step():
    import torch
    outs = []
    for every in (1, 5, 12):
        c, g, win, t0, target, target_d, tm_d, shape = make(12, every=every)
        _, tsn = win.forward(t0, t0)
        from nemo_gpu.adjoint import sst_cost
        torch.cuda.synchronize()
        _, gJ = sst_cost(tsn, target_d, tm_d, shape)
        ab, an = win.adjoint(torch.zeros_like(gJ), gJ)
        outs.append((ab + an).cpu().numpy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


def test_window_gradient_matches_finite_differences_without_advection():
    import torch
    from adj_autograd import WindowCost
    c, g, win, t0, target, target_d, tm_d, shape = make(10, every=3, advect=False)
    x = t0.clone().requires_grad_(True)
    J = WindowCost.apply(x, win, target_d, tm_d, shape)
    J.backward()
    grad = x.grad
    rng = np.random.default_rng(8)
    d = g.dev(np.asfortranarray(rng.standard_normal(c.s4) * c.tmask[..., None]))
    eps = 1e-3
    with torch.no_grad():
        Jp = WindowCost.apply(t0 + eps * d, win, target_d, tm_d, shape).item()
        Jm = WindowCost.apply(t0 - eps * d, win, target_d, tm_d, shape).item()
    fd = (Jp - Jm) / (2 * eps)
    gd = float(torch.dot(grad, d))
    assert abs(fd - gd) <= 1e-8 * abs(gd), (fd, gd)
