"""Restart snapshots: a run written at step n and read into a context whose
prognostic fields were scrambled continues bit for bit (GPU); the barotropic
velocities recomputed for a restart without them match dyn_nxt's (CPU)."""
import numpy as np
import pytest

from harness import Pair
from nemo_gpu import gyre, restart


def test_barotropic_velocities_recomputed_like_dyn_nxt():
    from oracle import ora
    dom = gyre.domain(1)
    nam = gyre.namelist()
    st = gyre.state(dom, nam, seed=52)
    o = ora.Oracle(dom, nam)
    f = {}
    for n in ("ua", "va", "un", "vn", "ub", "vb", "un_b", "vn_b", "ub_b", "vb_b"):
        f[n] = np.array(st[n], dtype=np.float64, order="F")
        o.bind(n.upper(), f[n])
    z = np.zeros((dom["jpi"], dom["jpj"]), order="F")
    o.bind("UA_B", z)
    o.bind("VA_B", z.copy(order="F"))
    o.dyn_nxt(5)

    class Ctx:
        pass
    c = Ctx()
    c.dom = dom
    v = {k: f[k] for k in ("un", "vn", "ub", "vb")}
    restart._barotropic(c, v)
    for k in ("un_b", "vn_b", "ub_b", "vb_b"):
        assert np.abs(v[k] - f[k]).max() <= 1e-12 * max(np.abs(f[k]).max(), 1e-30), k


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_restart_continues_bit_for_bit(tmp_path, prec):
    import torch
    p = Pair(nn=1, prec=prec, seed=51, neuler=0)
    p.bind_hotpath()
    for kt in (1, 2, 3):
        p.ctx.stp_model(kt)
    path = str(tmp_path / "restart.npz")
    restart.rst_write(p.ctx, path, 3)
    for kt in (4, 5):
        p.ctx.stp_model(kt)
    p.ctx.synchronize()
    names = ("TSN", "TSB", "UN", "VN", "UB", "VB", "SSHN", "SSHB", "UN_B", "VN_BF")
    a = {n: p.dev[n].clone() for n in names}
    # a second context on the same coefficients, its prognostic fields scrambled
    q = Pair(nn=1, prec=prec, seed=51, neuler=0)
    q.bind_hotpath()
    for f, _ in restart.STATE.values():
        q.dev[f].normal_()
    torch.cuda.synchronize()
    kt = restart.rst_read(q.ctx, path)
    assert kt == 3
    for kt in (4, 5):
        q.ctx.stp_model(kt)
    q.ctx.synchronize()
    for n in names:
        assert torch.equal(a[n], q.dev[n]), n
    with np.load(path) as z:
        assert {"rdt", "kt", "tb", "sn", "sshn", "ub2_b", "vn_bf", "tmask", "e3t_n"} <= set(z.files)
