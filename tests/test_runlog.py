"""The per-run metrics log (nemo_gpu/runlog.py), the counterpart of run.stat,
time.step and the timing report: on the CPU with a stand-in context (the line
layout, the sign convention of stp_ctl's zmax, the logging interval, the dia_hsb
drifts and the summary); on the GPU through the C ABI, where the logged extrema
must be those of the oracle's stp_ctl."""
import json

import numpy as np
import pytest

from nemo_gpu import _ffi
from nemo_gpu.runlog import RunLog


class FakeCtx:
    """the calls RunLog makes, with known answers"""

    def __init__(self, nmem=2):
        self.nmem = nmem
        self.syncs = 0

    def synchronize(self):
        self.syncs += 1

    def stp_ctl_result(self):
        self.syncs += 1
        z = np.array([[0.5 + m, 0.25, -34.0, 36.0, 1.0, 25.0] for m in range(self.nmem)])
        return z, np.zeros((self.nmem, _ffi.NEMO_CTL_NLOC), np.int32), np.array([0, -3][: self.nmem], np.int32)

    def dia_hsb_result(self):
        out = np.zeros((self.nmem, _ffi.NEMO_HSB_N))
        out[:, 5], out[:, 7], out[:, 8], out[:, 13] = 1e-3, 2e5, -3e2, 4e15
        return out

    def get_timing(self):
        return {"dyn_spg_ts": 4.0, "tra_adv": 2.0, "tra_ldf": 1.0, "tra_zdf": 0.5}, 2

    def get_kernel_timing(self):
        return {"spg_p2": (3.0, 2)}


def test_runlog_lines(tmp_path):
    ctx = FakeCtx()
    path = tmp_path / "run.jsonl"
    log = RunLog(ctx, str(path), cells=1000, every=2, hsb=True)
    for kt in range(1, 6):  # the first call opens the clock; lines after steps 3 and 5
        log.log(kt)
    log.close()
    lines = [json.loads(s) for s in path.read_text().splitlines()]
    assert [r.get("kt") for r in lines[:-1]] == [3, 5]
    for r in lines[:-1]:
        assert r["ms_per_step"] > 0 and r["cell_steps_per_s"] > 0
        m0, m1 = r["members"]
        assert m0["ssh_abs_max"] == 0.5 and m1["ssh_abs_max"] == 1.5
        assert m0["s_min"] == 34.0 and m0["s_max"] == 36.0  # zmax(3) is -S min
        assert m0["t_min"] == -1.0 and m0["t_max"] == 25.0
        assert (m0["kindic"], m1["kindic"]) == (0, -3)
        assert m0["zdiff_hc"] == 2e5 and m0["zvol_tot"] == 4e15
    s = lines[-1]
    assert s["summary"] and s["steps_logged"] == 4
    assert s["routine_ms_per_step"]["dyn_spg_ts"] == 2.0
    assert s["kernel_us_per_launch"]["spg_p2"] == 1500.0
    assert ctx.syncs == 3  # one to open the clock, one per line


def test_runlog_rejects_a_bad_interval(tmp_path):
    with pytest.raises(ValueError):
        RunLog(FakeCtx(), str(tmp_path / "x.jsonl"), cells=1, every=0)


@pytest.mark.gpu
def test_runlog_gpu_extrema_are_the_oracles(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from harness import Pair
    p = Pair(nn=2, prec="fp64", seed=17, nmem=2, neuler=0)
    p.bind_hotpath()
    path = tmp_path / "run.jsonl"
    cells = p.dom["jpi"] * p.dom["jpj"] * p.dom["jpk"] * p.nmem
    log = RunLog(p.ctx, str(path), cells=cells, every=1)
    log.log(4)
    for kt in (5, 6):
        for o in p.ora:
            o.stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
        p.ctx.stp_ctl(kt)
        log.log(kt)
    log.close()
    lines = [json.loads(s) for s in path.read_text().splitlines()]
    assert [r.get("kt") for r in lines[:-1]] == [5, 6]
    last = lines[-2]["members"]
    for m, o in enumerate(p.ora):
        rz, _rloc, rk = o.stp_ctl(6)
        got = last[m]
        ref = {"ssh_abs_max": rz[0], "u_abs_max": rz[1], "s_min": -rz[2], "s_max": rz[3], "t_min": -rz[4],
               "t_max": rz[5]}
        for k, v in ref.items():
            assert got[k] == pytest.approx(float(v), rel=1e-12, abs=1e-300), (m, k)
        assert got["kindic"] == int(rk)
