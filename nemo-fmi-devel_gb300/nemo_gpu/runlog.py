"""Per-run metrics as JSON lines: the counterpart of the reference's run.stat and
time.step (stpctl.F90:80-81, :106-109, written by stp_ctl every step), of its
timing report (timing.F90:89-212) and of the dia_hsb drifts it prints
(diahsb.F90:192-206).

``RunLog(ctx, path, cells, every)`` is handed the context after each step with
``log(kt)``. Every ``every`` steps it synchronises once and writes one line: the
step index, the wall time per step since the previous line and the cell-steps/s
it gives, and per member the extrema of the last stp_ctl (|ssh| max, |U| max,
S min/max, T min/max, kindic) and, when dia_hsb runs, its volume, heat and salt
drifts. ``close()`` writes a summary line with the per-routine and per-kernel
device times when the context's timing is on. Between logged steps nothing is
synchronised, so the log does not stall the pipeline of a run.
"""
import json
import time

# names of stp_ctl's zmax(1:6) (stpctl.F90:112-127) as the log reports them: the
# reference stores -S min and -T min
_CTL = ("ssh_abs_max", "u_abs_max", "s_min", "s_max", "t_min", "t_max")
_NEGATED = {"s_min", "t_min"}
# dia_hsb terms of nemo_gpu_dia_hsb_result reported in the log
_HSB = {"zdiff_v1": 5, "zdiff_hc": 7, "zdiff_sc": 8, "zvol_tot": 13}


class RunLog:
    def __init__(self, ctx, path, cells, every=1, hsb=False):
        if every < 1:
            raise ValueError("every must be >= 1")
        self.ctx, self.cells, self.every, self.hsb = ctx, cells, int(every), bool(hsb)
        self.f = open(path, "w")
        self.n = 0
        self.t0 = None

    def _line(self, rec):
        self.f.write(json.dumps(rec) + "\n")
        self.f.flush()

    def log(self, kt):
        """Call after each step kt (the step's stp_ctl has been enqueued)."""
        self.n += 1
        if self.t0 is None:  # the first call opens the clock
            self.ctx.synchronize()
            self.t0, self.n = time.perf_counter(), 0
            return
        if self.n % self.every:
            return
        zmax, _loc, kindic = self.ctx.stp_ctl_result()  # synchronises
        now = time.perf_counter()
        ms = 1e3 * (now - self.t0) / self.every
        self.t0 = now
        members = []
        for m in range(len(kindic)):
            rec = {k: (-float(zmax[m][i]) if k in _NEGATED else float(zmax[m][i])) for i, k in enumerate(_CTL)}
            rec["kindic"] = int(kindic[m])
            members.append(rec)
        if self.hsb:
            out = self.ctx.dia_hsb_result()
            for m, rec in enumerate(members):
                rec.update({k: float(out[m][i]) for k, i in _HSB.items()})
        self._line({"kt": int(kt), "ms_per_step": ms, "cell_steps_per_s": self.cells / (ms / 1e3),
                    "members": members})

    def close(self):
        rec = {"summary": True, "steps_logged": self.n}
        try:
            rt, ncalls = self.ctx.get_timing()
            if ncalls:
                rec["routine_ms_per_step"] = {k: v / ncalls for k, v in rt.items()}
                kt = self.ctx.get_kernel_timing()
                rec["kernel_us_per_launch"] = {k: 1e3 * ms / n for k, (ms, n) in kt.items() if n}
        except Exception as e:  # timing not available: the summary says so
            rec["timing"] = f"unavailable: {e}"
        self._line(rec)
        self.f.close()
