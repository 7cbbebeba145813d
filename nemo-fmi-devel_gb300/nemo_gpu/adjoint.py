"""Adjoint of a tracer window on the GPU, with checkpointing.

The window steps the tracer part of the hot path with the transports, the
diffusivities, the iso-neutral slopes and avt held fixed (an offline-tracer
configuration): each step kt runs, on the bound tsb / tsn / tsa of an FP64 context,

    tsa = 0; tra_adv_fct (FCT 2/2); tra_ldf_iso (or tra_ldf_lap); tra_zdf_imp; tra_nxt

as step.F90:230-257 orders them (without the salinity clamp of trazdf.F90:83, whose
derivative is 0 wherever it acts). Its adjoint runs the adjoint twins of those
routines (nemo_gpu_*_adj) in the reverse order, with each step's FCT limiter
multipliers recorded by a recomputation of the step's forward and held fixed.

Checkpointing (the two-level scheme of revolve-style adjoint drivers): the forward
sweep keeps (tsb, tsn) every `every` steps; the reverse sweep restores each segment's
checkpoint, recomputes the segment forwards while recording every step's limiter
multipliers, then runs the segment's adjoint steps backwards. Memory: the
checkpoints plus `every` tapes of 3 x 2 x jpi*jpj*jpk doubles per member; work: one
extra forward sweep.

The cost function of the window (C4 of the benchmark configurations) is
J = sum over wet surface points of (SST - target)^2 at the end of the window.
"""
from . import api


class TracerWindow:
    """A tracer window of nsteps steps from nit000 on an FP64 context.

    zun, zvn, zwn: device transports (tra_adv_fct's pun, pvn, pwn); gtsu, gtsv: the
    partial-step gradients (or None). The context must hold TSB, TSN, TSA and AVT
    bound, and for tra_ldf_iso the slopes, AH_WSLP2 and AKZ. every: steps between
    checkpoints.
    """

    def __init__(self, ctx, zun, zvn, zwn, nsteps, every=8, gtsu=None, gtsv=None):
        if ctx.prec != api._ffi.PREC_FP64:
            raise api.NemoError("the adjoint window needs an FP64 context")
        nam = ctx.nam
        if nam.get("nn_fct_h", 2) not in (0, 2) or nam.get("nn_fct_v", 2) not in (0, 2):
            raise api.NemoError("the adjoint window runs FCT 2/2")
        self.ctx, self.torch = ctx, ctx.torch
        self.zun, self.zvn, self.zwn = zun, zvn, zwn
        self.gtsu, self.gtsv = gtsu, gtsv
        self.n = nsteps
        self.every = max(1, min(every, nsteps))
        self.kit = nam["nit000"]
        self.iso = bool(nam["ln_traldf_iso"])
        for f in ("TSB", "TSN", "TSA"):
            if f not in ctx.bound:
                raise api.NemoError(f"the adjoint window needs {f} bound")
        self.tsb, self.tsn, self.tsa = ctx.bound["TSB"], ctx.bound["TSN"], ctx.bound["TSA"]
        numel = self.tsb.numel()
        self.tape_numel = 3 * numel
        self.checkpoints = {}
        # torch's own operations (zeroing, copies) are ordered with the context's
        # kernels when the context runs on torch's current stream; otherwise each
        # one is fenced by synchronisations
        st = getattr(ctx, "stream", None)
        self.same_stream = st is not None and st.cuda_stream == self.torch.cuda.current_stream().cuda_stream

    def _torch_op(self, fn):
        if self.same_stream:
            return fn()
        self.ctx.synchronize()
        out = fn()
        self.torch.cuda.synchronize()
        return out

    # ------------------------------------------------------------------ forward
    def p2dt(self, kt):
        nam = self.ctx.nam
        return nam["rn_rdt"] if (nam["neuler"] == 0 and kt == self.kit) else 2.0 * nam["rn_rdt"]

    def step(self, kt, tape=None):
        """One forward step on the bound fields; with a tape, FCT records its limiter."""
        c = self.ctx
        c.bind("FCT_TAPE", tape)
        self._torch_op(self.tsa.zero_)
        p2dt = self.p2dt(kt)
        c.tra_adv_fct(kt, self.kit, "TRA", p2dt, self.zun, self.zvn, self.zwn, self.tsb, self.tsn, self.tsa, 2, 2, 2)
        if tape is not None:
            c.bind("FCT_TAPE", None)
        if self.iso:
            c.tra_ldf_iso(kt, self.kit, "TRA", None, None, self.gtsu, self.gtsv, None, None, self.tsb, self.tsb,
                          self.tsa, 2, 1)
        else:
            c.tra_ldf_lap(kt, self.kit, "TRA", None, None, self.gtsu, self.gtsv, None, None, self.tsb, self.tsa, 2, 1)
        c.tra_zdf_imp(kt, self.kit, "TRA", p2dt, self.tsb, self.tsa, 2)
        c.tra_nxt(kt)

    def set_state(self, tsb, tsn):
        self._torch_op(lambda: (self.tsb.copy_(tsb), self.tsn.copy_(tsn)))

    def forward(self, tsb0, tsn0, tapes=None):
        """Run the window from (tsb0, tsn0), keeping the checkpoints; returns (tsb, tsn)
        at the end. With tapes (a list), every step's limiter multipliers are
        recorded and appended (for checks against a host tangent-linear)."""
        self.set_state(tsb0, tsn0)
        self.checkpoints = {}
        for s in range(self.n):
            if s % self.every == 0:
                self.checkpoints[s] = self._torch_op(lambda: (self.tsb.clone(), self.tsn.clone()))
            tape = None
            if tapes is not None:
                tape = self._torch_op(lambda: self.torch.zeros(self.tape_numel, dtype=self.torch.float64,
                                                               device=self.tsb.device))
                tapes.append(tape)
            self.step(self.kit + s, tape)
        out = self._torch_op(lambda: (self.tsb.clone(), self.tsn.clone()))
        self.ctx.synchronize()
        return out

    # ------------------------------------------------------------------ adjoint
    def adjoint_step(self, kt, tape, ab, an):
        """Adjoint of step kt: (ab, an), the adjoints of (tsb, tsn) after the step,
        become those before it."""
        c = self.ctx
        aa = self._torch_op(lambda: self.torch.zeros_like(ab))   # tsa after the step is not read later
        c.tra_nxt_adj(kt, ab, an, aa)
        p2dt = self.p2dt(kt)
        c.tra_zdf_imp_adj(kt, self.kit, "TRA", p2dt, ab, aa, 2)
        if self.iso:
            c.tra_ldf_iso_adj(kt, self.kit, "TRA", None, None, self.gtsu, self.gtsv, None, None, ab, None, aa, 2, 1)
        else:
            c.tra_ldf_lap_adj(kt, self.kit, "TRA", None, None, self.gtsu, self.gtsv, None, None, ab, aa, 2, 1)
        c.bind("FCT_TAPE", tape)
        c.tra_adv_fct_adj(kt, self.kit, "TRA", p2dt, self.zun, self.zvn, self.zwn, ab, an, aa, 2, 2, 2)
        c.bind("FCT_TAPE", None)

    def adjoint(self, ab, an):
        """Reverse sweep from the adjoints (ab, an) of the final (tsb, tsn); returns
        the adjoints of the initial (tsb0, tsn0). Uses the checkpoints of the last
        forward(); leaves the bound fields at the final state of the window."""
        if not self.checkpoints:
            raise api.NemoError("adjoint() needs a forward() first")
        torch = self.torch
        ab, an = self._torch_op(lambda: (ab.clone(), an.clone()))
        dev = self.tsb.device
        tapes = [torch.empty(self.tape_numel, dtype=torch.float64, device=dev) for _ in range(self.every)]
        starts = sorted(self.checkpoints)
        for s0 in reversed(starts):
            s1 = min(s0 + self.every, self.n)
            self.set_state(*self.checkpoints[s0])
            for s in range(s0, s1):
                self.step(self.kit + s, tapes[s - s0])
            for s in range(s1 - 1, s0 - 1, -1):
                self.adjoint_step(self.kit + s, tapes[s - s0], ab, an)
        self.ctx.synchronize()
        return ab, an


def sst_cost(tsn, target, tmask_surf, shape):
    """J = sum over wet surface points of (SST - target)^2, and dJ/dtsn (device tensors).

    tsn: (nmem * 2 * jpk * jpj * jpi) device tensor of the tracers; target: device
    tensor (nmem, jpj, jpi) of surface targets; tmask_surf: (jpj, jpi) 0/1 tensor."""
    jpi, jpj, jpk = shape
    t = tsn.view(-1, 2, jpk, jpj, jpi)
    d = (t[:, 0, 0] - target) * tmask_surf
    J = (d * d).sum()
    g = tsn.new_zeros(tsn.shape).view(-1, 2, jpk, jpj, jpi)
    g[:, 0, 0] = 2.0 * d
    return J, g.view(tsn.shape)
