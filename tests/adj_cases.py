"""Shared set-up of the adjoint tests: an oracle bound to a seeded GYRE (or shelf)
state, seeded perturbations, and the tangent-linear of each tracer routine
evaluated with the oracle (the forward routine itself for the linear ones, the
forward replaying the recorded limiter multipliers for FCT)."""
import numpy as np

from nemo_gpu import gyre, shelf
from oracle import ora


def inner(a, b):
    return float(np.dot(np.ravel(a, order="F"), np.ravel(b, order="F")))


def dot_test(lhs_parts, rhs_parts):
    """Relative mismatch of <TL x, y> (sum of lhs inner products) and <x, ADJ y>."""
    lhs = sum(inner(a, b) for a, b in lhs_parts)
    rhs = sum(inner(a, b) for a, b in rhs_parts)
    scale = max(abs(lhs), abs(rhs), 1e-300)
    return abs(lhs - rhs) / scale, lhs, rhs


class Case:
    """One oracle with the fields of the tracer routines bound."""

    def __init__(self, kind="gyre", seed=0, **nam_over):
        if kind == "gyre":
            self.dom = gyre.domain(1)
            self.nam = gyre.namelist(**nam_over)
            self.st = gyre.state(self.dom, self.nam, seed=seed)
        else:
            self.dom = shelf.domain(34, 26, jpk=21, seed=seed, e1=1000.0)
            self.nam = shelf.namelist(**nam_over)
            self.st = shelf.state(self.dom, self.nam, seed=seed)
        self.kind = kind
        self.jpi, self.jpj, self.jpk = self.dom["jpi"], self.dom["jpj"], self.dom["jpk"]
        self.s3 = (self.jpi, self.jpj, self.jpk)
        self.s4 = self.s3 + (2,)
        self.n3 = int(np.prod(self.s3))
        self.o = ora.Oracle(self.dom, self.nam)
        self.keep = {}
        for n in ("USLP", "VSLP", "WSLPI", "WSLPJ", "AVT"):
            self.bind(n, np.array(self.st[n.lower()], dtype=np.float64, order="F"))
        self.bind("AH_WSLP2", np.zeros(self.s3, order="F"))
        self.bind("AKZ", np.zeros(self.s3, order="F"))
        if not self.nam["ln_linssh"]:
            for n in ("E3T_B", "E3T_N", "E3T_A", "E3U_N", "E3V_N", "E3W_N"):
                self.bind(n, np.array(self.st[n.lower()], dtype=np.float64, order="F"))
        self.rng = np.random.default_rng([seed, 99])
        self.tmask = self.o.array("tmask", 3)
        un, vn, wn = (np.asfortranarray(self.st[k]) for k in ("un", "vn", "wn"))
        self.zun, self.zvn, self.zwn = self.o.tra_adv_trp(un, vn, wn)
        self.gtsu = np.asfortranarray(self.st.get("gtsu", np.zeros((self.jpi, self.jpj, 2))))
        self.gtsv = np.asfortranarray(self.st.get("gtsv", np.zeros((self.jpi, self.jpj, 2))))
        self.zero2 = np.zeros((self.jpi, self.jpj, 2), order="F")
        self.p2dt = 2.0 * self.nam["rn_rdt"]
        self.kit = self.nam["nit000"]

    def bind(self, name, a):
        self.keep[name] = a
        self.o.bind(name, a)

    def rand4(self, masked=True):
        x = self.rng.standard_normal(self.s4)
        if masked:
            x = x * self.tmask[..., None]
        return np.asfortranarray(x)

    def tsb(self):
        return np.array(self.st["tsb"], dtype=np.float64, order="F")

    def tsn(self):
        return np.array(self.st["tsn"], dtype=np.float64, order="F")

    # ---------------------------------------------------------- forward / TL
    def fct_record(self, tb=None, tn=None, kh=2, kv=2):
        """Forward FCT on the state, recording the limiter; returns (tape, ta)."""
        tape = np.zeros(3 * 2 * self.n3)
        self.o.set_fct_tape(tape, 1)
        ta = np.zeros(self.s4, order="F")
        self.o.tra_adv_fct(self.kit + 2, self.kit, "TRA", self.p2dt, self.zun, self.zvn, self.zwn,
                           self.tsb() if tb is None else tb, self.tsn() if tn is None else tn, ta, 2, kh, kv)
        self.o.set_fct_tape(None, 0)
        return tape, ta

    def fct_tl(self, tape, dtb, dtn, kh=2, kv=2):
        self.o.set_fct_tape(tape, 2)
        ta = np.zeros(self.s4, order="F")
        self.o.tra_adv_fct(self.kit + 2, self.kit, "TRA", self.p2dt, self.zun, self.zvn, self.zwn, dtb, dtn, ta, 2,
                           kh, kv)
        self.o.set_fct_tape(None, 0)
        return ta

    def fct_adj(self, tape, lam, kh=2, kv=2):
        tb_ad = np.zeros(self.s4, order="F")
        tn_ad = np.zeros(self.s4, order="F")
        self.o.set_fct_tape(tape, 2)
        self.o.tra_adv_fct_adj(self.kit + 2, self.kit, "TRA", self.p2dt, self.zun, self.zvn, self.zwn,
                               tb_ad, tn_ad, lam, 2, kh, kv)
        self.o.set_fct_tape(None, 0)
        return tb_ad, tn_ad

    def iso_coefficients(self):
        """kpass-1 call at kit000 so that ah_wslp2 / akz hold the slopes' values."""
        ta = np.zeros(self.s4, order="F")
        tb = self.tsb()
        self.o.tra_ldf_iso(self.kit, self.kit, "TRA", None, None, self.gtsu, self.gtsv, None, None, tb, tb, ta, 2, 1)


class GpuCase:
    """A GPU context (FP64) over the fields of a Case, for nmem copies of it."""

    def __init__(self, case, nmem=1):
        from nemo_gpu import api
        self.c = case
        self.nmem = nmem
        self.ctx = api.Context(case.dom, case.nam, nmembers=nmem, prec="fp64")
        self.torch = self.ctx.torch
        self.keep = {}
        for n in ("USLP", "VSLP", "WSLPI", "WSLPJ", "AVT"):
            self.bind(n, case.keep[n])
        for n in ("AH_WSLP2", "AKZ"):
            self.bind(n, np.zeros(case.s3, order="F"))
        if not case.nam["ln_linssh"]:
            for n in ("E3T_B", "E3T_N", "E3T_A", "E3U_N", "E3V_N", "E3W_N"):
                self.bind(n, case.keep[n])
        self.zun, self.zvn, self.zwn = (self.dev(a) for a in (case.zun, case.zvn, case.zwn))
        self.gtsu, self.gtsv = self.dev(case.gtsu), self.dev(case.gtsv)

    def dev(self, a, members=None):
        """Device tensor of nmem copies of a (or of the given list of members)."""
        return self.ctx.to_device(members if members is not None else [a] * self.nmem)

    def host(self, t, shape):
        self.ctx.synchronize()   # the context's kernels run on its own stream
        out = self.ctx.to_host(t, shape)
        return out if isinstance(out, list) else [out]

    def bind(self, name, a):
        t = self.dev(a)
        self.keep[name] = t
        self.ctx.bind(name, t)
        return t

    def iso_coefficients(self):
        tb = self.dev(self.c.tsb())
        ta = self.dev(np.zeros(self.c.s4, order="F"))
        k = self.c.kit
        self.ctx.tra_ldf_iso(k, k, "TRA", None, None, self.gtsu, self.gtsv, None, None, tb, tb, ta, 2, 1)
