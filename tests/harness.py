"""Shared set-up of the parity tests: one oracle per member and one GPU context
over the same seeded GYRE state, with the module-global fields bound on both."""
import numpy as np

from nemo_gpu import _ffi, gyre

FIELDS_3D = ("un", "vn", "wn", "ub", "vb", "ua", "va", "avt", "uslp", "vslp", "wslpi", "wslpj")
FIELDS_2D = ("sshn", "sshb", "un_b", "vn_b", "ub_b", "vb_b", "utau", "vtau", "emp")
ACC_2D = ("SSHA", "UA_B", "VA_B", "UN_ADV", "VN_ADV", "UB2_B", "VB2_B", "UN_BF", "VN_BF")
# variable volume (ln_linssh = 0): z* scale factors and depths of each state
ZSTAR = ("E3T_B", "E3T_N", "E3T_A", "E3U_N", "E3V_N", "E3W_N", "E3F_N", "HT_N", "HU_N", "HV_N",
         "R1_HU_N", "R1_HV_N", "HU_B", "HV_B", "R1_HU_B", "R1_HV_B")


# pointwise parity statistics of every compared field, by test and field name; the
# session writes them to $NEMO_PARITY_REPORT (JSON) when that is set (conftest.py)
REPORT = {}


def ordered_bits(a):
    """The FP64 values of a as integers in the order of the values (adjacent
    doubles differ by 1), so that |ordered(x) - ordered(y)| counts ulps."""
    i = np.ascontiguousarray(a, dtype=np.float64).view(np.int64)
    return np.where(i < 0, -(i & np.int64(0x7FFFFFFFFFFFFFFF)), i)


def pointwise(ref, got, floor=1e-6):
    """Pointwise statistics of got against ref: the largest |got - ref| / |ref| over
    the points with |ref| >= floor * max|ref|, the largest distance in FP64 ulps,
    and the fraction of bit-identical values."""
    ref = np.asarray(ref, dtype=np.float64).ravel()
    got = np.asarray(got, dtype=np.float64).ravel()
    if ref.size == 0:
        return {"max_rel": 0.0, "max_ulp": 0, "identical": 1.0, "n": 0}
    d = np.abs(got - ref)
    s = np.abs(ref).max()
    sel = np.abs(ref) >= floor * s if s > 0 else np.zeros(ref.shape, bool)
    max_rel = float((d[sel] / np.abs(ref[sel])).max()) if sel.any() else 0.0
    ulp = np.abs(ordered_bits(got).astype(np.float64) - ordered_bits(ref).astype(np.float64))
    return {"max_rel": max_rel, "max_ulp": float(ulp.max()), "identical": float((got == ref).mean()),
            "n": int(ref.size)}


def record(test, field, ref, got, normwise):
    st = pointwise(ref, got)
    st["normwise"] = float(normwise)
    REPORT.setdefault(test, {})[field] = st
    return st


def current_test():
    import os
    return os.environ.get("PYTEST_CURRENT_TEST", "?").split(" ")[0]


def relerr(ref, got, name=None):
    """Normwise relative error max|got - ref| / max|ref| (0 when both are 0); the
    pointwise statistics are recorded under `name` (name=False: not recorded)."""
    ref = np.asarray(ref, dtype=np.float64)
    got = np.asarray(got, dtype=np.float64)
    d = np.abs(got - ref).max() if ref.size else 0.0
    s = np.abs(ref).max() if ref.size else 0.0
    if not (np.isfinite(d) and np.isfinite(s)):  # a NaN or inf anywhere fails
        return float("inf")
    e = 0.0 if d == 0 else d / (s if s > 0 else 1.0)
    if name is not False and ref.size:
        t = current_test()
        k = name or f"value{len(REPORT.get(t, {}))}"
        record(t, k, ref, got, e)
    return e


class Pair:
    """Oracle(s) and a GPU context holding identical inputs."""

    def __init__(self, nn=1, prec="fp64", nmem=1, seed=0, states=None, jpk=31, dom=None, nam=None, sample=None,
                 **nam_over):
        from nemo_gpu import api
        from oracle import ora
        self.dom = dom or gyre.domain(nn, jpk=jpk)
        self.nam = nam or gyre.namelist(**nam_over)
        if states is not None and nmem == 1:
            nmem = len(states)  # one member per given state
        self.nmem = nmem
        self.states = states or [gyre.state(self.dom, self.nam, seed=seed, member=m) for m in range(nmem)]
        self.vvl = not self.nam["ln_linssh"]
        if self.vvl:
            for st in self.states:
                if "ht_n" not in st:
                    st.update(gyre.zstar(self.dom, st))
        # the members checked against an oracle (all by default; a sample of a large
        # ensemble): ora[i] and host[i] belong to member sample[i]
        self.sample = list(range(nmem)) if sample is None else list(sample)
        self.ora = [ora.Oracle(self.dom, self.nam) for _ in self.sample]
        self.ctx = api.Context(self.dom, self.nam, nmembers=nmem, prec=prec)
        self.torch = self.ctx.torch
        self.host = [dict() for _ in self.sample]  # arrays bound to each oracle
        self.dev = {}                                # tensors bound to the GPU context
        jpi, jpj, jpk = self.dom["jpi"], self.dom["jpj"], self.dom["jpk"]
        self.s2, self.s3, self.s4 = (jpi, jpj), (jpi, jpj, jpk), (jpi, jpj, jpk, 2)

    # -- helpers
    def to_dev(self, arrays, fp64=False):
        return self.ctx.to_device(arrays, dtype=self.torch.float64 if fp64 else None)

    def per_member(self, t, shape):
        out = self.ctx.to_host(t, shape)
        return out if isinstance(out, list) else [out]

    def bind(self, name, key=None, zero=False, shape=None, fp64=None):
        """Bind state[key] (or zeros) as field NAME on every oracle and on the GPU."""
        key = key or name.lower()
        arrs = []
        for m in range(self.nmem):
            if zero:
                a = np.zeros(shape, order="F")
            else:
                a = np.array(self.states[m][key], dtype=np.float64, order="F", copy=True)
            if m in self.sample:
                i = self.sample.index(m)
                self.host[i][name] = a
                self.ora[i].bind(name, a)
            arrs.append(a)
        if fp64 is None:
            fp64 = name in _ffi.FP64_FIELDS
        t = self.to_dev(arrs, fp64=fp64)
        self.dev[name] = t
        self.ctx.bind(name, t)
        return t

    def set(self, name, arrays):
        """New values of the bound field NAME on every member: the oracles' arrays in
        place, the device tensor by a copy ordered after the context's work and
        finished before its next call (the context's stream is not torch's)."""
        for i, m in enumerate(self.sample):
            self.host[i][name][...] = arrays[m]
        self.torch.cuda.synchronize()
        self.dev[name].copy_(self.to_dev(list(arrays), fp64=self.dev[name].dtype == self.torch.float64))
        self.torch.cuda.synchronize()

    def bind_iso(self):
        for n in ("USLP", "VSLP", "WSLPI", "WSLPJ"):
            self.bind(n)
        self.bind("AH_WSLP2", zero=True, shape=self.s3)
        self.bind("AKZ", zero=True, shape=self.s3)

    def bind_spg(self):
        for n in ("UA", "VA", "UN", "VN", "UB", "VB"):
            self.bind(n)
        for n in FIELDS_2D:
            self.bind(n.upper())
        self.bind("RCDU_BOT", key="rcdu_bot")
        for n in ACC_2D:
            self.bind(n, zero=True, shape=self.s2)
        if self.vvl:
            self.bind_zstar()

    def bind_zstar(self):
        for n in ZSTAR:
            self.bind(n)

    def bind_hotpath(self):
        self.bind("TSB", key="tsb")
        self.bind("TSN", key="tsn")
        self.bind("TSA", zero=True, shape=self.s4)
        self.bind("WN")
        self.bind("AVT")
        self.bind_iso()
        self.bind_spg()

    def compare(self, name, shape, tol, mask=None, report=None):
        """Check the GPU field NAME against every oracle member; return the worst error."""
        got = self.per_member(self.dev[name], shape)
        worst = 0.0
        exact = 0
        total = 0
        refs, gots = [], []
        for i, m in enumerate(self.sample):
            ref = self.host[i][name]
            g = got[m]
            if mask is not None:
                ref, g = ref[mask], g[mask]
            e = relerr(ref, g, name=False)
            worst = max(worst, e)
            exact += int((np.asarray(ref) == np.asarray(g)).sum())
            total += np.asarray(ref).size
            refs.append(np.asarray(ref).ravel())
            gots.append(np.asarray(g).ravel())
        record(current_test(), name, np.concatenate(refs), np.concatenate(gots), worst)
        if report is not None:
            report[name] = (worst, exact / max(total, 1))
        assert worst <= tol, f"{name}: relative error {worst:.3e} > {tol:.1e}"
        return worst
