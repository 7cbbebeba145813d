"""ctypes wrapper of the oracle library (test infrastructure only).

Mirrors the C ABI of include/nemo_gpu.h on host numpy arrays (one member).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "nemo-fmi-devel_gb300"))
from nemo_gpu import _ffi  # noqa: E402

from . import build as _build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build())
        vp, i, d, cp = C.c_void_p, C.c_int, C.c_double, C.c_char_p
        def P(name, argtypes, restype=C.c_int):
            f = getattr(L, name)
            f.argtypes, f.restype = argtypes, restype
        P("ora_create", [C.POINTER(_ffi.DomDesc), C.POINTER(_ffi.Namelist), C.POINTER(vp)])
        P("ora_destroy", [vp])
        P("ora_bind", [vp, i, vp])
        P("ora_spg_info", [vp, C.POINTER(i), C.POINTER(i), C.POINTER(d)])
        P("ora_array", [vp, cp], C.POINTER(C.c_double))
        P("ora_iarray", [vp, cp], C.POINTER(C.c_int))
        P("ora_tra_adv_trp", [vp, vp, vp, vp, vp, vp, vp])
        P("ora_tra_adv_fct", [vp, i, i, cp, d, vp, vp, vp, vp, vp, vp, i, i, i])
        P("ora_interp_4th_cpt", [vp, vp, vp])
        P("ora_interp_4th_cpt_adj", [vp, vp, vp])
        P("ora_tra_ldf_lap", [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
        P("ora_tra_ldf_iso", [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
        P("ora_tra_zdf_imp", [vp, i, i, cp, d, vp, vp, i])
        P("ora_tra_zdf", [vp, i])
        P("ora_dyn_spg_ts", [vp, i])
        P("ora_lbc_lnk", [vp, vp, i, i, C.c_char, d, d])
        P("ora_glob_sum", [vp, vp, i, C.POINTER(d)])
        P("ora_stp_hotpath", [vp, i])
        P("ora_set_poison", [i], None)
        P("ora_set_threads", [i])
        P("ora_stp_ctl", [vp, i, vp, vp, C.POINTER(i)])
        P("ora_zdf_phy", [vp, i])
        P("ora_sin_0pi", [d], d)
        P("ora_sin", [d], d)
        P("ora_cos", [d], d)
        P("ora_usrdef_sbc", [vp, i])
        P("ora_dia_hsb_init", [vp])
        P("ora_dia_hsb", [vp, i, vp])
        P("ora_stp_ctl_last", [vp, vp, vp, C.POINTER(i)])
        P("ora_dia_hsb_last", [vp, vp])
        P("ora_set_fct_tape", [vp, vp, i])
        P("ora_tra_adv_fct_adj", [vp, i, i, cp, d, vp, vp, vp, vp, vp, vp, i, i, i])
        P("ora_tra_ldf_lap_adj", [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
        P("ora_tra_ldf_iso_adj", [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
        P("ora_tra_zdf_imp_adj", [vp, i, i, cp, d, vp, vp, i])
        P("ora_tra_nxt", [vp, i])
        P("ora_tra_nxt_adj", [vp, i, vp, vp, vp])
        P("ora_dyn_spg_ts_adj", [vp, i, C.POINTER(_ffi.SpgAdj)])
        P("ora_dyn_nxt_adj", [vp, i, C.POINTER(_ffi.NxtAdj)])
        P("ora_wzv_adj", [vp, i, vp, vp, vp])
        P("ora_ssh_swp_adj", [vp, i, vp, vp, vp])
        for name in ("ora_wzv", "ora_dyn_zdf_step", "ora_dyn_nxt", "ora_ssh_swp", "ora_dom_vvl_sf_nxt",
                     "ora_dom_vvl_sf_swp", "ora_stp_model", "ora_tra_sbc", "ora_tra_qsr"):
            P(name, [vp, i])
        P("ora_ldf_slp", [vp, i, vp, vp])
        P("ora_ldf_slp_triad", [vp, i, vp])
        P("ora_tra_ldf_triad", [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
        P("ora_nksr", [vp], C.c_int)
        P("ora_eos_insitu", [vp, vp, vp, vp])
        P("ora_eos_insitu_pot", [vp, vp, vp, vp, vp])
        P("ora_rab_3d", [vp, vp, vp])
        P("ora_bn2", [vp, vp, vp, vp])
        P("ora_dyn_hpg", [vp, i])
        P("ora_zdf_mxl", [vp, i])
        P("ora_nlb10", [vp], C.c_int)
        P("ora_dyn_ldf_lap", [vp, i, vp, vp, vp, vp, i])
        P("ora_vor_ene", [vp, i, i, vp, vp, vp, vp])
        P("ora_dyn_keg", [vp, i, i])
        P("ora_dyn_zad", [vp, i])
        P("ora_tra_ldf_blp", [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
        P("ora_zps_hde", [vp, i, i, vp, vp, vp])
        P("ora_zps_hde_rd", [vp, i, vp, vp, vp, vp])
        _lib = L
    return _lib


def set_poison(on):
    """Start the oracle's automatic-array work buffers as NaN (1) or 0 (0)."""
    lib().ora_set_poison(int(on))


def set_threads(n):
    """OpenMP threads of the oracle's parallel loops (n < 1: unchanged); returns the setting."""
    return lib().ora_set_threads(int(n))


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim == 1), "oracle arrays: float64 Fortran order"
    return a.ctypes.data


class Oracle:
    """One oracle context (one member)."""

    def __init__(self, dom, nam):
        self.dom, self.nam = dom, nam
        self._desc = _ffi.make_desc(dom)
        self._nl = _ffi.make_namelist(nam)
        h = C.c_void_p()
        st = lib().ora_create(C.byref(self._desc), C.byref(self._nl), C.byref(h))
        if st:
            raise RuntimeError(f"ora_create failed ({st})")
        self.h = h
        self.bound = {}
        self.jpi, self.jpj, self.jpk = dom["jpi"], dom["jpj"], dom["jpk"]

    def close(self):
        if self.h:
            lib().ora_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def bind(self, name, arr):
        """Bind a float64 Fortran-order array to a module-global field (kept alive here);
        NMLN, the mixed-layer level, is an int32 array."""
        self.bound[name] = arr
        if name == "NMLN":
            assert arr.dtype == np.int32 and arr.flags.f_contiguous
            st = lib().ora_bind(self.h, _ffi.F[name], arr.ctypes.data)
        else:
            st = lib().ora_bind(self.h, _ffi.F[name], _p(arr))
        assert st == 0

    def spg_info(self):
        ic, nb, dt = C.c_int(), C.c_int(), C.c_double()
        lib().ora_spg_info(self.h, C.byref(ic), C.byref(nb), C.byref(dt))
        return ic.value, nb.value, dt.value

    def array(self, name, ndim=2):
        p = lib().ora_array(self.h, name.encode())
        if not p:
            raise KeyError(name)
        if name.startswith("wgtbtp"):
            n = 3 * self.spg_info()[1]
            return np.ctypeslib.as_array(p, shape=(n,)).copy()
        shape = (self.jpi, self.jpj, self.jpk) if ndim == 3 else (self.jpi, self.jpj)
        n = int(np.prod(shape))
        return np.ctypeslib.as_array(p, shape=(n,)).copy().reshape(shape, order="F")

    def iarray(self, name):
        p = lib().ora_iarray(self.h, name.encode())
        return np.ctypeslib.as_array(p, shape=(self.jpi * self.jpj,)).copy().reshape((self.jpi, self.jpj), order="F")

    def _ck(self, st, what):
        if st != 0:
            raise RuntimeError(f"{what} failed with status {st}")

    def tra_adv_trp(self, un, vn, wn):
        out = [np.zeros_like(un, order="F") for _ in range(3)]
        self._ck(lib().ora_tra_adv_trp(self.h, _p(un), _p(vn), _p(wn), *[_p(o) for o in out]), "tra_adv_trp")
        return out

    def tra_adv_fct(self, kt, kit000, cdtype, p2dt, pun, pvn, pwn, ptb, ptn, pta, kjpt, kh, kv):
        self._ck(lib().ora_tra_adv_fct(self.h, kt, kit000, cdtype.encode(), p2dt, _p(pun), _p(pvn), _p(pwn),
                                       _p(ptb), _p(ptn), _p(pta), kjpt, kh, kv), "tra_adv_fct")

    def interp_4th_cpt(self, pt_in):
        out = np.zeros_like(pt_in, order="F")
        self._ck(lib().ora_interp_4th_cpt(self.h, _p(pt_in), _p(out)), "interp_4th_cpt")
        return out

    def interp_4th_cpt_adj(self, pv, pt_ad):
        """pt_ad += the adjoint of interp_4th_cpt applied to pv"""
        self._ck(lib().ora_interp_4th_cpt_adj(self.h, _p(pv), _p(pt_ad)), "interp_4th_cpt_adj")
    def tra_ldf_lap(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, pta, kjpt, kpass):
        self._ck(lib().ora_tra_ldf_lap(self.h, kt, kit000, cdtype.encode(), _p(pahu), _p(pahv), _p(pgu), _p(pgv),
                                       _p(pgui), _p(pgvi), _p(ptb), _p(pta), kjpt, kpass), "tra_ldf_lap")

    def tra_ldf_iso(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, ptbb, pta, kjpt, kpass):
        self._ck(lib().ora_tra_ldf_iso(self.h, kt, kit000, cdtype.encode(), _p(pahu), _p(pahv), _p(pgu), _p(pgv),
                                       _p(pgui), _p(pgvi), _p(ptb), _p(ptbb), _p(pta), kjpt, kpass), "tra_ldf_iso")

    def tra_zdf_imp(self, kt, kit000, cdtype, p2dt, ptb, pta, kjpt):
        self._ck(lib().ora_tra_zdf_imp(self.h, kt, kit000, cdtype.encode(), p2dt, _p(ptb), _p(pta), kjpt),
                 "tra_zdf_imp")

    def tra_zdf(self, kt):
        self._ck(lib().ora_tra_zdf(self.h, kt), "tra_zdf")

    def dyn_spg_ts(self, kt):
        self._ck(lib().ora_dyn_spg_ts(self.h, kt), "dyn_spg_ts")

    def lbc_lnk(self, a, nat, pval=0.0):
        nk = 1 if a.ndim == 2 else int(np.prod(a.shape[2:]))
        self._ck(lib().ora_lbc_lnk(self.h, _p(a), nk, 1, nat.encode(), 1.0, pval), "lbc_lnk")

    def glob_sum(self, a):
        nk = 1 if a.ndim == 2 else a.shape[2]
        out = C.c_double()
        self._ck(lib().ora_glob_sum(self.h, _p(a), nk, C.byref(out)), "glob_sum")
        return out.value

    def stp_hotpath(self, kt):
        self._ck(lib().ora_stp_hotpath(self.h, kt), "stp_hotpath")

    def usrdef_sbc(self, kt):
        self._ck(lib().ora_usrdef_sbc(self.h, kt), "usrdef_sbc")

    def zdf_phy(self, kt):
        self._ck(lib().ora_zdf_phy(self.h, kt), "zdf_phy")

    # ---------------------------------------------------------------- stp_ctl, dia_hsb
    def stp_ctl(self, kt):
        """(zmax[6], loc[11], kindic) of stpctl.F90:112-184 on the bound fields"""
        z = np.zeros(_ffi.NEMO_CTL_N)
        loc = np.zeros(_ffi.NEMO_CTL_NLOC, dtype=np.int32)
        k = C.c_int(0)
        self._ck(lib().ora_stp_ctl(self.h, kt, _p(z), loc.ctypes.data, C.byref(k)), "stp_ctl")
        return z, loc, k.value

    def stp_ctl_last(self):
        z = np.zeros(_ffi.NEMO_CTL_N)
        loc = np.zeros(_ffi.NEMO_CTL_NLOC, dtype=np.int32)
        k = C.c_int(0)
        self._ck(lib().ora_stp_ctl_last(self.h, _p(z), loc.ctypes.data, C.byref(k)), "stp_ctl_last")
        return z, loc, k.value

    def dia_hsb_init(self):
        self._ck(lib().ora_dia_hsb_init(self.h), "dia_hsb_init")

    def dia_hsb(self, kt):
        out = np.zeros(_ffi.NEMO_HSB_N)
        self._ck(lib().ora_dia_hsb(self.h, kt, _p(out)), "dia_hsb")
        return out

    def dia_hsb_last(self):
        out = np.zeros(_ffi.NEMO_HSB_N)
        self._ck(lib().ora_dia_hsb_last(self.h, _p(out)), "dia_hsb_last")
        return out

    # ---------------------------------------------------------------- adjoint
    def set_fct_tape(self, tape, mode):
        """mode 1: tra_adv_fct records its limiter multipliers into tape; 2: replays
        them (the tangent-linear with the limiter frozen); 0: neither."""
        self._fct_tape = tape
        self._ck(lib().ora_set_fct_tape(self.h, _p(tape) if tape is not None else None, mode), "set_fct_tape")

    def tra_adv_fct_adj(self, kt, kit000, cdtype, p2dt, pun, pvn, pwn, ptb_ad, ptn_ad, pta_ad, kjpt, kh, kv):
        self._ck(lib().ora_tra_adv_fct_adj(self.h, kt, kit000, cdtype.encode(), p2dt, _p(pun), _p(pvn), _p(pwn),
                                           _p(ptb_ad), _p(ptn_ad), _p(pta_ad), kjpt, kh, kv), "tra_adv_fct_adj")

    def tra_ldf_lap_adj(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb_ad, pta_ad, kjpt, kpass):
        self._ck(lib().ora_tra_ldf_lap_adj(self.h, kt, kit000, cdtype.encode(), _p(pahu), _p(pahv), _p(pgu),
                                           _p(pgv), _p(pgui), _p(pgvi), _p(ptb_ad), _p(pta_ad), kjpt, kpass),
                 "tra_ldf_lap_adj")

    def tra_ldf_iso_adj(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb_ad, ptbb_ad, pta_ad, kjpt,
                        kpass):
        self._ck(lib().ora_tra_ldf_iso_adj(self.h, kt, kit000, cdtype.encode(), _p(pahu), _p(pahv), _p(pgu),
                                           _p(pgv), _p(pgui), _p(pgvi), _p(ptb_ad), _p(ptbb_ad), _p(pta_ad), kjpt,
                                           kpass), "tra_ldf_iso_adj")

    def tra_zdf_imp_adj(self, kt, kit000, cdtype, p2dt, ptb_ad, pta_ad, kjpt):
        self._ck(lib().ora_tra_zdf_imp_adj(self.h, kt, kit000, cdtype.encode(), p2dt, _p(ptb_ad), _p(pta_ad), kjpt),
                 "tra_zdf_imp_adj")

    def tra_nxt(self, kt):
        self._ck(lib().ora_tra_nxt(self.h, kt), "tra_nxt")

    def wzv_adj(self, kt, un_ad, vn_ad, wn_ad):
        self._ck(lib().ora_wzv_adj(self.h, kt, _p(un_ad), _p(vn_ad), _p(wn_ad)), "wzv_adj")

    def dyn_nxt_adj(self, kt, adj):
        s = _ffi.NxtAdj(*[_p(adj[n]) for n in _ffi.NXT_ADJ])
        self._ck(lib().ora_dyn_nxt_adj(self.h, kt, C.byref(s)), "dyn_nxt_adj")

    def ssh_swp_adj(self, kt, sshb_ad, sshn_ad, ssha_ad):
        self._ck(lib().ora_ssh_swp_adj(self.h, kt, _p(sshb_ad), _p(sshn_ad), _p(ssha_ad)), "ssh_swp_adj")

    def dyn_spg_ts_adj(self, kt, adj):
        """adj: dict of FP64 Fortran-order arrays keyed by the members of nemo_spg_adj."""
        s = _ffi.SpgAdj(*[_p(adj[n]) for n in _ffi.SPG_ADJ])
        self._ck(lib().ora_dyn_spg_ts_adj(self.h, kt, C.byref(s)), "dyn_spg_ts_adj")

    def tra_nxt_adj(self, kt, tsb_ad, tsn_ad, tsa_ad):
        self._ck(lib().ora_tra_nxt_adj(self.h, kt, _p(tsb_ad), _p(tsn_ad), _p(tsa_ad)), "tra_nxt_adj")

    # ------------------------------------------------------- rest of the step
    def wzv(self, kt):
        self._ck(lib().ora_wzv(self.h, kt), "wzv")

    def dyn_zdf_step(self, kt):
        self._ck(lib().ora_dyn_zdf_step(self.h, kt), "dyn_zdf_step")

    def dyn_nxt(self, kt):
        self._ck(lib().ora_dyn_nxt(self.h, kt), "dyn_nxt")

    def ssh_swp(self, kt):
        self._ck(lib().ora_ssh_swp(self.h, kt), "ssh_swp")

    def dom_vvl_sf_nxt(self, kt):
        self._ck(lib().ora_dom_vvl_sf_nxt(self.h, kt), "dom_vvl_sf_nxt")

    def dom_vvl_sf_swp(self, kt):
        self._ck(lib().ora_dom_vvl_sf_swp(self.h, kt), "dom_vvl_sf_swp")

    def stp_model(self, kt):
        self._ck(lib().ora_stp_model(self.h, kt), "stp_model")

    def tra_sbc(self, kt):
        self._ck(lib().ora_tra_sbc(self.h, kt), "tra_sbc")

    def tra_qsr(self, kt):
        self._ck(lib().ora_tra_qsr(self.h, kt), "tra_qsr")

    def eos_insitu(self, pts, prd, pdep):
        self._ck(lib().ora_eos_insitu(self.h, _p(pts), _p(prd), _p(pdep)), "eos_insitu")

    def eos_insitu_pot(self, pts, prd, prhop, pdep):
        self._ck(lib().ora_eos_insitu_pot(self.h, _p(pts), _p(prd), _p(prhop), _p(pdep)), "eos_insitu_pot")

    def rab_3d(self, pts, pab):
        self._ck(lib().ora_rab_3d(self.h, _p(pts), _p(pab)), "rab_3d")

    def bn2(self, pts, pab, pn2):
        self._ck(lib().ora_bn2(self.h, _p(pts), _p(pab), _p(pn2)), "bn2")

    def dyn_hpg(self, kt):
        self._ck(lib().ora_dyn_hpg(self.h, kt), "dyn_hpg")

    def zdf_mxl(self, kt):
        self._ck(lib().ora_zdf_mxl(self.h, kt), "zdf_mxl")

    def dyn_ldf_lap(self, kt, pub, pvb, pua, pva, kpass=1):
        self._ck(lib().ora_dyn_ldf_lap(self.h, kt, _p(pub), _p(pvb), _p(pua), _p(pva), kpass), "dyn_ldf_lap")

    def vor_ene(self, kt, kvor, pun, pvn, pua, pva):
        self._ck(lib().ora_vor_ene(self.h, kt, kvor, _p(pun), _p(pvn), _p(pua), _p(pva)), "vor_ene")

    def dyn_keg(self, kt, kscheme=0):
        self._ck(lib().ora_dyn_keg(self.h, kt, kscheme), "dyn_keg")

    def dyn_zad(self, kt):
        self._ck(lib().ora_dyn_zad(self.h, kt), "dyn_zad")

    def nlb10(self):
        return lib().ora_nlb10(self.h)

    def nksr(self):
        return lib().ora_nksr(self.h)

    def ldf_slp(self, kt, prd, pn2):
        self._ck(lib().ora_ldf_slp(self.h, kt, _p(prd), _p(pn2)), "ldf_slp")

    def ldf_slp_triad(self, kt, prab_b):
        self._ck(lib().ora_ldf_slp_triad(self.h, kt, _p(prab_b)), "ldf_slp_triad")

    def tra_ldf_triad(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, ptbb, pta, kjpt, kpass):
        self._ck(lib().ora_tra_ldf_triad(self.h, kt, kit000, cdtype.encode(), _p(pahu), _p(pahv), _p(pgu), _p(pgv),
                                         _p(pgui), _p(pgvi), _p(ptb), _p(ptbb), _p(pta), kjpt, kpass),
                 "tra_ldf_triad")

    def tra_ldf_blp(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, pta, kjpt, kldf):
        self._ck(lib().ora_tra_ldf_blp(self.h, kt, kit000, cdtype.encode(), _p(pahu), _p(pahv), _p(pgu), _p(pgv),
                                       _p(pgui), _p(pgvi), _p(ptb), _p(pta), kjpt, kldf), "tra_ldf_blp")

    def zps_hde(self, kt, kjpt, pta):
        gu = np.zeros((self.jpi, self.jpj, kjpt), order="F")
        gv = np.zeros((self.jpi, self.jpj, kjpt), order="F")
        self._ck(lib().ora_zps_hde(self.h, kt, kjpt, _p(pta), _p(gu), _p(gv)), "zps_hde")
        return gu, gv

    def zps_hde_rd(self, kt, pts, prd):
        """zps_hde's density part: (gru, grv) of the density of the interpolated T, S"""
        gu = np.zeros((self.jpi, self.jpj), order="F")
        gv = np.zeros((self.jpi, self.jpj), order="F")
        self._ck(lib().ora_zps_hde_rd(self.h, kt, _p(pts), _p(prd), _p(gu), _p(gv)), "zps_hde_rd")
        return gu, gv
