"""Host mirror of the reference's Fortran interfaces over the CUDA library.

Every method forwards to the C ABI (include/nemo_gpu.h) with device pointers; the
argument lists are the Fortran ones (traadv_fct.F90:54-80, traldf_lap_blp.F90:47-76,
traldf_iso.F90:50-103, trazdf.F90:109-135, dynspg_ts.F90:121, lbclnk.F90:81-102,
lib_fortran_generic.h90:32). Errors raise ``NemoError`` with the library's message,
as the reference's ctl_stop would stop the model. There is no CPU path: without the
compiled library or a GPU the constructor fails.

Tensors are torch tensors on the CUDA device whose memory is the Fortran array:
a (jpi,jpj,jpk[,kjpt]) field of m members is a C-contiguous tensor of shape
(m, [kjpt,] jpk, jpj, jpi) (or any contiguous tensor with that many elements).
"""
import ctypes as C

import numpy as np

from . import _ffi
from . import build as _build


class NemoError(RuntimeError):
    pass


_LIB = None


def library():
    """The loaded CUDA library (built in-tree on first use)."""
    global _LIB
    if _LIB is None:
        _LIB = _ffi.load(_build.build())
    return _LIB


def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise NemoError("fields must be contiguous CUDA tensors")
    return t.data_ptr()


class Context:
    """A nemo_gpu context: one domain, one namelist, nmembers ensemble members."""

    def __init__(self, dom, nam, nmembers=1, prec="fp64", stream=None):
        import torch
        if not torch.cuda.is_available():
            raise NemoError("a CUDA device is required (the library has no CPU path)")
        self.torch = torch
        self.lib = library()
        self.dom, self.nam = dom, dict(nam)
        self.nmem = nmembers
        self.prec = _ffi.PREC_FP64 if prec == "fp64" else _ffi.PREC_MIXED
        self.dtype = torch.float64 if self.prec == _ffi.PREC_FP64 else torch.float32
        self.jpi, self.jpj, self.jpk = dom["jpi"], dom["jpj"], dom["jpk"]
        desc = _ffi.make_desc(dom)
        nl = _ffi.make_namelist(self.nam)
        h = C.c_void_p()
        s = stream.cuda_stream if stream is not None else None
        st = self.lib.nemo_gpu_create(C.byref(desc), C.byref(nl), nmembers, self.prec, s, C.byref(h))
        if st != 0:
            raise NemoError(f"nemo_gpu_create failed with status {st}")
        self.h = h
        self.stream = stream
        self.bound = {}

    # ------------------------------------------------------------------ life cycle
    def close(self):
        if getattr(self, "h", None):
            self.lib.nemo_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st, what):
        if st != 0:
            msg = self.lib.nemo_gpu_last_error(self.h).decode()
            raise NemoError(f"{what}: status {st}: {msg}")

    def synchronize(self):
        self._ck(self.lib.nemo_gpu_synchronize(self.h), "synchronize")

    # ------------------------------------------------------------------ fields
    def field_dtype(self, name):
        if name == "NMLN":  # the mixed-layer level is an integer field
            return self.torch.int32
        return self.torch.float64 if self.lib.nemo_gpu_field_is_fp64(self.h, _ffi.F[name]) else self.torch.float32

    def field_numel(self, name):
        return int(self.lib.nemo_gpu_field_numel(self.h, _ffi.F[name]))

    def to_device(self, arr, dtype=None):
        """Device tensor holding a Fortran-order numpy array (or a list of members)."""
        torch = self.torch
        arrs = arr if isinstance(arr, (list, tuple)) else [arr]
        flat = np.concatenate([np.asarray(a).ravel(order="F") for a in arrs])
        return torch.from_numpy(flat).to(device="cuda", dtype=dtype or self.dtype).contiguous()

    def to_host(self, t, shape):
        """Fortran-order numpy array(s) (one per member) from a device tensor, after
        the device's work (the context's stream does not order with torch's)."""
        self.torch.cuda.synchronize()
        a = t.detach().to("cpu", self.torch.float64).numpy()
        n = int(np.prod(shape))
        if a.size == n:
            return a.reshape(shape, order="F")
        return [a[m * n:(m + 1) * n].reshape(shape, order="F") for m in range(a.size // n)]

    def bind(self, name, tensor):
        self.bound[name] = tensor
        self._ck(self.lib.nemo_gpu_bind(self.h, _ffi.F[name], _ptr(tensor)), f"bind {name}")

    def spg_info(self):
        ic, nb, dt = C.c_int(), C.c_int(), C.c_double()
        self._ck(self.lib.nemo_gpu_spg_info(self.h, C.byref(ic), C.byref(nb), C.byref(dt)), "spg_info")
        return ic.value, nb.value, dt.value

    def set_barrier_limit(self, max_spins, extra_arrivals=0):
        self._ck(self.lib.nemo_gpu_set_barrier_limit(self.h, max_spins, extra_arrivals), "set_barrier_limit")

    def set_fusion(self, on):
        self._ck(self.lib.nemo_gpu_set_fusion(self.h, int(on)), "set_fusion")

    def set_tma(self, on):
        self._ck(self.lib.nemo_gpu_set_tma(self.h, int(on)), "set_tma")

    # ---------------------------------------------------------------- stp_ctl, dia_hsb
    def stp_ctl(self, kt):
        self._ck(self.lib.nemo_gpu_stp_ctl(self.h, kt), "stp_ctl")

    def stp_ctl_result(self):
        """(zmax[nmem, 6], loc[nmem, 11], kindic[nmem]) of the last stp_ctl"""
        import numpy as np
        z = np.zeros((self.nmem, _ffi.NEMO_CTL_N))
        loc = np.zeros((self.nmem, _ffi.NEMO_CTL_NLOC), dtype=np.int32)
        k = np.zeros(self.nmem, dtype=np.int32)
        self._ck(self.lib.nemo_gpu_stp_ctl_result(self.h, z.ctypes.data, loc.ctypes.data, k.ctypes.data),
                 "stp_ctl_result")
        return z, loc, k

    def dia_hsb_init(self):
        self._ck(self.lib.nemo_gpu_dia_hsb_init(self.h), "dia_hsb_init")

    def dia_hsb(self, kt):
        self._ck(self.lib.nemo_gpu_dia_hsb(self.h, kt), "dia_hsb")

    def dia_hsb_result(self):
        """the terms of the last dia_hsb, [nmem, NEMO_HSB_N]"""
        import numpy as np
        out = np.zeros((self.nmem, _ffi.NEMO_HSB_N))
        self._ck(self.lib.nemo_gpu_dia_hsb_result(self.h, out.ctypes.data), "dia_hsb_result")
        return out

    def set_spg_specialised(self, on):
        self._ck(self.lib.nemo_gpu_set_spg_specialised(self.h, int(on)), "set_spg_specialised")

    def set_tma_poll_limit(self, max_polls):
        self._ck(self.lib.nemo_gpu_set_tma_poll_limit(self.h, int(max_polls)), "set_tma_poll_limit")

    def set_fct_fused(self, on):
        self._ck(self.lib.nemo_gpu_set_fct_fused(self.h, int(on)), "set_fct_fused")

    def autotune(self, kt, nrep=3):
        """Choose the block height of each tunable hot-path kernel by timing nrep steps
        per candidate at step kt; the bound state is left as it was."""
        self._ck(self.lib.nemo_gpu_autotune(self.h, kt, nrep), "autotune")

    def launch_shape(self):
        """{kernel name: block height} of the 32-wide hot-path launches."""
        nk = _ffi.K["COUNT"]
        ty = (C.c_int * nk)()
        self._ck(self.lib.nemo_gpu_get_launch_shape(self.h, ty, nk), "get_launch_shape")
        names = {v: k.lower() for k, v in _ffi.K.items() if k != "COUNT"}
        return {names[i]: ty[i] for i in range(nk)}

    def set_launch_shape(self, shape):
        """{kernel name: block height (4, 2 or 1)}; kernels not named keep 32 x 4."""
        nk = _ffi.K["COUNT"]
        ty = (C.c_int * nk)()
        for name, h in shape.items():
            ty[_ffi.K[name.upper()]] = int(h)
        self._ck(self.lib.nemo_gpu_set_launch_shape(self.h, ty, nk), "set_launch_shape")

    def set_timing(self, on):
        self._ck(self.lib.nemo_gpu_set_timing(self.h, int(on)), "set_timing")

    def get_timing(self):
        ms = (C.c_double * 4)()
        n = C.c_int()
        self._ck(self.lib.nemo_gpu_get_timing(self.h, ms, C.byref(n)), "get_timing")
        return dict(zip(("dyn_spg_ts", "tra_adv", "tra_ldf", "tra_zdf"), list(ms))), n.value

    def get_kernel_timing(self):
        """{kernel name: (cumulative ms, launches)} of the kernels timed since set_timing(True)."""
        nk = _ffi.K["COUNT"]
        ms = (C.c_double * nk)()
        cnt = (C.c_int * nk)()
        self._ck(self.lib.nemo_gpu_get_kernel_timing(self.h, ms, cnt, nk), "get_kernel_timing")
        names = {v: k.lower() for k, v in _ffi.K.items() if k != "COUNT"}
        return {names[i]: (ms[i], cnt[i]) for i in range(nk) if cnt[i] > 0}

    def upload(self, name, host):
        """nemo_gpu_field_upload from a (pinned) host torch tensor."""
        self._ck(self.lib.nemo_gpu_field_upload(self.h, _ffi.F[name], host.data_ptr()), f"upload {name}")

    def download(self, name, host):
        self._ck(self.lib.nemo_gpu_field_download(self.h, _ffi.F[name], host.data_ptr()), f"download {name}")

    # ------------------------------------------------------------------ routines
    def tra_adv_trp(self, un, vn, wn, zun, zvn, zwn):
        self._ck(self.lib.nemo_gpu_tra_adv_trp(self.h, *map(_ptr, (un, vn, wn, zun, zvn, zwn))), "tra_adv_trp")

    def tra_adv_fct(self, kt, kit000, cdtype, p2dt, pun, pvn, pwn, ptb, ptn, pta, kjpt, kn_fct_h, kn_fct_v):
        self._ck(self.lib.nemo_gpu_tra_adv_fct(self.h, kt, kit000, cdtype.encode(), p2dt, _ptr(pun), _ptr(pvn),
                                               _ptr(pwn), _ptr(ptb), _ptr(ptn), _ptr(pta), kjpt, kn_fct_h, kn_fct_v),
                 "tra_adv_fct")

    def tra_ldf_lap(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, pta, kjpt, kpass):
        self._ck(self.lib.nemo_gpu_tra_ldf_lap(self.h, kt, kit000, cdtype.encode(), *map(_ptr, (
            pahu, pahv, pgu, pgv, pgui, pgvi, ptb, pta)), kjpt, kpass), "tra_ldf_lap")

    def tra_ldf_iso(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, ptbb, pta, kjpt, kpass):
        self._ck(self.lib.nemo_gpu_tra_ldf_iso(self.h, kt, kit000, cdtype.encode(), *map(_ptr, (
            pahu, pahv, pgu, pgv, pgui, pgvi, ptb, ptbb, pta)), kjpt, kpass), "tra_ldf_iso")

    def tra_ldf_triad(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, ptbb, pta, kjpt, kpass):
        self._ck(self.lib.nemo_gpu_tra_ldf_triad(self.h, kt, kit000, cdtype.encode(), *map(_ptr, (
            pahu, pahv, pgu, pgv, pgui, pgvi, ptb, ptbb, pta)), kjpt, kpass), "tra_ldf_triad")

    def ldf_slp_triad(self, kt, prab_b):
        self._ck(self.lib.nemo_gpu_ldf_slp_triad(self.h, kt, _ptr(prab_b)), "ldf_slp_triad")

    def tra_ldf_blp(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, pta, kjpt, kldf):
        self._ck(self.lib.nemo_gpu_tra_ldf_blp(self.h, kt, kit000, cdtype.encode(), *map(_ptr, (
            pahu, pahv, pgu, pgv, pgui, pgvi, ptb, pta)), kjpt, kldf), "tra_ldf_blp")

    def zps_hde(self, kt, kjpt, pta, pgtu, pgtv):
        self._ck(self.lib.nemo_gpu_zps_hde(self.h, kt, kjpt, _ptr(pta), _ptr(pgtu), _ptr(pgtv)), "zps_hde")

    def zps_hde_rd(self, kt, pts, prd, pgru, pgrv):
        """zps_hde's density part: the bottom density gradients pgru, pgrv"""
        self._ck(self.lib.nemo_gpu_zps_hde_rd(self.h, kt, _ptr(pts), _ptr(prd), _ptr(pgru), _ptr(pgrv)),
                 "zps_hde_rd")

    def tra_zdf_imp(self, kt, kit000, cdtype, p2dt, ptb, pta, kjpt):
        self._ck(self.lib.nemo_gpu_tra_zdf_imp(self.h, kt, kit000, cdtype.encode(), p2dt, _ptr(ptb), _ptr(pta), kjpt),
                 "tra_zdf_imp")

    def tra_zdf(self, kt):
        self._ck(self.lib.nemo_gpu_tra_zdf(self.h, kt), "tra_zdf")

    def tra_nxt(self, kt):
        self._ck(self.lib.nemo_gpu_tra_nxt(self.h, kt), "tra_nxt")

    def ldf_slp(self, kt, prd, pn2):
        """ldf_slp (ldfslp.F90): the bound slope fields from the density anomaly and
        N^2 (device tensors) and the bound depths and mixed layer."""
        self._ck(self.lib.nemo_gpu_ldf_slp(self.h, kt, _ptr(prd), _ptr(pn2)), "ldf_slp")

    def wzv(self, kt):
        self._ck(self.lib.nemo_gpu_wzv(self.h, kt), "wzv")

    def dyn_zdf_step(self, kt):
        self._ck(self.lib.nemo_gpu_dyn_zdf_step(self.h, kt), "dyn_zdf_step")

    def dyn_nxt(self, kt):
        self._ck(self.lib.nemo_gpu_dyn_nxt(self.h, kt), "dyn_nxt")

    def ssh_swp(self, kt):
        self._ck(self.lib.nemo_gpu_ssh_swp(self.h, kt), "ssh_swp")

    def dom_vvl_sf_nxt(self, kt):
        self._ck(self.lib.nemo_gpu_dom_vvl_sf_nxt(self.h, kt), "dom_vvl_sf_nxt")

    def dom_vvl_sf_swp(self, kt):
        self._ck(self.lib.nemo_gpu_dom_vvl_sf_swp(self.h, kt), "dom_vvl_sf_swp")

    def tra_sbc(self, kt):
        self._ck(self.lib.nemo_gpu_tra_sbc(self.h, kt), "tra_sbc")

    def tra_qsr(self, kt):
        self._ck(self.lib.nemo_gpu_tra_qsr(self.h, kt), "tra_qsr")

    def eos_insitu(self, pts, prd, pdep):
        self._ck(self.lib.nemo_gpu_eos_insitu(self.h, _ptr(pts), _ptr(prd), _ptr(pdep)), "eos_insitu")

    def eos_insitu_pot(self, pts, prd, prhop, pdep):
        self._ck(self.lib.nemo_gpu_eos_insitu_pot(self.h, _ptr(pts), _ptr(prd), _ptr(prhop), _ptr(pdep)),
                 "eos_insitu_pot")

    def rab_3d(self, pts, pab):
        self._ck(self.lib.nemo_gpu_rab_3d(self.h, _ptr(pts), _ptr(pab)), "rab_3d")

    def bn2(self, pts, pab, pn2):
        self._ck(self.lib.nemo_gpu_bn2(self.h, _ptr(pts), _ptr(pab), _ptr(pn2)), "bn2")

    def dyn_ldf_lap(self, kt, pub, pvb, pua, pva, kpass=1):
        self._ck(self.lib.nemo_gpu_dyn_ldf_lap(self.h, kt, _ptr(pub), _ptr(pvb), _ptr(pua), _ptr(pva), kpass),
                 "dyn_ldf_lap")

    def vor_ene(self, kt, kvor, pun, pvn, pua, pva):
        self._ck(self.lib.nemo_gpu_vor_ene(self.h, kt, kvor, _ptr(pun), _ptr(pvn), _ptr(pua), _ptr(pva)), "vor_ene")

    def dyn_keg(self, kt, kscheme=0):
        self._ck(self.lib.nemo_gpu_dyn_keg(self.h, kt, kscheme), "dyn_keg")

    def dyn_zad(self, kt):
        self._ck(self.lib.nemo_gpu_dyn_zad(self.h, kt), "dyn_zad")

    def zdf_mxl(self, kt):
        self._ck(self.lib.nemo_gpu_zdf_mxl(self.h, kt), "zdf_mxl")

    def usrdef_sbc(self, kt):
        """GYRE's analytic surface forcing of step kt on the bound fields (usrdef_sbc.F90)"""
        self._ck(self.lib.nemo_gpu_usrdef_sbc(self.h, kt), "usrdef_sbc")

    def zdf_phy(self, kt):
        """zdf_sh2, the TKE closure and zdf_evd on the bound fields (zdfphy.F90:243-316)"""
        self._ck(self.lib.nemo_gpu_zdf_phy(self.h, kt), "zdf_phy")

    def dyn_hpg(self, kt):
        self._ck(self.lib.nemo_gpu_dyn_hpg(self.h, kt), "dyn_hpg")

    def stp_model(self, kt):
        """One model step: the hot path closed by wzv, the dyn_zdf time step, tra_nxt,
        dyn_nxt and ssh_swp (see nemo_gpu.h)."""
        self._ck(self.lib.nemo_gpu_stp_model(self.h, kt), "stp_model")

    # ------------------------------------------------------------------ adjoints
    # The adjoint twins of the tracer routines (FP64 contexts): the tracer arrays of
    # the forward's argument list are replaced by their adjoints; see nemo_gpu.h.
    def tra_adv_fct_adj(self, kt, kit000, cdtype, p2dt, pun, pvn, pwn, ptb_ad, ptn_ad, pta_ad, kjpt, kn_fct_h,
                        kn_fct_v):
        self._ck(self.lib.nemo_gpu_tra_adv_fct_adj(self.h, kt, kit000, cdtype.encode(), p2dt, _ptr(pun), _ptr(pvn),
                                                   _ptr(pwn), _ptr(ptb_ad), _ptr(ptn_ad), _ptr(pta_ad), kjpt,
                                                   kn_fct_h, kn_fct_v), "tra_adv_fct_adj")

    def tra_ldf_lap_adj(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb_ad, pta_ad, kjpt, kpass):
        self._ck(self.lib.nemo_gpu_tra_ldf_lap_adj(self.h, kt, kit000, cdtype.encode(), *map(_ptr, (
            pahu, pahv, pgu, pgv, pgui, pgvi, ptb_ad, pta_ad)), kjpt, kpass), "tra_ldf_lap_adj")

    def tra_ldf_iso_adj(self, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb_ad, ptbb_ad, pta_ad, kjpt,
                        kpass):
        self._ck(self.lib.nemo_gpu_tra_ldf_iso_adj(self.h, kt, kit000, cdtype.encode(), *map(_ptr, (
            pahu, pahv, pgu, pgv, pgui, pgvi, ptb_ad, ptbb_ad, pta_ad)), kjpt, kpass), "tra_ldf_iso_adj")

    def tra_zdf_imp_adj(self, kt, kit000, cdtype, p2dt, ptb_ad, pta_ad, kjpt):
        self._ck(self.lib.nemo_gpu_tra_zdf_imp_adj(self.h, kt, kit000, cdtype.encode(), p2dt, _ptr(ptb_ad),
                                                   _ptr(pta_ad), kjpt), "tra_zdf_imp_adj")

    def tra_nxt_adj(self, kt, tsb_ad, tsn_ad, tsa_ad):
        self._ck(self.lib.nemo_gpu_tra_nxt_adj(self.h, kt, _ptr(tsb_ad), _ptr(tsn_ad), _ptr(tsa_ad)), "tra_nxt_adj")

    def wzv_adj(self, kt, un_ad, vn_ad, wn_ad):
        self._ck(self.lib.nemo_gpu_wzv_adj(self.h, kt, _ptr(un_ad), _ptr(vn_ad), _ptr(wn_ad)), "wzv_adj")

    def dyn_nxt_adj(self, kt, adj):
        """adj: dict of device FP64 tensors keyed by the members of nemo_nxt_adj."""
        s = _ffi.NxtAdj(*[_ptr(adj[n]) for n in _ffi.NXT_ADJ])
        self._ck(self.lib.nemo_gpu_dyn_nxt_adj(self.h, kt, C.byref(s)), "dyn_nxt_adj")

    def ssh_swp_adj(self, kt, sshb_ad, sshn_ad, ssha_ad):
        self._ck(self.lib.nemo_gpu_ssh_swp_adj(self.h, kt, _ptr(sshb_ad), _ptr(sshn_ad), _ptr(ssha_ad)),
                 "ssh_swp_adj")

    def dyn_spg_ts_adj(self, kt, adj):
        """adj: dict of device FP64 tensors keyed by the members of nemo_spg_adj."""
        s = _ffi.SpgAdj(*[_ptr(adj[n]) for n in _ffi.SPG_ADJ])
        self._ck(self.lib.nemo_gpu_dyn_spg_ts_adj(self.h, kt, C.byref(s)), "dyn_spg_ts_adj")

    def dyn_spg_ts(self, kt):
        self._ck(self.lib.nemo_gpu_dyn_spg_ts(self.h, kt), "dyn_spg_ts")

    def lbc_lnk(self, t, nk, cd_nat, psgn=1.0, pval=0.0, nl=1):
        is64 = int(t.dtype == self.torch.float64)
        self._ck(self.lib.nemo_gpu_lbc_lnk(self.h, b"lbc", _ptr(t), nk, nl, cd_nat.encode(), psgn, pval, is64),
                 "lbc_lnk")

    def glob_sum(self, t, nk):
        out = (C.c_double * self.nmem)()
        is64 = int(t.dtype == self.torch.float64)
        self._ck(self.lib.nemo_gpu_glob_sum(self.h, b"glob_sum", _ptr(t), nk, is64, out), "glob_sum")
        return list(out)

    def stp_hotpath(self, kt):
        self._ck(self.lib.nemo_gpu_stp_hotpath(self.h, kt), "stp_hotpath")
