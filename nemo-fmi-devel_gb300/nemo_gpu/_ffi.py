"""ctypes binding of the C ABI declared in include/nemo_gpu.h.

The structures mirror ``nemo_dom_desc`` and ``nemo_namelist`` member for member;
the field ids are read from the header's ``enum nemo_field_id`` so the two cannot
drift apart.
"""
import ctypes as C
import os
import re

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                      "include", "nemo_gpu.h")

NEMO_OK, NEMO_ERR_ARG, NEMO_ERR_UNSUPPORTED, NEMO_ERR_UNBOUND = 0, 1, 2, 3
NEMO_ERR_CUDA, NEMO_ERR_TIMEOUT, NEMO_ERR_NOMEM, NEMO_ERR_STATE, NEMO_ERR_BLOWUP = 4, 5, 6, 7, 8
NEMO_CTL_N, NEMO_CTL_NLOC, NEMO_HSB_N = 6, 11, 16  # result sizes of stp_ctl and dia_hsb
PREC_FP64, PREC_MIXED = 0, 1
VOR = {"ENS": 0, "ENE": 1, "ENT": 2, "EET": 3, "EEN": 4, "MIX": 5}


def _enum(name, prefix):
    txt = open(HEADER).read()
    body = re.search(r"enum %s \{(.*?)\};" % name, txt, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = [n.split("=")[0].strip() for n in body.split(",")]
    names = [n for n in names if n]
    return {n[len(prefix):]: i for i, n in enumerate(names)}


F = _enum("nemo_field_id", "NEMO_F_")  # e.g. F["TSB"] == 0, F["COUNT"] == number of fields
K = _enum("nemo_kernel_id", "NEMO_K_")  # kernel ids of nemo_gpu_get_kernel_timing
FP64_FIELDS = {"SSHA", "UA_B", "VA_B", "UN_ADV", "VN_ADV", "UB2_B", "VB2_B", "UN_BF", "VN_BF"}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class DomDesc(C.Structure):
    _fields_ = [("jpi", C.c_int), ("jpj", C.c_int), ("jpk", C.c_int), ("jperio", C.c_int),
                ("e1t", _dp), ("e2t", _dp), ("e1u", _dp), ("e2u", _dp), ("e1v", _dp), ("e2v", _dp),
                ("e1f", _dp), ("e2f", _dp), ("ff_f", _dp), ("ff_t", _dp), ("k_top", _ip), ("k_bot", _ip),
                ("e3t_0", _dp), ("e3u_0", _dp), ("e3v_0", _dp), ("e3w_0", _dp), ("e3f_0", _dp)]


# members of nemo_spg_adj (the adjoint arrays of dyn_spg_ts), in order
SPG_ADJ = ("ua", "va", "un", "vn", "ssha", "ua_b", "va_b", "un_adv", "vn_adv", "ub2_b", "vb2_b", "un_bf", "vn_bf",
           "sshn", "un_b", "vn_b", "ub_b", "vb_b")


class SpgAdj(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in SPG_ADJ]


# members of nemo_nxt_adj (the adjoint arrays of dyn_nxt), in order
NXT_ADJ = ("ua", "va", "un", "vn", "ub", "vb", "un_b", "vn_b", "ub_b", "vb_b", "ua_b", "va_b")


class NxtAdj(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in NXT_ADJ]


class Namelist(C.Structure):
    _fields_ = [("rn_rdt", C.c_double), ("rn_atfp", C.c_double), ("nit000", C.c_int), ("neuler", C.c_int),
                ("ln_linssh", C.c_int), ("ln_zps", C.c_int), ("ln_isfcav", C.c_int),
                ("ln_traldf_lap", C.c_int), ("ln_traldf_blp", C.c_int), ("ln_traldf_iso", C.c_int),
                ("ln_traldf_msc", C.c_int), ("rn_aht_0", C.c_double), ("ln_zdfddm", C.c_int),
                ("ln_zad_Aimp", C.c_int), ("ln_bt_fw", C.c_int), ("ln_bt_av", C.c_int), ("nn_bt_flt", C.c_int),
                ("ln_bt_auto", C.c_int), ("nn_baro", C.c_int), ("rn_bt_cmax", C.c_double),
                ("rn_bt_alpha", C.c_double), ("nvor_scheme", C.c_int), ("nn_een_e3f", C.c_int),
                ("ln_dynadv_vec", C.c_int), ("ln_sco", C.c_int), ("ln_apr_dyn", C.c_int),
                ("rn_scal_load", C.c_double), ("grav", C.c_double), ("rau0", C.c_double),
                ("nn_fct_h", C.c_int), ("nn_fct_v", C.c_int), ("rn_slpmax", C.c_double),
                ("ln_traqsr", C.c_int), ("rn_abs", C.c_double), ("rn_si0", C.c_double), ("rn_si1", C.c_double),
                ("rcp", C.c_double), ("ln_seos", C.c_int), ("rn_a0", C.c_double), ("rn_b0", C.c_double),
                ("rn_lambda1", C.c_double), ("rn_lambda2", C.c_double), ("rn_mu1", C.c_double),
                ("rn_mu2", C.c_double), ("rn_nu", C.c_double), ("ln_eos80", C.c_int),
                ("ln_zdftke", C.c_int), ("ln_zdfevd", C.c_int), ("nn_evdm", C.c_int), ("rn_evd", C.c_double),
                ("rn_avm0", C.c_double), ("rn_avt0", C.c_double), ("rn_ediff", C.c_double),
                ("rn_ediss", C.c_double), ("rn_ebb", C.c_double), ("rn_emin", C.c_double),
                ("rn_emin0", C.c_double), ("rn_bshear", C.c_double), ("nn_pdl", C.c_int), ("nn_mxl", C.c_int),
                ("ln_mxl0", C.c_int), ("rn_mxl0", C.c_double), ("ln_lc", C.c_int), ("rn_lc", C.c_double),
                ("nn_etau", C.c_int), ("ln_drg_tke", C.c_int),
                ("ln_dynadv_OFF", C.c_int), ("nn_dynkeg", C.c_int), ("ln_usr", C.c_int),
                ("ln_traldf_triad", C.c_int), ("ln_triad_iso", C.c_int), ("ln_botmix_triad", C.c_int),
                ("rn_sw_triad", C.c_double)]


# members a namelist may leave out (&namtra_qsr of namelist_ref; rcp 0 selects 3991.86795711963)
NAMELIST_DEFAULTS = {"ln_traqsr": 0, "rn_abs": 0.58, "rn_si0": 0.35, "rn_si1": 23.0, "rcp": 0.0,
                     "ln_seos": 0, "rn_a0": 1.6550e-1, "rn_b0": 7.6554e-1, "rn_lambda1": 5.9520e-2,
                     "rn_lambda2": 7.4914e-4, "rn_mu1": 1.4970e-4, "rn_mu2": 1.1090e-5, "rn_nu": 2.4341e-3,
                     "ln_eos80": 0,
                     # &namzdf and &namzdf_tke of namelist_ref, with GYRE's namelist_cfg
                     # (TKE, EVD on tracers and momentum, rn_evd = 100, nn_etau = 0)
                     "ln_zdftke": 0, "ln_zdfevd": 0, "nn_evdm": 1, "rn_evd": 100.0, "rn_avm0": 1.2e-4,
                     "rn_avt0": 1.2e-5, "rn_ediff": 0.1, "rn_ediss": 0.7, "rn_ebb": 67.83, "rn_emin": 1.e-6,
                     "rn_emin0": 1.e-4, "rn_bshear": 1.e-20, "nn_pdl": 1, "nn_mxl": 2, "ln_mxl0": 1,
                     "rn_mxl0": 0.04, "ln_lc": 1, "rn_lc": 0.15, "nn_etau": 0, "ln_drg_tke": 0,
                     "ln_dynadv_OFF": 0, "nn_dynkeg": 0, "ln_usr": 0,
                     "ln_traldf_triad": 0, "ln_triad_iso": 0, "ln_botmix_triad": 0, "rn_sw_triad": 1.0}


def make_desc(dom):
    """DomDesc for a domain dict of Fortran-ordered float64/int32 numpy arrays.

    The numpy arrays must stay alive while the descriptor is used (creation only)."""
    import numpy as np
    d = DomDesc()
    d.jpi, d.jpj, d.jpk, d.jperio = dom["jpi"], dom["jpj"], dom["jpk"], dom.get("jperio", 0)
    keep = []
    for name in ("e1t", "e2t", "e1u", "e2u", "e1v", "e2v", "e1f", "e2f", "ff_f", "ff_t",
                 "e3t_0", "e3u_0", "e3v_0", "e3w_0", "e3f_0"):
        a = np.asfortranarray(dom[name], dtype=np.float64)
        keep.append(a)
        setattr(d, name, a.ctypes.data_as(_dp))
    for name in ("k_top", "k_bot"):
        a = np.asfortranarray(dom[name], dtype=np.int32)
        keep.append(a)
        setattr(d, name, a.ctypes.data_as(_ip))
    d._keep = keep
    return d


def make_namelist(nam):
    n = Namelist()
    for k, _ in Namelist._fields_:
        setattr(n, k, nam[k] if k in nam else NAMELIST_DEFAULTS[k])
    return n


def _proto(lib, name, restype, argtypes):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = argtypes
    return f


def load(path):
    """Load the CUDA library and declare the prototypes of every C ABI symbol."""
    lib = C.CDLL(path)
    vp, i, d, cp = C.c_void_p, C.c_int, C.c_double, C.c_char_p
    _proto(lib, "nemo_gpu_create", i, [C.POINTER(DomDesc), C.POINTER(Namelist), i, i, vp, C.POINTER(vp)])
    _proto(lib, "nemo_gpu_destroy", i, [vp])
    _proto(lib, "nemo_gpu_last_error", cp, [vp])
    _proto(lib, "nemo_gpu_synchronize", i, [vp])
    _proto(lib, "nemo_gpu_bind", i, [vp, i, vp])
    _proto(lib, "nemo_gpu_field_numel", C.c_size_t, [vp, i])
    _proto(lib, "nemo_gpu_field_is_fp64", i, [vp, i])
    _proto(lib, "nemo_gpu_spg_info", i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(d)])
    _proto(lib, "nemo_gpu_field_upload", i, [vp, i, vp])
    _proto(lib, "nemo_gpu_field_download", i, [vp, i, vp])
    _proto(lib, "nemo_gpu_tra_adv_trp", i, [vp, vp, vp, vp, vp, vp, vp])
    _proto(lib, "nemo_gpu_tra_adv_fct", i, [vp, i, i, cp, d, vp, vp, vp, vp, vp, vp, i, i, i])
    _proto(lib, "nemo_gpu_tra_ldf_lap", i, [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
    _proto(lib, "nemo_gpu_tra_ldf_iso", i, [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
    _proto(lib, "nemo_gpu_tra_zdf_imp", i, [vp, i, i, cp, d, vp, vp, i])
    _proto(lib, "nemo_gpu_tra_nxt", i, [vp, i])
    _proto(lib, "nemo_gpu_autotune", i, [vp, i, i])
    _proto(lib, "nemo_gpu_ldf_slp", i, [vp, i, vp, vp])
    _proto(lib, "nemo_gpu_ldf_slp_triad", i, [vp, i, vp])
    _proto(lib, "nemo_gpu_tra_ldf_triad", i, [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
    _proto(lib, "nemo_gpu_tra_ldf_blp", i, [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
    _proto(lib, "nemo_gpu_zps_hde", i, [vp, i, i, vp, vp, vp])
    _proto(lib, "nemo_gpu_get_launch_shape", i, [vp, _ip, i])
    _proto(lib, "nemo_gpu_set_launch_shape", i, [vp, _ip, i])
    _proto(lib, "nemo_gpu_eos_insitu", i, [vp, vp, vp, vp])
    _proto(lib, "nemo_gpu_eos_insitu_pot", i, [vp, vp, vp, vp, vp])
    _proto(lib, "nemo_gpu_rab_3d", i, [vp, vp, vp])
    _proto(lib, "nemo_gpu_bn2", i, [vp, vp, vp, vp])
    _proto(lib, "nemo_gpu_zps_hde_rd", i, [vp, i, vp, vp, vp, vp])
    _proto(lib, "nemo_gpu_dyn_ldf_lap", i, [vp, i, vp, vp, vp, vp, i])
    _proto(lib, "nemo_gpu_vor_ene", i, [vp, i, i, vp, vp, vp, vp])
    _proto(lib, "nemo_gpu_dyn_keg", i, [vp, i, i])
    _proto(lib, "nemo_gpu_dyn_zad", i, [vp, i])
    for name in ("nemo_gpu_tra_sbc", "nemo_gpu_tra_qsr", "nemo_gpu_dyn_hpg", "nemo_gpu_zdf_mxl",
                 "nemo_gpu_wzv", "nemo_gpu_dyn_zdf_step", "nemo_gpu_dyn_nxt", "nemo_gpu_ssh_swp",
                 "nemo_gpu_dom_vvl_sf_nxt", "nemo_gpu_dom_vvl_sf_swp",
                 "nemo_gpu_stp_model", "nemo_gpu_zdf_phy", "nemo_gpu_usrdef_sbc"):
        _proto(lib, name, i, [vp, i])
    _proto(lib, "nemo_gpu_tra_adv_fct_adj", i, [vp, i, i, cp, d, vp, vp, vp, vp, vp, vp, i, i, i])
    _proto(lib, "nemo_gpu_dyn_spg_ts_adj", i, [vp, i, C.POINTER(SpgAdj)])
    _proto(lib, "nemo_gpu_dyn_nxt_adj", i, [vp, i, C.POINTER(NxtAdj)])
    _proto(lib, "nemo_gpu_wzv_adj", i, [vp, i, vp, vp, vp])
    _proto(lib, "nemo_gpu_ssh_swp_adj", i, [vp, i, vp, vp, vp])
    _proto(lib, "nemo_gpu_tra_ldf_lap_adj", i, [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
    _proto(lib, "nemo_gpu_tra_ldf_iso_adj", i, [vp, i, i, cp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i])
    _proto(lib, "nemo_gpu_tra_zdf_imp_adj", i, [vp, i, i, cp, d, vp, vp, i])
    _proto(lib, "nemo_gpu_tra_nxt_adj", i, [vp, i, vp, vp, vp])
    _proto(lib, "nemo_gpu_tra_zdf", i, [vp, i])
    _proto(lib, "nemo_gpu_dyn_spg_ts", i, [vp, i])
    _proto(lib, "nemo_gpu_lbc_lnk", i, [vp, cp, vp, i, i, cp, d, d, i])
    _proto(lib, "nemo_gpu_lbc_lnk_multi", i, [vp, cp, i, C.POINTER(vp), C.POINTER(i), cp, C.POINTER(d), d, i])
    _proto(lib, "nemo_gpu_glob_sum", i, [vp, cp, vp, i, i, C.POINTER(d)])
    _proto(lib, "nemo_gpu_glob_sum_noalloc", i, [vp, vp, i, i, i, i, i, vp, vp])
    _proto(lib, "nemo_gpu_stp_hotpath", i, [vp, i])
    _proto(lib, "nemo_gpu_set_barrier_limit", i, [vp, C.c_longlong, i])
    _proto(lib, "nemo_gpu_set_timing", i, [vp, i])
    _proto(lib, "nemo_gpu_set_fusion", i, [vp, i])
    _proto(lib, "nemo_gpu_set_tma", i, [vp, i])
    _proto(lib, "nemo_gpu_set_tma_poll_limit", i, [vp, i])
    _proto(lib, "nemo_gpu_stp_ctl", i, [vp, i])
    _proto(lib, "nemo_gpu_stp_ctl_result", i, [vp, vp, vp, vp])
    _proto(lib, "nemo_gpu_dia_hsb_init", i, [vp])
    _proto(lib, "nemo_gpu_dia_hsb", i, [vp, i])
    _proto(lib, "nemo_gpu_dia_hsb_result", i, [vp, vp])
    _proto(lib, "nemo_gpu_set_spg_specialised", i, [vp, i])
    _proto(lib, "nemo_gpu_set_fct_fused", i, [vp, i])
    _proto(lib, "nemo_gpu_get_timing", i, [vp, C.POINTER(d), C.POINTER(i)])
    _proto(lib, "nemo_gpu_get_kernel_timing", i, [vp, C.POINTER(d), C.POINTER(i), i])
    return lib


def header_symbols():
    """Names of every function the header declares."""
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(nemo_gpu_\w+)\s*\(", txt)))
