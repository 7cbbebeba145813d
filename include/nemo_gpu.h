/*
 * nemo_gpu.h -- C ABI of the GB300 (sm_103a) implementation of NEMO's per-timestep
 * ocean stencil path: FCT tracer advection, laplacian / rotated-isopycnal lateral
 * diffusion, implicit vertical diffusion, the split-explicit barotropic sub-stepping
 * and the lbc_lnk halo fill, plus the compensated global sum.
 *
 * Conventions (identical to the Fortran arrays the entry points replace):
 *  - every field is a Fortran column-major array (jpi,jpj[,jpk][,kjpt]): i is the
 *    contiguous index, then j, then k, then the tracer index;
 *  - with an ensemble context (nmembers > 1) every field pointer addresses nmembers
 *    such arrays stored one after the other (member index outermost);
 *  - array arguments are DEVICE pointers (fields are resident on the GPU across
 *    timesteps); they are double* for a NEMO_PREC_FP64 context and float* for a
 *    NEMO_PREC_MIXED context, except the fields nemo_gpu_field_is_fp64() reports as
 *    FP64 (barotropic time-filter accumulators), which stay double* in both modes;
 *  - scalars (time steps, signs, land values) are always double;
 *  - every entry point returns a status (NEMO_OK = 0); it never aborts, traps or
 *    exits. The text of the last error is returned by nemo_gpu_last_error(). Errors
 *    of asynchronous kernels surface at the next nemo_gpu_synchronize().
 *  - one context = one CUDA stream; a context is not re-entrant.
 *
 * Each entry point cites the reference routine (file:line within NEMO 4.0 src/OCE)
 * whose body it replaces; the Fortran caller keeps the reference's argument list.
 */
#ifndef NEMO_GPU_H
#define NEMO_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
enum nemo_status {
  NEMO_OK = 0,
  NEMO_ERR_ARG = 1,          /* null pointer, bad size, unknown option value          */
  NEMO_ERR_UNSUPPORTED = 2,  /* reference option this path does not implement         */
  NEMO_ERR_UNBOUND = 3,      /* a module-global field the call reads is not bound     */
  NEMO_ERR_CUDA = 4,         /* CUDA runtime error                                    */
  NEMO_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up (barrier)          */
  NEMO_ERR_NOMEM = 6,        /* device allocation failed at context creation          */
  NEMO_ERR_STATE = 7,        /* call order violated (e.g. iso before its first pass)  */
  NEMO_ERR_BLOWUP = 8        /* stp_ctl: |ssh| > 20 m, |U| > 10 m/s, S <= 0, S >= 100
                                or NaN (stpctl.F90:149-157); reported by the next
                                nemo_gpu_synchronize after the check ran             */
};

/* ------------------------------------------------------------ precision modes */
enum nemo_prec {
  NEMO_PREC_FP64 = 0,   /* plain form: every field and every operation in FP64       */
  NEMO_PREC_MIXED = 1   /* FP32 bulk; FP64 barotropic accumulators and global sums    */
};

/* --------------------------------------------------------- vorticity schemes
 * Same integer values as dynvor.F90:65-70 (np_ENS ... np_MIX). */
enum nemo_vor { NEMO_VOR_ENS = 0, NEMO_VOR_ENE = 1, NEMO_VOR_ENT = 2,
                NEMO_VOR_EET = 3, NEMO_VOR_EEN = 4, NEMO_VOR_MIX = 5 };

/* --------------------------------------------------------- domain description
 * Host pointers, read once by nemo_gpu_create. The masks (tmask, umask, vmask,
 * wmask, ssmask, ssumask, ssvmask, tmask_i) and level indices (mikt, mbkt, mbku,
 * mbkv) are derived from k_top/k_bot exactly as dommsk.F90:133-238 and
 * domzgr.F90:292-314 derive them; the inverse/product metrics (e1e2t, r1_e1e2t,
 * e2_e1u, ...) as domhgr.F90:133-151; ht_0/hu_0/hv_0 and r1_hu_0/r1_hv_0 as
 * domain.F90:149-183. */
typedef struct nemo_dom_desc {
  int jpi, jpj, jpk;               /* par_oce.F90 domain sizes                           */
  int jperio;                      /* lateral b.c. (0 = closed basin; only 0 supported)  */
  const double *e1t, *e2t;         /* (jpi,jpj) horizontal scale factors [m]             */
  const double *e1u, *e2u;
  const double *e1v, *e2v;
  const double *e1f, *e2f;
  const double *ff_f, *ff_t;       /* (jpi,jpj) Coriolis parameter at f-/t-points [1/s]   */
  const int *k_top, *k_bot;        /* (jpi,jpj) first / last wet T-level, 0 over land    */
  const double *e3t_0, *e3u_0;     /* (jpi,jpj,jpk) rest-state vertical scale factors [m] */
  const double *e3v_0, *e3w_0;
  const double *e3f_0;
} nemo_dom_desc;

/* ------------------------------------------------------------ namelist subset
 * The members of the reference namelists (cfgs/SHARED/namelist_ref) read by the
 * routines on this path. Unsupported switches must be 0 (checked at creation). */
typedef struct nemo_namelist {
  double rn_rdt;          /* &namdom: baroclinic time step [s]                        */
  double rn_atfp;         /* &namdom: Asselin filter parameter                        */
  int nit000;             /* &namrun nn_it000: first time step                        */
  int neuler;             /* 0: Euler first step (no restart), 1: leapfrog restart   */
  int ln_linssh;          /* &namdom: linear free surface (fixed levels)              */
  int ln_zps;             /* partial-step bottom gradients in lap/iso (domzgr)        */
  int ln_isfcav;          /* ice-shelf cavities: must be 0                            */
  int ln_traldf_lap;      /* &namtra_ldf operator: laplacian                          */
  int ln_traldf_blp;      /*                       bilaplacian                        */
  int ln_traldf_iso;      /* direction: iso-neutral (standard operator)               */
  int ln_traldf_msc;      /* method of stabilizing correction                         */
  double rn_aht_0;        /* constant eddy diffusivity aht0 = 1/2 Ud Ld used when the
                             ahtu/ahtv fields are not bound (ldftra.F90:296-308) [m2/s] */
  int ln_zdfddm;          /* &namzdf: double diffusion (separate avs for salinity)    */
  int ln_zad_Aimp;        /* adaptive-implicit vertical advection: must be 0          */
  int ln_bt_fw;           /* &namdyn_spg: forward barotropic integration              */
  int ln_bt_av;           /*              time filtering of barotropic variables      */
  int nn_bt_flt;          /*              filter: 0 none, 1 boxcar nn_baro, 2 boxcar 2 */
  int ln_bt_auto;         /*              nn_baro from rn_bt_cmax                      */
  int nn_baro;            /*              sub-steps per rn_rdt when ln_bt_auto = 0     */
  double rn_bt_cmax;      /*              maximum barotropic Courant number            */
  double rn_bt_alpha;     /*              temporal diffusion parameter                 */
  int nvor_scheme;        /* &namdyn_vor: enum nemo_vor                                */
  int nn_een_e3f;         /*              e3f averaging of the EEN scheme              */
  int ln_dynadv_vec;      /* &namdyn_adv: vector-form momentum advection               */
  int ln_sco;             /* s-coordinate (dom_oce)                                    */
  int ln_apr_dyn;         /* &namsbc_apr: atmospheric pressure forcing in dyn          */
  double rn_scal_load;    /* &namsbc_tide scalar loading factor                        */
  double grav;            /* phycst.F90:38                                             */
  double rau0;            /* reference density (eosbn2)                                */
  int nn_fct_h;           /* &namtra_adv: FCT order in the horizontal (2 or 4; 0 = 2)  */
  int nn_fct_v;           /*              and the vertical (2 or 4; 0 = 2), used by
                             nemo_gpu_stp_hotpath                                       */
  double rn_slpmax;       /* &namtra_ldf: maximum iso-neutral slope (0 = 0.01)         */
  int    ln_traqsr;       /* &namsbc: solar radiation penetrates (tra_qsr, 2 bands)     */
  double rn_abs, rn_si0, rn_si1; /* &namtra_qsr: near-surface fraction, extinction depths */
  double rcp;             /* specific heat (eosbn2.F90:1245: 3991.86795711963; 0 = that) */
  int    ln_seos;         /* &nameos: the simplified equation of state (the only one here) */
  double rn_a0, rn_b0, rn_lambda1, rn_lambda2, rn_mu1, rn_mu2, rn_nu; /* &nameos S-EOS  */
  int    ln_eos80;        /* &nameos: the polynomial EOS-80 equation of state (GYRE's;
                             exclusive with ln_seos)                                   */
  /* &namzdf / &namzdf_tke (zdf_phy with the TKE closure and zdf_evd) */
  int    ln_zdftke;       /* TKE closure for avt, avm (zdftke.F90)                     */
  int    ln_zdfevd;       /* enhanced vertical diffusion where unstable (zdfevd.F90)   */
  int    nn_evdm;         /*   on tracers (0) or tracers and momentum (1)              */
  double rn_evd;          /*   mixing coefficient [m2/s]                               */
  double rn_avm0, rn_avt0;/* background viscosity and diffusivity [m2/s] (nn_avb = 0)  */
  double rn_ediff, rn_ediss, rn_ebb, rn_emin, rn_emin0, rn_bshear; /* TKE coefficients */
  int    nn_pdl;          /* Prandtl number a function of Ri (1) or not (0)           */
  int    nn_mxl;          /* mixing length: 0..3                                       */
  int    ln_mxl0;         /* surface mixing length from the wind stress               */
  double rn_mxl0;         /* surface mixing length minimum (ln_mxl0 = 0)              */
  int    ln_lc;           /* Langmuir cells (Axell 2002)                               */
  double rn_lc;
  int    nn_etau;         /* tke penetration below the mixed layer: 0 only here        */
  int    ln_drg_tke;      /* friction as TKE boundary condition (ln_drg): 0 only here */
  /* &namdyn_adv: the momentum advection of nemo_gpu_stp_model */
  int    ln_dynadv_OFF;   /* linear dynamics (no momentum advection; Coriolis only)    */
  int    nn_dynkeg;       /* grad(KE) scheme: 0 C2 (1, Hollingsworth: not supported)   */
  /* &namsbc: the user-defined (GYRE analytic) surface forcing, formed each model step */
  int    ln_usr;
  /* &namtra_ldf: the triad direction (exclusive with ln_traldf_iso) and its options */
  int    ln_traldf_triad;
  int    ln_triad_iso;    /* pure horizontal mixing in the mixed layer                 */
  int    ln_botmix_triad; /* lateral mixing on the bottom half cells                   */
  double rn_sw_triad;     /* 1 switching triads, 0 all four triads used                */
} nemo_namelist;

/* ------------------------------------------------------- module-global fields
 * Arrays the reference routines read from Fortran modules rather than from their
 * argument lists (oce.F90, dom_oce.F90, zdf_oce.F90, ldfslp.F90, sbc_oce.F90,
 * zdfdrg.F90, dynspg_ts.F90). The caller binds device arrays to them once; the
 * dimension of each is given in brackets. T = 3-D (jpi,jpj,jpk), S = 2-D (jpi,jpj),
 * TS = (jpi,jpj,jpk,2), G = (jpi,jpj,2). */
enum nemo_field_id {
  NEMO_F_TSB = 0,   /* [TS] before tracers tsb                         oce.F90        */
  NEMO_F_TSN,       /* [TS] now tracers tsn                                           */
  NEMO_F_TSA,       /* [TS] tracer trend / after tracers tsa                          */
  NEMO_F_UN, NEMO_F_VN, NEMO_F_WN,     /* [T] now velocities                          */
  NEMO_F_UB, NEMO_F_VB,                /* [T] before velocities                       */
  NEMO_F_UA, NEMO_F_VA,                /* [T] momentum trends                         */
  NEMO_F_AVT, NEMO_F_AVS,              /* [T] vertical diffusivities   zdf_oce.F90    */
  NEMO_F_AHTU, NEMO_F_AHTV,            /* [T] lateral diffusivities    ldftra.F90     */
  NEMO_F_USLP, NEMO_F_VSLP,            /* [T] iso-neutral slopes       ldfslp.F90     */
  NEMO_F_WSLPI, NEMO_F_WSLPJ,
  NEMO_F_AH_WSLP2, NEMO_F_AKZ,         /* [T] written by tra_ldf_iso, read by zdf     */
  NEMO_F_E3T_B, NEMO_F_E3T_N, NEMO_F_E3T_A,   /* [T] time-varying scale factors       */
  NEMO_F_E3U_N, NEMO_F_E3V_N, NEMO_F_E3W_N,
  NEMO_F_GTSU, NEMO_F_GTSV,            /* [G] partial-step bottom gradients (zpshde)  */
  NEMO_F_GTUI, NEMO_F_GTVI,            /* [G] partial-step top gradients              */
  NEMO_F_SSHB, NEMO_F_SSHN, NEMO_F_SSHA,      /* [S] sea surface height (ssha: FP64)  */
  NEMO_F_UB_B, NEMO_F_VB_B,            /* [S] before barotropic velocities            */
  NEMO_F_UN_B, NEMO_F_VN_B,            /* [S] now barotropic velocities               */
  NEMO_F_UA_B, NEMO_F_VA_B,            /* [S] after barotropic velocities (FP64)      */
  NEMO_F_UN_ADV, NEMO_F_VN_ADV,        /* [S] time-filtered transports (FP64)         */
  NEMO_F_UB2_B, NEMO_F_VB2_B,          /* [S] half-step fluxes, restart field (FP64)  */
  NEMO_F_UN_BF, NEMO_F_VN_BF,          /* [S] filtered half-step fluxes (FP64)        */
  NEMO_F_UTAU, NEMO_F_VTAU,            /* [S] wind stress                 sbc_oce.F90 */
  NEMO_F_UTAU_B, NEMO_F_VTAU_B,
  NEMO_F_EMP, NEMO_F_EMP_B,            /* [S] evaporation minus precipitation         */
  NEMO_F_RNF, NEMO_F_RNF_B,            /* [S] runoff                                  */
  NEMO_F_RCDU_BOT,                     /* [S] bottom drag coefficient x |U|  zdfdrg   */
  NEMO_F_SSH_IB, NEMO_F_SSH_IBB,       /* [S] inverse-barometer ssh       sbcapr.F90  */
  /* Variable volume (ln_linssh = 0) only, maintained by domvvl.F90 (:183-196,
   * :631-661); with ln_linssh = 1 the rest-state ht_0, hu_0, ... and e3f_0 are used
   * whether bound or not. */
  NEMO_F_HT_N,                         /* [S] now ocean depth at T-points             */
  NEMO_F_HU_N, NEMO_F_HV_N,            /* [S] now ocean depth at U-/V-points          */
  NEMO_F_R1_HU_N, NEMO_F_R1_HV_N,      /* [S] their masked inverses                   */
  NEMO_F_HU_B, NEMO_F_HV_B,            /* [S] before depths (centred integration or
                                              flux-form momentum, ln_dynadv_vec = 0)   */
  NEMO_F_R1_HU_B, NEMO_F_R1_HV_B,      /* [S] (centred integration)                   */
  NEMO_F_E3F_N,                        /* [T] now e3 at F-points (ENE/ENS/MIX schemes) */
  /* Adjoint support (FP64 contexts; no counterpart in the reference): while bound,
   * nemo_gpu_tra_adv_fct records its limiter multipliers here and
   * nemo_gpu_tra_adv_fct_adj reads them. 3 * kjpt * jpi*jpj*jpk doubles per
   * member, ordered (member, tracer, face x/y/z, k, j, i); 0 where the forward
   * zeroed the antidiffusive flux. */
  NEMO_F_FCT_TAPE,
  /* ldf_slp (ldfslp.F90) module inputs: depths of the now T- and W-points
   * (dom_oce gdept_n, gdepw_n), and the mixed layer of zdf_mxl (zdfmxl.F90): its
   * level nmln (int32 in both precisions), depth hmlp and the depth of its last
   * T-point hmlpt. */
  NEMO_F_GDEPT_N, NEMO_F_GDEPW_N,      /* [T]                                         */
  NEMO_F_NMLN, NEMO_F_HMLP, NEMO_F_HMLPT, /* [S]                                      */
  /* Surface boundary condition of the tracers (sbc_oce.F90): the non-solar and solar
   * heat fluxes qns, qsr [W/m2] and the salt flux sfx (with emp above); sbc_tsc and
   * sbc_tsc_b, the now and before tracer-content trends of the forcing,
   * (jpi,jpj,jpts) restart fields; qsr_hc and qsr_hc_b (jpi,jpj,jpk), the now and
   * before heat-content trends of the penetrating solar flux (restart fields);
   * fraqsr_1lev, the fraction of qsr absorbed in the first level. */
  NEMO_F_QNS, NEMO_F_QSR, NEMO_F_SFX,  /* [S]                                         */
  NEMO_F_SBC_TSC, NEMO_F_SBC_TSC_B,    /* [S] x jpts                                  */
  NEMO_F_QSR_HC, NEMO_F_QSR_HC_B,      /* [T]                                         */
  NEMO_F_FRAQSR_1LEV,                  /* [S]                                         */
  /* in situ density anomaly rhd (the input of dyn_hpg) and potential density rhop of
   * the model step's eos (oce.F90) */
  NEMO_F_RHD, NEMO_F_RHOP,             /* [T]                                         */
  /* zdf_mxl (zdfmxl.F90): its input, the before Brunt-Vaisala frequency rn2b
   * (zdf_oce), and its turbocline depth hmld (written when bound) */
  NEMO_F_RN2B,                         /* [T]                                         */
  NEMO_F_HMLD,                         /* [S]                                         */
  /* lateral eddy viscosity at T- and F-points (ldfdyn.F90 ahmt, ahmf, masked) */
  NEMO_F_AHMT, NEMO_F_AHMF,            /* [T]                                         */
  /* vertical physics (zdf_oce.F90, zdftke.F90): the vertical eddy viscosity avm, the
   * turbulent closure's coefficients avm_k, avt_k, the turbulent kinetic energy en
   * and its dissipation dissl (restart fields), the now Brunt-Vaisala frequency rn2
   * (the before one is NEMO_F_RN2B), the wind-stress module taum (sbc_oce.F90) and
   * the sea-ice fraction fr_i (unbound = 0) */
  NEMO_F_AVM, NEMO_F_AVM_K, NEMO_F_AVT_K, NEMO_F_EN, NEMO_F_DISSL, /* [T]            */
  NEMO_F_RN2,                          /* [T]                                         */
  NEMO_F_TAUM, NEMO_F_FR_I,            /* [S]                                         */
  /* latitudes of the T-, U- and V-points (dom_oce gphit, gphiu, gphiv) [degrees], read
   * by GYRE's analytic surface forcing (nemo_gpu_usrdef_sbc) */
  NEMO_F_GPHIT, NEMO_F_GPHIU, NEMO_F_GPHIV, /* [S]                                    */
  /* the horizontal gradients of the in situ density at the last ocean level of u- and
   * v-points (oce.F90 gru, grv; zps_hde with partial steps), read by ldf_slp */
  NEMO_F_GRU, NEMO_F_GRV,              /* [S]                                         */
  /* z* time stepping (domvvl.F90, dynnxt.F90; dom_oce.F90 names): the after scale
   * factors at u- and v-points and the after column depths of dom_vvl_sf_nxt, the
   * before (time-filtered) scale factors of dyn_nxt, the remaining now and before
   * scale factors, depths and gde3w of dom_vvl_sf_swp, and the rest-state e3uw_0,
   * e3vw_0 (domain-file inputs, read only when E3UW_N/E3VW_N are bound). */
  NEMO_F_E3U_A, NEMO_F_E3V_A,          /* [T]                                         */
  NEMO_F_HU_A, NEMO_F_HV_A, NEMO_F_R1_HU_A, NEMO_F_R1_HV_A, /* [S]                    */
  NEMO_F_E3U_B, NEMO_F_E3V_B, NEMO_F_E3W_B, /* [T]                                    */
  NEMO_F_E3UW_N, NEMO_F_E3VW_N, NEMO_F_E3UW_B, NEMO_F_E3VW_B, /* [T]                  */
  NEMO_F_GDEPT_B, NEMO_F_GDEPW_B, NEMO_F_GDE3W_N, /* [T]                              */
  NEMO_F_E3UW_0, NEMO_F_E3VW_0,        /* [T]                                         */
  /* the triad operator (ldfslp.F90 module arrays of ldf_slp_triad): the slopes of the
   * four i-k (j-k) triads of each T-point relative to geopotentials (triadi_g,
   * triadj_g) and to the model levels (triadi, triadj), each (jpi,jpj,jpk,0:1,0:1)
   * in Fortran order, i.e. 4 x jpi*jpj*jpk per member; wslp2 [T] */
  NEMO_F_TRIADI_G, NEMO_F_TRIADJ_G, NEMO_F_TRIADI, NEMO_F_TRIADJ,
  NEMO_F_WSLP2,
  NEMO_F_COUNT
};

typedef struct nemo_ctx nemo_ctx;

/* ------------------------------------------------------------- life cycle */

/* Create a context: uploads the domain (nemo_dom_desc) and the namelist subset,
 * derives masks and metrics, computes the barotropic sub-step count and weights
 * (dyn_spg_ts_init, dynspg_ts.F90:1466-1493, and ts_wgt, :1313-1388), and
 * allocates the library-owned work arrays (the reference's automatic arrays such
 * as zwx, zwy, zwz, zwi at traadv_fct.F90:86). stream is a cudaStream_t, or NULL
 * for a stream the context creates. Replaces the allocation/initialisation done
 * in nemo_init (nemogcm.F90:249-472) for the fields of this path. */
int nemo_gpu_create(const nemo_dom_desc *dom, const nemo_namelist *nam,
                    int nmembers, int prec, void *stream, nemo_ctx **out);
int nemo_gpu_destroy(nemo_ctx *ctx);

/* Text of the last error of this context ("" if none). */
const char *nemo_gpu_last_error(const nemo_ctx *ctx);

/* Wait for all work of the context; reports asynchronous kernel errors. */
int nemo_gpu_synchronize(nemo_ctx *ctx);

/* Bind a device array to a module-global field (enum nemo_field_id).
 * Passing NULL unbinds it (e.g. NEMO_F_AHTU = NULL selects the constant rn_aht_0,
 * the e3 fields = NULL select the rest-state e3*_0 of the domain). */
int nemo_gpu_bind(nemo_ctx *ctx, int field_id, void *dev_ptr);

/* Number of elements (per member) and precision of a field (1 = FP64, 0 = 4-byte
 * elements: FP32, or int32 for NEMO_F_NMLN). */
size_t nemo_gpu_field_numel(const nemo_ctx *ctx, int field_id);
int nemo_gpu_field_is_fp64(const nemo_ctx *ctx, int field_id);

/* Barotropic sub-step count icycle, and nn_baro after ln_bt_auto (dynspg_ts.F90:1491). */
int nemo_gpu_spg_info(const nemo_ctx *ctx, int *icycle, int *nn_baro, double *rdtbt);

/* Copy between a host buffer and a bound field (all members). Both are
 * asynchronous and ordered with the context's work per field. An upload of a field
 * of 1 MB or more copies the host buffer into a device staging buffer of the field
 * (made at its first upload) on a copy stream, as soon as the staging buffer's
 * previous contents are in the field; the work that next reads or writes the field,
 * or a download of it, first copies the staged data into the field on its own stream
 * (after the field's pending download). So the next step's uploads run while this
 * step still reads the fields, and of two uploads of a field with no work between
 * them the later one wins. A smaller field is copied straight into place after the
 * work already queued and its pending download. A download runs after the work already queued that writes the field (after
 * nemo_gpu_stp_hotpath: the fields dyn_spg_ts writes as soon as dyn_spg_ts ends) and
 * after a pending upload of it. Uploads run in call order on one copy stream and
 * downloads on another, so one step's downloads overlap the next step's uploads.
 * When nemo_gpu_stp_hotpath is called with copies in flight, each of its parts
 * waits only for the copies of the fields it reads or writes (dyn_spg_ts starts
 * while the tracers still upload); other routines wait for all pending copies.
 * Upload fields in the order the step reads them: dyn_spg_ts's (ua, va, the 2-D
 * fields), the slopes, un vn wn tsn, then the rest. Host memory should be pinned;
 * read a downloaded buffer, or reuse an uploaded one, only after
 * nemo_gpu_synchronize. */
int nemo_gpu_field_upload(nemo_ctx *ctx, int field_id, const void *host);
int nemo_gpu_field_download(nemo_ctx *ctx, int field_id, void *host);

/* -------------------------------------------------------------- hot path */

/* Effective transports zun = e2u e3u_n un, zvn = e1v e3v_n vn, zwn = e1e2t wn with
 * level jpk zeroed (traadv.F90:99-124, no Stokes drift / eiv / mle). */
int nemo_gpu_tra_adv_trp(nemo_ctx *ctx, const void *un, const void *vn, const void *wn,
                         void *zun, void *zvn, void *zwn);

/* tra_adv_fct (traadv_fct.F90:54-327) with nonosc (:330-428) and interp_4th_cpt
 * (:517-616). kn_fct_h in {2,4}, kn_fct_v in {2,4}. cdtype "TRA" or "TRC". */
int nemo_gpu_tra_adv_fct(nemo_ctx *ctx, int kt, int kit000, const char *cdtype, double p2dt,
                         const void *pun, const void *pvn, const void *pwn,
                         const void *ptb, const void *ptn, void *pta,
                         int kjpt, int kn_fct_h, int kn_fct_v);

/* tra_ldf_lap (traldf_lap_blp.F90:47-158). pahu/pahv NULL = rn_aht_0 * umask/vmask.
 * pgu..pgvi (jpi,jpj,kjpt) are read only when ln_zps (they may be NULL otherwise). */
int nemo_gpu_tra_ldf_lap(nemo_ctx *ctx, int kt, int kit000, const char *cdtype,
                         const void *pahu, const void *pahv,
                         const void *pgu, const void *pgv, const void *pgui, const void *pgvi,
                         const void *ptb, void *pta, int kjpt, int kpass);

/* tra_ldf_iso (traldf_iso.F90:50-382): reads the bound slopes, writes the bound
 * ah_wslp2 and akz on kpass = 1. */
int nemo_gpu_tra_ldf_iso(nemo_ctx *ctx, int kt, int kit000, const char *cdtype,
                         const void *pahu, const void *pahv,
                         const void *pgu, const void *pgv, const void *pgui, const void *pgvi,
                         const void *ptb, const void *ptbb, void *pta, int kjpt, int kpass);

/* tra_sbc (trasbc.F90:53-206): the surface forcing trend of the tracers. Reads the
 * bound qns, qsr, emp, sfx, tsn and e3t_n; swaps and fills the bound sbc_tsc_b,
 * sbc_tsc; adds zfact * (sbc_tsc_b + sbc_tsc) / e3t_n to the first level of the bound
 * tsa (zfact = 1 on an Euler first step, else 1/2). Without ln_traqsr, qsr is first
 * moved into qns (:76-79). Runoff (ln_rnf) and ice-shelf melt (ln_isf) are not
 * included; a restart start (neuler = 1 at nit000) keeps the bound sbc_tsc_b as the
 * restart's sbc_hc_b / sbc_sc_b. */
int nemo_gpu_tra_sbc(nemo_ctx *ctx, int kt);

/* tra_qsr (traqsr.F90:77-302), two-band light penetration (ln_qsr_2bd): swaps and
 * fills the bound qsr_hc_b, qsr_hc from the bound qsr and gdepw_n on levels 1..nksr
 * (nksr from trc_oce_ext_lev, trc_oce.F90:215-256, at context creation), adds
 * z1_2 * (qsr_hc_b + qsr_hc) / e3t_n to the temperature of the bound tsa, and sets
 * the bound fraqsr_1lev with its lbc_lnk. The RGB and bio-model bands are not
 * included. Needs ln_traqsr. */
int nemo_gpu_tra_qsr(nemo_ctx *ctx, int kt);

/* The simplified equation of state (ln_seos, eosbn2.F90 np_seos; Vallis 2006) on
 * levels 1..jpk-1 of every point; pts (jpi,jpj,jpk,2), pdep (jpi,jpj,jpk) depths:
 * eos_insitu (:188-301): prd = in situ density anomaly (rho - rau0) / rau0;
 * eos_insitu_pot (:304-470): prd and prhop, the potential density at the surface;
 * rab_3d (:566-676): pab (jpi,jpj,jpk,2) the thermal / haline expansion ratios at
 * the bound gdept_n; bn2 (:889-933): pn2 (jpi,jpj,jpk), the Brunt-Vaisala frequency
 * squared on levels 2..jpk-1 from the bound gdept_n, gdepw_n and e3w_n.
 * NEMO_ERR_UNSUPPORTED without ln_seos (the EOS-80 and TEOS-10 polynomials are not
 * included). */
int nemo_gpu_eos_insitu(nemo_ctx *ctx, const void *pts, void *prd, const void *pdep);
int nemo_gpu_eos_insitu_pot(nemo_ctx *ctx, const void *pts, void *prd, void *prhop, const void *pdep);
int nemo_gpu_rab_3d(nemo_ctx *ctx, const void *pts, void *pab);
int nemo_gpu_bn2(nemo_ctx *ctx, const void *pts, const void *pab, void *pn2);

/* dyn_hpg with hpg_zco (dynhpg.F90:258-323, z-coordinate with full steps): adds the
 * hydrostatic pressure gradient of the bound rhd to the bound ua, va. */
int nemo_gpu_dyn_hpg(nemo_ctx *ctx, int kt);

/* dyn_ldf_lap (dynldf_lap_blp.F90:37-104): adds the iso-level laplacian viscous
 * trend -curl(ahmf curl u) + grad(ahmt div u) of pub, pvb (jpi,jpj,jpk) to pua, pva,
 * with the bound ahmt and ahmf (kpass 2: the second pass of the bilaplacian, minus
 * sign). Linear free surface (e3*_b = e3*_n); e3f from the bound e3f_n or the rest
 * state. */
int nemo_gpu_dyn_ldf_lap(nemo_ctx *ctx, int kt, const void *pub, const void *pvb, void *pua, void *pva, int kpass);

/* vor_ene (dynvor.F90:324-429), the energy-conserving vorticity trend added to pua,
 * pva from the now velocities pun, pvn (jpi,jpj,jpk), z-coordinate without
 * ln_dynvor_msk: kvor 1 (np_COR, planetary), 2 (np_RVO, relative) or 4 (np_CRV,
 * both: dyn_vor's ntot with the vector-form momentum); the metric terms of the flux
 * form (3, 5) are NEMO_ERR_UNSUPPORTED. */
int nemo_gpu_vor_ene(nemo_ctx *ctx, int kt, int kvor, const void *pun, const void *pvn, void *pua, void *pva);

/* dyn_keg (dynkeg.F90, nkeg_C2 = 0): subtracts the gradient of the horizontal
 * kinetic energy of the bound un, vn from the bound ua, va; the Hollingsworth form
 * (kscheme 1) is NEMO_ERR_UNSUPPORTED. dyn_zad (dynzad.F90): subtracts the vertical
 * advection of the bound un, vn by the bound wn. */
int nemo_gpu_dyn_keg(nemo_ctx *ctx, int kt, int kscheme);
int nemo_gpu_dyn_zad(nemo_ctx *ctx, int kt);

/* zdf_mxl (zdfmxl.F90:59-141): the mixed layer of the bound rn2b (density criterion
 * rho_c = 0.01 integrated from the first W-level below 10 m, nlb10 of domzgr.F90:144-
 * 146) into the bound nmln (int32), hmlp and hmlpt, and the turbocline of the bound
 * avt (avt_c = 5e-4) into hmld when bound; reads the bound gdept_n and gdepw_n. */
int nemo_gpu_zdf_mxl(nemo_ctx *ctx, int kt);

/* zdf_phy (zdfphy.F90:243-316) with the TKE closure (ln_zdftke: tke_tke and tke_avn,
 * zdftke.F90:168-630, with Langmuir cells (ln_lc), the Prandtl number of nn_pdl and
 * the mixing lengths of nn_mxl; nn_etau = 0 and ln_drg off as in GYRE) and zdf_evd
 * (ln_zdfevd, nn_evdm, zdfevd.F90:40-121): the shear production zdf_sh2
 * (zdfsh2.F90:30-76) from the closure's avm_k of the last call, then en and dissl,
 * avm_k and avt_k, the ocean avm and avt on levels 2..jpk-1 with evd where N^2 or the
 * before N^2 is <= -1e-12, avs = avt, and the closed lbc_lnk of the five
 * coefficients. Linear free surface, z-levels. Bound: UB VB UN VN, AVM_K AVT_K AVM AVT
 * (AVS optional), EN DISSL, RN2 RN2B, TAUM, GDEPW_N (FR_I optional, else 0). A cold
 * start binds en = rn_emin wmask, dissl = 1e-12, avm_k = rn_avm0 wmask, avt_k =
 * rn_avt0 wmask (tke_rst, zdftke.F90:778-783, zdf_phy_init). nemo_gpu_stp_model runs it
 * at the head of the step, after rab_3d and bn2 of the before and now tracers (into
 * rn2b and rn2, step.F90:127-133), when an equation of state is selected and these
 * fields and GDEPT_N are bound. */
int nemo_gpu_zdf_phy(nemo_ctx *ctx, int kt);

/* usrdef_sbc_oce (usrdef_sbc.F90:62-190), GYRE's analytic surface forcing at time step
 * kt (year 1 of a 360-day calendar), preceded by sbc's swap of the before fields
 * UTAU_B, VTAU_B, EMP_B when bound and kt /= nit000 (sbcmod.F90:389-394): qsr, the
 * restoring qns from the before SST, E-P less its domain mean (GLOB_SUM) with its heat
 * content at the now SST in qns, sfx = 0, the wind stress utau, vtau and its modulus
 * taum. Bound: GPHIT GPHIU GPHIV TSB TSN QSR QNS EMP SFX UTAU VTAU TAUM. With ln_usr,
 * nemo_gpu_stp_model runs it first (step.F90:116). */
int nemo_gpu_usrdef_sbc(nemo_ctx *ctx, int kt);

/* zps_hde (zpshde.F90:41-148): pgtu, pgtv (jpi,jpj,kjpt) = the horizontal
 * gradients of pta (jpi,jpj,jpk,kjpt) at the partial-step bottom level of the u-
 * and v-points, with lbc_lnk. The optional density part (prd, pgru, pgrv) needs
 * eos and is not implemented. */
int nemo_gpu_zps_hde(nemo_ctx *ctx, int kt, int kjpt, const void *pta, void *pgtu, void *pgtv);

/* zps_hde's density part (zpshde.F90:150-184, the reference's optional arguments prd,
 * pgru, pgrv): pts (jpi,jpj,jpk,2) are T and S; each is interpolated to the shallower
 * bottom depth of the u- (v-) point as the tracer part does, its in situ density there
 * formed by eos_insitu_2d (eosbn2.F90:295-398, EOS-80 or the simplified eos) at
 * gdept_n of the shallower bottom cell, and pgru, pgrv (jpi,jpj) = its difference with
 * prd (jpi,jpj,jpk) on the deeper side, masked, edges 0. Bound: GDEPT_N. Bind the
 * results as NEMO_F_GRU, NEMO_F_GRV for nemo_gpu_ldf_slp with partial steps. */
int nemo_gpu_zps_hde_rd(nemo_ctx *ctx, int kt, const void *pts, const void *prd, void *pgru, void *pgrv);

/* tra_ldf_blp (traldf_lap_blp.F90:161-231): the bilaplacian as two passes of the
 * laplacian, kldf = 20 (np_blp: iso-level, tra_ldf_lap) or 21 (np_blp_i: rotated,
 * tra_ldf_iso), with lbc_lnk of the first laplacian and, with ln_zps, its zps_hde
 * gradients in between (pgu/pgv, the gradients of ptb, are then required). Not the
 * triad operator (kldf = 22). nemo_gpu_stp_hotpath calls it when ln_traldf_blp is
 * set (traldf.F90:75-76). */
int nemo_gpu_tra_ldf_blp(nemo_ctx *ctx, int kt, int kit000, const char *cdtype, const void *pahu,
                         const void *pahv, const void *pgu, const void *pgv, const void *pgui,
                         const void *pgvi, const void *ptb, void *pta, int kjpt, int kldf);

/* ldf_slp_triad (ldfslp.F90:377-617): the triad slopes from the before tracers and
 * their expansion ratios prab_b (jpi,jpj,jpk,2), eos_rab of tsb (step.F90:127), into
 * the bound TRIADI_G, TRIADJ_G, TRIADI, TRIADJ and, when bound, WSLP2. Reads the
 * bound TSB, GDEPT_N, GDEPW_N, NMLN (mixed-layer level) and the now scale factors.
 * No eddy-induced velocity; the partial-step bottom correction of the reference is
 * off (l_grad_zps = .FALSE.). Faces outside the reference's loops keep their values
 * except at levels 1 and jpk, which are zeroed. */
int nemo_gpu_ldf_slp_triad(nemo_ctx *ctx, int kt, const void *prab_b);
/* tra_ldf_triad (traldf_triad.F90:50-429), the same argument list as tra_ldf_iso
 * (pgu, pgv, pgui, pgvi are unread: l_grad_zps = .FALSE.): pass 1 writes the bound
 * AH_WSLP2 and AKZ from the triads (ln_traldf_msc: the stabilising akz), then per
 * tracer the triad fluxes, the 33 flux (laplacian: ah_wslp2 - akz; bilaplacian pass 1
 * ah_wslp2, pass 2 ah_wslp2 on ptb and akz on ptbb) and their divergence added to
 * pta (sign -1 in pass 2). Reads the bound triad arrays and GDEPT_N. */
int nemo_gpu_tra_ldf_triad(nemo_ctx *ctx, int kt, int kit000, const char *cdtype, const void *pahu,
                           const void *pahv, const void *pgu, const void *pgv, const void *pgui,
                           const void *pgvi, const void *ptb, const void *ptbb, void *pta, int kjpt, int kpass);

/* tra_zdf_imp (trazdf.F90:109-268): pta becomes the after tracer. Reads the bound
 * avt (avs), and ah_wslp2/akz when ln_traldf_iso. */
int nemo_gpu_tra_zdf_imp(nemo_ctx *ctx, int kt, int kit000, const char *cdtype, double p2dt,
                         const void *ptb, void *pta, int kjpt);

/* tra_zdf (trazdf.F90:46-106) on the bound tsb/tsa: r2dt choice (:66-68), the
 * implicit solve, then WHERE( tsa(:,:,:,jp_sal) < 0 ) tsa = 0.1 (:83). */
int nemo_gpu_tra_zdf(nemo_ctx *ctx, int kt);

/* tra_nxt (tranxt.F90:66-188) on the bound tsb, tsn, tsa: lbc_lnk of tsa, then at
 * the first step of an Euler start (neuler = 0, kt = nit000) tsn = tsa, otherwise
 * the leapfrog swap with the Asselin filter on the interior and lbc_lnk of tsb and
 * tsn. Linear free surface: tra_nxt_fix (:191-237), tsb = tsn + rn_atfp (tsa - 2 tsn
 * + tsb). Variable volume (ln_linssh = 0): tra_nxt_vvl (:240-380), the
 * thickness-weighted filter of E3T_B, E3T_N, E3T_A with the forcing removed at the
 * first level (EMP_B / EMP, RNF_B / RNF when bound, SBC_TSC / SBC_TSC_B) and, with
 * ln_traqsr, in the penetrating-light levels (QSR_HC / QSR_HC_B); no runoff depth,
 * ice-shelf melt or tracer runoff (ln_rnf). */
int nemo_gpu_tra_nxt(nemo_ctx *ctx, int kt);

/* ------------------------------------------------- the rest of a model step
 * The routines that close the path into a time step with the linear free surface
 * (step.F90:160-282), for a model run on the device. None is on the path itself. */

/* div_hor (divhor.F90:62-110) and wzv (sshwzv.F90:129-213) on the bound un, vn:
 * the horizontal divergence (0 on the closed edges), then wn integrated up from
 * wn(jpk) = 0, with the e3t_a - e3t_b term of z*. */
int nemo_gpu_wzv(nemo_ctx *ctx, int kt);
/* ldf_slp (ldfslp.F90:83-374, with ldf_slp_mxl :620-729): the iso-neutral slopes
 * uslp, vslp, wslpi, wslpj (the bound NEMO_F_USLP, ... fields, levels 2..jpk-1;
 * levels 1 and jpk are left as they are except on the closed edges) from the in
 * situ density anomaly prd and N^2 pn2 (3-D device arrays), the bound depths and
 * mixed layer. z-coordinate (z* with the now e3 and depths bound) without ice-shelf
 * cavities; with partial steps (ln_zps) the bottom level's density gradients are the
 * bound NEMO_F_GRU, NEMO_F_GRV of zps_hde (ldfslp.F90:144-151). */
int nemo_gpu_ldf_slp(nemo_ctx *ctx, int kt, const void *prd, const void *pn2);

/* dyn_zdf (dynzdf.F90:47-499). Its leap-frog time step ua = (ub + r2dt ua) umask, va
 * likewise (:109-114), or with a variable volume and flux-form momentum on the
 * thickness-weighted velocity, ua = (e3u_b ub + r2dt e3u_n ua) / e3u_a umask
 * (:115-120; E3U_B, E3U_N, E3U_A and the v ones bound); and, while the ocean viscosity NEMO_F_AVM is bound, the implicit
 * vertical viscosity of a linear free surface with the split-explicit free surface
 * and implicit bottom drag (ln_drgimp, the reference's default), iso-level lateral
 * mixing and ln_zad_Aimp off: the barotropic after velocity UA_B / VA_B of
 * dyn_spg_ts removed and its bottom stress (RCDU_BOT) added (:122-141), the
 * tridiagonal system of avm with the implicit drag on the bottom diagonal and the
 * wind stress (utau_b + utau) / 2 in the surface right-hand side (UTAU_B, VTAU_B when
 * bound, else UTAU, VTAU), solved per column (:205-302). nemo_gpu_stp_model runs it
 * after dyn_spg_ts. */
int nemo_gpu_dyn_zdf_step(nemo_ctx *ctx, int kt);
/* dyn_nxt (dynnxt.F90:66-377) with ln_dynspg_ts and ln_bt_fw: the barotropic part
 * of ua replaced by ua_b, lbc_lnk, the Euler swap or the Asselin filter and swap
 * with ub returned to the time-split estimate, then un_b, ub_b. Variable volume
 * (ln_linssh = 0) adds the time filter of E3T_B with the forcing removed at the
 * first level (:217-226), E3U_B / E3V_B interpolated from it, the filter on the
 * velocity (ln_dynadv_vec) or on the thickness-weighted velocity (flux form,
 * :277-307), HU_B, HV_B and their inverses, and at the Euler step the copy of
 * E3T_A, E3U_A, E3V_A into the now fields (:172-186); it reads E3U_A, E3V_A,
 * R1_HU_A, R1_HV_A of dom_vvl_sf_nxt and R1_HU_N, R1_HV_N. */
int nemo_gpu_dyn_nxt(nemo_ctx *ctx, int kt);
/* ssh_swp (sshwzv.F90:216-267); with variable volume the forcing (EMP_B - EMP,
 * RNF_B - RNF when bound) removed from the filtered before ssh (:254-258). */
int nemo_gpu_ssh_swp(nemo_ctx *ctx, int kt);
/* dom_vvl_sf_nxt (domvvl.F90:268-562) for z* (ln_vvl_zstar; z-tilde and layer
 * coordinates are not on this path): E3T_A = E3T_B + E3T_N z_scale on the wet
 * levels, z_scale = (ssha - sshb) ssmask / (ht_0 + sshn + 1 - ssmask); E3U_A, E3V_A
 * by dom_vvl_interpol (:678-782: surface-weighted means of the e3t_a change, lbc,
 * plus the rest state); HU_A, HV_A and R1_HU_A, R1_HV_A. Reads SSHA, SSHB, SSHN. */
int nemo_gpu_dom_vvl_sf_nxt(nemo_ctx *ctx, int kt);
/* dom_vvl_sf_swp (domvvl.F90:565-675, z*): GDEPT_B / GDEPW_B = the now depths (when
 * bound), E3T_N, E3U_N, E3V_N = the after fields, E3F_N from E3U_N, E3W_N from
 * E3T_N and E3W_B from E3T_B (and E3UW_N/E3VW_N, E3UW_B/E3VW_B from the u-/v-scale
 * factors when bound, with the rest-state E3UW_0/E3VW_0), the now depths GDEPT_N,
 * GDEPW_N and GDE3W_N (when bound), HU_N, HV_N, R1_HU_N, R1_HV_N = the after ones,
 * HT_N. No restart write (that is nemo_gpu/restart.py's). */
int nemo_gpu_dom_vvl_sf_swp(nemo_ctx *ctx, int kt);
/* One model step on the bound fields, in step.F90's order (:96-305):
 *  - the vertical physics (:127-133), with ln_zdftke, an equation of state and the
 *    fields of nemo_gpu_zdf_phy and gdept_n bound: rab_3d and bn2 of tsb and tsn into
 *    rn2b and rn2, then zdf_phy;
 *  - the iso-neutral slopes (:137-150), with rn2b, rhd, the depths, the mixed-layer
 *    fields and the slopes bound and ln_traldf_iso: (rab_3d and bn2 of tsb unless done
 *    above,) zdf_mxl, eos_insitu of tsb and ldf_slp;
 *  - div_hor + wzv of the now velocities (:156-160; ssha comes from dyn_spg_ts);
 *  - ua = va = 0; dyn_adv in the vector form (dyn_keg C2 + dyn_zad; none with
 *    ln_dynadv_OFF), dyn_vor (vor_ene of the total vorticity; the Coriolis term alone
 *    with ln_dynadv_OFF; the ENE scheme only), dyn_ldf (the iso-level laplacian of ub,
 *    vb, while ahmt and ahmf are bound) (:188-192);
 *  - with rhd and rhop bound: eos_insitu_pot of tsn at gdept_n and dyn_hpg (:165, :193);
 *  - dyn_spg_ts, div_hor + wzv, dyn_zdf (the implicit vertical viscosity while avm is
 *    bound), tsa = 0, tra_sbc and tra_qsr (when their fields are bound; tra_qsr with
 *    ln_traqsr), tra_adv, tra_ldf, tra_zdf (with the salinity clamp), tra_nxt,
 *    dyn_nxt, ssh_swp, dia_hsb (after nemo_gpu_dia_hsb_init), stp_ctl (:305).
 * With ln_usr the step opens with GYRE's analytic forcing (nemo_gpu_usrdef_sbc; its
 * time-dependent scalars are written to the device ahead of each step, so the
 * captured graph replays with the step's own). Captured into a CUDA graph like
 * nemo_gpu_stp_hotpath. Linear free surface with ln_bt_fw. */
int nemo_gpu_stp_model(nemo_ctx *ctx, int kt);

/* ------------------------------------------------------------ adjoint
 * Adjoints of the tracer routines with respect to their tracer arguments, in an
 * FP64 context (NEMO_ERR_ARG otherwise). NEMO has no adjoint of these routines in
 * its tree (its tangent-linear/adjoint, NEMOTAM, is a separate project), so these
 * entry points have no reference counterpart; each keeps the argument list of its
 * forward routine with the tracer arrays replaced by their adjoints, and is the
 * transpose of the forward's tangent-linear with the coefficients (transports,
 * diffusivities, slopes, scale factors, avt, ah_wslp2/akz as the forward left them)
 * held fixed. An adjoint accumulates into the adjoints of the inputs
 * (ptb_ad += ...); the adjoint of a trend array that the forward only adds to
 * (pta_ad of tra_adv_fct and tra_ldf_*) is read and left unchanged. */

/* FCT with the limiter multipliers the forward call recorded in NEMO_F_FCT_TAPE held
 * fixed: ptb_ad += A_b^T pta_ad, ptn_ad += A_n^T pta_ad. pun, pvn, pwn are the forward
 * call's transports; kn_fct_h = 2 or 4 (the 4th-order centred horizontal fluxes,
 * traadv_fct.F90:191-227), kn_fct_v = 2 or 4 (the compact 4th-order vertical
 * interpolation interp_4th_cpt, :517-616, transposed column by column). */
int nemo_gpu_tra_adv_fct_adj(nemo_ctx *ctx, int kt, int kit000, const char *cdtype, double p2dt,
                             const void *pun, const void *pvn, const void *pwn, void *ptb_ad,
                             void *ptn_ad, const void *pta_ad, int kjpt, int kn_fct_h, int kn_fct_v);
/* tra_ldf_lap: ptb_ad += L^T pta_ad. With ln_zps the bottom faces take the fixed
 * pgu/pgv, so nothing flows through them. */
int nemo_gpu_tra_ldf_lap_adj(nemo_ctx *ctx, int kt, int kit000, const char *cdtype, const void *pahu,
                             const void *pahv, const void *pgu, const void *pgv, const void *pgui,
                             const void *pgvi, void *ptb_ad, const void *pta_ad, int kjpt, int kpass);
/* tra_ldf_iso: ptb_ad += ..., and ptbb_ad += ... for kpass = 2 without
 * ln_traldf_lap (ptbb_ad may be NULL otherwise). Reads the bound ah_wslp2/akz. */
int nemo_gpu_tra_ldf_iso_adj(nemo_ctx *ctx, int kt, int kit000, const char *cdtype, const void *pahu,
                             const void *pahv, const void *pgu, const void *pgv, const void *pgui,
                             const void *pgvi, void *ptb_ad, void *ptbb_ad, const void *pta_ad, int kjpt,
                             int kpass);
/* tra_zdf_imp: on entry pta_ad is the adjoint of the after tracer, on exit that
 * of the trend the forward read; ptb_ad += e3t_b M^-T pta_ad. */
int nemo_gpu_tra_zdf_imp_adj(nemo_ctx *ctx, int kt, int kit000, const char *cdtype, double p2dt,
                             void *ptb_ad, void *pta_ad, int kjpt);
/* tra_nxt on three (jpi,jpj,jpk,2) adjoint arrays: on entry the adjoints of the
 * swapped tsb, tsn, tsa, on exit those of the fields before the swap. */
int nemo_gpu_tra_nxt_adj(nemo_ctx *ctx, int kt, void *tsb_ad, void *tsn_ad, void *tsa_ad);

/* Adjoint arrays of dyn_spg_ts (FP64, laid out like the fields they shadow, per
 * member): of the outputs only -- ssha, ua_b, va_b, un_adv, vn_adv: read, then
 * zeroed (the forward overwrites them); in and out -- ua, va, un, vn (3-D) and ub2_b,
 * vb2_b, un_bf, vn_bf: on entry the adjoint of the value after the call, on exit
 * that of the value before; of the inputs only -- sshn, un_b, vn_b, ub_b, vb_b:
 * accumulated. */
typedef struct nemo_spg_adj {
  void *ua, *va, *un, *vn;
  void *ssha, *ua_b, *va_b, *un_adv, *vn_adv;
  void *ub2_b, *vb2_b, *un_bf, *vn_bf;
  void *sshn, *un_b, *vn_b, *ub_b, *vb_b;
} nemo_spg_adj;
/* dyn_spg_ts_adj: the adjoint of nemo_gpu_dyn_spg_ts (dynspg_ts.F90:121-1310) with
 * respect to the state, with the forcing (wind stress, E-P, runoff, atmospheric
 * pressure), the bottom drag coefficient and the Coriolis factors held fixed: phase
 * 3, the sub-steps in reverse order, phase 1. Linear free surface, ln_bt_fw and
 * ln_bt_av (every step starts the sub-steps from sshn, un_b, vn_b), the vorticity
 * schemes ENE, ENS, EEN and MIX (not ENT: NEMO_ERR_UNSUPPORTED). Uses the sub-step
 * count and weights of the forward's last call: run nemo_gpu_dyn_spg_ts(kt) first. */
int nemo_gpu_dyn_spg_ts_adj(nemo_ctx *ctx, int kt, const nemo_spg_adj *adj);

/* The adjoints of the time stepping of the model step, linear free surface, FP64.
 * wzv_adj (sshwzv.F90:129-213 with divhor.F90:62-110): un_ad, vn_ad += the transpose
 * of the map (un, vn) -> wn applied to wn_ad; wn_ad (of the output only) is zeroed.
 * The thickness-change term is a constant of the map. */
int nemo_gpu_wzv_adj(nemo_ctx *ctx, int kt, void *un_ad, void *vn_ad, void *wn_ad);
/* Adjoint arrays of dyn_nxt: in and out -- ua, va, un, vn, ub, vb (3-D) and un_b,
 * vn_b; of the outputs only -- ub_b, vb_b (read, then zeroed); of the inputs only --
 * ua_b, va_b (FP64 like the forward's, accumulated). */
typedef struct nemo_nxt_adj {
  void *ua, *va, *un, *vn, *ub, *vb;
  void *un_b, *vn_b, *ub_b, *vb_b;
  void *ua_b, *va_b;
} nemo_nxt_adj;
/* dyn_nxt_adj: the adjoint of nemo_gpu_dyn_nxt (dynnxt.F90:66-377) for ln_linssh with
 * ln_dynspg_ts and ln_bt_fw, one column per thread. */
int nemo_gpu_dyn_nxt_adj(nemo_ctx *ctx, int kt, const nemo_nxt_adj *adj);
/* ssh_swp_adj (sshwzv.F90:216-267, linear free surface): on entry the adjoints of the
 * swapped sshb, sshn and of ssha, on exit those of the values before the swap. */
int nemo_gpu_ssh_swp_adj(nemo_ctx *ctx, int kt, void *sshb_ad, void *sshn_ad, void *ssha_ad);

/* dyn_spg_ts (dynspg_ts.F90:121-1310) on the bound fields: phase 1 forcing,
 * icycle barotropic sub-steps in one persistent kernel, phase 3 correction. */
int nemo_gpu_dyn_spg_ts(nemo_ctx *ctx, int kt);

/* lbc_lnk for one array of nk levels (nk = 1 for a 2-D array) and nl 4th-dim
 * slices, closed-basin branch of lbc_lnk_generic.h90:80-105. cd_nat in
 * T,U,V,W,F; psgn is only used across a north fold (not supported). The array
 * is FP64 when is_fp64 != 0, else FP32. */
int nemo_gpu_lbc_lnk(nemo_ctx *ctx, const char *cdname, void *ptab, int nk, int nl,
                     const char *cd_nat, double psgn, double pval, int is_fp64);

/* lbc_lnk_multi (lbc_lnk_multi_generic.h90:16-40): kfld arrays in one launch. */
int nemo_gpu_lbc_lnk_multi(nemo_ctx *ctx, const char *cdname, int kfld, void *const *ptabs,
                           const int *nk, const char *cd_nats, const double *psgns,
                           double pval, int is_fp64);

/* glob_sum (lib_fortran_generic.h90:32-65 with DDPDD, lib_fortran.F90:300-332):
 * sum of ptab(:,:,k) * tmask_i over nk levels in double-double arithmetic, one
 * result per member written to the host array out[nmembers]. ptab is FP64 when
 * is_fp64 != 0. */
int nemo_gpu_glob_sum(nemo_ctx *ctx, const char *cdname, const void *ptab, int nk,
                      int is_fp64, double *out);

/* glob_sum without any device allocation, for callers that cannot allocate at
 * the point of the call: hosts whose device memory belongs to another runtime
 * (OpenACC / CUDA Fortran data regions, a coupler's caching allocator), which must
 * not see allocations made behind its back, and set-ups that fix their device
 * footprint at start-up. This entry point has no counterpart in the reference
 * (whose glob_sum is lib_fortran_generic.h90:32-65); it computes the same masked
 * double-double sum as nemo_gpu_glob_sum but needs no context: ptab holds nmembers
 * consecutive (jpi,jpj,nk) fields (FP64 when is_fp64 != 0, else FP32), tmask_i is
 * the (jpi,jpj) FP64 interior mask, and out receives nmembers sums -- all three are
 * DEVICE pointers; stream is a cudaStream_t or NULL. The block partial sums live
 * in a static device array of the library (about 1 MB, held by every GPU that
 * loads it until the process exits), so at most 64 members per call; larger
 * requests return NEMO_ERR_ARG. The first call on each device looks up that
 * array's device address (cudaGetSymbolAddress); make it before any stream
 * capture. Calls that overlap on the GPU (other streams, other host threads)
 * share the array and race: serialise them. */
int nemo_gpu_glob_sum_noalloc(const void *ptab, const double *tmask_i, int jpi, int jpj, int nk,
                              int nmembers, int is_fp64, void *stream, double *out);

/* ------------------------------------------------ run control and budgets */

/* Sizes of the per-member results of stp_ctl and dia_hsb below. */
#define NEMO_CTL_N 6
#define NEMO_CTL_NLOC 11
#define NEMO_HSB_N 16

/* stp_ctl (stpctl.F90:44-194): the test of extrema of every member on the device
 * (:112-127): |ssh| max, |U| max (zonal velocity, every point), and the maxima of
 * -S, S, -T, T over tmask = 1 (a NaN makes its extremum NaN); then the blow-up test
 * (:149-157) when the domain has ocean points. Enqueued on the context's stream; no
 * host synchronisation. If it fires for a member, the next nemo_gpu_synchronize
 * returns NEMO_ERR_BLOWUP (the reference's ctl_stop / kindic = -3), and
 * nemo_gpu_stp_ctl_result gives the values and positions. nemo_gpu_stp_model runs
 * it at the end of every step (step.F90:305). */
int nemo_gpu_stp_ctl(nemo_ctx *ctx, int kt);
/* The last stp_ctl's results (synchronises): per member m, zmax[NEMO_CTL_N*m ..] =
 * |ssh| max, |U| max, -S min, S max, -T min, T max (the reference's zmax(1:6));
 * loc[NEMO_CTL_NLOC*m ..] = the 1-based positions of :158-170 (i j of |ssh| max,
 * i j k of |U| max, S min, S max; 0 when the test did not fire); kindic[m] = -3 when
 * it fired, else 0. Each pointer may be NULL. */
int nemo_gpu_stp_ctl_result(nemo_ctx *ctx, double *zmax, int *loc, int *kindic);

/* dia_hsb (diahsb.F90): heat, salt and volume budgets with FP64 compensated
 * (double-double) global sums, in both precisions. nemo_gpu_dia_hsb_init is
 * dia_hsb_rst( nit000, 'READ' ) of a run without restart (:283-311): it records the
 * initial ssh, scale factors and contents of the bound fields and zeroes the
 * forcing sums; after it nemo_gpu_stp_model runs dia_hsb after ssh_swp
 * (step.F90:282). nemo_gpu_dia_hsb is one call of :60-239 (without runoff, ice-shelf
 * and geothermal inputs; rnf enters the volume flux where bound); it reads SSHN,
 * TSN, TSB, E3T_N (or the rest state), EMP, SBC_TSC, WN (ln_linssh) and QSR
 * (ln_traqsr), and masks tsn and tsb in place as the reference does (:88-89). */
int nemo_gpu_dia_hsb_init(nemo_ctx *ctx);
int nemo_gpu_dia_hsb(nemo_ctx *ctx, int kt);
/* The last dia_hsb's terms (synchronises): per member m, out[NEMO_HSB_N*m ..] =
 * frc_v, frc_t, frc_s, frc_wn_t, frc_wn_s (the accumulated forcing), zdiff_v1,
 * zdiff_v2, zdiff_hc, zdiff_sc (drifts after the forcing, :174-178), zdiff_hc1,
 * zdiff_sc1, zerr_hc1, zerr_sc1 (linear free surface, :179-185, else 0), zvol_tot,
 * surf_tot, 0. The reference's diagnostics follow from them, e.g. the temperature
 * drift bgtemper = zdiff_hc1 / zvol_tot (linear free surface). */
int nemo_gpu_dia_hsb_result(nemo_ctx *ctx, double *out);

/* The path of one timestep stp (step.F90:194-257) on the bound fields, in the
 * reference's order: dyn_spg_ts, tsa = 0 (:234), tra_adv (transports + FCT),
 * tra_ldf (lap or iso, per the namelist), tra_zdf (implicit + salinity clamp).
 * The first call for a class of kt (Euler start, leapfrog) is captured in a CUDA
 * graph that later calls replay. */
int nemo_gpu_stp_hotpath(nemo_ctx *ctx, int kt);

/* ------------------------------------------------------------ timing */

/* Per-routine device timing of nemo_gpu_stp_hotpath, the counterpart of the
 * reference's ln_timing (timing.F90:89-212, timing_start/stop around tra_adv,
 * tra_ldf, tra_zdf, dyn_spg). While on, the hot path runs without graph replay and
 * records CUDA events between routines. ms[0..3] = cumulative milliseconds in
 * dyn_spg_ts, tra_adv, tra_ldf, tra_zdf since timing was switched on. Where the
 * iso-neutral operator is fused into FCT (ln_traldf_iso without blp), tra_ldf is
 * the iso-neutral flux kernel and tra_adv the three FCT stages, the last of which
 * also adds the iso-neutral divergence. */
int nemo_gpu_set_timing(nemo_ctx *ctx, int on);
int nemo_gpu_get_timing(nemo_ctx *ctx, double *ms, int *ncalls);

/* The kernels of the library, for per-kernel timing. */
enum nemo_kernel_id {
  NEMO_K_ADV_TRP, NEMO_K_INTERP4, NEMO_K_FCT_A, NEMO_K_FCT_B, NEMO_K_FCT_C, NEMO_K_LDF_LAP,
  NEMO_K_ISO_FLUX, NEMO_K_ISO_DIV, NEMO_K_ISO_AKZ_EDGES, NEMO_K_ISO_MSC_EDGES, NEMO_K_ZDF_IMP,
  NEMO_K_CLAMP, NEMO_K_SPG_P1A, NEMO_K_SPG_P1B, NEMO_K_SPG_P2, NEMO_K_SPG_P3,
  NEMO_K_SPG_COR,   /* variable volume: Coriolis factors of the step */
  NEMO_K_ISO_FLUX_TMA, /* iso-neutral fluxes with TMA-staged tracer planes */
  NEMO_K_FCT_FUSED,    /* FCT stages a, b, c in one kernel, TMA-staged inputs */
  NEMO_K_FCT_A_TMA, NEMO_K_FCT_B_TMA, /* FCT stages a, b with TMA-staged planes */
  NEMO_K_FCT_ADJ, NEMO_K_LAP_ADJ, NEMO_K_ISO_ADJ, NEMO_K_ZDF_ADJ, /* adjoints */
  NEMO_K_TRA_NXT, NEMO_K_TRA_NXT_ADJ,
  NEMO_K_WZV, NEMO_K_DYN_ZDF_STEP, NEMO_K_DYN_NXT, NEMO_K_SSH_SWP, /* rest of the model step */
  NEMO_K_LDF_SLP,      /* the three iso-neutral slope kernels */
  NEMO_K_ZPS_HDE,      /* partial-step bottom gradients */
  NEMO_K_TRA_SBC, NEMO_K_TRA_QSR, /* surface forcing of the tracers */
  NEMO_K_EOS, NEMO_K_BN2, NEMO_K_DYN_HPG, /* equation of state, N^2, pressure gradient */
  NEMO_K_ZDF_MXL,      /* mixed-layer depth */
  NEMO_K_DYN_LDF,      /* lateral viscosity */
  NEMO_K_DYN_VOR,      /* vorticity trend */
  NEMO_K_DYN_KEG, NEMO_K_DYN_ZAD, /* momentum advection, vector form */
  NEMO_K_STP_CTL, NEMO_K_DIA_HSB, /* run control extrema, conservation budgets */
  NEMO_K_ZDF_PHY,      /* shear production, TKE closure, enhanced vertical diffusion */
  NEMO_K_USR_SBC,      /* GYRE's analytic surface forcing */
  NEMO_K_VVL_SF,       /* z*: the after scale factors and the swap (dom_vvl_sf_nxt/_swp) */
  NEMO_K_VVL_NXT,      /* z*: tra_nxt_vvl, dyn_nxt's filter of e3 and velocities, ssh_swp */
  NEMO_K_TRIAD,        /* the triad operator: slopes, coefficients, fluxes, divergence */
  NEMO_K_SPG_ADJ,      /* the adjoint of dyn_spg_ts (phase 3, reverse sub-steps, phase 1) */
  NEMO_K_STEP_ADJ,     /* the adjoints of wzv, dyn_nxt, ssh_swp */
  NEMO_K_COUNT
};

/* Autotuner of the hot path's launch shapes (no counterpart in the reference):
 * runs nrep timed steps of nemo_gpu_stp_hotpath at step kt (> nit000 + 1) for each
 * candidate block height (32 x 4, 32 x 2, 32 x 1) of the 32-wide kernels and keeps,
 * per kernel, the fastest; every bound field the step writes is put back before
 * each trial and at the end, so the state is as before the call. The TMA-staged
 * kernels and the persistent sub-step kernel keep their fixed tiles. */
int nemo_gpu_autotune(nemo_ctx *ctx, int kt, int nrep);
/* The block heights in use, ty[id] per nemo_kernel_id (n entries). */
int nemo_gpu_get_launch_shape(const nemo_ctx *ctx, int *ty, int n);
/* Set them (n entries from kernel id 0): 0 or 4 = 32 x 4; 2 or 1 only for the
 * kernels the autotuner tunes (NEMO_ERR_ARG otherwise). The results do not depend
 * on the shape: a test runs the step under each and requires the same bits. */
int nemo_gpu_set_launch_shape(nemo_ctx *ctx, const int *ty, int n);

/* Per-kernel device timing of nemo_gpu_stp_hotpath while timing is on (no
 * counterpart in the reference, whose timing stops at routines): a CUDA event is
 * recorded on the context's stream after every kernel launch, so
 * ms[id] = cumulative milliseconds between the end of the previous kernel and the
 * end of kernel id, launches[id] = how many launches of it were timed. Both arrays
 * hold NEMO_K_COUNT entries; n is their length (entries past NEMO_K_COUNT are 0). */
int nemo_gpu_get_kernel_timing(nemo_ctx *ctx, double *ms, int *launches, int n);

/* ------------------------------------------------------------ kernel choice */

/* on = 1 (default): in a mixed-precision context whose configuration allows it
 * (FCT 2/2, linear free surface, z-coordinate, constant eddy diffusivity,
 * iso-neutral laplacian) nemo_gpu_stp_hotpath runs FCT advection and iso-neutral
 * diffusion as one fused kernel; on = 0 forces the per-routine kernels. */
int nemo_gpu_set_fusion(nemo_ctx *ctx, int on);

/* on = 1 (default): in a mixed-precision context, the iso-neutral flux kernel of that
 * configuration stages the tracer planes in shared memory with tensor copies (TMA)
 * when jpi is a multiple of 4; on = 0 forces the kernel without TMA. Same results. */
int nemo_gpu_set_tma(nemo_ctx *ctx, int on);

/* on = 1: with TMA on (nemo_gpu_set_tma), the three FCT stages of that configuration
 * run as ONE kernel that keeps the intermediates (monotone guess, antidiffusive
 * fluxes, limiter coefficients) in shared memory and recomputes them on the tile
 * halos instead of storing them; on = 0 (default): three kernels. Same results. */
int nemo_gpu_set_fct_fused(nemo_ctx *ctx, int on);

/* The sub-step kernel of dyn_spg_ts in the mixed form with a linear free surface
 * and the ENE/MIX vorticity scheme: on (default) the specialised kernel where the
 * grid allows it, off the general one (both compute the same sub-steps; tests
 * compare them). No counterpart in the reference. */
int nemo_gpu_set_spg_specialised(nemo_ctx *ctx, int on);

/* ------------------------------------------------------------ test hook */

/* Bound of the grid barriers of the persistent sub-step kernel: each wait gives up
 * after max_spins polls and the next nemo_gpu_synchronize() returns
 * NEMO_ERR_TIMEOUT. extra_arrivals > 0 makes every barrier wait for blocks that do
 * not exist, so that the timeout path can be exercised without faulting the GPU. */
int nemo_gpu_set_barrier_limit(nemo_ctx *ctx, long long max_spins, int extra_arrivals);

/* Bound of each wait of the TMA-staged tracer kernels on their tensor copies:
 * max_polls polls of at most ~1 us each (default 65536). When a wait gives up, the
 * kernel records the failure, still waits (with its own fixed bound) for every copy
 * it has issued, and returns; the next nemo_gpu_synchronize() returns
 * NEMO_ERR_TIMEOUT. max_polls = 0 makes the first wait give up at once, so that the
 * timeout path can be exercised without faulting the GPU. */
int nemo_gpu_set_tma_poll_limit(nemo_ctx *ctx, int max_polls);

#ifdef __cplusplus
}
#endif
#endif /* NEMO_GPU_H */
