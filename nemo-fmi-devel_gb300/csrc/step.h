// step.h -- host launchers of the rest-of-step kernels (k_step.cuh), defined in
// inst_step.cu for both precisions.
#pragma once
#include "k_diag.cuh"
#include "k_tra.cuh"
#include "k_vvl.cuh"

namespace nemo {

template <class T, class A>
struct NxtArgs {
  T *ua, *va, *un, *vn, *ub, *vb;   // (jpi,jpj,jpk) per member
  T *un_b, *vn_b, *ub_b, *vb_b;     // (jpi,jpj) per member
  const A *ua_b, *va_b;             // after barotropic velocities of dyn_spg_ts
  T atfp;
  int euler;
};

template <class T>
struct SlpArgs {
  const T *prd, *pn2;                  // in situ density anomaly, N^2 (3-D per member)
  const T *gdept, *gdepw;              // depths of the now T-, W-points (3-D)
  const int* nmln;                     // mixed-layer level (2-D, int)
  const T *hmlp, *hmlpt;               // mixed-layer depth, depth of its last T-point
  const T *gru_b, *grv_b;              // partial steps: zps_hde's bottom gradients (2-D), else null
  T *uslp, *vslp, *wslpi, *wslpj;      // out
  T *uml, *vml, *wiml, *wjml, *hu, *hv;  // work (2-D): slopes below the mixed layer
  T *zu, *zv, *zwi, *zwj;              // work (3-D): slopes before the filter
  T zeps, zm1_g, zm1_2g, z1_slpmax;
};

// tra_sbc: mode 0 swaps sbc_tsc into sbc_tsc_b, 1 zeroes both (Euler first step),
// 2 zeroes sbc_tsc and keeps sbc_tsc_b (restart first step)
template <class T>
struct SbcArgs {
  T *qns, *qsr;                       // (jpi,jpj) per member; qsr moved into qns without ln_traqsr
  const T *emp, *sfx, *tsn;
  T *tsc, *tsc_b;                     // (jpi,jpj,2) per member
  T* tsa;
  T r1_rau0, r1_rau0_rcp, zfact;
  int traqsr, linssh, mode;
};

// tra_qsr, two bands: mode as for tra_sbc (qsr_hc into qsr_hc_b)
template <class T>
struct QsrArgs {
  const T *qsr, *gdepw;
  T *hc, *hc_b, *fraq, *tsa;
  T zz0, zz1, xsi0r, xsi1r, z1_2, r1_rau0_rcp;
  int nksr, mode;
};

// The simplified equation of state (np_seos), rab_3d and bn2; member strides are
// those of the bound fields (2 x n3 for pts and pab, n3 for the others).
template <class T>
struct EosArgs {
  const T *pts, *pdep, *gdept, *gdepw, *pab_in;
  T *prd, *prhop, *pab, *pn2;
  T a0, b0, lambda1, lambda2, mu1, mu2, nu, rau0, r1_rau0, grav;
  int what;  // 0 eos_insitu, 1 eos_insitu_pot, 2 rab_3d, 3 bn2
  // EOS-80 (ln_eos80): FP64 evaluates the reference's table in its association
  // (e80_raw: [table][k][i][j], eos80.h); FP32 the same polynomials re-expanded about
  // the salinity 35 (e80_tay, same layout, in s' = zs - e80_s0), the density's
  // constant term kept apart (e80_rho0, and e80_anom = e80_rho0 - rau0)
  int eos80;
  const double* e80_raw;
  const float* e80_tay;
  float e80_s0, e80_rho0, e80_anom;
};

template <class T>
struct MxlArgs {
  const T *rn2b, *avt, *gdept, *gdepw;
  int* nmln;
  T *hmlp, *hmlpt, *hmld;  // hmld may be null
  T zn2_c, avt_c;
  int nlb10;
};

// dyn_zdf with the implicit vertical viscosity: the ocean avm, the bottom drag
// rcdu (2-D), the wind stress (utau_b may be utau), the barotropic after velocity of
// dyn_spg_ts (FP64 in both precisions); work: the diagonal and upper diagonal of the
// system, n3 per member each (u and v in turn)
template <class T>
struct DynZdfArgs {
  const T *ub, *vb, *avm, *rcdu, *utau, *vtau, *utau_b, *vtau_b;
  const double *ua_b, *va_b;
  T *ua, *va, *zwd, *zws;
  T r2dt, zdt, rau0;
};

// GYRE's analytic surface forcing (usrdef_sbc.F90). s: the step's scalars formed on
// the host (usr_scalars): the amplitude and the denominator of T*, 23.5 zcos_sais1,
// the two seasonal factors of E-P, ztaun, and the swap flag (kt /= nit000); gsum:
// glob_sum of the raw E-P per member; the before fields may be null.
template <class T>
struct UsrSbcArgs {
  const T *gphit, *gphiu, *gphiv, *tsb, *tsn;
  T *qsr, *qns, *emp, *sfx, *utau, *vtau, *taum, *utau_b, *vtau_b, *emp_b;
  const double *s, *gsum;
  double zsurf, rcp;
};

// zdf_phy with the TKE closure and zdf_evd. Member strides n3 (3-D) and n2 (taum,
// fr_i). Work arrays (n3 per member): sh2, apdlr (the inverse Prandtl number), and
// the three diagonals of the TKE system, whose storage the mixing lengths zmxlm
// (zdiag) and zmxld (zd_up) take over once the system is solved.
template <class T>
struct ZphyArgs {
  const T *ub, *vb, *un, *vn, *rn2, *rn2b, *taum, *gdepw, *fr_i;  // fr_i may be null
  T *avm_k, *avt_k, *avm, *avt, *avs, *en, *dissl;                 // avs may be null
  T *sh2, *apdlr, *zdiag, *zd_up, *zd_lw;
  T rdt, zbbrau, zfact1, zfact2, zfact3, rn_emin, rn_emin0, rn_bshear, rn_ediff, rn_lc, rn_evd;
  T rn_avm0, rn_avt0, ri_cri, rmxl_min, rn_mxl0, zraug, rsmall, lc_cof1, lc_cof2, rpi;
  int nn_pdl, nn_mxl, ln_mxl0, ln_lc, ln_zdfevd, nn_evdm;
};

template <class T>
cudaError_t launch_dyn_ldf_lap(const Dom<T>& d, const T* ahmt, const T* ahmf, const T* pub, const T* pvb, T* pua, T* pva,
                               T zsign, cudaStream_t s);
template <class T>
cudaError_t launch_vor_ene(const Dom<T>& d, int kvor, const T* pun, const T* pvn, T* pua, T* pva, cudaStream_t s);
template <class T>
cudaError_t launch_dyn_keg(const Dom<T>& d, const T* un, const T* vn, T* ua, T* va, cudaStream_t s);
template <class T>
cudaError_t launch_dyn_zad(const Dom<T>& d, const T* un, const T* vn, const T* wn, T* ua, T* va, cudaStream_t s);
template <class T>
cudaError_t launch_zdf_mxl(const Dom<T>& d, const MxlArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_dyn_zdf_imp(const Dom<T>& d, const DynZdfArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_usr_sbc_a(const Dom<T>& d, const UsrSbcArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_usr_sbc_b(const Dom<T>& d, const UsrSbcArgs<T>& a, cudaStream_t s);
cudaError_t launch_usr_put(double* dst, const double* v, cudaStream_t s);
template <class T>
cudaError_t launch_zdf_phy(const Dom<T>& d, const ZphyArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_eos(const Dom<T>& d, const EosArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_dyn_hpg(const Dom<T>& d, const T* rhd, T* ua, T* va, T zcoef0, cudaStream_t s);
template <class T>
cudaError_t launch_tra_sbc(const Dom<T>& d, const SbcArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_tra_qsr(const Dom<T>& d, const QsrArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_zps_hde_rd(const Dom<T>& d, const EosArgs<T>& a, const T* prd, T* pgru, T* pgrv, cudaStream_t s);
template <class T>
cudaError_t launch_zps_hde(const Dom<T>& d, const T* pta, T* pgtu, T* pgtv, int kjpt, cudaStream_t s);
template <class T>
cudaError_t launch_ldf_slp(const Dom<T>& d, const SlpArgs<T>& a, cudaStream_t s);

template <class T>
cudaError_t launch_wzv(const Dom<T>& d, const T* un, const T* vn, T* wn, T z1_2dt, cudaStream_t s);
template <class T>
// e3u_b ... e3v_a null: the time step on the velocity; else on the thickness-weighted
// velocity (variable volume, flux-form momentum)
cudaError_t launch_dyn_zdf_step(const Dom<T>& d, const T* ub, const T* vb, T* ua, T* va, T r2dt, const T* e3u_b,
                                const T* e3v_b, const T* e3u_a, const T* e3v_a, cudaStream_t s);
template <class T>
cudaError_t launch_dyn_nxt(const Dom<T>& d, const NxtArgs<T, double>& a, cudaStream_t s);
template <class T>
cudaError_t launch_ssh_swp(const Dom<T>& d, T* sshb, T* sshn, const double* ssha, T atfp, int euler, cudaStream_t s);
// z* time stepping (k_vvl.cuh); d0: the domain with the rest-state scale factors
template <class T>
cudaError_t launch_vvl_sf_nxt(const Dom<T>& d0, const VvlArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_vvl_sf_swp(const Dom<T>& d0, const VvlArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_tra_nxt_vvl(const Dom<T>& d0, const VvlArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_dyn_nxt_vvl(const Dom<T>& d0, const VvlArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_ssh_swp_vvl(const Dom<T>& d0, const VvlArgs<T>& a, T* sshb, T* sshn, cudaStream_t s);
// stp_ctl: block partials part (nblk x nmem records), results out (32 doubles a member)
template <class T>
cudaError_t launch_stp_ctl(const Dom<T>& d, const T* sshn, const T* un, const T* ts, double* part, int nblk,
                           int someoce, double* out, unsigned long long* idx, int* flag, cudaStream_t s);
// dia_hsb: the initial fields, and one call (block partials part: nblk x nmem x 13 pairs)
template <class T>
cudaError_t launch_hsb_init(const Dom<T>& d, const HsbArgs<T>& a, int nblk, cudaStream_t s);
template <class T>
cudaError_t launch_dia_hsb(const Dom<T>& d, const HsbArgs<T>& a, double* part, int nblk, cudaStream_t s);

}  // namespace nemo
