/*
 * nemo_oracle.h -- CPU FP64 restatement of NEMO 4.0's per-timestep stencil path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker the parity tests, the smoke test
 * and the CPU-baseline leg of the benchmark compare the CUDA library against; it is
 * never linked into, loaded by or called from the product path.
 *
 * Parity status: UNPINNED against the reference's own outputs. NEMO cannot be built
 * in this environment (no Fortran compiler, MPI or NetCDF) and its tree ships no
 * golden vectors or known-answer tests for these routines. Each function below
 * restates the cited Fortran line for line (same loop bounds, same expression
 * association, no FMA contraction: build with -ffp-contract=off) and is pinned by
 * the analytic known-answer properties in tests/test_oracle_kat.py.
 *
 * The functions mirror the C ABI of include/nemo_gpu.h with host pointers and an
 * ora_ prefix, for one ensemble member; the module-global fields are bound with
 * ora_bind() using the same enum nemo_field_id.
 */
#ifndef NEMO_ORACLE_H
#define NEMO_ORACLE_H

#include "../include/nemo_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_ctx ora_ctx;

int ora_create(const nemo_dom_desc *dom, const nemo_namelist *nam, ora_ctx **out);
int ora_destroy(ora_ctx *c);
int ora_bind(ora_ctx *c, int field_id, double *host_ptr);
int ora_spg_info(const ora_ctx *c, int *icycle, int *nn_baro, double *rdtbt);
/* OpenMP threads of the parallel loops (n < 1: unchanged); returns the setting. */
int ora_set_threads(int n);
/* Derived domain arrays for inspection: name in tmask, umask, vmask, wmask (3-D),
 * ssmask, ssumask, ssvmask, tmask_i, ht_0, hu_0, hv_0, r1_hu_0, r1_hv_0, e1e2t,
 * r1_e1e2t (2-D), wgtbtp1, wgtbtp2 (3*nn_baro). Returns NULL for an unknown name. */
const double *ora_array(const ora_ctx *c, const char *name);
const int *ora_iarray(const ora_ctx *c, const char *name); /* mikt mbkt mbku mbkv */

int ora_tra_adv_trp(ora_ctx *c, const double *un, const double *vn, const double *wn,
                    double *zun, double *zvn, double *zwn);
int ora_tra_adv_fct(ora_ctx *c, int kt, int kit000, const char *cdtype, double p2dt,
                    const double *pun, const double *pvn, const double *pwn,
                    const double *ptb, const double *ptn, double *pta,
                    int kjpt, int kn_fct_h, int kn_fct_v);
int ora_interp_4th_cpt(ora_ctx *c, const double *pt_in, double *pt_out);
int ora_interp_4th_cpt_adj(ora_ctx *c, const double *pv, double *pt_ad);
int ora_tra_ldf_lap(ora_ctx *c, int kt, int kit000, const char *cdtype,
                    const double *pahu, const double *pahv,
                    const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                    const double *ptb, double *pta, int kjpt, int kpass);
int ora_tra_ldf_iso(ora_ctx *c, int kt, int kit000, const char *cdtype,
                    const double *pahu, const double *pahv,
                    const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                    const double *ptb, const double *ptbb, double *pta, int kjpt, int kpass);
int ora_zps_hde_rd(ora_ctx *c, int kt, const double *pts, const double *prd, double *pgru, double *pgrv);
int ora_zps_hde(ora_ctx *c, int kt, int kjpt, const double *pta, double *pgtu, double *pgtv);
int ora_tra_ldf_blp(ora_ctx *c, int kt, int kit000, const char *cdtype,
                    const double *pahu, const double *pahv,
                    const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                    const double *ptb, double *pta, int kjpt, int kldf);
int ora_tra_zdf_imp(ora_ctx *c, int kt, int kit000, const char *cdtype, double p2dt,
                    const double *ptb, double *pta, int kjpt);
int ora_tra_zdf(ora_ctx *c, int kt);
int ora_dyn_spg_ts(ora_ctx *c, int kt);
int ora_lbc_lnk(ora_ctx *c, double *ptab, int nk, int nl, char cd_nat, double psgn, double pval);
/* zdf_phy with zdf_sh2, the TKE closure and zdf_evd (see nemo_gpu_zdf_phy) */
double ora_sin(double x);
double ora_cos(double x);
int ora_usrdef_sbc(ora_ctx *c, int kt);
double ora_sin_0pi(double x);
int ora_zdf_phy(ora_ctx *c, int kt);
/* stp_ctl (stpctl.F90:44-194): zmax[NEMO_CTL_N], loc[NEMO_CTL_NLOC], kindic */
int ora_stp_ctl(ora_ctx *c, int kt, double *zmax, int *loc, int *kindic);
/* dia_hsb (diahsb.F90): the initial state of the budgets, then one step's budget
 * terms out[NEMO_HSB_N] (see nemo_gpu_dia_hsb_result) */
int ora_dia_hsb_init(ora_ctx *c);
int ora_dia_hsb(ora_ctx *c, int kt, double *out);
/* stp_ctl and dia_hsb of the last ora_stp_model */
int ora_stp_ctl_last(const ora_ctx *c, double *zmax, int *loc, int *kindic);
int ora_dia_hsb_last(const ora_ctx *c, double *out);
int ora_glob_sum(ora_ctx *c, const double *ptab, int nk, double *out);
int ora_stp_hotpath(ora_ctx *c, int kt);
/* Adjoints with respect to the tracer arguments (the coefficients held fixed).
 * tape: 3 * kjpt * jpi*jpj*jpk doubles of FCT limiter multipliers; mode 1 makes
 * ora_tra_adv_fct record them, mode 2 replay them (tangent-linear), 0 neither. */
int ora_set_fct_tape(ora_ctx *c, double *tape, int mode);
int ora_tra_adv_fct_adj(ora_ctx *c, int kt, int kit000, const char *cdtype, double p2dt,
                        const double *pun, const double *pvn, const double *pwn,
                        double *ptb_ad, double *ptn_ad, const double *pta_ad,
                        int kjpt, int kn_fct_h, int kn_fct_v);
int ora_tra_ldf_lap_adj(ora_ctx *c, int kt, int kit000, const char *cdtype,
                        const double *pahu, const double *pahv,
                        const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                        double *ptb_ad, const double *pta_ad, int kjpt, int kpass);
int ora_tra_ldf_iso_adj(ora_ctx *c, int kt, int kit000, const char *cdtype,
                        const double *pahu, const double *pahv,
                        const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                        double *ptb_ad, double *ptbb_ad, const double *pta_ad, int kjpt, int kpass);
int ora_tra_zdf_imp_adj(ora_ctx *c, int kt, int kit000, const char *cdtype, double p2dt,
                        double *ptb_ad, double *pta_ad, int kjpt);
int ora_tra_nxt(ora_ctx *c, int kt);
int ora_tra_nxt_adj(ora_ctx *c, int kt, double *tsb_ad, double *tsn_ad, double *tsa_ad);
/* adjoint of ora_dyn_spg_ts; the arrays of nemo_spg_adj are double * */
int ora_dyn_spg_ts_adj(ora_ctx *c, int kt, const nemo_spg_adj *adj);
/* adjoints of the step's time stepping (linear free surface) */
int ora_wzv_adj(ora_ctx *c, int kt, double *un_ad, double *vn_ad, double *wn_ad);
int ora_dyn_nxt_adj(ora_ctx *c, int kt, const nemo_nxt_adj *adj);
int ora_ssh_swp_adj(ora_ctx *c, int kt, double *sshb_ad, double *sshn_ad, double *ssha_ad);
/* The rest of a linear-free-surface step, and one model step built from them and
 * the path (momentum trends outside the path and vertical viscosity held at 0). */
int ora_wzv(ora_ctx *c, int kt);
int ora_dyn_zdf_step(ora_ctx *c, int kt);
int ora_dyn_nxt(ora_ctx *c, int kt);
int ora_ssh_swp(ora_ctx *c, int kt);
/* z* time stepping: dom_vvl_sf_nxt (domvvl.F90:268-562) and dom_vvl_sf_swp (:565-675) */
int ora_dom_vvl_sf_nxt(ora_ctx *c, int kt);
int ora_dom_vvl_sf_swp(ora_ctx *c, int kt);
int ora_stp_model(ora_ctx *c, int kt);
/* ldf_slp with ldf_slp_mxl (z-coordinate, no cavities, no partial steps); NMLN is
 * bound as an int array. */
/* the triad operator: ldf_slp_triad (ldfslp.F90:377-617), tra_ldf_triad (traldf_triad.F90:50-429) */
int ora_ldf_slp_triad(ora_ctx *c, int kt, const double *prab_b);
int ora_tra_ldf_triad(ora_ctx *c, int kt, int kit000, const char *cdtype, const double *pahu,
                      const double *pahv, const double *pgu, const double *pgv, const double *pgui,
                      const double *pgvi, const double *ptb, const double *ptbb, double *pta, int kjpt, int kpass);
int ora_ldf_slp(ora_ctx *c, int kt, const double *prd, const double *pn2);
/* tra_sbc and tra_qsr (two bands) on the bound surface forcing; nksr: the level of
 * light extinction found at creation. */
int ora_tra_sbc(ora_ctx *c, int kt);
int ora_tra_qsr(ora_ctx *c, int kt);
int ora_nksr(const ora_ctx *c);
/* the simplified equation of state, N^2 and hpg_zco */
int ora_eos_insitu(ora_ctx *c, const double *pts, double *prd, const double *pdep);
int ora_eos_insitu_pot(ora_ctx *c, const double *pts, double *prd, double *prhop, const double *pdep);
int ora_rab_3d(ora_ctx *c, const double *pts, double *pab);
int ora_bn2(ora_ctx *c, const double *pts, const double *pab, double *pn2);
int ora_dyn_hpg(ora_ctx *c, int kt);
/* zdf_mxl; nlb10, the first W-level below 10 m */
int ora_zdf_mxl(ora_ctx *c, int kt);
int ora_nlb10(const ora_ctx *c);
int ora_dyn_keg(ora_ctx *c, int kt, int kscheme);
int ora_dyn_zad(ora_ctx *c, int kt);
int ora_vor_ene(ora_ctx *c, int kt, int kvor, const double *pun, const double *pvn, double *pua, double *pva);
int ora_dyn_ldf_lap(ora_ctx *c, int kt, const double *pub, const double *pvb, double *pua, double *pva, int kpass);
/* 1: start the work arrays standing for Fortran automatic arrays as NaN */
void ora_set_poison(int on);

#ifdef __cplusplus
}
#endif
#endif
