/*
 * nemo_oracle.c -- CPU FP64 restatement of NEMO 4.0's stencil hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; see nemo_oracle.h). Parity is UNPINNED
 * against the reference's own outputs (NEMO cannot be built here and ships no
 * golden vectors); it is pinned by analytic known-answer tests.
 *
 * Every routine restates the cited Fortran loop nest with the same loop bounds and
 * the same left-to-right association of + - * /. Arrays are Fortran column-major
 * with 1-based index helpers I2/I3/I4. Automatic Fortran work arrays that the
 * reference leaves undefined outside the loop ranges are zero-filled here; the
 * routines never read those points (this is checked by the NaN-poisoning test).
 * Compile with -ffp-contract=off so that no multiply-add is fused.
 */
#include "nemo_oracle.h"
#include "../nemo-fmi-devel_gb300/csrc/eos80.h"
#include "../nemo-fmi-devel_gb300/csrc/nemo_sin.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* Loops whose iterations write disjoint points run in parallel for the CPU
 * baseline; every point is computed by the same operations in the same order. */
#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

#define I2(i, j) ((size_t)((i)-1) + (size_t)jpi * (size_t)((j)-1))
#define I3(i, j, k) (I2(i, j) + (size_t)jpi * (size_t)jpj * (size_t)((k)-1))
#define I4(i, j, k, n) (I3(i, j, k) + (size_t)jpi * (size_t)jpj * (size_t)jpk * (size_t)((n)-1))

struct ora_ctx {
  int jpi, jpj, jpk;
  nemo_namelist nam;
  double *e1t, *e2t, *e1u, *e2u, *e1v, *e2v, *e1f, *e2f, *ff_f, *ff_t;
  double *r1_e1t, *r1_e2t, *r1_e1u, *r1_e2u, *r1_e1v, *r1_e2v;
  double *e1e2t, *r1_e1e2t, *e1e2u, *e1e2v, *r1_e1e2u, *r1_e1e2v, *e2_e1u, *e1_e2v;
  int *mikt, *mbkt, *mbku, *mbkv;
  double *tmask, *umask, *vmask, *wmask;
  double *ssmask, *ssumask, *ssvmask, *tmask_h, *tmask_i;
  double *e3t_0, *e3u_0, *e3v_0, *e3w_0, *e3f_0;
  double *ht_0, *hu_0, *hv_0, *r1_hu_0, *r1_hv_0;
  double *ahtu_c, *ahtv_c; /* constant masked diffusivity (ldftra.F90:292-372) */
  /* dyn_spg_ts module state */
  int nn_baro, icycle;
  int nksr;  /* level of light extinction of tra_qsr's two bands */
  double rdtbt;
  double *wgtbtp1, *wgtbtp2, *zwz, *ftne, *ftnw, *ftse, *ftsw;
  double *sshn_e, *sshb_e, *sshbb_e, *un_e, *ub_e, *ubb_e, *vn_e, *vb_e, *vbb_e;
  double *ssha_e, *ua_e, *va_e, *hu_e, *hv_e, *hur_e, *hvr_e;
  double r2dt;
  double *f[NEMO_F_COUNT];
  /* FCT limiter multipliers (3 faces x kjpt fields): 1 = record, 2 = replay */
  double *fct_tape;
  int fct_tape_mode;
  /* dia_hsb module state (diahsb.F90:40-52): set by ora_dia_hsb_init */
  int hsb_on;
  double surf_tot, frc_v, frc_t, frc_s, frc_wn_t, frc_wn_s;
  double *surf, *surf_ini, *ssh_ini, *ssh_hc_loc_ini, *ssh_sc_loc_ini, *e3t_ini, *hc_loc_ini, *sc_loc_ini;
  double hsb_out[NEMO_HSB_N];
  /* the last stp_ctl of the model step */
  double ctl_zmax[NEMO_CTL_N];
  int ctl_loc[NEMO_CTL_NLOC], ctl_kindic;
};

static void spg_coriolis_factors(ora_ctx *c, const double *ht_n, const double *e3f_n);

/* Work arrays of the routines come from a small per-thread pool of freed blocks
 * (a block of the same length is reused), so that a time loop over the routines
 * allocates only on its first step, as the reference's automatic arrays live on
 * the stack. The pool keeps at most WP_SLOTS blocks and WP_BYTES bytes. */
#define WP_SLOTS 96
#define WP_BYTES ((size_t)6 << 30)
static _Thread_local struct { double *p[WP_SLOTS]; size_t n[WP_SLOTS]; int cnt; size_t bytes; } g_wpool;

static double *pool_take(size_t n) {
  for (int s = g_wpool.cnt - 1; s >= 0; --s)
    if (g_wpool.n[s] == n) {
      double *p = g_wpool.p[s];
      g_wpool.bytes -= n * sizeof(double);
      g_wpool.p[s] = g_wpool.p[g_wpool.cnt - 1];
      g_wpool.n[s] = g_wpool.n[g_wpool.cnt - 1];
      g_wpool.cnt--;
      return p;
    }
  return (double *)malloc(n * sizeof(double));
}
/* return a block of n doubles from zalloc / walloc to the pool */
static void wfree_n(double *p, size_t n) {
  if (!p) return;
  if (g_wpool.cnt < WP_SLOTS && g_wpool.bytes + n * sizeof(double) <= WP_BYTES) {
    g_wpool.p[g_wpool.cnt] = p;
    g_wpool.n[g_wpool.cnt] = n;
    g_wpool.cnt++;
    g_wpool.bytes += n * sizeof(double);
  } else {
    free(p);
  }
}
/* the length of each block handed out, kept in a header in front of it */
static double *blk_new(size_t n) {
  double *b = pool_take(n + 2);
  if (!b) return NULL;
  b[0] = (double)n;
  return b + 2;
}
static void wfree(double *p) {
  if (p) wfree_n(p - 2, (size_t)p[-2] + 2);
}
/* zero-filled: arrays the reference sets to 0 itself (or reads as 0) */
static double *zalloc(size_t n) {
  n = n ? n : 1;
  double *p = blk_new(n);
  if (!p) return NULL;
  OMP_FOR
  for (size_t i = 0; i < n; ++i) p[i] = 0.0;
  return p;
}

/* Work arrays that stand for the reference's automatic arrays (undefined until
 * written): not cleared. With ora_set_poison(1) they start as NaN, so a test can
 * show that no routine reads a point the reference leaves undefined. */
static int g_poison = 0;
void ora_set_poison(int on) { g_poison = on; }
static double *walloc(size_t n) {
  n = n ? n : 1;
  double *p = blk_new(n);
  if (p && g_poison)
    for (size_t i = 0; i < n; ++i) p[i] = NAN;
  return p;
}

/* OpenMP threads of the routines' parallel loops (the CPU baseline's 1-thread and
 * all-core figures); n < 1 keeps the current setting. */
#ifdef _OPENMP
#include <omp.h>
#endif
int ora_set_threads(int n) {
#ifdef _OPENMP
  if (n >= 1) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

/* SIGN(a,b) of lib_fortran.F90:339-351 (key_nosignedzero): b >= 0 gives |a|. */
static inline double sign_nsz(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }
static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }

/* ------------------------------------------------------------------ lbc_lnk */
/* Closed-basin branch of lbc_lnk_generic.h90:80-105 (jperio = 0): columns 1 and
 * jpi, rows 1 and jpj take pval, except that F-point arrays keep column/row 1. */
static void lbc_closed(int jpi, int jpj, double *a, int nslices, char nat, double pval) {
  for (int s = 0; s < nslices; ++s) {
    double *p = a + (size_t)s * jpi * jpj;
    for (int jj = 1; jj <= jpj; ++jj) {
      if (nat != 'F') p[I2(1, jj)] = pval;
      p[I2(jpi, jj)] = pval;
    }
    for (int ji = 1; ji <= jpi; ++ji) {
      if (nat != 'F') p[I2(ji, 1)] = pval;
      p[I2(ji, jpj)] = pval;
    }
  }
}

int ora_lbc_lnk(ora_ctx *c, double *ptab, int nk, int nl, char cd_nat, double psgn, double pval) {
  (void)psgn;
  if (!c || !ptab || nk < 1 || nl < 1) return NEMO_ERR_ARG;
  lbc_closed(c->jpi, c->jpj, ptab, nk * nl, cd_nat, pval);
  return NEMO_OK;
}

/* ------------------------------------------------------------------ ts_wgt */
/* dynspg_ts.F90:1313-1388 */
static void ts_wgt(ora_ctx *c, int ll_av, int ll_fw, int *jpit, double *zwgt1, double *zwgt2) {
  int nn_baro = c->nn_baro, jic, n3 = 3 * nn_baro;
  for (int i = 0; i < n3; ++i) { zwgt1[i] = 0.0; zwgt2[i] = 0.0; }
  jic = ll_fw ? nn_baro : 2 * nn_baro;
  if (ll_av) {
    switch (c->nam.nn_bt_flt) {
      case 0: zwgt1[jic - 1] = 1.0; *jpit = jic; break;
      case 1:
        for (int jn = 1; jn <= n3; ++jn) {
          double za1 = fabs((double)(jn - jic)) / (double)nn_baro;
          if (za1 < 0.5) { zwgt1[jn - 1] = 1.0; *jpit = jn; }
        }
        break;
      default:
        for (int jn = 1; jn <= n3; ++jn) {
          double za1 = fabs((double)(jn - jic)) / (double)nn_baro;
          if (za1 < 1.0) { zwgt1[jn - 1] = 1.0; *jpit = jn; }
        }
        break;
    }
  } else {
    zwgt1[jic - 1] = 1.0;
    *jpit = jic;
  }
  for (int jn = 1; jn <= *jpit; ++jn)
    for (int ji = jn; ji <= *jpit; ++ji) zwgt2[jn - 1] = zwgt2[jn - 1] + zwgt1[ji - 1];
  double s1 = 0.0, s2 = 0.0;
  for (int jn = 1; jn <= *jpit; ++jn) { s1 += zwgt1[jn - 1]; s2 += zwgt2[jn - 1]; }
  double za1 = 1.0 / s1, za2 = 1.0 / s2;
  for (int jn = 1; jn <= *jpit; ++jn) {
    zwgt1[jn - 1] = zwgt1[jn - 1] * za1;
    zwgt2[jn - 1] = zwgt2[jn - 1] * za2;
  }
}

/* ------------------------------------------------------------------ create */
/* trc_oce_ext_lev (trc_oce.F90:215-256): the last T-level reached by a fraction
 * pqsr_frc of the light with longest extinction depth prldex, or the sea bed. The
 * rest-state W-depths come from e3t_0 as e3_to_depth forms them (DOM/depth_e3.F90):
 * gdepw_0(1) = 0, gdepw_0(k) = gdepw_0(k-1) + e3t_0(k-1). */
static int ext_lev(const ora_ctx *c, const double *e3t_0, double prldex, double pqsr_frc) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  const double zhext = prldex * (log(10.0) * 15.0 + log(pqsr_frc));
  double *gdepw = zalloc(n2 * jpk);
  for (int jk = 2; jk <= jpk; ++jk)
    for (size_t p = 0; p < n2; ++p) gdepw[p + n2 * (jk - 1)] = gdepw[p + n2 * (jk - 2)] + e3t_0[p + n2 * (jk - 2)];
  int pjl = jpk - 1;
  for (int jk = jpk - 1; jk >= 1; --jk) {
    double sum = 0.0, zem = -1e300;
    for (size_t p = 0; p < n2; ++p) sum += c->tmask[p + n2 * (jk - 1)];
    if (sum > 0) {
      for (size_t p = 0; p < n2; ++p) zem = dmax(zem, gdepw[p + n2 * jk] * c->tmask[p + n2 * (jk - 1)]);
      if (zem >= zhext) pjl = jk;
    } else {
      pjl = jk;
    }
  }
  wfree(gdepw);
  return pjl;
}

int ora_create(const nemo_dom_desc *d, const nemo_namelist *nam, ora_ctx **out) {
  if (!d || !nam || !out) return NEMO_ERR_ARG;
  if (d->jpi < 4 || d->jpj < 4 || d->jpk < 3 || d->jperio != 0) return NEMO_ERR_UNSUPPORTED;
  ora_ctx *c = (ora_ctx *)calloc(1, sizeof(ora_ctx));
  const int jpi = d->jpi, jpj = d->jpj, jpk = d->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  c->jpi = jpi; c->jpj = jpj; c->jpk = jpk; c->nam = *nam;
#define CP2(dst, src) do { c->dst = zalloc(n2); memcpy(c->dst, d->src, n2 * sizeof(double)); } while (0)
#define CP3(dst, src) do { c->dst = zalloc(n3); memcpy(c->dst, d->src, n3 * sizeof(double)); } while (0)
  CP2(e1t, e1t); CP2(e2t, e2t); CP2(e1u, e1u); CP2(e2u, e2u); CP2(e1v, e1v); CP2(e2v, e2v);
  CP2(e1f, e1f); CP2(e2f, e2f); CP2(ff_f, ff_f); CP2(ff_t, ff_t);
  CP3(e3t_0, e3t_0); CP3(e3u_0, e3u_0); CP3(e3v_0, e3v_0); CP3(e3w_0, e3w_0); CP3(e3f_0, e3f_0);
#undef CP2
#undef CP3
  /* domhgr.F90:133-151 */
  c->r1_e1t = zalloc(n2); c->r1_e2t = zalloc(n2); c->r1_e1u = zalloc(n2); c->r1_e2u = zalloc(n2);
  c->r1_e1v = zalloc(n2); c->r1_e2v = zalloc(n2); c->e1e2t = zalloc(n2); c->r1_e1e2t = zalloc(n2);
  c->e1e2u = zalloc(n2); c->e1e2v = zalloc(n2); c->r1_e1e2u = zalloc(n2); c->r1_e1e2v = zalloc(n2);
  c->e2_e1u = zalloc(n2); c->e1_e2v = zalloc(n2);
  for (size_t p = 0; p < n2; ++p) {
    c->r1_e1t[p] = 1.0 / c->e1t[p]; c->r1_e2t[p] = 1.0 / c->e2t[p];
    c->r1_e1u[p] = 1.0 / c->e1u[p]; c->r1_e2u[p] = 1.0 / c->e2u[p];
    c->r1_e1v[p] = 1.0 / c->e1v[p]; c->r1_e2v[p] = 1.0 / c->e2v[p];
    c->e1e2t[p] = c->e1t[p] * c->e2t[p]; c->r1_e1e2t[p] = 1.0 / c->e1e2t[p];
    c->e1e2u[p] = c->e1u[p] * c->e2u[p]; c->e1e2v[p] = c->e1v[p] * c->e2v[p];
    c->r1_e1e2u[p] = 1.0 / c->e1e2u[p]; c->r1_e1e2v[p] = 1.0 / c->e1e2v[p];
    c->e2_e1u[p] = c->e2u[p] / c->e1u[p]; c->e1_e2v[p] = c->e1v[p] / c->e2v[p];
  }
  /* dommsk.F90:133-145 tmask from k_top/k_bot, then lbc_lnk 'T' */
  c->tmask = zalloc(n3); c->umask = zalloc(n3); c->vmask = zalloc(n3); c->wmask = zalloc(n3);
  for (int jj = 1; jj <= jpj; ++jj)
    for (int ji = 1; ji <= jpi; ++ji) {
      int kt = d->k_top[I2(ji, jj)], kb = d->k_bot[I2(ji, jj)];
      if (kt != 0)
        for (int jk = kt; jk <= kb; ++jk) c->tmask[I3(ji, jj, jk)] = 1.0;
    }
  lbc_closed(jpi, jpj, c->tmask, jpk, 'T', 0.0);
  /* dommsk.F90:172-183 umask/vmask (fmask not used on this path), lbc 'U'/'V' */
  for (int jk = 1; jk <= jpk; ++jk)
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        c->umask[I3(ji, jj, jk)] = c->tmask[I3(ji, jj, jk)] * c->tmask[I3(ji + 1, jj, jk)];
        c->vmask[I3(ji, jj, jk)] = c->tmask[I3(ji, jj, jk)] * c->tmask[I3(ji, jj + 1, jk)];
      }
  lbc_closed(jpi, jpj, c->umask, jpk, 'U', 0.0);
  lbc_closed(jpi, jpj, c->vmask, jpk, 'V', 0.0);
  /* dommsk.F90:189-194 */
  for (size_t p = 0; p < n2; ++p) c->wmask[p] = c->tmask[p];
  for (int jk = 2; jk <= jpk; ++jk)
    for (size_t p = 0; p < n2; ++p) c->wmask[p + n2 * (jk - 1)] = c->tmask[p + n2 * (jk - 1)] * c->tmask[p + n2 * (jk - 2)];
  c->nksr = ext_lev(c, d->e3t_0, c->nam.rn_si1 > 0 ? c->nam.rn_si1 : 23.0, 100.0);
  /* dommsk.F90:201-238 */
  c->ssmask = zalloc(n2); c->ssumask = zalloc(n2); c->ssvmask = zalloc(n2);
  c->tmask_h = zalloc(n2); c->tmask_i = zalloc(n2);
  for (size_t p = 0; p < n2; ++p) {
    double a = 0, b = 0, e = 0;
    for (int jk = 0; jk < jpk; ++jk) {
      a = dmax(a, c->tmask[p + n2 * jk]); b = dmax(b, c->umask[p + n2 * jk]); e = dmax(e, c->vmask[p + n2 * jk]);
    }
    c->ssmask[p] = a; c->ssumask[p] = b; c->ssvmask[p] = e;
  }
  for (int jj = 1; jj <= jpj; ++jj)
    for (int ji = 1; ji <= jpi; ++ji)
      c->tmask_h[I2(ji, jj)] = (ji == 1 || ji == jpi || jj == 1 || jj == jpj) ? 0.0 : 1.0;
  for (size_t p = 0; p < n2; ++p) c->tmask_i[p] = c->ssmask[p] * c->tmask_h[p];
  /* domzgr.F90:292-314 */
  c->mikt = (int *)calloc(n2, sizeof(int)); c->mbkt = (int *)calloc(n2, sizeof(int));
  c->mbku = (int *)calloc(n2, sizeof(int)); c->mbkv = (int *)calloc(n2, sizeof(int));
  for (size_t p = 0; p < n2; ++p) {
    c->mikt[p] = d->k_top[p] > 1 ? d->k_top[p] : 1;
    c->mbkt[p] = d->k_bot[p] > 1 ? d->k_bot[p] : 1;
  }
  for (int jj = 1; jj <= jpj - 1; ++jj)
    for (int ji = 1; ji <= jpi - 1; ++ji) {
      int a = c->mbkt[I2(ji + 1, jj)], b = c->mbkt[I2(ji, jj)], e = c->mbkt[I2(ji, jj + 1)];
      c->mbku[I2(ji, jj)] = a < b ? a : b;
      c->mbkv[I2(ji, jj)] = e < b ? e : b;
    }
  for (int jj = 1; jj <= jpj; ++jj)
    for (int ji = 1; ji <= jpi; ++ji)
      if (ji == 1 || ji == jpi || jj == 1 || jj == jpj) { c->mbku[I2(ji, jj)] = 1; c->mbkv[I2(ji, jj)] = 1; }
      else {
        if (c->mbku[I2(ji, jj)] < 1) c->mbku[I2(ji, jj)] = 1;
        if (c->mbkv[I2(ji, jj)] < 1) c->mbkv[I2(ji, jj)] = 1;
      }
  /* domain.F90:149-183 */
  c->ht_0 = zalloc(n2); c->hu_0 = zalloc(n2); c->hv_0 = zalloc(n2);
  c->r1_hu_0 = zalloc(n2); c->r1_hv_0 = zalloc(n2);
  for (int jk = 0; jk < jpk; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      c->ht_0[p] = c->ht_0[p] + c->e3t_0[p + n2 * jk] * c->tmask[p + n2 * jk];
      c->hu_0[p] = c->hu_0[p] + c->e3u_0[p + n2 * jk] * c->umask[p + n2 * jk];
      c->hv_0[p] = c->hv_0[p] + c->e3v_0[p + n2 * jk] * c->vmask[p + n2 * jk];
    }
  for (size_t p = 0; p < n2; ++p) {
    c->r1_hu_0[p] = c->ssumask[p] / (c->hu_0[p] + 1.0 - c->ssumask[p]);
    c->r1_hv_0[p] = c->ssvmask[p] / (c->hv_0[p] + 1.0 - c->ssvmask[p]);
  }
  /* ldftra.F90:292-372 constant masked diffusivity */
  c->ahtu_c = zalloc(n3); c->ahtv_c = zalloc(n3);
  {
    double a0 = nam->ln_traldf_blp ? sqrt(nam->rn_aht_0) : nam->rn_aht_0;
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (size_t p = 0; p < n2; ++p) {
        c->ahtu_c[p + n2 * (jk - 1)] = a0 * c->umask[p + n2 * (jk - 1)];
        c->ahtv_c[p + n2 * (jk - 1)] = a0 * c->vmask[p + n2 * (jk - 1)];
      }
  }
  /* dyn_spg_ts_init, dynspg_ts.F90:1479-1493 */
  {
    double zcmax = -1.0e300;
    for (size_t p = 0; p < n2; ++p) {
      double zxr2 = c->r1_e1t[p] * c->r1_e1t[p];
      double zyr2 = c->r1_e2t[p] * c->r1_e2t[p];
      double zcu = sqrt(nam->grav * dmax(c->ht_0[p], 0.0) * (zxr2 + zyr2));
      zcmax = dmax(zcmax, zcu);
    }
    c->nn_baro = nam->ln_bt_auto ? (int)ceil(nam->rn_rdt / nam->rn_bt_cmax * zcmax) : nam->nn_baro;
    if (c->nn_baro < 1) c->nn_baro = 1;
    c->rdtbt = nam->rn_rdt / (double)c->nn_baro;
  }
  c->wgtbtp1 = zalloc(3 * (size_t)c->nn_baro); c->wgtbtp2 = zalloc(3 * (size_t)c->nn_baro);
  c->zwz = zalloc(n2); c->ftne = zalloc(n2); c->ftnw = zalloc(n2); c->ftse = zalloc(n2); c->ftsw = zalloc(n2);
  c->sshn_e = zalloc(n2); c->sshb_e = zalloc(n2); c->sshbb_e = zalloc(n2);
  c->un_e = zalloc(n2); c->ub_e = zalloc(n2); c->ubb_e = zalloc(n2);
  c->vn_e = zalloc(n2); c->vb_e = zalloc(n2); c->vbb_e = zalloc(n2);
  c->ssha_e = zalloc(n2); c->ua_e = zalloc(n2); c->va_e = zalloc(n2);
  c->hu_e = zalloc(n2); c->hv_e = zalloc(n2); c->hur_e = zalloc(n2); c->hvr_e = zalloc(n2);
  {
    /* icycle for the steady leapfrog case; dyn_spg_ts recomputes it at nit000 */
    int jpit = 0;
    ts_wgt(c, nam->ln_bt_av, nam->ln_bt_fw, &jpit, c->wgtbtp1, c->wgtbtp2);
    c->icycle = jpit;
  }
  c->r2dt = 2.0 * nam->rn_rdt;
  spg_coriolis_factors(c, c->ht_0, c->e3f_0);
  *out = c;
  return NEMO_OK;
}

int ora_destroy(ora_ctx *c) {
  if (!c) return NEMO_OK;
  double **dp[] = {&c->e1t, &c->e2t, &c->e1u, &c->e2u, &c->e1v, &c->e2v, &c->e1f, &c->e2f, &c->ff_f, &c->ff_t,
                   &c->r1_e1t, &c->r1_e2t, &c->r1_e1u, &c->r1_e2u, &c->r1_e1v, &c->r1_e2v, &c->e1e2t,
                   &c->r1_e1e2t, &c->e1e2u, &c->e1e2v, &c->r1_e1e2u, &c->r1_e1e2v, &c->e2_e1u, &c->e1_e2v,
                   &c->tmask, &c->umask, &c->vmask, &c->wmask, &c->ssmask, &c->ssumask, &c->ssvmask,
                   &c->tmask_h, &c->tmask_i, &c->e3t_0, &c->e3u_0, &c->e3v_0, &c->e3w_0, &c->e3f_0,
                   &c->ht_0, &c->hu_0, &c->hv_0, &c->r1_hu_0, &c->r1_hv_0, &c->ahtu_c, &c->ahtv_c,
                   &c->wgtbtp1, &c->wgtbtp2, &c->zwz, &c->ftne, &c->ftnw, &c->ftse, &c->ftsw,
                   &c->sshn_e, &c->sshb_e, &c->sshbb_e, &c->un_e, &c->ub_e, &c->ubb_e, &c->vn_e, &c->vb_e,
                   &c->vbb_e, &c->ssha_e, &c->ua_e, &c->va_e, &c->hu_e, &c->hv_e, &c->hur_e, &c->hvr_e,
                   &c->surf, &c->surf_ini, &c->ssh_ini, &c->ssh_hc_loc_ini, &c->ssh_sc_loc_ini, &c->e3t_ini,
                   &c->hc_loc_ini, &c->sc_loc_ini};
  for (size_t i = 0; i < sizeof(dp) / sizeof(dp[0]); ++i) wfree(*dp[i]);
  free(c->mikt); free(c->mbkt); free(c->mbku); free(c->mbkv);
  free(c);
  return NEMO_OK;
}

int ora_bind(ora_ctx *c, int id, double *p) {
  if (!c || id < 0 || id >= NEMO_F_COUNT) return NEMO_ERR_ARG;
  c->f[id] = p;
  return NEMO_OK;
}

int ora_spg_info(const ora_ctx *c, int *icycle, int *nn_baro, double *rdtbt) {
  if (!c) return NEMO_ERR_ARG;
  if (icycle) *icycle = c->icycle;
  if (nn_baro) *nn_baro = c->nn_baro;
  if (rdtbt) *rdtbt = c->rdtbt;
  return NEMO_OK;
}

const double *ora_array(const ora_ctx *c, const char *name) {
#define R(n) if (!strcmp(name, #n)) return c->n
  R(tmask); R(umask); R(vmask); R(wmask); R(ssmask); R(ssumask); R(ssvmask); R(tmask_i); R(tmask_h);
  R(ht_0); R(hu_0); R(hv_0); R(r1_hu_0); R(r1_hv_0); R(e1e2t); R(r1_e1e2t); R(wgtbtp1); R(wgtbtp2);
  R(zwz); R(e2_e1u); R(e1_e2v); R(r1_e1u); R(r1_e2v);
#undef R
  return NULL;
}

const int *ora_iarray(const ora_ctx *c, const char *name) {
  if (!strcmp(name, "mikt")) return c->mikt;
  if (!strcmp(name, "mbkt")) return c->mbkt;
  if (!strcmp(name, "mbku")) return c->mbku;
  if (!strcmp(name, "mbkv")) return c->mbkv;
  return NULL;
}

/* Field accessors with the rest-state default of the e3 fields and depths (ln_linssh). */
static const double *fld(const ora_ctx *c, int id) {
  if (c->f[id]) return c->f[id];
  switch (id) {
    case NEMO_F_E3T_B: case NEMO_F_E3T_N: case NEMO_F_E3T_A: return c->e3t_0;
    case NEMO_F_E3U_N: return c->e3u_0;
    case NEMO_F_E3V_N: return c->e3v_0;
    case NEMO_F_E3W_N: return c->e3w_0;
    case NEMO_F_E3F_N: return c->e3f_0;
    case NEMO_F_HT_N: return c->ht_0;
    case NEMO_F_HU_N: case NEMO_F_HU_B: return c->hu_0;
    case NEMO_F_HV_N: case NEMO_F_HV_B: return c->hv_0;
    case NEMO_F_R1_HU_N: case NEMO_F_R1_HU_B: return c->r1_hu_0;
    case NEMO_F_R1_HV_N: case NEMO_F_R1_HV_B: return c->r1_hv_0;
    default: return NULL;
  }
}

/* ----------------------------------------------------------- tra_adv transports */
/* traadv.F90:99-124 (no Stokes drift, no vvl z-tilde, no eiv/mle) */
int ora_tra_adv_trp(ora_ctx *c, const double *un, const double *vn, const double *wn,
                    double *zun, double *zvn, double *zwn) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N);
  for (size_t p = 0; p < n2; ++p) { zun[p + n2 * (jpk - 1)] = 0; zvn[p + n2 * (jpk - 1)] = 0; zwn[p + n2 * (jpk - 1)] = 0; }
  OMP_FOR
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      size_t q = p + n2 * (jk - 1);
      zun[q] = c->e2u[p] * e3u[q] * un[q];
      zvn[q] = c->e1v[p] * e3v[q] * vn[q];
      zwn[q] = c->e1e2t[p] * wn[q];
    }
  return NEMO_OK;
}

/* ------------------------------------------------------------ interp_4th_cpt */
/* traadv_fct.F90:517-616 (ln_isfcav = F). pt_out is defined on the interior
 * columns, levels 2..jpkm1, exactly where the reference defines it. */
int ora_interp_4th_cpt(ora_ctx *c, const double *pt_in, double *pt_out) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n3 = (size_t)jpi * jpj * jpk;
  double *zwd = walloc(n3), *zwi = walloc(n3), *zws = walloc(n3), *zwrm = walloc(n3), *zwt = walloc(n3);
  const double *wmask = c->wmask;
  for (int jk = 3; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        zwd[q] = 3.0 * wmask[q] + 1.0;
        zwi[q] = wmask[q];
        zws[q] = wmask[q];
        zwrm[q] = 3.0 * wmask[q] * (pt_in[q] + pt_in[I3(ji, jj, jk - 1)]);
      }
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      int ikt = c->mikt[I2(ji, jj)] + 1;
      int ikb = c->mbkt[I2(ji, jj)];
      size_t q = I3(ji, jj, ikt);
      zwd[q] = 1.0; zwi[q] = 0.0; zws[q] = 0.0;
      zwrm[q] = 0.5 * (pt_in[I3(ji, jj, ikt - 1)] + pt_in[I3(ji, jj, ikt)]);
      q = I3(ji, jj, ikb);
      zwd[q] = 1.0; zwi[q] = 0.0; zws[q] = 0.0;
      /* over land ikb = 1 and the reference reads pt_in(:,:,0) into an unused
       * zwrm(:,:,1); 0 stands in for that value here */
      zwrm[q] = ikb >= 2 ? 0.5 * (pt_in[I3(ji, jj, ikb - 1)] + pt_in[I3(ji, jj, ikb)]) : 0.0;
    }
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) zwt[I3(ji, jj, 2)] = zwd[I3(ji, jj, 2)];
  for (int jk = 3; jk <= jpk - 1; ++jk)
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji)
        zwt[I3(ji, jj, jk)] = zwd[I3(ji, jj, jk)] - zwi[I3(ji, jj, jk)] * zws[I3(ji, jj, jk - 1)] / zwt[I3(ji, jj, jk - 1)];
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) pt_out[I3(ji, jj, 2)] = zwrm[I3(ji, jj, 2)];
  for (int jk = 3; jk <= jpk - 1; ++jk)
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji)
        pt_out[I3(ji, jj, jk)] = zwrm[I3(ji, jj, jk)] - zwi[I3(ji, jj, jk)] / zwt[I3(ji, jj, jk - 1)] * pt_out[I3(ji, jj, jk - 1)];
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji)
      pt_out[I3(ji, jj, jpk - 1)] = pt_out[I3(ji, jj, jpk - 1)] / zwt[I3(ji, jj, jpk - 1)];
  for (int jk = jpk - 2; jk >= 2; --jk)
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji)
        pt_out[I3(ji, jj, jk)] = (pt_out[I3(ji, jj, jk)] - zws[I3(ji, jj, jk)] * pt_out[I3(ji, jj, jk + 1)]) / zwt[I3(ji, jj, jk)];
  wfree(zwd); wfree(zwi); wfree(zws); wfree(zwrm); wfree(zwt);
  return NEMO_OK;
}

/* The adjoint of ora_interp_4th_cpt with respect to pt_in: pv holds the adjoint of
 * pt_out on the interior columns, levels 2..jpkm1; pt_ad accumulates R^T M^-T pv, M
 * the tridiagonal matrix and R the right-hand-side operator the forward builds (the
 * same rows, pivots zwt and special top and bottom rows), the back substitution
 * undone forwards and the elimination backwards. */
int ora_interp_4th_cpt_adj(ora_ctx *c, const double *pv, double *pt_ad) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const double *wmask = c->wmask;
  double *d = malloc(sizeof(double) * jpk), *wi = malloc(sizeof(double) * jpk), *ws = malloc(sizeof(double) * jpk);
  double *w = malloc(sizeof(double) * jpk), *zwt = malloc(sizeof(double) * jpk), *xa = malloc(sizeof(double) * jpk);
  double *za = malloc(sizeof(double) * jpk);
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      const size_t p = I2(ji, jj);
      const int ikt = c->mikt[p] + 1, ikb = c->mbkt[p];
      for (int jk = 2; jk <= jpk - 1; ++jk) {  /* the forward's rows (:535-565) */
        const double wm = wmask[I3(ji, jj, jk)];
        if (jk == ikt || jk == ikb) { d[jk] = 1.0; wi[jk] = 0.0; ws[jk] = 0.0; w[jk] = 0.5; }
        else if (jk >= 3) { d[jk] = 3.0 * wm + 1.0; wi[jk] = wm; ws[jk] = wm; w[jk] = 3.0 * wm; }
        else { d[jk] = 0.0; wi[jk] = 0.0; ws[jk] = 0.0; w[jk] = 0.0; }
      }
      zwt[2] = d[2];
      for (int jk = 3; jk <= jpk - 1; ++jk) zwt[jk] = d[jk] - wi[jk] * ws[jk - 1] / zwt[jk - 1];
      for (int jk = 2; jk <= jpk - 1; ++jk) xa[jk] = pv[I3(ji, jj, jk)];
      for (int jk = 2; jk <= jpk - 2; ++jk) {  /* back substitution, undone (:596-607) */
        za[jk] = xa[jk] / zwt[jk];
        xa[jk + 1] = xa[jk + 1] - ws[jk] * za[jk];
      }
      za[jpk - 1] = xa[jpk - 1] / zwt[jpk - 1];
      for (int jk = jpk - 1; jk >= 3; --jk)  /* elimination, undone (:584-593) */
        za[jk - 1] = za[jk - 1] - wi[jk] / zwt[jk - 1] * za[jk];
      for (int jk = 2; jk <= jpk - 1; ++jk) {  /* the right-hand side, transposed */
        pt_ad[I3(ji, jj, jk)] += w[jk] * za[jk];
        pt_ad[I3(ji, jj, jk - 1)] += w[jk] * za[jk];
      }
    }
  free(d); free(wi); free(ws); free(w); free(zwt); free(xa); free(za);
  return NEMO_OK;
}

/* -------------------------------------------------------------------- nonosc */
/* traadv_fct.F90:330-428 */
static void nonosc(ora_ctx *c, const double *pbef, double *paa, double *pbb, double *pcc,
                   const double *paft, double p2dt, double *tape) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n3 = (size_t)jpi * jpj * jpk;
  const double *tmask = c->tmask, *e3t_n = fld(c, NEMO_F_E3T_N);
  const double zbig = 1.e+40, zrtrn = 1.e-15;
  double *zbetup = zalloc(n3), *zbetdo = zalloc(n3), *zbup = walloc(n3), *zbdo = walloc(n3);
  for (size_t q = 0; q < n3; ++q) {
    zbup[q] = dmax(pbef[q] * tmask[q] - zbig * (1.0 - tmask[q]), paft[q] * tmask[q] - zbig * (1.0 - tmask[q]));
    zbdo[q] = dmin(pbef[q] * tmask[q] + zbig * (1.0 - tmask[q]), paft[q] * tmask[q] + zbig * (1.0 - tmask[q]));
  }
  OMP_FOR
  for (int jk = 1; jk <= jpk - 1; ++jk) {
    int ikm1 = jk - 1 > 1 ? jk - 1 : 1;
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        double zup = zbup[I3(ji, jj, jk)];
        zup = dmax(zup, zbup[I3(ji - 1, jj, jk)]); zup = dmax(zup, zbup[I3(ji + 1, jj, jk)]);
        zup = dmax(zup, zbup[I3(ji, jj - 1, jk)]); zup = dmax(zup, zbup[I3(ji, jj + 1, jk)]);
        zup = dmax(zup, zbup[I3(ji, jj, ikm1)]); zup = dmax(zup, zbup[I3(ji, jj, jk + 1)]);
        double zdo = zbdo[I3(ji, jj, jk)];
        zdo = dmin(zdo, zbdo[I3(ji - 1, jj, jk)]); zdo = dmin(zdo, zbdo[I3(ji + 1, jj, jk)]);
        zdo = dmin(zdo, zbdo[I3(ji, jj - 1, jk)]); zdo = dmin(zdo, zbdo[I3(ji, jj + 1, jk)]);
        zdo = dmin(zdo, zbdo[I3(ji, jj, ikm1)]); zdo = dmin(zdo, zbdo[I3(ji, jj, jk + 1)]);
        double zpos = dmax(0., paa[I3(ji - 1, jj, jk)]) - dmin(0., paa[I3(ji, jj, jk)])
                    + dmax(0., pbb[I3(ji, jj - 1, jk)]) - dmin(0., pbb[I3(ji, jj, jk)])
                    + dmax(0., pcc[I3(ji, jj, jk + 1)]) - dmin(0., pcc[I3(ji, jj, jk)]);
        double zneg = dmax(0., paa[I3(ji, jj, jk)]) - dmin(0., paa[I3(ji - 1, jj, jk)])
                    + dmax(0., pbb[I3(ji, jj, jk)]) - dmin(0., pbb[I3(ji, jj - 1, jk)])
                    + dmax(0., pcc[I3(ji, jj, jk)]) - dmin(0., pcc[I3(ji, jj, jk + 1)]);
        double zbt = c->e1e2t[I2(ji, jj)] * e3t_n[I3(ji, jj, jk)] / p2dt;
        zbetup[I3(ji, jj, jk)] = (zup - paft[I3(ji, jj, jk)]) / (zpos + zrtrn) * zbt;
        zbetdo[I3(ji, jj, jk)] = (paft[I3(ji, jj, jk)] - zdo) / (zneg + zrtrn) * zbt;
      }
  }
  lbc_closed(jpi, jpj, zbetup, jpk, 'T', 0.0);
  lbc_closed(jpi, jpj, zbetdo, jpk, 'T', 0.0);
  if (tape) memset(tape, 0, 3 * n3 * sizeof(double));
  OMP_FOR
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        double zau = dmin(1.0, dmin(zbetdo[I3(ji, jj, jk)], zbetup[I3(ji + 1, jj, jk)]));
        double zbu = dmin(1.0, dmin(zbetup[I3(ji, jj, jk)], zbetdo[I3(ji + 1, jj, jk)]));
        double zcu = (0.5 + sign_nsz(0.5, paa[I3(ji, jj, jk)]));
        paa[I3(ji, jj, jk)] = paa[I3(ji, jj, jk)] * (zcu * zau + (1.0 - zcu) * zbu);
        if (tape) tape[I3(ji, jj, jk)] = zcu * zau + (1.0 - zcu) * zbu;
        double zav = dmin(1.0, dmin(zbetdo[I3(ji, jj, jk)], zbetup[I3(ji, jj + 1, jk)]));
        double zbv = dmin(1.0, dmin(zbetup[I3(ji, jj, jk)], zbetdo[I3(ji, jj + 1, jk)]));
        double zcv = (0.5 + sign_nsz(0.5, pbb[I3(ji, jj, jk)]));
        pbb[I3(ji, jj, jk)] = pbb[I3(ji, jj, jk)] * (zcv * zav + (1.0 - zcv) * zbv);
        if (tape) tape[n3 + I3(ji, jj, jk)] = zcv * zav + (1.0 - zcv) * zbv;
        double za = dmin(1., dmin(zbetdo[I3(ji, jj, jk + 1)], zbetup[I3(ji, jj, jk)]));
        double zb = dmin(1., dmin(zbetup[I3(ji, jj, jk + 1)], zbetdo[I3(ji, jj, jk)]));
        double zc = (0.5 + sign_nsz(0.5, pcc[I3(ji, jj, jk + 1)]));
        pcc[I3(ji, jj, jk + 1)] = pcc[I3(ji, jj, jk + 1)] * (zc * za + (1.0 - zc) * zb);
        if (tape) tape[2 * n3 + I3(ji, jj, jk + 1)] = zc * za + (1.0 - zc) * zb;
      }
  lbc_closed(jpi, jpj, paa, jpk, 'U', 0.0);
  lbc_closed(jpi, jpj, pbb, jpk, 'V', 0.0);
  wfree(zbetup); wfree(zbetdo); wfree(zbup); wfree(zbdo);
}

/* --------------------------------------------------------------- tra_adv_fct */
/* traadv_fct.F90:54-327 (no trend / ptr / hst diagnostics, ln_isfcav = F) */
int ora_tra_adv_fct(ora_ctx *c, int kt, int kit000, const char *cdtype, double p2dt,
                    const double *pun, const double *pvn, const double *pwn,
                    const double *ptb, const double *ptn, double *pta,
                    int kjpt, int kn_fct_h, int kn_fct_v) {
  (void)kt; (void)kit000; (void)cdtype;
  if ((kn_fct_h != 2 && kn_fct_h != 4) || (kn_fct_v != 2 && kn_fct_v != 4) || kjpt < 1) return NEMO_ERR_ARG;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const double *tmask = c->tmask, *umask = c->umask, *vmask = c->vmask, *wmask = c->wmask;
  const double *e3t_b = fld(c, NEMO_F_E3T_B), *e3t_n = fld(c, NEMO_F_E3T_N), *e3t_a = fld(c, NEMO_F_E3T_A);
  const double r1_6 = 1.0 / 6.0;
  double *zwi = zalloc(n3), *zwx = walloc(n3), *zwy = walloc(n3), *zwz = walloc(n3);
  double *ztu = walloc(n3), *ztv = walloc(n3), *zltu = walloc(n3), *zltv = walloc(n3), *ztw = walloc(n3);
  for (size_t p = 0; p < n2; ++p) {
    zwz[p] = 0.0;
    zwx[p + n2 * (jpk - 1)] = 0.0; zwy[p + n2 * (jpk - 1)] = 0.0; zwz[p + n2 * (jpk - 1)] = 0.0;
  }
  memset(zwi, 0, n3 * sizeof(double));
  for (int jn = 1; jn <= kjpt; ++jn) {
    const double *tb = ptb + n3 * (jn - 1), *tn = ptn + n3 * (jn - 1);
    double *ta = pta + n3 * (jn - 1);
    /* upstream fluxes (:123-135) */
    OMP_FOR
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double zfp_ui = pun[q] + fabs(pun[q]);
          double zfm_ui = pun[q] - fabs(pun[q]);
          double zfp_vj = pvn[q] + fabs(pvn[q]);
          double zfm_vj = pvn[q] - fabs(pvn[q]);
          zwx[q] = 0.5 * (zfp_ui * tb[q] + zfm_ui * tb[I3(ji + 1, jj, jk)]);
          zwy[q] = 0.5 * (zfp_vj * tb[q] + zfm_vj * tb[I3(ji, jj + 1, jk)]);
        }
    /* (:137-145) */
    OMP_FOR
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj; ++jj)
        for (int ji = 1; ji <= jpi; ++ji) {
          size_t q = I3(ji, jj, jk);
          double zfp_wk = pwn[q] + fabs(pwn[q]);
          double zfm_wk = pwn[q] - fabs(pwn[q]);
          zwz[q] = 0.5 * (zfp_wk * tb[q] + zfm_wk * tb[I3(ji, jj, jk - 1)]) * wmask[q];
        }
    /* (:146-156) linear free surface, no cavities */
    if (c->nam.ln_linssh)
      for (size_t p = 0; p < n2; ++p) zwz[p] = pwn[p] * tb[p];
    /* (:158-170) */
    OMP_FOR
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double ztra = -(zwx[q] - zwx[I3(ji - 1, jj, jk)] + zwy[q] - zwy[I3(ji, jj - 1, jk)]
                          + zwz[q] - zwz[I3(ji, jj, jk + 1)]) * c->r1_e1e2t[I2(ji, jj)];
          ta[q] = ta[q] + ztra / e3t_n[q] * tmask[q];
          zwi[q] = (e3t_b[q] * tb[q] + p2dt * ztra) / e3t_a[q] * tmask[q];
        }
    /* horizontal antidiffusive fluxes (:180-251) */
    if (kn_fct_h == 2) {
      OMP_FOR
      for (int jk = 1; jk <= jpk - 1; ++jk)
        for (int jj = 1; jj <= jpj - 1; ++jj)
          for (int ji = 1; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            zwx[q] = 0.5 * pun[q] * (tn[q] + tn[I3(ji + 1, jj, jk)]) - zwx[q];
            zwy[q] = 0.5 * pvn[q] * (tn[q] + tn[I3(ji, jj + 1, jk)]) - zwy[q];
          }
    } else {
      for (size_t p = 0; p < n2; ++p) { zltu[p + n2 * (jpk - 1)] = 0.0; zltv[p + n2 * (jpk - 1)] = 0.0; }
      OMP_FOR
      for (int jk = 1; jk <= jpk - 1; ++jk) {
        for (int jj = 1; jj <= jpj - 1; ++jj)
          for (int ji = 1; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            ztu[q] = (tn[I3(ji + 1, jj, jk)] - tn[q]) * umask[q];
            ztv[q] = (tn[I3(ji, jj + 1, jk)] - tn[q]) * vmask[q];
          }
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            zltu[q] = (ztu[q] + ztu[I3(ji - 1, jj, jk)]) * r1_6;
            zltv[q] = (ztv[q] + ztv[I3(ji, jj - 1, jk)]) * r1_6;
          }
      }
      lbc_closed(jpi, jpj, zltu, jpk, 'T', 0.0);
      lbc_closed(jpi, jpj, zltv, jpk, 'T', 0.0);
      OMP_FOR
      for (int jk = 1; jk <= jpk - 1; ++jk)
        for (int jj = 1; jj <= jpj - 1; ++jj)
          for (int ji = 1; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            double zC2t_u = tn[q] + tn[I3(ji + 1, jj, jk)];
            double zC2t_v = tn[q] + tn[I3(ji, jj + 1, jk)];
            zwx[q] = 0.5 * pun[q] * (zC2t_u + zltu[q] - zltu[I3(ji + 1, jj, jk)]) - zwx[q];
            zwy[q] = 0.5 * pvn[q] * (zC2t_v + zltv[q] - zltv[I3(ji, jj + 1, jk)]) - zwy[q];
          }
    }
    /* vertical antidiffusive fluxes (:253-275) */
    if (kn_fct_v == 2) {
      OMP_FOR
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            zwz[q] = (pwn[q] * 0.5 * (tn[q] + tn[I3(ji, jj, jk - 1)]) - zwz[q]) * wmask[q];
          }
    } else {
      ora_interp_4th_cpt(c, tn, ztw);
      OMP_FOR
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            zwz[q] = (pwn[q] * ztw[q] - zwz[q]) * wmask[q];
          }
    }
    if (c->nam.ln_linssh)
      for (size_t p = 0; p < n2; ++p) zwz[p] = 0.0;
    /* (:280) */
    lbc_closed(jpi, jpj, zwi, jpk, 'T', 0.0);
    lbc_closed(jpi, jpj, zwx, jpk, 'U', 0.0);
    lbc_closed(jpi, jpj, zwy, jpk, 'V', 0.0);
    lbc_closed(jpi, jpj, zwz, jpk, 'W', 0.0);
    /* (:284) the limiter; with a tape in replay mode the recorded multipliers
     * instead (the tangent-linear with the limiter frozen) */
    double *tp = c->fct_tape ? c->fct_tape + 3 * n3 * (size_t)(jn - 1) : NULL;
    if (c->fct_tape_mode == 2) {
      for (size_t q = 0; q < n3; ++q) {
        zwx[q] = zwx[q] * tp[q];
        zwy[q] = zwy[q] * tp[n3 + q];
        zwz[q] = zwz[q] * tp[2 * n3 + q];
      }
    } else {
      nonosc(c, tb, zwx, zwy, zwz, zwi, p2dt, c->fct_tape_mode == 1 ? tp : NULL);
    }
    /* (:288-297) */
    OMP_FOR
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          ta[q] = ta[q] - (zwx[q] - zwx[I3(ji - 1, jj, jk)] + zwy[q] - zwy[I3(ji, jj - 1, jk)]
                           + zwz[q] - zwz[I3(ji, jj, jk + 1)]) * c->r1_e1e2t[I2(ji, jj)] / e3t_n[q];
        }
  }
  wfree(zwi); wfree(zwx); wfree(zwy); wfree(zwz); wfree(ztu); wfree(ztv); wfree(zltu); wfree(zltv); wfree(ztw);
  return NEMO_OK;
}

/* --------------------------------------------------------------- tra_ldf_lap */
/* traldf_lap_blp.F90:47-158 (ln_isfcav = F; no ptr/hst diagnostics) */
int ora_tra_ldf_lap(ora_ctx *c, int kt, int kit000, const char *cdtype,
                    const double *pahu, const double *pahv,
                    const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                    const double *ptb, double *pta, int kjpt, int kpass) {
  (void)kt; (void)kit000; (void)cdtype; (void)pgui; (void)pgvi;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  if (!pahu) pahu = c->ahtu_c;
  if (!pahv) pahv = c->ahtv_c;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N), *e3t_n = fld(c, NEMO_F_E3T_N);
  double zsign = kpass == 1 ? 1.0 : -1.0;
  double *ztu = walloc(n3), *ztv = walloc(n3), *zaheeu = walloc(n3), *zaheev = walloc(n3);
  OMP_FOR
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        zaheeu[q] = zsign * pahu[q] * c->e2_e1u[I2(ji, jj)] * e3u[q];
        zaheev[q] = zsign * pahv[q] * c->e1_e2v[I2(ji, jj)] * e3v[q];
      }
  for (int jn = 1; jn <= kjpt; ++jn) {
    const double *tb = ptb + n3 * (jn - 1);
    double *ta = pta + n3 * (jn - 1);
    OMP_FOR
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          ztu[q] = zaheeu[q] * (tb[I3(ji + 1, jj, jk)] - tb[q]);
          ztv[q] = zaheev[q] * (tb[I3(ji, jj + 1, jk)] - tb[q]);
        }
    if (c->nam.ln_zps)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          int ku = c->mbku[I2(ji, jj)], kv = c->mbkv[I2(ji, jj)];
          ztu[I3(ji, jj, ku)] = zaheeu[I3(ji, jj, ku)] * pgu[I2(ji, jj) + n2 * (jn - 1)];
          ztv[I3(ji, jj, kv)] = zaheev[I3(ji, jj, kv)] * pgv[I2(ji, jj) + n2 * (jn - 1)];
        }
    OMP_FOR
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          ta[q] = ta[q] + (ztu[q] - ztu[I3(ji - 1, jj, jk)] + ztv[q] - ztv[I3(ji, jj - 1, jk)])
                              / (c->e1e2t[I2(ji, jj)] * e3t_n[q]);
        }
  }
  wfree(ztu); wfree(ztv); wfree(zaheeu); wfree(zaheev);
  return NEMO_OK;
}

/* --------------------------------------------------------------- tra_ldf_iso */
/* traldf_iso.F90:50-382 (ln_isfcav = F; no ptr/hst diagnostics) */
int ora_tra_ldf_iso(ora_ctx *c, int kt, int kit000, const char *cdtype,
                    const double *pahu, const double *pahv,
                    const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                    const double *ptb, const double *ptbb, double *pta, int kjpt, int kpass) {
  (void)cdtype; (void)pgui; (void)pgvi;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const nemo_namelist *nm = &c->nam;
  double *ah_wslp2 = c->f[NEMO_F_AH_WSLP2], *akz = c->f[NEMO_F_AKZ];
  const double *uslp = c->f[NEMO_F_USLP], *vslp = c->f[NEMO_F_VSLP];
  const double *wslpi = c->f[NEMO_F_WSLPI], *wslpj = c->f[NEMO_F_WSLPJ];
  if (!ah_wslp2 || !akz || !uslp || !vslp || !wslpi || !wslpj) return NEMO_ERR_UNBOUND;
  if (!pahu) pahu = c->ahtu_c;
  if (!pahv) pahv = c->ahtv_c;
  const double *tmask = c->tmask, *umask = c->umask, *vmask = c->vmask, *wmask = c->wmask;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N), *e3t_n = fld(c, NEMO_F_E3T_N);
  const double *e3w = fld(c, NEMO_F_E3W_N);
  (void)tmask;
  if (kpass == 1 && kt == kit000) {
    memset(akz, 0, n3 * sizeof(double));
    memset(ah_wslp2, 0, n3 * sizeof(double));
  }
  double z2dt = (nm->neuler == 0 && kt == nm->nit000) ? nm->rn_rdt : 2. * nm->rn_rdt;
  double z1_2dt = 1.0 / z2dt;
  double zsign = kpass == 1 ? 1.0 : -1.0;
  if (kpass == 1) {
    OMP_FOR
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double zmsku = wmask[q] / dmax(umask[I3(ji, jj, jk - 1)] + umask[I3(ji - 1, jj, jk)]
                                         + umask[I3(ji - 1, jj, jk - 1)] + umask[q], 1.0);
          double zmskv = wmask[q] / dmax(vmask[I3(ji, jj, jk - 1)] + vmask[I3(ji, jj - 1, jk)]
                                         + vmask[I3(ji, jj - 1, jk - 1)] + vmask[q], 1.0);
          double zahu_w = (pahu[I3(ji, jj, jk - 1)] + pahu[I3(ji - 1, jj, jk)]
                           + pahu[I3(ji - 1, jj, jk - 1)] + pahu[q]) * zmsku;
          double zahv_w = (pahv[I3(ji, jj, jk - 1)] + pahv[I3(ji, jj - 1, jk)]
                           + pahv[I3(ji, jj - 1, jk - 1)] + pahv[q]) * zmskv;
          ah_wslp2[q] = zahu_w * wslpi[q] * wslpi[q] + zahv_w * wslpj[q] * wslpj[q];
        }
    if (nm->ln_traldf_msc) {
      OMP_FOR
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            double e1u0 = c->e1u[I2(ji, jj)], e1um = c->e1u[I2(ji - 1, jj)];
            double e2v0 = c->e2v[I2(ji, jj)], e2vm = c->e2v[I2(ji, jj - 1)];
            akz[q] = 0.25 * ((pahu[q] + pahu[I3(ji, jj, jk - 1)]) / (e1u0 * e1u0)
                             + (pahu[I3(ji - 1, jj, jk)] + pahu[I3(ji - 1, jj, jk - 1)]) / (e1um * e1um)
                             + (pahv[q] + pahv[I3(ji, jj, jk - 1)]) / (e2v0 * e2v0)
                             + (pahv[I3(ji, jj - 1, jk)] + pahv[I3(ji, jj - 1, jk - 1)]) / (e2vm * e2vm));
          }
      if (nm->ln_traldf_blp) {
        OMP_FOR
        for (int jk = 2; jk <= jpk - 1; ++jk)
          for (int jj = 1; jj <= jpj - 1; ++jj)
            for (int ji = 1; ji <= jpi - 1; ++ji) {
              size_t q = I3(ji, jj, jk);
              akz[q] = 16.0 * ah_wslp2[q] * (akz[q] + ah_wslp2[q] / (e3w[q] * e3w[q]));
            }
      } else if (nm->ln_traldf_lap) {
        OMP_FOR
        for (int jk = 2; jk <= jpk - 1; ++jk)
          for (int jj = 1; jj <= jpj - 1; ++jj)
            for (int ji = 1; ji <= jpi - 1; ++ji) {
              size_t q = I3(ji, jj, jk);
              double ze3w_2 = e3w[q] * e3w[q];
              double zcoef0 = z2dt * (akz[q] + ah_wslp2[q] / ze3w_2);
              akz[q] = dmax(zcoef0 - 0.5, 0.0) * ze3w_2 * z1_2dt;
            }
      }
    } else {
      memcpy(akz, ah_wslp2, n3 * sizeof(double));
    }
  }
  double *zdit = walloc(n3), *zdjt = walloc(n3), *zftu = walloc(n3), *zftv = walloc(n3), *ztfw = walloc(n3);
  double *zdkt = walloc(n2), *zdk1t = walloc(n2);
  for (int jn = 1; jn <= kjpt; ++jn) {
    const double *tb = ptb + n3 * (jn - 1), *tbb = ptbb + n3 * (jn - 1);
    double *ta = pta + n3 * (jn - 1);
    for (int jk = 1; jk <= jpk; ++jk)
      for (int jj = 1; jj <= jpj; ++jj) {
        zdit[I3(1, jj, jk)] = 0.0; zdit[I3(jpi, jj, jk)] = 0.0;
        zdjt[I3(1, jj, jk)] = 0.0; zdjt[I3(jpi, jj, jk)] = 0.0;
      }
    OMP_FOR
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          zdit[q] = (tb[I3(ji + 1, jj, jk)] - tb[q]) * umask[q];
          zdjt[q] = (tb[I3(ji, jj + 1, jk)] - tb[q]) * vmask[q];
        }
    if (nm->ln_zps)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          zdit[I3(ji, jj, c->mbku[I2(ji, jj)])] = pgu[I2(ji, jj) + n2 * (jn - 1)];
          zdjt[I3(ji, jj, c->mbkv[I2(ji, jj)])] = pgv[I2(ji, jj) + n2 * (jn - 1)];
        }
    for (int jk = 1; jk <= jpk - 1; ++jk) {
      for (size_t p = 0; p < n2; ++p)
        zdk1t[p] = (tb[p + n2 * (jk - 1)] - tb[p + n2 * jk]) * wmask[p + n2 * jk];
      if (jk == 1) memcpy(zdkt, zdk1t, n2 * sizeof(double));
      else
        for (size_t p = 0; p < n2; ++p)
          zdkt[p] = (tb[p + n2 * (jk - 2)] - tb[p + n2 * (jk - 1)]) * wmask[p + n2 * (jk - 1)];
      OMP_FOR
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double zabe1 = pahu[q] * c->e2_e1u[I2(ji, jj)] * e3u[q];
          double zabe2 = pahv[q] * c->e1_e2v[I2(ji, jj)] * e3v[q];
          double zmsku = 1. / dmax(wmask[I3(ji + 1, jj, jk)] + wmask[I3(ji, jj, jk + 1)]
                                   + wmask[I3(ji + 1, jj, jk + 1)] + wmask[q], 1.);
          double zmskv = 1. / dmax(wmask[I3(ji, jj + 1, jk)] + wmask[I3(ji, jj, jk + 1)]
                                   + wmask[I3(ji, jj + 1, jk + 1)] + wmask[q], 1.);
          double zcof1 = -pahu[q] * c->e2u[I2(ji, jj)] * uslp[q] * zmsku;
          double zcof2 = -pahv[q] * c->e1v[I2(ji, jj)] * vslp[q] * zmskv;
          zftu[q] = (zabe1 * zdit[q] + zcof1 * (zdkt[I2(ji + 1, jj)] + zdk1t[I2(ji, jj)]
                                                + zdk1t[I2(ji + 1, jj)] + zdkt[I2(ji, jj)])) * umask[q];
          zftv[q] = (zabe2 * zdjt[q] + zcof2 * (zdkt[I2(ji, jj + 1)] + zdk1t[I2(ji, jj)]
                                                + zdk1t[I2(ji, jj + 1)] + zdkt[I2(ji, jj)])) * vmask[q];
        }
      OMP_FOR
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          ta[q] = ta[q] + zsign * (zftu[q] - zftu[I3(ji - 1, jj, jk)] + zftv[q] - zftv[I3(ji, jj - 1, jk)])
                              * c->r1_e1e2t[I2(ji, jj)] / e3t_n[q];
        }
    }
    for (int jk = 1; jk <= jpk; ++jk)
      for (int jj = 1; jj <= jpj; ++jj) { ztfw[I3(1, jj, jk)] = 0.0; ztfw[I3(jpi, jj, jk)] = 0.0; }
    for (size_t p = 0; p < n2; ++p) { ztfw[p] = 0.0; ztfw[p + n2 * (jpk - 1)] = 0.0; }
    OMP_FOR
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double zmsku = wmask[q] / dmax(umask[I3(ji, jj, jk - 1)] + umask[I3(ji - 1, jj, jk)]
                                         + umask[I3(ji - 1, jj, jk - 1)] + umask[q], 1.0);
          double zmskv = wmask[q] / dmax(vmask[I3(ji, jj, jk - 1)] + vmask[I3(ji, jj - 1, jk)]
                                         + vmask[I3(ji, jj - 1, jk - 1)] + vmask[q], 1.0);
          double zahu_w = (pahu[I3(ji, jj, jk - 1)] + pahu[I3(ji - 1, jj, jk)]
                           + pahu[I3(ji - 1, jj, jk - 1)] + pahu[q]) * zmsku;
          double zahv_w = (pahv[I3(ji, jj, jk - 1)] + pahv[I3(ji, jj - 1, jk)]
                           + pahv[I3(ji, jj - 1, jk - 1)] + pahv[q]) * zmskv;
          double zcoef3 = -zahu_w * c->e2t[I2(ji, jj)] * zmsku * wslpi[q];
          double zcoef4 = -zahv_w * c->e1t[I2(ji, jj)] * zmskv * wslpj[q];
          ztfw[q] = zcoef3 * (zdit[I3(ji, jj, jk - 1)] + zdit[I3(ji - 1, jj, jk)]
                              + zdit[I3(ji - 1, jj, jk - 1)] + zdit[q])
                  + zcoef4 * (zdjt[I3(ji, jj, jk - 1)] + zdjt[I3(ji, jj - 1, jk)]
                              + zdjt[I3(ji, jj - 1, jk - 1)] + zdjt[q]);
        }
    if (nm->ln_traldf_lap) {
      OMP_FOR
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 1; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            ztfw[q] = ztfw[q] + c->e1e2t[I2(ji, jj)] / e3w[q] * wmask[q]
                                    * (ah_wslp2[q] - akz[q]) * (tb[I3(ji, jj, jk - 1)] - tb[q]);
          }
    } else if (kpass == 1) {
      OMP_FOR
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 1; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            ztfw[q] = ztfw[q] + ah_wslp2[q] * c->e1e2t[I2(ji, jj)] * (tb[I3(ji, jj, jk - 1)] - tb[q]) / e3w[q] * wmask[q];
          }
    } else {
      OMP_FOR
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 1; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            ztfw[q] = ztfw[q] + c->e1e2t[I2(ji, jj)] / e3w[q] * wmask[q]
                                    * (ah_wslp2[q] * (tb[I3(ji, jj, jk - 1)] - tb[q])
                                       + akz[q] * (tbb[I3(ji, jj, jk - 1)] - tbb[q]));
          }
    }
    OMP_FOR
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          ta[q] = ta[q] + zsign * (ztfw[q] - ztfw[I3(ji, jj, jk + 1)]) * c->r1_e1e2t[I2(ji, jj)] / e3t_n[q];
        }
  }
  wfree(zdit); wfree(zdjt); wfree(zftu); wfree(zftv); wfree(ztfw); wfree(zdkt); wfree(zdk1t);
  return NEMO_OK;
}

/* Matrix of the implicit vertical diffusion and its LU pivots (trazdf.F90:153-234,
 * ln_zad_Aimp = F): zwi, zws the sub- and super-diagonals, zwt the pivots. */
static void zdf_lu(ora_ctx *c, const double *coef, double p2dt, double *zwi, double *zwt, double *zwd,
                   double *zws) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const nemo_namelist *nm = &c->nam;
  const double *akz = c->f[NEMO_F_AKZ], *ah_wslp2 = c->f[NEMO_F_AH_WSLP2];
  const double *e3t_a = fld(c, NEMO_F_E3T_A), *e3w = fld(c, NEMO_F_E3W_N);
  const int l_ldfslp = nm->ln_traldf_iso || nm->ln_traldf_triad;   /* ldftra.F90:253-255 */
  for (int jk = 2; jk <= jpk; ++jk)
    for (int jj = 1; jj <= jpj; ++jj)
      for (int ji = 1; ji <= jpi; ++ji) zwt[I3(ji, jj, jk)] = coef[I3(ji, jj, jk)];
  for (int jj = 1; jj <= jpj; ++jj)
    for (int ji = 1; ji <= jpi; ++ji) zwt[I3(ji, jj, 1)] = 0.0;
  if (l_ldfslp) {
    const double *add = nm->ln_traldf_msc ? akz : ah_wslp2;
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) zwt[I3(ji, jj, jk)] = zwt[I3(ji, jj, jk)] + add[I3(ji, jj, jk)];
  }
  OMP_FOR
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        zwi[q] = -p2dt * zwt[q] / e3w[q];
        zws[q] = -p2dt * zwt[I3(ji, jj, jk + 1)] / e3w[I3(ji, jj, jk + 1)];
        zwd[q] = e3t_a[q] - zwi[q] - zws[q];
      }
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) zwt[I3(ji, jj, 1)] = zwd[I3(ji, jj, 1)];
  for (int jk = 2; jk <= jpk - 1; ++jk)
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji)
        zwt[I3(ji, jj, jk)] = zwd[I3(ji, jj, jk)] - zwi[I3(ji, jj, jk)] * zws[I3(ji, jj, jk - 1)] / zwt[I3(ji, jj, jk - 1)];
}

/* --------------------------------------------------------------- tra_zdf_imp */
/* trazdf.F90:109-268 (ln_zad_Aimp = F) */
int ora_tra_zdf_imp(ora_ctx *c, int kt, int kit000, const char *cdtype, double p2dt,
                    const double *ptb, double *pta, int kjpt) {
  (void)kt; (void)kit000;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n3 = (size_t)jpi * jpj * jpk;
  const nemo_namelist *nm = &c->nam;
  const int is_trc = cdtype && cdtype[0] == 'T' && cdtype[1] == 'R' && cdtype[2] == 'C';
  const double *avt = c->f[NEMO_F_AVT], *avs = c->f[NEMO_F_AVS];
  const double *akz = c->f[NEMO_F_AKZ], *ah_wslp2 = c->f[NEMO_F_AH_WSLP2];
  const double *e3t_b = fld(c, NEMO_F_E3T_B), *e3t_n = fld(c, NEMO_F_E3T_N), *tmask = c->tmask;
  const int l_ldfslp = nm->ln_traldf_iso || nm->ln_traldf_triad;   /* ldftra.F90:253-255 */
  if (!avt && !is_trc) return NEMO_ERR_UNBOUND;
  if (l_ldfslp && ((nm->ln_traldf_msc && !akz) || (!nm->ln_traldf_msc && !ah_wslp2))) return NEMO_ERR_UNBOUND;
  double *zwi = walloc(n3), *zwt = walloc(n3), *zwd = walloc(n3), *zws = walloc(n3);
  for (int jn = 1; jn <= kjpt; ++jn) {
    const double *tb = ptb + n3 * (jn - 1);
    double *ta = pta + n3 * (jn - 1);
    if ((!is_trc && (jn == 1 || (jn == 2 && nm->ln_zdfddm))) || (is_trc && jn == 1)) {
      const double *coef = (!is_trc && jn == 1) ? avt : avs;
      if (!coef) { wfree(zwi); wfree(zwt); wfree(zwd); wfree(zws); return NEMO_ERR_UNBOUND; }
      zdf_lu(c, coef, p2dt, zwi, zwt, zwd, zws);
    }
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, 1);
        ta[q] = e3t_b[q] * tb[q] + p2dt * e3t_n[q] * ta[q];
      }
    for (int jk = 2; jk <= jpk - 1; ++jk)
      OMP_FOR
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double zrhs = e3t_b[q] * tb[q] + p2dt * e3t_n[q] * ta[q];
          ta[q] = zrhs - zwi[q] / zwt[I3(ji, jj, jk - 1)] * ta[I3(ji, jj, jk - 1)];
        }
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jpk - 1);
        ta[q] = ta[q] / zwt[q] * tmask[q];
      }
    for (int jk = jpk - 2; jk >= 1; --jk)
      OMP_FOR
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          ta[q] = (ta[q] - zws[q] * ta[I3(ji, jj, jk + 1)]) / zwt[q] * tmask[q];
        }
  }
  wfree(zwi); wfree(zwt); wfree(zwd); wfree(zws);
  return NEMO_OK;
}

/* trazdf.F90:46-106 on the bound tsb / tsa (no trend diagnostics) */
int ora_tra_zdf(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  double *tsb = c->f[NEMO_F_TSB], *tsa = c->f[NEMO_F_TSA];
  if (!tsb || !tsa) return NEMO_ERR_UNBOUND;
  if (nm->neuler == 0 && kt == nm->nit000) c->r2dt = nm->rn_rdt;
  else if (kt <= nm->nit000 + 1) c->r2dt = 2. * nm->rn_rdt;
  int st = ora_tra_zdf_imp(c, kt, nm->nit000, "TRA", c->r2dt, tsb, tsa, 2);
  if (st) return st;
  const size_t n3 = (size_t)c->jpi * c->jpj * c->jpk;
  double *sa = tsa + n3;
  for (size_t q = 0; q < n3; ++q)
    if (sa[q] < 0.0) sa[q] = 0.1;
  return NEMO_OK;
}

/* Coriolis factors of dyn_spg_ts (dynspg_ts.F90:241-342): zwz = ff_f / hf
 * (ENE/ENS/MIX) or the EEN/EET triads, from the now depths ht_n and e3f_n. The
 * reference computes them at kt = nit000 for a linear free surface (rest-state
 * depths; they depend only on the domain, so they are also computed at context
 * creation to give calls that start later the same values) and at every step
 * otherwise. */
static void spg_coriolis_factors(ora_ctx *c, const double *ht_n, const double *e3f_n) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  const nemo_namelist *nm = &c->nam;
  const double *umask = c->umask, *ssmask = c->ssmask;
  double *zhf = zalloc(n2);
  const int sc = nm->nvor_scheme;
  if (sc == NEMO_VOR_EEN) {
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        double z;
        if (nm->nn_een_e3f == 0)
          z = (ht_n[I2(ji, jj + 1)] + ht_n[I2(ji + 1, jj + 1)] + ht_n[I2(ji, jj)] + ht_n[I2(ji + 1, jj)]) * 0.25;
        else
          z = (ht_n[I2(ji, jj + 1)] + ht_n[I2(ji + 1, jj + 1)] + ht_n[I2(ji, jj)] + ht_n[I2(ji + 1, jj)])
              / dmax(1.0, ssmask[I2(ji, jj + 1)] + ssmask[I2(ji + 1, jj + 1)] + ssmask[I2(ji, jj)] + ssmask[I2(ji + 1, jj)]);
        if (z != 0.0) z = c->ff_f[I2(ji, jj)] / z;
        c->zwz[I2(ji, jj)] = z;
      }
    lbc_closed(jpi, jpj, c->zwz, 1, 'F', 0.0);
    for (int jj = 1; jj <= jpj; ++jj) {
      c->ftne[I2(1, jj)] = 0; c->ftnw[I2(1, jj)] = 0; c->ftse[I2(1, jj)] = 0; c->ftsw[I2(1, jj)] = 0;
    }
    for (int jj = 2; jj <= jpj; ++jj)
      for (int ji = 2; ji <= jpi; ++ji) {
        const double *w = c->zwz;
        c->ftne[I2(ji, jj)] = w[I2(ji - 1, jj)] + w[I2(ji, jj)] + w[I2(ji, jj - 1)];
        c->ftnw[I2(ji, jj)] = w[I2(ji - 1, jj - 1)] + w[I2(ji - 1, jj)] + w[I2(ji, jj)];
        c->ftse[I2(ji, jj)] = w[I2(ji, jj)] + w[I2(ji, jj - 1)] + w[I2(ji - 1, jj - 1)];
        c->ftsw[I2(ji, jj)] = w[I2(ji, jj - 1)] + w[I2(ji - 1, jj - 1)] + w[I2(ji - 1, jj)];
      }
  } else if (sc == NEMO_VOR_EET) {
    const double *ff = c->ff_f;
    for (int jj = 1; jj <= jpj; ++jj) {
      c->ftne[I2(1, jj)] = 0; c->ftnw[I2(1, jj)] = 0; c->ftse[I2(1, jj)] = 0; c->ftsw[I2(1, jj)] = 0;
    }
    for (int jj = 2; jj <= jpj; ++jj)
      for (int ji = 2; ji <= jpi; ++ji) {
        double z1_ht = ssmask[I2(ji, jj)] / (ht_n[I2(ji, jj)] + 1.0 - ssmask[I2(ji, jj)]);
        c->ftne[I2(ji, jj)] = (ff[I2(ji - 1, jj)] + ff[I2(ji, jj)] + ff[I2(ji, jj - 1)]) * z1_ht;
        c->ftnw[I2(ji, jj)] = (ff[I2(ji - 1, jj - 1)] + ff[I2(ji - 1, jj)] + ff[I2(ji, jj)]) * z1_ht;
        c->ftse[I2(ji, jj)] = (ff[I2(ji, jj)] + ff[I2(ji, jj - 1)] + ff[I2(ji - 1, jj - 1)]) * z1_ht;
        c->ftsw[I2(ji, jj)] = (ff[I2(ji, jj - 1)] + ff[I2(ji - 1, jj - 1)] + ff[I2(ji - 1, jj)]) * z1_ht;
      }
  } else if (sc == NEMO_VOR_ENE || sc == NEMO_VOR_ENS || sc == NEMO_VOR_MIX) {
    for (size_t p = 0; p < n2; ++p) { c->zwz[p] = 0.0; zhf[p] = 0.0; }
    if (nm->ln_sco) {
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji)
          zhf[I2(ji, jj)] = (c->ht_0[I2(ji, jj)] + c->ht_0[I2(ji + 1, jj)] + c->ht_0[I2(ji, jj + 1)] + c->ht_0[I2(ji + 1, jj + 1)])
                            / dmax(ssmask[I2(ji, jj)] + ssmask[I2(ji + 1, jj)] + ssmask[I2(ji, jj + 1)] + ssmask[I2(ji + 1, jj + 1)], 1.0);
    }
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi; ++ji)
        zhf[I2(ji, jj)] = zhf[I2(ji, jj)] * (1.0 - umask[I3(ji, jj, 1)] * umask[I3(ji, jj + 1, 1)]);
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi; ++ji)
          zhf[I2(ji, jj)] = zhf[I2(ji, jj)] + e3f_n[I3(ji, jj, jk)] * umask[I3(ji, jj, jk)] * umask[I3(ji, jj + 1, jk)];
    lbc_closed(jpi, jpj, zhf, 1, 'F', 0.0);
    for (size_t p = 0; p < n2; ++p)
      if (zhf[p] != 0.0) c->zwz[p] = 1.0 / zhf[p];
    for (size_t p = 0; p < n2; ++p) c->zwz[p] = c->ff_f[p] * c->zwz[p];
  }
  wfree(zhf);
}

/* ---------------------------------------------------------------- dyn_spg_ts */
/* dynspg_ts.F90:121-1310 without isf, wetting/drying, tides, bdy, agrif, Stokes
 * drift or assimilation increments. Linear (ln_linssh) or variable-volume free
 * surface; with a variable volume, vector-form (ln_dynadv_vec) or flux-form
 * momentum. */
int ora_dyn_spg_ts(ora_ctx *c, int kt) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  const nemo_namelist *nm = &c->nam;
  double *const *F = c->f;
  double *ua = F[NEMO_F_UA], *va = F[NEMO_F_VA], *un = F[NEMO_F_UN], *vn = F[NEMO_F_VN];
  double *ub = F[NEMO_F_UB], *vb = F[NEMO_F_VB];
  double *sshn = F[NEMO_F_SSHN], *sshb = F[NEMO_F_SSHB], *ssha = F[NEMO_F_SSHA];
  double *un_b = F[NEMO_F_UN_B], *vn_b = F[NEMO_F_VN_B], *ub_b = F[NEMO_F_UB_B], *vb_b = F[NEMO_F_VB_B];
  double *ua_b = F[NEMO_F_UA_B], *va_b = F[NEMO_F_VA_B];
  double *un_adv = F[NEMO_F_UN_ADV], *vn_adv = F[NEMO_F_VN_ADV];
  double *ub2_b = F[NEMO_F_UB2_B], *vb2_b = F[NEMO_F_VB2_B], *un_bf = F[NEMO_F_UN_BF], *vn_bf = F[NEMO_F_VN_BF];
  double *utau = F[NEMO_F_UTAU], *vtau = F[NEMO_F_VTAU], *utau_b = F[NEMO_F_UTAU_B], *vtau_b = F[NEMO_F_VTAU_B];
  double *emp = F[NEMO_F_EMP], *emp_b = F[NEMO_F_EMP_B], *rnf = F[NEMO_F_RNF], *rnf_b = F[NEMO_F_RNF_B];
  double *rCdU_bot = F[NEMO_F_RCDU_BOT], *ssh_ib = F[NEMO_F_SSH_IB], *ssh_ibb = F[NEMO_F_SSH_IBB];
  if (!ua || !va || !un || !vn || !sshn || !ssha || !un_b || !vn_b || !ub_b || !vb_b || !ua_b || !va_b ||
      !un_adv || !vn_adv || !ub2_b || !vb2_b || !un_bf || !vn_bf || !utau || !vtau || !emp || !rCdU_bot)
    return NEMO_ERR_UNBOUND;
  if (!nm->ln_bt_fw && (!ub || !vb || !sshb || !utau_b || !vtau_b || !emp_b)) return NEMO_ERR_UNBOUND;
  if (nm->ln_apr_dyn && (!ssh_ib || (!nm->ln_bt_fw && !ssh_ibb))) return NEMO_ERR_UNBOUND;
  const double *umask = c->umask, *vmask = c->vmask, *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N);
  /* depths: the rest state for a linear free surface (domain.F90:149-183), the
   * bound now / before depths of domvvl.F90 otherwise */
  const int vvl = !nm->ln_linssh, flux = vvl && !nm->ln_dynadv_vec;
  const double *hu_n = c->hu_0, *hv_n = c->hv_0, *r1_hu_n = c->r1_hu_0, *r1_hv_n = c->r1_hv_0, *ht_n = c->ht_0;
  const double *hu_b = c->hu_0, *hv_b = c->hv_0, *r1_hu_b = c->r1_hu_0, *r1_hv_b = c->r1_hv_0;
  const double *e3f_n = c->e3f_0;
  const int sc = nm->nvor_scheme;
  if (vvl) {
    hu_n = F[NEMO_F_HU_N]; hv_n = F[NEMO_F_HV_N]; r1_hu_n = F[NEMO_F_R1_HU_N]; r1_hv_n = F[NEMO_F_R1_HV_N];
    ht_n = F[NEMO_F_HT_N];
    if (!hu_n || !hv_n || !r1_hu_n || !r1_hv_n || !ht_n) return NEMO_ERR_UNBOUND;
    if (sc == NEMO_VOR_ENE || sc == NEMO_VOR_ENS || sc == NEMO_VOR_MIX) {
      e3f_n = F[NEMO_F_E3F_N];
      if (!e3f_n) return NEMO_ERR_UNBOUND;
    }
    if (!nm->ln_bt_fw || flux) {
      hu_b = F[NEMO_F_HU_B]; hv_b = F[NEMO_F_HV_B];
      if (!hu_b || !hv_b) return NEMO_ERR_UNBOUND;
    }
    if (!nm->ln_bt_fw) {
      r1_hu_b = F[NEMO_F_R1_HU_B]; r1_hv_b = F[NEMO_F_R1_HV_B];
      if (!r1_hu_b || !r1_hv_b) return NEMO_ERR_UNBOUND;
    }
  }
  const double *ssumask = c->ssumask, *ssvmask = c->ssvmask, *ssmask = c->ssmask;
  const double r1_2 = 0.5, r1_4 = 0.25, r1_8 = 0.125, r1_12 = 1.0 / 12.0;
  const double grav = nm->grav, r1_rau0 = 1.0 / nm->rau0, rdtbt = c->rdtbt;
  const int ln_bt_fw = nm->ln_bt_fw, ln_dynadv_vec = nm->ln_dynadv_vec;
  double *zu_frc = walloc(n2), *zv_frc = walloc(n2), *zu_trd = walloc(n2), *zv_trd = walloc(n2);
  double *zwx = walloc(n2), *zwy = walloc(n2), *zssh_frc = walloc(n2), *zhdiv = walloc(n2);
  double *zsshp2_e = walloc(n2), *zCdU_u = walloc(n2), *zCdU_v = walloc(n2);
  double *zhup2_e = walloc(n2), *zhvp2_e = walloc(n2), *zhtp2_e = walloc(n2);
  double *zsshu_a = walloc(n2), *zsshv_a = walloc(n2), *zhust_e = walloc(n2), *zhvst_e = walloc(n2);
  double z2dt_bf = (kt == nm->nit000 && nm->neuler == 0) ? nm->rn_rdt : 2.0 * nm->rn_rdt;
  double r1_2dt_b = 1.0 / z2dt_bf;
  int ll_init = nm->ln_bt_av, ll_fw_start = 0;
  if (kt == nm->nit000) {
    if (nm->neuler == 0) ll_init = 1;
    ll_fw_start = (nm->ln_bt_fw || nm->neuler == 0) ? 1 : 0;
    ts_wgt(c, nm->ln_bt_av, ll_fw_start, &c->icycle, c->wgtbtp1, c->wgtbtp2);
  }
  /* (:225-231) bottom friction only */
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      zCdU_u[I2(ji, jj)] = r1_2 * (rCdU_bot[I2(ji + 1, jj)] + rCdU_bot[I2(ji, jj)]);
      zCdU_v[I2(ji, jj)] = r1_2 * (rCdU_bot[I2(ji, jj + 1)] + rCdU_bot[I2(ji, jj)]);
    }
  /* (:241-343) at nit000, and at every step with a variable volume */
  if (kt == nm->nit000 || vvl) spg_coriolis_factors(c, ht_n, e3f_n);
  if (!nm->ln_bt_fw && (nm->neuler == 0 && kt == nm->nit000 + 1)) {
    ll_fw_start = 0;
    ts_wgt(c, nm->ln_bt_av, ll_fw_start, &c->icycle, c->wgtbtp1, c->wgtbtp2);
  }
  /* Phase 1 (:358-378) */
  for (size_t p = 0; p < n2; ++p) { zu_frc[p] = 0.0; zv_frc[p] = 0.0; }
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      size_t q = p + n2 * (jk - 1);
      zu_frc[p] = zu_frc[p] + e3u[q] * ua[q] * umask[q];
      zv_frc[p] = zv_frc[p] + e3v[q] * va[q] * vmask[q];
    }
  for (size_t p = 0; p < n2; ++p) { zu_frc[p] = zu_frc[p] * r1_hu_n[p]; zv_frc[p] = zv_frc[p] * r1_hv_n[p]; }
  OMP_FOR
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        ua[q] = ua[q] - zu_frc[I2(ji, jj)] * umask[q];
        va[q] = va[q] - zv_frc[I2(ji, jj)] * vmask[q];
      }
  /* barotropic Coriolis (:387-443) */
  for (size_t p = 0; p < n2; ++p) {
    zwx[p] = un_b[p] * hu_n[p] * c->e2u[p];
    zwy[p] = vn_b[p] * hv_n[p] * c->e1v[p];
  }
  OMP_FOR
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      size_t p = I2(ji, jj);
      if (sc == NEMO_VOR_ENT) {
        const double *e = c->e1e2t, *h = ht_n, *ft = c->ff_t;
        zu_trd[p] = +r1_4 * c->r1_e1e2u[p] * r1_hu_n[p]
                    * (e[I2(ji + 1, jj)] * h[I2(ji + 1, jj)] * ft[I2(ji + 1, jj)] * (vn_b[I2(ji + 1, jj)] + vn_b[I2(ji + 1, jj - 1)])
                       + e[p] * h[p] * ft[p] * (vn_b[p] + vn_b[I2(ji, jj - 1)]));
        zv_trd[p] = -r1_4 * c->r1_e1e2v[p] * r1_hv_n[p]
                    * (e[I2(ji, jj + 1)] * h[I2(ji, jj + 1)] * ft[I2(ji, jj + 1)] * (un_b[I2(ji, jj + 1)] + un_b[I2(ji - 1, jj + 1)])
                       + e[p] * h[p] * ft[p] * (un_b[p] + un_b[I2(ji - 1, jj)]));
      } else if (sc == NEMO_VOR_ENE || sc == NEMO_VOR_MIX) {
        double zy1 = (zwy[I2(ji, jj - 1)] + zwy[I2(ji + 1, jj - 1)]) * c->r1_e1u[p];
        double zy2 = (zwy[p] + zwy[I2(ji + 1, jj)]) * c->r1_e1u[p];
        double zx1 = (zwx[I2(ji - 1, jj)] + zwx[I2(ji - 1, jj + 1)]) * c->r1_e2v[p];
        double zx2 = (zwx[p] + zwx[I2(ji, jj + 1)]) * c->r1_e2v[p];
        zu_trd[p] = r1_4 * (c->zwz[I2(ji, jj - 1)] * zy1 + c->zwz[p] * zy2);
        zv_trd[p] = -r1_4 * (c->zwz[I2(ji - 1, jj)] * zx1 + c->zwz[p] * zx2);
      } else if (sc == NEMO_VOR_ENS) {
        double zy1 = r1_8 * (zwy[I2(ji, jj - 1)] + zwy[I2(ji + 1, jj - 1)] + zwy[p] + zwy[I2(ji + 1, jj)]) * c->r1_e1u[p];
        double zx1 = -r1_8 * (zwx[I2(ji - 1, jj)] + zwx[I2(ji - 1, jj + 1)] + zwx[p] + zwx[I2(ji, jj + 1)]) * c->r1_e2v[p];
        zu_trd[p] = zy1 * (c->zwz[I2(ji, jj - 1)] + c->zwz[p]);
        zv_trd[p] = zx1 * (c->zwz[I2(ji - 1, jj)] + c->zwz[p]);
      } else {
        zu_trd[p] = +r1_12 * c->r1_e1u[p] * (c->ftne[p] * zwy[p] + c->ftnw[I2(ji + 1, jj)] * zwy[I2(ji + 1, jj)]
                                              + c->ftse[p] * zwy[I2(ji, jj - 1)] + c->ftsw[I2(ji + 1, jj)] * zwy[I2(ji + 1, jj - 1)]);
        zv_trd[p] = -r1_12 * c->r1_e2v[p] * (c->ftsw[I2(ji, jj + 1)] * zwx[I2(ji - 1, jj + 1)] + c->ftse[I2(ji, jj + 1)] * zwx[I2(ji, jj + 1)]
                                              + c->ftnw[p] * zwx[I2(ji - 1, jj)] + c->ftne[p] * zwx[p]);
      }
    }
  /* variable volume: remove the surface pressure gradient (:447-509) */
  if (vvl)
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj);
        zu_trd[p] = zu_trd[p] - grav * (sshn[I2(ji + 1, jj)] - sshn[p]) * c->r1_e1u[p];
        zv_trd[p] = zv_trd[p] - grav * (sshn[I2(ji, jj + 1)] - sshn[p]) * c->r1_e2v[p];
      }
  /* (:511-516) */
  OMP_FOR
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      size_t p = I2(ji, jj);
      zu_frc[p] = zu_frc[p] - zu_trd[p] * ssumask[p];
      zv_frc[p] = zv_frc[p] - zv_trd[p] * ssvmask[p];
    }
  /* bottom stress from baroclinic velocities (:519-557) */
  OMP_FOR
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      size_t p = I2(ji, jj);
      int ikbu = c->mbku[p], ikbv = c->mbkv[p];
      if (ln_bt_fw) {
        zwx[p] = un[I3(ji, jj, ikbu)] - un_b[p];
        zwy[p] = vn[I3(ji, jj, ikbv)] - vn_b[p];
      } else {
        zwx[p] = ub[I3(ji, jj, ikbu)] - ub_b[p];
        zwy[p] = vb[I3(ji, jj, ikbv)] - vb_b[p];
      }
    }
  OMP_FOR
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      size_t p = I2(ji, jj);
      zu_frc[p] = zu_frc[p] + r1_hu_n[p] * r1_2 * (rCdU_bot[I2(ji + 1, jj)] + rCdU_bot[p]) * zwx[p];
      zv_frc[p] = zv_frc[p] + r1_hv_n[p] * r1_2 * (rCdU_bot[I2(ji, jj + 1)] + rCdU_bot[p]) * zwy[p];
    }
  /* wind (:589-604) */
  OMP_FOR
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      size_t p = I2(ji, jj);
      if (ln_bt_fw) {
        zu_frc[p] = zu_frc[p] + r1_rau0 * utau[p] * r1_hu_n[p];
        zv_frc[p] = zv_frc[p] + r1_rau0 * vtau[p] * r1_hv_n[p];
      } else {
        double zztmp = r1_rau0 * r1_2;
        zu_frc[p] = zu_frc[p] + zztmp * (utau_b[p] + utau[p]) * r1_hu_n[p];
        zv_frc[p] = zv_frc[p] + zztmp * (vtau_b[p] + vtau[p]) * r1_hv_n[p];
      }
    }
  /* atmospheric pressure (:606-629) */
  if (nm->ln_apr_dyn)
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj);
        double zu_spg, zv_spg;
        if (ln_bt_fw) {
          zu_spg = grav * (ssh_ib[I2(ji + 1, jj)] - ssh_ib[p]) * c->r1_e1u[p];
          zv_spg = grav * (ssh_ib[I2(ji, jj + 1)] - ssh_ib[p]) * c->r1_e2v[p];
        } else {
          double zztmp = grav * r1_2;
          zu_spg = zztmp * (ssh_ib[I2(ji + 1, jj)] - ssh_ib[p] + ssh_ibb[I2(ji + 1, jj)] - ssh_ibb[p]) * c->r1_e1u[p];
          zv_spg = zztmp * (ssh_ib[I2(ji, jj + 1)] - ssh_ib[p] + ssh_ibb[I2(ji, jj + 1)] - ssh_ibb[p]) * c->r1_e2v[p];
        }
        zu_frc[p] = zu_frc[p] + zu_spg;
        zv_frc[p] = zv_frc[p] + zv_spg;
      }
  /* ssh forcing (:633-639), rnf / fwfisf absent when not bound */
  for (size_t p = 0; p < n2; ++p) {
    double r = rnf ? rnf[p] : 0.0;
    if (ln_bt_fw) zssh_frc[p] = r1_rau0 * (emp[p] - r + 0.0);
    else {
      double rb = rnf_b ? rnf_b[p] : 0.0;
      zssh_frc[p] = r1_rau0 * r1_2 * (emp[p] + emp_b[p] - r - rb + 0.0 + 0.0);
    }
  }
  /* Phase 2 initialisation (:665-702) */
  if (ll_init)
    for (size_t p = 0; p < n2; ++p) {
      c->sshbb_e[p] = 0; c->ubb_e[p] = 0; c->vbb_e[p] = 0; c->sshb_e[p] = 0; c->ub_e[p] = 0; c->vb_e[p] = 0;
    }
  for (size_t p = 0; p < n2; ++p) {
    if (ln_bt_fw) {
      c->sshn_e[p] = sshn[p]; c->un_e[p] = un_b[p]; c->vn_e[p] = vn_b[p];
      c->hu_e[p] = hu_n[p]; c->hv_e[p] = hv_n[p]; c->hur_e[p] = r1_hu_n[p]; c->hvr_e[p] = r1_hv_n[p];
    } else {
      c->sshn_e[p] = sshb[p]; c->un_e[p] = ub_b[p]; c->vn_e[p] = vb_b[p];
      c->hu_e[p] = hu_b[p]; c->hv_e[p] = hv_b[p]; c->hur_e[p] = r1_hu_b[p]; c->hvr_e[p] = r1_hv_b[p];
    }
    ua_b[p] = 0; va_b[p] = 0; ssha[p] = 0; un_adv[p] = 0; vn_adv[p] = 0;
  }
  /* sub-step loop (:712-1207) */
  for (int jn = 1; jn <= c->icycle; ++jn) {
    double za0, za1, za2, za3;
    if (jn < 3 && ll_init) { za1 = 1.0; za2 = 0.0; za3 = 0.0; }
    else { za1 = 1.781105; za2 = -1.06221; za3 = 0.281105; }
    OMP_FOR
    for (size_t p = 0; p < n2; ++p) {
      c->ua_e[p] = za1 * c->un_e[p] + za2 * c->ub_e[p] + za3 * c->ubb_e[p];
      c->va_e[p] = za1 * c->vn_e[p] + za2 * c->vb_e[p] + za3 * c->vbb_e[p];
    }
    /* ocean depth of the predictor (:738-792): from the extrapolated ssh with a
     * variable volume, the now depth otherwise */
    if (vvl) {
      OMP_FOR
      for (size_t p = 0; p < n2; ++p)
        zsshp2_e[p] = za1 * c->sshn_e[p] + za2 * c->sshb_e[p] + za3 * c->sshbb_e[p];
      OMP_FOR
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t p = I2(ji, jj);
          zwx[p] = r1_2 * ssumask[p] * c->r1_e1e2u[p]
                   * (c->e1e2t[p] * zsshp2_e[p] + c->e1e2t[I2(ji + 1, jj)] * zsshp2_e[I2(ji + 1, jj)]);
          zwy[p] = r1_2 * ssvmask[p] * c->r1_e1e2v[p]
                   * (c->e1e2t[p] * zsshp2_e[p] + c->e1e2t[I2(ji, jj + 1)] * zsshp2_e[I2(ji, jj + 1)]);
        }
      lbc_closed(jpi, jpj, zwx, 1, 'U', 0.0);
      lbc_closed(jpi, jpj, zwy, 1, 'V', 0.0);
      for (size_t p = 0; p < n2; ++p) {
        zhup2_e[p] = c->hu_0[p] + zwx[p];
        zhvp2_e[p] = c->hv_0[p] + zwy[p];
        zhtp2_e[p] = c->ht_0[p] + zsshp2_e[p];
      }
    } else
      for (size_t p = 0; p < n2; ++p) { zhup2_e[p] = hu_n[p]; zhvp2_e[p] = hv_n[p]; zhtp2_e[p] = ht_n[p]; }
    /* fluxes at jn + 1/2 (:799-800) */
    OMP_FOR
    for (size_t p = 0; p < n2; ++p) {
      zwx[p] = c->e2u[p] * c->ua_e[p] * zhup2_e[p];
      zwy[p] = c->e1v[p] * c->va_e[p] * zhvp2_e[p];
    }
    za2 = c->wgtbtp2[jn - 1];
    OMP_FOR
    for (size_t p = 0; p < n2; ++p) {
      un_adv[p] = un_adv[p] + za2 * zwx[p] * c->r1_e2u[p];
      vn_adv[p] = vn_adv[p] + za2 * zwy[p] * c->r1_e1v[p];
    }
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj);
        zhdiv[p] = (zwx[p] - zwx[I2(ji - 1, jj)] + zwy[p] - zwy[I2(ji, jj - 1)]) * c->r1_e1e2t[p];
      }
    OMP_FOR
    for (size_t p = 0; p < n2; ++p) c->ssha_e[p] = (c->sshn_e[p] - rdtbt * (zssh_frc[p] + zhdiv[p])) * ssmask[p];
    lbc_closed(jpi, jpj, c->ssha_e, 1, 'T', 0.0);
    /* ssh at u- and v-points of the new level (:888-900) */
    if (vvl) {
      OMP_FOR
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t p = I2(ji, jj);
          zsshu_a[p] = r1_2 * ssumask[p] * c->r1_e1e2u[p]
                       * (c->e1e2t[p] * c->ssha_e[p] + c->e1e2t[I2(ji + 1, jj)] * c->ssha_e[I2(ji + 1, jj)]);
          zsshv_a[p] = r1_2 * ssvmask[p] * c->r1_e1e2v[p]
                       * (c->e1e2t[p] * c->ssha_e[p] + c->e1e2t[I2(ji, jj + 1)] * c->ssha_e[I2(ji, jj + 1)]);
        }
      lbc_closed(jpi, jpj, zsshu_a, 1, 'U', 0.0);
      lbc_closed(jpi, jpj, zsshv_a, 1, 'V', 0.0);
    }
    if (jn == 1 && ll_init) { za0 = 1.0; za1 = 0.0; za2 = 0.0; za3 = 0.0; }
    else if (jn == 2 && ll_init) { za0 = 1.0833333333333; za1 = -0.1666666666666; za2 = 0.0833333333333; za3 = 0.0; }
    else if (nm->rn_bt_alpha == 0.0) { za0 = 0.614; za1 = 0.285; za2 = 0.088; za3 = 0.013; }
    else {
      double zepsilon = 0.00976186 - 0.13451357 * nm->rn_bt_alpha;
      double zgamma = 0.08344500 - 0.51358400 * nm->rn_bt_alpha;
      za0 = 0.5 + zgamma + 2.0 * nm->rn_bt_alpha + 2.0 * zepsilon;
      za1 = 1.0 - za0 - zgamma - zepsilon;
      za2 = zgamma;
      za3 = zepsilon;
    }
    OMP_FOR
    for (size_t p = 0; p < n2; ++p)
      zsshp2_e[p] = za0 * c->ssha_e[p] + za1 * c->sshn_e[p] + za2 * c->sshb_e[p] + za3 * c->sshbb_e[p];
    /* flux form: depth at u- and v-points of the AM4 ssh (:973-991) */
    if (flux)
      OMP_FOR
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t p = I2(ji, jj);
          double zx1 = r1_2 * ssumask[p] * c->r1_e1e2u[p]
                       * (c->e1e2t[p] * zsshp2_e[p] + c->e1e2t[I2(ji + 1, jj)] * zsshp2_e[I2(ji + 1, jj)]);
          double zy1 = r1_2 * ssvmask[p] * c->r1_e1e2v[p]
                       * (c->e1e2t[p] * zsshp2_e[p] + c->e1e2t[I2(ji, jj + 1)] * zsshp2_e[I2(ji, jj + 1)]);
          zhust_e[p] = c->hu_0[p] + zx1;
          zhvst_e[p] = c->hv_0[p] + zy1;
        }
    /* Coriolis (:1000-1056) */
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj);
        if (sc == NEMO_VOR_ENT) {
          const double *e = c->e1e2t, *h = zhtp2_e, *ft = c->ff_t;
          double z1_hu = ssumask[p] / (zhup2_e[p] + 1.0 - ssumask[p]);
          double z1_hv = ssvmask[p] / (zhvp2_e[p] + 1.0 - ssvmask[p]);
          zu_trd[p] = +r1_4 * c->r1_e1e2u[p] * z1_hu
                      * (e[I2(ji + 1, jj)] * h[I2(ji + 1, jj)] * ft[I2(ji + 1, jj)] * (c->va_e[I2(ji + 1, jj)] + c->va_e[I2(ji + 1, jj - 1)])
                         + e[p] * h[p] * ft[p] * (c->va_e[p] + c->va_e[I2(ji, jj - 1)]));
          zv_trd[p] = -r1_4 * c->r1_e1e2v[p] * z1_hv
                      * (e[I2(ji, jj + 1)] * h[I2(ji, jj + 1)] * ft[I2(ji, jj + 1)] * (c->ua_e[I2(ji, jj + 1)] + c->ua_e[I2(ji - 1, jj + 1)])
                         + e[p] * h[p] * ft[p] * (c->ua_e[p] + c->ua_e[I2(ji - 1, jj)]));
        } else if (sc == NEMO_VOR_ENE || sc == NEMO_VOR_MIX) {
          double zy1 = (zwy[I2(ji, jj - 1)] + zwy[I2(ji + 1, jj - 1)]) * c->r1_e1u[p];
          double zy2 = (zwy[p] + zwy[I2(ji + 1, jj)]) * c->r1_e1u[p];
          double zx1 = (zwx[I2(ji - 1, jj)] + zwx[I2(ji - 1, jj + 1)]) * c->r1_e2v[p];
          double zx2 = (zwx[p] + zwx[I2(ji, jj + 1)]) * c->r1_e2v[p];
          zu_trd[p] = r1_4 * (c->zwz[I2(ji, jj - 1)] * zy1 + c->zwz[p] * zy2);
          zv_trd[p] = -r1_4 * (c->zwz[I2(ji - 1, jj)] * zx1 + c->zwz[p] * zx2);
        } else if (sc == NEMO_VOR_ENS) {
          double zy1 = r1_8 * (zwy[I2(ji, jj - 1)] + zwy[I2(ji + 1, jj - 1)] + zwy[p] + zwy[I2(ji + 1, jj)]) * c->r1_e1u[p];
          double zx1 = -r1_8 * (zwx[I2(ji - 1, jj)] + zwx[I2(ji - 1, jj + 1)] + zwx[p] + zwx[I2(ji, jj + 1)]) * c->r1_e2v[p];
          zu_trd[p] = zy1 * (c->zwz[I2(ji, jj - 1)] + c->zwz[p]);
          zv_trd[p] = zx1 * (c->zwz[I2(ji - 1, jj)] + c->zwz[p]);
        } else {
          zu_trd[p] = +r1_12 * c->r1_e1u[p] * (c->ftne[p] * zwy[p] + c->ftnw[I2(ji + 1, jj)] * zwy[I2(ji + 1, jj)]
                                                + c->ftse[p] * zwy[I2(ji, jj - 1)] + c->ftsw[I2(ji + 1, jj)] * zwy[I2(ji + 1, jj - 1)]);
          zv_trd[p] = -r1_12 * c->r1_e2v[p] * (c->ftsw[I2(ji, jj + 1)] * zwx[I2(ji - 1, jj + 1)] + c->ftse[I2(ji, jj + 1)] * zwx[I2(ji, jj + 1)]
                                                + c->ftnw[p] * zwx[I2(ji - 1, jj)] + c->ftne[p] * zwx[p]);
        }
      }
    /* bottom stress (:1072-1079) */
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj);
        zu_trd[p] = zu_trd[p] + zCdU_u[p] * c->un_e[p] * c->hur_e[p];
        zv_trd[p] = zv_trd[p] + zCdU_v[p] * c->vn_e[p] * c->hvr_e[p];
      }
    /* surface pressure gradient (:1093-1101) */
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj);
        double zu_spg = -grav * (zsshp2_e[I2(ji + 1, jj)] - zsshp2_e[p]) * c->r1_e1u[p];
        double zv_spg = -grav * (zsshp2_e[I2(ji, jj + 1)] - zsshp2_e[p]) * c->r1_e2v[p];
        zwx[p] = (1.0 - nm->rn_scal_load) * zu_spg;
        zwy[p] = (1.0 - nm->rn_scal_load) * zv_spg;
      }
    /* next velocities, vector form (:1106-1122) or flux form (:1124-1147) */
    OMP_FOR
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj);
        if (!flux) {
          c->ua_e[p] = (c->un_e[p] + rdtbt * (zwx[p] + zu_trd[p] + zu_frc[p])) * ssumask[p];
          c->va_e[p] = (c->vn_e[p] + rdtbt * (zwy[p] + zv_trd[p] + zv_frc[p])) * ssvmask[p];
        } else {
          double zhura = c->hu_0[p] + zsshu_a[p];
          double zhvra = c->hv_0[p] + zsshv_a[p];
          zhura = ssumask[p] / (zhura + 1.0 - ssumask[p]);
          zhvra = ssvmask[p] / (zhvra + 1.0 - ssvmask[p]);
          c->ua_e[p] = (c->hu_e[p] * c->un_e[p]
                        + rdtbt * (zhust_e[p] * zwx[p] + zhup2_e[p] * zu_trd[p] + hu_n[p] * zu_frc[p])) * zhura;
          c->va_e[p] = (c->hv_e[p] * c->vn_e[p]
                        + rdtbt * (zhvst_e[p] * zwy[p] + zhvp2_e[p] * zv_trd[p] + hv_n[p] * zv_frc[p])) * zhvra;
        }
      }
    /* depth of the new level (:1159-1165) */
    if (vvl)
      OMP_FOR
      for (size_t p = 0; p < n2; ++p) {
        c->hu_e[p] = c->hu_0[p] + zsshu_a[p];
        c->hv_e[p] = c->hv_0[p] + zsshv_a[p];
        c->hur_e[p] = ssumask[p] / (c->hu_e[p] + 1.0 - ssumask[p]);
        c->hvr_e[p] = ssvmask[p] / (c->hv_e[p] + 1.0 - ssvmask[p]);
      }
    lbc_closed(jpi, jpj, c->ua_e, 1, 'U', 0.0);
    lbc_closed(jpi, jpj, c->va_e, 1, 'V', 0.0);
    /* swap (:1176-1186) */
    OMP_FOR
    for (size_t p = 0; p < n2; ++p) {
      c->ubb_e[p] = c->ub_e[p]; c->ub_e[p] = c->un_e[p]; c->un_e[p] = c->ua_e[p];
      c->vbb_e[p] = c->vb_e[p]; c->vb_e[p] = c->vn_e[p]; c->vn_e[p] = c->va_e[p];
      c->sshbb_e[p] = c->sshb_e[p]; c->sshb_e[p] = c->sshn_e[p]; c->sshn_e[p] = c->ssha_e[p];
    }
    /* sums of velocities or transports (:1190-1204) */
    za1 = c->wgtbtp1[jn - 1];
    OMP_FOR
    for (size_t p = 0; p < n2; ++p) {
      if (!flux) {
        ua_b[p] = ua_b[p] + za1 * c->ua_e[p];
        va_b[p] = va_b[p] + za1 * c->va_e[p];
      } else {
        ua_b[p] = ua_b[p] + za1 * c->ua_e[p] * c->hu_e[p];
        va_b[p] = va_b[p] + za1 * c->va_e[p] * c->hv_e[p];
      }
      ssha[p] = ssha[p] + za1 * c->ssha_e[p];
    }
  }
  (void)ln_dynadv_vec;
  /* Phase 3 (:1214-1269) */
  if (ln_bt_fw) {
    OMP_FOR
    for (size_t p = 0; p < n2; ++p) {
      zwx[p] = un_adv[p];
      zwy[p] = vn_adv[p];
      if (!(kt == nm->nit000 && nm->neuler == 0)) {
        un_adv[p] = r1_2 * (ub2_b[p] + zwx[p] - nm->rn_atfp * un_bf[p]);
        vn_adv[p] = r1_2 * (vb2_b[p] + zwy[p] - nm->rn_atfp * vn_bf[p]);
        un_bf[p] = nm->rn_atfp * un_bf[p] + (zwx[p] - ub2_b[p]);
        vn_bf[p] = nm->rn_atfp * vn_bf[p] + (zwy[p] - vb2_b[p]);
      } else {
        un_bf[p] = 0.0;
        vn_bf[p] = 0.0;
      }
      ub2_b[p] = zwx[p];
      vb2_b[p] = zwy[p];
    }
  }
  if (!flux) {  /* (:1233-1240) */
    OMP_FOR
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (size_t p = 0; p < n2; ++p) {
        size_t q = p + n2 * (jk - 1);
        ua[q] = ua[q] + (ua_b[p] - ub_b[p]) * r1_2dt_b;
        va[q] = va[q] + (va_b[p] - vb_b[p]) * r1_2dt_b;
      }
  } else {     /* (:1241-1262) */
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj);
        zsshu_a[p] = r1_2 * ssumask[p] * c->r1_e1e2u[p] * (c->e1e2t[p] * ssha[p] + c->e1e2t[I2(ji + 1, jj)] * ssha[I2(ji + 1, jj)]);
        zsshv_a[p] = r1_2 * ssvmask[p] * c->r1_e1e2v[p] * (c->e1e2t[p] * ssha[p] + c->e1e2t[I2(ji, jj + 1)] * ssha[I2(ji, jj + 1)]);
      }
    lbc_closed(jpi, jpj, zsshu_a, 1, 'U', 0.0);
    lbc_closed(jpi, jpj, zsshv_a, 1, 'V', 0.0);
    OMP_FOR
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (size_t p = 0; p < n2; ++p) {
        size_t q = p + n2 * (jk - 1);
        ua[q] = ua[q] + r1_hu_n[p] * (ua_b[p] - ub_b[p] * hu_b[p]) * r1_2dt_b;
        va[q] = va[q] + r1_hv_n[p] * (va_b[p] - vb_b[p] * hv_b[p]) * r1_2dt_b;
      }
    for (size_t p = 0; p < n2; ++p) {
      ua_b[p] = ua_b[p] / (c->hu_0[p] + zsshu_a[p] + 1.0 - ssumask[p]);
      va_b[p] = va_b[p] / (c->hv_0[p] + zsshv_a[p] + 1.0 - ssvmask[p]);
    }
  }
  OMP_FOR
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      size_t q = p + n2 * (jk - 1);
      un[q] = (un[q] + un_adv[p] * r1_hu_n[p] - un_b[p]) * umask[q];
      vn[q] = (vn[q] + vn_adv[p] * r1_hv_n[p] - vn_b[p]) * vmask[q];
    }
  wfree(zu_frc); wfree(zv_frc); wfree(zu_trd); wfree(zv_trd); wfree(zwx); wfree(zwy); wfree(zssh_frc); wfree(zhdiv);
  wfree(zsshp2_e); wfree(zCdU_u); wfree(zCdU_v);
  wfree(zhup2_e); wfree(zhvp2_e); wfree(zhtp2_e); wfree(zsshu_a); wfree(zsshv_a); wfree(zhust_e); wfree(zhvst_e);
  return NEMO_OK;
}

/* ---------------------------------------------------------------- glob_sum */
/* DDPDD, lib_fortran.F90:300-332 */
static void ddpdd(double a_re, double *b_re, double *b_im) {
  double zt1 = a_re + *b_re;
  double zerr = zt1 - a_re;
  double zt2 = ((*b_re - zerr) + (a_re - (zt1 - zerr))) + 0.0 + *b_im;
  double s = zt1 + zt2;
  *b_im = zt2 - ((zt1 + zt2) - zt1);
  *b_re = s;
}

/* lib_fortran_generic.h90:32-65 (OPERATION_GLOBSUM: mask tmask_i) */
int ora_glob_sum(ora_ctx *c, const double *ptab, int nk, double *out) {
  const int jpi = c->jpi, jpj = c->jpj;
  double re = 0.0, im = 0.0;
  for (int jk = 1; jk <= nk; ++jk)
    for (int jj = 1; jj <= jpj; ++jj)
      for (int ji = 1; ji <= jpi; ++ji) {
        double ztmp = ptab[I2(ji, jj) + (size_t)jpi * jpj * (jk - 1)] * c->tmask_i[I2(ji, jj)];
        ddpdd(ztmp, &re, &im);
      }
  *out = re;
  return NEMO_OK;
}

/* the shared sines and cosine (nemo_sin.h), exported for their accuracy tests */
double ora_sin_0pi(double x) { return nemo_sin_0pi(x); }
double ora_sin(double x) { return nemo_sin(x); }
double ora_cos(double x) { return nemo_cos(x); }

/* ---------------------------------------------------------------- usrdef_sbc */
/* GYRE's analytic surface forcing, usrdef_sbc_oce (usrdef_sbc.F90:62-190) at time
 * step kt, year 1 of a 360-day calendar, preceded by sbc's swap of the before fields
 * (sbcmod.F90:389-394) when kt /= nit000 and they are bound: qsr and the restoring
 * qns from the before SST, E-P (its domain mean removed, GLOB_SUM) and its heat
 * content at the now SST (sst_m of sbc_ssm with nn_fsbc = 1), sfx = 0, the wind
 * stress and its modulus taum (interior, closed lbc_lnk). SIN and COS are the shared
 * evaluations of nemo_sin.h. Bound: GPHIT GPHIU GPHIV TSB TSN, QSR QNS EMP SFX UTAU
 * VTAU TAUM; UTAU_B VTAU_B EMP_B optional. */
int ora_usrdef_sbc(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj;
  const size_t n2 = (size_t)jpi * jpj;
  double **F = c->f;
  const double *gphit = F[NEMO_F_GPHIT], *gphiu = F[NEMO_F_GPHIU], *gphiv = F[NEMO_F_GPHIV];
  const double *tsb = F[NEMO_F_TSB], *tsn = F[NEMO_F_TSN];
  double *qsr = F[NEMO_F_QSR], *qns = F[NEMO_F_QNS], *emp = F[NEMO_F_EMP], *sfx = F[NEMO_F_SFX];
  double *utau = F[NEMO_F_UTAU], *vtau = F[NEMO_F_VTAU], *taum = F[NEMO_F_TAUM];
  if (!gphit || !gphiu || !gphiv || !tsb || !tsn || !qsr || !qns || !emp || !sfx || !utau || !vtau || !taum)
    return NEMO_ERR_UNBOUND;
  if (kt != nm->nit000) {  /* sbcmod.F90:389-394 */
    if (F[NEMO_F_UTAU_B]) memcpy(F[NEMO_F_UTAU_B], utau, n2 * sizeof(double));
    if (F[NEMO_F_VTAU_B]) memcpy(F[NEMO_F_VTAU_B], vtau, n2 * sizeof(double));
    if (F[NEMO_F_EMP_B]) memcpy(F[NEMO_F_EMP_B], emp, n2 * sizeof(double));
  }
  const double rpi = 3.141592653589793, rcp = nm->rcp > 0 ? nm->rcp : 3991.86795711963;
  const double zyydd = 360.0, rjjhh = 24.0;
  const double ztime = (double)kt * nm->rn_rdt / (60.0 * 60.0);  /* hours; year 1: no years to subtract */
  const double ztimemax1 = ((5. * 30.) + 21.) * 24., ztimemin1 = ztimemax1 + rjjhh * zyydd / 2;
  const double ztimemax2 = ((6. * 30.) + 21.) * 24., ztimemin2 = ztimemax2 - rjjhh * zyydd / 2;
  const double zemp_S = 0.7, zemp_N = 0.8, zemp_sais = 0.1, zTstar = 28.3;
  const double zcos_sais1 = nemo_cos((ztime - ztimemax1) / (ztimemin1 - ztimemax1) * rpi);
  const double zcos_sais2 = nemo_cos((ztime - ztimemax2) / (ztimemax2 - ztimemin2) * rpi);
  const double ztrp = -40.e0, zconv = 3.16e-5;
  for (size_t p = 0; p < n2; ++p) {  /* (:113-135) */
    const double g = gphit[p];
    const double t_star = zTstar * (1. + 1. / 50. * zcos_sais2) * nemo_cos(rpi * (g - 5.) / (53.5 * (1 + 11 / 53.5 * zcos_sais2) * 2.));
    qsr[p] = 230 * nemo_cos(3.1415 * (g - 23.5 * zcos_sais1) / (0.9 * 180));
    qns[p] = ztrp * (tsb[p] - t_star) - qsr[p];
    if (g >= 14.845 && 37.2 >= g)
      emp[p] = zemp_S * zconv * nemo_sin(rpi / 2 * (g - 37.2) / (24.6 - 37.2)) * (1 - zemp_sais / zemp_S * zcos_sais1);
    else
      emp[p] = -zemp_N * zconv * nemo_sin(rpi / 2 * (g - 37.2) / (46.8 - 37.2)) * (1 - zemp_sais / zemp_N * zcos_sais1);
  }
  double zsumemp, zsurf;  /* (:137-139) */
  ora_glob_sum(c, emp, 1, &zsumemp);
  ora_glob_sum(c, c->tmask, 1, &zsurf);
  zsumemp = zsumemp / zsurf;
  for (size_t p = 0; p < n2; ++p) {  /* (:142-144) */
    emp[p] = emp[p] - zsumemp * c->tmask[p];
    sfx[p] = 0.0;
    qns[p] = qns[p] - emp[p] * tsn[p] * rcp;
  }
  /* the wind stress (:160-172) and its modulus (:176-186) */
  const double ztimemax = ((5. * 30.) + 21.) * 24., ztimemin = ztimemax + rjjhh * zyydd / 2;
  const double ztau = 0.105 / sqrt(2.), ztau_sais = 0.015;
  const double ztaun = ztau - ztau_sais * nemo_cos((ztime - ztimemax) / (ztimemin - ztimemax) * rpi);
  for (size_t p = 0; p < n2; ++p) {
    utau[p] = -ztaun * nemo_sin(rpi * (gphiu[p] - 15.) / (29. - 15.));
    vtau[p] = ztaun * nemo_sin(rpi * (gphiv[p] - 15.) / (29. - 15.));
  }
  for (size_t p = 0; p < n2; ++p) taum[p] = 0.0;
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      const double ztx = utau[I2(ji - 1, jj)] + utau[I2(ji, jj)];
      const double zty = vtau[I2(ji, jj - 1)] + vtau[I2(ji, jj)];
      taum[I2(ji, jj)] = 0.5 * sqrt(ztx * ztx + zty * zty);
    }
  return NEMO_OK;
}

/* ---------------------------------------------------------------- zdf_phy */
/* zdf_phy (zdfphy.F90:243-291) for the TKE closure: zdf_sh2 (zdfsh2.F90:30-76)
 * with the closure's avm_k, zdf_tke = tke_tke + tke_avn (zdftke.F90:168-630) for
 * ln_drg = .false., no ice-shelf cavities and nn_etau = 0 (GYRE), then avt, avm
 * from the closure on levels 2..jpk-1, zdf_evd (zdfevd.F90:40-121) and avs = avt.
 * Bound: UB VB UN VN, AVM_K AVT_K AVM AVT (and AVS), EN DISSL (restart fields; a
 * cold start sets en = rn_emin wmask, dissl = 1e-12), RN2 RN2B, TAUM, GDEPW_N; FR_I
 * optional (0). The rest-state e3uw/e3vw are the minima of the neighbouring e3w_0
 * (equal to e3w_0 on full steps, usrdef_zgr.F90:241-242). The five coefficients get
 * the closed lbc_lnk of a W-point field at the end. */
int ora_zdf_phy(ora_ctx *c, int kt) {
  (void)kt;
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  double *ub = c->f[NEMO_F_UB], *vb = c->f[NEMO_F_VB], *un = c->f[NEMO_F_UN], *vn = c->f[NEMO_F_VN];
  double *avm_k = c->f[NEMO_F_AVM_K], *avt_k = c->f[NEMO_F_AVT_K], *avm = c->f[NEMO_F_AVM], *avt = c->f[NEMO_F_AVT];
  double *avs = c->f[NEMO_F_AVS], *en = c->f[NEMO_F_EN], *dissl = c->f[NEMO_F_DISSL];
  const double *rn2 = c->f[NEMO_F_RN2], *rn2b = c->f[NEMO_F_RN2B], *taum = c->f[NEMO_F_TAUM];
  const double *pdepw = c->f[NEMO_F_GDEPW_N], *fr_i = c->f[NEMO_F_FR_I];
  if (!ub || !vb || !un || !vn || !avm_k || !avt_k || !avm || !avt || !en || !dissl || !rn2 || !rn2b || !taum || !pdepw)
    return NEMO_ERR_UNBOUND;
  if (!nm->ln_zdftke || nm->nn_etau != 0 || nm->ln_drg_tke || nm->ln_isfcav || !nm->ln_linssh)
    return NEMO_ERR_UNSUPPORTED;
  const double *e3t = fld(c, NEMO_F_E3T_N), *e3w = fld(c, NEMO_F_E3W_N);
  const double *tmask = c->tmask, *wmask = c->wmask, *umask = c->umask, *vmask = c->vmask;
  const double rdt = nm->rn_rdt, rau0 = nm->rau0, grav = nm->grav;
  const double rpi = 3.141592653589793, vkarmn = 0.4, rsmall = 0.5 * 2.220446049250313e-16;
  const double ri_cri = 2.0 / (2.0 + nm->rn_ediss / nm->rn_ediff);
  const double rmxl_min = 1.e-6 / (nm->rn_ediff * sqrt(nm->rn_emin));
  const double rn_mxl0 = nm->ln_mxl0 ? rmxl_min : nm->rn_mxl0;
  double *sh2 = zalloc(n3), *apdlr = zalloc(n3), *zdiag = zalloc(n3), *zd_up = zalloc(n3), *zd_lw = zalloc(n3);
  double *zpelc = zalloc(n3), *zmxlm = zalloc(n3), *zmxld = zalloc(n3), *zhlc = zalloc(n2), *zfr_i = zalloc(n2);
  double *zsh2u = zalloc(n2), *zsh2v = zalloc(n2);
#define E3UW(ji, jj, jk) dmin(e3w[I3(ji, jj, jk)], e3w[I3((ji) + 1, jj, jk)])
#define E3VW(ji, jj, jk) dmin(e3w[I3(ji, jj, jk)], e3w[I3(ji, (jj) + 1, jk)])
#define WUM(ji, jj, jk) (umask[I3(ji, jj, jk)] * umask[I3(ji, jj, (jk) - 1)])
#define WVM(ji, jj, jk) (vmask[I3(ji, jj, jk)] * vmask[I3(ji, jj, (jk) - 1)])
  /* zdf_sh2 (zdfsh2.F90:57-74), p_avm = avm_k */
  for (int jk = 2; jk <= jpk - 1; ++jk) {
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        zsh2u[I2(ji, jj)] = (avm_k[I3(ji + 1, jj, jk)] + avm_k[I3(ji, jj, jk)]) *
                            (un[I3(ji, jj, jk - 1)] - un[I3(ji, jj, jk)]) *
                            (ub[I3(ji, jj, jk - 1)] - ub[I3(ji, jj, jk)]) / (E3UW(ji, jj, jk) * E3UW(ji, jj, jk)) *
                            WUM(ji, jj, jk);
        zsh2v[I2(ji, jj)] = (avm_k[I3(ji, jj + 1, jk)] + avm_k[I3(ji, jj, jk)]) *
                            (vn[I3(ji, jj, jk - 1)] - vn[I3(ji, jj, jk)]) *
                            (vb[I3(ji, jj, jk - 1)] - vb[I3(ji, jj, jk)]) / (E3VW(ji, jj, jk) * E3VW(ji, jj, jk)) *
                            WVM(ji, jj, jk);
      }
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji)
        sh2[I3(ji, jj, jk)] =
            0.25 * ((zsh2u[I2(ji - 1, jj)] + zsh2u[I2(ji, jj)]) * (2. - umask[I3(ji - 1, jj, jk)] * umask[I3(ji, jj, jk)]) +
                    (zsh2v[I2(ji, jj - 1)] + zsh2v[I2(ji, jj)]) * (2. - vmask[I3(ji, jj - 1, jk)] * vmask[I3(ji, jj, jk)]));
  }
  /* ---- tke_tke (zdftke.F90:168-440), p_avm = avm_k, p_avt = avt_k */
  const double zbbrau = nm->rn_ebb / rau0, zfact1 = -.5 * rdt, zfact2 = 1.5 * rdt * nm->rn_ediss;
  const double zfact3 = 0.5 * nm->rn_ediss;
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji)
      en[I3(ji, jj, 1)] = dmax(nm->rn_emin0, zbbrau * taum[I2(ji, jj)]) * tmask[I3(ji, jj, 1)];
  if (nm->ln_lc) {  /* Langmuir circulation (:243-311) */
    const double zrhoa = 1.22, zcdrag = 1.5e-3;
    for (size_t p = 0; p < n2; ++p) zpelc[p] = dmax(rn2b[p], 0.) * pdepw[p] * e3w[p];
    for (int jk = 2; jk <= jpk; ++jk)
      for (size_t p = 0; p < n2; ++p) {
        const size_t q = p + n2 * (jk - 1);
        zpelc[q] = zpelc[q - n2] + dmax(rn2b[q], 0.) * pdepw[q] * e3w[q];
      }
    double zcof = 0.5 * 0.016 * 0.016 / (zrhoa * zcdrag);
    for (size_t p = 0; p < n2; ++p) {
      int imlc = c->mbkt[p] + 1;
      for (int jk = jpk - 1; jk >= 2; --jk) {
        const double zus = zcof * taum[p];
        if (zpelc[p + n2 * (jk - 1)] > zus) imlc = jk;
      }
      zhlc[p] = pdepw[p + n2 * (imlc - 1)];
    }
    zcof = 0.016 / sqrt(zrhoa * zcdrag);
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj);
        const double zus = zcof * sqrt(taum[p]);
        zfr_i[p] = (1. - 4. * (fr_i ? fr_i[p] : 0.)) * zus * zus * zus * tmask[p];
        if (zfr_i[p] < 0.) zfr_i[p] = 0.;
      }
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t p = I2(ji, jj), q = I3(ji, jj, jk);
          if (zfr_i[p] != 0.) {
            if (pdepw[q] - zhlc[p] < 0 && wmask[q] != 0.) {
              /* SIN by the evaluation the CUDA kernels share (nemo_sin.h) */
              const double zwlc = nm->rn_lc * nemo_sin_0pi(rpi * pdepw[q] / zhlc[p]);
              en[q] = en[q] + rdt * zfr_i[p] * (zwlc * zwlc * zwlc) / zhlc[p];
            }
          }
        }
  }
  if (nm->nn_pdl == 1)  /* (:323-334) */
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          const double zri = dmax(rn2b[q], 0.) * avm_k[q] / (sh2[q] + nm->rn_bshear);
          apdlr[q] = dmax(0.1, ri_cri / dmax(ri_cri, zri));
        }
  for (int jk = 2; jk <= jpk - 1; ++jk)  /* matrix and right-hand side (:336-356) */
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jk);
        const double zcof = zfact1 * tmask[q];
        const double zzd_up = zcof * dmax(avm_k[q + n2] + avm_k[q], 2.e-5) / (e3t[q] * e3w[q]);
        const double zzd_lw = zcof * dmax(avm_k[q] + avm_k[q - n2], 2.e-5) / (e3t[q - n2] * e3w[q]);
        zd_up[q] = zzd_up;
        zd_lw[q] = zzd_lw;
        zdiag[q] = 1. - zzd_lw - zzd_up + zfact2 * dissl[q] * wmask[q];
        en[q] = en[q] + rdt * (sh2[q] - avt_k[q] * rn2[q] + zfact3 * dissl[q] * en[q]) * wmask[q];
      }
  for (int jk = 3; jk <= jpk - 1; ++jk)  /* recurrences (:358-390) */
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jk);
        zdiag[q] = zdiag[q] - zd_lw[q] * zd_up[q - n2] / zdiag[q - n2];
      }
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji)
      zd_lw[I3(ji, jj, 2)] = en[I3(ji, jj, 2)] - zd_lw[I3(ji, jj, 2)] * en[I3(ji, jj, 1)];
  for (int jk = 3; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jk);
        zd_lw[q] = en[q] - zd_lw[q] / zdiag[q - n2] * zd_lw[q - n2];
      }
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji)
      en[I3(ji, jj, jpk - 1)] = zd_lw[I3(ji, jj, jpk - 1)] / zdiag[I3(ji, jj, jpk - 1)];
  for (int jk = jpk - 2; jk >= 2; --jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jk);
        en[q] = (zd_lw[q] - zd_up[q] * en[q + n2]) / zdiag[q];
      }
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jk);
        en[q] = dmax(en[q], nm->rn_emin) * wmask[q];
      }
  /* ---- tke_avn (zdftke.F90:443-630) */
  for (size_t q = 0; q < n3; ++q) { zmxlm[q] = rmxl_min; zmxld[q] = rmxl_min; }
  if (nm->ln_mxl0) {
    const double zraug = vkarmn * 2.e5 / (rau0 * grav);
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji)
        zmxlm[I2(ji, jj)] = dmax(rn_mxl0, zraug * taum[I2(ji, jj)] * tmask[I2(ji, jj)]);
  } else {
    for (size_t p = 0; p < n2; ++p) zmxlm[p] = rn_mxl0;
  }
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jk);
        const double zrn2 = dmax(rn2[q], rsmall);
        zmxlm[q] = dmax(rmxl_min, sqrt(2. * en[q] / zrn2));
      }
  for (size_t p = 0; p < n2; ++p) { zmxld[p] = zmxlm[p]; zmxld[p + n2 * (jpk - 1)] = rmxl_min; }
  switch (nm->nn_mxl) {
    case 0:
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            const size_t p = I2(ji, jj), q = I3(ji, jj, jk);
            const double a = pdepw[q] - pdepw[p + n2 * (c->mikt[p] - 1)], b = pdepw[p + n2 * c->mbkt[p]] - pdepw[q];
            const double zemxl = dmin(dmin(a, zmxlm[q]), b);
            zmxlm[q] = zemxl * wmask[q] + dmin(zmxlm[q], e3w[q]) * (1 - wmask[q]);
            zmxld[q] = zemxl * wmask[q] + dmin(zmxlm[q], e3w[q]) * (1 - wmask[q]);
          }
      break;
    case 1:
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            const size_t q = I3(ji, jj, jk);
            const double zemxl = dmin(e3w[q], zmxlm[q]);
            zmxlm[q] = zemxl;
            zmxld[q] = zemxl;
          }
      break;
    case 2:
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            const size_t q = I3(ji, jj, jk);
            zmxlm[q] = dmin(zmxlm[q - n2] + e3t[q - n2], zmxlm[q]);
          }
      for (int jk = jpk - 1; jk >= 2; --jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            const size_t q = I3(ji, jj, jk);
            const double zemxl = dmin(zmxlm[q + n2] + e3t[q + n2], zmxlm[q]);
            zmxlm[q] = zemxl;
            zmxld[q] = zemxl;
          }
      break;
    default:  /* 3 */
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            const size_t q = I3(ji, jj, jk);
            zmxld[q] = dmin(zmxld[q - n2] + e3t[q - n2], zmxlm[q]);
          }
      for (int jk = jpk - 1; jk >= 2; --jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            const size_t q = I3(ji, jj, jk);
            zmxlm[q] = dmin(zmxlm[q + n2] + e3t[q + n2], zmxlm[q]);
          }
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            const size_t q = I3(ji, jj, jk);
            const double zemlm = dmin(zmxld[q], zmxlm[q]), zemlp = sqrt(zmxld[q] * zmxlm[q]);
            zmxlm[q] = zemlm;
            zmxld[q] = zemlp;
          }
      break;
  }
  for (int jk = 1; jk <= jpk - 1; ++jk)  /* avm_k, avt_k, dissl (:610-620), nn_avb = nn_havtb = 0 */
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jk);
        const double zsqen = sqrt(en[q]);
        const double zav = nm->rn_ediff * zmxlm[q] * zsqen;
        avm_k[q] = dmax(zav, nm->rn_avm0) * wmask[q];
        avt_k[q] = dmax(zav, 1.0 * nm->rn_avt0) * wmask[q];
        dissl[q] = zsqen / zmxld[q];
      }
  if (nm->nn_pdl == 1)
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          avt_k[q] = dmax(apdlr[q] * avt_k[q], 1.0 * nm->rn_avt0) * tmask[q];
        }
  /* ---- zdf_phy: ocean Kz from the closure (zdfphy.F90:269-291) */
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      const size_t q = p + n2 * (jk - 1);
      avt[q] = avt_k[q];
      avm[q] = avm_k[q];
    }
  if (nm->ln_zdfevd)  /* zdfevd.F90:76-109 */
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          if (dmin(rn2[q], rn2b[q]) <= -1.e-12) {
            avt[q] = nm->rn_evd * wmask[q];
            if (nm->nn_evdm == 1) avm[q] = nm->rn_evd * wmask[q];
          }
        }
  if (avs)
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) avs[I3(ji, jj, jk)] = avt[I3(ji, jj, jk)];
  /* closed lateral boundaries of the five coefficients (zdfphy.F90:301-303) */
  lbc_closed(jpi, jpj, avm_k, jpk, 'W', 0.0);
  lbc_closed(jpi, jpj, avt_k, jpk, 'W', 0.0);
  lbc_closed(jpi, jpj, avm, jpk, 'W', 0.0);
  lbc_closed(jpi, jpj, avt, jpk, 'W', 0.0);
  if (avs) lbc_closed(jpi, jpj, avs, jpk, 'W', 0.0);
#undef E3UW
#undef E3VW
#undef WUM
#undef WVM
  wfree(sh2); wfree(apdlr); wfree(zdiag); wfree(zd_up); wfree(zd_lw); wfree(zpelc); wfree(zmxlm); wfree(zmxld);
  wfree(zhlc); wfree(zfr_i); wfree(zsh2u); wfree(zsh2v);
  return NEMO_OK;
}

/* ---------------------------------------------------------------- stp_ctl */
/* stp_ctl (stpctl.F90:44-194), the test of extrema (:112-127) and the blow-up
 * conditions (:149-157): zmax = |ssh| max, |U| max (zonal, every point), then the
 * maxima of -S, S, -T, T over tmask = 1. MAXVAL of values that include a NaN is
 * taken as NaN here (the NaN test of :155 then fires). On a blow-up the positions
 * (:158-170) are MAXLOC(|ssh|), MAXLOC(|un|), MINLOC(S), MAXLOC(S) (1-based, first
 * in Fortran order; a NaN counts as the extreme) and kindic = -3 (:184). */
int ora_stp_ctl(ora_ctx *c, int kt, double *zmax, int *loc, int *kindic) {
  (void)kt;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const double *sshn = c->f[NEMO_F_SSHN], *un = c->f[NEMO_F_UN], *ts = c->f[NEMO_F_TSN];
  if (!sshn || !un || !ts || !zmax) return NEMO_ERR_UNBOUND;
  const double huge = 1.7976931348623157e308;
  int lsomeoce = 0;
  for (size_t p = 0; p < n2; ++p) lsomeoce |= c->ssmask[p] == 1.0;
  double z[6] = {-huge, -huge, -huge, -huge, -huge, -huge};
  int nan1 = 0, nan2 = 0, nan3 = 0;
  for (size_t p = 0; p < n2; ++p) {
    const double v = fabs(sshn[p]);
    if (isnan(v)) nan1 = 1; else if (v > z[0]) z[0] = v;
  }
  for (size_t q = 0; q < n3; ++q) {
    const double v = fabs(un[q]);
    if (isnan(v)) nan2 = 1; else if (v > z[1]) z[1] = v;
    if (c->tmask[q] == 1.0) {
      const double sv = ts[q + n3], tv = ts[q];
      if (isnan(sv)) nan3 = 1;
      else { if (-sv > z[2]) z[2] = -sv; if (sv > z[3]) z[3] = sv; }
      if (!isnan(tv)) { if (-tv > z[4]) z[4] = -tv; if (tv > z[5]) z[5] = tv; }
    }
  }
  if (nan1) z[0] = NAN;
  if (nan2) z[1] = NAN;
  if (nan3) { z[2] = NAN; z[3] = NAN; }
  for (int i = 0; i < 6; ++i) zmax[i] = z[i];
  const int trip = lsomeoce && (z[0] > 20.0 || z[1] > 10.0 || z[2] >= 0.0 || z[3] >= 100.0 || z[3] < 0.0 ||
                                isnan(z[0] + z[1] + z[2]));
  if (kindic) *kindic = trip ? -3 : 0;
  if (loc) {
    for (int i = 0; i < NEMO_CTL_NLOC; ++i) loc[i] = 0;
    if (trip) {
      size_t best = 0;
      double bv = -INFINITY;
      for (size_t p = 0; p < n2; ++p) {  /* MAXLOC(ABS(sshn)) */
        const double v = isnan(sshn[p]) ? INFINITY : fabs(sshn[p]);
        if (v > bv) { bv = v; best = p; }
      }
      loc[0] = (int)(best % jpi) + 1; loc[1] = (int)(best / jpi) + 1;
      best = 0; bv = -INFINITY;
      for (size_t q = 0; q < n3; ++q) {  /* MAXLOC(ABS(un)) */
        const double v = isnan(un[q]) ? INFINITY : fabs(un[q]);
        if (v > bv) { bv = v; best = q; }
      }
      loc[2] = (int)(best % jpi) + 1; loc[3] = (int)((best / jpi) % jpj) + 1; loc[4] = (int)(best / n2) + 1;
      size_t bmin = 0, bmax = 0;
      double vmin = INFINITY, vmax = -INFINITY;
      int any = 0;
      for (size_t q = 0; q < n3; ++q) {  /* MINLOC / MAXLOC(S, mask = tmask == 1) */
        if (c->tmask[q] != 1.0) continue;
        const double sv = ts[q + n3];
        const double lo = isnan(sv) ? -INFINITY : sv, hi = isnan(sv) ? INFINITY : sv;
        if (!any || lo < vmin) { vmin = lo; bmin = q; }
        if (!any || hi > vmax) { vmax = hi; bmax = q; }
        any = 1;
      }
      if (any) {
        loc[5] = (int)(bmin % jpi) + 1; loc[6] = (int)((bmin / jpi) % jpj) + 1; loc[7] = (int)(bmin / n2) + 1;
        loc[8] = (int)(bmax % jpi) + 1; loc[9] = (int)((bmax / jpi) % jpj) + 1; loc[10] = (int)(bmax / n2) + 1;
      }
    }
  }
  return NEMO_OK;
}

/* ---------------------------------------------------------------- dia_hsb */
static double gsum(const ora_ctx *c, const double *x, int nk, const double *mask) {
  const size_t n2 = (size_t)c->jpi * c->jpj;
  double re = 0.0, im = 0.0;
  for (int jk = 0; jk < nk; ++jk)
    for (size_t p = 0; p < n2; ++p) ddpdd(x[p + n2 * jk] * mask[p], &re, &im);
  return re;
}

/* dia_hsb_init (diahsb.F90:411-412) and dia_hsb_rst( nit000, 'READ' ) without a
 * restart (:283-311): the masked cell area, the initial ssh, scale factors, heat and
 * salt contents, and zero forcing sums. */
int ora_dia_hsb_init(ora_ctx *c) {
  const int jpk = c->jpk;
  const size_t n2 = (size_t)c->jpi * c->jpj, n3 = n2 * jpk;
  const double *sshn = c->f[NEMO_F_SSHN], *ts = c->f[NEMO_F_TSN];
  if (!sshn || !ts) return NEMO_ERR_UNBOUND;
  const double *e3t = fld(c, NEMO_F_E3T_N);
  if (!c->surf) {
    c->surf = zalloc(n2); c->surf_ini = zalloc(n2); c->ssh_ini = zalloc(n2);
    c->ssh_hc_loc_ini = zalloc(n2); c->ssh_sc_loc_ini = zalloc(n2);
    c->e3t_ini = zalloc(n3); c->hc_loc_ini = zalloc(n3); c->sc_loc_ini = zalloc(n3);
  }
  for (size_t p = 0; p < n2; ++p) c->surf[p] = c->e1e2t[p] * c->tmask_i[p];
  c->surf_tot = gsum(c, c->surf, 1, c->tmask_i);
  for (size_t p = 0; p < n2; ++p) {
    c->surf_ini[p] = c->e1e2t[p] * c->tmask_i[p];
    c->ssh_ini[p] = sshn[p];
  }
  for (size_t q = 0; q < n3; ++q) {
    c->e3t_ini[q] = e3t[q] * c->tmask[q];
    c->hc_loc_ini[q] = ts[q] * e3t[q] * c->tmask[q];
    c->sc_loc_ini[q] = ts[q + n3] * e3t[q] * c->tmask[q];
  }
  c->frc_v = c->frc_t = c->frc_s = 0.0;
  if (c->nam.ln_linssh) {
    for (size_t p = 0; p < n2; ++p) {
      c->ssh_hc_loc_ini[p] = ts[p] * sshn[p];
      c->ssh_sc_loc_ini[p] = ts[p + n3] * sshn[p];
    }
    c->frc_wn_t = c->frc_wn_s = 0.0;
  }
  c->hsb_on = 1;
  return NEMO_OK;
}

/* dia_hsb (diahsb.F90:60-239) without runoff, ice-shelf and geothermal inputs
 * (ln_rnf, ln_isf, ln_trabbc off; rnf enters the volume flux where bound): the
 * forcing sums (:93-123), the content variations (:130-169), the drifts (:174-185)
 * and the total volume (:190-193). out[NEMO_HSB_N] = frc_v, frc_t, frc_s, frc_wn_t,
 * frc_wn_s, zdiff_v1, zdiff_v2, zdiff_hc, zdiff_sc, zdiff_hc1, zdiff_sc1, zerr_hc1,
 * zerr_sc1, zvol_tot, surf_tot (the last four of the first group of the linear free
 * surface only, else 0). tsn and tsb are masked in place (:88-89). */
int ora_dia_hsb(ora_ctx *c, int kt, double *out) {
  (void)kt;
  const int jpk = c->jpk;
  const size_t n2 = (size_t)c->jpi * c->jpj, n3 = n2 * jpk;
  double *tsn = c->f[NEMO_F_TSN], *tsb = c->f[NEMO_F_TSB];
  const double *sshn = c->f[NEMO_F_SSHN], *emp = c->f[NEMO_F_EMP], *rnf = c->f[NEMO_F_RNF];
  const double *tsc = c->f[NEMO_F_SBC_TSC], *qsr = c->f[NEMO_F_QSR], *wn = c->f[NEMO_F_WN];
  if (!c->hsb_on) return NEMO_ERR_STATE;
  if (!tsn || !tsb || !sshn || !emp || !tsc || !wn || (c->nam.ln_traqsr && !qsr)) return NEMO_ERR_UNBOUND;
  const double *e3t = fld(c, NEMO_F_E3T_N);
  const double rdt = c->nam.rn_rdt, rau0 = c->nam.rau0;
  const double rcp = c->nam.rcp > 0 ? c->nam.rcp : 3991.86795711963;
  const double r1_rau0 = 1.0 / rau0, r1_rau0_rcp = 1.0 / (rau0 * rcp);
  for (size_t q = 0; q < n3; ++q) {
    tsn[q] = tsn[q] * c->tmask[q]; tsb[q] = tsb[q] * c->tmask[q];
    tsn[q + n3] = tsn[q + n3] * c->tmask[q]; tsb[q + n3] = tsb[q + n3] * c->tmask[q];
  }
  double *z2d0 = walloc(n2), *z2d1 = walloc(n2), *zwrk = walloc(n2 * (jpk - 1));
  /* 1 - trends due to forcing */
  for (size_t p = 0; p < n2; ++p) z2d0[p] = -(emp[p] - (rnf ? rnf[p] : 0.0) + 0.0) * c->surf[p];
  const double z_frc_trd_v = r1_rau0 * gsum(c, z2d0, 1, c->tmask_i);
  for (size_t p = 0; p < n2; ++p) z2d0[p] = tsc[p] * c->surf[p];
  double z_frc_trd_t = gsum(c, z2d0, 1, c->tmask_i);
  for (size_t p = 0; p < n2; ++p) z2d0[p] = tsc[p + n2] * c->surf[p];
  const double z_frc_trd_s = gsum(c, z2d0, 1, c->tmask_i);
  if (c->nam.ln_traqsr) {
    for (size_t p = 0; p < n2; ++p) z2d0[p] = qsr[p] * c->surf[p];
    z_frc_trd_t = z_frc_trd_t + r1_rau0_rcp * gsum(c, z2d0, 1, c->tmask_i);
  }
  double z_wn_trd_t = 0.0, z_wn_trd_s = 0.0;
  if (c->nam.ln_linssh) {
    for (size_t p = 0; p < n2; ++p) {
      z2d0[p] = c->surf[p] * wn[p] * tsb[p];
      z2d1[p] = c->surf[p] * wn[p] * tsb[p + n3];
    }
    z_wn_trd_t = -gsum(c, z2d0, 1, c->tmask_i);
    z_wn_trd_s = -gsum(c, z2d1, 1, c->tmask_i);
  }
  c->frc_v = c->frc_v + z_frc_trd_v * rdt;
  c->frc_t = c->frc_t + z_frc_trd_t * rdt;
  c->frc_s = c->frc_s + z_frc_trd_s * rdt;
  if (c->nam.ln_linssh) {
    c->frc_wn_t = c->frc_wn_t + z_wn_trd_t * rdt;
    c->frc_wn_s = c->frc_wn_s + z_wn_trd_s * rdt;
  }
  /* 2 - content variations (glob_sum_full: mask tmask_h) */
  for (size_t p = 0; p < n2; ++p) z2d0[p] = c->surf[p] * sshn[p] - c->surf_ini[p] * c->ssh_ini[p];
  double zdiff_v1 = gsum(c, z2d0, 1, c->tmask_h);
  double z_ssh_hc = 0.0, z_ssh_sc = 0.0;
  if (c->nam.ln_linssh) {
    for (size_t p = 0; p < n2; ++p) {
      z2d0[p] = c->surf[p] * (tsn[p] * sshn[p] - c->ssh_hc_loc_ini[p]);
      z2d1[p] = c->surf[p] * (tsn[p + n3] * sshn[p] - c->ssh_sc_loc_ini[p]);
    }
    z_ssh_hc = gsum(c, z2d0, 1, c->tmask_h);
    z_ssh_sc = gsum(c, z2d1, 1, c->tmask_h);
  }
  for (size_t q = 0; q < n2 * (jpk - 1); ++q) {
    const size_t p = q % n2;
    zwrk[q] = (c->surf[p] * e3t[q] - c->surf_ini[p] * c->e3t_ini[q]) * c->tmask[q];
  }
  double zdiff_v2 = gsum(c, zwrk, jpk - 1, c->tmask_h);
  for (size_t q = 0; q < n2 * (jpk - 1); ++q) {
    const size_t p = q % n2;
    zwrk[q] = (c->surf[p] * e3t[q] * tsn[q] - c->surf_ini[p] * c->hc_loc_ini[q]) * c->tmask[q];
  }
  double zdiff_hc = gsum(c, zwrk, jpk - 1, c->tmask_h);
  for (size_t q = 0; q < n2 * (jpk - 1); ++q) {
    const size_t p = q % n2;
    zwrk[q] = (c->surf[p] * e3t[q] * tsn[q + n3] - c->surf_ini[p] * c->sc_loc_ini[q]) * c->tmask[q];
  }
  double zdiff_sc = gsum(c, zwrk, jpk - 1, c->tmask_h);
  /* 3 - drifts */
  zdiff_v1 = zdiff_v1 - c->frc_v;
  if (!c->nam.ln_linssh) zdiff_v2 = zdiff_v2 - c->frc_v;
  zdiff_hc = zdiff_hc - c->frc_t;
  zdiff_sc = zdiff_sc - c->frc_s;
  double zdiff_hc1 = 0.0, zdiff_sc1 = 0.0, zerr_hc1 = 0.0, zerr_sc1 = 0.0;
  if (c->nam.ln_linssh) {
    zdiff_hc1 = zdiff_hc + z_ssh_hc;
    zdiff_sc1 = zdiff_sc + z_ssh_sc;
    zerr_hc1 = z_ssh_hc - c->frc_wn_t;
    zerr_sc1 = z_ssh_sc - c->frc_wn_s;
  }
  /* 4 - total volume */
  for (size_t q = 0; q < n2 * (jpk - 1); ++q) zwrk[q] = c->surf[q % n2] * e3t[q] * c->tmask[q];
  const double zvol_tot = gsum(c, zwrk, jpk - 1, c->tmask_h);
  wfree(z2d0); wfree(z2d1); wfree(zwrk);
  double *o = c->hsb_out;
  o[0] = c->frc_v; o[1] = c->frc_t; o[2] = c->frc_s; o[3] = c->frc_wn_t; o[4] = c->frc_wn_s;
  o[5] = zdiff_v1; o[6] = zdiff_v2; o[7] = zdiff_hc; o[8] = zdiff_sc; o[9] = zdiff_hc1; o[10] = zdiff_sc1;
  o[11] = zerr_hc1; o[12] = zerr_sc1; o[13] = zvol_tot; o[14] = c->surf_tot; o[15] = 0.0;
  if (out) memcpy(out, o, NEMO_HSB_N * sizeof(double));
  return NEMO_OK;
}

/* the last model step's stp_ctl and dia_hsb */
int ora_stp_ctl_last(const ora_ctx *c, double *zmax, int *loc, int *kindic) {
  if (zmax) memcpy(zmax, c->ctl_zmax, sizeof(c->ctl_zmax));
  if (loc) memcpy(loc, c->ctl_loc, sizeof(c->ctl_loc));
  if (kindic) *kindic = c->ctl_kindic;
  return NEMO_OK;
}
int ora_dia_hsb_last(const ora_ctx *c, double *out) {
  if (!c->hsb_on) return NEMO_ERR_STATE;
  memcpy(out, c->hsb_out, sizeof(c->hsb_out));
  return NEMO_OK;
}

/* ---------------------------------------------------------- one hot-path step */
/* step.F90:194-257 on the bound fields: dyn_spg_ts, tsa = 0, tra_adv (transports
 * + FCT), tra_ldf (iso or lap), tra_zdf. FCT orders from nn_fct_h/v (0 = 2). */
/* zps_hde (zpshde.F90:41-148): the horizontal gradients of the tracers at the last
 * (partial-step) ocean level of u- and v-points, each tracer interpolated to the
 * shallower of the two bottom depths; lbc_lnk. The density part is ora_zps_hde_rd. */
int ora_zps_hde(ora_ctx *c, int kt, int kjpt, const double *pta, double *pgtu, double *pgtv) {
  (void)kt;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const double *e3w = fld(c, NEMO_F_E3W_N), *umask = c->umask, *vmask = c->vmask;
  memset(pgtu, 0, n2 * kjpt * sizeof(double));
  memset(pgtv, 0, n2 * kjpt * sizeof(double));
  for (int jn = 1; jn <= kjpt; ++jn) {
    const double *t = pta + n3 * (jn - 1);
    double *gu = pgtu + n2 * (jn - 1), *gv = pgtv + n2 * (jn - 1);
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj);
        int iku = c->mbku[p], ikum1 = iku - 1 > 1 ? iku - 1 : 1;
        int ikv = c->mbkv[p], ikvm1 = ikv - 1 > 1 ? ikv - 1 : 1;
        double ze3wu = e3w[I3(ji + 1, jj, iku)] - e3w[I3(ji, jj, iku)];
        double ze3wv = e3w[I3(ji, jj + 1, ikv)] - e3w[I3(ji, jj, ikv)];
        if (ze3wu >= 0.0) {
          double zmaxu = ze3wu / e3w[I3(ji + 1, jj, iku)];
          double zti = t[I3(ji + 1, jj, iku)] + zmaxu * (t[I3(ji + 1, jj, ikum1)] - t[I3(ji + 1, jj, iku)]);
          gu[p] = umask[p] * (zti - t[I3(ji, jj, iku)]);
        } else {
          double zmaxu = -ze3wu / e3w[I3(ji, jj, iku)];
          double zti = t[I3(ji, jj, iku)] + zmaxu * (t[I3(ji, jj, ikum1)] - t[I3(ji, jj, iku)]);
          gu[p] = umask[p] * (t[I3(ji + 1, jj, iku)] - zti);
        }
        if (ze3wv >= 0.0) {
          double zmaxv = ze3wv / e3w[I3(ji, jj + 1, ikv)];
          double ztj = t[I3(ji, jj + 1, ikv)] + zmaxv * (t[I3(ji, jj + 1, ikvm1)] - t[I3(ji, jj + 1, ikv)]);
          gv[p] = vmask[p] * (ztj - t[I3(ji, jj, ikv)]);
        } else {
          double zmaxv = -ze3wv / e3w[I3(ji, jj, ikv)];
          double ztj = t[I3(ji, jj, ikv)] + zmaxv * (t[I3(ji, jj, ikvm1)] - t[I3(ji, jj, ikv)]);
          gv[p] = vmask[p] * (t[I3(ji, jj + 1, ikv)] - ztj);
        }
      }
  }
  lbc_closed(jpi, jpj, pgtu, kjpt, 'U', 0.0);
  lbc_closed(jpi, jpj, pgtv, kjpt, 'V', 0.0);
  return NEMO_OK;
}

/* eos_insitu_2d (eosbn2.F90:295-398): the unmasked in situ density anomaly of one
 * (T, S, depth) with EOS-80 or the simplified equation of state */
static double eos_rd_2d(const ora_ctx *c, double t, double sal, double dep);

/* zps_hde's density part (zpshde.F90:150-184): T and S interpolated to the shallower
 * bottom depth of each u- (v-) point as the tracer part does, their density at that
 * depth (gdept_n of the shallower bottom cell) by eos_insitu_2d, its difference with
 * the bound prd of the deeper side; the closed lbc_lnk. pts: T and S (jpi,jpj,jpk,2),
 * out: pgru, pgrv (jpi,jpj). Bound: GDEPT_N. */
int ora_zps_hde_rd(ora_ctx *c, int kt, const double *pts, const double *prd, double *pgru, double *pgrv) {
  (void)kt;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const double *e3w = fld(c, NEMO_F_E3W_N), *gdept = c->f[NEMO_F_GDEPT_N], *umask = c->umask, *vmask = c->vmask;
  if (!pts || !prd || !pgru || !pgrv) return NEMO_ERR_ARG;
  if (!gdept) return NEMO_ERR_UNBOUND;
  if (!c->nam.ln_seos && !c->nam.ln_eos80) return NEMO_ERR_UNSUPPORTED;
  memset(pgru, 0, n2 * sizeof(double));
  memset(pgrv, 0, n2 * sizeof(double));
  for (int jj = 1; jj <= jpj - 1; ++jj)
    for (int ji = 1; ji <= jpi - 1; ++ji) {
      const size_t p = I2(ji, jj);
      const int iku = c->mbku[p], ikum1 = iku - 1 > 1 ? iku - 1 : 1;
      const int ikv = c->mbkv[p], ikvm1 = ikv - 1 > 1 ? ikv - 1 : 1;
      const double ze3wu = e3w[I3(ji + 1, jj, iku)] - e3w[I3(ji, jj, iku)];
      const double ze3wv = e3w[I3(ji, jj + 1, ikv)] - e3w[I3(ji, jj, ikv)];
      double zti[2], ztj[2];
      for (int jn = 0; jn < 2; ++jn) {  /* the tracer part's interpolation (:108-140) */
        const double *t = pts + n3 * jn;
        if (ze3wu >= 0.0) {
          const double zmaxu = ze3wu / e3w[I3(ji + 1, jj, iku)];
          zti[jn] = t[I3(ji + 1, jj, iku)] + zmaxu * (t[I3(ji + 1, jj, ikum1)] - t[I3(ji + 1, jj, iku)]);
        } else {
          const double zmaxu = -ze3wu / e3w[I3(ji, jj, iku)];
          zti[jn] = t[I3(ji, jj, iku)] + zmaxu * (t[I3(ji, jj, ikum1)] - t[I3(ji, jj, iku)]);
        }
        if (ze3wv >= 0.0) {
          const double zmaxv = ze3wv / e3w[I3(ji, jj + 1, ikv)];
          ztj[jn] = t[I3(ji, jj + 1, ikv)] + zmaxv * (t[I3(ji, jj + 1, ikvm1)] - t[I3(ji, jj + 1, ikv)]);
        } else {
          const double zmaxv = -ze3wv / e3w[I3(ji, jj, ikv)];
          ztj[jn] = t[I3(ji, jj, ikv)] + zmaxv * (t[I3(ji, jj, ikvm1)] - t[I3(ji, jj, ikv)]);
        }
      }
      const double zhi = ze3wu >= 0.0 ? gdept[I3(ji, jj, iku)] : gdept[I3(ji + 1, jj, iku)];
      const double zhj = ze3wv >= 0.0 ? gdept[I3(ji, jj, ikv)] : gdept[I3(ji, jj + 1, ikv)];
      /* eos of the interpolated tracers; its lbc_lnk zeroes the edge values, which
         only the edge gradients read and the final lbc_lnk zeroes too */
      const double zri = (ji == 1 || jj == 1) ? 0.0 : eos_rd_2d(c, zti[0], zti[1], zhi);
      const double zrj = (ji == 1 || jj == 1) ? 0.0 : eos_rd_2d(c, ztj[0], ztj[1], zhj);
      pgru[p] = ze3wu >= 0.0 ? umask[p] * (zri - prd[I3(ji, jj, iku)]) : umask[p] * (prd[I3(ji + 1, jj, iku)] - zri);
      pgrv[p] = ze3wv >= 0.0 ? vmask[p] * (zrj - prd[I3(ji, jj, ikv)]) : vmask[p] * (prd[I3(ji, jj + 1, ikv)] - zrj);
    }
  lbc_closed(jpi, jpj, pgru, 1, 'U', 0.0);
  lbc_closed(jpi, jpj, pgrv, 1, 'V', 0.0);
  return NEMO_OK;
}

/* tra_ldf_blp (traldf_lap_blp.F90:161-231): the first laplacian (kldf 20
 * iso-level, 21 rotated) of ptb into zlap, lbc_lnk, with partial steps zps_hde of
 * zlap, the second laplacian of zlap into pta. */
int ora_tra_ldf_blp(ora_ctx *c, int kt, int kit000, const char *cdtype,
                    const double *pahu, const double *pahv,
                    const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                    const double *ptb, double *pta, int kjpt, int kldf) {
  if (kldf != 20 && kldf != 21 && kldf != 22) return NEMO_ERR_UNSUPPORTED;
  if (c->nam.ln_zps && (!pgu || !pgv)) return NEMO_ERR_ARG;
  const size_t n2 = (size_t)c->jpi * c->jpj, n3 = n2 * c->jpk;
  double *zlap = zalloc(n3 * (size_t)kjpt), *zglu = zalloc(n2 * kjpt), *zglv = zalloc(n2 * kjpt);
  int st = kldf == 20 ? ora_tra_ldf_lap(c, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, zlap, kjpt, 1)
         : kldf == 21 ? ora_tra_ldf_iso(c, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, ptb, zlap, kjpt, 1)
                      : ora_tra_ldf_triad(c, kt, kit000, cdtype, pahu, pahv, pgu, pgv, pgui, pgvi, ptb, ptb, zlap, kjpt, 1);
  if (!st) {
    lbc_closed(c->jpi, c->jpj, zlap, c->jpk * kjpt, 'T', 0.0);
    if (c->nam.ln_zps) ora_zps_hde(c, kt, kjpt, zlap, zglu, zglv);   /* GRADh(zlap) at the partial steps */
    st = kldf == 20 ? ora_tra_ldf_lap(c, kt, kit000, cdtype, pahu, pahv, zglu, zglv, NULL, NULL, zlap, pta, kjpt, 2)
       : kldf == 21 ? ora_tra_ldf_iso(c, kt, kit000, cdtype, pahu, pahv, zglu, zglv, NULL, NULL, zlap, ptb, pta, kjpt, 2)
                    : ora_tra_ldf_triad(c, kt, kit000, cdtype, pahu, pahv, zglu, zglv, NULL, NULL, zlap, ptb, pta, kjpt, 2);
  }
  wfree(zlap); wfree(zglu); wfree(zglv);
  return st;
}

/* The tracer part of the step: tsa = 0, tra_adv (transports + FCT), tra_ldf, tra_zdf. */
int ora_tra_sbc(ora_ctx *c, int kt);
int ora_tra_qsr(ora_ctx *c, int kt);
/* The model step runs tra_sbc (and tra_qsr) when the surface forcing is bound. */
static int sbc_bound(const ora_ctx *c) {
  return c->f[NEMO_F_QNS] && c->f[NEMO_F_QSR] && c->f[NEMO_F_SFX] && c->f[NEMO_F_SBC_TSC] && c->f[NEMO_F_SBC_TSC_B];
}

static int stp_tracers(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  const size_t n3 = (size_t)c->jpi * c->jpj * c->jpk;
  double *tsb = c->f[NEMO_F_TSB], *tsn = c->f[NEMO_F_TSN], *tsa = c->f[NEMO_F_TSA];
  int st;
  memset(tsa, 0, 2 * n3 * sizeof(double));
  if (sbc_bound(c)) {                                        /* step.F90:232-233 */
    if ((st = ora_tra_sbc(c, kt))) return st;
    if (nm->ln_traqsr && (st = ora_tra_qsr(c, kt))) return st;
  }
  double r2dt = (nm->neuler == 0 && kt == nm->nit000) ? nm->rn_rdt : 2.0 * nm->rn_rdt;
  double *zun = zalloc(n3), *zvn = zalloc(n3), *zwn = zalloc(n3);
  ora_tra_adv_trp(c, c->f[NEMO_F_UN], c->f[NEMO_F_VN], c->f[NEMO_F_WN], zun, zvn, zwn);
  st = ora_tra_adv_fct(c, kt, nm->nit000, "TRA", r2dt, zun, zvn, zwn, tsb, tsn, tsa, 2, nm->nn_fct_h ? nm->nn_fct_h : 2,
                       nm->nn_fct_v ? nm->nn_fct_v : 2);
  wfree(zun); wfree(zvn); wfree(zwn);
  if (st) return st;
  const double *ahtu = c->f[NEMO_F_AHTU], *ahtv = c->f[NEMO_F_AHTV];
  if (nm->ln_traldf_blp)   /* traldf.F90:75-76 */
    st = ora_tra_ldf_blp(c, kt, nm->nit000, "TRA", ahtu, ahtv, c->f[NEMO_F_GTSU], c->f[NEMO_F_GTSV],
                         c->f[NEMO_F_GTUI], c->f[NEMO_F_GTVI], tsb, tsa, 2,
                         nm->ln_traldf_iso ? 21 : nm->ln_traldf_triad ? 22 : 20);
  else if (nm->ln_traldf_triad)   /* np_lap_it (traldf.F90:73-74) */
    st = ora_tra_ldf_triad(c, kt, nm->nit000, "TRA", ahtu, ahtv, c->f[NEMO_F_GTSU], c->f[NEMO_F_GTSV],
                           c->f[NEMO_F_GTUI], c->f[NEMO_F_GTVI], tsb, tsb, tsa, 2, 1);
  else if (nm->ln_traldf_iso)
    st = ora_tra_ldf_iso(c, kt, nm->nit000, "TRA", ahtu, ahtv, c->f[NEMO_F_GTSU], c->f[NEMO_F_GTSV],
                         c->f[NEMO_F_GTUI], c->f[NEMO_F_GTVI], tsb, tsb, tsa, 2, 1);
  else
    st = ora_tra_ldf_lap(c, kt, nm->nit000, "TRA", ahtu, ahtv, c->f[NEMO_F_GTSU], c->f[NEMO_F_GTSV],
                         c->f[NEMO_F_GTUI], c->f[NEMO_F_GTVI], tsb, tsa, 2, 1);
  if (st) return st;
  return ora_tra_zdf(c, kt);
}

int ora_stp_hotpath(ora_ctx *c, int kt) {
  double *tsb = c->f[NEMO_F_TSB], *tsn = c->f[NEMO_F_TSN], *tsa = c->f[NEMO_F_TSA];
  if (!tsb || !tsn || !tsa || !c->f[NEMO_F_UN] || !c->f[NEMO_F_VN] || !c->f[NEMO_F_WN]) return NEMO_ERR_UNBOUND;
  int st = ora_dyn_spg_ts(c, kt);
  if (st) return st;
  return stp_tracers(c, kt);
}

/* =================================================================== adjoint */
/* Adjoints of the tracer routines with respect to their tracer arguments. NEMO
 * itself has none (its tangent-linear and adjoint, NEMOTAM, is a separate
 * project), so these follow the forward routines above: each is the transpose of
 * the forward's tangent-linear, written as the forward loops run backwards with
 * every assignment's partial derivatives scattered onto its operands. The
 * coefficients (transports, diffusivities, slopes, scale factors, avt, the
 * partial-step bottom gradients pgu/pgv) are held fixed, and so are the FCT
 * limiter multipliers, which the forward records (ora_set_fct_tape mode 1).
 * Replaying them (mode 2) turns ora_tra_adv_fct into the tangent-linear with the
 * limiter frozen; lap, iso, zdf and nxt are linear in the tracers, so their
 * forward routines are their own tangent-linears. Conventions: an adjoint
 * accumulates into the adjoints of the inputs (ptb_ad += ...), and the adjoint
 * of a trend array pta that the forward only adds to is left unchanged. */

int ora_set_fct_tape(ora_ctx *c, double *tape, int mode) {
  if (!c || mode < 0 || mode > 2 || (mode && !tape)) return NEMO_ERR_ARG;
  c->fct_tape = mode ? tape : NULL;
  c->fct_tape_mode = mode;
  return NEMO_OK;
}

/* Adjoint of ora_tra_adv_fct (kn_fct_h = kn_fct_v = 2) with the recorded limiter. */
int ora_tra_adv_fct_adj(ora_ctx *c, int kt, int kit000, const char *cdtype, double p2dt,
                        const double *pun, const double *pvn, const double *pwn,
                        double *ptb_ad, double *ptn_ad, const double *pta_ad,
                        int kjpt, int kn_fct_h, int kn_fct_v) {
  (void)kt; (void)kit000; (void)cdtype; (void)p2dt;
  if ((kn_fct_h != 2 && kn_fct_h != 4) || (kn_fct_v != 2 && kn_fct_v != 4) || kjpt < 1) return NEMO_ERR_ARG;
  if (!c->fct_tape) return NEMO_ERR_UNBOUND;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const double *tmask = c->tmask, *wmask = c->wmask, *e3t_n = fld(c, NEMO_F_E3T_N);
  const double *umask = c->umask, *vmask = c->vmask, r1_6 = 1. / 6.;
  double *ax = zalloc(n3), *ay = zalloc(n3), *az = zalloc(n3);
  double *fx = zalloc(n3), *fy = zalloc(n3), *fz = zalloc(n3);
  double *zlu = zalloc(n3), *zlv = zalloc(n3), *zv = zalloc(n3);
  for (int jn = 1; jn <= kjpt; ++jn) {
    const double *lam = pta_ad + n3 * (jn - 1), *tp = c->fct_tape + 3 * n3 * (size_t)(jn - 1);
    double *tb_ad = ptb_ad + n3 * (jn - 1), *tn_ad = ptn_ad + n3 * (jn - 1);
    memset(ax, 0, n3 * sizeof(double)); memset(ay, 0, n3 * sizeof(double)); memset(az, 0, n3 * sizeof(double));
    /* (:288-297) trend of the limited fluxes */
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double g = lam[q] * c->r1_e1e2t[I2(ji, jj)] / e3t_n[q];
          ax[q] -= g; ax[I3(ji - 1, jj, jk)] += g;
          ay[q] -= g; ay[I3(ji, jj - 1, jk)] += g;
          az[q] -= g; az[I3(ji, jj, jk + 1)] += g;
        }
    /* (:284 nonosc, :280 lbc) the recorded multipliers, 0 where the flux was zeroed */
    for (size_t q = 0; q < n3; ++q) { ax[q] *= tp[q]; ay[q] *= tp[n3 + q]; az[q] *= tp[2 * n3 + q]; }
    /* (:276-278) linear free surface: no antidiffusive flux through the surface */
    if (c->nam.ln_linssh)
      for (size_t p = 0; p < n2; ++p) az[p] = 0.0;
    /* (:253-275) vertical antidiffusive flux = centred (C2, or the compact 4th-order
     * interpolation ztw) - upstream, interior columns */
    memcpy(fz, az, n3 * sizeof(double));
    if (kn_fct_v == 4) memset(zv, 0, n3 * sizeof(double));
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double a = az[q] * wmask[q];
          if (kn_fct_v == 2) {
            tn_ad[q] += pwn[q] * 0.5 * a;
            tn_ad[I3(ji, jj, jk - 1)] += pwn[q] * 0.5 * a;
          } else {
            zv[q] = pwn[q] * a;  /* the adjoint of ztw */
          }
          fz[q] = -a;
        }
    if (kn_fct_v == 4) ora_interp_4th_cpt_adj(c, zv, tn_ad);
    /* (:182-190, :191-227) horizontal antidiffusive fluxes, C2 or C4 */
    memcpy(fx, ax, n3 * sizeof(double));
    memcpy(fy, ay, n3 * sizeof(double));
    if (kn_fct_h == 4) { memset(zlu, 0, n3 * sizeof(double)); memset(zlv, 0, n3 * sizeof(double)); }
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          const double su = 0.5 * pun[q] * ax[q], sv = 0.5 * pvn[q] * ay[q];
          tn_ad[q] += su;
          tn_ad[I3(ji + 1, jj, jk)] += su;
          tn_ad[q] += sv;
          tn_ad[I3(ji, jj + 1, jk)] += sv;
          if (kn_fct_h == 4) {  /* + zltu(ji) - zltu(ji+1) */
            zlu[q] += su; zlu[I3(ji + 1, jj, jk)] -= su;
            zlv[q] += sv; zlv[I3(ji, jj + 1, jk)] -= sv;
          }
          fx[q] = -ax[q];
          fy[q] = -ay[q];
        }
    if (kn_fct_h == 4) {
      /* zltu, zltv: only the interior values enter the fluxes (their lbc_lnk zeroes
       * the edges); zltu = (ztu(ji) + ztu(ji-1)) / 6, ztu = (tn(ji+1) - tn(ji)) umask */
      for (int jk = 1; jk <= jpk - 1; ++jk)
        for (int jj = 2; jj <= jpj - 1; ++jj)
          for (int ji = 2; ji <= jpi - 1; ++ji) {
            size_t q = I3(ji, jj, jk);
            const double zu = zlu[q] * r1_6, zw = zlv[q] * r1_6;
            const size_t qw = I3(ji - 1, jj, jk), qs = I3(ji, jj - 1, jk);
            tn_ad[I3(ji + 1, jj, jk)] += zu * umask[q];
            tn_ad[q] -= zu * umask[q];
            tn_ad[q] += zu * umask[qw];
            tn_ad[qw] -= zu * umask[qw];
            tn_ad[I3(ji, jj + 1, jk)] += zw * vmask[q];
            tn_ad[q] -= zw * vmask[q];
            tn_ad[q] += zw * vmask[qs];
            tn_ad[qs] -= zw * vmask[qs];
          }
    }
    /* (:158-170) upstream trend (zwi, used only by the frozen limiter, drops out) */
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double h = lam[q] * tmask[q] / e3t_n[q] * c->r1_e1e2t[I2(ji, jj)];
          fx[q] -= h; fx[I3(ji - 1, jj, jk)] += h;
          fy[q] -= h; fy[I3(ji, jj - 1, jk)] += h;
          fz[q] -= h; fz[I3(ji, jj, jk + 1)] += h;
        }
    /* (:146-156) surface flux of the linear free surface */
    if (c->nam.ln_linssh)
      for (size_t p = 0; p < n2; ++p) tb_ad[p] += pwn[p] * fz[p];
    /* (:137-145) vertical upstream flux */
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj; ++jj)
        for (int ji = 1; ji <= jpi; ++ji) {
          size_t q = I3(ji, jj, jk);
          double a = 0.5 * fz[q] * wmask[q];
          tb_ad[q] += (pwn[q] + fabs(pwn[q])) * a;
          tb_ad[I3(ji, jj, jk - 1)] += (pwn[q] - fabs(pwn[q])) * a;
        }
    /* (:123-135) horizontal upstream fluxes */
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          tb_ad[q] += 0.5 * (pun[q] + fabs(pun[q])) * fx[q];
          tb_ad[I3(ji + 1, jj, jk)] += 0.5 * (pun[q] - fabs(pun[q])) * fx[q];
          tb_ad[q] += 0.5 * (pvn[q] + fabs(pvn[q])) * fy[q];
          tb_ad[I3(ji, jj + 1, jk)] += 0.5 * (pvn[q] - fabs(pvn[q])) * fy[q];
        }
  }
  wfree(ax); wfree(ay); wfree(az); wfree(fx); wfree(fy); wfree(fz); wfree(zlu); wfree(zlv); wfree(zv);
  return NEMO_OK;
}

/* Adjoint of ora_tra_ldf_lap. The partial-step bottom faces (ln_zps) take the
 * fixed pgu/pgv, so nothing flows from them to tb. */
int ora_tra_ldf_lap_adj(ora_ctx *c, int kt, int kit000, const char *cdtype,
                        const double *pahu, const double *pahv,
                        const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                        double *ptb_ad, const double *pta_ad, int kjpt, int kpass) {
  (void)kt; (void)kit000; (void)cdtype; (void)pgu; (void)pgv; (void)pgui; (void)pgvi;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n3 = (size_t)jpi * jpj * jpk;
  if (!pahu) pahu = c->ahtu_c;
  if (!pahv) pahv = c->ahtv_c;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N), *e3t_n = fld(c, NEMO_F_E3T_N);
  const double zsign = kpass == 1 ? 1.0 : -1.0;
  double *ztu = zalloc(n3), *ztv = zalloc(n3);
  for (int jn = 1; jn <= kjpt; ++jn) {
    const double *lam = pta_ad + n3 * (jn - 1);
    double *tb_ad = ptb_ad + n3 * (jn - 1);
    memset(ztu, 0, n3 * sizeof(double)); memset(ztv, 0, n3 * sizeof(double));
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double g = lam[q] / (c->e1e2t[I2(ji, jj)] * e3t_n[q]);
          ztu[q] += g; ztu[I3(ji - 1, jj, jk)] -= g;
          ztv[q] += g; ztv[I3(ji, jj - 1, jk)] -= g;
        }
    if (c->nam.ln_zps)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          ztu[I3(ji, jj, c->mbku[I2(ji, jj)])] = 0.0;
          ztv[I3(ji, jj, c->mbkv[I2(ji, jj)])] = 0.0;
        }
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double au = zsign * pahu[q] * c->e2_e1u[I2(ji, jj)] * e3u[q] * ztu[q];
          double av = zsign * pahv[q] * c->e1_e2v[I2(ji, jj)] * e3v[q] * ztv[q];
          tb_ad[I3(ji + 1, jj, jk)] += au; tb_ad[q] -= au;
          tb_ad[I3(ji, jj + 1, jk)] += av; tb_ad[q] -= av;
        }
  }
  wfree(ztu); wfree(ztv);
  return NEMO_OK;
}

/* Adjoint of ora_tra_ldf_iso with respect to ptb (and ptbb, which only kpass = 2
 * without ln_traldf_lap reads). ah_wslp2 and akz are read as the forward left
 * them; the adjoint does not modify them. */
int ora_tra_ldf_iso_adj(ora_ctx *c, int kt, int kit000, const char *cdtype,
                        const double *pahu, const double *pahv,
                        const double *pgu, const double *pgv, const double *pgui, const double *pgvi,
                        double *ptb_ad, double *ptbb_ad, const double *pta_ad, int kjpt, int kpass) {
  (void)kt; (void)kit000; (void)cdtype; (void)pgu; (void)pgv; (void)pgui; (void)pgvi;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const nemo_namelist *nm = &c->nam;
  const double *ah_wslp2 = c->f[NEMO_F_AH_WSLP2], *akz = c->f[NEMO_F_AKZ];
  const double *uslp = c->f[NEMO_F_USLP], *vslp = c->f[NEMO_F_VSLP];
  const double *wslpi = c->f[NEMO_F_WSLPI], *wslpj = c->f[NEMO_F_WSLPJ];
  if (!ah_wslp2 || !akz || !uslp || !vslp || !wslpi || !wslpj) return NEMO_ERR_UNBOUND;
  const int use_tbb = !nm->ln_traldf_lap && kpass != 1;
  if (use_tbb && !ptbb_ad) return NEMO_ERR_ARG;
  if (!pahu) pahu = c->ahtu_c;
  if (!pahv) pahv = c->ahtv_c;
  const double *umask = c->umask, *vmask = c->vmask, *wmask = c->wmask;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N), *e3t_n = fld(c, NEMO_F_E3T_N);
  const double *e3w = fld(c, NEMO_F_E3W_N);
  const double zsign = kpass == 1 ? 1.0 : -1.0;
  double *dit = zalloc(n3), *djt = zalloc(n3), *tfw = zalloc(n3);
  double *dkt = zalloc(n2), *dk1t = zalloc(n2), *ftu = zalloc(n2), *ftv = zalloc(n2);
  for (int jn = 1; jn <= kjpt; ++jn) {
    const double *lam = pta_ad + n3 * (jn - 1);
    double *tb_ad = ptb_ad + n3 * (jn - 1);
    double *tbb_ad = use_tbb ? ptbb_ad + n3 * (jn - 1) : NULL;
    memset(dit, 0, n3 * sizeof(double)); memset(djt, 0, n3 * sizeof(double)); memset(tfw, 0, n3 * sizeof(double));
    /* (:359-366) divergence of the vertical fluxes */
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double g = zsign * lam[q] * c->r1_e1e2t[I2(ji, jj)] / e3t_n[q];
          tfw[q] += g; tfw[I3(ji, jj, jk + 1)] -= g;
        }
    /* the flux zeroed at the surface, the bottom and the edge columns (:294-296) */
    for (int jk = 1; jk <= jpk; ++jk)
      for (int jj = 1; jj <= jpj; ++jj) { tfw[I3(1, jj, jk)] = 0.0; tfw[I3(jpi, jj, jk)] = 0.0; }
    for (size_t p = 0; p < n2; ++p) { tfw[p] = 0.0; tfw[p + n2 * (jpk - 1)] = 0.0; }
    /* (:323-357) vertical laplacian part, jj from 1 */
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk), qu = I3(ji, jj, jk - 1);
          double f = c->e1e2t[I2(ji, jj)] / e3w[q] * wmask[q] * tfw[q];
          if (nm->ln_traldf_lap) {
            double a = (ah_wslp2[q] - akz[q]) * f;
            tb_ad[qu] += a; tb_ad[q] -= a;
          } else if (kpass == 1) {
            double a = ah_wslp2[q] * f;
            tb_ad[qu] += a; tb_ad[q] -= a;
          } else {
            double a = ah_wslp2[q] * f, b = akz[q] * f;
            tb_ad[qu] += a; tb_ad[q] -= a;
            tbb_ad[qu] += b; tbb_ad[q] -= b;
          }
        }
    /* (:298-321) rotated vertical flux from the four surrounding horizontal gradients */
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double zmsku = wmask[q] / dmax(umask[I3(ji, jj, jk - 1)] + umask[I3(ji - 1, jj, jk)]
                                         + umask[I3(ji - 1, jj, jk - 1)] + umask[q], 1.0);
          double zmskv = wmask[q] / dmax(vmask[I3(ji, jj, jk - 1)] + vmask[I3(ji, jj - 1, jk)]
                                         + vmask[I3(ji, jj - 1, jk - 1)] + vmask[q], 1.0);
          double zahu_w = (pahu[I3(ji, jj, jk - 1)] + pahu[I3(ji - 1, jj, jk)]
                           + pahu[I3(ji - 1, jj, jk - 1)] + pahu[q]) * zmsku;
          double zahv_w = (pahv[I3(ji, jj, jk - 1)] + pahv[I3(ji, jj - 1, jk)]
                           + pahv[I3(ji, jj - 1, jk - 1)] + pahv[q]) * zmskv;
          double a3 = -zahu_w * c->e2t[I2(ji, jj)] * zmsku * wslpi[q] * tfw[q];
          double a4 = -zahv_w * c->e1t[I2(ji, jj)] * zmskv * wslpj[q] * tfw[q];
          dit[I3(ji, jj, jk - 1)] += a3; dit[I3(ji - 1, jj, jk)] += a3;
          dit[I3(ji - 1, jj, jk - 1)] += a3; dit[q] += a3;
          djt[I3(ji, jj, jk - 1)] += a4; djt[I3(ji, jj - 1, jk)] += a4;
          djt[I3(ji, jj - 1, jk - 1)] += a4; djt[q] += a4;
        }
    /* (:243-285) level by level: horizontal rotated fluxes and their divergence */
    for (int jk = jpk - 1; jk >= 1; --jk) {
      memset(ftu, 0, n2 * sizeof(double)); memset(ftv, 0, n2 * sizeof(double));
      memset(dkt, 0, n2 * sizeof(double)); memset(dk1t, 0, n2 * sizeof(double));
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double g = zsign * lam[q] * c->r1_e1e2t[I2(ji, jj)] / e3t_n[q];
          ftu[I2(ji, jj)] += g; ftu[I2(ji - 1, jj)] -= g;
          ftv[I2(ji, jj)] += g; ftv[I2(ji, jj - 1)] -= g;
        }
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double zabe1 = pahu[q] * c->e2_e1u[I2(ji, jj)] * e3u[q];
          double zabe2 = pahv[q] * c->e1_e2v[I2(ji, jj)] * e3v[q];
          double zmsku = 1. / dmax(wmask[I3(ji + 1, jj, jk)] + wmask[I3(ji, jj, jk + 1)]
                                   + wmask[I3(ji + 1, jj, jk + 1)] + wmask[q], 1.);
          double zmskv = 1. / dmax(wmask[I3(ji, jj + 1, jk)] + wmask[I3(ji, jj, jk + 1)]
                                   + wmask[I3(ji, jj + 1, jk + 1)] + wmask[q], 1.);
          double zcof1 = -pahu[q] * c->e2u[I2(ji, jj)] * uslp[q] * zmsku;
          double zcof2 = -pahv[q] * c->e1v[I2(ji, jj)] * vslp[q] * zmskv;
          double fu = ftu[I2(ji, jj)] * umask[q], fv = ftv[I2(ji, jj)] * vmask[q];
          dit[q] += zabe1 * fu;
          djt[q] += zabe2 * fv;
          double u1 = zcof1 * fu, v1 = zcof2 * fv;
          dkt[I2(ji + 1, jj)] += u1; dk1t[I2(ji, jj)] += u1; dk1t[I2(ji + 1, jj)] += u1; dkt[I2(ji, jj)] += u1;
          dkt[I2(ji, jj + 1)] += v1; dk1t[I2(ji, jj)] += v1; dk1t[I2(ji, jj + 1)] += v1; dkt[I2(ji, jj)] += v1;
        }
      /* zdkt: (tb(k-1) - tb(k)) * wmask(k), or zdk1t at the surface (:246-251) */
      if (jk == 1) {
        for (size_t p = 0; p < n2; ++p) dk1t[p] += dkt[p];
      } else {
        for (size_t p = 0; p < n2; ++p) {
          double a = dkt[p] * wmask[p + n2 * (jk - 1)];
          tb_ad[p + n2 * (jk - 2)] += a; tb_ad[p + n2 * (jk - 1)] -= a;
        }
      }
      /* zdk1t: (tb(k) - tb(k+1)) * wmask(k+1) */
      for (size_t p = 0; p < n2; ++p) {
        double a = dk1t[p] * wmask[p + n2 * jk];
        tb_ad[p + n2 * (jk - 1)] += a; tb_ad[p + n2 * jk] -= a;
      }
    }
    /* (:228-241) the partial-step bottom gradients are fixed inputs */
    if (nm->ln_zps)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          dit[I3(ji, jj, c->mbku[I2(ji, jj)])] = 0.0;
          djt[I3(ji, jj, c->mbkv[I2(ji, jj)])] = 0.0;
        }
    /* (:218-227) masked horizontal gradients */
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double a = dit[q] * umask[q], b = djt[q] * vmask[q];
          tb_ad[I3(ji + 1, jj, jk)] += a; tb_ad[q] -= a;
          tb_ad[I3(ji, jj + 1, jk)] += b; tb_ad[q] -= b;
        }
  }
  wfree(dit); wfree(djt); wfree(tfw); wfree(dkt); wfree(dk1t); wfree(ftu); wfree(ftv);
  return NEMO_OK;
}

/* Adjoint of ora_tra_zdf_imp: pta_ad (adjoint of the after tracer) becomes the
 * adjoint of the trend that entered, ptb_ad accumulates the before tracer's. */
int ora_tra_zdf_imp_adj(ora_ctx *c, int kt, int kit000, const char *cdtype, double p2dt,
                        double *ptb_ad, double *pta_ad, int kjpt) {
  (void)kt; (void)kit000;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n3 = (size_t)jpi * jpj * jpk;
  const nemo_namelist *nm = &c->nam;
  const int is_trc = cdtype && cdtype[0] == 'T' && cdtype[1] == 'R' && cdtype[2] == 'C';
  const double *avt = c->f[NEMO_F_AVT], *avs = c->f[NEMO_F_AVS];
  const double *e3t_b = fld(c, NEMO_F_E3T_B), *e3t_n = fld(c, NEMO_F_E3T_N), *tmask = c->tmask;
  if (!avt && !is_trc) return NEMO_ERR_UNBOUND;
  if ((nm->ln_traldf_iso || nm->ln_traldf_triad) &&
      ((nm->ln_traldf_msc && !c->f[NEMO_F_AKZ]) || (!nm->ln_traldf_msc && !c->f[NEMO_F_AH_WSLP2])))
    return NEMO_ERR_UNBOUND;
  double *zwi = zalloc(n3), *zwt = zalloc(n3), *zwd = zalloc(n3), *zws = zalloc(n3);
  for (int jn = 1; jn <= kjpt; ++jn) {
    double *tb_ad = ptb_ad + n3 * (jn - 1), *lam = pta_ad + n3 * (jn - 1);
    if ((!is_trc && (jn == 1 || (jn == 2 && nm->ln_zdfddm))) || (is_trc && jn == 1)) {
      const double *coef = (!is_trc && jn == 1) ? avt : avs;
      if (!coef) { wfree(zwi); wfree(zwt); wfree(zwd); wfree(zws); return NEMO_ERR_UNBOUND; }
      zdf_lu(c, coef, p2dt, zwi, zwt, zwd, zws);
    }
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        /* back-substitution (:252-264), run forwards */
        for (int jk = 1; jk <= jpk - 2; ++jk) {
          size_t q = I3(ji, jj, jk);
          double a = lam[q] * tmask[q] / zwt[q];
          lam[I3(ji, jj, jk + 1)] -= zws[q] * a;
          lam[q] = a;
        }
        size_t qb = I3(ji, jj, jpk - 1);
        lam[qb] = lam[qb] * tmask[qb] / zwt[qb];
        /* forward elimination with the right-hand side (:238-250), run backwards */
        for (int jk = jpk - 1; jk >= 2; --jk) {
          size_t q = I3(ji, jj, jk);
          lam[I3(ji, jj, jk - 1)] -= zwi[q] / zwt[I3(ji, jj, jk - 1)] * lam[q];
          tb_ad[q] += e3t_b[q] * lam[q];
          lam[q] = p2dt * e3t_n[q] * lam[q];
        }
        size_t q1 = I3(ji, jj, 1);
        tb_ad[q1] += e3t_b[q1] * lam[q1];
        lam[q1] = p2dt * e3t_n[q1] * lam[q1];
      }
  }
  wfree(zwi); wfree(zwt); wfree(zwd); wfree(zws);
  return NEMO_OK;
}

/* ------------------------------------------------------ dyn_spg_ts adjoint */
/* The barotropic Coriolis trend of dyn_spg_ts (dynspg_ts.F90:387-443, :1000-1056)
 * as weights of four neighbouring fluxes: zu_trd(p) = sum_t cu(t,p) zwy(p + du_t)
 * with du = (0,-1), (1,-1), (0,0), (1,0), and zv_trd(p) = sum_t cv(t,p) zwx(p + dv_t)
 * with dv = (-1,0), (-1,1), (0,0), (0,1); ENE (and MIX), ENS, EEN. */
static const int SPG_DUI[4] = {0, 1, 0, 1}, SPG_DUJ[4] = {-1, -1, 0, 0};
static const int SPG_DVI[4] = {-1, -1, 0, 0}, SPG_DVJ[4] = {0, 1, 0, 1};
static double spg_cu(const ora_ctx *c, int sc, int t, int ji, int jj) {
  const int jpi = c->jpi;
  const size_t p = I2(ji, jj);
  if (sc == NEMO_VOR_ENS) return 0.125 * c->r1_e1u[p] * (c->zwz[I2(ji, jj - 1)] + c->zwz[p]);
  if (sc == NEMO_VOR_EEN) {
    const double f = t == 0 ? c->ftse[p] : t == 1 ? c->ftsw[I2(ji + 1, jj)] : t == 2 ? c->ftne[p] : c->ftnw[I2(ji + 1, jj)];
    return (1.0 / 12.0) * c->r1_e1u[p] * f;
  }
  return 0.25 * (t < 2 ? c->zwz[I2(ji, jj - 1)] : c->zwz[p]) * c->r1_e1u[p];
}
static double spg_cv(const ora_ctx *c, int sc, int t, int ji, int jj) {
  const int jpi = c->jpi;
  const size_t p = I2(ji, jj);
  if (sc == NEMO_VOR_ENS) return -0.125 * c->r1_e2v[p] * (c->zwz[I2(ji - 1, jj)] + c->zwz[p]);
  if (sc == NEMO_VOR_EEN) {
    const double f = t == 0 ? c->ftnw[p] : t == 1 ? c->ftsw[I2(ji, jj + 1)] : t == 2 ? c->ftne[p] : c->ftse[I2(ji, jj + 1)];
    return -(1.0 / 12.0) * c->r1_e2v[p] * f;
  }
  return -0.25 * (t < 2 ? c->zwz[I2(ji - 1, jj)] : c->zwz[p]) * c->r1_e2v[p];
}
/* the transpose: the flux adjoints zwxa, zwya += C^T (gu, gv) for trend adjoints gu,
 * gv on the interior */
static void spg_cor_adj(const ora_ctx *c, int sc, const double *gu, const double *gv, double *zwxa, double *zwya) {
  const int jpi = c->jpi, jpj = c->jpj;
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      const size_t p = I2(ji, jj);
      for (int t = 0; t < 4; ++t) {
        zwya[I2(ji + SPG_DUI[t], jj + SPG_DUJ[t])] += spg_cu(c, sc, t, ji, jj) * gu[p];
        zwxa[I2(ji + SPG_DVI[t], jj + SPG_DVJ[t])] += spg_cv(c, sc, t, ji, jj) * gv[p];
      }
    }
}

/* Adjoint of ora_dyn_spg_ts (the argument roles of nemo_spg_adj in nemo_gpu.h) for a
 * linear free surface with ln_bt_fw and ln_bt_av: the forward's operations in
 * reverse order -- phase 3 (:1214-1269), the sub-steps from the last (:712-1207:
 * sums, swap, lbc, next velocities, bottom stress, pressure gradient, Coriolis, AM4
 * ssh, ssh update, divergence, flux sums, fluxes, AB3 extrapolation), the start of
 * the sub-steps from sshn, un_b, vn_b (:665-702), phase 1 (:358-557). The forcing
 * terms are constants of the map. The weights are those of the last forward call. */
int ora_dyn_spg_ts_adj(ora_ctx *c, int kt, const nemo_spg_adj *A) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  if (!A) return NEMO_ERR_ARG;
  double *ua_ad = A->ua, *va_ad = A->va, *un_ad = A->un, *vn_ad = A->vn;
  double *ssha_ad = A->ssha, *uab_ad = A->ua_b, *vab_ad = A->va_b, *unadv_ad = A->un_adv, *vnadv_ad = A->vn_adv;
  double *ub2_ad = A->ub2_b, *vb2_ad = A->vb2_b, *unbf_ad = A->un_bf, *vnbf_ad = A->vn_bf;
  double *sshn_ad = A->sshn, *unb_ad = A->un_b, *vnb_ad = A->vn_b, *ubb_ad = A->ub_b, *vbb_ad = A->vb_b;
  if (!ua_ad || !va_ad || !un_ad || !vn_ad || !ssha_ad || !uab_ad || !vab_ad || !unadv_ad || !vnadv_ad || !ub2_ad ||
      !vb2_ad || !unbf_ad || !vnbf_ad || !sshn_ad || !unb_ad || !vnb_ad || !ubb_ad || !vbb_ad)
    return NEMO_ERR_ARG;
  const int sc = nm->nvor_scheme;
  if (!nm->ln_linssh || !nm->ln_bt_fw || !nm->ln_bt_av || sc == NEMO_VOR_ENT) return NEMO_ERR_UNSUPPORTED;
  const double *rCdU_bot = c->f[NEMO_F_RCDU_BOT];
  if (!rCdU_bot) return NEMO_ERR_UNBOUND;
  const int euler = kt == nm->nit000 && nm->neuler == 0;
  const double r1_2dt_b = 1.0 / (euler ? nm->rn_rdt : 2.0 * nm->rn_rdt), atfp = nm->rn_atfp;
  const double rdtbt = c->rdtbt, grav = nm->grav, sl = nm->rn_scal_load, r1_2 = 0.5;
  const double *umask = c->umask, *vmask = c->vmask, *e3u = c->e3u_0, *e3v = c->e3v_0;
  const double *hu = c->hu_0, *hv = c->hv_0, *r1_hu = c->r1_hu_0, *r1_hv = c->r1_hv_0;
  const double *ssumask = c->ssumask, *ssvmask = c->ssvmask, *ssmask = c->ssmask;
  double *X = zalloc(n2), *Y = zalloc(n2), *uab = zalloc(n2), *vab = zalloc(n2);
  double *Au = zalloc(n2), *Aub = zalloc(n2), *Aubb = zalloc(n2), *Av = zalloc(n2), *Avb = zalloc(n2), *Avbb = zalloc(n2);
  double *Sn = zalloc(n2), *Sb = zalloc(n2), *Sbb = zalloc(n2);
  double *Nu = zalloc(n2), *Nub = zalloc(n2), *Nubb = zalloc(n2), *Nv = zalloc(n2), *Nvb = zalloc(n2), *Nvbb = zalloc(n2);
  double *Nsn = zalloc(n2), *Nsb = zalloc(n2), *Nsbb = zalloc(n2);
  double *Fu = zalloc(n2), *Fv = zalloc(n2), *gu = zalloc(n2), *gv = zalloc(n2);
  double *uae = zalloc(n2), *vae = zalloc(n2), *sae = zalloc(n2), *zsp = zalloc(n2), *zhd = zalloc(n2);
  double *zwxa = zalloc(n2), *zwya = zalloc(n2);
  /* phase 3 */
  for (size_t p = 0; p < n2; ++p) {
    double su = 0.0, sv = 0.0, ta = 0.0, tb = 0.0;
    for (int jk = 1; jk <= jpk - 1; ++jk) {
      const size_t q = p + n2 * (jk - 1);
      su += un_ad[q] * umask[q]; sv += vn_ad[q] * vmask[q];
      ta += ua_ad[q]; tb += va_ad[q];
      un_ad[q] = un_ad[q] * umask[q]; vn_ad[q] = vn_ad[q] * vmask[q];
    }
    const double adu = unadv_ad[p] + su * r1_hu[p], adv = vnadv_ad[p] + sv * r1_hv[p];
    unb_ad[p] -= su; vnb_ad[p] -= sv;
    uab[p] = uab_ad[p] + ta * r1_2dt_b; vab[p] = vab_ad[p] + tb * r1_2dt_b;
    ubb_ad[p] -= ta * r1_2dt_b; vbb_ad[p] -= tb * r1_2dt_b;
    if (!euler) {
      X[p] = 0.5 * adu + unbf_ad[p] + ub2_ad[p];
      Y[p] = 0.5 * adv + vnbf_ad[p] + vb2_ad[p];
      const double u2 = 0.5 * adu - unbf_ad[p], v2 = 0.5 * adv - vnbf_ad[p];
      unbf_ad[p] = -0.5 * atfp * adu + atfp * unbf_ad[p];
      vnbf_ad[p] = -0.5 * atfp * adv + atfp * vnbf_ad[p];
      ub2_ad[p] = u2; vb2_ad[p] = v2;
    } else {
      X[p] = adu + ub2_ad[p]; Y[p] = adv + vb2_ad[p];
      ub2_ad[p] = 0.0; vb2_ad[p] = 0.0; unbf_ad[p] = 0.0; vnbf_ad[p] = 0.0;
    }
  }
  /* the sub-steps, last first */
  for (int jn = c->icycle; jn >= 1; --jn) {
    const double w1 = c->wgtbtp1[jn - 1], w2 = c->wgtbtp2[jn - 1];
    double zb1, zb2, zb3, za0, za1, za2, za3;
    if (jn < 3) { zb1 = 1.0; zb2 = 0.0; zb3 = 0.0; }
    else { zb1 = 1.781105; zb2 = -1.06221; zb3 = 0.281105; }
    if (jn == 1) { za0 = 1.0; za1 = 0.0; za2 = 0.0; za3 = 0.0; }
    else if (jn == 2) { za0 = 1.0833333333333; za1 = -0.1666666666666; za2 = 0.0833333333333; za3 = 0.0; }
    else if (nm->rn_bt_alpha == 0.0) { za0 = 0.614; za1 = 0.285; za2 = 0.088; za3 = 0.013; }
    else {
      const double zepsilon = 0.00976186 - 0.13451357 * nm->rn_bt_alpha;
      const double zgamma = 0.08344500 - 0.51358400 * nm->rn_bt_alpha;
      za0 = 0.5 + zgamma + 2.0 * nm->rn_bt_alpha + 2.0 * zepsilon;
      za1 = 1.0 - za0 - zgamma - zepsilon;
      za2 = zgamma;
      za3 = zepsilon;
    }
    for (size_t p = 0; p < n2; ++p) {       /* sums and swap (:1176-1204) */
      uae[p] = Au[p] + w1 * uab[p]; vae[p] = Av[p] + w1 * vab[p];
      sae[p] = Sn[p] + w1 * ssha_ad[p];
      Nu[p] = Aub[p]; Nub[p] = Aubb[p]; Nubb[p] = 0.0;
      Nv[p] = Avb[p]; Nvb[p] = Avbb[p]; Nvbb[p] = 0.0;
      Nsn[p] = Sb[p]; Nsb[p] = Sbb[p]; Nsbb[p] = 0.0;
      gu[p] = 0.0; gv[p] = 0.0; zsp[p] = 0.0; zwxa[p] = 0.0; zwya[p] = 0.0;
    }
    lbc_closed(jpi, jpj, uae, 1, 'U', 0.0);   /* (:1167) */
    lbc_closed(jpi, jpj, vae, 1, 'V', 0.0);
    for (int jj = 2; jj <= jpj - 1; ++jj)    /* next velocities (:1106-1122), bottom stress (:1072-1079) */
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj);
        const double tu = uae[p] * ssumask[p], tv = vae[p] * ssvmask[p];
        gu[p] = rdtbt * tu; gv[p] = rdtbt * tv;
        Fu[p] += gu[p]; Fv[p] += gv[p];
        Nu[p] += tu + r1_2 * (rCdU_bot[I2(ji + 1, jj)] + rCdU_bot[p]) * r1_hu[p] * gu[p];
        Nv[p] += tv + r1_2 * (rCdU_bot[I2(ji, jj + 1)] + rCdU_bot[p]) * r1_hv[p] * gv[p];
        /* surface pressure gradient (:1093-1101) */
        const double ku = (1.0 - sl) * (-grav) * c->r1_e1u[p] * gu[p];
        const double kv = (1.0 - sl) * (-grav) * c->r1_e2v[p] * gv[p];
        zsp[I2(ji + 1, jj)] += ku; zsp[p] -= ku;
        zsp[I2(ji, jj + 1)] += kv; zsp[p] -= kv;
      }
    spg_cor_adj(c, sc, gu, gv, zwxa, zwya);  /* Coriolis of the fluxes (:1000-1056) */
    for (size_t p = 0; p < n2; ++p) {        /* AM4 ssh (:904-931) */
      sae[p] += za0 * zsp[p]; Nsn[p] += za1 * zsp[p]; Nsb[p] += za2 * zsp[p]; Nsbb[p] += za3 * zsp[p];
    }
    lbc_closed(jpi, jpj, sae, 1, 'T', 0.0);  /* (:879) */
    for (size_t p = 0; p < n2; ++p) {        /* ssh update (:871-877) */
      const double t = sae[p] * ssmask[p];
      Nsn[p] += t;
      zhd[p] = -rdtbt * t;
    }
    for (int jj = 2; jj <= jpj - 1; ++jj)    /* divergence (:866-869) */
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj);
        const double t = zhd[p] * c->r1_e1e2t[p];
        zwxa[p] += t; zwxa[I2(ji - 1, jj)] -= t;
        zwya[p] += t; zwya[I2(ji, jj - 1)] -= t;
      }
    for (size_t p = 0; p < n2; ++p) {        /* flux sums (:860-862), fluxes (:799-800), AB3 (:724-736) */
      zwxa[p] += w2 * X[p] * c->r1_e2u[p];
      zwya[p] += w2 * Y[p] * c->r1_e1v[p];
      const double eu = zwxa[p] * c->e2u[p] * hu[p], ev = zwya[p] * c->e1v[p] * hv[p];
      Nu[p] += zb1 * eu; Nub[p] += zb2 * eu; Nubb[p] += zb3 * eu;
      Nv[p] += zb1 * ev; Nvb[p] += zb2 * ev; Nvbb[p] += zb3 * ev;
    }
    double *t;
    t = Au; Au = Nu; Nu = t;  t = Aub; Aub = Nub; Nub = t;  t = Aubb; Aubb = Nubb; Nubb = t;
    t = Av; Av = Nv; Nv = t;  t = Avb; Avb = Nvb; Nvb = t;  t = Avbb; Avbb = Nvbb; Nvbb = t;
    t = Sn; Sn = Nsn; Nsn = t;  t = Sb; Sb = Nsb; Nsb = t;  t = Sbb; Sbb = Nsbb; Nsbb = t;
  }
  for (size_t p = 0; p < n2; ++p) {          /* the start from sshn, un_b, vn_b (:688-693) */
    unb_ad[p] += Au[p]; vnb_ad[p] += Av[p]; sshn_ad[p] += Sn[p];
  }
  /* phase 1: bottom stress of the baroclinic velocities (:519-557) */
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      const size_t p = I2(ji, jj);
      const double tu = r1_hu[p] * r1_2 * (rCdU_bot[I2(ji + 1, jj)] + rCdU_bot[p]) * Fu[p];
      const double tv = r1_hv[p] * r1_2 * (rCdU_bot[I2(ji, jj + 1)] + rCdU_bot[p]) * Fv[p];
      un_ad[I3(ji, jj, c->mbku[p])] += tu; unb_ad[p] -= tu;
      vn_ad[I3(ji, jj, c->mbkv[p])] += tv; vnb_ad[p] -= tv;
    }
  /* Coriolis of un_b, vn_b (:387-443) removed from the forcing (:511-516) */
  for (size_t p = 0; p < n2; ++p) { gu[p] = 0.0; gv[p] = 0.0; zwxa[p] = 0.0; zwya[p] = 0.0; }
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      const size_t p = I2(ji, jj);
      gu[p] = -Fu[p] * ssumask[p]; gv[p] = -Fv[p] * ssvmask[p];
    }
  spg_cor_adj(c, sc, gu, gv, zwxa, zwya);
  for (size_t p = 0; p < n2; ++p) { unb_ad[p] += zwxa[p] * hu[p] * c->e2u[p]; vnb_ad[p] += zwya[p] * hv[p] * c->e1v[p]; }
  /* the baroclinic trend's vertical mean (:358-378) */
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      const size_t p = I2(ji, jj);
      double su = Fu[p], sv = Fv[p];
      for (int jk = 1; jk <= jpk - 1; ++jk) {
        const size_t q = p + n2 * (jk - 1);
        su -= ua_ad[q] * umask[q]; sv -= va_ad[q] * vmask[q];
      }
      for (int jk = 1; jk <= jpk - 1; ++jk) {
        const size_t q = p + n2 * (jk - 1);
        ua_ad[q] += e3u[q] * umask[q] * r1_hu[p] * su;
        va_ad[q] += e3v[q] * vmask[q] * r1_hv[p] * sv;
      }
    }
  for (size_t p = 0; p < n2; ++p) {          /* the outputs the forward overwrites */
    ssha_ad[p] = 0.0; uab_ad[p] = 0.0; vab_ad[p] = 0.0; unadv_ad[p] = 0.0; vnadv_ad[p] = 0.0;
  }
  double *w[] = {X, Y, uab, vab, Au, Aub, Aubb, Av, Avb, Avbb, Sn, Sb, Sbb, Nu, Nub, Nubb, Nv, Nvb, Nvbb, Nsn, Nsb, Nsbb,
                 Fu, Fv, gu, gv, uae, vae, sae, zsp, zhd, zwxa, zwya};
  for (size_t i = 0; i < sizeof w / sizeof w[0]; ++i) wfree(w[i]);
  return NEMO_OK;
}

/* ---------------------------------------------------------------- tra_nxt */
/* tra_nxt_vvl (tranxt.F90:240-380) for the active tracers, p2dt = rdt as tra_nxt
 * passes it (:161): the thickness-weighted Asselin filter with the forcing removed at
 * the first level (emp, rnf without ln_rnf_depth, sbc_tsc) and in the levels of
 * penetrating light (qsr_hc, ln_traqsr); no ice-shelf melt, no tracer runoff. */
static int tra_nxt_vvl(ora_ctx *c, double *tsb, double *tsn, const double *tsa) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const double *e3t_b = c->f[NEMO_F_E3T_B], *e3t_n = c->f[NEMO_F_E3T_N], *e3t_a = c->f[NEMO_F_E3T_A];
  const double *emp = c->f[NEMO_F_EMP], *emp_b = c->f[NEMO_F_EMP_B];
  const double *rnf = c->f[NEMO_F_RNF], *rnf_b = c->f[NEMO_F_RNF_B];
  const double *tsc = c->f[NEMO_F_SBC_TSC], *tsc_b = c->f[NEMO_F_SBC_TSC_B];
  const double *hc = c->f[NEMO_F_QSR_HC], *hc_b = c->f[NEMO_F_QSR_HC_B];
  if (!e3t_b || !e3t_n || !e3t_a || !emp || !emp_b || !tsc || !tsc_b) return NEMO_ERR_UNBOUND;
  if ((rnf == NULL) != (rnf_b == NULL)) return NEMO_ERR_UNBOUND;
  if (nm->ln_traqsr && (!hc || !hc_b)) return NEMO_ERR_UNBOUND;
  const double atfp = nm->rn_atfp, r1_rau0 = 1.0 / nm->rau0;
  const double zfact1 = atfp * nm->rn_rdt, zfact2 = zfact1 * r1_rau0;   /* :293-295 */
  for (int jn = 1; jn <= 2; ++jn)
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t p = I2(ji, jj), q = I3(ji, jj, jk), o = q + n3 * (jn - 1);
          const double ze3t_b = e3t_b[q], ze3t_n = e3t_n[q], ze3t_a = e3t_a[q];
          const double ztc_b = tsb[o] * ze3t_b, ztc_n = tsn[o] * ze3t_n, ztc_a = tsa[o] * ze3t_a;
          const double ze3t_d = ze3t_a - 2. * ze3t_n + ze3t_b;
          const double ztc_d = ztc_a - 2. * ztc_n + ztc_b;
          double ze3t_f = ze3t_n + atfp * ze3t_d;
          double ztc_f = ztc_n + atfp * ztc_d;
          if (jk == c->mikt[p]) {                               /* :314-319 */
            ze3t_f = ze3t_f - zfact2 * (emp_b[p] - emp[p]);
            ztc_f = ztc_f - zfact1 * (tsc[p + n2 * (jn - 1)] - tsc_b[p + n2 * (jn - 1)]);
            if (rnf) ze3t_f = ze3t_f - zfact2 * (-(rnf_b[p] - rnf[p]));   /* :325-329 */
          }
          if (nm->ln_traqsr && jn == 1 && jk <= c->nksr)        /* :333-334 */
            ztc_f = ztc_f - zfact1 * (hc[q] - hc_b[q]);
          ze3t_f = 1.e0 / ze3t_f;
          tsb[o] = ztc_f * ze3t_f;
          tsn[o] = tsa[o];
        }
  return NEMO_OK;
}

/* tranxt.F90:66-188 with tra_nxt_fix (:191-237) or, with a variable volume,
 * tra_nxt_vvl on the bound tsb, tsn, tsa (no trend diagnostics, bdy or agrif). */
int ora_tra_nxt(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n3 = (size_t)jpi * jpj * jpk;
  double *tsb = c->f[NEMO_F_TSB], *tsn = c->f[NEMO_F_TSN], *tsa = c->f[NEMO_F_TSA];
  if (!tsb || !tsn || !tsa) return NEMO_ERR_UNBOUND;
  lbc_closed(jpi, jpj, tsa, 2 * jpk, 'T', 0.0);          /* :109 */
  if (nm->neuler == 0 && kt == nm->nit000) {               /* :144-149 Euler: swap only */
    for (int jn = 0; jn < 2; ++jn)
      memcpy(tsn + n3 * jn, tsa + n3 * jn, (n3 - (size_t)jpi * jpj) * sizeof(double));
    return NEMO_OK;
  }
  if (!nm->ln_linssh) {                                     /* :160-162 */
    const int st = tra_nxt_vvl(c, tsb, tsn, tsa);
    if (st) return st;
    lbc_closed(jpi, jpj, tsb, 2 * jpk, 'T', 0.0);
    lbc_closed(jpi, jpj, tsn, 2 * jpk, 'T', 0.0);
    return NEMO_OK;
  }
  const double atfp = nm->rn_atfp;
  for (int jn = 0; jn < 2; ++jn) {                          /* :221-234 */
    double *tb = tsb + n3 * jn, *tn = tsn + n3 * jn, *ta = tsa + n3 * jn;
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double ztn = tn[q];
          double ztd = ta[q] - 2.0 * ztn + tb[q];
          tb[q] = ztn + atfp * ztd;
          tn[q] = ta[q];
        }
  }
  lbc_closed(jpi, jpj, tsb, 2 * jpk, 'T', 0.0);          /* :165-167 */
  lbc_closed(jpi, jpj, tsn, 2 * jpk, 'T', 0.0);
  return NEMO_OK;
}

/* Adjoint of ora_tra_nxt on three adjoint arrays (jpi,jpj,jpk,2): on entry the
 * adjoints of the after-swap tsb, tsn, tsa; on exit those of the before-swap ones. */
int ora_tra_nxt_adj(ora_ctx *c, int kt, double *tsb_ad, double *tsn_ad, double *tsa_ad) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  if (!tsb_ad || !tsn_ad || !tsa_ad) return NEMO_ERR_ARG;
  if (!nm->ln_linssh) return NEMO_ERR_ARG;
  if (nm->neuler == 0 && kt == nm->nit000) {
    for (int jn = 0; jn < 2; ++jn)
      for (size_t q = 0; q < n3 - n2; ++q) {
        tsa_ad[n3 * jn + q] += tsn_ad[n3 * jn + q];
        tsn_ad[n3 * jn + q] = 0.0;
      }
    lbc_closed(jpi, jpj, tsa_ad, 2 * jpk, 'T', 0.0);
    return NEMO_OK;
  }
  const double atfp = nm->rn_atfp;
  lbc_closed(jpi, jpj, tsb_ad, 2 * jpk, 'T', 0.0);
  lbc_closed(jpi, jpj, tsn_ad, 2 * jpk, 'T', 0.0);
  lbc_closed(jpi, jpj, tsa_ad, 2 * jpk, 'T', 0.0);
  for (int jn = 0; jn < 2; ++jn) {
    double *bb = tsb_ad + n3 * jn, *nn = tsn_ad + n3 * jn, *aa = tsa_ad + n3 * jn;
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          size_t q = I3(ji, jj, jk);
          double b = bb[q], n = nn[q];
          aa[q] += n + atfp * b;
          nn[q] = b - 2.0 * atfp * b;
          bb[q] = atfp * b;
        }
  }
  lbc_closed(jpi, jpj, tsa_ad, 2 * jpk, 'T', 0.0);
  return NEMO_OK;
}

/* ------------------------------------- adjoints of the step's time stepping */
/* Adjoint of ora_wzv for the linear free surface: the transpose of (un, vn) -> wn
 * (sshwzv.F90:129-213 with divhor.F90:62-110): hdivn_ad(l) = -e3t_n tmask times the
 * sum of wn_ad over levels 1..l, then the transposed divergence. wn_ad is zeroed. */
int ora_wzv_adj(ora_ctx *c, int kt, double *un_ad, double *vn_ad, double *wn_ad) {
  (void)kt;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  if (!un_ad || !vn_ad || !wn_ad) return NEMO_ERR_ARG;
  if (!c->nam.ln_linssh) return NEMO_ERR_UNSUPPORTED;
  const double *e3u = c->e3u_0, *e3v = c->e3v_0, *e3t = c->e3t_0;
  double *G = zalloc(n3);
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      double C = 0.0;
      for (int jk = 1; jk <= jpk - 1; ++jk) {
        const size_t q = I3(ji, jj, jk);
        C += wn_ad[q];
        const double hd = -(e3t[q] * c->tmask[q]) * C;
        G[q] = hd * c->r1_e1e2t[I2(ji, jj)] / e3t[q];
      }
    }
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jk), p = I2(ji, jj);
        un_ad[q] += c->e2u[p] * e3u[q] * G[q];
        un_ad[I3(ji - 1, jj, jk)] -= c->e2u[I2(ji - 1, jj)] * e3u[I3(ji - 1, jj, jk)] * G[q];
        vn_ad[q] += c->e1v[p] * e3v[q] * G[q];
        vn_ad[I3(ji, jj - 1, jk)] -= c->e1v[I2(ji, jj - 1)] * e3v[I3(ji, jj - 1, jk)] * G[q];
      }
  memset(wn_ad, 0, n3 * sizeof(double));
  wfree(G);
  return NEMO_OK;
}

/* Adjoint of ora_dyn_nxt (dynnxt.F90:66-377, linear free surface, ln_bt_fw), the
 * roles of nemo_nxt_adj. Reverse order: the barotropic velocities, the return of ub
 * to the time-split estimate, the Asselin filter and swap (or the Euler swap), the
 * lbc and the replacement of the barotropic part of ua by ua_b. */
int ora_dyn_nxt_adj(ora_ctx *c, int kt, const nemo_nxt_adj *A) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  if (!A || !A->ua || !A->va || !A->un || !A->vn || !A->ub || !A->vb || !A->un_b || !A->vn_b || !A->ub_b ||
      !A->vb_b || !A->ua_b || !A->va_b)
    return NEMO_ERR_ARG;
  if (!nm->ln_linssh || !nm->ln_bt_fw) return NEMO_ERR_UNSUPPORTED;
  const int euler = nm->neuler == 0 && kt == nm->nit000;
  const double atfp = nm->rn_atfp;
  for (int dir = 0; dir < 2; ++dir) {
    double *ua = dir ? A->va : A->ua, *un = dir ? A->vn : A->un, *ub = dir ? A->vb : A->ub;
    double *unb = dir ? A->vn_b : A->un_b, *ubb = dir ? A->vb_b : A->ub_b, *uab = dir ? A->va_b : A->ua_b;
    const double *e3 = dir ? c->e3v_0 : c->e3u_0, *msk = dir ? c->vmask : c->umask, *r1h = dir ? c->r1_hv_0 : c->r1_hu_0;
    const char nat = dir ? 'V' : 'U';
    for (size_t p = 0; p < n2; ++p) {
      /* (:345-358) the barotropic velocities of the next step */
      double su = 0.0;
      for (int jk = 1; jk <= jpk - 1; ++jk) {
        const size_t q = p + n2 * (jk - 1);
        un[q] += e3[q] * msk[q] * r1h[p] * unb[p];
        ub[q] += e3[q] * msk[q] * r1h[p] * ubb[p];
      }
      unb[p] = 0.0; ubb[p] = 0.0;
      if (!euler) {
        /* (:312-324) ub returned to the time-split estimate */
        for (int jk = 1; jk <= jpk - 1; ++jk) su += ub[p + n2 * (jk - 1)] * msk[p + n2 * (jk - 1)];
        unb[p] += su;
        const double zad = -su * r1h[p];
        for (int jk = 1; jk <= jpk - 1; ++jk) {
          const size_t q = p + n2 * (jk - 1);
          ub[q] += e3[q] * msk[q] * zad;
          /* (:197-211) the Asselin filter and swap */
          const double b = ub[q];
          ua[q] += un[q] + atfp * b;
          un[q] = (1.0 - 2.0 * atfp) * b;
          ub[q] = atfp * b;
        }
      } else {
        for (int jk = 1; jk <= jpk - 1; ++jk) {   /* (:168-171) */
          const size_t q = p + n2 * (jk - 1);
          ua[q] += un[q];
          un[q] = 0.0;
        }
      }
    }
    lbc_closed(jpi, jpj, ua, jpk, nat, 0.0);   /* (:146) */
    for (size_t p = 0; p < n2; ++p) {           /* (:114-126) */
      double s = 0.0;
      for (int jk = 1; jk <= jpk - 1; ++jk) {
        const size_t q = p + n2 * (jk - 1);
        ua[q] = ua[q] * msk[q];
        s += ua[q];
      }
      uab[p] += s;
      const double zad = -s * r1h[p];
      for (int jk = 1; jk <= jpk - 1; ++jk) {
        const size_t q = p + n2 * (jk - 1);
        ua[q] += e3[q] * msk[q] * zad;
      }
    }
  }
  return NEMO_OK;
}

/* Adjoint of ora_ssh_swp (sshwzv.F90:216-267), linear free surface. */
int ora_ssh_swp_adj(ora_ctx *c, int kt, double *sshb_ad, double *sshn_ad, double *ssha_ad) {
  const nemo_namelist *nm = &c->nam;
  const size_t n2 = (size_t)c->jpi * c->jpj;
  if (!sshb_ad || !sshn_ad || !ssha_ad) return NEMO_ERR_ARG;
  if (!nm->ln_linssh) return NEMO_ERR_UNSUPPORTED;
  const double atfp = nm->rn_atfp;
  for (size_t p = 0; p < n2; ++p) {
    if (nm->neuler == 0 && kt == nm->nit000) {
      ssha_ad[p] += sshn_ad[p];
      sshn_ad[p] = 0.0;
    } else {
      const double b = sshb_ad[p];
      ssha_ad[p] += sshn_ad[p] + atfp * b;
      sshn_ad[p] = (1.0 - 2.0 * atfp) * b;
      sshb_ad[p] = atfp * b;
    }
  }
  return NEMO_OK;
}

/* ======================================================= the rest of the step */
/* The parts of stp (step.F90:96-305) that close the path into a time step with the
 * linear free surface: the vertical velocity, the time step and the swaps of the
 * momentum and the sea surface height. */

/* div_hor (divhor.F90:62-110) and wzv (sshwzv.F90:129-213) on the bound un, vn, wn. */
int ora_wzv(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const double *un = c->f[NEMO_F_UN], *vn = c->f[NEMO_F_VN];
  double *wn = c->f[NEMO_F_WN];
  if (!un || !vn || !wn) return NEMO_ERR_UNBOUND;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N), *e3t_n = fld(c, NEMO_F_E3T_N);
  const double *e3t_a = fld(c, NEMO_F_E3T_A), *e3t_b = fld(c, NEMO_F_E3T_B);
  double *hdivn = zalloc(n3);
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        hdivn[q] = (c->e2u[I2(ji, jj)] * e3u[q] * un[q] - c->e2u[I2(ji - 1, jj)] * e3u[I3(ji - 1, jj, jk)] * un[I3(ji - 1, jj, jk)]
                    + c->e1v[I2(ji, jj)] * e3v[q] * vn[q] - c->e1v[I2(ji, jj - 1)] * e3v[I3(ji, jj - 1, jk)] * vn[I3(ji, jj - 1, jk)])
                   * c->r1_e1e2t[I2(ji, jj)] / e3t_n[q];
      }
  lbc_closed(jpi, jpj, hdivn, jpk, 'T', 0.0);
  double z1_2dt = 1. / (2. * nm->rn_rdt);
  if (nm->neuler == 0 && kt == nm->nit000) z1_2dt = 1. / nm->rn_rdt;
  for (size_t p = 0; p < n2; ++p) wn[p + n2 * (jpk - 1)] = 0.0;
  for (int jk = jpk - 1; jk >= 1; --jk)
    for (size_t p = 0; p < n2; ++p) {
      size_t q = p + n2 * (jk - 1);
      wn[q] = wn[q + n2] - (e3t_n[q] * hdivn[q] + z1_2dt * (e3t_a[q] - e3t_b[q])) * c->tmask[q];
    }
  wfree(hdivn);
  return NEMO_OK;
}

/* dyn_zdf (dynzdf.F90:47-499). The leap-frog time step ua = (ub + r2dt ua) umask
 * (:112); then, where the ocean viscosity AVM is bound, the implicit vertical
 * viscosity of a linear free surface with the split-explicit free surface and
 * implicit bottom drag (ln_drgimp, the reference's default), iso-level lateral
 * mixing and no adaptive-implicit advection: the barotropic after velocity ua_b
 * removed (:122-126) and its bottom stress added (:127-141), the matrix of avm
 * (:205-232) with the implicit drag on the bottom diagonal (:243-250), and the
 * Thomas solve with the wind stress (utau_b + utau) / 2 in the surface right-hand
 * side (:266-302); u then v. utau_b, vtau_b: the bound ones, else utau, vtau. The
 * U- and V-W scale factors are the MIN of the neighbouring e3w_0 (domzgr). */
int ora_dyn_zdf_step(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n3 = (size_t)jpi * jpj * jpk, n2 = (size_t)jpi * jpj;
  double *ua = c->f[NEMO_F_UA], *va = c->f[NEMO_F_VA];
  const double *ub = c->f[NEMO_F_UB], *vb = c->f[NEMO_F_VB];
  if (!ua || !va || !ub || !vb) return NEMO_ERR_UNBOUND;
  const double r2dt = (nm->neuler == 0 && kt == nm->nit000) ? nm->rn_rdt : 2. * nm->rn_rdt;
  if (!nm->ln_linssh && !nm->ln_dynadv_vec) {   /* (:115-120) on the thickness-weighted velocity */
    const double *e3u_b = c->f[NEMO_F_E3U_B], *e3v_b = c->f[NEMO_F_E3V_B], *e3u_a = c->f[NEMO_F_E3U_A];
    const double *e3v_a = c->f[NEMO_F_E3V_A], *e3u_n = c->f[NEMO_F_E3U_N], *e3v_n = c->f[NEMO_F_E3V_N];
    if (!e3u_b || !e3v_b || !e3u_a || !e3v_a || !e3u_n || !e3v_n) return NEMO_ERR_UNBOUND;
    for (size_t q = 0; q < n3 - n2; ++q) {
      ua[q] = (e3u_b[q] * ub[q] + r2dt * e3u_n[q] * ua[q]) / e3u_a[q] * c->umask[q];
      va[q] = (e3v_b[q] * vb[q] + r2dt * e3v_n[q] * va[q]) / e3v_a[q] * c->vmask[q];
    }
  } else {                                        /* (:109-114) */
    for (size_t q = 0; q < n3 - n2; ++q) {
      ua[q] = (ub[q] + r2dt * ua[q]) * c->umask[q];
      va[q] = (vb[q] + r2dt * va[q]) * c->vmask[q];
    }
  }
  const double *avm = c->f[NEMO_F_AVM];
  if (!avm) return NEMO_OK;
  const double *ua_b = c->f[NEMO_F_UA_B], *va_b = c->f[NEMO_F_VA_B], *rcdu = c->f[NEMO_F_RCDU_BOT];
  const double *utau = c->f[NEMO_F_UTAU], *vtau = c->f[NEMO_F_VTAU];
  const double *utau_b = c->f[NEMO_F_UTAU_B] ? c->f[NEMO_F_UTAU_B] : utau;
  const double *vtau_b = c->f[NEMO_F_VTAU_B] ? c->f[NEMO_F_VTAU_B] : vtau;
  if (!ua_b || !va_b || !rcdu || !utau || !vtau) return NEMO_ERR_UNBOUND;
  if (!nm->ln_linssh || nm->ln_isfcav || nm->ln_zad_Aimp) return NEMO_ERR_UNSUPPORTED;
  const double *umask = c->umask, *vmask = c->vmask;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N), *e3w = fld(c, NEMO_F_E3W_N);
  const double zdt = r2dt * 0.5, rau0 = nm->rau0;
  for (int jk = 1; jk <= jpk - 1; ++jk)  /* (:122-126) */
    for (size_t p = 0; p < n2; ++p) {
      const size_t q = p + n2 * (jk - 1);
      ua[q] = (ua[q] - ua_b[p]) * umask[q];
      va[q] = (va[q] - va_b[p]) * vmask[q];
    }
  for (int jj = 2; jj <= jpj - 1; ++jj)  /* (:127-141) */
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      const size_t p = I2(ji, jj);
      const int iku = c->mbku[p], ikv = c->mbkv[p];
      ua[I3(ji, jj, iku)] = ua[I3(ji, jj, iku)] +
                            r2dt * 0.5 * (rcdu[I2(ji + 1, jj)] + rcdu[p]) * ua_b[p] / e3u[I3(ji, jj, iku)];
      va[I3(ji, jj, ikv)] = va[I3(ji, jj, ikv)] +
                            r2dt * 0.5 * (rcdu[I2(ji, jj + 1)] + rcdu[p]) * va_b[p] / e3v[I3(ji, jj, ikv)];
    }
  double *zwi = zalloc(n3), *zwd = zalloc(n3), *zws = zalloc(n3);
  for (int comp = 0; comp < 2; ++comp) {
    const int u = comp == 0;
    double *pa = u ? ua : va;
    const double *mask = u ? umask : vmask, *e3 = u ? e3u : e3v, *tau = u ? utau : vtau, *tau_b = u ? utau_b : vtau_b;
    const int *mbk = u ? c->mbku : c->mbkv;
    const size_t nb = u ? 1 : (size_t)jpi;  /* the neighbour across the U- (V-) point */
#define WXM(q, jk) ((jk) == 1 ? mask[q] : mask[q] * mask[(q) - n2])
#define E3XW(q) dmin(e3w[q], e3w[(q) + nb])
    for (int jk = 1; jk <= jpk - 1; ++jk)  /* matrix (:222-232) */
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          const double ze3a = e3[q];
          const double zzwi = -zdt * (avm[q + nb] + avm[q]) / (ze3a * E3XW(q)) * WXM(q, jk);
          const double zzws = -zdt * (avm[q + n2 + nb] + avm[q + n2]) / (ze3a * E3XW(q + n2)) * WXM(q + n2, jk + 1);
          zwi[q] = zzwi;
          zws[q] = zzws;
          zwd[q] = 1. - zzwi - zzws;
        }
    for (int jj = 2; jj <= jpj - 1; ++jj)  /* surface (:234-239), implicit bottom drag (:243-250) */
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj), qb = I3(ji, jj, mbk[p]);
        zwi[p] = 0.;
        zwd[p] = 1. - zws[p];
        zwd[qb] = zwd[qb] - r2dt * 0.5 * (rcdu[p + nb] + rcdu[p]) / e3[qb];
      }
    for (int jk = 2; jk <= jpk - 1; ++jk)  /* first recurrence (:266-272) */
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          zwd[q] = zwd[q] - zwi[q] * zws[q - n2] / zwd[q - n2];
        }
    for (int jj = 2; jj <= jpj - 1; ++jj)  /* wind stress (:274-279) */
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj);
        pa[p] = pa[p] + r2dt * 0.5 * (tau_b[p] + tau[p]) / (e3[p] * rau0) * mask[p];
      }
    for (int jk = 2; jk <= jpk - 1; ++jk)  /* second recurrence (:280-286) */
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          pa[q] = pa[q] - zwi[q] / zwd[q - n2] * pa[q - n2];
        }
    for (int jj = 2; jj <= jpj - 1; ++jj)  /* third recurrence (:288-299) */
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jpk - 1);
        pa[q] = pa[q] / zwd[q];
      }
    for (int jk = jpk - 2; jk >= 1; --jk)
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          pa[q] = (pa[q] - zws[q] * pa[q + n2]) / zwd[q];
        }
#undef WXM
#undef E3XW
  }
  wfree(zwi); wfree(zwd); wfree(zws);
  return NEMO_OK;
}

/* ----------------------------------------------------- z* scale factors */
/* dom_vvl_interpol (domvvl.F90:678-782) without wetting and drying (zlnwd = 0): the
 * scale factor at the out point is its rest state plus the change of pe3_in,
 * surface-weighted between two neighbours ('U', 'V', 'F', then lbc_lnk) or averaged
 * between two levels ('W', 'UW', 'VW'). */
static int vvl_interpol(const ora_ctx *c, const double *in, double *out, char pout, int w) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  if (!w) {                                               /* U, V, F: :705-742 */
    const double *in0 = pout == 'F' ? c->e3u_0 : c->e3t_0;
    const double *out0 = pout == 'U' ? c->e3u_0 : pout == 'V' ? c->e3v_0 : c->e3f_0;
    for (int jk = 1; jk <= jpk; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          const size_t p = I2(ji, jj), q = I3(ji, jj, jk);
          if (pout == 'U') {
            const size_t p1 = I2(ji + 1, jj), q1 = I3(ji + 1, jj, jk);
            out[q] = 0.5 * (c->umask[q] * (1.0 - 0.0) + 0.0) * c->r1_e1e2u[p] *
                     (c->e1e2t[p] * (in[q] - in0[q]) + c->e1e2t[p1] * (in[q1] - in0[q1]));
          } else if (pout == 'V') {
            const size_t p1 = I2(ji, jj + 1), q1 = I3(ji, jj + 1, jk);
            out[q] = 0.5 * (c->vmask[q] * (1.0 - 0.0) + 0.0) * c->r1_e1e2v[p] *
                     (c->e1e2t[p] * (in[q] - in0[q]) + c->e1e2t[p1] * (in[q1] - in0[q1]));
          } else {
            const size_t p1 = I2(ji, jj + 1), q1 = I3(ji, jj + 1, jk);
            const double r1_e1e2f = 1.0 / (c->e1f[p] * c->e2f[p]);
            out[q] = 0.5 * (c->umask[q] * c->umask[q1] * (1.0 - 0.0) + 0.0) * r1_e1e2f *
                     (c->e1e2u[p] * (in[q] - in0[q]) + c->e1e2u[p1] * (in[q1] - in0[q1]));
          }
        }
    lbc_closed(jpi, jpj, out, jpk, pout, 0.0);
    for (size_t q = 0; q < n2 * jpk; ++q) out[q] = out[q] + out0[q];
    return NEMO_OK;
  }
  /* W, UW, VW: :744-779 */
  const double *out0 = pout == 'W' ? c->e3w_0 : pout == 'U' ? c->f[NEMO_F_E3UW_0] : c->f[NEMO_F_E3VW_0];
  const double *in0 = pout == 'W' ? c->e3t_0 : pout == 'U' ? c->e3u_0 : c->e3v_0;
  const double *msk = pout == 'W' ? c->tmask : pout == 'U' ? c->umask : c->vmask;
  if (!out0) return NEMO_ERR_UNBOUND;
  for (size_t p = 0; p < n2; ++p) out[p] = out0[p] + in[p] - in0[p];
  for (int jk = 2; jk <= jpk; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      const size_t q = p + n2 * (jk - 1), qm = q - n2;
      const double m = msk[q] * (1.0 - 0.0) + 0.0;
      out[q] = out0[q] + (1.0 - 0.5 * m) * (in[qm] - in0[qm]) + 0.5 * m * (in[q] - in0[q]);
    }
  return NEMO_OK;
}

/* a column depth and its masked inverse: h = sum of e3 mask over the levels 1..jpkm1,
 * r1_h = ssmask / (h + 1 - ssmask) (domvvl.F90:549-558) */
static void vvl_depth(const ora_ctx *c, const double *e3, const double *msk, const double *ssm, double *h,
                      double *r1_h) {
  const size_t n2 = (size_t)c->jpi * c->jpj;
  for (size_t p = 0; p < n2; ++p) h[p] = e3[p] * msk[p];
  for (int jk = 2; jk <= c->jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) h[p] = h[p] + e3[p + n2 * (jk - 1)] * msk[p + n2 * (jk - 1)];
  if (r1_h)
    for (size_t p = 0; p < n2; ++p) r1_h[p] = ssm[p] / (h[p] + 1.0 - ssm[p]);
}

/* dom_vvl_sf_nxt (domvvl.F90:268-562), z*: the after scale factors from the ssh
 * increment (:323-327), at u- and v-points (:542-543), the after column depths. */
int ora_dom_vvl_sf_nxt(ora_ctx *c, int kt) {
  (void)kt;
  double **F = c->f;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  if (c->nam.ln_linssh) return NEMO_ERR_ARG;
  const double *ssha = F[NEMO_F_SSHA], *sshb = F[NEMO_F_SSHB], *sshn = F[NEMO_F_SSHN];
  const double *e3t_b = F[NEMO_F_E3T_B], *e3t_n = F[NEMO_F_E3T_N];
  double *e3t_a = F[NEMO_F_E3T_A], *e3u_a = F[NEMO_F_E3U_A], *e3v_a = F[NEMO_F_E3V_A];
  double *hu_a = F[NEMO_F_HU_A], *hv_a = F[NEMO_F_HV_A], *r1_hu_a = F[NEMO_F_R1_HU_A], *r1_hv_a = F[NEMO_F_R1_HV_A];
  if (!ssha || !sshb || !sshn || !e3t_b || !e3t_n || !e3t_a || !e3u_a || !e3v_a || !hu_a || !hv_a || !r1_hu_a ||
      !r1_hv_a)
    return NEMO_ERR_UNBOUND;
  (void)jpi; (void)jpj;
  for (size_t p = 0; p < n2; ++p) {
    const double z_scale = (ssha[p] - sshb[p]) * c->ssmask[p] / (c->ht_0[p] + sshn[p] + 1. - c->ssmask[p]);
    for (int jk = 1; jk <= jpk - 1; ++jk) {
      const size_t q = p + n2 * (jk - 1);
      e3t_a[q] = e3t_b[q] + e3t_n[q] * z_scale * c->tmask[q];
    }
  }
  vvl_interpol(c, e3t_a, e3u_a, 'U', 0);
  vvl_interpol(c, e3t_a, e3v_a, 'V', 0);
  vvl_depth(c, e3u_a, c->umask, c->ssumask, hu_a, r1_hu_a);
  vvl_depth(c, e3v_a, c->vmask, c->ssvmask, hv_a, r1_hv_a);
  return NEMO_OK;
}

/* dom_vvl_sf_swp (domvvl.F90:565-675), z*: the swap of the scale factors, the now
 * and before e3 at w-, f-, uw- and vw-points, the now depths and column depths. The
 * optional outputs are formed when bound. */
int ora_dom_vvl_sf_swp(ora_ctx *c, int kt) {
  (void)kt;
  double **F = c->f;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  if (c->nam.ln_linssh) return NEMO_ERR_ARG;
  double *e3t_n = F[NEMO_F_E3T_N], *e3u_n = F[NEMO_F_E3U_N], *e3v_n = F[NEMO_F_E3V_N], *e3w_n = F[NEMO_F_E3W_N];
  const double *e3t_a = F[NEMO_F_E3T_A], *e3u_a = F[NEMO_F_E3U_A], *e3v_a = F[NEMO_F_E3V_A], *e3t_b = F[NEMO_F_E3T_B];
  const double *sshn = F[NEMO_F_SSHN];
  if (!e3t_n || !e3u_n || !e3v_n || !e3w_n || !e3t_a || !e3u_a || !e3v_a || !e3t_b || !sshn || !F[NEMO_F_HU_A] ||
      !F[NEMO_F_HV_A] || !F[NEMO_F_R1_HU_A] || !F[NEMO_F_R1_HV_A] || !F[NEMO_F_HU_N] || !F[NEMO_F_HV_N] ||
      !F[NEMO_F_R1_HU_N] || !F[NEMO_F_R1_HV_N] || !F[NEMO_F_HT_N])
    return NEMO_ERR_UNBOUND;
  if ((F[NEMO_F_E3UW_N] || F[NEMO_F_E3UW_B]) && !F[NEMO_F_E3UW_0]) return NEMO_ERR_UNBOUND;
  if ((F[NEMO_F_E3VW_N] || F[NEMO_F_E3VW_B]) && !F[NEMO_F_E3VW_0]) return NEMO_ERR_UNBOUND;
  if ((F[NEMO_F_E3UW_B] && !F[NEMO_F_E3U_B]) || (F[NEMO_F_E3VW_B] && !F[NEMO_F_E3V_B])) return NEMO_ERR_UNBOUND;
  double *gdept = F[NEMO_F_GDEPT_N], *gdepw = F[NEMO_F_GDEPW_N], *gde3w = F[NEMO_F_GDE3W_N];
  if (F[NEMO_F_GDEPT_B] && gdept) memcpy(F[NEMO_F_GDEPT_B], gdept, n3 * sizeof(double));   /* :617-618 */
  if (F[NEMO_F_GDEPW_B] && gdepw) memcpy(F[NEMO_F_GDEPW_B], gdepw, n3 * sizeof(double));
  memcpy(e3t_n, e3t_a, n3 * sizeof(double));                                               /* :620-622 */
  memcpy(e3u_n, e3u_a, n3 * sizeof(double));
  memcpy(e3v_n, e3v_a, n3 * sizeof(double));
  if (F[NEMO_F_E3F_N]) vvl_interpol(c, e3u_n, F[NEMO_F_E3F_N], 'F', 0);                     /* :631 */
  vvl_interpol(c, e3t_n, e3w_n, 'W', 1);                                                    /* :634-640 */
  if (F[NEMO_F_E3UW_N]) vvl_interpol(c, e3u_n, F[NEMO_F_E3UW_N], 'U', 1);
  if (F[NEMO_F_E3VW_N]) vvl_interpol(c, e3v_n, F[NEMO_F_E3VW_N], 'V', 1);
  if (F[NEMO_F_E3W_B]) vvl_interpol(c, e3t_b, F[NEMO_F_E3W_B], 'W', 1);
  if (F[NEMO_F_E3UW_B]) vvl_interpol(c, F[NEMO_F_E3U_B], F[NEMO_F_E3UW_B], 'U', 1);
  if (F[NEMO_F_E3VW_B]) vvl_interpol(c, F[NEMO_F_E3V_B], F[NEMO_F_E3VW_B], 'V', 1);
  if (gdept && gdepw) {                                                                     /* :642-657 */
    for (size_t p = 0; p < n2; ++p) {
      gdept[p] = 0.5 * e3w_n[p];
      gdepw[p] = 0.0;
      if (gde3w) gde3w[p] = gdept[p] - sshn[p];
    }
    for (int jk = 2; jk <= jpk; ++jk)
      for (size_t p = 0; p < n2; ++p) {
        const size_t q = p + n2 * (jk - 1), qm = q - n2;
        const double zcoef = c->tmask[q] - c->wmask[q];
        gdepw[q] = gdepw[qm] + e3t_n[qm];
        gdept[q] = zcoef * (gdepw[q] + 0.5 * e3w_n[q]) + (1 - zcoef) * (gdept[qm] + e3w_n[q]);
        if (gde3w) gde3w[q] = gdept[q] - sshn[p];
      }
  }
  memcpy(F[NEMO_F_HU_N], F[NEMO_F_HU_A], n2 * sizeof(double));                              /* :661-662 */
  memcpy(F[NEMO_F_R1_HU_N], F[NEMO_F_R1_HU_A], n2 * sizeof(double));
  memcpy(F[NEMO_F_HV_N], F[NEMO_F_HV_A], n2 * sizeof(double));
  memcpy(F[NEMO_F_R1_HV_N], F[NEMO_F_R1_HV_A], n2 * sizeof(double));
  vvl_depth(c, e3t_n, c->tmask, NULL, F[NEMO_F_HT_N], NULL);                                /* :664-667 */
  return NEMO_OK;
}

/* dyn_nxt (dynnxt.F90:66-377) with ln_dynspg_ts and ln_bt_fw; with a variable
 * volume the after e3 and column depths of dom_vvl_sf_nxt, the time filter of e3t_b
 * (:217-226, runoff only with ln_rnf: not on this path), e3u_b / e3v_b from it, and
 * the filter on the velocity (ln_dynadv_vec) or on the thickness-weighted velocity. */
int ora_dyn_nxt(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  double **F = c->f;
  double *ua = F[NEMO_F_UA], *va = F[NEMO_F_VA], *un = F[NEMO_F_UN], *vn = F[NEMO_F_VN];
  double *ub = F[NEMO_F_UB], *vb = F[NEMO_F_VB];
  double *un_b = F[NEMO_F_UN_B], *vn_b = F[NEMO_F_VN_B], *ub_b = F[NEMO_F_UB_B], *vb_b = F[NEMO_F_VB_B];
  const double *ua_b = F[NEMO_F_UA_B], *va_b = F[NEMO_F_VA_B];
  if (!ua || !va || !un || !vn || !ub || !vb || !un_b || !vn_b || !ub_b || !vb_b || !ua_b || !va_b)
    return NEMO_ERR_UNBOUND;
  if (!nm->ln_bt_fw) return NEMO_ERR_ARG;
  const int vvl = !nm->ln_linssh;
  const double *umask = c->umask, *vmask = c->vmask;
  const double *e3u_a = c->e3u_0, *e3v_a = c->e3v_0, *r1_hu_a = c->r1_hu_0, *r1_hv_a = c->r1_hv_0;
  const double *r1_hu_n = c->r1_hu_0, *r1_hv_n = c->r1_hv_0;
  double *e3u_b = c->e3u_0, *e3v_b = c->e3v_0, *r1_hu_b = c->r1_hu_0, *r1_hv_b = c->r1_hv_0;
  if (vvl) {
    const int need[] = {NEMO_F_E3T_B, NEMO_F_E3T_N, NEMO_F_E3T_A, NEMO_F_E3U_N, NEMO_F_E3V_N, NEMO_F_E3U_A,
                        NEMO_F_E3V_A, NEMO_F_E3U_B, NEMO_F_E3V_B, NEMO_F_R1_HU_A, NEMO_F_R1_HV_A, NEMO_F_R1_HU_N,
                        NEMO_F_R1_HV_N, NEMO_F_HU_B, NEMO_F_HV_B, NEMO_F_R1_HU_B, NEMO_F_R1_HV_B, NEMO_F_EMP,
                        NEMO_F_EMP_B};
    for (size_t i = 0; i < sizeof need / sizeof need[0]; ++i)
      if (!F[need[i]]) return NEMO_ERR_UNBOUND;
    e3u_a = F[NEMO_F_E3U_A]; e3v_a = F[NEMO_F_E3V_A]; r1_hu_a = F[NEMO_F_R1_HU_A]; r1_hv_a = F[NEMO_F_R1_HV_A];
    r1_hu_n = F[NEMO_F_R1_HU_N]; r1_hv_n = F[NEMO_F_R1_HV_N];
    e3u_b = F[NEMO_F_E3U_B]; e3v_b = F[NEMO_F_E3V_B]; r1_hu_b = F[NEMO_F_R1_HU_B]; r1_hv_b = F[NEMO_F_R1_HV_B];
  }
  const double atfp = nm->rn_atfp;
  double *zue = zalloc(n2), *zve = zalloc(n2);
  /* (:114-126) the barotropic part of the after velocity from the sub-steps */
  for (size_t p = 0; p < n2; ++p) { zue[p] = e3u_a[p] * ua[p] * umask[p]; zve[p] = e3v_a[p] * va[p] * vmask[p]; }
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      size_t q = p + n2 * (jk - 1);
      zue[p] = zue[p] + e3u_a[q] * ua[q] * umask[q];
      zve[p] = zve[p] + e3v_a[q] * va[q] * vmask[q];
    }
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      size_t q = p + n2 * (jk - 1);
      ua[q] = (ua[q] - zue[p] * r1_hu_a[p] + ua_b[p]) * umask[q];
      va[q] = (va[q] - zve[p] * r1_hv_a[p] + va_b[p]) * vmask[q];
    }
  lbc_closed(jpi, jpj, ua, jpk, 'U', 0.0);                    /* :146 */
  lbc_closed(jpi, jpj, va, jpk, 'V', 0.0);
  if (nm->neuler == 0 && kt == nm->nit000) {                 /* :168-188 Euler: swap only */
    memcpy(un, ua, (size_t)(jpk - 1) * n2 * sizeof(double));
    memcpy(vn, va, (size_t)(jpk - 1) * n2 * sizeof(double));
    if (vvl) {                                                /* :172-186 */
      memcpy(F[NEMO_F_E3T_N], F[NEMO_F_E3T_A], (size_t)(jpk - 1) * n2 * sizeof(double));
      memcpy(F[NEMO_F_E3U_N], F[NEMO_F_E3U_A], (size_t)(jpk - 1) * n2 * sizeof(double));
      memcpy(F[NEMO_F_E3V_N], F[NEMO_F_E3V_A], (size_t)(jpk - 1) * n2 * sizeof(double));
    }
  } else {
    double *ze3u_f = NULL, *ze3v_f = NULL;
    if (vvl) {                                                /* :217-226 e3t_b filtered */
      double *e3t_b = F[NEMO_F_E3T_B];
      const double *e3t_n = F[NEMO_F_E3T_N], *e3t_a = F[NEMO_F_E3T_A];
      for (size_t q = 0; q < n3 - n2; ++q) e3t_b[q] = e3t_n[q] + atfp * (e3t_b[q] - 2. * e3t_n[q] + e3t_a[q]);
      const double zcoef = atfp * nm->rn_rdt * (1.0 / nm->rau0);
      const double *emp = F[NEMO_F_EMP], *emp_b = F[NEMO_F_EMP_B];
      for (size_t p = 0; p < n2; ++p) e3t_b[p] = e3t_b[p] - zcoef * (emp_b[p] - emp[p]) * c->tmask[p];
      if (nm->ln_dynadv_vec) {                                /* :262-263 */
        vvl_interpol(c, e3t_b, e3u_b, 'U', 0);
        vvl_interpol(c, e3t_b, e3v_b, 'V', 0);
      } else {                                                /* :282-283 */
        ze3u_f = walloc(n3); ze3v_f = walloc(n3);
        vvl_interpol(c, e3t_b, ze3u_f, 'U', 0);
        vvl_interpol(c, e3t_b, ze3v_f, 'V', 0);
      }
    }
    if (!ze3u_f) {                                            /* :195-211, :264-276 */
      for (int jk = 1; jk <= jpk - 1; ++jk)
        for (size_t p = 0; p < n2; ++p) {
          size_t q = p + n2 * (jk - 1);
          double zuf = un[q] + atfp * (ub[q] - 2.0 * un[q] + ua[q]);
          double zvf = vn[q] + atfp * (vb[q] - 2.0 * vn[q] + va[q]);
          ub[q] = zuf; vb[q] = zvf;
          un[q] = ua[q]; vn[q] = va[q];
        }
    } else {                                                  /* :284-305 thickness-weighted */
      const double *e3u_n = F[NEMO_F_E3U_N], *e3v_n = F[NEMO_F_E3V_N];
      for (size_t q = 0; q < n3 - n2; ++q) {
        const double zue3a = e3u_a[q] * ua[q], zve3a = e3v_a[q] * va[q];
        const double zue3n = e3u_n[q] * un[q], zve3n = e3v_n[q] * vn[q];
        const double zue3b = e3u_b[q] * ub[q], zve3b = e3v_b[q] * vb[q];
        const double zuf = (zue3n + atfp * (zue3b - 2. * zue3n + zue3a)) / ze3u_f[q];
        const double zvf = (zve3n + atfp * (zve3b - 2. * zve3n + zve3a)) / ze3v_f[q];
        ub[q] = zuf; vb[q] = zvf;
        un[q] = ua[q]; vn[q] = va[q];
      }
      memcpy(e3u_b, ze3u_f, (n3 - n2) * sizeof(double));      /* :304-305 */
      memcpy(e3v_b, ze3v_f, (n3 - n2) * sizeof(double));
      wfree(ze3u_f); wfree(ze3v_f);
    }
    /* (:312-324) the before velocity back to the time-split barotropic estimate */
    for (size_t p = 0; p < n2; ++p) { zue[p] = e3u_b[p] * ub[p] * umask[p]; zve[p] = e3v_b[p] * vb[p] * vmask[p]; }
    for (int jk = 2; jk <= jpk - 1; ++jk)
      for (size_t p = 0; p < n2; ++p) {
        size_t q = p + n2 * (jk - 1);
        zue[p] = zue[p] + e3u_b[q] * ub[q] * umask[q];
        zve[p] = zve[p] + e3v_b[q] * vb[q] * vmask[q];
      }
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (size_t p = 0; p < n2; ++p) {
        size_t q = p + n2 * (jk - 1);
        ub[q] = ub[q] - (zue[p] * r1_hu_n[p] - un_b[p]) * umask[q];
        vb[q] = vb[q] - (zve[p] * r1_hv_n[p] - vn_b[p]) * vmask[q];
      }
  }
  if (vvl) {                                                  /* :334-343 */
    vvl_depth(c, e3u_b, umask, c->ssumask, F[NEMO_F_HU_B], r1_hu_b);
    vvl_depth(c, e3v_b, vmask, c->ssvmask, F[NEMO_F_HV_B], r1_hv_b);
  }
  /* (:345-358) now and before barotropic velocities for the next step */
  for (size_t p = 0; p < n2; ++p) {
    un_b[p] = e3u_a[p] * un[p] * umask[p]; ub_b[p] = e3u_b[p] * ub[p] * umask[p];
    vn_b[p] = e3v_a[p] * vn[p] * vmask[p]; vb_b[p] = e3v_b[p] * vb[p] * vmask[p];
  }
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      size_t q = p + n2 * (jk - 1);
      un_b[p] = un_b[p] + e3u_a[q] * un[q] * umask[q]; ub_b[p] = ub_b[p] + e3u_b[q] * ub[q] * umask[q];
      vn_b[p] = vn_b[p] + e3v_a[q] * vn[q] * vmask[q]; vb_b[p] = vb_b[p] + e3v_b[q] * vb[q] * vmask[q];
    }
  for (size_t p = 0; p < n2; ++p) {
    un_b[p] = un_b[p] * r1_hu_a[p]; vn_b[p] = vn_b[p] * r1_hv_a[p];
    ub_b[p] = ub_b[p] * r1_hu_b[p]; vb_b[p] = vb_b[p] * r1_hv_b[p];
  }
  wfree(zue); wfree(zve);
  return NEMO_OK;
}

/* ssh_swp (sshwzv.F90:216-267); with a variable volume the forcing is removed from
 * the filtered before ssh (:254-258; rnf when bound, no ice-shelf melt). */
int ora_ssh_swp(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  const size_t n2 = (size_t)c->jpi * c->jpj;
  double *sshb = c->f[NEMO_F_SSHB], *sshn = c->f[NEMO_F_SSHN];
  const double *ssha = c->f[NEMO_F_SSHA];
  const double *emp = c->f[NEMO_F_EMP], *emp_b = c->f[NEMO_F_EMP_B];
  const double *rnf = c->f[NEMO_F_RNF], *rnf_b = c->f[NEMO_F_RNF_B];
  if (!sshb || !sshn || !ssha) return NEMO_ERR_UNBOUND;
  if (!nm->ln_linssh && (!emp || !emp_b || (rnf == NULL) != (rnf_b == NULL))) return NEMO_ERR_UNBOUND;
  if (nm->neuler == 0 && kt == nm->nit000) {
    memcpy(sshn, ssha, n2 * sizeof(double));
  } else {
    const double zcoef = nm->rn_atfp * nm->rn_rdt * (1.0 / nm->rau0);
    for (size_t p = 0; p < n2; ++p) {
      sshb[p] = sshn[p] + nm->rn_atfp * (sshb[p] - 2 * sshn[p] + ssha[p]);
      if (!nm->ln_linssh) {
        double zf = emp_b[p] - emp[p];
        if (rnf) zf = zf - rnf_b[p] + rnf[p];
        sshb[p] = sshb[p] - zcoef * zf * c->ssmask[p];
      }
      sshn[p] = ssha[p];
    }
  }
  return NEMO_OK;
}

/* ------------------------------------------------------- surface forcing */
static double rcp_of(const nemo_namelist *nm) { return nm->rcp > 0 ? nm->rcp : 3991.86795711963; }

/* tra_sbc (trasbc.F90:53-206) without runoff and ice-shelf melt: bound QNS, QSR, EMP,
 * SFX, SBC_TSC, SBC_TSC_B (jpi,jpj,2), TSN, TSA. */
int ora_tra_sbc(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj;
  const size_t n2 = (size_t)jpi * jpj;
  double *qns = c->f[NEMO_F_QNS], *qsr = c->f[NEMO_F_QSR];
  const double *emp = c->f[NEMO_F_EMP], *sfx = c->f[NEMO_F_SFX], *tsn = c->f[NEMO_F_TSN];
  double *tsc = c->f[NEMO_F_SBC_TSC], *tsc_b = c->f[NEMO_F_SBC_TSC_B], *tsa = c->f[NEMO_F_TSA];
  if (!qns || !qsr || !emp || !sfx || !tsn || !tsc || !tsc_b || !tsa) return NEMO_ERR_UNBOUND;
  const double *e3t_n = fld(c, NEMO_F_E3T_N);
  const size_t n3 = n2 * c->jpk;
  const double rau0 = nm->rau0, r1_rau0 = 1.0 / rau0, rau0_rcp = rau0 * rcp_of(nm), r1_rau0_rcp = 1.0 / rau0_rcp;
  if (!nm->ln_traqsr)                                        /* :76-79 */
    for (size_t p = 0; p < n2; ++p) { qns[p] = qns[p] + qsr[p]; qsr[p] = 0.0; }
  double zfact;
  if (kt == nm->nit000) {                                    /* :81-96 */
    if (nm->neuler != 0) {              /* restart: sbc_tsc_b holds the restart's sbc_hc_b, sbc_sc_b */
      zfact = 0.5;
      memset(tsc, 0, 2 * n2 * sizeof(double));
    } else {
      zfact = 1.0;
      memset(tsc, 0, 2 * n2 * sizeof(double));
      memset(tsc_b, 0, 2 * n2 * sizeof(double));
    }
  } else {                                                   /* :97-100 */
    zfact = 0.5;
    memcpy(tsc_b, tsc, 2 * n2 * sizeof(double));
  }
  for (int jj = 2; jj <= jpj; ++jj)                          /* :104-109 */
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      tsc[I2(ji, jj)] = r1_rau0_rcp * qns[I2(ji, jj)];
      tsc[n2 + I2(ji, jj)] = r1_rau0 * sfx[I2(ji, jj)];
    }
  if (nm->ln_linssh)                                         /* :111-118 */
    for (int jj = 2; jj <= jpj; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        tsc[I2(ji, jj)] = tsc[I2(ji, jj)] + r1_rau0 * emp[I2(ji, jj)] * tsn[I2(ji, jj)];
        tsc[n2 + I2(ji, jj)] = tsc[n2 + I2(ji, jj)] + r1_rau0 * emp[I2(ji, jj)] * tsn[n3 + I2(ji, jj)];
      }
  for (int jn = 0; jn < 2; ++jn)                             /* :123-129 */
    for (int jj = 2; jj <= jpj; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj);
        tsa[n3 * jn + p] = tsa[n3 * jn + p] + zfact * (tsc_b[n2 * jn + p] + tsc[n2 * jn + p]) / e3t_n[p];
      }
  return NEMO_OK;
}

/* tra_qsr (traqsr.F90:77-302), two bands (np_2BD): bound QSR, QSR_HC, QSR_HC_B,
 * FRAQSR_1LEV, GDEPW_N, TSA. */
int ora_tra_qsr(ora_ctx *c, int kt) {
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const double *qsr = c->f[NEMO_F_QSR], *gdepw = c->f[NEMO_F_GDEPW_N];
  double *hc = c->f[NEMO_F_QSR_HC], *hc_b = c->f[NEMO_F_QSR_HC_B], *fraq = c->f[NEMO_F_FRAQSR_1LEV];
  double *tsa = c->f[NEMO_F_TSA];
  if (!qsr || !gdepw || !hc || !hc_b || !fraq || !tsa) return NEMO_ERR_UNBOUND;
  if (!nm->ln_traqsr) return NEMO_ERR_ARG;
  const double *e3t_n = fld(c, NEMO_F_E3T_N), *wmask = c->wmask;
  const double r1_rau0_rcp = 1.0 / (nm->rau0 * rcp_of(nm));
  const double rn_abs = nm->rn_abs, xsi0r = 1.0 / nm->rn_si0, xsi1r = 1.0 / nm->rn_si1;
  const int nksr = c->nksr;
  double z1_2;
  if (kt == nm->nit000) {                                    /* :134-143 */
    if (nm->neuler != 0) z1_2 = 0.5;    /* restart: qsr_hc_b holds the restart's qsr_hc_b */
    else { z1_2 = 1.0; memset(hc_b, 0, n3 * sizeof(double)); }
  } else {                                                   /* :144-147 */
    z1_2 = 0.5;
    memcpy(hc_b, hc, n3 * sizeof(double));
  }
  const double zz0 = rn_abs * r1_rau0_rcp, zz1 = (1. - rn_abs) * r1_rau0_rcp;   /* :245-255 */
  for (int jk = 1; jk <= nksr; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const double g0 = gdepw[I3(ji, jj, jk)], g1 = gdepw[I3(ji, jj, jk + 1)];
        const double zc0 = zz0 * exp(-g0 * xsi0r) + zz1 * exp(-g0 * xsi1r);
        const double zc1 = zz0 * exp(-g1 * xsi0r) + zz1 * exp(-g1 * xsi1r);
        hc[I3(ji, jj, jk)] = qsr[I2(ji, jj)] * (zc0 * wmask[I3(ji, jj, jk)] - zc1 * wmask[I3(ji, jj, jk + 1)]);
      }
  for (int jk = 1; jk <= nksr; ++jk)                         /* :260-267 */
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t q = I3(ji, jj, jk);
        tsa[q] = tsa[q] + z1_2 * (hc_b[q] + hc[q]) / e3t_n[q];
      }
  for (int jj = 2; jj <= jpj - 1; ++jj)                      /* :270-277 */
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      const size_t p = I2(ji, jj);
      fraq[p] = qsr[p] != 0.0 ? hc[p] / (r1_rau0_rcp * qsr[p]) : 1.0;
    }
  lbc_closed(jpi, jpj, fraq, 1, 'T', 0.0);
  return NEMO_OK;
}

int ora_nksr(const ora_ctx *c) { return c->nksr; }

/* nlb10 (domzgr.F90:144-146): the shallowest W-level deeper than 10 m less a tenth of
 * the thinnest W-layer, on the 1-D reference profile (the rest-state column with
 * the most wet levels: gdepw_1d from its e3t_0 as e3_to_depth sums them). */
static int nlb10_of(const ora_ctx *c) {
  const size_t n2 = (size_t)c->jpi * c->jpj;
  size_t best = 0;
  for (size_t p = 0; p < n2; ++p)
    if (c->mbkt[p] > c->mbkt[best]) best = p;
  double e3wmin = 1e300, gdepw = 0.0;
  for (int jk = 1; jk <= c->jpk; ++jk) e3wmin = dmin(e3wmin, c->e3w_0[best + n2 * (jk - 1)]);
  const double zrefdep = 10.0 - 0.1 * e3wmin;
  for (int jk = 1; jk <= c->jpk; ++jk) {
    if (gdepw > zrefdep) return jk;
    gdepw = gdepw + c->e3t_0[best + n2 * (jk - 1)];
  }
  return c->jpk;
}

/* zdf_mxl (zdfmxl.F90:59-141): bound RN2B, AVT, GDEPT_N, GDEPW_N -> NMLN (int),
 * HMLP, HMLPT, HMLD (when bound). */
int ora_zdf_mxl(ora_ctx *c, int kt) {
  (void)kt;
  const nemo_namelist *nm = &c->nam;
  const int jpk = c->jpk;
  const size_t n2 = (size_t)c->jpi * c->jpj;
  const double *rn2b = c->f[NEMO_F_RN2B], *avt = c->f[NEMO_F_AVT];
  const double *gdept = c->f[NEMO_F_GDEPT_N], *gdepw = c->f[NEMO_F_GDEPW_N];
  int *nmln = (int *)c->f[NEMO_F_NMLN];
  double *hmlp = c->f[NEMO_F_HMLP], *hmlpt = c->f[NEMO_F_HMLPT], *hmld = c->f[NEMO_F_HMLD];
  if (!rn2b || !avt || !gdept || !gdepw || !nmln || !hmlp || !hmlpt) return NEMO_ERR_UNBOUND;
  const double *e3w = fld(c, NEMO_F_E3W_N);
  const int nlb10 = nlb10_of(c);
  const double rho_c = 0.01, avt_c = 5.e-4;
  const double zN2_c = nm->grav * rho_c * (1.0 / nm->rau0);
  for (size_t p = 0; p < n2; ++p) { nmln[p] = nlb10; hmlp[p] = 0.0; }
  for (int jk = nlb10; jk <= jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      const int ikt = c->mbkt[p];
      hmlp[p] = hmlp[p] + dmax(rn2b[p + n2 * (jk - 1)], 0.0) * e3w[p + n2 * (jk - 1)];
      if (hmlp[p] < zN2_c) nmln[p] = (jk < ikt ? jk : ikt) + 1;
    }
  for (size_t p = 0; p < n2; ++p) {
    int imld = c->mbkt[p] + 1;
    for (int jk = jpk - 1; jk >= nlb10; --jk)
      if (avt[p + n2 * (jk - 1)] < avt_c * c->wmask[p + n2 * (jk - 1)]) imld = jk;
    const int iikn = nmln[p];
    if (hmld) hmld[p] = gdepw[p + n2 * (imld - 1)] * c->ssmask[p];
    hmlp[p] = gdepw[p + n2 * (iikn - 1)] * c->ssmask[p];
    hmlpt[p] = gdept[p + n2 * (iikn - 2)] * c->ssmask[p];
  }
  return NEMO_OK;
}

int ora_nlb10(const ora_ctx *c) { return nlb10_of(c); }

/* dyn_keg (dynkeg.F90), nkeg_C2: bound UN, VN, UA, VA. */
int ora_dyn_keg(ora_ctx *c, int kt, int kscheme) {
  (void)kt;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  const double *un = c->f[NEMO_F_UN], *vn = c->f[NEMO_F_VN];
  double *ua = c->f[NEMO_F_UA], *va = c->f[NEMO_F_VA];
  if (!un || !vn || !ua || !va) return NEMO_ERR_UNBOUND;
  if (kscheme != 0) return NEMO_ERR_UNSUPPORTED;
  double *zhke = zalloc(n2);
  for (int jk = 1; jk <= jpk - 1; ++jk) {
    for (int jj = 2; jj <= jpj; ++jj)
      for (int ji = 2; ji <= jpi; ++ji) {
        const size_t q = I3(ji, jj, jk);
        const double zu = un[q - 1] * un[q - 1] + un[q] * un[q];
        const double zv = vn[q - jpi] * vn[q - jpi] + vn[q] * vn[q];
        zhke[I2(ji, jj)] = 0.25 * (zv + zu);
      }
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj), q = I3(ji, jj, jk);
        ua[q] = ua[q] - (zhke[p + 1] - zhke[p]) / c->e1u[p];
        va[q] = va[q] - (zhke[p + jpi] - zhke[p]) / c->e2v[p];
      }
  }
  wfree(zhke);
  return NEMO_OK;
}

/* dyn_zad (dynzad.F90): bound UN, VN, WN, UA, VA. */
int ora_dyn_zad(ora_ctx *c, int kt) {
  (void)kt;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  const double *un = c->f[NEMO_F_UN], *vn = c->f[NEMO_F_VN], *wn = c->f[NEMO_F_WN];
  double *ua = c->f[NEMO_F_UA], *va = c->f[NEMO_F_VA];
  if (!un || !vn || !wn || !ua || !va) return NEMO_ERR_UNBOUND;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N);
  double *zww = zalloc(n2), *zwuw = zalloc(n3), *zwvw = zalloc(n3);
  for (int jk = 2; jk <= jpk - 1; ++jk) {
    for (int jj = 2; jj <= jpj; ++jj)
      for (int ji = 2; ji <= jpi; ++ji) zww[I2(ji, jj)] = 0.25 * c->e1e2t[I2(ji, jj)] * wn[I3(ji, jj, jk)];
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj), q = I3(ji, jj, jk);
        zwuw[q] = (zww[p + 1] + zww[p]) * (un[q - n2] - un[q]);
        zwvw[q] = (zww[p + jpi] + zww[p]) * (vn[q - n2] - vn[q]);
      }
  }
  for (int jk = 1; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj), q = I3(ji, jj, jk);
        ua[q] = ua[q] - (zwuw[q] + zwuw[q + n2]) * c->r1_e1e2u[p] / e3u[q];
        va[q] = va[q] - (zwvw[q] + zwvw[q + n2]) * c->r1_e1e2v[p] / e3v[q];
      }
  wfree(zww); wfree(zwuw); wfree(zwvw);
  return NEMO_OK;
}

/* vor_ene (dynvor.F90:324-429), z-coordinate, no ln_dynvor_msk; kvor 1, 2 or 4. */
int ora_vor_ene(ora_ctx *c, int kt, int kvor, const double *pun, const double *pvn, double *pua, double *pva) {
  (void)kt;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  if (kvor != 1 && kvor != 2 && kvor != 4) return NEMO_ERR_UNSUPPORTED;
  if (c->nam.ln_sco) return NEMO_ERR_UNSUPPORTED;
  double *zwz = zalloc(n2), *zwx = zalloc(n2), *zwy = zalloc(n2);
  const double r1_4 = 0.250;
  for (int jk = 1; jk <= jpk - 1; ++jk) {
    const double *un = pun + n2 * (jk - 1), *vn = pvn + n2 * (jk - 1);
    if (kvor == 1) {
      memcpy(zwz, c->ff_f, n2 * sizeof(double));
    } else {
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          const size_t p = I2(ji, jj);
          const double rv = (c->e2v[I2(ji + 1, jj)] * vn[I2(ji + 1, jj)] - c->e2v[p] * vn[p]
                             - c->e1u[I2(ji, jj + 1)] * un[I2(ji, jj + 1)] + c->e1u[p] * un[p])
                            * (1.0 / (c->e1f[p] * c->e2f[p]));
          zwz[p] = kvor == 2 ? rv : c->ff_f[p] + (c->e2v[I2(ji + 1, jj)] * vn[I2(ji + 1, jj)] - c->e2v[p] * vn[p]
                                                  - c->e1u[I2(ji, jj + 1)] * un[I2(ji, jj + 1)] + c->e1u[p] * un[p])
                                                     * (1.0 / (c->e1f[p] * c->e2f[p]));
        }
    }
    for (size_t p = 0; p < n2; ++p) { zwx[p] = c->e2u[p] * un[p]; zwy[p] = c->e1v[p] * vn[p]; }
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj), q = p + n2 * (jk - 1);
        const double zy1 = zwy[I2(ji, jj - 1)] + zwy[I2(ji + 1, jj - 1)];
        const double zy2 = zwy[p] + zwy[I2(ji + 1, jj)];
        const double zx1 = zwx[I2(ji - 1, jj)] + zwx[I2(ji - 1, jj + 1)];
        const double zx2 = zwx[p] + zwx[I2(ji, jj + 1)];
        pua[q] = pua[q] + r1_4 * c->r1_e1u[p] * (zwz[I2(ji, jj - 1)] * zy1 + zwz[p] * zy2);
        pva[q] = pva[q] - r1_4 * c->r1_e2v[p] * (zwz[I2(ji - 1, jj)] * zx1 + zwz[p] * zx2);
      }
  }
  wfree(zwz); wfree(zwx); wfree(zwy);
  return NEMO_OK;
}

/* dyn_ldf_lap (dynldf_lap_blp.F90:37-104), linear free surface (e3*_b = e3*_0):
 * bound AHMT, AHMF. */
int ora_dyn_ldf_lap(ora_ctx *c, int kt, const double *pub, const double *pvb, double *pua, double *pva, int kpass) {
  (void)kt;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj;
  const double *ahmt = c->f[NEMO_F_AHMT], *ahmf = c->f[NEMO_F_AHMF];
  if (!ahmt || !ahmf) return NEMO_ERR_UNBOUND;
  if (!c->nam.ln_linssh) return NEMO_ERR_UNSUPPORTED;
  const double *e3f = fld(c, NEMO_F_E3F_N), *e3t_b = fld(c, NEMO_F_E3T_B);
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N);
  const double zsign = kpass == 1 ? 1.0 : -1.0;
  double *zcur = zalloc(n2), *zdiv = zalloc(n2);
  for (int jk = 1; jk <= jpk - 1; ++jk) {
    for (int jj = 2; jj <= jpj; ++jj)
      for (int ji = 2; ji <= jpi; ++ji) {
        const size_t pm = I2(ji - 1, jj - 1), qm = I3(ji - 1, jj - 1, jk);
        zcur[pm] = ahmf[qm] * e3f[qm] * (1.0 / (c->e1f[pm] * c->e2f[pm]))
                 * (c->e2v[I2(ji, jj - 1)] * pvb[I3(ji, jj - 1, jk)] - c->e2v[pm] * pvb[qm]
                    - c->e1u[I2(ji - 1, jj)] * pub[I3(ji - 1, jj, jk)] + c->e1u[pm] * pub[qm]);
        const size_t p = I2(ji, jj), q = I3(ji, jj, jk);
        zdiv[p] = ahmt[q] * c->r1_e1e2t[p] / e3t_b[q]
                * (c->e2u[p] * e3u[q] * pub[q] - c->e2u[I2(ji - 1, jj)] * e3u[I3(ji - 1, jj, jk)] * pub[I3(ji - 1, jj, jk)]
                   + c->e1v[p] * e3v[q] * pvb[q] - c->e1v[I2(ji, jj - 1)] * e3v[I3(ji, jj - 1, jk)] * pvb[I3(ji, jj - 1, jk)]);
      }
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj), q = I3(ji, jj, jk);
        pua[q] = pua[q] + zsign * (-(zcur[p] - zcur[I2(ji, jj - 1)]) * c->r1_e2u[p] / e3u[q]
                                   + (zdiv[I2(ji + 1, jj)] - zdiv[p]) * c->r1_e1u[p]);
        pva[q] = pva[q] + zsign * ((zcur[p] - zcur[I2(ji - 1, jj)]) * c->r1_e1v[p] / e3v[q]
                                   + (zdiv[I2(ji, jj + 1)] - zdiv[p]) * c->r1_e2v[p]);
      }
  }
  wfree(zcur); wfree(zdiv);
  return NEMO_OK;
}

/* ------------------------------------------- simplified equation of state */
/* eos_insitu (eosbn2.F90:276-292), np_seos: levels 1..jpk-1 of every point. */
/* ---- EOS-80 (np_eos80): the polynomial of eosbn2.F90:236-270 (density), :588-642
 * (expansion coefficients), written in the reference's association: for one power
 * k of the depth, acc = C(0,D); then for j = D-1 .. 0, acc = (acc*zt + H_j*zs) +
 * C(0,j) with H_j = (..(C(n,j)*zs + C(n-1,j))*zs .. + C(1,j)), n = D - j. */
static const double eos80_c[3][4][7][7] = NEMO_EOS80_TABLE;

static double eos80_zn(int t, int k, int deg, double zt, double zs) {
  const double (*C)[7] = eos80_c[t][k];
  double acc = C[0][deg];
  for (int j = deg - 1; j >= 0; --j) {
    const int n = deg - j;
    double h = C[n][j];
    for (int i = n - 1; i >= 1; --i) h = h * zs + C[i][j];
    acc = (acc * zt + h * zs) + C[0][j];
  }
  return acc;
}
/* zn = ((zn3*zh + zn2)*zh + zn1)*zh + zn0 of table t (0 EOS: degrees 6 4 2 1 in zt;
 * 1 ALP, 2 BET: 5 3 1 0); *zn0 = the surface part */
static double eos80_poly(int t, double zt, double zs, double zh, double *zn0) {
  const int d0 = t == 0 ? 6 : 5, d1 = t == 0 ? 4 : 3, d2 = t == 0 ? 2 : 1, d3 = t == 0 ? 1 : 0;
  const double z3 = eos80_zn(t, 3, d3, zt, zs), z2 = eos80_zn(t, 2, d2, zt, zs);
  const double z1 = eos80_zn(t, 1, d1, zt, zs), z0 = eos80_zn(t, 0, d0, zt, zs);
  if (zn0) *zn0 = z0;
  return ((z3 * zh + z2) * zh + z1) * zh + z0;
}
static void eos80_vars(double t, double s, double dep, double *zt, double *zs, double *zh) {
  *zh = dep * NEMO_EOS80_R1_Z0;
  *zt = t * NEMO_EOS80_R1_T0;
  *zs = sqrt(fabs(s + NEMO_EOS80_RDELTAS) * NEMO_EOS80_R1_S0);
}

static double eos_rd_2d(const ora_ctx *c, double t, double sal, double dep) {
  const nemo_namelist *nm = &c->nam;
  const double r1_rau0 = 1.0 / nm->rau0;
  if (nm->ln_eos80) {  /* eosbn2.F90:318-347 */
    double zt, zs, zh;
    eos80_vars(t, sal, dep, &zt, &zs, &zh);
    return eos80_poly(0, zt, zs, zh, NULL) * r1_rau0 - 1.0;
  }
  const double zt = t - 10., zs = sal - 35., zh = dep;  /* :366-376 */
  const double zn = -nm->rn_a0 * (1. + 0.5 * nm->rn_lambda1 * zt + nm->rn_mu1 * zh) * zt
                    + nm->rn_b0 * (1. - 0.5 * nm->rn_lambda2 * zs - nm->rn_mu2 * zh) * zs
                    - nm->rn_nu * zt * zs;
  return zn * r1_rau0;
}

int ora_eos_insitu(ora_ctx *c, const double *pts, double *prd, const double *pdep) {
  const nemo_namelist *nm = &c->nam;
  if (nm->ln_eos80) {  /* eosbn2.F90:236-270 */
    const size_t n3 = (size_t)c->jpi * c->jpj * c->jpk, nl = (size_t)c->jpi * c->jpj * (c->jpk - 1);
    const double r1_rau0 = 1.0 / nm->rau0;
    for (size_t q = 0; q < nl; ++q) {
      double zt, zs, zh;
      eos80_vars(pts[q], pts[n3 + q], pdep[q], &zt, &zs, &zh);
      const double zn = eos80_poly(0, zt, zs, zh, NULL);
      prd[q] = (zn * r1_rau0 - 1.0) * c->tmask[q];
    }
    return NEMO_OK;
  }
  if (!nm->ln_seos) return NEMO_ERR_UNSUPPORTED;
  const size_t n3 = (size_t)c->jpi * c->jpj * c->jpk, nl = (size_t)c->jpi * c->jpj * (c->jpk - 1);
  const double r1_rau0 = 1.0 / nm->rau0;
  for (size_t q = 0; q < nl; ++q) {
    const double zt = pts[q] - 10., zs = pts[n3 + q] - 35., zh = pdep[q], ztm = c->tmask[q];
    const double zn = -nm->rn_a0 * (1. + 0.5 * nm->rn_lambda1 * zt + nm->rn_mu1 * zh) * zt
                      + nm->rn_b0 * (1. - 0.5 * nm->rn_lambda2 * zs - nm->rn_mu2 * zh) * zs
                      - nm->rn_nu * zt * zs;
    prd[q] = zn * r1_rau0 * ztm;
  }
  return NEMO_OK;
}

/* eos_insitu_pot (eosbn2.F90:440-462), np_seos. */
int ora_eos_insitu_pot(ora_ctx *c, const double *pts, double *prd, double *prhop, const double *pdep) {
  const nemo_namelist *nm = &c->nam;
  if (nm->ln_eos80) {  /* eosbn2.F90:400-436 (ln_sto_eos off) */
    const size_t n3 = (size_t)c->jpi * c->jpj * c->jpk, nl = (size_t)c->jpi * c->jpj * (c->jpk - 1);
    const double r1_rau0 = 1.0 / nm->rau0;
    for (size_t q = 0; q < nl; ++q) {
      double zt, zs, zh, zn0;
      eos80_vars(pts[q], pts[n3 + q], pdep[q], &zt, &zs, &zh);
      const double zn = eos80_poly(0, zt, zs, zh, &zn0);
      prhop[q] = zn0 * c->tmask[q];
      prd[q] = (zn * r1_rau0 - 1.0) * c->tmask[q];
    }
    return NEMO_OK;
  }
  if (!nm->ln_seos) return NEMO_ERR_UNSUPPORTED;
  const size_t n3 = (size_t)c->jpi * c->jpj * c->jpk, nl = (size_t)c->jpi * c->jpj * (c->jpk - 1);
  const double r1_rau0 = 1.0 / nm->rau0;
  for (size_t q = 0; q < nl; ++q) {
    const double zt = pts[q] - 10., zs = pts[n3 + q] - 35., zh = pdep[q], ztm = c->tmask[q];
    double zn = -nm->rn_a0 * (1. + 0.5 * nm->rn_lambda1 * zt) * zt
                + nm->rn_b0 * (1. - 0.5 * nm->rn_lambda2 * zs) * zs
                - nm->rn_nu * zt * zs;
    prhop[q] = (nm->rau0 + zn) * ztm;
    zn = zn - (nm->rn_a0 * nm->rn_mu1 * zt + nm->rn_b0 * nm->rn_mu2 * zs) * zh;
    prd[q] = zn * r1_rau0 * ztm;
  }
  return NEMO_OK;
}

/* rab_3d (eosbn2.F90:645-661), np_seos, at the bound GDEPT_N. */
int ora_rab_3d(ora_ctx *c, const double *pts, double *pab) {
  const nemo_namelist *nm = &c->nam;
  const double *gdept = c->f[NEMO_F_GDEPT_N];
  if (nm->ln_eos80) {  /* eosbn2.F90:588-642 */
    if (!gdept) return NEMO_ERR_UNBOUND;
    const size_t n3 = (size_t)c->jpi * c->jpj * c->jpk, nl = (size_t)c->jpi * c->jpj * (c->jpk - 1);
    const double r1_rau0 = 1.0 / nm->rau0;
    for (size_t q = 0; q < nl; ++q) {
      double zt, zs, zh;
      eos80_vars(pts[q], pts[n3 + q], gdept[q], &zt, &zs, &zh);
      const double ztm = c->tmask[q];
      double zn = eos80_poly(1, zt, zs, zh, NULL);
      pab[q] = zn * r1_rau0 * ztm;
      zn = eos80_poly(2, zt, zs, zh, NULL);
      pab[n3 + q] = zn / zs * r1_rau0 * ztm;
    }
    return NEMO_OK;
  }
  if (!nm->ln_seos) return NEMO_ERR_UNSUPPORTED;
  if (!gdept) return NEMO_ERR_UNBOUND;
  const size_t n3 = (size_t)c->jpi * c->jpj * c->jpk, nl = (size_t)c->jpi * c->jpj * (c->jpk - 1);
  const double r1_rau0 = 1.0 / nm->rau0;
  for (size_t q = 0; q < nl; ++q) {
    const double zt = pts[q] - 10., zs = pts[n3 + q] - 35., zh = gdept[q], ztm = c->tmask[q];
    double zn = nm->rn_a0 * (1. + nm->rn_lambda1 * zt + nm->rn_mu1 * zh) + nm->rn_nu * zs;
    pab[q] = zn * r1_rau0 * ztm;
    zn = nm->rn_b0 * (1. - nm->rn_lambda2 * zs - nm->rn_mu2 * zh) - nm->rn_nu * zt;
    pab[n3 + q] = zn * r1_rau0 * ztm;
  }
  return NEMO_OK;
}

/* bn2 (eosbn2.F90:889-933): levels 2..jpk-1 of every point. */
int ora_bn2(ora_ctx *c, const double *pts, const double *pab, double *pn2) {
  const nemo_namelist *nm = &c->nam;
  const double *gdept = c->f[NEMO_F_GDEPT_N], *gdepw = c->f[NEMO_F_GDEPW_N];
  if (!gdept || !gdepw) return NEMO_ERR_UNBOUND;
  const double *e3w = fld(c, NEMO_F_E3W_N);
  const size_t n2 = (size_t)c->jpi * c->jpj, n3 = n2 * c->jpk;
  for (int jk = 2; jk <= c->jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      const size_t q = p + n2 * (jk - 1), qu = q - n2;
      const double zrw = (gdepw[q] - gdept[q]) / (gdept[qu] - gdept[q]);
      const double zaw = pab[q] * (1. - zrw) + pab[qu] * zrw;
      const double zbw = pab[n3 + q] * (1. - zrw) + pab[n3 + qu] * zrw;
      pn2[q] = nm->grav * (zaw * (pts[qu] - pts[q]) - zbw * (pts[n3 + qu] - pts[n3 + q])) / e3w[q] * c->wmask[q];
    }
  return NEMO_OK;
}

/* dyn_hpg with hpg_zco (dynhpg.F90:258-323): bound RHD, UA, VA. */
int ora_dyn_hpg(ora_ctx *c, int kt) {
  (void)kt;
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const double *rhd = c->f[NEMO_F_RHD];
  double *ua = c->f[NEMO_F_UA], *va = c->f[NEMO_F_VA];
  if (!rhd || !ua || !va) return NEMO_ERR_UNBOUND;
  if (nm->ln_zps || nm->ln_sco || nm->ln_isfcav) return NEMO_ERR_UNSUPPORTED;
  const double *e3w = fld(c, NEMO_F_E3W_N);
  const double zcoef0 = -nm->grav * 0.5;
  const size_t n2 = (size_t)jpi * jpj;
  double *zhpi = zalloc(n2), *zhpj = zalloc(n2);
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      const size_t p = I2(ji, jj);
      const double zcoef1 = zcoef0 * e3w[p];
      zhpi[p] = zcoef1 * (rhd[I2(ji + 1, jj)] - rhd[p]) * c->r1_e1u[p];
      zhpj[p] = zcoef1 * (rhd[I2(ji, jj + 1)] - rhd[p]) * c->r1_e2v[p];
      ua[p] = ua[p] + zhpi[p];
      va[p] = va[p] + zhpj[p];
    }
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj), q = I3(ji, jj, jk), qu = q - n2;
        const double zcoef1 = zcoef0 * e3w[q];
        zhpi[p] = zhpi[p] + zcoef1 * ((rhd[q + 1] + rhd[qu + 1]) - (rhd[q] + rhd[qu])) * c->r1_e1u[p];
        zhpj[p] = zhpj[p] + zcoef1 * ((rhd[q + jpi] + rhd[qu + jpi]) - (rhd[q] + rhd[qu])) * c->r1_e2v[p];
        ua[q] = ua[q] + zhpi[p];
        va[q] = va[q] + zhpj[p];
      }
  wfree(zhpi); wfree(zhpj);
  return NEMO_OK;
}

/* the model step's vertical physics is on: the TKE closure selected as zdf_phy
 * covers it, an equation of state and every field of zdf_phy bound */
static int vphys_on(const ora_ctx *c) {
  const nemo_namelist *nm = &c->nam;
  static const int ids[] = {NEMO_F_UB, NEMO_F_VB, NEMO_F_UN, NEMO_F_VN, NEMO_F_AVM_K, NEMO_F_AVT_K, NEMO_F_AVM,
                            NEMO_F_AVT, NEMO_F_EN, NEMO_F_DISSL, NEMO_F_RN2, NEMO_F_RN2B, NEMO_F_TAUM,
                            NEMO_F_GDEPW_N, NEMO_F_GDEPT_N};
  if (!nm->ln_zdftke || !(nm->ln_seos || nm->ln_eos80) || nm->nn_etau != 0 || nm->ln_drg_tke || !nm->ln_linssh ||
      nm->ln_isfcav || nm->ln_sco || nm->ln_zps)
    return 0;
  for (size_t i = 0; i < sizeof(ids) / sizeof(ids[0]); ++i)
    if (!c->f[ids[i]]) return 0;
  return 1;
}

/* One model step (step.F90:96-305) with the path and the routines above: the
 * GYRE analytic forcing (ln_usr), the vertical physics (rab_3d and bn2 of the
 * before and now tracers, zdf_phy), the
 * iso-neutral slopes, div_hor + wzv, ua = va = 0, dyn_adv (keg + zad), dyn_vor (vor_ene), dyn_ldf,
 * eos + dyn_hpg, dyn_spg_ts, div_hor + wzv, dyn_zdf, tsa = 0, tra_sbc, tra_qsr,
 * tra_adv, tra_ldf, tra_zdf, tra_nxt, dyn_nxt, ssh_swp, dia_hsb, stp_ctl; the
 * optional ones where their fields are bound. */
int ora_stp_model(ora_ctx *c, int kt) {
  const size_t n3 = (size_t)c->jpi * c->jpj * c->jpk;
  if (!c->f[NEMO_F_UA] || !c->f[NEMO_F_VA]) return NEMO_ERR_UNBOUND;
  int st = 0;
  const nemo_namelist *nm = &c->nam;
  if (nm->ln_usr) {                                               /* step.F90:116: sbc */
    st = ora_usrdef_sbc(c, kt);
    if (st) return st;
  }
  const int vphys = vphys_on(c);
  if (vphys) {                                                    /* step.F90:127-133 */
    double *rab = zalloc(2 * n3);
    st = ora_rab_3d(c, c->f[NEMO_F_TSB], rab);
    if (!st) st = ora_bn2(c, c->f[NEMO_F_TSB], rab, c->f[NEMO_F_RN2B]);
    if (!st) st = ora_rab_3d(c, c->f[NEMO_F_TSN], rab);
    if (!st) st = ora_bn2(c, c->f[NEMO_F_TSN], rab, c->f[NEMO_F_RN2]);
    wfree(rab);
    if (!st) st = ora_zdf_phy(c, kt);
    if (st) return st;
  }
  if ((nm->ln_seos || nm->ln_eos80) && nm->ln_traldf_iso && !nm->ln_zps && !nm->ln_sco && !nm->ln_isfcav && c->f[NEMO_F_RN2B] &&
      c->f[NEMO_F_RHD] && c->f[NEMO_F_GDEPT_N] && c->f[NEMO_F_GDEPW_N] && c->f[NEMO_F_NMLN] && c->f[NEMO_F_HMLP] &&
      c->f[NEMO_F_HMLPT] && c->f[NEMO_F_USLP] && c->f[NEMO_F_VSLP] && c->f[NEMO_F_WSLPI] && c->f[NEMO_F_WSLPJ] &&
      c->f[NEMO_F_AVT]) {                                          /* step.F90:127-150 */
    if (!vphys) {  /* (rn2b comes from the vertical physics otherwise) */
      double *rab = zalloc(2 * n3);
      st = ora_rab_3d(c, c->f[NEMO_F_TSB], rab);
      if (!st) st = ora_bn2(c, c->f[NEMO_F_TSB], rab, c->f[NEMO_F_RN2B]);
      wfree(rab);
    }
    if (!st) st = ora_zdf_mxl(c, kt);
    if (!st) st = ora_eos_insitu(c, c->f[NEMO_F_TSB], c->f[NEMO_F_RHD], c->f[NEMO_F_GDEPT_N]);
    if (!st) st = ora_ldf_slp(c, kt, c->f[NEMO_F_RHD], c->f[NEMO_F_RN2B]);
    if (st) return st;
  }
  /* ssh_nxt's div_hor and wzv (step.F90:156-160): the now vertical velocity of dyn_adv
   * (ssha is dyn_spg_ts's with the split-explicit free surface) */
  st = ora_wzv(c, kt);
  if (st) return st;
  memset(c->f[NEMO_F_UA], 0, n3 * sizeof(double));
  memset(c->f[NEMO_F_VA], 0, n3 * sizeof(double));
  /* dyn_adv, dyn_vor (step.F90:190-191): the vector form, keg (C2) + zad, and vor_ene
   * of the total vorticity (dynvor.F90:904-913: Coriolis alone for linear dynamics) */
  if (!nm->ln_dynadv_OFF) {
    if (!nm->ln_dynadv_vec || nm->nn_dynkeg != 0) return NEMO_ERR_UNSUPPORTED;
    st = ora_dyn_keg(c, kt, 0);
    if (!st) st = ora_dyn_zad(c, kt);
  }
  if (nm->nvor_scheme != NEMO_VOR_ENE) return NEMO_ERR_UNSUPPORTED;
  if (!st) st = ora_vor_ene(c, kt, nm->ln_dynadv_OFF ? 1 : 4, c->f[NEMO_F_UN], c->f[NEMO_F_VN], c->f[NEMO_F_UA],
                            c->f[NEMO_F_VA]);
  /* dyn_ldf (:192): the iso-level laplacian where the viscosity AHMT, AHMF is bound */
  if (!st && c->f[NEMO_F_AHMT] && c->f[NEMO_F_AHMF])
    st = ora_dyn_ldf_lap(c, kt, c->f[NEMO_F_UB], c->f[NEMO_F_VB], c->f[NEMO_F_UA], c->f[NEMO_F_VA], 1);
  if (st) return st;
  if (c->f[NEMO_F_RHD] && c->f[NEMO_F_RHOP] && (c->nam.ln_seos || c->nam.ln_eos80)) {  /* step.F90:165, :193 */
    if (!c->f[NEMO_F_GDEPT_N]) return NEMO_ERR_UNBOUND;
    st = ora_eos_insitu_pot(c, c->f[NEMO_F_TSN], c->f[NEMO_F_RHD], c->f[NEMO_F_RHOP], c->f[NEMO_F_GDEPT_N]);
    if (!st) st = ora_dyn_hpg(c, kt);
  }
  if (!st) st = ora_dyn_spg_ts(c, kt);
  if (!st) st = ora_wzv(c, kt);
  if (!st) st = ora_dyn_zdf_step(c, kt);
  if (!st) st = stp_tracers(c, kt);
  if (!st) st = ora_tra_nxt(c, kt);
  if (!st) st = ora_dyn_nxt(c, kt);
  if (!st) st = ora_ssh_swp(c, kt);
  if (!st && c->hsb_on) st = ora_dia_hsb(c, kt, NULL);                  /* step.F90:282 */
  if (!st && c->f[NEMO_F_SSHN] && c->f[NEMO_F_UN] && c->f[NEMO_F_TSN])  /* :305 */
    st = ora_stp_ctl(c, kt, c->ctl_zmax, c->ctl_loc, &c->ctl_kindic);
  return st;
}

/* -------------------------------------------------------- the triad operator */
/* offset of (ji,jj,jk,a,b) in a (jpi,jpj,jpk,0:1,0:1) triad array */
#define TRI(ji, jj, jk, a, b) (I3(ji, jj, jk) + n3 * (size_t)((a) + 2 * (b)))
static inline double dmin3(double a, double b, double c) { double m = a < b ? a : b; return m < c ? m : c; }

/* ldf_slp_triad (ldfslp.F90:377-617): the slopes of the four i-k and four j-k
 * Griffies triads of each T-point relative to geopotentials (triadi_g, triadj_g) and
 * to the model levels (triadi, triadj), and wslp2. The density gradients use the
 * before expansion ratios prab_b (jpi,jpj,jpk,2: eos_rab of tsb) at the triad's
 * T-point; inside the mixed layer the slope tapers linearly from its value just
 * below the mixed-layer base. No eddy-induced velocity; l_grad_zps is .FALSE. (the
 * reference never sets it, ldfslp.F90:54). Bound: TSB, GDEPT_N, GDEPW_N, NMLN and
 * the outputs TRIADI_G, TRIADJ_G, TRIADI, TRIADJ (jpi,jpj,jpk,2,2), WSLP2 when
 * bound. Entries of faces outside the reference's loops keep their values, except
 * levels 1 and jpk, which are zeroed (:480-483; triadi's jpk level too). */
int ora_ldf_slp_triad(ora_ctx *c, int kt, const double *prab_b) {
  (void)kt;
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  double **F = c->f;
  const double *tsb = F[NEMO_F_TSB], *gdept = F[NEMO_F_GDEPT_N], *gdepw = F[NEMO_F_GDEPW_N];
  const int *nmln = (const int *)F[NEMO_F_NMLN];
  double *tig = F[NEMO_F_TRIADI_G], *tjg = F[NEMO_F_TRIADJ_G], *ti = F[NEMO_F_TRIADI], *tj = F[NEMO_F_TRIADJ];
  double *wslp2 = F[NEMO_F_WSLP2];
  if (!prab_b) return NEMO_ERR_ARG;
  if (!tsb || !gdept || !gdepw || !nmln || !tig || !tjg || !ti || !tj) return NEMO_ERR_UNBOUND;
  if (nm->ln_isfcav) return NEMO_ERR_UNSUPPORTED;
  const double repsln = 1.e-25, slpmax = nm->rn_slpmax > 0 ? nm->rn_slpmax : 0.01, sw = nm->rn_sw_triad;
  const double *e3w = fld(c, NEMO_F_E3W_N), *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N);
  const double *tt = tsb, *ts = tsb + n3, *ra = prab_b, *rb = prab_b + n3;
  const double *umask = c->umask, *vmask = c->vmask;
  double *zdxrho = zalloc(2 * n3), *zdyrho = zalloc(2 * n3), *zdzrho = zalloc(2 * n3);
  double *zti_mlb = zalloc(4 * n2), *ztj_mlb = zalloc(4 * n2), *z1_mlbw = zalloc(n2);
  for (int jl = 0; jl <= 1; ++jl) {                                      /* :415-429 */
    const int ip = jl, jp = jl;
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          const double zdit = tt[I3(ji + 1, jj, jk)] - tt[I3(ji, jj, jk)];
          const double zdis = ts[I3(ji + 1, jj, jk)] - ts[I3(ji, jj, jk)];
          const double zdjt = tt[I3(ji, jj + 1, jk)] - tt[I3(ji, jj, jk)];
          const double zdjs = ts[I3(ji, jj + 1, jk)] - ts[I3(ji, jj, jk)];
          const double xr = (-ra[I3(ji + ip, jj, jk)] * zdit + rb[I3(ji + ip, jj, jk)] * zdis) * c->r1_e1u[I2(ji, jj)];
          const double yr = (-ra[I3(ji, jj + jp, jk)] * zdjt + rb[I3(ji, jj + jp, jk)] * zdjs) * c->r1_e2v[I2(ji, jj)];
          zdxrho[I3(ji + ip, jj, jk) + n3 * (1 - ip)] = sign_nsz(repsln > fabs(xr) ? repsln : fabs(xr), xr);
          zdyrho[I3(ji, jj + jp, jk) + n3 * (1 - jp)] = sign_nsz(repsln > fabs(yr) ? repsln : fabs(yr), yr);
        }
  }
  for (int kp = 0; kp <= 1; ++kp)                                        /* :446-463 */
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (size_t p = 0; p < n2; ++p) {
        const int k = jk + kp;
        const size_t q = p + n2 * (k - 1);
        double zdkt = 0.0, zdks = 0.0;
        if (k > 1) { zdkt = tt[q - n2] - tt[q]; zdks = ts[q - n2] - ts[q]; }
        const double zr = (-ra[q] * zdkt + rb[q] * zdks) / e3w[q];
        zdzrho[p + n2 * (jk - 1) + n3 * kp] = -(-repsln < zr ? -repsln : zr);
      }
  for (int jj = 1; jj <= jpj; ++jj)                                      /* :465-470 */
    for (int ji = 1; ji <= jpi; ++ji) {
      const size_t p = I2(ji, jj);
      int jk = (nmln[p] < c->mbkt[p] ? nmln[p] : c->mbkt[p]) + 1;
      jk = jk < 1 ? 1 : jk;   /* kept in the column whatever nmln holds */
      z1_mlbw[p] = 1.0 / gdepw[I3(ji, jj, jk)];
    }
  if (wslp2) memset(wslp2, 0, n3 * sizeof(double));                     /* :478-483 */
  for (int a = 0; a < 4; ++a)
    for (size_t p = 0; p < n2; ++p) {
      tig[p + n3 * a] = 0.0; tig[p + n2 * (jpk - 1) + n3 * a] = 0.0;
      tjg[p + n3 * a] = 0.0; tjg[p + n2 * (jpk - 1) + n3 * a] = 0.0;
      ti[p + n3 * a] = 0.0; ti[p + n2 * (jpk - 1) + n3 * a] = 0.0;
      tj[p + n3 * a] = 0.0; tj[p + n2 * (jpk - 1) + n3 * a] = 0.0;
    }
  for (int jl = 0; jl <= 1; ++jl)                                        /* :489-521 */
    for (int kp = 0; kp <= 1; ++kp)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          const int ip = jl, jp = jl;
          int jk = nmln[I2(ji + ip, jj)] + 1;
          double *mi = &zti_mlb[I2(ji + ip, jj) + n2 * ((1 - ip) + 2 * kp)];
          if (jk > c->mbkt[I2(ji + ip, jj)] || jk - kp < 1) {   /* (jk - kp >= 1 for nmln >= 1) */
            *mi = 0.0;
          } else {
            const double g = (zdxrho[I3(ji + ip, jj, jk - kp) + n3 * (1 - ip)] / zdzrho[I3(ji + ip, jj, jk - kp) + n3 * kp]
                              - (gdept[I3(ji + 1, jj, jk - kp)] - gdept[I3(ji, jj, jk - kp)]) * c->r1_e1u[I2(ji, jj)])
                             * umask[I3(ji, jj, jk)];
            const double ze3_e1 = e3w[I3(ji + ip, jj, jk - kp)] * c->r1_e1u[I2(ji, jj)];
            *mi = sign_nsz(dmin3(slpmax, 5.0 * ze3_e1, fabs(g)), g);
          }
          jk = nmln[I2(ji, jj + jp)] + 1;
          double *mj = &ztj_mlb[I2(ji, jj + jp) + n2 * ((1 - jp) + 2 * kp)];
          if (jk > c->mbkt[I2(ji, jj + jp)] || jk - kp < 1) {
            *mj = 0.0;
          } else {
            const double g = (zdyrho[I3(ji, jj + jp, jk - kp) + n3 * (1 - jp)] / zdzrho[I3(ji, jj + jp, jk - kp) + n3 * kp]
                              - (gdept[I3(ji, jj + 1, jk - kp)] - gdept[I3(ji, jj, jk - kp)]) / c->e2v[I2(ji, jj)])
                             * vmask[I3(ji, jj, jk)];
            const double ze3_e2 = e3w[I3(ji, jj + jp, jk - kp)] / c->e2v[I2(ji, jj)];
            *mj = sign_nsz(dmin3(slpmax, 5.0 * ze3_e2, fabs(g)), g);
          }
        }
  for (int kp = 0; kp <= 1; ++kp)                                        /* :527-609 */
    for (int jl = 0; jl <= 1; ++jl) {
      const int ip = jl, jp = jl;
      for (int jk = 1; jk <= jpk - 1; ++jk) {
        const double znot = (jk + kp == 1) ? 0.0 : 1.0;
        for (int jj = 1; jj <= jpj - 1; ++jj)
          for (int ji = 1; ji <= jpi - 1; ++ji) {
            const size_t pi = I2(ji + ip, jj), pj = I2(ji, jj + jp), pu = I2(ji, jj);
            const double dxr = zdxrho[I3(ji + ip, jj, jk) + n3 * (1 - ip)];
            const double dyr = zdyrho[I3(ji, jj + jp, jk) + n3 * (1 - jp)];
            double zti_raw = dxr / zdzrho[I3(ji + ip, jj, jk) + n3 * kp];
            double ztj_raw = dyr / zdzrho[I3(ji, jj + jp, jk) + n3 * kp];
            const double zti_coord = znot * (gdept[I3(ji + 1, jj, jk)] - gdept[I3(ji, jj, jk)]) * c->r1_e1u[pu];
            const double ztj_coord = znot * (gdept[I3(ji, jj + 1, jk)] - gdept[I3(ji, jj, jk)]) * c->r1_e2v[pu];
            const double zti_g_raw = zti_raw - zti_coord, ztj_g_raw = ztj_raw - ztj_coord;
            const double ze3_e1 = e3w[I3(ji + ip, jj, jk + kp)] * c->r1_e1u[pu];
            const double ze3_e2 = e3w[I3(ji, jj + jp, jk + kp)] * c->r1_e2v[pu];
            double zti_g_lim = sign_nsz(dmin3(slpmax, 5.0 * ze3_e1, fabs(zti_g_raw)), zti_g_raw);
            double ztj_g_lim = sign_nsz(dmin3(slpmax, 5.0 * ze3_e2, fabs(ztj_g_raw)), ztj_g_raw);
            const double zfacti = (jk + kp - 1 >= nmln[pi]) ? 1.0 : 0.0;
            const double zfactj = (jk + kp - 1 >= nmln[pj]) ? 1.0 : 0.0;
            zti_g_lim = (zfacti * zti_g_lim + (1.0 - zfacti) * zti_mlb[pi + n2 * ((1 - ip) + 2 * kp)] *
                         gdepw[I3(ji + ip, jj, jk + kp)] * z1_mlbw[pi]) * umask[I3(ji, jj, jk + kp)];
            ztj_g_lim = (zfactj * ztj_g_lim + (1.0 - zfactj) * ztj_mlb[pj + n2 * ((1 - jp) + 2 * kp)] *
                         gdepw[I3(ji, jj + jp, jk + kp)] * z1_mlbw[pj]) * vmask[I3(ji, jj, jk + kp)];
            tig[TRI(ji + ip, jj, jk, 1 - ip, kp)] = zti_g_lim;
            tjg[TRI(ji, jj + jp, jk, 1 - jp, kp)] = ztj_g_lim;
            double zti_lim = (zti_g_lim + zti_coord) * umask[I3(ji, jj, jk + kp)];
            double ztj_lim = (ztj_g_lim + ztj_coord) * vmask[I3(ji, jj, jk + kp)];
            if (nm->ln_triad_iso) {                                      /* :581-588 */
              zti_raw = zti_lim * zti_lim / zti_raw;
              ztj_raw = ztj_lim * ztj_lim / ztj_raw;
              zti_raw = sign_nsz(fabs(zti_lim) < fabs(zti_raw) ? fabs(zti_lim) : fabs(zti_raw), zti_raw);
              ztj_raw = sign_nsz(fabs(ztj_lim) < fabs(ztj_raw) ? fabs(ztj_lim) : fabs(ztj_raw), ztj_raw);
              zti_lim = zfacti * zti_lim + (1.0 - zfacti) * zti_raw;
              ztj_lim = zfactj * ztj_lim + (1.0 - zfactj) * ztj_raw;
            }
            const double zisw = (1.0 - sw) + sw * 2.0 * fabs(0.5 - kp - (0.5 - ip) * sign_nsz(1.0, dxr));
            const double zjsw = (1.0 - sw) + sw * 2.0 * fabs(0.5 - kp - (0.5 - jp) * sign_nsz(1.0, dyr));
            ti[TRI(ji + ip, jj, jk, 1 - ip, kp)] = zti_lim * zisw;
            tj[TRI(ji, jj + jp, jk, 1 - jp, kp)] = ztj_lim * zjsw;
            if (wslp2) {
              const double zbu = c->e1e2u[pu] * e3u[I3(ji, jj, jk)], zbv = c->e1e2v[pu] * e3v[I3(ji, jj, jk)];
              const double zbti = c->e1e2t[pi] * e3w[I3(ji + ip, jj, jk + kp)];
              const double zbtj = c->e1e2t[pj] * e3w[I3(ji, jj + jp, jk + kp)];
              wslp2[I3(ji + ip, jj, jk + kp)] += 0.25 * zbu / zbti * zti_g_lim * zti_g_lim;
              wslp2[I3(ji, jj + jp, jk + kp)] += 0.25 * zbv / zbtj * ztj_g_lim * ztj_g_lim;
            }
          }
      }
    }
  if (wslp2) {                                                           /* :611-613 */
    memset(wslp2, 0, n2 * sizeof(double));
    lbc_closed(jpi, jpj, wslp2, jpk, 'W', 0.0);
  }
  wfree(zdxrho); wfree(zdyrho); wfree(zdzrho); wfree(zti_mlb); wfree(ztj_mlb); wfree(z1_mlbw);
  return NEMO_OK;
}

/* tra_ldf_triad (traldf_triad.F90:50-429), no eddy-induced velocity, l_grad_zps =
 * .FALSE. (pgu, pgv, pgui, pgvi unread): in the first pass ah_wslp2 and akz from the
 * triads (:135-222); per tracer the horizontal fluxes of the four triads of each
 * u- (v-) face and their vertical counterparts at the triads' w-points, masked by
 * the face's mask at the w-level unless ln_botmix_triad (:260-358), the horizontal
 * divergence added level by level, then the 33 flux and the vertical divergence
 * (:370-410). Reads the bound triad arrays and writes the bound AH_WSLP2, AKZ. */
int ora_tra_ldf_triad(ora_ctx *c, int kt, int kit000, const char *cdtype, const double *pahu,
                      const double *pahv, const double *pgu, const double *pgv, const double *pgui,
                      const double *pgvi, const double *ptb, const double *ptbb, double *pta, int kjpt, int kpass) {
  (void)cdtype; (void)pgu; (void)pgv; (void)pgui; (void)pgvi;
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  double **F = c->f;
  double *ah_wslp2 = F[NEMO_F_AH_WSLP2], *akz = F[NEMO_F_AKZ];
  const double *tig = F[NEMO_F_TRIADI_G], *tjg = F[NEMO_F_TRIADJ_G], *ti = F[NEMO_F_TRIADI], *tj = F[NEMO_F_TRIADJ];
  if (!ptb || !pta || kjpt < 1 || (kpass != 1 && kpass != 2) || (kpass == 2 && !ptbb)) return NEMO_ERR_ARG;
  if (!ah_wslp2 || !akz || !tig || !tjg || !ti || !tj) return NEMO_ERR_UNBOUND;
  if (!pahu) pahu = c->ahtu_c;
  if (!pahv) pahv = c->ahtv_c;
  const double *tmask = c->tmask, *umask = c->umask, *vmask = c->vmask;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N), *e3t = fld(c, NEMO_F_E3T_N);
  const double *e3w = fld(c, NEMO_F_E3W_N), *gdept = fld(c, NEMO_F_GDEPT_N);
  if (!gdept) return NEMO_ERR_UNBOUND;
  const double z2dt = (nm->neuler == 0 && kt == kit000) ? nm->rn_rdt : 2. * nm->rn_rdt;   /* :117-120 */
  const double z1_2dt = 1.0 / z2dt;
  const double zsign = kpass == 1 ? 1.0 : -1.0;
  if (kpass == 1) {                                                      /* :131-222 */
    memset(akz, 0, n3 * sizeof(double));
    memset(ah_wslp2, 0, n3 * sizeof(double));
    for (int ip = 0; ip <= 1; ++ip)
      for (int kp = 0; kp <= 1; ++kp)
        for (int jk = 1; jk <= jpk - 1; ++jk)
          for (int jj = 1; jj <= jpj - 1; ++jj)
            for (int ji = 1; ji <= jpi - 1; ++ji) {
              const size_t pu = I2(ji, jj), w = I3(ji + ip, jj, jk + kp);
              const double ze3wr = 1.0 / e3w[w];
              const double zbu = c->e1e2u[pu] * e3u[I3(ji, jj, jk)];
              const double zah = 0.25 * pahu[I3(ji, jj, jk)];
              const double skew = tig[TRI(ji + ip, jj, jk, 1 - ip, kp)];
              double s2 = skew + (gdept[I3(ji + 1, jj, jk)] - gdept[I3(ji, jj, jk)]) * c->r1_e1u[pu] * umask[I3(ji, jj, jk + kp)];
              s2 = s2 * s2;
              ah_wslp2[w] = ah_wslp2[w] + zah * zbu * ze3wr * c->r1_e1e2t[I2(ji + ip, jj)] * s2;
              akz[w] = akz[w] + zah * c->r1_e1u[pu] * c->r1_e1u[pu] * umask[I3(ji, jj, jk + kp)];
            }
    for (int jp = 0; jp <= 1; ++jp)
      for (int kp = 0; kp <= 1; ++kp)
        for (int jk = 1; jk <= jpk - 1; ++jk)
          for (int jj = 1; jj <= jpj - 1; ++jj)
            for (int ji = 1; ji <= jpi - 1; ++ji) {
              const size_t pv = I2(ji, jj), w = I3(ji, jj + jp, jk + kp);
              const double ze3wr = 1.0 / e3w[w];
              const double zbv = c->e1e2v[pv] * e3v[I3(ji, jj, jk)];
              const double zah = 0.25 * pahv[I3(ji, jj, jk)];
              const double skew = tjg[TRI(ji, jj + jp, jk, 1 - jp, kp)];
              double s2 = skew + (gdept[I3(ji, jj + 1, jk)] - gdept[I3(ji, jj, jk)]) * c->r1_e2v[pv] * vmask[I3(ji, jj, jk + kp)];
              s2 = s2 * s2;
              ah_wslp2[w] = ah_wslp2[w] + zah * zbv * ze3wr * c->r1_e1e2t[I2(ji, jj + jp)] * s2;
              akz[w] = akz[w] + zah * c->r1_e2v[pv] * c->r1_e2v[pv] * vmask[I3(ji, jj, jk + kp)];
            }
    if (nm->ln_traldf_msc) {                                             /* :190-212 */
      for (int jk = 2; jk <= jpk - 1; ++jk)
        for (int jj = 1; jj <= jpj - 1; ++jj)
          for (int ji = 1; ji <= jpi - 1; ++ji) {
            const size_t q = I3(ji, jj, jk);
            if (nm->ln_traldf_blp) {
              akz[q] = 16.0 * ah_wslp2[q] * (akz[q] + ah_wslp2[q] / (e3w[q] * e3w[q]));
            } else {
              const double ze3w_2 = e3w[q] * e3w[q];
              const double zcoef0 = z2dt * (akz[q] + ah_wslp2[q] / ze3w_2);
              akz[q] = (zcoef0 - 0.5 > 0.0 ? zcoef0 - 0.5 : 0.0) * ze3w_2 * z1_2dt;
            }
          }
    } else {                                                             /* :214-215 */
      memcpy(akz, ah_wslp2, n3 * sizeof(double));
    }
  }
  double *zdit = zalloc(n3), *zdjt = zalloc(n3), *zftu = walloc(n3), *zftv = walloc(n3), *ztfw = walloc(n3);
  double *zdk0 = walloc(n2), *zdk1 = walloc(n2);
  for (int jn = 0; jn < kjpt; ++jn) {
    const double *tb = ptb + n3 * jn, *tbb = kpass == 2 ? ptbb + n3 * jn : NULL;
    double *ta = pta + n3 * jn;
    memset(ztfw, 0, n3 * sizeof(double));
    memset(zftu, 0, n3 * sizeof(double));
    memset(zftv, 0, n3 * sizeof(double));
    for (int jk = 1; jk <= jpk - 1; ++jk)                                /* :234-241 */
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          zdit[q] = (tb[I3(ji + 1, jj, jk)] - tb[q]) * umask[q];
          zdjt[q] = (tb[I3(ji, jj + 1, jk)] - tb[q]) * vmask[q];
        }
    for (int jk = 1; jk <= jpk - 1; ++jk) {                              /* :263-364 */
      for (size_t p = 0; p < n2; ++p) {
        const size_t q = p + n2 * (jk - 1);
        zdk1[p] = (tb[q] - tb[q + n2]) * tmask[q + n2];
        zdk0[p] = jk == 1 ? zdk1[p] : (tb[q - n2] - tb[q]) * tmask[q];
      }
      for (int ip = 0; ip <= 1; ++ip)
        for (int kp = 0; kp <= 1; ++kp)
          for (int jj = 1; jj <= jpj - 1; ++jj)
            for (int ji = 1; ji <= jpi - 1; ++ji) {
              const size_t pu = I2(ji, jj), q = I3(ji, jj, jk), w = I3(ji + ip, jj, jk + kp);
              const double ze1ur = c->r1_e1u[pu];
              const double zdxt = zdit[q] * ze1ur;
              const double ze3wr = 1.0 / e3w[w];
              const double zdzt = (kp ? zdk1 : zdk0)[I2(ji + ip, jj)] * ze3wr;
              const double zslope_iso = ti[TRI(ji + ip, jj, jk, 1 - ip, kp)];
              const double zbu = 0.25 * c->e1e2u[pu] * e3u[q];
              const double zah = nm->ln_botmix_triad ? pahu[q] : pahu[q] * umask[I3(ji, jj, jk + kp)];
              const double zah_slp = zah * zslope_iso;
              const double zaei_slp = 0.0;
              zftu[q] = zftu[q] - (zah * zdxt + (zah_slp - zaei_slp) * zdzt) * zbu * ze1ur;
              ztfw[w] = ztfw[w] - (zah_slp + zaei_slp) * zdxt * zbu * ze3wr;
            }
      for (int jp = 0; jp <= 1; ++jp)
        for (int kp = 0; kp <= 1; ++kp)
          for (int jj = 1; jj <= jpj - 1; ++jj)
            for (int ji = 1; ji <= jpi - 1; ++ji) {
              const size_t pv = I2(ji, jj), q = I3(ji, jj, jk), w = I3(ji, jj + jp, jk + kp);
              const double ze2vr = c->r1_e2v[pv];
              const double zdyt = zdjt[q] * ze2vr;
              const double ze3wr = 1.0 / e3w[w];
              const double zdzt = (kp ? zdk1 : zdk0)[I2(ji, jj + jp)] * ze3wr;
              const double zslope_iso = tj[TRI(ji, jj + jp, jk, 1 - jp, kp)];
              const double zbv = 0.25 * c->e1e2v[pv] * e3v[q];
              const double zah = nm->ln_botmix_triad ? pahv[q] : pahv[q] * vmask[I3(ji, jj, jk + kp)];
              const double zah_slp = zah * zslope_iso;
              const double zaei_slp = 0.0;
              zftv[q] = zftv[q] - (zah * zdyt + (zah_slp - zaei_slp) * zdzt) * zbv * ze2vr;
              ztfw[w] = ztfw[w] - (zah_slp + zaei_slp) * zdyt * zbv * ze3wr;
            }
      for (int jj = 2; jj <= jpj - 1; ++jj)                              /* :356-363 */
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          ta[q] = ta[q] + zsign * (zftu[I3(ji - 1, jj, jk)] - zftu[q] + zftv[I3(ji, jj - 1, jk)] - zftv[q]) /
                              (c->e1e2t[I2(ji, jj)] * e3t[q]);
        }
    }
    for (int jk = 2; jk <= jpk - 1; ++jk)                                /* :368-402 */
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk), p = I2(ji, jj);
          if (nm->ln_traldf_lap)
            ztfw[q] = ztfw[q] - c->e1e2t[p] / e3w[q] * tmask[q] * (ah_wslp2[q] - akz[q]) * (tb[q - n2] - tb[q]);
          else if (kpass == 1)
            ztfw[q] = ztfw[q] - c->e1e2t[p] / e3w[q] * tmask[q] * ah_wslp2[q] * (tb[q - n2] - tb[q]);
          else
            ztfw[q] = ztfw[q] - c->e1e2t[p] / e3w[q] * tmask[q] *
                                    (ah_wslp2[q] * (tb[q - n2] - tb[q]) + akz[q] * (tbb[q - n2] - tbb[q]));
        }
    for (int jk = 1; jk <= jpk - 1; ++jk)                                /* :404-410 */
      for (int jj = 2; jj <= jpj - 1; ++jj)
        for (int ji = 2; ji <= jpi - 1; ++ji) {
          const size_t q = I3(ji, jj, jk);
          ta[q] = ta[q] + zsign * (ztfw[q + n2] - ztfw[q]) / (c->e1e2t[I2(ji, jj)] * e3t[q]);
        }
  }
  wfree(zdit); wfree(zdjt); wfree(zftu); wfree(zftv); wfree(ztfw); wfree(zdk0); wfree(zdk1);
  return NEMO_OK;
}
#undef TRI

/* ---------------------------------------------------------------- ldf_slp */
/* ldf_slp (ldfslp.F90:83-374) with ldf_slp_mxl (:620-729): z-coordinate without
 * ice-shelf cavities (risfdep = 0, mikt = miku = mikv = 1) and without the
 * s-coordinate level slope; with partial steps (ln_zps) the density gradients of the
 * bottom level are the bound GRU, GRV of zps_hde (:144-151). prd, pn2: in situ density
 * anomaly and N^2; bound: GDEPT_N, GDEPW_N, NMLN (int), HMLP, HMLPT; out: USLP, VSLP,
 * WSLPI, WSLPJ on levels 2..jpk-1 of the interior, then lbc_lnk on every level. */
int ora_ldf_slp(ora_ctx *c, int kt, const double *prd, const double *pn2) {
  (void)kt;
  const nemo_namelist *nm = &c->nam;
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = (size_t)jpi * jpj, n3 = n2 * jpk;
  double *uslp = c->f[NEMO_F_USLP], *vslp = c->f[NEMO_F_VSLP], *wslpi = c->f[NEMO_F_WSLPI], *wslpj = c->f[NEMO_F_WSLPJ];
  const double *gdept = c->f[NEMO_F_GDEPT_N], *gdepw = c->f[NEMO_F_GDEPW_N];
  const double *hmlp = c->f[NEMO_F_HMLP], *hmlpt = c->f[NEMO_F_HMLPT];
  const int *nmln = (const int *)c->f[NEMO_F_NMLN];
  if (!prd || !pn2) return NEMO_ERR_ARG;
  if (!uslp || !vslp || !wslpi || !wslpj || !gdept || !gdepw || !hmlp || !hmlpt || !nmln) return NEMO_ERR_UNBOUND;
  const double *gru = c->f[NEMO_F_GRU], *grv = c->f[NEMO_F_GRV];
  if (nm->ln_isfcav || nm->ln_sco) return NEMO_ERR_UNSUPPORTED;
  if (nm->ln_zps && (!gru || !grv)) return NEMO_ERR_UNBOUND;
  const double *tmask = c->tmask, *umask = c->umask, *vmask = c->vmask, *wmask = c->wmask;
  const double *e3u = fld(c, NEMO_F_E3U_N), *e3v = fld(c, NEMO_F_E3V_N), *e3w = fld(c, NEMO_F_E3W_N);
  const double zeps = 1.e-20, z1_16 = 1.0 / 16., zm1_g = -1.0 / nm->grav, zm1_2g = -0.5 / nm->grav;
  const double z1_slpmax = 1. / (nm->rn_slpmax > 0 ? nm->rn_slpmax : 0.01);
  double *zgru = zalloc(n3), *zgrv = zalloc(n3), *zdzr = zalloc(n3);
  double *zwz = zalloc(n3), *zww = zalloc(n3);
  double *uml = zalloc(n2), *vml = zalloc(n2), *wiml = zalloc(n2), *wjml = zalloc(n2);
  double *hu = zalloc(n2), *hv = zalloc(n2);
#define OML(ji, jj, jk) ((jk) <= nmln[I2(ji, jj)] - 1 ? 1.0 : 0.0)
  /* (:136-143) */
  for (int jk = 1; jk <= jpk; ++jk)
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        zgru[q] = umask[q] * (prd[I3(ji + 1, jj, jk)] - prd[q]);
        zgrv[q] = vmask[q] * (prd[I3(ji, jj + 1, jk)] - prd[q]);
      }
  if (nm->ln_zps)  /* the partial-step gradients at the bottom level (:144-151) */
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        const size_t p = I2(ji, jj);
        zgru[I3(ji, jj, c->mbku[p])] = gru[p];
        zgrv[I3(ji, jj, c->mbkv[p])] = grv[p];
      }
  /* (:161-171) */
  for (size_t p = 0; p < n2; ++p) zdzr[p] = 0.0;
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      size_t q = p + n2 * (jk - 1);
      zdzr[q] = zm1_g * (prd[q] + 1.0) * (pn2[q] + pn2[q + n2]) * (1.0 - 0.5 * tmask[q + n2]);
    }
  /* ldf_slp_mxl (:660-726) */
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      size_t p = I2(ji, jj);
      int n0 = nmln[p], ne = nmln[I2(ji + 1, jj)], nn_ = nmln[I2(ji, jj + 1)];
      int iku = n0 > ne ? n0 : ne; if (iku < 1) iku = 1; if (iku > jpk - 1) iku = jpk - 1;
      int ikv = n0 > nn_ ? n0 : nn_; if (ikv < 1) ikv = 1; if (ikv > jpk - 1) ikv = jpk - 1;
      double zbu = 0.5 * (zdzr[I3(ji, jj, iku)] + zdzr[I3(ji + 1, jj, iku)]);
      double zbv = 0.5 * (zdzr[I3(ji, jj, ikv)] + zdzr[I3(ji, jj + 1, ikv)]);
      double zau = zgru[I3(ji, jj, iku)] * c->r1_e1u[p];
      double zav = zgrv[I3(ji, jj, ikv)] * c->r1_e2v[p];
      zbu = dmin(dmin(zbu, -z1_slpmax * fabs(zau)), -7.e+3 / e3u[I3(ji, jj, iku)] * fabs(zau));
      zbv = dmin(dmin(zbv, -z1_slpmax * fabs(zav)), -7.e+3 / e3v[I3(ji, jj, ikv)] * fabs(zav));
      uml[p] = zau / (zbu - zeps) * umask[I3(ji, jj, iku)];
      vml[p] = zav / (zbv - zeps) * vmask[I3(ji, jj, ikv)];
      int ik = n0 + 1 < jpk ? n0 + 1 : jpk;
      int ikm1 = ik - 1 > 1 ? ik - 1 : 1;
      double zbw = zm1_2g * pn2[I3(ji, jj, ik)] * (prd[I3(ji, jj, ik)] + prd[I3(ji, jj, ikm1)] + 2.);
      double zci = dmax(umask[I3(ji - 1, jj, ik)] + umask[I3(ji, jj, ik)] + umask[I3(ji - 1, jj, ikm1)]
                        + umask[I3(ji, jj, ikm1)], zeps) * c->e1t[p];
      double zcj = dmax(vmask[I3(ji, jj - 1, ik)] + vmask[I3(ji, jj, ik)] + vmask[I3(ji, jj - 1, ikm1)]
                        + vmask[I3(ji, jj, ikm1)], zeps) * c->e2t[p];
      double zai = (zgru[I3(ji - 1, jj, ik)] + zgru[I3(ji, jj, ik)] + zgru[I3(ji - 1, jj, ikm1)]
                    + zgru[I3(ji, jj, ikm1)]) / zci * tmask[I3(ji, jj, ik)];
      double zaj = (zgrv[I3(ji, jj - 1, ik)] + zgrv[I3(ji, jj, ik)] + zgrv[I3(ji, jj - 1, ikm1)]
                    + zgrv[I3(ji, jj, ikm1)]) / zcj * tmask[I3(ji, jj, ik)];
      double zbi = dmin(dmin(zbw, -100. * fabs(zai)), -7.e+3 / e3w[I3(ji, jj, ik)] * fabs(zai));
      double zbj = dmin(dmin(zbw, -100. * fabs(zaj)), -7.e+3 / e3w[I3(ji, jj, ik)] * fabs(zaj));
      wiml[p] = zai / (zbi - zeps) * tmask[I3(ji, jj, ik)];
      wjml[p] = zaj / (zbj - zeps) * tmask[I3(ji, jj, ik)];
    }
  lbc_closed(jpi, jpj, uml, 1, 'U', 0.0); lbc_closed(jpi, jpj, vml, 1, 'V', 0.0);
  lbc_closed(jpi, jpj, wiml, 1, 'W', 0.0); lbc_closed(jpi, jpj, wjml, 1, 'W', 0.0);
  /* (:188-194) */
  for (int jj = 2; jj <= jpj - 1; ++jj)
    for (int ji = 2; ji <= jpi - 1; ++ji) {
      size_t p = I2(ji, jj);
      hu[p] = uml[p] / dmax(dmax(hmlpt[p], hmlpt[I2(ji + 1, jj)]), 5.0);
      hv[p] = vml[p] / dmax(dmax(hmlpt[p], hmlpt[I2(ji, jj + 1)]), 5.0);
    }
  /* (:197-233) slopes at u- and v-points */
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj), q = I3(ji, jj, jk);
        double zau = zgru[q] * c->r1_e1u[p];
        double zav = zgrv[q] * c->r1_e2v[p];
        double zbu = 0.5 * (zdzr[q] + zdzr[I3(ji + 1, jj, jk)]);
        double zbv = 0.5 * (zdzr[q] + zdzr[I3(ji, jj + 1, jk)]);
        zbu = dmin(dmin(zbu, -z1_slpmax * fabs(zau)), -7.e+3 / e3u[q] * fabs(zau));
        zbv = dmin(dmin(zbv, -z1_slpmax * fabs(zav)), -7.e+3 / e3v[q] * fabs(zav));
        double zfi = dmax(OML(ji, jj, jk), OML(ji + 1, jj, jk));
        double zfj = dmax(OML(ji, jj, jk), OML(ji, jj + 1, jk));
        double zdepu = 0.5 * ((gdept[q] + gdept[I3(ji + 1, jj, jk)]) - 2 * 0.0 - e3u[I3(ji, jj, 1)]);
        double zdepv = 0.5 * ((gdept[q] + gdept[I3(ji, jj + 1, jk)]) - 2 * 0.0 - e3v[I3(ji, jj, 1)]);
        zwz[q] = ((1. - zfi) * zau / (zbu - zeps) + zfi * zdepu * hu[p]) * umask[q];
        zww[q] = ((1. - zfj) * zav / (zbv - zeps) + zfj * zdepv * hv[p]) * vmask[q];
      }
  lbc_closed(jpi, jpj, zwz, jpk, 'U', 0.0);
  lbc_closed(jpi, jpj, zww, jpk, 'V', 0.0);
  /* (:236-275) Shapiro filter, decrease along coastal boundaries */
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        uslp[q] = z1_16 * (zwz[I3(ji - 1, jj - 1, jk)] + zwz[I3(ji + 1, jj - 1, jk)]
                           + zwz[I3(ji - 1, jj + 1, jk)] + zwz[I3(ji + 1, jj + 1, jk)]
                           + 2. * (zwz[I3(ji, jj - 1, jk)] + zwz[I3(ji - 1, jj, jk)]
                                   + zwz[I3(ji + 1, jj, jk)] + zwz[I3(ji, jj + 1, jk)])
                           + 4. * zwz[q]);
        vslp[q] = z1_16 * (zww[I3(ji - 1, jj - 1, jk)] + zww[I3(ji + 1, jj - 1, jk)]
                           + zww[I3(ji - 1, jj + 1, jk)] + zww[I3(ji + 1, jj + 1, jk)]
                           + 2. * (zww[I3(ji, jj - 1, jk)] + zww[I3(ji - 1, jj, jk)]
                                   + zww[I3(ji + 1, jj, jk)] + zww[I3(ji, jj + 1, jk)])
                           + 4. * zww[q]);
      }
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        uslp[q] = uslp[q] * (umask[I3(ji, jj + 1, jk)] + umask[I3(ji, jj - 1, jk)]) * 0.5
                          * (umask[q] + umask[I3(ji, jj, jk + 1)]) * 0.5;
        vslp[q] = vslp[q] * (vmask[I3(ji + 1, jj, jk)] + vmask[I3(ji - 1, jj, jk)]) * 0.5
                          * (vmask[q] + vmask[I3(ji, jj, jk + 1)]) * 0.5;
      }
  /* (:281-315) slopes at w-points */
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t p = I2(ji, jj), q = I3(ji, jj, jk);
        double zbw = zm1_2g * pn2[q] * (prd[q] + prd[I3(ji, jj, jk - 1)] + 2.);
        double zci = dmax(umask[I3(ji - 1, jj, jk)] + umask[q] + umask[I3(ji - 1, jj, jk - 1)]
                          + umask[I3(ji, jj, jk - 1)], zeps) * c->e1t[p];
        double zcj = dmax(vmask[I3(ji, jj - 1, jk)] + vmask[I3(ji, jj, jk - 1)] + vmask[I3(ji, jj - 1, jk - 1)]
                          + vmask[q], zeps) * c->e2t[p];
        double zai = (zgru[I3(ji - 1, jj, jk)] + zgru[I3(ji, jj, jk - 1)] + zgru[I3(ji - 1, jj, jk - 1)]
                      + zgru[q]) / zci * wmask[q];
        double zaj = (zgrv[I3(ji, jj - 1, jk)] + zgrv[I3(ji, jj, jk - 1)] + zgrv[I3(ji, jj - 1, jk - 1)]
                      + zgrv[q]) / zcj * wmask[q];
        double zbi = dmin(dmin(zbw, -100. * fabs(zai)), -7.e+3 / e3w[q] * fabs(zai));
        double zbj = dmin(dmin(zbw, -100. * fabs(zaj)), -7.e+3 / e3w[q] * fabs(zaj));
        double zfk = dmax(OML(ji, jj, jk), OML(ji, jj, jk - 1));
        double zck = (gdepw[q] - gdepw[I3(ji, jj, 1)]) / dmax(hmlp[p] - gdepw[I3(ji, jj, 1)], 10.);
        zwz[q] = (zai / (zbi - zeps) * (1. - zfk) + zck * wiml[p] * zfk) * wmask[q];
        zww[q] = (zaj / (zbj - zeps) * (1. - zfk) + zck * wjml[p] * zfk) * wmask[q];
      }
  lbc_closed(jpi, jpj, zwz, jpk, 'T', 0.0);
  lbc_closed(jpi, jpj, zww, jpk, 'T', 0.0);
  /* (:318-361) */
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        double zcofw = wmask[q] * z1_16;
        wslpi[q] = (zwz[I3(ji - 1, jj - 1, jk)] + zwz[I3(ji + 1, jj - 1, jk)]
                    + zwz[I3(ji - 1, jj + 1, jk)] + zwz[I3(ji + 1, jj + 1, jk)]
                    + 2. * (zwz[I3(ji, jj - 1, jk)] + zwz[I3(ji - 1, jj, jk)]
                            + zwz[I3(ji + 1, jj, jk)] + zwz[I3(ji, jj + 1, jk)])
                    + 4. * zwz[q]) * zcofw;
        wslpj[q] = (zww[I3(ji - 1, jj - 1, jk)] + zww[I3(ji + 1, jj - 1, jk)]
                    + zww[I3(ji - 1, jj + 1, jk)] + zww[I3(ji + 1, jj + 1, jk)]
                    + 2. * (zww[I3(ji, jj - 1, jk)] + zww[I3(ji - 1, jj, jk)]
                            + zww[I3(ji + 1, jj, jk)] + zww[I3(ji, jj + 1, jk)])
                    + 4. * zww[q]) * zcofw;
      }
  for (int jk = 2; jk <= jpk - 1; ++jk)
    for (int jj = 2; jj <= jpj - 1; ++jj)
      for (int ji = 2; ji <= jpi - 1; ++ji) {
        size_t q = I3(ji, jj, jk);
        double zck = (umask[q] + umask[I3(ji - 1, jj, jk)]) * (vmask[q] + vmask[I3(ji, jj - 1, jk)]) * 0.25;
        wslpi[q] = wslpi[q] * zck;
        wslpj[q] = wslpj[q] * zck;
      }
  /* (:365) */
  lbc_closed(jpi, jpj, uslp, jpk, 'U', 0.0); lbc_closed(jpi, jpj, vslp, jpk, 'V', 0.0);
  lbc_closed(jpi, jpj, wslpi, jpk, 'W', 0.0); lbc_closed(jpi, jpj, wslpj, jpk, 'W', 0.0);
#undef OML
  wfree(zgru); wfree(zgrv); wfree(zdzr); wfree(zwz); wfree(zww);
  wfree(uml); wfree(vml); wfree(wiml); wfree(wjml); wfree(hu); wfree(hv);
  return NEMO_OK;
}
