// k_dyn.cuh -- split-explicit free surface (dyn_spg_ts, dynspg_ts.F90:121-1310) for a
// linear or a variable-volume free surface, plus lbc_lnk and the compensated global sum.
//
// Phase 1 (forcing of the 2-D system) and phase 3 (correction of the 3-D fields)
// are column kernels. Phase 2, the icycle barotropic sub-steps, is ONE persistent
// cooperative kernel with one bounded grid barrier per sub-step (each block
// recomputes the new ssh of a one-point halo instead of waiting for its owner). The
// three time levels of ssh, u, v
// and the new level live in a ring of 4 slots, so the reference's swap
// (:1176-1186) is an index rotation and no stage overwrites a level a neighbouring
// point still reads. T is the bulk type; the time-filter accumulators ssha, ua_b,
// va_b, un_adv, vn_adv (and the restart fields ub2_b, vb2_b, un_bf, vn_bf) are FP64
// in both precision modes.
#pragma once
#include "nemo_common.cuh"

namespace nemo {

constexpr int KCH3 = 8;  // levels per thread of the phase-3 kernel

template <class T>
struct SpgArgs {
  // 3-D
  T *ua, *va, *un, *vn;
  RO<T> ub, vb;
  // 2-D inputs
  RO<T> sshn, sshb, un_b, vn_b, ub_b, vb_b;
  RO<T> utau, vtau, utau_b, vtau_b, emp, emp_b, rnf, rnf_b;
  RO<T> rCdU_bot, ssh_ib, ssh_ibb;
  // FP64 accumulators / restart fields
  double *ssha, *ua_b, *va_b, *un_adv, *vn_adv, *ub2_b, *vb2_b, *un_bf, *vn_bf;
  // library work arrays (2-D, per member)
  T *zu_frc, *zv_frc, *zssh_frc, *zCdU_u, *zCdU_v;
  T *ring_ssh, *ring_u, *ring_v;  // 4 slots each
  T *fx, *fy;                     // 2 slots each: predictor fluxes zwx, zwy of a sub-step
  T *du, *dv, *cu, *cv;           // phase-3 column terms, computed at the end of phase 2
  T *zmu, *zmv;                   // phase-1 column means, subtracted from ua, va by phase 3
  float* ff;                      // mixed form: the five sums as (hi, lo) float pairs, 10 x nmem2
  RO<double> wgt1, wgt2;
  RO<float> wgtf;                 // mixed form: wgt1 hi | wgt1 lo | wgt2, nwgt entries each
  int nwgt;
  int ln_bt_fw, ln_apr_dyn, nvor, ll_init, icycle, ring0, phase3_filter;
  int cache;  // mixed form, ENE/MIX: the sub-step constants cached in shared memory
  int hot;    // mixed form, linear free surface, ENE/MIX: k_spg_p2_ene instead of k_spg_p2
  // Column depths (2-D): for a linear free surface the rest-state ht_0, hu_0, ...
  // shared by all members (member stride hs = 0); with a variable volume the bound
  // now / before depths of each member (hs = points per member). The Coriolis
  // factors (:241-343) follow the same rule: the domain's, or those k_spg_cor
  // computes from the now depths at every step.
  RO<T> ht_n, hu_n, hv_n, r1_hu_n, r1_hv_n, hu_b, hv_b, r1_hu_b, r1_hv_b;
  RO<T> zwz, ftne, ftnw, ftse, ftsw;
  RO<T> e3f_n;   // (jpi,jpj,jpk) per member: variable volume, ENE/ENS/MIX schemes
  T* cor_w[5];   // k_spg_cor output: zwz, ftne, ftnw, ftse, ftsw per member
  long hs;
  int vvl, flux;  // variable volume; flux-form momentum (variable volume, !ln_dynadv_vec)
  int een_e3f, sco;
  T rdtbt, grav, r1_rau0, scal_load, rn_bt_alpha;
  double rn_atfp, r1_2dt_b;
};

template <class T>
__device__ __forceinline__ long pt_ij(const Dom<T>& d, int i, int j) { return (long)(i - 1) + (long)(j - 1) * d.jpi; }

// ---------------------------------------------------------------------------------
// Phase 1a (:358-367): zu_frc = SUM_k e3u*ua*umask * r1_hu_n. One thread per column,
// all columns. The removal of the mean from ua (:371-378) is left to phase 3, the next
// kernel that touches ua (nothing between reads the 3-D trend): it applies
// (ua - zu_frc*umask) + (ua_b - ub_b)/2dt, the reference's two roundings, in one pass.
template <class T>
__global__ void k_spg_p1a(Dom<T> d, SpgArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int m = blockIdx.z;
  if (i > d.jpi || j > d.jpj) return;
  const long ij = pt_ij(d, i, j), n2 = d.n2, m3 = (long)m * d.n3, m2 = (long)m * n2;
  const ColInfo ci = d.ci[ij];
  T su = T(0), sv = T(0);
  for (int k = 1; k <= d.jpk - 1; ++k) {
    const long q = m3 + ij + (long)(k - 1) * n2;
    su = su + d.e3u_n(ij, k, m) * a.ua[q] * umsk<T>(ci, k);
    sv = sv + d.e3v_n(ij, k, m) * a.va[q] * vmsk<T>(ci, k);
  }
  su = su * a.r1_hu_n[m * a.hs + ij];
  sv = sv * a.r1_hv_n[m * a.hs + ij];
  a.zu_frc[m2 + ij] = su;
  a.zv_frc[m2 + ij] = sv;
  a.zmu[m2 + ij] = su;
  a.zmv[m2 + ij] = sv;
}

// Coriolis factors of one member (:241-343).
template <class T>
struct CorF {
  RO<T> zwz, ftne, ftnw, ftse, ftsw;
};
// hm: member offset of the 2-D depth and factor arrays (m * hs)
template <class T>
__device__ __forceinline__ CorF<T> cor_of(const SpgArgs<T>& a, long hm) {
  return CorF<T>{a.zwz + hm, a.ftne + hm, a.ftnw + hm, a.ftse + hm, a.ftsw + hm};
}

// Barotropic Coriolis trend of a flux field (ENE/MIX, ENS, EET/EEN, ENT) at an
// interior point (:390-443 and :1000-1056). Every scheme reads the same eight
// neighbours, passed preloaded: x[0..3] = zwx at p-1, p, p-1+jpi, p+jpi and
// y[0..3] = zwy at p-jpi, p+1-jpi, p, p+1; for ENT xu / yv are the velocities at
// the same points, h[0..2] the depths at p, p+1, p+jpi and z1_hu / z1_hv the
// inverse depths at the u- / v-point.
template <class T>
__device__ __forceinline__ void coriolis(const Dom<T>& d, const CorF<T>& f, int nvor, long p, const T (&x)[4],
                                         const T (&y)[4], const T (&xu)[4], const T (&yv)[4], const T (&h)[3],
                                         T z1_hu, T z1_hv, T& zu_trd, T& zv_trd) {
  const int jpi = d.jpi;
  const T r1_4 = T(0.25), r1_8 = T(0.125), r1_12 = T(1) / T(12);
  if (nvor == 2) {  // ENT
    const RO<T> e = d.e1e2t;
    const RO<T> ft = d.ff_t;
    zu_trd = +r1_4 * d.r1_e1e2u[p] * z1_hu *
             (e[p + 1] * h[1] * ft[p + 1] * (yv[3] + yv[1]) + e[p] * h[0] * ft[p] * (yv[2] + yv[0]));
    zv_trd = -r1_4 * d.r1_e1e2v[p] * z1_hv *
             (e[p + jpi] * h[2] * ft[p + jpi] * (xu[3] + xu[2]) + e[p] * h[0] * ft[p] * (xu[1] + xu[0]));
  } else if (nvor == 1 || nvor == 5) {  // ENE, MIX
    const T zy1 = (y[0] + y[1]) * d.r1_e1u[p];
    const T zy2 = (y[2] + y[3]) * d.r1_e1u[p];
    const T zx1 = (x[0] + x[2]) * d.r1_e2v[p];
    const T zx2 = (x[1] + x[3]) * d.r1_e2v[p];
    zu_trd = r1_4 * (f.zwz[p - jpi] * zy1 + f.zwz[p] * zy2);
    zv_trd = -r1_4 * (f.zwz[p - 1] * zx1 + f.zwz[p] * zx2);
  } else if (nvor == 0) {  // ENS
    const T zy1 = r1_8 * (y[0] + y[1] + y[2] + y[3]) * d.r1_e1u[p];
    const T zx1 = -r1_8 * (x[0] + x[2] + x[1] + x[3]) * d.r1_e2v[p];
    zu_trd = zy1 * (f.zwz[p - jpi] + f.zwz[p]);
    zv_trd = zx1 * (f.zwz[p - 1] + f.zwz[p]);
  } else {  // EET, EEN
    zu_trd = +r1_12 * d.r1_e1u[p] *
             (f.ftne[p] * y[2] + f.ftnw[p + 1] * y[3] + f.ftse[p] * y[0] + f.ftsw[p + 1] * y[1]);
    zv_trd = -r1_12 * d.r1_e2v[p] *
             (f.ftsw[p + jpi] * x[2] + f.ftse[p + jpi] * x[3] + f.ftnw[p] * x[0] + f.ftne[p] * x[1]);
  }
}

// Coriolis factors of a variable-volume step (:241-343, recomputed at every step
// when ln_linssh = .false.) from the now depths: ht_n for EEN and EET, e3f_n for
// ENE, ENS and MIX. One thread per point and member; the F-point lbc (:265) is
// folded in (column jpi and row jpj are 0).
template <class T>
__global__ void k_spg_cor(Dom<T> d, SpgArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int m = blockIdx.z;
  const int jpi = d.jpi, jpj = d.jpj;
  if (i > jpi || j > jpj) return;
  const long p = pt_ij(d, i, j), m2 = (long)m * d.n2;
  const RO<T> ht = a.ht_n + m2;
  const RO<T> ff = d.ff_f;
  const int sc = a.nvor;
  T zwz = T(0), ne = T(0), nw = T(0), se = T(0), sw = T(0);
  if (sc == 4) {  // EEN: ff_f over the averaged depth at F-points (:249-263)
    auto zw = [&](long q, int ii, int jj) -> T {
      if (ii > jpi - 1 || jj > jpj - 1) return T(0);
      T z = ht[q + jpi] + ht[q + jpi + 1] + ht[q] + ht[q + 1];
      if (a.een_e3f == 0) z = z * T(0.25);
      else z = z / fmx(T(1), d.ssmask[q + jpi] + d.ssmask[q + jpi + 1] + d.ssmask[q] + d.ssmask[q + 1]);
      if (z != T(0)) z = ff[q] / z;
      return z;
    };
    zwz = zw(p, i, j);
    if (i >= 2 && j >= 2) {  // (:267-275)
      const T w_ij = zwz, w_wj = zw(p - 1, i - 1, j), w_is = zw(p - jpi, i, j - 1), w_ws = zw(p - 1 - jpi, i - 1, j - 1);
      ne = w_wj + w_ij + w_is;
      nw = w_ws + w_wj + w_ij;
      se = w_ij + w_is + w_ws;
      sw = w_is + w_ws + w_wj;
    }
  } else if (sc == 3) {  // EET (:278-287)
    if (i >= 2 && j >= 2) {
      const T z1_ht = d.ssmask[p] / (ht[p] + T(1) - d.ssmask[p]);
      ne = (ff[p - 1] + ff[p] + ff[p - jpi]) * z1_ht;
      nw = (ff[p - 1 - jpi] + ff[p - 1] + ff[p]) * z1_ht;
      se = (ff[p] + ff[p - jpi] + ff[p - 1 - jpi]) * z1_ht;
      sw = (ff[p - jpi] + ff[p - 1 - jpi] + ff[p - 1]) * z1_ht;
    }
  } else {  // ENE, ENS, MIX: ff_f / hf with hf the wet e3f_n column (:289-341)
    T zhf = T(0);
    if (i <= jpi - 1 && j <= jpj - 1) {
      if (a.sco)
        zhf = (d.ht_0[p] + d.ht_0[p + 1] + d.ht_0[p + jpi] + d.ht_0[p + jpi + 1]) /
              fmx(d.ssmask[p] + d.ssmask[p + 1] + d.ssmask[p + jpi] + d.ssmask[p + jpi + 1], T(1));
      const ColInfo c0 = d.ci[p], c1 = d.ci[p + jpi];
      zhf = zhf * (T(1) - umsk<T>(c0, 1) * umsk<T>(c1, 1));
      const RO<T> e3f = a.e3f_n + (long)m * d.n3 + p;
      for (int k = 1; k <= d.jpk - 1; ++k) zhf = zhf + e3f[(long)(k - 1) * d.n2] * umsk<T>(c0, k) * umsk<T>(c1, k);
    }
    T r = T(0);
    if (zhf != T(0)) r = T(1) / zhf;
    zwz = ff[p] * r;
  }
  a.cor_w[0][m2 + p] = zwz;
  a.cor_w[1][m2 + p] = ne;
  a.cor_w[2][m2 + p] = nw;
  a.cor_w[3][m2 + p] = se;
  a.cor_w[4][m2 + p] = sw;
}

// the eight neighbours of p that coriolis() reads, of a point function f
template <class T, class F>
__device__ __forceinline__ void nbx(F f, long p, int jpi, T (&x)[4]) {
  x[0] = f(p - 1); x[1] = f(p); x[2] = f(p - 1 + jpi); x[3] = f(p + jpi);
}
template <class T, class F>
__device__ __forceinline__ void nby(F f, long p, int jpi, T (&y)[4]) {
  y[0] = f(p - jpi); y[1] = f(p + 1 - jpi); y[2] = f(p); y[3] = f(p + 1);
}

// Phase 1b (:387-702): Coriolis of the now barotropic flow, bottom stress, wind,
// atmospheric pressure, ssh forcing, initial barotropic levels, zeroed sums.
template <class T>
__device__ __forceinline__ void spg_p1b_point(const Dom<T>& d, const SpgArgs<T>& a, int i, int j, int m) {
  const long p = pt_ij(d, i, j), n2 = d.n2, m2 = (long)m * n2, m3 = (long)m * d.n3, hm = (long)m * a.hs;
  const T r1_2 = T(0.5);
  const bool interior = i >= 2 && i <= d.jpi - 1 && j >= 2 && j <= d.jpj - 1;
  if (interior) {
    const RO<T> unb = a.un_b + m2;
    const RO<T> vnb = a.vn_b + m2;
    const RO<T> hun = a.hu_n + hm, hvn = a.hv_n + hm, r1hu = a.r1_hu_n + hm, r1hv = a.r1_hv_n + hm;
    auto fx = [&](long q) -> T { return unb[q] * hun[q] * d.e2u[q]; };
    auto fy = [&](long q) -> T { return vnb[q] * hvn[q] * d.e1v[q]; };
    auto fu = [&](long q) -> T { return unb[q]; };
    auto fv = [&](long q) -> T { return vnb[q]; };
    T x[4], y[4], xu[4] = {}, yv[4] = {};
    nbx(fx, p, d.jpi, x);
    nby(fy, p, d.jpi, y);
    if (a.nvor == 2) {
      nbx(fu, p, d.jpi, xu);
      nby(fv, p, d.jpi, yv);
    }
    T h[3] = {};
    if (a.nvor == 2) {
      const RO<T> ht = a.ht_n + hm;
      h[0] = ht[p]; h[1] = ht[p + 1]; h[2] = ht[p + d.jpi];
    }
    T zu_trd, zv_trd;
    coriolis(d, cor_of(a, hm), a.nvor, p, x, y, xu, yv, h, r1hu[p], r1hv[p], zu_trd, zv_trd);
    if (a.vvl) {  // variable volume: remove the surface pressure gradient (:447-509)
      const RO<T> sn = a.sshn + m2;
      zu_trd = zu_trd - a.grav * (sn[p + 1] - sn[p]) * d.r1_e1u[p];
      zv_trd = zv_trd - a.grav * (sn[p + d.jpi] - sn[p]) * d.r1_e2v[p];
    }
    T zu = a.zu_frc[m2 + p] - zu_trd * d.ssumask[p];
    T zv = a.zv_frc[m2 + p] - zv_trd * d.ssvmask[p];
    // bottom stress from the baroclinic bottom velocity (:519-557)
    const ColInfo ci = d.ci[p];
    const long qu = m3 + p + (long)(ci.mbku - 1) * n2, qv = m3 + p + (long)(ci.mbkv - 1) * n2;
    T zwx, zwy;
    if (a.ln_bt_fw) { zwx = a.un[qu] - unb[p]; zwy = a.vn[qv] - vnb[p]; }
    else { zwx = a.ub[qu] - a.ub_b[m2 + p]; zwy = a.vb[qv] - a.vb_b[m2 + p]; }
    const RO<T> cdu = a.rCdU_bot + m2;
    zu = zu + r1hu[p] * r1_2 * (cdu[p + 1] + cdu[p]) * zwx;
    zv = zv + r1hv[p] * r1_2 * (cdu[p + d.jpi] + cdu[p]) * zwy;
    // wind (:589-604)
    if (a.ln_bt_fw) {
      zu = zu + a.r1_rau0 * a.utau[m2 + p] * r1hu[p];
      zv = zv + a.r1_rau0 * a.vtau[m2 + p] * r1hv[p];
    } else {
      const T zztmp = a.r1_rau0 * r1_2;
      zu = zu + zztmp * (a.utau_b[m2 + p] + a.utau[m2 + p]) * r1hu[p];
      zv = zv + zztmp * (a.vtau_b[m2 + p] + a.vtau[m2 + p]) * r1hv[p];
    }
    // atmospheric pressure (:606-629)
    if (a.ln_apr_dyn) {
      const RO<T> ib = a.ssh_ib + m2;
      T zu_spg, zv_spg;
      if (a.ln_bt_fw) {
        zu_spg = a.grav * (ib[p + 1] - ib[p]) * d.r1_e1u[p];
        zv_spg = a.grav * (ib[p + d.jpi] - ib[p]) * d.r1_e2v[p];
      } else {
        const RO<T> ibb = a.ssh_ibb + m2;
        const T zztmp = a.grav * r1_2;
        zu_spg = zztmp * (ib[p + 1] - ib[p] + ibb[p + 1] - ibb[p]) * d.r1_e1u[p];
        zv_spg = zztmp * (ib[p + d.jpi] - ib[p] + ibb[p + d.jpi] - ibb[p]) * d.r1_e2v[p];
      }
      zu = zu + zu_spg;
      zv = zv + zv_spg;
    }
    a.zu_frc[m2 + p] = zu;
    a.zv_frc[m2 + p] = zv;
    a.zCdU_u[m2 + p] = r1_2 * (cdu[p + 1] + cdu[p]);
    a.zCdU_v[m2 + p] = r1_2 * (cdu[p + d.jpi] + cdu[p]);
  }
  // ssh forcing (:633-639); rnf / fwfisf are 0 when absent
  {
    const T r = a.rnf ? a.rnf[m2 + p] : T(0);
    T f;
    if (a.ln_bt_fw) f = a.r1_rau0 * (a.emp[m2 + p] - r + T(0));
    else {
      const T rb = a.rnf_b ? a.rnf_b[m2 + p] : T(0);
      f = a.r1_rau0 * r1_2 * (a.emp[m2 + p] + a.emp_b[m2 + p] - r - rb + T(0) + T(0));
    }
    a.zssh_frc[m2 + p] = f;
  }
  // initial barotropic levels (:665-693) in ring slots n = ring0, b, bb
  const long nmem2 = (long)d.nmem * n2;
  const int sn = a.ring0 & 3, sb = (a.ring0 + 1) & 3, sbb = (a.ring0 + 2) & 3;
  if (a.ll_init) {
    a.ring_ssh[sbb * nmem2 + m2 + p] = T(0); a.ring_u[sbb * nmem2 + m2 + p] = T(0); a.ring_v[sbb * nmem2 + m2 + p] = T(0);
    a.ring_ssh[sb * nmem2 + m2 + p] = T(0); a.ring_u[sb * nmem2 + m2 + p] = T(0); a.ring_v[sb * nmem2 + m2 + p] = T(0);
  }
  if (a.ln_bt_fw) {
    a.ring_ssh[sn * nmem2 + m2 + p] = a.sshn[m2 + p];
    a.ring_u[sn * nmem2 + m2 + p] = a.un_b[m2 + p];
    a.ring_v[sn * nmem2 + m2 + p] = a.vn_b[m2 + p];
  } else {
    a.ring_ssh[sn * nmem2 + m2 + p] = a.sshb[m2 + p];
    a.ring_u[sn * nmem2 + m2 + p] = a.ub_b[m2 + p];
    a.ring_v[sn * nmem2 + m2 + p] = a.vb_b[m2 + p];
  }
  a.ua_b[m2 + p] = 0.0; a.va_b[m2 + p] = 0.0; a.ssha[m2 + p] = 0.0;
  a.un_adv[m2 + p] = 0.0; a.vn_adv[m2 + p] = 0.0;
}

template <class T>
__global__ void k_spg_p1b(Dom<T> d, SpgArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  spg_p1b_point(d, a, i, j, (int)blockIdx.z);
}

// Phase 1a for FP32 and jpk = NK known at compile time: the column of ua / va is
// loaded whole into registers and summed in the reference's order, so all loads are
// in flight together.
template <int NK>
__global__ void __launch_bounds__(128, 8) k_spg_p1a_reg(Dom<float> d, SpgArgs<float> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int m = blockIdx.z;
  if (i > d.jpi || j > d.jpj) return;
  const long ij = pt_ij(d, i, j), n2 = d.n2, m2 = (long)m * n2;
  const ColInfo ci = d.ci[ij];
  // read-only loads (this kernel writes neither ua nor va)
  const float* ua = a.ua + (long)m * d.n3 + ij;
  const float* va = a.va + (long)m * d.n3 + ij;
  float u[NK - 1], v[NK - 1];
#pragma unroll
  for (int k = 1; k <= NK - 1; ++k) {
    u[k - 1] = __ldg(ua + (k - 1) * n2);
    v[k - 1] = __ldg(va + (k - 1) * n2);
  }
  float su = 0.f, sv = 0.f;
#pragma unroll
  for (int k = 1; k <= NK - 1; ++k) {
    su = su + d.e3u_n(ij, k, m) * u[k - 1] * umsk<float>(ci, k);
    sv = sv + d.e3v_n(ij, k, m) * v[k - 1] * vmsk<float>(ci, k);
  }
  su = su * a.r1_hu_n[m * a.hs + ij];
  sv = sv * a.r1_hv_n[m * a.hs + ij];
  a.zu_frc[m2 + ij] = su;
  a.zv_frc[m2 + ij] = sv;
  a.zmu[m2 + ij] = su;
  a.zmv[m2 + ij] = sv;
}


// Predictor (AB3) and AM4 coefficients of sub-step jn (:724-732, :904-928).
template <class T>
__device__ __forceinline__ void ab3(int jn, int ll_init, T& za1, T& za2, T& za3) {
  if (jn < 3 && ll_init) { za1 = T(1); za2 = T(0); za3 = T(0); }
  else { za1 = T(1.781105); za2 = T(-1.06221); za3 = T(0.281105); }
}
template <class T>
__device__ __forceinline__ void am4(int jn, int ll_init, T alpha, T& za0, T& za1, T& za2, T& za3) {
  if (jn == 1 && ll_init) { za0 = T(1); za1 = T(0); za2 = T(0); za3 = T(0); }
  else if (jn == 2 && ll_init) { za0 = T(1.0833333333333); za1 = T(-0.1666666666666); za2 = T(0.0833333333333); za3 = T(0); }
  else if (alpha == T(0)) { za0 = T(0.614); za1 = T(0.285); za2 = T(0.088); za3 = T(0.013); }
  else {
    const T zepsilon = T(0.00976186) - T(0.13451357) * alpha;
    const T zgamma = T(0.08344500) - T(0.51358400) * alpha;
    za0 = T(0.5) + zgamma + T(2) * alpha + T(2) * zepsilon;
    za1 = T(1) - za0 - zgamma - zepsilon;
    za2 = zgamma;
    za3 = zepsilon;
  }
}

// Phase 2 (:664-1207): the icycle sub-steps in one persistent cooperative kernel,
// ONE grid barrier per sub-step. Blocks own 32 x 8 tiles of points. In sub-step jn
// a block first computes, for its tile and a one-point halo to the east and north,
// the new ssh (ssha_e, :871-879) and the AM4 ssh zsshp2_e (:930-931) into shared
// memory -- from the predictor fluxes and ssh levels published before the last
// barrier -- and keeps ssha_e and the ssha sum (:1204) of the points it owns; then,
// per owned point, the Coriolis, drag and pressure-gradient trends, ua_e / va_e and
// their sums (:1000-1204), and the predictor fluxes of sub-step jn+1 (:724-800) with
// their un_adv / vn_adv sums (:860-862). Reads and writes of one sub-step never
// touch the same ring slot or flux buffer, so one barrier separates sub-steps.
constexpr int P2_TX = 32, P2_TY = 8;
// Constant cache of the mixed form (ENE/MIX vorticity): P2_NC floats per point of
// each of up to P2_MAXT tiles a block owns, in dynamic shared memory.
constexpr int P2_NC = 16, P2_MAXT = 3;
constexpr size_t P2_CACHE_BYTES = (size_t)P2_NC * P2_MAXT * 256 * sizeof(float);

// The time-filter sums of the sub-steps (ssha, ua_b, va_b :1202-1204; un_adv,
// vn_adv :860-862). FP64 form: the reference's FP64 accumulation. Mixed form: each
// sum is a float pair hi + lo, updated with an exact product (the FMA residual) and
// a two-sum on the FP32 pipe -- error ~2^-46 of the sum, far below the FP32 storage
// of the summed values -- and converted to the FP64 fields once, at the end of the
// kernel. (FP64 arithmetic runs at 1/64 of the FP32 rate on this GPU, and five FP64
// sums per point per sub-step would occupy its FP64 pipe.) The intrinsics keep the
// compiler from contracting the compensated steps.
struct FF {
  float h, l;
};
// s += p + e, with |e| small against p
__device__ __forceinline__ void ff_add(FF& s, float p, float e) {
  const float t = __fadd_rn(s.h, p);
  const float bp = __fadd_rn(t, -s.h);
  const float err = __fadd_rn(__fadd_rn(s.h, -__fadd_rn(t, -bp)), __fadd_rn(p, -bp));
  s.l = __fadd_rn(s.l, __fadd_rn(err, e));
  s.h = t;
}
// s += w * x with the FP64 weight w split as wh + wl
__device__ __forceinline__ void ff_add_w(FF& s, float wh, float wl, float x) {
  const float p = __fmul_rn(wh, x);
  const float e = __fadd_rn(__fmaf_rn(wh, x, -p), __fmul_rn(wl, x));
  ff_add(s, p, e);
}
// index of the hi / lo float of sum `which` (0 ssha, 1 ua_b, 2 va_b, 3 un_adv,
// 4 vn_adv) at point g
__device__ __forceinline__ long ffi(int which, int part, int nmem2, int g) {
  return (long)(2 * which + part) * nmem2 + g;
}

template <class T>
__device__ __forceinline__ int p2_tiles(const Dom<T>& d) {
  return ((d.jpi + P2_TX - 1) / P2_TX) * ((d.jpj + P2_TY - 1) / P2_TY) * d.nmem;
}

template <class T, bool VVL>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) k_spg_p2(Dom<T> d, SpgArgs<T> a, GridBar bar) {
  unsigned int bar_epoch = 0;  // barriers passed by this block
  // two buffers, alternating between a block's tiles: a warp may start the next
  // tile while others still read this one's (the block barrier between the two
  // stages of the next tile orders the reuse)
  __shared__ T zs_b[2][P2_TY + 1][P2_TX + 1];
  // Variable volume: the new ssh ssha_e [0], the predictor ssh of the next sub-step
  // [1] and the now ssh [2] of the tile and its halo, for the depths at u- and
  // v-points that average two neighbouring T-points.
  __shared__ T vv_b[2][VVL ? 3 : 1][P2_TY + 1][P2_TX + 1];
  const int n2 = (int)d.n2;
  const int nmem2 = d.nmem * n2;
  const int jpi = d.jpi, jpj = d.jpj;
  const int ntx = (jpi + P2_TX - 1) / P2_TX, nty = (jpj + P2_TY - 1) / P2_TY;
  const int ntile = ntx * nty * d.nmem;
  const int tx = threadIdx.x % P2_TX, ty = threadIdx.x / P2_TX;
  const T grav = a.grav, rdtbt = a.rdtbt;
  // forcing of the sub-steps, written by phase 1 and only read here
  const RO<T> zssh_frc = a.zssh_frc, zu_frc = a.zu_frc, zv_frc = a.zv_frc, zCdU_u = a.zCdU_u, zCdU_v = a.zCdU_v;
  int r = a.ring0;
  auto interior = [&](int i, int j) -> bool { return i >= 2 && i <= jpi - 1 && j >= 2 && j <= jpj - 1; };
  // tile t -> member offset m2 and the 1-based indices of its first point
  auto tile = [&](int t, int& m2, int& i0, int& j0) {
    const int m = t / (ntx * nty), tt = t - m * (ntx * nty);
    m2 = m * n2;
    i0 = (tt % ntx) * P2_TX + 1;
    j0 = (tt / ntx) * P2_TY + 1;
  };
  // ssh averaged to the u- / v-point of interior point p from its values at p and
  // at the east / north neighbour (:766-773, :888-895, :976-983)
  const T r1_2 = T(0.5);
  auto ssh_u = [&](int p, T s0, T se) -> T {
    return r1_2 * d.ssumask[p] * d.r1_e1e2u[p] * (d.e1e2t[p] * s0 + d.e1e2t[p + 1] * se);
  };
  auto ssh_v = [&](int p, T s0, T sn) -> T {
    return r1_2 * d.ssvmask[p] * d.r1_e1e2v[p] * (d.e1e2t[p] * s0 + d.e1e2t[p + jpi] * sn);
  };
  // predictor fluxes of sub-step jn from the owner's levels (:724-800) and their
  // un_adv / vn_adv sums (:860-862)
  auto predictor = [&](int jn, int rr, int m2, int p, bool inner) {
    const int g = m2 + p;
    T za1, za2, za3;
    ab3(jn, a.ll_init, za1, za2, za3);
    const int sn = rr & 3, sb = (rr + 1) & 3, sbb = (rr + 2) & 3;
    const T ua_e = za1 * a.ring_u[sn * nmem2 + g] + za2 * a.ring_u[sb * nmem2 + g] + za3 * a.ring_u[sbb * nmem2 + g];
    const T va_e = za1 * a.ring_v[sn * nmem2 + g] + za2 * a.ring_v[sb * nmem2 + g] + za3 * a.ring_v[sbb * nmem2 + g];
    T hu = d.hu_0[p], hv = d.hv_0[p];
    if constexpr (VVL) {  // depth from the extrapolated ssh (:738-792)
      if (inner) {
        auto s_at = [&](int q) -> T {
          return za1 * a.ring_ssh[sn * nmem2 + m2 + q] + za2 * a.ring_ssh[sb * nmem2 + m2 + q] +
                 za3 * a.ring_ssh[sbb * nmem2 + m2 + q];
        };
        const T s0 = s_at(p);
        hu = hu + ssh_u(p, s0, s_at(p + 1));
        hv = hv + ssh_v(p, s0, s_at(p + jpi));
      }
    }
    const T zwx = d.e2u[p] * ua_e * hu;
    const T zwy = d.e1v[p] * va_e * hv;
    a.fx[(jn & 1) * nmem2 + g] = zwx;
    a.fy[(jn & 1) * nmem2 + g] = zwy;
    T w2;
    if constexpr (sizeof(T) == 8) w2 = a.wgt2[jn - 1];
    else w2 = a.wgtf[2 * a.nwgt + jn - 1];
    if constexpr (sizeof(T) == 8) {
      a.un_adv[g] = a.un_adv[g] + (double)(w2 * zwx * d.r1_e2u[p]);
      a.vn_adv[g] = a.vn_adv[g] + (double)(w2 * zwy * d.r1_e1v[p]);
    } else {  // first predictor of the kernel: the sums start here
      for (int w = 0; w < 10; ++w) a.ff[(long)w * nmem2 + g] = 0.0f;
      a.ff[ffi(3, 0, nmem2, g)] = w2 * zwx * d.r1_e2u[p];
      a.ff[ffi(4, 0, nmem2, g)] = w2 * zwy * d.r1_e1v[p];
    }
  };
  if (a.icycle >= 1)
    for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
      int m2, i0, j0;
      tile(t, m2, i0, j0);
      const int i = i0 + tx, j = j0 + ty;
      if (i <= jpi && j <= jpj) {
        const int p = (i - 1) + (j - 1) * jpi;
        predictor(1, r, m2, p, interior(i, j));
      }
    }
  // Mixed form with the ENE/MIX scheme and a linear free surface: the per-point
  // constants of the Coriolis, drag, pressure-gradient and predictor terms, combined
  // once and kept in shared memory for the whole kernel (the barrier's acquire
  // empties L1 every sub-step, so they would otherwise come from L2 after each
  // tile's __syncthreads). Each thread writes and reads only its own entries. FP32
  // products in another association than the general path below: within the mixed
  // form's tolerance.
  extern __shared__ float p2c[];
  const bool cache = !VVL && sizeof(T) == 4 && a.cache;
  if (cache) {
    int slot = 0;
    for (int t = blockIdx.x; t < ntile && slot < P2_MAXT; t += gridDim.x, ++slot) {
      int m2, i0, j0;
      tile(t, m2, i0, j0);
      const int i = i0 + tx, j = j0 + ty;
      float cv[P2_NC] = {};
      if (i <= jpi && j <= jpj) {
        const int p = (i - 1) + (j - 1) * jpi, g = m2 + p;
        if (interior(i, j)) {
          const float su = (float)(T(1) - a.scal_load) * (float)(-grav);
          cv[0] = 0.25f * (float)d.zwz[p - jpi] * (float)d.r1_e1u[p];  // times fy(p-jpi) + fy(p+1-jpi)
          cv[1] = 0.25f * (float)d.zwz[p] * (float)d.r1_e1u[p];        // times fy(p) + fy(p+1)
          cv[2] = -0.25f * (float)d.zwz[p - 1] * (float)d.r1_e2v[p];   // times fx(p-1) + fx(p-1+jpi)
          cv[3] = -0.25f * (float)d.zwz[p] * (float)d.r1_e2v[p];       // times fx(p) + fx(p+jpi)
          cv[4] = (float)zCdU_u[g] * (float)d.r1_hu_0[p];
          cv[5] = (float)zCdU_v[g] * (float)d.r1_hv_0[p];
          cv[6] = su * (float)d.r1_e1u[p];
          cv[7] = su * (float)d.r1_e2v[p];
          cv[8] = (float)zu_frc[g];
          cv[9] = (float)zv_frc[g];
          cv[10] = (float)d.ssumask[p];
          cv[11] = (float)d.ssvmask[p];
        }
        cv[12] = (float)d.e2u[p] * (float)d.hu_0[p];
        cv[13] = (float)d.e1v[p] * (float)d.hv_0[p];
        cv[14] = (float)d.r1_e2u[p];
        cv[15] = (float)d.r1_e1v[p];
      }
#pragma unroll
      for (int cc = 0; cc < P2_NC; ++cc) p2c[(cc * P2_MAXT + slot) * 256 + threadIdx.x] = cv[cc];
    }
  }
  if (!grid_barrier(bar, bar_epoch)) return;
  for (int jn = 1; jn <= a.icycle; ++jn) {
    const int sn = r & 3, sb = (r + 1) & 3, sbb = (r + 2) & 3, sa = (r + 3) & 3;
    const T* fx = a.fx + (jn & 1) * nmem2;
    const T* fy = a.fy + (jn & 1) * nmem2;
    double w1 = 0.0;         // FP64 form
    float w1h = 0.f, w1l = 0.f;  // mixed form: w1 = w1h + w1l
    if constexpr (sizeof(T) == 8) {
      w1 = a.wgt1[jn - 1];
    } else {
      w1h = a.wgtf[jn - 1];
      w1l = a.wgtf[a.nwgt + jn - 1];
    }
    T zb0, zb1, zb2, zb3;
    am4(jn, a.ll_init, a.rn_bt_alpha, zb0, zb1, zb2, zb3);
    T zc1 = T(0), zc2 = T(0), zc3 = T(0);  // predictor coefficients of sub-step jn+1
    if constexpr (VVL) ab3(jn + 1, a.ll_init, zc1, zc2, zc3);
    int slot = 0;  // the tile's place in the constant cache
    for (int t = blockIdx.x; t < ntile; t += gridDim.x, ++slot) {
      int m2, i0, j0;
      tile(t, m2, i0, j0);
      auto& zs_s = zs_b[slot & 1];
      auto& vv_s = vv_b[slot & 1];
      const long hm = VVL ? m2 : 0;  // member offset of the depths and Coriolis factors
      // Every value this tile reads that the sub-step does not produce is loaded
      // first, so the loads of both stages are in flight together.
      const int i = i0 + tx, j = j0 + ty;
      const bool own = i <= jpi && j <= jpj;
      const bool inner = own && interior(i, j);
      const int p = own ? (i - 1) + (j - 1) * jpi : 0, g = m2 + p;
      T x[4] = {}, y[4] = {}, xu[4] = {}, yv[4] = {};
      T sn0 = T(0), sb0 = T(0), sbb0 = T(0), un_e = T(0), vn_e = T(0), ub_e = T(0), vb_e = T(0);
      // ENT / flux form: the predictor depths of sub-step jn at the u- and v-point
      // and at p, p+1, p+jpi (:738-792)
      T hup = T(0), hvp = T(0), hq[3] = {};
      double acc_s = 0.0, acc_u = 0.0, acc_v = 0.0, acc_au = 0.0, acc_av = 0.0;  // FP64 form
      FF f_s{}, f_u{}, f_v{}, f_au{}, f_av{};                                    // mixed form
      if (own) {
        sn0 = a.ring_ssh[sn * nmem2 + g];
        sb0 = a.ring_ssh[sb * nmem2 + g];
        sbb0 = a.ring_ssh[sbb * nmem2 + g];
        un_e = a.ring_u[sn * nmem2 + g];
        vn_e = a.ring_v[sn * nmem2 + g];
        ub_e = a.ring_u[sb * nmem2 + g];
        vb_e = a.ring_v[sb * nmem2 + g];
        if constexpr (sizeof(T) == 8) {
          acc_s = a.ssha[g]; acc_u = a.ua_b[g]; acc_v = a.va_b[g];
          acc_au = a.un_adv[g]; acc_av = a.vn_adv[g];
        } else {
          f_s = FF{a.ff[ffi(0, 0, nmem2, g)], a.ff[ffi(0, 1, nmem2, g)]};
          f_u = FF{a.ff[ffi(1, 0, nmem2, g)], a.ff[ffi(1, 1, nmem2, g)]};
          f_v = FF{a.ff[ffi(2, 0, nmem2, g)], a.ff[ffi(2, 1, nmem2, g)]};
          f_au = FF{a.ff[ffi(3, 0, nmem2, g)], a.ff[ffi(3, 1, nmem2, g)]};
          f_av = FF{a.ff[ffi(4, 0, nmem2, g)], a.ff[ffi(4, 1, nmem2, g)]};
        }
        if (inner) {
          nbx([&](long q) { return fx[m2 + q]; }, (long)p, jpi, x);
          nby([&](long q) { return fy[m2 + q]; }, (long)p, jpi, y);
          T za1, za2, za3;
          ab3(jn, a.ll_init, za1, za2, za3);
          if (a.nvor == 2) {  // the ENT scheme uses the extrapolated velocities
            auto uext = [&](long q) -> T {
              return za1 * a.ring_u[sn * nmem2 + m2 + q] + za2 * a.ring_u[sb * nmem2 + m2 + q] +
                     za3 * a.ring_u[sbb * nmem2 + m2 + q];
            };
            auto vext = [&](long q) -> T {
              return za1 * a.ring_v[sn * nmem2 + m2 + q] + za2 * a.ring_v[sb * nmem2 + m2 + q] +
                     za3 * a.ring_v[sbb * nmem2 + m2 + q];
            };
            nbx(uext, (long)p, jpi, xu);
            nby(vext, (long)p, jpi, yv);
          }
          if constexpr (VVL) {
            if (a.nvor == 2 || a.flux) {
              auto s_at = [&](int q) -> T {
                return za1 * a.ring_ssh[sn * nmem2 + m2 + q] + za2 * a.ring_ssh[sb * nmem2 + m2 + q] +
                       za3 * a.ring_ssh[sbb * nmem2 + m2 + q];
              };
              const T s0 = za1 * sn0 + za2 * sb0 + za3 * sbb0, se = s_at(p + 1), so = s_at(p + jpi);
              hup = d.hu_0[p] + ssh_u(p, s0, se);
              hvp = d.hv_0[p] + ssh_v(p, s0, so);
              hq[0] = d.ht_0[p] + s0;
              hq[1] = d.ht_0[p + 1] + se;
              hq[2] = d.ht_0[p + jpi] + so;
            }
          }
        }
      }
      // the halo position of this thread, if any: the east column (9) and the
      // north row (32) of the tile
      int hti = -1, htj = -1;
      if (threadIdx.x < P2_TY + 1) { hti = P2_TX; htj = threadIdx.x; }
      else if (threadIdx.x < P2_TY + 1 + P2_TX) { hti = threadIdx.x - (P2_TY + 1); htj = P2_TY; }
      const int hi_ = i0 + hti, hj_ = j0 + htj;
      const bool halo = hti >= 0 && hi_ <= jpi && hj_ <= jpj;
      const int hp = halo ? (hi_ - 1) + (hj_ - 1) * jpi : 0, hg = m2 + hp;
      T h_fx0 = T(0), h_fxw = T(0), h_fy0 = T(0), h_fys = T(0), h_sn = T(0), h_sb = T(0), h_sbb = T(0);
      if (halo) {
        h_sn = a.ring_ssh[sn * nmem2 + hg];
        h_sb = a.ring_ssh[sb * nmem2 + hg];
        h_sbb = a.ring_ssh[sbb * nmem2 + hg];
        if (interior(hi_, hj_)) {
          h_fx0 = fx[hg]; h_fxw = fx[hg - 1]; h_fy0 = fy[hg]; h_fys = fy[hg - jpi];
        }
      }
      // ---- ssha_e (:871-879) and zsshp2_e (:930-931) of the owned point and the halo
      // position; the owned point's new level and ssha sum (:1204)
      if (own) {
        T ssha_e = T(0);
        if (inner) {
          const T zhdiv = (x[1] - x[0] + y[2] - y[0]) * d.r1_e1e2t[p];
          ssha_e = (sn0 - rdtbt * (zssh_frc[g] + zhdiv)) * d.ssmask[p];
        }
        zs_s[ty][tx] = zb0 * ssha_e + zb1 * sn0 + zb2 * sb0 + zb3 * sbb0;
        if constexpr (VVL) {
          vv_s[0][ty][tx] = ssha_e;
          vv_s[1][ty][tx] = zc1 * ssha_e + zc2 * sn0 + zc3 * sb0;
          vv_s[2][ty][tx] = sn0;
        }
        a.ring_ssh[sa * nmem2 + g] = ssha_e;
        if constexpr (sizeof(T) == 8) {
          a.ssha[g] = acc_s + w1 * (double)ssha_e;
        } else {
          ff_add_w(f_s, w1h, w1l, ssha_e);
          a.ff[ffi(0, 0, nmem2, g)] = f_s.h;
          a.ff[ffi(0, 1, nmem2, g)] = f_s.l;
        }
      }
      if (halo) {
        T ssha_e = T(0);
        if (interior(hi_, hj_)) {
          const T zhdiv = (h_fx0 - h_fxw + h_fy0 - h_fys) * d.r1_e1e2t[hp];
          ssha_e = (h_sn - rdtbt * (zssh_frc[hg] + zhdiv)) * d.ssmask[hp];
        }
        zs_s[htj][hti] = zb0 * ssha_e + zb1 * h_sn + zb2 * h_sb + zb3 * h_sbb;
        if constexpr (VVL) {
          vv_s[0][htj][hti] = ssha_e;
          vv_s[1][htj][hti] = zc1 * ssha_e + zc2 * h_sn + zc3 * h_sb;
          vv_s[2][htj][hti] = h_sn;
        }
      }
      __syncthreads();
      // ---- Coriolis, drag, pressure gradient, ua_e/va_e and their sums (:1000-1204),
      // then the predictor of sub-step jn+1 (:724-800) and its sums (:860-862)
      if (own) {
        T ua_e = T(0), va_e = T(0);
        // variable volume: depth of the new level, hu_0 + zsshu_a (:888-900, :1159-1165)
        T hu_a = d.hu_0[p], hv_a = d.hv_0[p];
        if constexpr (VVL) {
          if (inner) {
            hu_a = d.hu_0[p] + ssh_u(p, vv_s[0][ty][tx], vv_s[0][ty][tx + 1]);
            hv_a = d.hv_0[p] + ssh_v(p, vv_s[0][ty][tx], vv_s[0][ty + 1][tx]);
          }
        }
        // the cached constants of this point: C[c * P2_MAXT * 256]
        const float* C = p2c + slot * 256 + threadIdx.x;
        constexpr int CS = P2_MAXT * 256;
        if (inner && cache) {
          const T s0 = zs_s[ty][tx];
          const T zu_trd = C[0] * (y[0] + y[1]) + C[CS] * (y[2] + y[3]) + C[4 * CS] * un_e;
          const T zv_trd = C[2 * CS] * (x[0] + x[2]) + C[3 * CS] * (x[1] + x[3]) + C[5 * CS] * vn_e;
          const T wxs = C[6 * CS] * (zs_s[ty][tx + 1] - s0);
          const T wys = C[7 * CS] * (zs_s[ty + 1][tx] - s0);
          ua_e = (un_e + rdtbt * (wxs + zu_trd + C[8 * CS])) * C[10 * CS];
          va_e = (vn_e + rdtbt * (wys + zv_trd + C[9 * CS])) * C[11 * CS];
        } else if (inner) {
          T z1_hu = T(0), z1_hv = T(0);
          if constexpr (!VVL) {  // rest-state depths, loaded here to keep them out of stage A
            if (a.nvor == 2) {
              hup = d.hu_0[p];
              hvp = d.hv_0[p];
              hq[0] = d.ht_0[p];
              hq[1] = d.ht_0[p + 1];
              hq[2] = d.ht_0[p + jpi];
            }
          }
          if (a.nvor == 2) {
            z1_hu = d.ssumask[p] / (hup + T(1) - d.ssumask[p]);
            z1_hv = d.ssvmask[p] / (hvp + T(1) - d.ssvmask[p]);
          }
          T zu_trd, zv_trd;
          coriolis(d, cor_of(a, hm), a.nvor, (long)p, x, y, xu, yv, hq, z1_hu, z1_hv, zu_trd, zv_trd);
          // depth of the current level hu_e and its inverse hur_e (:689-693, :1159-1165)
          T hue = d.hu_0[p], hve = d.hv_0[p], hur = d.r1_hu_0[p], hvr = d.r1_hv_0[p];
          if constexpr (VVL) {
            if (jn == 1) {
              hue = (a.ln_bt_fw ? a.hu_n : a.hu_b)[hm + p];
              hve = (a.ln_bt_fw ? a.hv_n : a.hv_b)[hm + p];
              hur = (a.ln_bt_fw ? a.r1_hu_n : a.r1_hu_b)[hm + p];
              hvr = (a.ln_bt_fw ? a.r1_hv_n : a.r1_hv_b)[hm + p];
            } else {  // from ssha_e of sub-step jn-1 = the now ssh
              hue = d.hu_0[p] + ssh_u(p, vv_s[2][ty][tx], vv_s[2][ty][tx + 1]);
              hve = d.hv_0[p] + ssh_v(p, vv_s[2][ty][tx], vv_s[2][ty + 1][tx]);
              hur = d.ssumask[p] / (hue + T(1) - d.ssumask[p]);
              hvr = d.ssvmask[p] / (hve + T(1) - d.ssvmask[p]);
            }
          }
          zu_trd = zu_trd + zCdU_u[g] * un_e * hur;
          zv_trd = zv_trd + zCdU_v[g] * vn_e * hvr;
          const T s0 = zs_s[ty][tx];
          const T zu_spg = -grav * (zs_s[ty][tx + 1] - s0) * d.r1_e1u[p];
          const T zv_spg = -grav * (zs_s[ty + 1][tx] - s0) * d.r1_e2v[p];
          const T wxs = (T(1) - a.scal_load) * zu_spg;
          const T wys = (T(1) - a.scal_load) * zv_spg;
          if (!VVL || !a.flux) {  // vector form (:1106-1123)
            ua_e = (un_e + rdtbt * (wxs + zu_trd + zu_frc[g])) * d.ssumask[p];
            va_e = (vn_e + rdtbt * (wys + zv_trd + zv_frc[g])) * d.ssvmask[p];
          } else {  // flux form (:973-991, :1124-1147)
            const T zhust = d.hu_0[p] + ssh_u(p, s0, zs_s[ty][tx + 1]);
            const T zhvst = d.hv_0[p] + ssh_v(p, s0, zs_s[ty + 1][tx]);
            const T zhura = d.ssumask[p] / (hu_a + T(1) - d.ssumask[p]);
            const T zhvra = d.ssvmask[p] / (hv_a + T(1) - d.ssvmask[p]);
            ua_e = (hue * un_e + rdtbt * (zhust * wxs + hup * zu_trd + a.hu_n[hm + p] * zu_frc[g])) * zhura;
            va_e = (hve * vn_e + rdtbt * (zhvst * wys + hvp * zv_trd + a.hv_n[hm + p] * zv_frc[g])) * zhvra;
          }
        }
        a.ring_u[sa * nmem2 + g] = ua_e;
        a.ring_v[sa * nmem2 + g] = va_e;
        // velocities, or transports with the new depth in flux form (:1190-1201)
        const bool tr = VVL && a.flux;
        if constexpr (sizeof(T) == 8) {
          a.ua_b[g] = tr ? acc_u + w1 * (double)ua_e * (double)hu_a : acc_u + w1 * (double)ua_e;
          a.va_b[g] = tr ? acc_v + w1 * (double)va_e * (double)hv_a : acc_v + w1 * (double)va_e;
        } else {
          ff_add_w(f_u, w1h, w1l, tr ? ua_e * hu_a : ua_e);
          ff_add_w(f_v, w1h, w1l, tr ? va_e * hv_a : va_e);
          a.ff[ffi(1, 0, nmem2, g)] = f_u.h;
          a.ff[ffi(1, 1, nmem2, g)] = f_u.l;
          a.ff[ffi(2, 0, nmem2, g)] = f_v.h;
          a.ff[ffi(2, 1, nmem2, g)] = f_v.l;
        }
        if (jn < a.icycle) {
          // levels of sub-step jn+1: n = ua_e (new), b = un_e, bb = ub_e
          T za1, za2, za3;
          ab3(jn + 1, a.ll_init, za1, za2, za3);
          const T uex = za1 * ua_e + za2 * un_e + za3 * ub_e;
          const T vex = za1 * va_e + za2 * vn_e + za3 * vb_e;
          T hu = d.hu_0[p], hv = d.hv_0[p];
          if constexpr (VVL) {  // depth from the extrapolated ssh (:738-792)
            if (inner) {
              hu = hu + ssh_u(p, vv_s[1][ty][tx], vv_s[1][ty][tx + 1]);
              hv = hv + ssh_v(p, vv_s[1][ty][tx], vv_s[1][ty + 1][tx]);
            }
          }
          const T zwx = cache ? (T)C[12 * CS] * uex : d.e2u[p] * uex * hu;
          const T zwy = cache ? (T)C[13 * CS] * vex : d.e1v[p] * vex * hv;
          const T r1e2u = cache ? (T)C[14 * CS] : d.r1_e2u[p];
          const T r1e1v = cache ? (T)C[15 * CS] : d.r1_e1v[p];
          a.fx[((jn + 1) & 1) * nmem2 + g] = zwx;
          a.fy[((jn + 1) & 1) * nmem2 + g] = zwy;
          T w2;
          if constexpr (sizeof(T) == 8) w2 = a.wgt2[jn];
          else w2 = a.wgtf[2 * a.nwgt + jn];
          if constexpr (sizeof(T) == 8) {
            a.un_adv[g] = acc_au + (double)(w2 * zwx * d.r1_e2u[p]);
            a.vn_adv[g] = acc_av + (double)(w2 * zwy * d.r1_e1v[p]);
          } else {
            ff_add(f_au, w2 * zwx * r1e2u, 0.0f);
            ff_add(f_av, w2 * zwy * r1e1v, 0.0f);
            a.ff[ffi(3, 0, nmem2, g)] = f_au.h;
            a.ff[ffi(3, 1, nmem2, g)] = f_au.l;
            a.ff[ffi(4, 0, nmem2, g)] = f_av.h;
            a.ff[ffi(4, 1, nmem2, g)] = f_av.l;
          }
        }
      }
    }
    r = (r + 3) & 3;
    if (!grid_barrier(bar, bar_epoch)) return;
  }
  // ---- phase 3, per column (:1214-1262, :1266-1269): time-filtered transports
  // and the two depth-independent terms each level adds
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  // the time-averaged ssh at point g (final after the last barrier)
  auto ssha_at = [&](int gg) -> double {
    if constexpr (sizeof(T) == 4)
      return (double)a.ff[ffi(0, 0, nmem2, gg)] + (double)a.ff[ffi(0, 1, nmem2, gg)];
    else
      return a.ssha[gg];
  };
  for (int g = tid; g < nmem2; g += nth) {
    const int m2 = (g / n2) * n2, p = g - m2;
    const long hm = VVL ? m2 : 0;
    if constexpr (sizeof(T) == 4) {  // the compensated sums into the FP64 fields
      auto sum = [&](int w) { return (double)a.ff[ffi(w, 0, nmem2, g)] + (double)a.ff[ffi(w, 1, nmem2, g)]; };
      a.ssha[g] = sum(0);
      a.ua_b[g] = sum(1);
      a.va_b[g] = sum(2);
      a.un_adv[g] = sum(3);
      a.vn_adv[g] = sum(4);
    }
    double uadv = a.un_adv[g], vadv = a.vn_adv[g];
    if (a.ln_bt_fw) {
      const double zwx = uadv, zwy = vadv;
      if (a.phase3_filter) {
        uadv = 0.5 * (a.ub2_b[g] + zwx - a.rn_atfp * a.un_bf[g]);
        vadv = 0.5 * (a.vb2_b[g] + zwy - a.rn_atfp * a.vn_bf[g]);
        a.un_bf[g] = a.rn_atfp * a.un_bf[g] + (zwx - a.ub2_b[g]);
        a.vn_bf[g] = a.rn_atfp * a.vn_bf[g] + (zwy - a.vb2_b[g]);
      } else {
        a.un_bf[g] = 0.0;
        a.vn_bf[g] = 0.0;
      }
      a.ub2_b[g] = zwx;
      a.vb2_b[g] = zwy;
      a.un_adv[g] = uadv;
      a.vn_adv[g] = vadv;
    }
    double r1hu = (double)d.r1_hu_0[p], r1hv = (double)d.r1_hv_0[p];
    if constexpr (VVL) {
      r1hu = (double)a.r1_hu_n[hm + p];
      r1hv = (double)a.r1_hv_n[hm + p];
    }
    if (!VVL || !a.flux) {
      a.du[g] = (T)((a.ua_b[g] - (double)a.ub_b[g]) * a.r1_2dt_b);
      a.dv[g] = (T)((a.va_b[g] - (double)a.vb_b[g]) * a.r1_2dt_b);
    } else {  // flux form: summed transports to velocities (:1241-1262)
      a.du[g] = (T)(r1hu * (a.ua_b[g] - (double)a.ub_b[g] * (double)a.hu_b[hm + p]) * a.r1_2dt_b);
      a.dv[g] = (T)(r1hv * (a.va_b[g] - (double)a.vb_b[g] * (double)a.hv_b[hm + p]) * a.r1_2dt_b);
      const int i = p % jpi + 1, j = p / jpi + 1;
      double zsu = 0.0, zsv = 0.0;
      if (interior(i, j)) {
        const double s0 = ssha_at(g);
        zsu = 0.5 * (double)d.ssumask[p] * (double)d.r1_e1e2u[p] *
              ((double)d.e1e2t[p] * s0 + (double)d.e1e2t[p + 1] * ssha_at(g + 1));
        zsv = 0.5 * (double)d.ssvmask[p] * (double)d.r1_e1e2v[p] *
              ((double)d.e1e2t[p] * s0 + (double)d.e1e2t[p + jpi] * ssha_at(g + jpi));
      }
      a.ua_b[g] = a.ua_b[g] / ((double)d.hu_0[p] + zsu + 1.0 - (double)d.ssumask[p]);
      a.va_b[g] = a.va_b[g] / ((double)d.hv_0[p] + zsv + 1.0 - (double)d.ssvmask[p]);
    }
    a.cu[g] = (T)(uadv * r1hu);
    a.cv[g] = (T)(vadv * r1hv);
  }
}

// ---------------------------------------------------------------------------------
// The sub-steps of the mixed form for a linear free surface with the ENE or MIX
// vorticity scheme (GYRE's configuration), specialised for a short critical path:
// the sub-step time is set by the slowest block, i.e. by the tiles a block owns, so
// this kernel keeps to <= 48 registers for 5 co-resident blocks per SM and owns at
// most P2H_MAXT = 2 tiles a block (GYRE nn_GYRE=25: 1512 tiles on 760 blocks),
// where the general kernel runs 4 blocks per SM with up to 3 tiles. Per point it
// keeps in shared memory the constants of both stages (those of k_spg_p2's cache,
// plus rdtbt * zssh_frc and rdtbt / e1e2t of the new ssh), and it packs the five
// compensated sums of a point into three float4 (one 16-byte access each instead
// of ten 4-byte ones). Same steps as k_spg_p2 (:712-1207): the east/north halo of
// the new ssh recomputed by each block, one grid barrier per sub-step.
constexpr int P2H_MAXT = 2;
constexpr int P2H_NC = 18;
constexpr size_t P2H_CACHE_BYTES = (size_t)P2H_NC * P2H_MAXT * 256 * sizeof(float);

// the packed sums: plane 0 = {ssha hi, lo, ua_b hi, lo}, 1 = {va_b hi, lo, un_adv hi,
// lo}, 2 = {vn_adv hi, lo, 0, 0}; plane q of point g at ff4[q * nmem2 + g]
__device__ __forceinline__ void ff4_add_w(float& h, float& l, float wh, float wl, float x) {
  FF s{h, l};
  ff_add_w(s, wh, wl, x);
  h = s.h;
  l = s.l;
}

template <class T>
__global__ void __launch_bounds__(256, 5) k_spg_p2_ene(Dom<T> d, SpgArgs<T> a, GridBar bar) {
  unsigned int bar_epoch = 0;  // barriers passed by this block
  static_assert(sizeof(T) == 4, "the mixed form's kernel");
  __shared__ float zs_s[P2_TY + 1][P2_TX + 1];
  extern __shared__ float p2h[];
  const int n2 = (int)d.n2, nmem2 = d.nmem * n2, jpi = d.jpi, jpj = d.jpj;
  const int ntx = (jpi + P2_TX - 1) / P2_TX, nty = (jpj + P2_TY - 1) / P2_TY;
  const int ntile = ntx * nty * d.nmem;
  const int tx = threadIdx.x % P2_TX, ty = threadIdx.x / P2_TX;
  const float rdtbt = a.rdtbt;
  float4* const ff4 = reinterpret_cast<float4*>(a.ff);
  constexpr int CS = P2H_MAXT * 256;  // stride of one constant in the cache
  auto interior = [&](int i, int j) -> bool { return i >= 2 && i <= jpi - 1 && j >= 2 && j <= jpj - 1; };
  auto tile = [&](int t, int& m2, int& i0, int& j0) {
    const int m = t / (ntx * nty), tt = t - m * (ntx * nty);
    m2 = m * n2;
    i0 = (tt % ntx) * P2_TX + 1;
    j0 = (tt / ntx) * P2_TY + 1;
  };
  int r = a.ring0;
  // ---- the constants of the owned points, the predictor of sub-step 1 (:724-800)
  // and the sums started with its un_adv / vn_adv terms (:860-862)
  {
    float za1, za2, za3;
    ab3(1, a.ll_init, za1, za2, za3);
    const int sn = r & 3, sb = (r + 1) & 3, sbb = (r + 2) & 3;
    const float w2 = a.wgtf[2 * a.nwgt];
    int slot = 0;
    for (int t = blockIdx.x; t < ntile && slot < P2H_MAXT; t += gridDim.x, ++slot) {
      int m2, i0, j0;
      tile(t, m2, i0, j0);
      const int i = i0 + tx, j = j0 + ty;
      float cv[P2H_NC] = {};
      if (i <= jpi && j <= jpj) {
        const int p = (i - 1) + (j - 1) * jpi, g = m2 + p;
        if (interior(i, j)) {
          const float su = (1.0f - a.scal_load) * (-a.grav);
          cv[0] = 0.25f * d.zwz[p - jpi] * d.r1_e1u[p];
          cv[1] = 0.25f * d.zwz[p] * d.r1_e1u[p];
          cv[2] = -0.25f * d.zwz[p - 1] * d.r1_e2v[p];
          cv[3] = -0.25f * d.zwz[p] * d.r1_e2v[p];
          cv[4] = a.zCdU_u[g] * d.r1_hu_0[p];
          cv[5] = a.zCdU_v[g] * d.r1_hv_0[p];
          cv[6] = su * d.r1_e1u[p];
          cv[7] = su * d.r1_e2v[p];
          cv[8] = a.zu_frc[g];
          cv[9] = a.zv_frc[g];
          cv[10] = d.ssumask[p];
          cv[11] = d.ssvmask[p];
          cv[16] = __fmul_rn(rdtbt, a.zssh_frc[g]);
          cv[17] = __fmul_rn(rdtbt, d.r1_e1e2t[p]);
        }
        cv[12] = d.e2u[p] * d.hu_0[p];
        cv[13] = d.e1v[p] * d.hv_0[p];
        cv[14] = d.r1_e2u[p];
        cv[15] = d.r1_e1v[p];
        const float ua_e = za1 * a.ring_u[sn * nmem2 + g] + za2 * a.ring_u[sb * nmem2 + g] +
                           za3 * a.ring_u[sbb * nmem2 + g];
        const float va_e = za1 * a.ring_v[sn * nmem2 + g] + za2 * a.ring_v[sb * nmem2 + g] +
                           za3 * a.ring_v[sbb * nmem2 + g];
        const float zwx = d.e2u[p] * ua_e * d.hu_0[p];
        const float zwy = d.e1v[p] * va_e * d.hv_0[p];
        a.fx[nmem2 + g] = zwx;  // slot (1 & 1)
        a.fy[nmem2 + g] = zwy;
        ff4[g] = make_float4(0.f, 0.f, 0.f, 0.f);
        ff4[nmem2 + g] = make_float4(0.f, 0.f, w2 * zwx * d.r1_e2u[p], 0.f);
        ff4[2 * nmem2 + g] = make_float4(w2 * zwy * d.r1_e1v[p], 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int cc = 0; cc < P2H_NC; ++cc) p2h[cc * CS + slot * 256 + threadIdx.x] = cv[cc];
    }
  }
  // the halo position of this thread, if any: the east column (9) and the north row
  // (32) of the tile
  int hti = -1, htj = -1;
  if (threadIdx.x < P2_TY + 1) { hti = P2_TX; htj = threadIdx.x; }
  else if (threadIdx.x < P2_TY + 1 + P2_TX) { hti = threadIdx.x - (P2_TY + 1); htj = P2_TY; }
  if (!grid_barrier(bar, bar_epoch)) return;
  for (int jn = 1; jn <= a.icycle; ++jn) {
    const int sn = r & 3, sb = (r + 1) & 3, sbb = (r + 2) & 3, sa = (r + 3) & 3;
    const float* fx = a.fx + (jn & 1) * nmem2;
    const float* fy = a.fy + (jn & 1) * nmem2;
    const float w1h = a.wgtf[jn - 1], w1l = a.wgtf[a.nwgt + jn - 1];
    float zb0, zb1, zb2, zb3;
    am4(jn, a.ll_init, a.rn_bt_alpha, zb0, zb1, zb2, zb3);
    int slot = 0;
    for (int t = blockIdx.x; t < ntile; t += gridDim.x, ++slot) {
      int m2, i0, j0;
      tile(t, m2, i0, j0);
      const int i = i0 + tx, j = j0 + ty;
      const bool own = i <= jpi && j <= jpj;
      const bool inner = own && interior(i, j);
      const int p = own ? (i - 1) + (j - 1) * jpi : 0, g = m2 + p;
      const float* C = p2h + slot * 256 + threadIdx.x;
      // the values of both stages first, so that their loads are in flight together;
      // those of the sums and the predictor's before levels at the start of stage B
      // (fewer registers live across the block barrier)
      float x[4] = {}, y[4] = {};
      float sn0 = 0.f, sb0 = 0.f, sbb0 = 0.f, un_e = 0.f, vn_e = 0.f;
      float4 f0 = {};
      if (own) {
        sn0 = a.ring_ssh[sn * nmem2 + g];
        sb0 = a.ring_ssh[sb * nmem2 + g];
        sbb0 = a.ring_ssh[sbb * nmem2 + g];
        un_e = a.ring_u[sn * nmem2 + g];
        vn_e = a.ring_v[sn * nmem2 + g];
        f0 = ff4[g];
        if (inner) {
          nbx([&](long q) { return fx[m2 + q]; }, (long)p, jpi, x);
          nby([&](long q) { return fy[m2 + q]; }, (long)p, jpi, y);
        }
      }
      const int hi_ = i0 + hti, hj_ = j0 + htj;
      const bool halo = hti >= 0 && hi_ <= jpi && hj_ <= jpj;
      // ---- ssha_e (:871-879) and zsshp2_e (:930-931) of the owned point and the halo
      // the owner of a point and the blocks whose halo it is form its values with the
      // same rounded operations (explicit intrinsics: no contraction choices)
      auto ssha_of = [&](float s0, float frc, float div, float dv, float msk) {
        return __fmul_rn(__fsub_rn(s0, __fmaf_rn(div, dv, frc)), msk);
      };
      auto zs_of = [&](float e, float s0, float s1, float s2) {
        return __fmaf_rn(zb3, s2, __fmaf_rn(zb2, s1, __fmaf_rn(zb1, s0, __fmul_rn(zb0, e))));
      };
      if (own) {
        float ssha_e = 0.f;
        if (inner) {
          const float dv = __fsub_rn(__fadd_rn(__fsub_rn(x[1], x[0]), y[2]), y[0]);
          ssha_e = ssha_of(sn0, C[16 * CS], C[17 * CS], dv, d.ssmask[p]);
        }
        zs_s[ty][tx] = zs_of(ssha_e, sn0, sb0, sbb0);
        a.ring_ssh[sa * nmem2 + g] = ssha_e;
        ff4_add_w(f0.x, f0.y, w1h, w1l, ssha_e);
      }
      if (halo) {
        const int hp = (hi_ - 1) + (hj_ - 1) * jpi, hg = m2 + hp;
        const float h_sn = a.ring_ssh[sn * nmem2 + hg];
        float ssha_e = 0.f;
        if (interior(hi_, hj_)) {
          const float dv = __fsub_rn(__fadd_rn(__fsub_rn(fx[hg], fx[hg - 1]), fy[hg]), fy[hg - jpi]);
          ssha_e = ssha_of(h_sn, __fmul_rn(rdtbt, a.zssh_frc[hg]), __fmul_rn(rdtbt, d.r1_e1e2t[hp]), dv,
                           d.ssmask[hp]);
        }
        zs_s[htj][hti] = zs_of(ssha_e, h_sn, a.ring_ssh[sb * nmem2 + hg], a.ring_ssh[sbb * nmem2 + hg]);
      }
      __syncthreads();
      // ---- Coriolis, drag, pressure gradient, ua_e / va_e and their sums
      // (:1000-1204), the predictor of sub-step jn+1 (:724-800) and its sums (:860-862)
      if (own) {
        float4 f1 = ff4[nmem2 + g];
        const float ub_e = a.ring_u[sb * nmem2 + g], vb_e = a.ring_v[sb * nmem2 + g];
        float ua_e = 0.f, va_e = 0.f;
        if (inner) {
          const float s0 = zs_s[ty][tx];
          const float zu_trd = C[0] * (y[0] + y[1]) + C[CS] * (y[2] + y[3]) + C[4 * CS] * un_e;
          const float zv_trd = C[2 * CS] * (x[0] + x[2]) + C[3 * CS] * (x[1] + x[3]) + C[5 * CS] * vn_e;
          const float wxs = C[6 * CS] * (zs_s[ty][tx + 1] - s0);
          const float wys = C[7 * CS] * (zs_s[ty + 1][tx] - s0);
          ua_e = (un_e + rdtbt * (wxs + zu_trd + C[8 * CS])) * C[10 * CS];
          va_e = (vn_e + rdtbt * (wys + zv_trd + C[9 * CS])) * C[11 * CS];
        }
        a.ring_u[sa * nmem2 + g] = ua_e;
        a.ring_v[sa * nmem2 + g] = va_e;
        ff4_add_w(f0.z, f0.w, w1h, w1l, ua_e);
        ff4_add_w(f1.x, f1.y, w1h, w1l, va_e);
        ff4[g] = f0;
        if (jn < a.icycle) {
          float2 f2 = reinterpret_cast<float2*>(ff4 + 2 * nmem2)[2 * g];
          float za1, za2, za3;
          ab3(jn + 1, a.ll_init, za1, za2, za3);
          const float uex = za1 * ua_e + za2 * un_e + za3 * ub_e;
          const float vex = za1 * va_e + za2 * vn_e + za3 * vb_e;
          const float zwx = C[12 * CS] * uex;
          const float zwy = C[13 * CS] * vex;
          a.fx[((jn + 1) & 1) * nmem2 + g] = zwx;
          a.fy[((jn + 1) & 1) * nmem2 + g] = zwy;
          const float w2 = a.wgtf[2 * a.nwgt + jn];
          FF s{f1.z, f1.w};
          ff_add(s, w2 * zwx * C[14 * CS], 0.0f);
          f1.z = s.h;
          f1.w = s.l;
          s = FF{f2.x, f2.y};
          ff_add(s, w2 * zwy * C[15 * CS], 0.0f);
          f2.x = s.h;
          f2.y = s.l;
          reinterpret_cast<float2*>(ff4 + 2 * nmem2)[2 * g] = f2;
        }
        ff4[nmem2 + g] = f1;
      }
      __syncthreads();  // zs_s is rewritten by the next tile
    }
    r = (r + 3) & 3;
    if (!grid_barrier(bar, bar_epoch)) return;
  }
  // ---- phase 3, per column (:1214-1240, :1266-1269): the sums into the FP64 fields,
  // the time-filtered transports and the two depth-independent terms of each level
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  for (int g = tid; g < nmem2; g += nth) {
    const int p = g % n2;
    const float4 f0 = ff4[g], f1 = ff4[nmem2 + g], f2 = ff4[2 * nmem2 + g];
    a.ssha[g] = (double)f0.x + (double)f0.y;
    const double uab = (double)f0.z + (double)f0.w, vab = (double)f1.x + (double)f1.y;
    a.ua_b[g] = uab;
    a.va_b[g] = vab;
    double uadv = (double)f1.z + (double)f1.w, vadv = (double)f2.x + (double)f2.y;
    if (a.ln_bt_fw) {
      const double zwx = uadv, zwy = vadv;
      if (a.phase3_filter) {
        uadv = 0.5 * (a.ub2_b[g] + zwx - a.rn_atfp * a.un_bf[g]);
        vadv = 0.5 * (a.vb2_b[g] + zwy - a.rn_atfp * a.vn_bf[g]);
        a.un_bf[g] = a.rn_atfp * a.un_bf[g] + (zwx - a.ub2_b[g]);
        a.vn_bf[g] = a.rn_atfp * a.vn_bf[g] + (zwy - a.vb2_b[g]);
      } else {
        a.un_bf[g] = 0.0;
        a.vn_bf[g] = 0.0;
      }
      a.ub2_b[g] = zwx;
      a.vb2_b[g] = zwy;
    }
    a.un_adv[g] = uadv;
    a.vn_adv[g] = vadv;
    a.du[g] = (float)((uab - (double)a.ub_b[g]) * a.r1_2dt_b);
    a.dv[g] = (float)((vab - (double)a.vb_b[g]) * a.r1_2dt_b);
    a.cu[g] = (float)(uadv * (double)d.r1_hu_0[p]);
    a.cv[g] = (float)(vadv * (double)d.r1_hv_0[p]);
  }
}

// Phase 3 (:1236-1240, :1266-1269), with phase 1's removal of the column mean from
// ua, va on the interior (:371-378): the barotropic trend added to ua, va and the now
// velocities corrected to the time-filtered transports; one thread walks a chunk of
// levels of one column, the column terms loaded once.
template <class T>
__global__ void __launch_bounds__(128) k_spg_p3(Dom<T> d, SpgArgs<T> a) {
  const int nch = (d.jpk + KCH3 - 1) / KCH3;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int m = (int)(blockIdx.z / (unsigned)nch);
  const int k0 = ((int)blockIdx.z - m * nch) * KCH3 + 1;
  if (i > d.jpi || j > d.jpj) return;
  const int k1 = k0 + KCH3 - 1 < d.jpk - 1 ? k0 + KCH3 - 1 : d.jpk - 1;
  const long p = pt_ij(d, i, j), m2 = (long)m * d.n2;
  const ColInfo ci = d.ci[p];
  const RO<T> du = a.du, dv = a.dv, cu = a.cu, cv = a.cv;  // written by phase 2
  const T du0 = du[m2 + p], dv0 = dv[m2 + p], cu0 = cu[m2 + p], cv0 = cv[m2 + p];
  const T unb = a.un_b[m2 + p], vnb = a.vn_b[m2 + p];
  const bool interior = i >= 2 && i <= d.jpi - 1 && j >= 2 && j <= d.jpj - 1;
  const T zm_u = interior ? a.zmu[m2 + p] : T(0), zm_v = interior ? a.zmv[m2 + p] : T(0);
  const long base = (long)m * d.n3 + p;
  // all levels of the chunk loaded before the first store (the stores may alias the
  // loads for the compiler, which would otherwise keep one level in flight)
  T lua[KCH3], lva[KCH3], lun[KCH3], lvn[KCH3];
#pragma unroll
  for (int kk = 0; kk < KCH3; ++kk) {
    if (k0 + kk > k1) break;
    const long q = base + (long)(k0 + kk - 1) * d.n2;
    lua[kk] = a.ua[q];
    lva[kk] = a.va[q];
    lun[kk] = a.un[q];
    lvn[kk] = a.vn[q];
  }
#pragma unroll
  for (int kk = 0; kk < KCH3; ++kk) {
    const int k = k0 + kk;
    if (k > k1) break;
    const long q = base + (long)(k - 1) * d.n2;
    T ua = lua[kk], va = lva[kk];
    const T un = lun[kk], vn = lvn[kk];
    if (interior) {
      ua = ua - zm_u * umsk<T>(ci, k);
      va = va - zm_v * vmsk<T>(ci, k);
    }
    a.ua[q] = ua + du0;
    a.va[q] = va + dv0;
    a.un[q] = (un + cu0 - unb) * umsk<T>(ci, k);
    a.vn[q] = (vn + cv0 - vnb) * vmsk<T>(ci, k);
  }
}

// ---------------------------------------------------------------------------------
// lbc_lnk closed branch (lbc_lnk_generic.h90:88-101) on nslab (i,j) slices: columns
// 1 and jpi, rows 1 and jpj take pval; F-point arrays keep column and row 1.
template <class T>
__global__ void k_lbc_closed(T* p, int jpi, int jpj, long nslab, int is_f, T pval) {
  const long per = 2L * jpi + 2L * jpj;
  const long s = blockIdx.y;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < per; e += (long)gridDim.x * blockDim.x) {
    for (long sl = s; sl < nslab; sl += gridDim.y) {
      T* a = p + sl * (long)jpi * jpj;
      long i, j;
      bool first;  // on column 1 or row 1
      if (e < jpj) { i = 1; j = e + 1; first = true; }
      else if (e < 2L * jpj) { i = jpi; j = e - jpj + 1; first = false; }
      else if (e < 2L * jpj + jpi) { i = e - 2L * jpj + 1; j = 1; first = true; }
      else { i = e - 2L * jpj - jpi + 1; j = jpj; first = false; }
      if (first && is_f) continue;
      a[(i - 1) + (j - 1) * (long)jpi] = pval;
    }
  }
}

// ---------------------------------------------------------------------------------
// glob_sum (lib_fortran_generic.h90:32-65): sum of x*tmask_i in double-double
// arithmetic (the compensated pair (sum, err) of DDPDD, lib_fortran.F90:300-332),
// combined across threads with the same two-sum, one result per member.
__device__ __forceinline__ void dd_add(double& hi, double& lo, double a_hi, double a_lo) {
  const double zt1 = a_hi + hi;
  const double zerr = zt1 - a_hi;
  const double zt2 = ((hi - zerr) + (a_hi - (zt1 - zerr))) + a_lo + lo;
  hi = zt1 + zt2;
  lo = zt2 - ((zt1 + zt2) - zt1);
}

template <class T>
__global__ void k_globsum_partial(const T* __restrict__ x, const double* __restrict__ tmask_i, long n2, int nk,
                                  double* __restrict__ part) {
  const int m = blockIdx.y;
  const long n = n2 * nk;
  const T* xm = x + (long)m * n;
  double hi = 0.0, lo = 0.0;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    dd_add(hi, lo, (double)xm[e] * tmask_i[e % n2], 0.0);
  __shared__ double sh[2][256];
  sh[0][threadIdx.x] = hi;
  sh[1][threadIdx.x] = lo;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      double h = sh[0][threadIdx.x], l = sh[1][threadIdx.x];
      dd_add(h, l, sh[0][threadIdx.x + s], sh[1][threadIdx.x + s]);
      sh[0][threadIdx.x] = h;
      sh[1][threadIdx.x] = l;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * ((long)m * gridDim.x + blockIdx.x)] = sh[0][0];
    part[2 * ((long)m * gridDim.x + blockIdx.x) + 1] = sh[1][0];
  }
}

static __global__ void k_globsum_final(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  const int m = blockIdx.x;
  double hi = 0.0, lo = 0.0;
  __shared__ double sh[2][256];
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) dd_add(hi, lo, part[2 * ((long)m * nblk + b)], part[2 * ((long)m * nblk + b) + 1]);
  sh[0][threadIdx.x] = hi;
  sh[1][threadIdx.x] = lo;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      double h = sh[0][threadIdx.x], l = sh[1][threadIdx.x];
      dd_add(h, l, sh[0][threadIdx.x + s], sh[1][threadIdx.x + s]);
      sh[0][threadIdx.x] = h;
      sh[1][threadIdx.x] = l;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[m] = sh[0][0];
}

}  // namespace nemo
