// k_spg_adj.cuh -- the adjoint of dyn_spg_ts (dynspg_ts.F90:121-1310) for the linear
// free surface with ln_bt_fw and ln_bt_av, FP64.
//
// The forward is affine in the state; its adjoint runs phase 3, the barotropic
// sub-steps from the last to the first, then phase 1. Each reverse sub-step is three
// point kernels (one (i,j) per thread) in gather form: a thread forms the adjoint of
// its own point from its neighbours' values of the previous kernel, so no two
// threads write one element and no atomics are needed; a launch boundary separates
// a value from its neighbours' reads, so nothing waits inside a kernel.
//   S1 -- the adjoint of the new velocity (the sums of ua_b, the swap, the lbc):
//         gu = rdtbt ssumask ua_e_ad, the forcing adjoint Fu += gu;
//   S2 -- the ssh: the pressure-gradient adjoint gathered from the neighbouring gu,
//         the AM4 ssh, the ssh update (lbc, ssmask), the divergence adjoint zhd;
//   S3 -- the fluxes: the un_adv sums, the divergence (from the neighbouring zhd) and
//         the Coriolis trend (from the neighbouring gu) transposed, then the AB3
//         extrapolation and the new carried adjoints of un_e, ub_e, ubb_e.
#pragma once
#include "../../include/nemo_gpu.h"
#include "adj.h"

namespace nemo {

__device__ __forceinline__ bool spg_in(const Dom<double>& d, int i, int j) {
  return i >= 2 && i <= d.jpi - 1 && j >= 2 && j <= d.jpj - 1;
}
// Coriolis weights (the oracle's restatement of :387-443, :1000-1056): zu_trd(p) =
// sum_t cu(t,p) zwy(p + du_t), du = (0,-1), (1,-1), (0,0), (1,0); zv_trd(p) =
// sum_t cv(t,p) zwx(p + dv_t), dv = (-1,0), (-1,1), (0,0), (0,1)
__device__ __forceinline__ double spg_cu(const Dom<double>& d, int sc, int t, long p) {
  const long nb = d.jpi;
  if (sc == NEMO_VOR_ENS) return 0.125 * d.r1_e1u[p] * (d.zwz[p - nb] + d.zwz[p]);
  if (sc == NEMO_VOR_EEN) {
    const double f = t == 0 ? d.ftse[p] : t == 1 ? d.ftsw[p + 1] : t == 2 ? d.ftne[p] : d.ftnw[p + 1];
    return (1.0 / 12.0) * d.r1_e1u[p] * f;
  }
  return 0.25 * (t < 2 ? d.zwz[p - nb] : d.zwz[p]) * d.r1_e1u[p];
}
__device__ __forceinline__ double spg_cv(const Dom<double>& d, int sc, int t, long p) {
  const long nb = d.jpi;
  if (sc == NEMO_VOR_ENS) return -0.125 * d.r1_e2v[p] * (d.zwz[p - 1] + d.zwz[p]);
  if (sc == NEMO_VOR_EEN) {
    const double f = t == 0 ? d.ftnw[p] : t == 1 ? d.ftsw[p + nb] : t == 2 ? d.ftne[p] : d.ftse[p + nb];
    return -(1.0 / 12.0) * d.r1_e2v[p] * f;
  }
  return -0.25 * (t < 2 ? d.zwz[p - 1] : d.zwz[p]) * d.r1_e2v[p];
}
// the flux adjoints at point (i,j) from the trend adjoints gu, gv (member offset o)
// of the interior points whose trends read that flux
__device__ __forceinline__ void spg_cor_gather(const Dom<double>& d, int sc, const double* gu, const double* gv,
                                               long o, int i, int j, double& xa, double& ya) {
  const long nb = d.jpi, q = (long)(i - 1) + (long)(j - 1) * nb;
  // zwya(q): trends at q - du_t
  const int pui[4] = {0, -1, 0, -1}, puj[4] = {1, 1, 0, 0};
  const int pvi[4] = {1, 1, 0, 0}, pvj[4] = {0, -1, 0, -1};
  for (int t = 0; t < 4; ++t) {
    const int ii = i + pui[t], jj = j + puj[t];
    if (spg_in(d, ii, jj)) {
      const long p = q + pui[t] + puj[t] * nb;
      ya += spg_cu(d, sc, t, p) * gu[o + p];
    }
    const int vi = i + pvi[t], vj = j + pvj[t];
    if (spg_in(d, vi, vj)) {
      const long p = q + pvi[t] + pvj[t] * nb;
      xa += spg_cv(d, sc, t, p) * gv[o + p];
    }
  }
}

// phase 3 (:1214-1269) per column: the un and ua updates and the restart fields
__global__ void k_spg_adj_p3(Dom<double> d, SpgAdjArgs a) {
  const ColIdx<double> c = col_index(d);
  if (!c.valid) return;
  const long p = (long)c.m * d.n2 + c.ij, o = (long)c.m * d.n3 + c.ij;
  const ColInfo ci = d.ci[c.ij];
  double su = 0.0, sv = 0.0, ta = 0.0, tb = 0.0;
  for (int k = 1; k <= d.jpk - 1; ++k) {
    const long q = o + (long)(k - 1) * d.n2;
    const double um = umsk<double>(ci, k), vm = vmsk<double>(ci, k);
    su += a.un[q] * um; sv += a.vn[q] * vm;
    ta += a.ua[q]; tb += a.va[q];
    a.un[q] = a.un[q] * um; a.vn[q] = a.vn[q] * vm;
  }
  const double adu = a.un_adv[p] + su * d.r1_hu_0[c.ij], adv = a.vn_adv[p] + sv * d.r1_hv_0[c.ij];
  a.un_b[p] -= su; a.vn_b[p] -= sv;
  a.uab[p] = a.ua_b[p] + ta * a.r1_2dt_b; a.vab[p] = a.va_b[p] + tb * a.r1_2dt_b;
  a.ub_b[p] -= ta * a.r1_2dt_b; a.vb_b[p] -= tb * a.r1_2dt_b;
  if (!a.euler) {
    a.X[p] = 0.5 * adu + a.un_bf[p] + a.ub2_b[p];
    a.Y[p] = 0.5 * adv + a.vn_bf[p] + a.vb2_b[p];
    const double u2 = 0.5 * adu - a.un_bf[p], v2 = 0.5 * adv - a.vn_bf[p];
    a.un_bf[p] = -0.5 * a.atfp * adu + a.atfp * a.un_bf[p];
    a.vn_bf[p] = -0.5 * a.atfp * adv + a.atfp * a.vn_bf[p];
    a.ub2_b[p] = u2; a.vb2_b[p] = v2;
  } else {
    a.X[p] = adu + a.ub2_b[p]; a.Y[p] = adv + a.vb2_b[p];
    a.ub2_b[p] = 0.0; a.vb2_b[p] = 0.0; a.un_bf[p] = 0.0; a.vn_bf[p] = 0.0;
  }
  a.Au[p] = 0.0; a.Aub[p] = 0.0; a.Aubb[p] = 0.0; a.Av[p] = 0.0; a.Avb[p] = 0.0; a.Avbb[p] = 0.0;
  a.Sn[p] = 0.0; a.Sb[p] = 0.0; a.Sbb[p] = 0.0; a.Fu[p] = 0.0; a.Fv[p] = 0.0;
}

// the adjoint of the new velocity ua_e before the lbc (:1167-1204), on the interior
__device__ __forceinline__ double spg_uae(const Dom<double>& d, const SpgAdjArgs& a, const SpgAdjStep& s, long p,
                                          int i, int j, bool u) {
  if (!spg_in(d, i, j)) return 0.0;
  return u ? a.Au[p] + s.w1 * a.uab[p] : a.Av[p] + s.w1 * a.vab[p];
}

__global__ void k_spg_adj_s1(Dom<double> d, SpgAdjArgs a, SpgAdjStep s) {
  const ColIdx<double> c = col_index(d);
  if (!c.valid) return;
  const long p = (long)c.m * d.n2 + c.ij;
  double gu = 0.0, gv = 0.0;
  if (c.interior) {
    gu = a.rdtbt * (spg_uae(d, a, s, p, c.i, c.j, true) * d.ssumask[c.ij]);
    gv = a.rdtbt * (spg_uae(d, a, s, p, c.i, c.j, false) * d.ssvmask[c.ij]);
    a.Fu[p] += gu;
    a.Fv[p] += gv;
  }
  a.gu[p] = gu;
  a.gv[p] = gv;
}

__global__ void k_spg_adj_s2(Dom<double> d, SpgAdjArgs a, SpgAdjStep s) {
  const ColIdx<double> c = col_index(d);
  if (!c.valid) return;
  const long o = (long)c.m * d.n2, p = o + c.ij, nb = d.jpi;
  const double kg = (1.0 - a.sl) * (-a.grav);
  // the pressure-gradient adjoint (:1093-1101): zsshp2(i+1) - zsshp2(i) of the faces
  double zsp = 0.0;
  if (spg_in(d, c.i - 1, c.j)) zsp += kg * d.r1_e1u[c.ij - 1] * a.gu[p - 1];
  if (c.interior) zsp -= kg * d.r1_e1u[c.ij] * a.gu[p];
  if (spg_in(d, c.i, c.j - 1)) zsp += kg * d.r1_e2v[c.ij - nb] * a.gv[p - nb];
  if (c.interior) zsp -= kg * d.r1_e2v[c.ij] * a.gv[p];
  double sae = a.Sn[p] + s.w1 * a.ssha[p] + s.za0 * zsp;
  if (!c.interior) sae = 0.0;  // lbc of ssha_e (:879)
  const double t = sae * d.ssmask[c.ij];
  a.zhd[p] = -a.rdtbt * t;
  const double nsn = a.Sb[p] + s.za1 * zsp + t, nsb = a.Sbb[p] + s.za2 * zsp, nsbb = s.za3 * zsp;
  a.Sn[p] = nsn; a.Sb[p] = nsb; a.Sbb[p] = nsbb;
}

__global__ void k_spg_adj_s3(Dom<double> d, SpgAdjArgs a, SpgAdjStep s) {
  const ColIdx<double> c = col_index(d);
  if (!c.valid) return;
  const long o = (long)c.m * d.n2, p = o + c.ij, nb = d.jpi;
  double xa = 0.0, ya = 0.0;
  spg_cor_gather(d, a.sc, a.gu, a.gv, o, c.i, c.j, xa, ya);
  // the divergence (:866-869) of the interior points p and p + 1 (p + jpi)
  if (c.interior) {
    const double t = a.zhd[p] * d.r1_e1e2t[c.ij];
    xa += t; ya += t;
  }
  if (spg_in(d, c.i + 1, c.j)) xa -= a.zhd[p + 1] * d.r1_e1e2t[c.ij + 1];
  if (spg_in(d, c.i, c.j + 1)) ya -= a.zhd[p + nb] * d.r1_e1e2t[c.ij + nb];
  // the un_adv sums (:860-862) and the fluxes (:799-800)
  xa += s.w2 * a.X[p] * d.r1_e2u[c.ij];
  ya += s.w2 * a.Y[p] * d.r1_e1v[c.ij];
  const double eu = xa * d.e2u[c.ij] * d.hu_0[c.ij], ev = ya * d.e1v[c.ij] * d.hv_0[c.ij];
  // the next velocity's dependence on un_e (:1106-1122) and the bottom stress (:1072-1079)
  double tu = 0.0, tv = 0.0;
  if (c.interior) {
    const double gu = a.gu[p], gv = a.gv[p];
    tu = spg_uae(d, a, s, p, c.i, c.j, true) * d.ssumask[c.ij] +
         0.5 * (a.rcdu[p + 1] + a.rcdu[p]) * d.r1_hu_0[c.ij] * gu;
    tv = spg_uae(d, a, s, p, c.i, c.j, false) * d.ssvmask[c.ij] +
         0.5 * (a.rcdu[p + nb] + a.rcdu[p]) * d.r1_hv_0[c.ij] * gv;
  }
  const double nu = a.Aub[p] + tu + s.zb1 * eu, nub = a.Aubb[p] + s.zb2 * eu, nubb = s.zb3 * eu;
  const double nv = a.Avb[p] + tv + s.zb1 * ev, nvb = a.Avbb[p] + s.zb2 * ev, nvbb = s.zb3 * ev;
  a.Au[p] = nu; a.Aub[p] = nub; a.Aubb[p] = nubb;
  a.Av[p] = nv; a.Avb[p] = nvb; a.Avbb[p] = nvbb;
}

// phase 1 (:358-557) per column, after the start of the sub-steps (:688-693)
__global__ void k_spg_adj_p1(Dom<double> d, SpgAdjArgs a) {
  const ColIdx<double> c = col_index(d);
  if (!c.valid) return;
  const long o2 = (long)c.m * d.n2, p = o2 + c.ij, o3 = (long)c.m * d.n3 + c.ij, nb = d.jpi;
  const ColInfo ci = d.ci[c.ij];
  double ub = a.un_b[p] + a.Au[p], vb = a.vn_b[p] + a.Av[p];
  a.sshn[p] += a.Sn[p];
  // the Coriolis trend of un_b, vn_b removed from the forcing (:387-443, :511-516):
  // the trend adjoints -Fu ssumask of the neighbouring interior points
  {
    double xa = 0.0, ya = 0.0;
    const int pui[4] = {0, -1, 0, -1}, puj[4] = {1, 1, 0, 0};
    const int pvi[4] = {1, 1, 0, 0}, pvj[4] = {0, -1, 0, -1};
    for (int t = 0; t < 4; ++t) {
      if (spg_in(d, c.i + pui[t], c.j + puj[t])) {
        const long q = c.ij + pui[t] + puj[t] * nb;
        ya += spg_cu(d, a.sc, t, q) * (-a.Fu[o2 + q] * d.ssumask[q]);
      }
      if (spg_in(d, c.i + pvi[t], c.j + pvj[t])) {
        const long q = c.ij + pvi[t] + pvj[t] * nb;
        xa += spg_cv(d, a.sc, t, q) * (-a.Fv[o2 + q] * d.ssvmask[q]);
      }
    }
    ub += xa * d.hu_0[c.ij] * d.e2u[c.ij];
    vb += ya * d.hv_0[c.ij] * d.e1v[c.ij];
  }
  if (c.interior) {
    // the bottom stress of the baroclinic velocities (:519-557)
    const double fu = a.Fu[p], fv = a.Fv[p];
    const double tu = d.r1_hu_0[c.ij] * 0.5 * (a.rcdu[p + 1] + a.rcdu[p]) * fu;
    const double tv = d.r1_hv_0[c.ij] * 0.5 * (a.rcdu[p + nb] + a.rcdu[p]) * fv;
    a.un[o3 + (long)(ci.mbku - 1) * d.n2] += tu;
    a.vn[o3 + (long)(ci.mbkv - 1) * d.n2] += tv;
    ub -= tu; vb -= tv;
    // the vertical mean of the baroclinic trend (:358-378)
    double su = fu, sv = fv;
    for (int k = 1; k <= d.jpk - 1; ++k) {
      const long q = o3 + (long)(k - 1) * d.n2;
      su -= a.ua[q] * umsk<double>(ci, k);
      sv -= a.va[q] * vmsk<double>(ci, k);
    }
    for (int k = 1; k <= d.jpk - 1; ++k) {
      const long q = o3 + (long)(k - 1) * d.n2;
      a.ua[q] += d.e3u_n(c.ij, k, c.m) * umsk<double>(ci, k) * d.r1_hu_0[c.ij] * su;
      a.va[q] += d.e3v_n(c.ij, k, c.m) * vmsk<double>(ci, k) * d.r1_hv_0[c.ij] * sv;
    }
  }
  a.un_b[p] = ub;
  a.vn_b[p] = vb;
  a.ssha[p] = 0.0; a.ua_b[p] = 0.0; a.va_b[p] = 0.0; a.un_adv[p] = 0.0; a.vn_adv[p] = 0.0;
}

}  // namespace nemo
