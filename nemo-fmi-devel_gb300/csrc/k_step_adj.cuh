// k_step_adj.cuh -- the adjoints of the time stepping of the model step for the linear
// free surface, FP64: wzv (sshwzv.F90:129-213 with divhor.F90:62-110), dyn_nxt
// (dynnxt.F90:66-377, ln_bt_fw) and ssh_swp (sshwzv.F90:216-267). Gather form: a
// thread writes only its own column (point).
#pragma once
#include "adj.h"

namespace nemo {

// wzv, first kernel (one column per thread): G(l) = hdivn_ad(l) r1_e1e2t / e3t_n with
// hdivn_ad(l) = -e3t_n tmask times the sum of wn_ad over the levels 1..l; wn_ad zeroed
__global__ void k_wzv_adj_g(Dom<double> d, double* wn_ad, double* G) {
  const ColIdx<double> c = col_index(d);
  if (!c.valid) return;
  const long o = (long)c.m * d.n3 + c.ij;
  const ColInfo ci = d.ci[c.ij];
  double C = 0.0;
  for (int k = 1; k <= d.jpk; ++k) {
    const long q = o + (long)(k - 1) * d.n2;
    if (k <= d.jpk - 1) {
      C += wn_ad[q];
      double g = 0.0;
      if (c.interior) {
        const double e3 = d.e3t_n(c.ij, k, c.m);
        const double hd = -(e3 * tmsk<double>(ci, k)) * C;
        g = hd * d.r1_e1e2t[c.ij] / e3;
      }
      G[q] = g;
    } else {
      G[q] = 0.0;
    }
    wn_ad[q] = 0.0;
  }
}

// wzv, second kernel (one point per thread): the transposed divergence of the fluxes
// e2u e3u un and e1v e3v vn
__global__ void k_wzv_adj_uv(Dom<double> d, double* un_ad, double* vn_ad, const double* G) {
  const PtIdx c = pt_index(d);
  if (!c.valid || c.k > d.jpk - 1) return;
  const long o = (long)c.m * d.n3, q = o + c.q, nb = d.jpi;
  const double fu = d.e2u[c.ij] * d.e3u_n(c.ij, c.k, c.m), fv = d.e1v[c.ij] * d.e3v_n(c.ij, c.k, c.m);
  double u = un_ad[q], v = vn_ad[q];
  const bool in = c.interior;
  if (in) u += fu * G[q];
  if (c.i + 1 <= d.jpi - 1 && c.j >= 2 && c.j <= d.jpj - 1 && c.i + 1 >= 2) u -= fu * G[q + 1];
  if (in) v += fv * G[q];
  if (c.j + 1 <= d.jpj - 1 && c.i >= 2 && c.i <= d.jpi - 1 && c.j + 1 >= 2) v -= fv * G[q + nb];
  un_ad[q] = u;
  vn_ad[q] = v;
}


// dyn_nxt, one (i,j) column of u and of v per thread, the forward's steps reversed:
// the barotropic velocities (:345-358), the return of ub to the time-split estimate
// (:312-324), the Asselin filter and swap (:197-211) or the Euler swap (:168-171), the
// lbc of ua (:146) and the replacement of its barotropic part (:114-126)
__global__ void k_dyn_nxt_adj(Dom<double> d, NxtAdjArgs a) {
  const ColIdx<double> c = col_index(d);
  if (!c.valid) return;
  const long p = (long)c.m * d.n2 + c.ij, o = (long)c.m * d.n3 + c.ij;
  const ColInfo ci = d.ci[c.ij];
  for (int dir = 0; dir < 2; ++dir) {
    double *ua = dir ? a.va : a.ua, *un = dir ? a.vn : a.un, *ub = dir ? a.vb : a.ub;
    double *unb = dir ? a.vn_b : a.un_b, *ubb = dir ? a.vb_b : a.ub_b, *uab = dir ? a.va_b : a.ua_b;
    const double r1h = dir ? d.r1_hv_0[c.ij] : d.r1_hu_0[c.ij];
    auto msk = [&](int k) { return dir ? vmsk<double>(ci, k) : umsk<double>(ci, k); };
    auto e3 = [&](int k) { return dir ? d.e3v_n(c.ij, k, c.m) : d.e3u_n(c.ij, k, c.m); };
    const double bn = unb[p], bb = ubb[p];
    double su = 0.0;
    for (int k = 1; k <= d.jpk - 1; ++k) {
      const long q = o + (long)(k - 1) * d.n2;
      un[q] += e3(k) * msk(k) * r1h * bn;
      ub[q] += e3(k) * msk(k) * r1h * bb;
      su += ub[q] * msk(k);
    }
    unb[p] = 0.0;
    ubb[p] = 0.0;
    if (!a.euler) {
      unb[p] += su;
      const double zad = -su * r1h;
      for (int k = 1; k <= d.jpk - 1; ++k) {
        const long q = o + (long)(k - 1) * d.n2;
        ub[q] += e3(k) * msk(k) * zad;
        const double b = ub[q];
        ua[q] += un[q] + a.atfp * b;
        un[q] = (1.0 - 2.0 * a.atfp) * b;
        ub[q] = a.atfp * b;
      }
    } else {
      for (int k = 1; k <= d.jpk - 1; ++k) {
        const long q = o + (long)(k - 1) * d.n2;
        ua[q] += un[q];
        un[q] = 0.0;
      }
    }
    if (!c.interior) {
      for (int k = 1; k <= d.jpk; ++k) ua[o + (long)(k - 1) * d.n2] = 0.0;
    }
    double s = 0.0;
    for (int k = 1; k <= d.jpk - 1; ++k) {
      const long q = o + (long)(k - 1) * d.n2;
      ua[q] = ua[q] * msk(k);
      s += ua[q];
    }
    uab[p] += s;
    const double zad = -s * r1h;
    for (int k = 1; k <= d.jpk - 1; ++k) {
      const long q = o + (long)(k - 1) * d.n2;
      ua[q] += e3(k) * msk(k) * zad;
    }
  }
}

// ssh_swp, one point per thread
__global__ void k_ssh_swp_adj(Dom<double> d, double* sb, double* sn, double* sa, double atfp, int euler) {
  const ColIdx<double> c = col_index(d);
  if (!c.valid) return;
  const long p = (long)c.m * d.n2 + c.ij;
  if (euler) {
    sa[p] += sn[p];
    sn[p] = 0.0;
  } else {
    const double b = sb[p];
    sa[p] += sn[p] + atfp * b;
    sn[p] = (1.0 - 2.0 * atfp) * b;
    sb[p] = atfp * b;
  }
}

}  // namespace nemo
