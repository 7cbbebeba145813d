// k_step.cuh -- the parts of the time step (step.F90:96-305) that close the path into
// a model step with the linear free surface: the vertical velocity from the
// horizontal divergence, the time step of dyn_zdf without vertical viscosity, the
// Asselin filter and swap of the momentum and of the sea surface height. The
// momentum trends outside the path (dyn_adv, dyn_vor, dyn_ldf, dyn_hpg) are held at
// 0 by the caller. T is the bulk type, A the type of the barotropic accumulators
// (ua_b, va_b, ssha: double in both forms).
#pragma once
#include "step.h"

namespace nemo {

// div_hor (divhor.F90:76-106: the horizontal divergence of the interior, 0 on the
// closed edges) and wzv (sshwzv.F90:172-189: w integrated up from w(jpk) = 0), one
// column per thread.
template <class T>
__global__ void k_wzv(Dom<T> d, RO<T> un, RO<T> vn, T* wn, T z1_2dt) {
  ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk;
  const long n2 = d.n2, m3 = (long)c.m * d.n3, ij = c.ij;
  const ColInfo ci = d.ci[ij];
  wn[m3 + ij + (long)(jpk - 1) * n2] = T(0);
  T w = T(0);
  for (int k = jpk - 1; k >= 1; --k) {
    const long q = m3 + ij + (long)(k - 1) * n2;
    const T e3n = d.e3t_n(ij, k, c.m);
    T hdiv = T(0);
    if (c.interior)
      hdiv = (d.e2u[ij] * d.e3u_n(ij, k, c.m) * un[q] - d.e2u[ij - 1] * d.e3u_n(ij - 1, k, c.m) * un[q - 1] +
              d.e1v[ij] * d.e3v_n(ij, k, c.m) * vn[q] - d.e1v[ij - jpi] * d.e3v_n(ij - jpi, k, c.m) * vn[q - jpi]) *
             d.r1_e1e2t[ij] / e3n;
    w = w - (e3n * hdiv + z1_2dt * (d.e3t_a(ij, k, c.m) - d.e3t_b(ij, k, c.m))) * tmsk<T>(ci, k);
    wn[q] = w;
  }
}

// The time step of dyn_zdf (dynzdf.F90:112) with no vertical viscosity or drag.
template <class T>
__global__ void k_dyn_zdf_step(Dom<T> d, RO<T> ub, RO<T> vb, T* ua, T* va, T r2dt) {
  const PtIdx c = pt_index(d);
  if (!c.valid || c.k > d.jpk - 1) return;
  const long q = (long)c.m * d.n3 + c.q;
  const ColInfo ci = d.ci[c.ij];
  ua[q] = (ub[q] + r2dt * ua[q]) * umsk<T>(ci, c.k);
  va[q] = (vb[q] + r2dt * va[q]) * vmsk<T>(ci, c.k);
}

// dyn_nxt (dynnxt.F90:114-358; linear free surface, ln_dynspg_ts with ln_bt_fw),
// one (i,j) column of u and of v per thread: the barotropic part of the after
// velocity replaced by the sub-steps' ua_b; lbc of ua, va (the closed edges 0);
// the Euler swap or the Asselin filter and swap with the before velocity returned
// to the time-split barotropic estimate; the now and before barotropic velocities.
template <class T, class A>
__global__ void k_dyn_nxt(Dom<T> d, NxtArgs<T, A> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const int jpk = d.jpk;
  const long n2 = d.n2, m3 = (long)c.m * d.n3, m2 = (long)c.m * n2, ij = c.ij;
  const ColInfo ci = d.ci[ij];
  const T r1u = d.r1_hu_0[ij], r1v = d.r1_hv_0[ij];
  const T uab = T(a.ua_b[m2 + ij]), vab = T(a.va_b[m2 + ij]);
  T* ua = a.ua + m3;
  T* va = a.va + m3;
  T* un = a.un + m3;
  T* vn = a.vn + m3;
  T* ub = a.ub + m3;
  T* vb = a.vb + m3;
  auto Q = [&](int k) { return ij + (long)(k - 1) * n2; };
  // (:114-126)
  T zue = T(0), zve = T(0);
  for (int k = 1; k <= jpk - 1; ++k) {
    const long q = Q(k);
    zue = zue + d.e3u_n(ij, k, c.m) * ua[q] * umsk<T>(ci, k);
    zve = zve + d.e3v_n(ij, k, c.m) * va[q] * vmsk<T>(ci, k);
  }
  for (int k = 1; k <= jpk - 1; ++k) {
    const long q = Q(k);
    ua[q] = (ua[q] - zue * r1u + uab) * umsk<T>(ci, k);
    va[q] = (va[q] - zve * r1v + vab) * vmsk<T>(ci, k);
  }
  if (!c.interior)  // lbc_lnk of ua, va (:146): the closed edges, every level
    for (int k = 1; k <= jpk; ++k) {
      ua[Q(k)] = T(0);
      va[Q(k)] = T(0);
    }
  if (a.euler) {  // (:168-171)
    for (int k = 1; k <= jpk - 1; ++k) {
      un[Q(k)] = ua[Q(k)];
      vn[Q(k)] = va[Q(k)];
    }
  } else {  // (:197-211), then (:312-324)
    T sb = T(0), tb = T(0);
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = Q(k);
      // FP32: the time laplacian from differences (see k_tra_nxt)
      const T zuf = un[q] + a.atfp * (sizeof(T) == 4 ? (ua[q] - un[q]) - (un[q] - ub[q]) : ub[q] - T(2) * un[q] + ua[q]);
      const T zvf = vn[q] + a.atfp * (sizeof(T) == 4 ? (va[q] - vn[q]) - (vn[q] - vb[q]) : vb[q] - T(2) * vn[q] + va[q]);
      ub[q] = zuf;
      vb[q] = zvf;
      un[q] = ua[q];
      vn[q] = va[q];
      sb = sb + d.e3u_n(ij, k, c.m) * zuf * umsk<T>(ci, k);
      tb = tb + d.e3v_n(ij, k, c.m) * zvf * vmsk<T>(ci, k);
    }
    const T unb = a.un_b[m2 + ij], vnb = a.vn_b[m2 + ij];
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = Q(k);
      ub[q] = ub[q] - (sb * r1u - unb) * umsk<T>(ci, k);
      vb[q] = vb[q] - (tb * r1v - vnb) * vmsk<T>(ci, k);
    }
  }
  // (:345-358)
  T sun = T(0), sub = T(0), svn = T(0), svb = T(0);
  for (int k = 1; k <= jpk - 1; ++k) {
    const long q = Q(k);
    const T eu = d.e3u_n(ij, k, c.m), ev = d.e3v_n(ij, k, c.m), um = umsk<T>(ci, k), vm = vmsk<T>(ci, k);
    sun = sun + eu * un[q] * um;
    sub = sub + eu * ub[q] * um;
    svn = svn + ev * vn[q] * vm;
    svb = svb + ev * vb[q] * vm;
  }
  a.un_b[m2 + ij] = sun * r1u;
  a.ub_b[m2 + ij] = sub * r1u;
  a.vn_b[m2 + ij] = svn * r1v;
  a.vb_b[m2 + ij] = svb * r1v;
}

// ssh_swp (sshwzv.F90:216-267), linear free surface, one point per thread.
template <class T, class A>
__global__ void k_ssh_swp(Dom<T> d, T* sshb, T* sshn, const A* __restrict__ ssha, T atfp, int euler) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const long p = (long)blockIdx.z * d.n2 + (long)(i - 1) + (long)(j - 1) * d.jpi;
  const T sa = T(ssha[p]);
  if (!euler)
    sshb[p] = sshn[p] + atfp * (sizeof(T) == 4 ? (sa - sshn[p]) - (sshn[p] - sshb[p]) : sshb[p] - T(2) * sshn[p] + sa);
  sshn[p] = sa;
}

}  // namespace nemo
