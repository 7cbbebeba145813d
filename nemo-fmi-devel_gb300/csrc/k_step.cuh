// k_step.cuh -- the parts of the time step (step.F90:96-305) that close the path into
// a model step with the linear free surface: the vertical velocity from the
// horizontal divergence, the time step of dyn_zdf without vertical viscosity, the
// Asselin filter and swap of the momentum and of the sea surface height. The
// momentum trends outside the path (dyn_adv, dyn_vor, dyn_ldf, dyn_hpg) are held at
// 0 by the caller. T is the bulk type, A the type of the barotropic accumulators
// (ua_b, va_b, ssha: double in both forms).
#pragma once
#include "nemo_sin.h"
#include "step.h"

namespace nemo {

// div_hor (divhor.F90:76-106: the horizontal divergence of the interior, 0 on the
// closed edges) and wzv (sshwzv.F90:172-189: w integrated up from w(jpk) = 0), one
// column per thread. The loads of a level do not depend on the running sum, so the
// unrolled k-loops keep several levels' loads in flight (the column kernels of this
// file are otherwise bound by one memory round trip per level).
template <class T>
__global__ void k_wzv(Dom<T> d, RO<T> un, RO<T> vn, T* wn, T z1_2dt) {
  ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk;
  const long n2 = d.n2, m3 = (long)c.m * d.n3, ij = c.ij;
  const ColInfo ci = d.ci[ij];
  wn[m3 + ij + (long)(jpk - 1) * n2] = T(0);
  T w = T(0);
  #pragma unroll 4
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
__global__ void k_dyn_zdf_step(Dom<T> d, RO<T> ub, RO<T> vb, T* ua, T* va, T r2dt, RO<T> e3u_b, RO<T> e3v_b,
                               RO<T> e3u_a, RO<T> e3v_a) {
  const PtIdx c = pt_index(d);
  if (!c.valid || c.k > d.jpk - 1) return;
  const long q = (long)c.m * d.n3 + c.q;
  const ColInfo ci = d.ci[c.ij];
  if (e3u_b) {  // flux form with a variable volume: on the thickness-weighted velocity (:115-120)
    ua[q] = (e3u_b[q] * ub[q] + r2dt * d.e3u_n(c.ij, c.k, c.m) * ua[q]) / e3u_a[q] * umsk<T>(ci, c.k);
    va[q] = (e3v_b[q] * vb[q] + r2dt * d.e3v_n(c.ij, c.k, c.m) * va[q]) / e3v_a[q] * vmsk<T>(ci, c.k);
  } else {      // on the velocity (:109-114)
    ua[q] = (ub[q] + r2dt * ua[q]) * umsk<T>(ci, c.k);
    va[q] = (vb[q] + r2dt * va[q]) * vmsk<T>(ci, c.k);
  }
}

// The implicit vertical viscosity of one U- (V-) column of dyn_zdf
// (dynzdf.F90:127-141, :205-302) after its time step: the bottom stress of the
// barotropic after velocity ab, then the system of avm (iso-level lateral mixing,
// no adaptive-implicit advection) with the surface condition, the implicit drag on
// the bottom diagonal and the wind stress in the surface right-hand side, assembled
// and forward-eliminated in one downward sweep (its diagonals kept in zwd, zws) and
// back-substituted upwards. The W-point scale factor across the U- (V-) point is the
// MIN of the neighbouring e3w (the rest state of a linear free surface).
template <bool U, class T>
__device__ __forceinline__ void dyn_zdf_column(const Dom<T>& d, const DynZdfArgs<T>& a, long ij, int m,
                                               const ColInfo& ci, T* pa, const double* ab, const T* tau,
                                               const T* tau_b) {
  const long n2 = d.n2, m3 = (long)m * d.n3 + ij, p2 = (long)m * d.n2 + ij;
  const long nb = U ? 1 : d.jpi;
  const int jpk = d.jpk, kb = U ? ci.mbku : ci.mbkv;
  auto mk = [&](int k) { return U ? umsk<T>(ci, k) : vmsk<T>(ci, k); };
  auto e3 = [&](int k) { return U ? d.e3u_n(ij, k, m) : d.e3v_n(ij, k, m); };
  auto e3xw = [&](int k) { return fmn(d.e3w_n(ij, k, m), d.e3w_n(ij + nb, k, m)); };
  auto wxm = [&](int k) { return k == 1 ? mk(1) : mk(k) * mk(k - 1); };
  const T rc = a.rcdu[p2 + nb] + a.rcdu[p2];
  {
    const long q = m3 + (long)(kb - 1) * n2;
    pa[q] = pa[q] + a.r2dt * T(0.5) * rc * (T)ab[p2] / e3(kb);
  }
  T wd_p = T(1), ws_p = T(0), x_p = T(0);
  for (int k = 1; k <= jpk - 1; ++k) {
    const long q = m3 + (long)(k - 1) * n2;
    const T ze3a = e3(k);
    const T zzws = -a.zdt * (a.avm[q + n2 + nb] + a.avm[q + n2]) / (ze3a * e3xw(k + 1)) * wxm(k + 1);
    T wd, x = pa[q];
    if (k == 1) {
      wd = T(1) - zzws;
      if (k == kb) wd = wd - a.r2dt * T(0.5) * rc / e3(kb);
      x = x + a.r2dt * T(0.5) * (tau_b[p2] + tau[p2]) / (ze3a * a.rau0) * mk(1);
    } else {
      const T zzwi = -a.zdt * (a.avm[q + nb] + a.avm[q]) / (ze3a * e3xw(k)) * wxm(k);
      wd = T(1) - zzwi - zzws;
      if (k == kb) wd = wd - a.r2dt * T(0.5) * rc / e3(kb);
      wd = wd - zzwi * ws_p / wd_p;
      x = x - zzwi / wd_p * x_p;
    }
    a.zwd[q] = wd;
    a.zws[q] = zzws;
    pa[q] = x;
    wd_p = wd; ws_p = zzws; x_p = x;
  }
  T nxt = T(0);
  for (int k = jpk - 1; k >= 1; --k) {
    const long q = m3 + (long)(k - 1) * n2;
    const T x = (k == jpk - 1) ? pa[q] / a.zwd[q] : (pa[q] - a.zws[q] * nxt) / a.zwd[q];
    pa[q] = x;
    nxt = x;
  }
}

// dyn_zdf (dynzdf.F90:47-499) with the implicit vertical viscosity, one column per
// thread: the time step and the removal of the barotropic after velocity on every
// column (:112, :122-126), then the u and v systems of the interior columns.
template <class T>
__global__ void k_dyn_zdf_imp(Dom<T> d, DynZdfArgs<T> a) {
  const ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const long n2 = d.n2, m3 = (long)c.m * d.n3 + c.ij, p2 = (long)c.m * d.n2 + c.ij;
  const ColInfo ci = d.ci[c.ij];
  const T uab = (T)a.ua_b[p2], vab = (T)a.va_b[p2];
  for (int k = 1; k <= d.jpk - 1; ++k) {
    const long q = m3 + (long)(k - 1) * n2;
    const T um = umsk<T>(ci, k), vm = vmsk<T>(ci, k);
    a.ua[q] = ((a.ub[q] + a.r2dt * a.ua[q]) * um - uab) * um;
    a.va[q] = ((a.vb[q] + a.r2dt * a.va[q]) * vm - vab) * vm;
  }
  if (!c.interior) return;
  dyn_zdf_column<true>(d, a, c.ij, c.m, ci, a.ua, a.ua_b, a.utau, a.utau_b);
  dyn_zdf_column<false>(d, a, c.ij, c.m, ci, a.va, a.va_b, a.vtau, a.vtau_b);
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
  // six distinct arrays: restrict lets the unrolled loops load ahead of the stores
  T* __restrict__ ua = a.ua + m3;
  T* __restrict__ va = a.va + m3;
  T* __restrict__ un = a.un + m3;
  T* __restrict__ vn = a.vn + m3;
  T* __restrict__ ub = a.ub + m3;
  T* __restrict__ vb = a.vb + m3;
  auto Q = [&](int k) { return ij + (long)(k - 1) * n2; };
  // (:114-126)
  T zue = T(0), zve = T(0);
  #pragma unroll 4
  for (int k = 1; k <= jpk - 1; ++k) {
    const long q = Q(k);
    zue = zue + d.e3u_n(ij, k, c.m) * ua[q] * umsk<T>(ci, k);
    zve = zve + d.e3v_n(ij, k, c.m) * va[q] * vmsk<T>(ci, k);
  }
  #pragma unroll 4
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
  // the now and before barotropic velocities (:345-358) are summed where un and ub
  // take their final values, level by level in the same order
  T sun = T(0), sub = T(0), svn = T(0), svb = T(0);
  if (a.euler) {  // (:168-171)
    #pragma unroll 4
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = Q(k);
      const T eu = d.e3u_n(ij, k, c.m), ev = d.e3v_n(ij, k, c.m), um = umsk<T>(ci, k), vm = vmsk<T>(ci, k);
      const T u = ua[q], v = va[q];
      un[q] = u;
      vn[q] = v;
      sun = sun + eu * u * um;
      sub = sub + eu * ub[q] * um;
      svn = svn + ev * v * vm;
      svb = svb + ev * vb[q] * vm;
    }
  } else {  // (:197-211), then (:312-324)
    T sb = T(0), tb = T(0);
    #pragma unroll 4
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = Q(k);
      const T eu = d.e3u_n(ij, k, c.m), ev = d.e3v_n(ij, k, c.m), um = umsk<T>(ci, k), vm = vmsk<T>(ci, k);
      const T u = ua[q], v = va[q];
      // FP32: the time laplacian from differences (see k_tra_nxt)
      const T zuf = un[q] + a.atfp * (sizeof(T) == 4 ? (u - un[q]) - (un[q] - ub[q]) : ub[q] - T(2) * un[q] + u);
      const T zvf = vn[q] + a.atfp * (sizeof(T) == 4 ? (v - vn[q]) - (vn[q] - vb[q]) : vb[q] - T(2) * vn[q] + v);
      ub[q] = zuf;
      vb[q] = zvf;
      un[q] = u;
      vn[q] = v;
      sb = sb + eu * zuf * um;
      tb = tb + ev * zvf * vm;
      sun = sun + eu * u * um;
      svn = svn + ev * v * vm;
    }
    const T unb = a.un_b[m2 + ij], vnb = a.vn_b[m2 + ij];
    #pragma unroll 4
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = Q(k);
      const T eu = d.e3u_n(ij, k, c.m), ev = d.e3v_n(ij, k, c.m), um = umsk<T>(ci, k), vm = vmsk<T>(ci, k);
      const T ubk = ub[q] - (sb * r1u - unb) * um;
      const T vbk = vb[q] - (tb * r1v - vnb) * vm;
      ub[q] = ubk;
      vb[q] = vbk;
      sub = sub + eu * ubk * um;
      svb = svb + ev * vbk * vm;
    }
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


// ----------------------------------------------------------------------- ldf_slp
// ldf_slp (ldfslp.F90:83-374) with ldf_slp_mxl (:620-729), z-coordinate with or
// without partial steps, without cavities, in three kernels: the slopes just below the mixed
// layer (one column per thread), the slopes before the Shapiro filter at u-, v- and
// w-points (one point per thread), the filter with the coastal decrease and lbc.
// The density gradients zgru, zgrv and zdzr of the reference's work arrays are
// formed where they are read, from the same operands in the same order.
template <class T, bool ZPS = false>
struct SlpPt {
  const Dom<T>& d;
  const SlpArgs<T>& a;
  long m3;
  int m;
  __device__ __forceinline__ long Q(int i, int j, int k) const {
    return (long)(i - 1) + (long)(j - 1) * d.jpi + (long)(k - 1) * d.n2;
  }
  __device__ __forceinline__ T um(int i, int j, int k) const { return umsk<T>(d.ci[Q(i, j, 1)], k); }
  __device__ __forceinline__ T vm(int i, int j, int k) const { return vmsk<T>(d.ci[Q(i, j, 1)], k); }
  __device__ __forceinline__ T tm(int i, int j, int k) const { return tmsk<T>(d.ci[Q(i, j, 1)], k); }
  __device__ __forceinline__ T wm(int i, int j, int k) const { return wmsk<T>(d.ci[Q(i, j, 1)], k); }
  __device__ __forceinline__ T prd(int i, int j, int k) const { return a.prd[m3 + Q(i, j, k)]; }
  // with partial steps (ZPS) the bottom level's gradients are zps_hde's
  // (ldfslp.F90:144-151); the z-coordinate form compiles without the test
  __device__ __forceinline__ T gru(int i, int j, int k) const {
    if constexpr (ZPS) {
      if (k == d.ci[Q(i, j, 1)].mbku) return a.gru_b[(long)m * d.n2 + Q(i, j, 1)];
    }
    return um(i, j, k) * (prd(i + 1, j, k) - prd(i, j, k));
  }
  __device__ __forceinline__ T grv(int i, int j, int k) const {
    if constexpr (ZPS) {
      if (k == d.ci[Q(i, j, 1)].mbkv) return a.grv_b[(long)m * d.n2 + Q(i, j, 1)];
    }
    return vm(i, j, k) * (prd(i, j + 1, k) - prd(i, j, k));
  }
  __device__ __forceinline__ T dzr(int i, int j, int k) const {
    if (k == 1) return T(0);
    const long q = m3 + Q(i, j, k);
    return a.zm1_g * (a.prd[q] + T(1)) * (a.pn2[q] + a.pn2[q + d.n2]) * (T(1) - T(0.5) * tm(i, j, k + 1));
  }
  __device__ __forceinline__ T oml(int i, int j, int k) const {
    return k <= a.nmln[(long)m * d.n2 + Q(i, j, 1)] - 1 ? T(1) : T(0);
  }
};

template <class T, bool ZPS>
__global__ void k_slp_mxl(Dom<T> d, SlpArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const long p = (long)c.m * d.n2 + c.ij;
  if (!c.interior) {  // lbc_lnk of the four mixed-layer slopes: the closed edges 0
    a.uml[p] = T(0); a.vml[p] = T(0); a.wiml[p] = T(0); a.wjml[p] = T(0);
    a.hu[p] = T(0); a.hv[p] = T(0);
    return;
  }
  const SlpPt<T, ZPS> P{d, a, (long)c.m * d.n3, c.m};
  const int i = c.i, j = c.j, jpk = d.jpk, jpi = d.jpi;
  const long ij = c.ij, m2 = (long)c.m * d.n2;
  const int n0 = a.nmln[m2 + ij], ne = a.nmln[m2 + ij + 1], nn = a.nmln[m2 + ij + jpi];
  int iku = n0 > ne ? n0 : ne;
  iku = iku < 1 ? 1 : (iku > jpk - 1 ? jpk - 1 : iku);
  int ikv = n0 > nn ? n0 : nn;
  ikv = ikv < 1 ? 1 : (ikv > jpk - 1 ? jpk - 1 : ikv);
  T zbu = T(0.5) * (P.dzr(i, j, iku) + P.dzr(i + 1, j, iku));
  T zbv = T(0.5) * (P.dzr(i, j, ikv) + P.dzr(i, j + 1, ikv));
  const T zau = P.gru(i, j, iku) * d.r1_e1u[ij];
  const T zav = P.grv(i, j, ikv) * d.r1_e2v[ij];
  zbu = fmn(fmn(zbu, -a.z1_slpmax * fabs(zau)), T(-7.e+3) / d.e3u_n(ij, iku, c.m) * fabs(zau));
  zbv = fmn(fmn(zbv, -a.z1_slpmax * fabs(zav)), T(-7.e+3) / d.e3v_n(ij, ikv, c.m) * fabs(zav));
  const T uml = zau / (zbu - a.zeps) * P.um(i, j, iku);
  const T vml = zav / (zbv - a.zeps) * P.vm(i, j, ikv);
  const int ik = n0 + 1 < jpk ? n0 + 1 : jpk;
  const int ikm1 = ik - 1 > 1 ? ik - 1 : 1;
  const T zbw = a.zm1_2g * a.pn2[P.m3 + P.Q(i, j, ik)] * (P.prd(i, j, ik) + P.prd(i, j, ikm1) + T(2));
  const T zci = fmx(P.um(i - 1, j, ik) + P.um(i, j, ik) + P.um(i - 1, j, ikm1) + P.um(i, j, ikm1), a.zeps) * d.e1t[ij];
  const T zcj = fmx(P.vm(i, j - 1, ik) + P.vm(i, j, ik) + P.vm(i, j - 1, ikm1) + P.vm(i, j, ikm1), a.zeps) * d.e2t[ij];
  const T tmk = P.tm(i, j, ik);
  const T zai = (P.gru(i - 1, j, ik) + P.gru(i, j, ik) + P.gru(i - 1, j, ikm1) + P.gru(i, j, ikm1)) / zci * tmk;
  const T zaj = (P.grv(i, j - 1, ik) + P.grv(i, j, ik) + P.grv(i, j - 1, ikm1) + P.grv(i, j, ikm1)) / zcj * tmk;
  const T e3w = d.e3w_n(ij, ik, c.m);
  const T zbi = fmn(fmn(zbw, T(-100) * fabs(zai)), T(-7.e+3) / e3w * fabs(zai));
  const T zbj = fmn(fmn(zbw, T(-100) * fabs(zaj)), T(-7.e+3) / e3w * fabs(zaj));
  a.uml[p] = uml;
  a.vml[p] = vml;
  a.wiml[p] = zai / (zbi - a.zeps) * tmk;
  a.wjml[p] = zaj / (zbj - a.zeps) * tmk;
  // (:188-194) the mixed-layer slope over the depth of the last T-point in it
  const T h0 = a.hmlpt[p], he = a.hmlpt[p + 1], hn = a.hmlpt[p + jpi];
  a.hu[p] = uml / fmx(fmx(h0, he), T(5));
  a.hv[p] = vml / fmx(fmx(h0, hn), T(5));
}

// The slopes before the filter: u, v (:197-233) and w (:281-315) at levels 2..jpkm1;
// 0 on the closed edges (the lbc_lnk of :234 and :316).
template <class T, bool ZPS>
__global__ void k_slp_pre(Dom<T> d, SlpArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid || c.k < 2 || c.k > d.jpk - 1) return;
  const long o = (long)c.m * d.n3 + c.q;
  if (!c.interior) {
    a.zu[o] = T(0); a.zv[o] = T(0); a.zwi[o] = T(0); a.zwj[o] = T(0);
    return;
  }
  const SlpPt<T, ZPS> P{d, a, (long)c.m * d.n3, c.m};
  const int i = c.i, j = c.j, k = c.k, jpi = d.jpi;
  const long ij = c.ij, p = (long)c.m * d.n2 + ij;
  // u- and v-points
  {
    const T zau = P.gru(i, j, k) * d.r1_e1u[ij];
    const T zav = P.grv(i, j, k) * d.r1_e2v[ij];
    const T dz0 = P.dzr(i, j, k);
    T zbu = T(0.5) * (dz0 + P.dzr(i + 1, j, k));
    T zbv = T(0.5) * (dz0 + P.dzr(i, j + 1, k));
    zbu = fmn(fmn(zbu, -a.z1_slpmax * fabs(zau)), T(-7.e+3) / d.e3u_n(ij, k, c.m) * fabs(zau));
    zbv = fmn(fmn(zbv, -a.z1_slpmax * fabs(zav)), T(-7.e+3) / d.e3v_n(ij, k, c.m) * fabs(zav));
    const T o0 = P.oml(i, j, k);
    const T zfi = fmx(o0, P.oml(i + 1, j, k));
    const T zfj = fmx(o0, P.oml(i, j + 1, k));
    const long m3 = P.m3;
    const T g0 = a.gdept[m3 + c.q];
    const T zdepu = T(0.5) * ((g0 + a.gdept[m3 + c.q + 1]) - T(2) * T(0) - d.e3u_n(ij, 1, c.m));
    const T zdepv = T(0.5) * ((g0 + a.gdept[m3 + c.q + jpi]) - T(2) * T(0) - d.e3v_n(ij, 1, c.m));
    a.zu[o] = ((T(1) - zfi) * zau / (zbu - a.zeps) + zfi * zdepu * a.hu[p]) * P.um(i, j, k);
    a.zv[o] = ((T(1) - zfj) * zav / (zbv - a.zeps) + zfj * zdepv * a.hv[p]) * P.vm(i, j, k);
  }
  // w-points
  {
    const long q = P.m3 + c.q;
    const T zbw = a.zm1_2g * a.pn2[q] * (a.prd[q] + a.prd[q - d.n2] + T(2));
    const T zci = fmx(P.um(i - 1, j, k) + P.um(i, j, k) + P.um(i - 1, j, k - 1) + P.um(i, j, k - 1), a.zeps) * d.e1t[ij];
    const T zcj = fmx(P.vm(i, j - 1, k) + P.vm(i, j, k - 1) + P.vm(i, j - 1, k - 1) + P.vm(i, j, k), a.zeps) * d.e2t[ij];
    const T wmk = P.wm(i, j, k);
    const T zai = (P.gru(i - 1, j, k) + P.gru(i, j, k - 1) + P.gru(i - 1, j, k - 1) + P.gru(i, j, k)) / zci * wmk;
    const T zaj = (P.grv(i, j - 1, k) + P.grv(i, j, k - 1) + P.grv(i, j - 1, k - 1) + P.grv(i, j, k)) / zcj * wmk;
    const T e3w = d.e3w_n(ij, k, c.m);
    const T zbi = fmn(fmn(zbw, T(-100) * fabs(zai)), T(-7.e+3) / e3w * fabs(zai));
    const T zbj = fmn(fmn(zbw, T(-100) * fabs(zaj)), T(-7.e+3) / e3w * fabs(zaj));
    const T zfk = fmx(P.oml(i, j, k), P.oml(i, j, k - 1));
    const T gw1 = a.gdepw[P.m3 + ij];
    const T zck = (a.gdepw[q] - gw1) / fmx(a.hmlp[p] - gw1, T(10));
    a.zwi[o] = (zai / (zbi - a.zeps) * (T(1) - zfk) + zck * a.wiml[p] * zfk) * wmk;
    a.zwj[o] = (zaj / (zbj - a.zeps) * (T(1) - zfk) + zck * a.wjml[p] * zfk) * wmk;
  }
}

// 1-2-1 Shapiro filter of the nine neighbours at level k (:237-275, :319-353)
template <class T>
__device__ __forceinline__ T shapiro(const T* __restrict__ z, long q, int jpi) {
  return z[q - 1 - jpi] + z[q + 1 - jpi] + z[q - 1 + jpi] + z[q + 1 + jpi] +
         T(2) * (z[q - jpi] + z[q - 1] + z[q + 1] + z[q + jpi]) + T(4) * z[q];
}

// The filtered slopes with the decrease near coasts and topography (:237-361) on
// the interior of levels 2..jpkm1; lbc_lnk (:365): 0 on the closed edges, every level.
template <class T>
__global__ void k_slp_filter(Dom<T> d, SlpArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const long o = (long)c.m * d.n3 + c.q;
  if (!c.interior) {
    a.uslp[o] = T(0); a.vslp[o] = T(0); a.wslpi[o] = T(0); a.wslpj[o] = T(0);
    return;
  }
  if (c.k < 2 || c.k > d.jpk - 1) return;
  const SlpPt<T> P{d, a, (long)c.m * d.n3, c.m};
  const int i = c.i, j = c.j, k = c.k, jpi = d.jpi;
  const T z1_16 = T(1) / T(16);
  T u = z1_16 * shapiro(a.zu, o, jpi);
  T v = z1_16 * shapiro(a.zv, o, jpi);
  u = u * (P.um(i, j + 1, k) + P.um(i, j - 1, k)) * T(0.5) * (P.um(i, j, k) + P.um(i, j, k + 1)) * T(0.5);
  v = v * (P.vm(i + 1, j, k) + P.vm(i - 1, j, k)) * T(0.5) * (P.vm(i, j, k) + P.vm(i, j, k + 1)) * T(0.5);
  const T zcofw = P.wm(i, j, k) * z1_16;
  T wi = shapiro(a.zwi, o, jpi) * zcofw;
  T wj = shapiro(a.zwj, o, jpi) * zcofw;
  const T zck = (P.um(i, j, k) + P.um(i - 1, j, k)) * (P.vm(i, j, k) + P.vm(i, j - 1, k)) * T(0.25);
  a.uslp[o] = u;
  a.vslp[o] = v;
  a.wslpi[o] = wi * zck;
  a.wslpj[o] = wj * zck;
}

// zps_hde (zpshde.F90:41-148): the horizontal gradients of the tracers at the last
// ocean level of the u- and v-points (the partial step), each tracer interpolated
// to the shallower bottom; the loop of the reference covers i <= jpim1, j <= jpjm1
// and lbc_lnk then zeroes the closed edges, so only the interior is nonzero.
template <class T>
__global__ void k_zps_hde(Dom<T> d, RO<T> pta, T* __restrict__ pgtu, T* __restrict__ pgtv, int kjpt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const int m = blockIdx.z, jpi = d.jpi;
  const long ij = (long)(i - 1) + (long)(j - 1) * jpi, n2 = d.n2, n3 = d.n3;
  const bool inner = i >= 2 && i <= jpi - 1 && j >= 2 && j <= d.jpj - 1;
  const ColInfo ci = d.ci[ij];
  const int iku = ci.mbku, ikum1 = iku - 1 > 1 ? iku - 1 : 1;
  const int ikv = ci.mbkv, ikvm1 = ikv - 1 > 1 ? ikv - 1 : 1;
  for (int n = 0; n < kjpt; ++n) {
    const long g = ((long)m * kjpt + n) * n2 + ij;
    if (!inner) {
      pgtu[g] = T(0);
      pgtv[g] = T(0);
      continue;
    }
    const RO<T> t = pta + ((long)m * kjpt + n) * n3;
    auto Q = [&](long o, int k) { return o + (long)(k - 1) * d.n2; };
    const T ze3wu = d.e3w_n(ij + 1, iku, m) - d.e3w_n(ij, iku, m);
    const T ze3wv = d.e3w_n(ij + jpi, ikv, m) - d.e3w_n(ij, ikv, m);
    T gu, gv;
    if (ze3wu >= T(0)) {
      const T zmaxu = ze3wu / d.e3w_n(ij + 1, iku, m);
      const T zti = t[Q(ij + 1, iku)] + zmaxu * (t[Q(ij + 1, ikum1)] - t[Q(ij + 1, iku)]);
      gu = umsk<T>(ci, 1) * (zti - t[Q(ij, iku)]);
    } else {
      const T zmaxu = -ze3wu / d.e3w_n(ij, iku, m);
      const T zti = t[Q(ij, iku)] + zmaxu * (t[Q(ij, ikum1)] - t[Q(ij, iku)]);
      gu = umsk<T>(ci, 1) * (t[Q(ij + 1, iku)] - zti);
    }
    if (ze3wv >= T(0)) {
      const T zmaxv = ze3wv / d.e3w_n(ij + jpi, ikv, m);
      const T ztj = t[Q(ij + jpi, ikv)] + zmaxv * (t[Q(ij + jpi, ikvm1)] - t[Q(ij + jpi, ikv)]);
      gv = vmsk<T>(ci, 1) * (ztj - t[Q(ij, ikv)]);
    } else {
      const T zmaxv = -ze3wv / d.e3w_n(ij, ikv, m);
      const T ztj = t[Q(ij, ikv)] + zmaxv * (t[Q(ij, ikvm1)] - t[Q(ij, ikv)]);
      gv = vmsk<T>(ci, 1) * (t[Q(ij + jpi, ikv)] - ztj);
    }
    pgtu[g] = gu;
    pgtv[g] = gv;
  }
}

// The unmasked in situ density anomaly of one (T, S, depth), eos_insitu_2d
// (eosbn2.F90:295-398): EOS-80 or the simplified equation of state
template <class T>
__device__ __forceinline__ T eos_rd_2d(const EosArgs<T>& a, T t, T sal, T dep);

// zps_hde's density part (zpshde.F90:150-184), one (i,j) a thread: T and S
// interpolated to the shallower bottom depth of the u- (v-) point as k_zps_hde does,
// their density there (eos_insitu_2d at gdept_n of the shallower bottom cell), its
// difference with prd on the deeper side; the closed edges 0 (lbc_lnk)
template <class T>
__global__ void k_zps_hde_rd(Dom<T> d, EosArgs<T> a, RO<T> prd, T* __restrict__ pgru, T* __restrict__ pgrv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const int m = blockIdx.z, jpi = d.jpi;
  const long ij = (long)(i - 1) + (long)(j - 1) * jpi, n2 = d.n2, n3 = d.n3;
  const long g = (long)m * n2 + ij;
  if (!(i >= 2 && i <= jpi - 1 && j >= 2 && j <= d.jpj - 1)) {
    pgru[g] = T(0);
    pgrv[g] = T(0);
    return;
  }
  const ColInfo ci = d.ci[ij];
  const int iku = ci.mbku, ikum1 = iku - 1 > 1 ? iku - 1 : 1;
  const int ikv = ci.mbkv, ikvm1 = ikv - 1 > 1 ? ikv - 1 : 1;
  auto Q = [&](long o, int k) { return o + (long)(k - 1) * n2; };
  const T ze3wu = d.e3w_n(ij + 1, iku, m) - d.e3w_n(ij, iku, m);
  const T ze3wv = d.e3w_n(ij + jpi, ikv, m) - d.e3w_n(ij, ikv, m);
  T zti[2], ztj[2];
  for (int n = 0; n < 2; ++n) {
    const RO<T> t = a.pts + ((long)m * 2 + n) * n3;
    if (ze3wu >= T(0)) {
      const T zmaxu = ze3wu / d.e3w_n(ij + 1, iku, m);
      zti[n] = t[Q(ij + 1, iku)] + zmaxu * (t[Q(ij + 1, ikum1)] - t[Q(ij + 1, iku)]);
    } else {
      const T zmaxu = -ze3wu / d.e3w_n(ij, iku, m);
      zti[n] = t[Q(ij, iku)] + zmaxu * (t[Q(ij, ikum1)] - t[Q(ij, iku)]);
    }
    if (ze3wv >= T(0)) {
      const T zmaxv = ze3wv / d.e3w_n(ij + jpi, ikv, m);
      ztj[n] = t[Q(ij + jpi, ikv)] + zmaxv * (t[Q(ij + jpi, ikvm1)] - t[Q(ij + jpi, ikv)]);
    } else {
      const T zmaxv = -ze3wv / d.e3w_n(ij, ikv, m);
      ztj[n] = t[Q(ij, ikv)] + zmaxv * (t[Q(ij, ikvm1)] - t[Q(ij, ikv)]);
    }
  }
  const long m3 = (long)m * n3;
  const T zhi = ze3wu >= T(0) ? a.gdept[m3 + Q(ij, iku)] : a.gdept[m3 + Q(ij + 1, iku)];
  const T zhj = ze3wv >= T(0) ? a.gdept[m3 + Q(ij, ikv)] : a.gdept[m3 + Q(ij + jpi, ikv)];
  const T zri = eos_rd_2d(a, zti[0], zti[1], zhi), zrj = eos_rd_2d(a, ztj[0], ztj[1], zhj);
  const T um1 = umsk<T>(ci, 1), vm1 = vmsk<T>(ci, 1);
  pgru[g] = ze3wu >= T(0) ? um1 * (zri - prd[m3 + Q(ij, iku)]) : um1 * (prd[m3 + Q(ij + 1, iku)] - zri);
  pgrv[g] = ze3wv >= T(0) ? vm1 * (zrj - prd[m3 + Q(ij, ikv)]) : vm1 * (prd[m3 + Q(ij + jpi, ikv)] - zrj);
}

// ------------------------------------------------------------ surface forcing
// tra_sbc (trasbc.F90:53-206) without runoff and ice-shelf melt, one (i,j) point per
// thread: the move of qsr into qns without penetration (:76-79), the swap of the
// forcing trends (:81-100), the trends of the heat and salt fluxes with the
// concentration/dilution of the linear free surface (:104-118) and their addition to
// the first level of tsa (:123-129), on the reference's index ranges.
template <class T>
__global__ void k_tra_sbc(Dom<T> d, SbcArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const int m = blockIdx.z;
  const long ij = (long)(i - 1) + (long)(j - 1) * d.jpi;
  const long p = (long)m * d.n2 + ij, pt = 2 * (long)m * d.n2 + ij, ps = pt + d.n2;
  T qns = a.qns[p];
  if (!a.traqsr) {
    qns = qns + a.qsr[p];
    a.qns[p] = qns;
    a.qsr[p] = T(0);
  }
  T bt, bs;
  if (a.mode == 0) {
    bt = a.tsc[pt];
    bs = a.tsc[ps];
  } else if (a.mode == 1) {
    bt = T(0);
    bs = T(0);
  } else {
    bt = a.tsc_b[pt];
    bs = a.tsc_b[ps];
  }
  if (a.mode != 2) {
    a.tsc_b[pt] = bt;
    a.tsc_b[ps] = bs;
  }
  if (i < 2 || i > d.jpi - 1 || j < 2) {
    if (a.mode != 0) {  // first step: sbc_tsc = 0 everywhere
      a.tsc[pt] = T(0);
      a.tsc[ps] = T(0);
    }
    return;
  }
  T tt = a.r1_rau0_rcp * qns;
  T ts = a.r1_rau0 * a.sfx[p];
  if (a.linssh) {
    const long q = 2 * (long)m * d.n3 + ij;
    const T e = a.emp[p];
    tt = tt + a.r1_rau0 * e * a.tsn[q];
    ts = ts + a.r1_rau0 * e * a.tsn[q + d.n3];
  }
  a.tsc[pt] = tt;
  a.tsc[ps] = ts;
  const long q = 2 * (long)m * d.n3 + ij;
  const T e3 = d.e3t_n(ij, 1, m);
  a.tsa[q] = a.tsa[q] + a.zfact * (bt + tt) / e3;
  a.tsa[q + d.n3] = a.tsa[q + d.n3] + a.zfact * (bs + ts) / e3;
}

// tra_qsr (traqsr.F90:77-302) with two bands (np_2BD, :243-256), one column per
// thread: the swap of the heat-content trend over the whole column (:134-147), the
// absorbed flux of levels 1..nksr, whose lower-interface attenuation is the next
// level's upper one (the same expression of the same depth, so computed once), the
// temperature trend (:260-267) and the first-level fraction with the closed lbc_lnk
// (:270-277: 0 on the domain edge).
template <class T>
__global__ void k_tra_qsr(Dom<T> d, QsrArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const int m = blockIdx.z;
  const long ij = (long)(i - 1) + (long)(j - 1) * d.jpi;
  const long c3 = (long)m * d.n3 + ij;
  const bool inner = i >= 2 && i <= d.jpi - 1 && j >= 2 && j <= d.jpj - 1;
  if (a.mode != 2) {
    const int k1 = inner ? a.nksr + 1 : 1;  // levels the solve below does not read
    for (int k = k1; k <= d.jpk; ++k) {
      const long q = c3 + (long)(k - 1) * d.n2;
      a.hc_b[q] = a.mode == 0 ? a.hc[q] : T(0);
    }
  }
  if (!inner) {
    a.fraq[(long)m * d.n2 + ij] = T(0);
    return;
  }
  const ColInfo ci = d.ci[ij];
  const T qsr = a.qsr[(long)m * d.n2 + ij];
  T* ta = a.tsa + 2 * (long)m * d.n3 + ij;  // temperature
  T g = a.gdepw[c3];
  T zc0 = a.zz0 * exp(-g * a.xsi0r) + a.zz1 * exp(-g * a.xsi1r);
  T h1 = T(0);
  for (int k = 1; k <= a.nksr; ++k) {
    const long q = c3 + (long)(k - 1) * d.n2;
    g = a.gdepw[q + d.n2];
    const T zc1 = a.zz0 * exp(-g * a.xsi0r) + a.zz1 * exp(-g * a.xsi1r);
    const T hb = a.mode == 0 ? a.hc[q] : (a.mode == 1 ? T(0) : a.hc_b[q]);
    if (a.mode != 2) a.hc_b[q] = hb;
    const T h = qsr * (zc0 * wmsk<T>(ci, k) - zc1 * wmsk<T>(ci, k + 1));
    a.hc[q] = h;
    const long qt = (long)(k - 1) * d.n2;
    ta[qt] = ta[qt] + a.z1_2 * (hb + h) / d.e3t_n(ij, k, m);
    if (k == 1) h1 = h;
    zc0 = zc1;
  }
  a.fraq[(long)m * d.n2 + ij] = qsr != T(0) ? h1 / (a.r1_rau0_rcp * qsr) : T(1);
}

// ------------------------------------------- the simplified equation of state
// eos_insitu (eosbn2.F90:276-292), eos_insitu_pot (:440-462), rab_3d (:645-661)
// with np_seos, and bn2 (:889-933), one point per thread, each expression in the
// reference's association.
// ---- EOS-80. FP64: one power k of the depth of a table in the reference's
// association (eosbn2.F90:242-265): acc = C(0,D); for j = D-1 .. 0,
// acc = (acc*zt + H_j*zs) + C(0,j), H_j = (..(C(n,j)*zs + C(n-1,j))*zs .. + C(1,j)),
// n = D - j. C points at [i][j] (7 x 7) of that k.
template <int D>
__device__ __forceinline__ double e80_zn(const double* __restrict__ C, double zt, double zs) {
  double acc = __ldg(C + D);
#pragma unroll
  for (int j = D - 1; j >= 0; --j) {
    const int n = D - j;
    double h = __ldg(C + n * 7 + j);
#pragma unroll
    for (int i = n - 1; i >= 1; --i) h = h * zs + __ldg(C + i * 7 + j);
    acc = (acc * zt + h * zs) + __ldg(C + j);
  }
  return acc;
}
// table t (0 EOS: degrees 6 4 2 1 in zt; 1 ALP, 2 BET: 5 3 1 0), all depth powers
template <int D0, int D1, int D2, int D3>
__device__ __forceinline__ double e80_poly(const double* __restrict__ tab, double zt, double zs, double zh,
                                           double& zn0) {
  const double z3 = e80_zn<D3>(tab + 3 * 49, zt, zs), z2 = e80_zn<D2>(tab + 2 * 49, zt, zs);
  const double z1 = e80_zn<D1>(tab + 49, zt, zs);
  zn0 = e80_zn<D0>(tab, zt, zs);
  return ((z3 * zh + z2) * zh + z1) * zh + zn0;
}
// FP32: the re-expanded table (in s' = zs - s0), Horner in s', zt, zh; skip00 leaves
// out the constant term of the surface part (the density's, added apart)
template <int D>
__device__ __forceinline__ float e80_q32(const float* __restrict__ C, float zt, float sp, bool skip00) {
  float acc = 0.f;
#pragma unroll
  for (int j = D; j >= 0; --j) {
    float h = 0.f;
#pragma unroll
    for (int i = D - j; i >= 0; --i) h = h * sp + ((skip00 && i == 0 && j == 0) ? 0.f : __ldg(C + i * 7 + j));
    acc = acc * zt + h;
  }
  return acc;
}
template <int D0, int D1, int D2, int D3>
__device__ __forceinline__ float e80_poly32(const float* __restrict__ tab, float zt, float sp, float zh,
                                            bool skip00, float& zn0) {
  const float z3 = e80_q32<D3>(tab + 3 * 49, zt, sp, false), z2 = e80_q32<D2>(tab + 2 * 49, zt, sp, false);
  const float z1 = e80_q32<D1>(tab + 49, zt, sp, false);
  zn0 = e80_q32<D0>(tab, zt, sp, skip00);
  return ((z3 * zh + z2) * zh + z1) * zh + zn0;
}

// eos_insitu, eos_insitu_pot and rab_3d with EOS-80 (eosbn2.F90:236-270, :400-436,
// :588-642) at point q (temperature qt, salinity qs)
template <class T>
__device__ __forceinline__ void eos80_point(const EosArgs<T>& a, long q, long qt, long qs, T ztm) {
  constexpr double r1_Z0 = 1.e-4, r1_T0 = 1.0 / 40.0, r1_S0 = 1.0 / 40.0, rdeltaS = 20.0;
  const T dep = a.what == 2 ? a.gdept[q] : a.pdep[q];
  if constexpr (sizeof(T) == 8) {
    const double zh = dep * r1_Z0, zt = a.pts[qt] * r1_T0;
    const double zs = sqrt(fabs(a.pts[qs] + rdeltaS) * r1_S0);
    double zn0;
    if (a.what == 2) {
      double zn = e80_poly<5, 3, 1, 0>(a.e80_raw + 196, zt, zs, zh, zn0);
      a.pab[qt] = zn * a.r1_rau0 * ztm;
      zn = e80_poly<5, 3, 1, 0>(a.e80_raw + 392, zt, zs, zh, zn0);
      a.pab[qs] = zn / zs * a.r1_rau0 * ztm;
    } else {
      const double zn = e80_poly<6, 4, 2, 1>(a.e80_raw, zt, zs, zh, zn0);
      if (a.what == 1) a.prhop[q] = zn0 * ztm;
      a.prd[q] = (zn * a.r1_rau0 - 1.0) * ztm;
    }
  } else {
    const float zh = dep * (float)r1_Z0, zt = a.pts[qt] * (float)r1_T0;
    const float x = fabsf(a.pts[qs] + (float)rdeltaS) * (float)r1_S0;
    const float zs = sqrtf(x);
    const float sp = (x - a.e80_s0 * a.e80_s0) / (zs + a.e80_s0);  // zs - s0 without cancellation
    float zn0;
    if (a.what == 2) {
      float zn = e80_poly32<5, 3, 1, 0>(a.e80_tay + 196, zt, sp, zh, false, zn0);
      a.pab[qt] = zn * a.r1_rau0 * ztm;
      zn = e80_poly32<5, 3, 1, 0>(a.e80_tay + 392, zt, sp, zh, false, zn0);
      a.pab[qs] = zn / zs * a.r1_rau0 * ztm;
    } else {
      // the anomaly of the density about its value at (35 psu, 0 degC, 0 m) first
      const float zn = e80_poly32<6, 4, 2, 1>(a.e80_tay, zt, sp, zh, true, zn0);
      if (a.what == 1) a.prhop[q] = (zn0 + a.e80_rho0) * ztm;
      a.prd[q] = ((zn + a.e80_anom) * a.r1_rau0) * ztm;
    }
  }
}

template <class T>
__device__ __forceinline__ T eos_rd_2d(const EosArgs<T>& a, T t, T sal, T dep) {
  if (a.eos80) {
    constexpr double r1_Z0 = 1.e-4, r1_T0 = 1.0 / 40.0, r1_S0 = 1.0 / 40.0, rdeltaS = 20.0;
    if constexpr (sizeof(T) == 8) {
      const double zh = dep * r1_Z0, zt = t * r1_T0, zs = sqrt(fabs(sal + rdeltaS) * r1_S0);
      double zn0;
      return e80_poly<6, 4, 2, 1>(a.e80_raw, zt, zs, zh, zn0) * a.r1_rau0 - 1.0;
    } else {
      const float zh = dep * (float)r1_Z0, zt = t * (float)r1_T0;
      const float x = fabsf(sal + (float)rdeltaS) * (float)r1_S0;
      const float zs = sqrtf(x);
      const float sp = (x - a.e80_s0 * a.e80_s0) / (zs + a.e80_s0);
      float zn0;
      return (e80_poly32<6, 4, 2, 1>(a.e80_tay, zt, sp, zh, true, zn0) + a.e80_anom) * a.r1_rau0;
    }
  }
  const T zt = t - T(10), zs = sal - T(35);
  const T zn = -a.a0 * (T(1) + T(0.5) * a.lambda1 * zt + a.mu1 * dep) * zt +
               a.b0 * (T(1) - T(0.5) * a.lambda2 * zs - a.mu2 * dep) * zs - a.nu * zt * zs;
  return zn * a.r1_rau0;
}

template <class T>
__global__ void k_eos(Dom<T> d, EosArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid || c.k > d.jpk - 1) return;
  const long q = (long)c.m * d.n3 + c.q;          // one 3-D field
  const long qt = 2 * (long)c.m * d.n3 + c.q;     // temperature of (jpi,jpj,jpk,2)
  const long qs = qt + d.n3;
  const ColInfo ci = d.ci[c.ij];
  if (a.eos80 && a.what != 3) {
    eos80_point(a, q, qt, qs, tmsk<T>(ci, c.k));
    return;
  }
  if (a.what == 3) {
    if (c.k < 2) return;
    const T zrw = (a.gdepw[q] - a.gdept[q]) / (a.gdept[q - d.n2] - a.gdept[q]);
    const T zaw = a.pab_in[qt] * (T(1) - zrw) + a.pab_in[qt - d.n2] * zrw;
    const T zbw = a.pab_in[qs] * (T(1) - zrw) + a.pab_in[qs - d.n2] * zrw;
    a.pn2[q] = a.grav * (zaw * (a.pts[qt - d.n2] - a.pts[qt]) - zbw * (a.pts[qs - d.n2] - a.pts[qs])) /
               d.e3w_n(c.ij, c.k, c.m) * wmsk<T>(ci, c.k);
    return;
  }
  const T zt = a.pts[qt] - T(10), zs = a.pts[qs] - T(35), ztm = tmsk<T>(ci, c.k);
  if (a.what == 2) {
    const T zh = a.gdept[q];
    T zn = a.a0 * (T(1) + a.lambda1 * zt + a.mu1 * zh) + a.nu * zs;
    a.pab[qt] = zn * a.r1_rau0 * ztm;
    zn = a.b0 * (T(1) - a.lambda2 * zs - a.mu2 * zh) - a.nu * zt;
    a.pab[qs] = zn * a.r1_rau0 * ztm;
    return;
  }
  const T zh = a.pdep[q];
  if (a.what == 0) {
    const T zn = -a.a0 * (T(1) + T(0.5) * a.lambda1 * zt + a.mu1 * zh) * zt +
                 a.b0 * (T(1) - T(0.5) * a.lambda2 * zs - a.mu2 * zh) * zs - a.nu * zt * zs;
    a.prd[q] = zn * a.r1_rau0 * ztm;
  } else {
    T zn = -a.a0 * (T(1) + T(0.5) * a.lambda1 * zt) * zt + a.b0 * (T(1) - T(0.5) * a.lambda2 * zs) * zs -
           a.nu * zt * zs;
    a.prhop[q] = (a.rau0 + zn) * ztm;
    zn = zn - (a.a0 * a.mu1 * zt + a.b0 * a.mu2 * zs) * zh;
    a.prd[q] = zn * a.r1_rau0 * ztm;
  }
}

// hpg_zco (dynhpg.F90:258-323), one interior column per thread: the pressure
// gradient integrated downwards from the surface in registers.
template <class T>
__global__ void k_hpg_zco(Dom<T> d, const T* __restrict__ rhd, T* ua, T* va, T zcoef0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i < 2 || i > d.jpi - 1 || j < 2 || j > d.jpj - 1) return;
  const int m = blockIdx.z;
  const long ij = (long)(i - 1) + (long)(j - 1) * d.jpi;
  const long c3 = (long)m * d.n3 + ij;
  const T r1u = d.r1_e1u[ij], r1v = d.r1_e2v[ij];
  T zcoef1 = zcoef0 * d.e3w_n(ij, 1, m);
  T zhpi = zcoef1 * (rhd[c3 + 1] - rhd[c3]) * r1u;
  T zhpj = zcoef1 * (rhd[c3 + d.jpi] - rhd[c3]) * r1v;
  ua[c3] = ua[c3] + zhpi;
  va[c3] = va[c3] + zhpj;
  for (int k = 2; k <= d.jpk - 1; ++k) {
    const long q = c3 + (long)(k - 1) * d.n2, qu = q - d.n2;
    zcoef1 = zcoef0 * d.e3w_n(ij, k, m);
    zhpi = zhpi + zcoef1 * ((rhd[q + 1] + rhd[qu + 1]) - (rhd[q] + rhd[qu])) * r1u;
    zhpj = zhpj + zcoef1 * ((rhd[q + d.jpi] + rhd[qu + d.jpi]) - (rhd[q] + rhd[qu])) * r1v;
    ua[q] = ua[q] + zhpi;
    va[q] = va[q] + zhpj;
  }
}

// zdf_mxl (zdfmxl.F90:59-141), one (i,j) column per thread: N^2 integrated
// downwards from nlb10 against the density criterion, the turbocline searched upwards
// from the bottom, then the depths of the two levels.
template <class T>
__global__ void k_zdf_mxl(Dom<T> d, MxlArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const int m = blockIdx.z;
  const long ij = (long)(i - 1) + (long)(j - 1) * d.jpi;
  const long c3 = (long)m * d.n3 + ij, c2 = (long)m * d.n2 + ij;
  const int ikt = d.mbkt[ij];
  const ColInfo ci = d.ci[ij];
  int nmln = a.nlb10;
  T h = T(0);
  for (int k = a.nlb10; k <= d.jpk - 1; ++k) {
    const T n2 = a.rn2b[c3 + (long)(k - 1) * d.n2];
    h = h + (n2 > T(0) ? n2 : T(0)) * d.e3w_n(ij, k, m);
    if (h < a.zn2_c) nmln = (k < ikt ? k : ikt) + 1;
  }
  const T ssm = d.ssmask[ij];
  if (a.hmld) {
    int imld = ikt + 1;
    for (int k = d.jpk - 1; k >= a.nlb10; --k)
      if (a.avt[c3 + (long)(k - 1) * d.n2] < a.avt_c * wmsk<T>(ci, k)) imld = k;
    a.hmld[c2] = a.gdepw[c3 + (long)(imld - 1) * d.n2] * ssm;
  }
  a.nmln[c2] = nmln;
  a.hmlp[c2] = a.gdepw[c3 + (long)(nmln - 1) * d.n2] * ssm;
  a.hmlpt[c2] = a.gdept[c3 + (long)(nmln - 2) * d.n2] * ssm;
}

// dyn_ldf_lap (dynldf_lap_blp.F90:37-104), linear free surface (e3*_b = e3*_n),
// one (i,j,k) point per thread: -curl(curl) + grad(div) of the before velocity.
// The relative vorticity zcur and divergence zdiv a point needs (three of each) are
// formed where read, each with the reference's expression.
template <class T>
struct LdfDyn {
  const Dom<T>& d;
  const T *ahmt, *ahmf, *pub, *pvb;
  long m3;
  int k, m;
  __device__ __forceinline__ long P(int i, int j) const { return (long)(i - 1) + (long)(j - 1) * d.jpi; }
  __device__ __forceinline__ T cur(int a, int b) const {
    const long p = P(a, b), q = m3 + p + (long)(k - 1) * d.n2;
    return a_(ahmf, q) * d.e3f_n(p, k, m) * d.r1_e1e2f[p] *
           (d.e2v[p + 1] * a_(pvb, q + 1) - d.e2v[p] * a_(pvb, q) - d.e1u[p + d.jpi] * a_(pub, q + d.jpi) +
            d.e1u[p] * a_(pub, q));
  }
  __device__ __forceinline__ T div(int a, int b) const {
    const long p = P(a, b), q = m3 + p + (long)(k - 1) * d.n2;
    return a_(ahmt, q) * d.r1_e1e2t[p] / d.e3t_b(p, k, m) *
           (d.e2u[p] * d.e3u_n(p, k, m) * a_(pub, q) - d.e2u[p - 1] * d.e3u_n(p - 1, k, m) * a_(pub, q - 1) +
            d.e1v[p] * d.e3v_n(p, k, m) * a_(pvb, q) - d.e1v[p - d.jpi] * d.e3v_n(p - d.jpi, k, m) * a_(pvb, q - d.jpi));
  }
  __device__ __forceinline__ static T a_(const T* x, long q) { return __ldg(x + q); }
};

template <class T>
__global__ void k_dyn_ldf_lap(Dom<T> d, const T* __restrict__ ahmt, const T* __restrict__ ahmf,
                              const T* __restrict__ pub, const T* __restrict__ pvb, T* pua, T* pva, T zsign) {
  const PtIdx c = pt_index(d);
  if (!c.valid || c.k > d.jpk - 1 || c.i < 2 || c.i > d.jpi - 1 || c.j < 2 || c.j > d.jpj - 1) return;
  const LdfDyn<T> L{d, ahmt, ahmf, pub, pvb, (long)c.m * d.n3, c.k, c.m};
  const int i = c.i, j = c.j;
  const long q = (long)c.m * d.n3 + c.q;
  const T zc = L.cur(i, j), zd = L.div(i, j);
  pua[q] = pua[q] + zsign * (-((zc - L.cur(i, j - 1)) * d.r1_e2u[c.ij] / d.e3u_n(c.ij, c.k, c.m)) +
                             (L.div(i + 1, j) - zd) * d.r1_e1u[c.ij]);
  pva[q] = pva[q] + zsign * ((zc - L.cur(i - 1, j)) * d.r1_e1v[c.ij] / d.e3v_n(c.ij, c.k, c.m) +
                             (L.div(i, j + 1) - zd) * d.r1_e2v[c.ij]);
}

// vor_ene (dynvor.F90:324-429), z-coordinate without ln_dynvor_msk, one (i,j,k)
// point per thread; the vorticities zwz and transports zwx, zwy of the four
// surrounding points are formed where read, each with the reference's expression.
template <class T>
__global__ void k_vor_ene(Dom<T> d, int kvor, const T* __restrict__ pun, const T* __restrict__ pvn, T* pua,
                          T* pva) {
  const PtIdx c = pt_index(d);
  if (!c.valid || c.k > d.jpk - 1 || c.i < 2 || c.i > d.jpi - 1 || c.j < 2 || c.j > d.jpj - 1) return;
  const long o = (long)c.m * d.n3 + (long)(c.k - 1) * d.n2;  // this level of this member
  const long J = d.jpi;
  auto zwz = [&](long p) -> T {
    if (kvor == 1) return d.ff_f[p];
    const T rv = (d.e2v[p + 1] * __ldg(pvn + o + p + 1) - d.e2v[p] * __ldg(pvn + o + p) -
                  d.e1u[p + J] * __ldg(pun + o + p + J) + d.e1u[p] * __ldg(pun + o + p)) *
                 d.r1_e1e2f[p];
    if (kvor == 2) return rv;
    return d.ff_f[p] + (d.e2v[p + 1] * __ldg(pvn + o + p + 1) - d.e2v[p] * __ldg(pvn + o + p) -
                        d.e1u[p + J] * __ldg(pun + o + p + J) + d.e1u[p] * __ldg(pun + o + p)) *
                           d.r1_e1e2f[p];
  };
  auto zwx = [&](long p) -> T { return d.e2u[p] * __ldg(pun + o + p); };
  auto zwy = [&](long p) -> T { return d.e1v[p] * __ldg(pvn + o + p); };
  const long p = c.ij, q = o + p;
  const T zy1 = zwy(p - J) + zwy(p + 1 - J);
  const T zy2 = zwy(p) + zwy(p + 1);
  const T zx1 = zwx(p - 1) + zwx(p - 1 + J);
  const T zx2 = zwx(p) + zwx(p + J);
  const T zc = zwz(p);
  pua[q] = pua[q] + T(0.25) * d.r1_e1u[p] * (zwz(p - J) * zy1 + zc * zy2);
  pva[q] = pva[q] - T(0.25) * d.r1_e2v[p] * (zwz(p - 1) * zx1 + zc * zx2);
}

// dyn_keg (dynkeg.F90, nkeg_C2), one (i,j,k) interior point per thread: the kinetic
// energy of the point and of its east / north neighbours formed where read.
template <class T>
__global__ void k_dyn_keg(Dom<T> d, const T* __restrict__ un, const T* __restrict__ vn, T* ua, T* va) {
  const PtIdx c = pt_index(d);
  if (!c.valid || c.k > d.jpk - 1 || c.i < 2 || c.i > d.jpi - 1 || c.j < 2 || c.j > d.jpj - 1) return;
  const long q = (long)c.m * d.n3 + c.q, J = d.jpi;
  auto hke = [&](long r) -> T {
    const T u0 = __ldg(un + r - 1), u1 = __ldg(un + r), v0 = __ldg(vn + r - J), v1 = __ldg(vn + r);
    const T zu = u0 * u0 + u1 * u1;
    const T zv = v0 * v0 + v1 * v1;
    return T(0.25) * (zv + zu);
  };
  const T h = hke(q);
  ua[q] = ua[q] - (hke(q + 1) - h) / d.e1u[c.ij];
  va[q] = va[q] - (hke(q + J) - h) / d.e2v[c.ij];
}

// dyn_zad (dynzad.F90), one interior column per thread: the w-level momentum fluxes
// of the column carried down, each formed once.
template <class T>
__global__ void k_dyn_zad(Dom<T> d, const T* __restrict__ un, const T* __restrict__ vn, const T* __restrict__ wn,
                          T* ua, T* va) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i < 2 || i > d.jpi - 1 || j < 2 || j > d.jpj - 1) return;
  const int m = blockIdx.z;
  const long ij = (long)(i - 1) + (long)(j - 1) * d.jpi, J = d.jpi;
  const long c3 = (long)m * d.n3 + ij;
  const T e0 = d.e1e2t[ij], e1 = d.e1e2t[ij + 1], e2 = d.e1e2t[ij + J];
  const T r1u = d.r1_e1e2u[ij], r1v = d.r1_e1e2v[ij];
  T wu = T(0), wv = T(0);  // zwuw, zwvw at the top of level k
  for (int k = 1; k <= d.jpk - 1; ++k) {
    const long q = c3 + (long)(k - 1) * d.n2;
    T wu1 = T(0), wv1 = T(0);  // at its bottom (w-level k+1), 0 at jpk
    if (k + 1 <= d.jpk - 1) {
      const long qb = q + d.n2;
      const T z0 = T(0.25) * e0 * __ldg(wn + qb), zi = T(0.25) * e1 * __ldg(wn + qb + 1),
              zj = T(0.25) * e2 * __ldg(wn + qb + J);
      wu1 = (zi + z0) * (__ldg(un + q) - __ldg(un + qb));
      wv1 = (zj + z0) * (__ldg(vn + q) - __ldg(vn + qb));
    }
    ua[q] = ua[q] - (wu + wu1) * r1u / d.e3u_n(ij, k, m);
    va[q] = va[q] - (wv + wv1) * r1v / d.e3v_n(ij, k, m);
    wu = wu1;
    wv = wv1;
  }
}

// ---------------------------------------------------------------- usrdef_sbc (GYRE)
// SIN and COS of the analytic forcing: FP64 by the evaluations the test oracle shares
// (nemo_sin.h), FP32 by the library
template <class T> __device__ __forceinline__ T usr_sin(T x);
template <class T> __device__ __forceinline__ T usr_cos(T x);
template <> __device__ __forceinline__ double usr_sin<double>(double x) { return nemo_sin(x); }
template <> __device__ __forceinline__ double usr_cos<double>(double x) { return nemo_cos(x); }
template <> __device__ __forceinline__ float usr_sin<float>(float x) { return sinf(x); }
template <> __device__ __forceinline__ float usr_cos<float>(float x) { return cosf(x); }

// The point part of usrdef_sbc_oce (usrdef_sbc.F90:113-135, :160-172), one (i,j) a
// thread: sbc's swap of the before fields, qsr, the restoring qns from the before SST,
// the raw E-P, the wind stress
template <class T>
__global__ void k_usr_sbc_a(Dom<T> d, UsrSbcArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const int m = blockIdx.z;
  const long ij = (long)(i - 1) + (long)(j - 1) * d.jpi, p = (long)m * d.n2 + ij;
  const long q = (long)m * 2 * d.n3 + ij;  // surface temperature of the member
  if (a.s[6] != 0.0) {
    if (a.utau_b) a.utau_b[p] = a.utau[p];
    if (a.vtau_b) a.vtau_b[p] = a.vtau[p];
    if (a.emp_b) a.emp_b[p] = a.emp[p];
  }
  const T rpi = T(3.141592653589793);
  const T g = a.gphit[p];
  const T t_star = T(a.s[0]) * usr_cos<T>(rpi * (g - T(5.)) / T(a.s[1]));
  const T qsr = T(230) * usr_cos<T>(T(3.1415) * (g - T(a.s[2])) / T(0.9 * 180));
  a.qsr[p] = qsr;
  a.qns[p] = T(-40.e0) * (a.tsb[q] - t_star) - qsr;
  T emp;
  if (g >= T(14.845) && T(37.2) >= g)
    emp = T(0.7) * T(3.16e-5) * usr_sin<T>(rpi / T(2) * (g - T(37.2)) / T(24.6 - 37.2)) * T(a.s[3]);
  else
    emp = -T(0.8) * T(3.16e-5) * usr_sin<T>(rpi / T(2) * (g - T(37.2)) / T(46.8 - 37.2)) * T(a.s[4]);
  a.emp[p] = emp;
  const T ztaun = T(a.s[5]);
  a.utau[p] = -ztaun * usr_sin<T>(rpi * (a.gphiu[p] - T(15.)) / T(29. - 15.));
  a.vtau[p] = ztaun * usr_sin<T>(rpi * (a.gphiv[p] - T(15.)) / T(29. - 15.));
}

// The rest (usrdef_sbc.F90:137-144, :176-186): E-P less its domain mean, sfx = 0, the
// heat content of E-P at the now SST in qns, the wind-stress modulus (interior; the
// closed lbc_lnk zeroes the edges)
template <class T>
__global__ void k_usr_sbc_b(Dom<T> d, UsrSbcArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const int m = blockIdx.z;
  const long ij = (long)(i - 1) + (long)(j - 1) * d.jpi, p = (long)m * d.n2 + ij;
  const long q = (long)m * 2 * d.n3 + ij;
  const double zsumemp = a.gsum[m] / a.zsurf;
  const T tm = tmsk<T>(d.ci[ij], 1);
  const T emp = (T)((double)a.emp[p] - zsumemp * (double)tm);
  a.emp[p] = emp;
  a.sfx[p] = T(0);
  a.qns[p] = a.qns[p] - emp * a.tsn[q] * T(a.rcp);
  T tau = T(0);
  if (i >= 2 && i <= d.jpi - 1 && j >= 2 && j <= d.jpj - 1) {
    const T ztx = a.utau[p - 1] + a.utau[p];
    const T zty = a.vtau[p - d.jpi] + a.vtau[p];
    tau = T(0.5) * sqrt(ztx * ztx + zty * zty);
  }
  a.taum[p] = tau;
}

// the step's scalars of the forcing into device memory (a launch outside any
// captured graph, so a replay reads the values of its own step)
__global__ void k_usr_put(double* dst, double s0, double s1, double s2, double s3, double s4, double s5,
                          double s6) {
  dst[0] = s0; dst[1] = s1; dst[2] = s2; dst[3] = s3; dst[4] = s4; dst[5] = s5; dst[6] = s6;
}

// ---------------------------------------------------------------- zdf_phy (TKE)
// SIN of the Langmuir-cell source: FP64 by the evaluation the test oracle shares
// (nemo_sin.h), FP32 by the library
__device__ __forceinline__ double lc_sin(double x) { return nemo_sin_0pi(x); }
__device__ __forceinline__ float lc_sin(float x) { return sinf(x); }

// 2 x the shear production at the uw-point (i+1/2, j, k) and the vw-point
// (i, j+1/2, k) of column ij (zdfsh2.F90:57-66) with the closure's avm_k. With a
// linear free surface e3uw_n = e3uw_b = the rest-state MIN of the neighbouring e3w.
template <class T>
__device__ __forceinline__ T zsh2_u(const Dom<T>& d, const ZphyArgs<T>& a, long m3, long ij, int k, int m) {
  const ColInfo c = d.ci[ij];
  const long q = m3 + ij + (long)(k - 1) * d.n2;
  const T e = fmn(d.e3w_n(ij, k, m), d.e3w_n(ij + 1, k, m));
  return (a.avm_k[q + 1] + a.avm_k[q]) * (a.un[q - d.n2] - a.un[q]) * (a.ub[q - d.n2] - a.ub[q]) / (e * e) *
         (umsk<T>(c, k) * umsk<T>(c, k - 1));
}
template <class T>
__device__ __forceinline__ T zsh2_v(const Dom<T>& d, const ZphyArgs<T>& a, long m3, long ij, int k, int m) {
  const ColInfo c = d.ci[ij];
  const long q = m3 + ij + (long)(k - 1) * d.n2;
  const T e = fmn(d.e3w_n(ij, k, m), d.e3w_n(ij + d.jpi, k, m));
  return (a.avm_k[q + d.jpi] + a.avm_k[q]) * (a.vn[q - d.n2] - a.vn[q]) * (a.vb[q - d.n2] - a.vb[q]) / (e * e) *
         (vmsk<T>(c, k) * vmsk<T>(c, k - 1));
}

// zdf_sh2 (zdfsh2.F90:67-74): the shear production at the interior w-points of
// levels 2..jpk-1, one point per thread; each of the four uw/vw terms it averages is
// formed where read (two threads form each).
template <class T>
__global__ void k_zdf_sh2(Dom<T> d, ZphyArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid || !c.interior || c.k < 2 || c.k > d.jpk - 1) return;
  const long m3 = (long)c.m * d.n3;
  const int k = c.k;
  const T u0 = zsh2_u(d, a, m3, c.ij - 1, k, c.m), u1 = zsh2_u(d, a, m3, c.ij, k, c.m);
  const T v0 = zsh2_v(d, a, m3, c.ij - d.jpi, k, c.m), v1 = zsh2_v(d, a, m3, c.ij, k, c.m);
  const ColInfo cw = d.ci[c.ij - 1], ch = d.ci[c.ij], cs = d.ci[c.ij - d.jpi];
  a.sh2[m3 + c.q] = T(0.25) * ((u0 + u1) * (T(2) - umsk<T>(cw, k) * umsk<T>(ch, k)) +
                               (v0 + v1) * (T(2) - vmsk<T>(cs, k) * vmsk<T>(ch, k)));
}

// The column part of zdf_phy, one water column per thread (its levels are coupled
// by the implicit TKE equation and the mixing-length limits):
//  tke_tke (zdftke.F90:168-440): surface value of en, Langmuir cells, the inverse
//    Prandtl number apdlr, the implicit system assembled and forward-eliminated in
//    one downward sweep, back-substituted upwards, the floor rn_emin;
//  tke_avn (:443-630): the buoyancy length sqrt(2 en / N^2), limited by nn_mxl in a
//    downward and an upward sweep, and on that upward sweep avm_k, avt_k, dissl, the
//    Prandtl correction of avt_k, then zdf_phy's avt, avm (zdfphy.F90:269-270),
//    zdf_evd (zdfevd.F90:76-109) and avs = avt (:284).
// Edge columns get the closed lbc_lnk of the five coefficients (zdfphy.F90:301-303).
// Each expression keeps the reference's association.
template <class T>
__global__ void k_zdf_tke(Dom<T> d, ZphyArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const int m = blockIdx.z, jpk = d.jpk;
  const long n2 = d.n2;
  const long ij = (long)(i - 1) + (long)(j - 1) * d.jpi;
  const long c3 = (long)m * d.n3 + ij, c2 = (long)m * d.n2 + ij;
  if (i == 1 || i == d.jpi || j == 1 || j == d.jpj) {
    for (int k = 1; k <= jpk; ++k) {
      const long q = c3 + (long)(k - 1) * n2;
      a.avm_k[q] = T(0); a.avt_k[q] = T(0); a.avm[q] = T(0); a.avt[q] = T(0);
      if (a.avs) a.avs[q] = T(0);
    }
    return;
  }
  const ColInfo ci = d.ci[ij];
  const T tm1 = tmsk<T>(ci, 1);
  const T taum = a.taum[c2];
  const T en1 = fmx(a.rn_emin0, a.zbbrau * taum) * tm1;  // surface boundary condition
  a.en[c3] = en1;
  // Langmuir cells: the depth zhlc of the first w-level whose cumulated potential
  // energy exceeds the Stokes-drift scale, and the source amplitude zfr
  T zhlc = T(1), zfr = T(0);
  if (a.ln_lc) {
    const T zus = a.lc_cof1 * taum;
    T zpelc = fmx(a.rn2b[c3], T(0)) * a.gdepw[c3] * d.e3w_n(ij, 1, m);
    int imlc = d.mbkt[ij] + 1;
    for (int k = 2; k <= jpk - 1; ++k) {
      const long q = c3 + (long)(k - 1) * n2;
      zpelc = zpelc + fmx(a.rn2b[q], T(0)) * a.gdepw[q] * d.e3w_n(ij, k, m);
      if (zpelc > zus) { imlc = k; break; }
    }
    zhlc = a.gdepw[c3 + (long)(imlc - 1) * n2];
    const T zs = a.lc_cof2 * sqrt(taum);
    zfr = (T(1) - T(4) * (a.fr_i ? a.fr_i[c2] : T(0))) * zs * zs * zs * tm1;
    if (zfr < T(0)) zfr = T(0);
  }
  // downward sweep: right-hand side, matrix, forward elimination
  T dg_p = T(1), up_p = T(0), lw_p = T(0);
  T avm_km1 = a.avm_k[c3];
  for (int k = 2; k <= jpk - 1; ++k) {
    const long q = c3 + (long)(k - 1) * n2;
    const T wm = wmsk<T>(ci, k), tm = tmsk<T>(ci, k);
    T en = a.en[q];
    if (zfr != T(0)) {
      const T dep = a.gdepw[q];
      if (dep - zhlc < T(0) && wm != T(0)) {
        const T zwlc = a.rn_lc * lc_sin(a.rpi * dep / zhlc);
        en = en + a.rdt * zfr * (zwlc * zwlc * zwlc) / zhlc;
      }
    }
    const T avm_k = a.avm_k[q], avm_kp1 = a.avm_k[q + n2];
    const T sh2 = a.sh2[q], dissl = a.dissl[q], rn2 = a.rn2[q];
    if (a.nn_pdl == 1) {
      const T zri = fmx(a.rn2b[q], T(0)) * avm_k / (sh2 + a.rn_bshear);
      a.apdlr[q] = fmx(T(0.1), a.ri_cri / fmx(a.ri_cri, zri));
    }
    const T zcof = a.zfact1 * tm;
    const T e3w = d.e3w_n(ij, k, m);
    const T up = zcof * fmx(avm_kp1 + avm_k, T(2.e-5)) / (d.e3t_n(ij, k, m) * e3w);
    const T lw = zcof * fmx(avm_k + avm_km1, T(2.e-5)) / (d.e3t_n(ij, k - 1, m) * e3w);
    T dg = T(1) - lw - up + a.zfact2 * dissl * wm;
    const T rhs = en + a.rdt * (sh2 - a.avt_k[q] * rn2 + a.zfact3 * dissl * en) * wm;
    T lf;
    if (k == 2) {
      lf = rhs - lw * en1;
    } else {
      dg = dg - lw * up_p / dg_p;
      lf = rhs - lw / dg_p * lw_p;
    }
    a.zdiag[q] = dg; a.zd_up[q] = up; a.zd_lw[q] = lf;
    dg_p = dg; up_p = up; lw_p = lf;
    avm_km1 = avm_k;
  }
  // upward sweep: back substitution, the floor, and the buoyancy length (into zdiag)
  T en_p = T(0);
  for (int k = jpk - 1; k >= 2; --k) {
    const long q = c3 + (long)(k - 1) * n2;
    const T en = (k == jpk - 1) ? a.zd_lw[q] / a.zdiag[q] : (a.zd_lw[q] - a.zd_up[q] * en_p) / a.zdiag[q];
    en_p = en;
    const T e = fmx(en, a.rn_emin) * wmsk<T>(ci, k);
    a.en[q] = e;
    a.zdiag[q] = fmx(a.rmxl_min, sqrt(T(2) * e / fmx(a.rn2[q], a.rsmall)));
  }
  T* zmxlm = a.zdiag;
  T* zmxld = a.zd_up;
  const T mxl1 = a.ln_mxl0 ? fmx(a.rn_mxl0, a.zraug * taum * tm1) : a.rn_mxl0;
  // downward limits of nn_mxl = 2 (zmxlm) and 3 (zmxld, from the unlimited zmxlm)
  if (a.nn_mxl == 2) {
    T p = mxl1;
    for (int k = 2; k <= jpk - 1; ++k) {
      const long q = c3 + (long)(k - 1) * n2;
      p = fmn(p + d.e3t_n(ij, k - 1, m), zmxlm[q]);
      zmxlm[q] = p;
    }
  } else if (a.nn_mxl == 3) {
    T p = mxl1;
    for (int k = 2; k <= jpk - 1; ++k) {
      const long q = c3 + (long)(k - 1) * n2;
      p = fmn(p + d.e3t_n(ij, k - 1, m), zmxlm[q]);
      zmxld[q] = p;
    }
  }
  // upward sweep: the limited lengths, the coefficients, the ocean Kz
  const T evd = a.rn_evd;
  T nxt = a.rmxl_min;  // zmxlm(jpk)
  for (int k = jpk - 1; k >= 2; --k) {
    const long q = c3 + (long)(k - 1) * n2;
    const T wm = wmsk<T>(ci, k), tm = tmsk<T>(ci, k);
    const T raw = zmxlm[q];
    T lm, ld;
    if (a.nn_mxl == 2) {
      lm = fmn(nxt + d.e3t_n(ij, k + 1, m), raw);
      ld = lm;
      nxt = lm;
    } else if (a.nn_mxl == 3) {
      const T dn = fmn(nxt + d.e3t_n(ij, k + 1, m), raw);
      nxt = dn;
      const T lu = zmxld[q];
      lm = fmn(lu, dn);
      ld = sqrt(lu * dn);
    } else if (a.nn_mxl == 1) {
      lm = fmn(d.e3w_n(ij, k, m), raw);
      ld = lm;
    } else {  // 0: bounded by the distances to the surface (mikt = 1) and the bottom
      const T dep = a.gdepw[q], e3w = d.e3w_n(ij, k, m);
      const T z = fmn(fmn(dep - a.gdepw[c3], raw), a.gdepw[c3 + (long)d.mbkt[ij] * n2] - dep);
      lm = z * wm + fmn(raw, e3w) * (T(1) - wm);
      ld = z * wm + fmn(lm, e3w) * (T(1) - wm);
    }
    const T zsqen = sqrt(a.en[q]);
    const T zav = a.rn_ediff * lm * zsqen;
    const T avmk = fmx(zav, a.rn_avm0) * wm;
    T avtk = fmx(zav, a.rn_avt0) * wm;
    a.dissl[q] = zsqen / ld;
    if (a.nn_pdl == 1) avtk = fmx(a.apdlr[q] * avtk, a.rn_avt0) * tm;
    a.avm_k[q] = avmk;
    a.avt_k[q] = avtk;
    T avt = avtk, avm = avmk;
    if (a.ln_zdfevd && fmn(a.rn2[q], a.rn2b[q]) <= T(-1.e-12)) {
      avt = evd * wm;
      if (a.nn_evdm == 1) avm = evd * wm;
    }
    a.avt[q] = avt;
    a.avm[q] = avm;
    if (a.avs) a.avs[q] = avt;
  }
  // the surface level: coefficients from en(1) and the surface length; avt, avm
  // keep their values there unless zdf_evd acts
  {
    const T wm = tm1;
    const T zsqen = sqrt(en1);
    const T zav = a.rn_ediff * mxl1 * zsqen;
    a.avm_k[c3] = fmx(zav, a.rn_avm0) * wm;
    a.avt_k[c3] = fmx(zav, a.rn_avt0) * wm;
    a.dissl[c3] = zsqen / mxl1;
    T avt = a.avt[c3];
    if (a.ln_zdfevd && fmn(a.rn2[c3], a.rn2b[c3]) <= T(-1.e-12)) {
      avt = evd * wm;
      a.avt[c3] = avt;
      if (a.nn_evdm == 1) a.avm[c3] = evd * wm;
    }
    if (a.avs) a.avs[c3] = avt;
  }
}

}  // namespace nemo
