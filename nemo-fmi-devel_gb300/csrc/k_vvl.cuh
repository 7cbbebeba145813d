// k_vvl.cuh -- z* time stepping of a variable-volume (ln_linssh = .false.) model:
// the after scale factors (dom_vvl_sf_nxt), the thickness-weighted Asselin filter of
// the tracers (tra_nxt_vvl), the filter of the before scale factors and velocities
// (dyn_nxt), the forcing removed from the filtered before ssh (ssh_swp) and the swap
// with the depths of the next step (dom_vvl_sf_swp).
//
// One (i,j) water column per thread, marching down k; the tracer filter one point per
// thread. The rest-state scale factors come from the context's domain (the e3 fields
// of a Dom built without the bound time-varying ones); the time-varying fields are
// the bound arrays, member-strided by n3 (n2 for the 2-D ones). Every kernel writes
// only its own column (point), so a kernel that reads a neighbour's value reads a
// field that no thread of the same launch writes.
#pragma once
#include "k_tra.cuh"

namespace nemo {

template <class T>
struct VvlArgs {
  const double* ssha;                      // after ssh of dyn_spg_ts (FP64)
  const T *sshb, *sshn;
  const T *emp, *emp_b, *rnf, *rnf_b;      // forcing; rnf, rnf_b may be null
  T *e3t_b, *e3t_n, *e3t_a;
  T *e3u_n, *e3v_n, *e3u_a, *e3v_a, *e3u_b, *e3v_b;
  T *e3w_n, *e3f_n, *e3w_b, *e3uw_n, *e3vw_n, *e3uw_b, *e3vw_b;  // outputs of the swap; null = not formed
  const T *e3uw_0, *e3vw_0;
  T *hu_a, *hv_a, *r1_hu_a, *r1_hv_a;
  T *hu_n, *hv_n, *r1_hu_n, *r1_hv_n, *ht_n;
  T *hu_b, *hv_b, *r1_hu_b, *r1_hv_b;
  T *gdept_n, *gdepw_n, *gde3w_n, *gdept_b, *gdepw_b;
  // dyn_nxt
  T *ua, *va, *un, *vn, *ub, *vb;
  T *un_b, *vn_b, *ub_b, *vb_b;
  const double *ua_b, *va_b;
  // tra_nxt_vvl
  T *tsb, *tsn, *tsa;
  const T *tsc, *tsc_b, *qsr_hc, *qsr_hc_b;
  T atfp, zfact1, zfact2;                  // zfact1 = atfp rdt, zfact2 = zfact1 / rau0
  int euler, vec, traqsr, nksr;
};

// ------------------------------------------------------------ dom_vvl_interpol
// domvvl.F90:678-782 with zlnwd = 0. Horizontal cases at (i,j,k) of member m; the
// value of a point that lbc_lnk closes (i = 1, jpi or j = 1, jpj for U and V; i = jpi
// or j = jpj for F) is the rest state.
template <class T>
__device__ __forceinline__ T vvl_to_u(const Dom<T>& d, const T* pe3, const ColInfo& ci, int i, int j, long ij,
                                      int k, long mo) {
  T x = T(0);
  if (i >= 2 && i <= d.jpi - 1 && j >= 2 && j <= d.jpj - 1) {
    const long q = mo + ij + (long)(k - 1) * d.n2;
    x = T(0.5) * umsk<T>(ci, k) * d.r1_e1e2u[ij] *
        (d.e1e2t[ij] * (pe3[q] - d.e3t_n(ij, k, 0)) + d.e1e2t[ij + 1] * (pe3[q + 1] - d.e3t_n(ij + 1, k, 0)));
  }
  return x + d.e3u_n(ij, k, 0);
}
template <class T>
__device__ __forceinline__ T vvl_to_v(const Dom<T>& d, const T* pe3, const ColInfo& ci, int i, int j, long ij,
                                      int k, long mo) {
  T x = T(0);
  if (i >= 2 && i <= d.jpi - 1 && j >= 2 && j <= d.jpj - 1) {
    const long q = mo + ij + (long)(k - 1) * d.n2, nb = d.jpi;
    x = T(0.5) * vmsk<T>(ci, k) * d.r1_e1e2v[ij] *
        (d.e1e2t[ij] * (pe3[q] - d.e3t_n(ij, k, 0)) + d.e1e2t[ij + nb] * (pe3[q + nb] - d.e3t_n(ij + nb, k, 0)));
  }
  return x + d.e3v_n(ij, k, 0);
}
// 'F' from the u-point field pe3
template <class T>
__device__ __forceinline__ T vvl_to_f(const Dom<T>& d, const T* pe3, const ColInfo& ci, const ColInfo& cn, int i,
                                      int j, long ij, int k, long mo) {
  T x = T(0);
  if (i <= d.jpi - 1 && j <= d.jpj - 1) {
    const long q = mo + ij + (long)(k - 1) * d.n2, nb = d.jpi;
    x = T(0.5) * (umsk<T>(ci, k) * umsk<T>(cn, k)) * d.r1_e1e2f[ij] *
        (d.e1e2u[ij] * (pe3[q] - d.e3u_n(ij, k, 0)) + d.e1e2u[ij + nb] * (pe3[q + nb] - d.e3u_n(ij + nb, k, 0)));
  }
  return x + d.e3f_n(ij, k, 0);
}
// the vertical cases 'W', 'UW', 'VW' for one column: out(k) from in(k-1), in(k), the
// rest states in0 (at the in points) and out0, and the mask of the in points
template <class T, class In0, class Out0, class Msk>
__device__ __forceinline__ void vvl_to_w(const Dom<T>& d, const T* in, T* out, long o, In0 in0, Out0 out0, Msk msk) {
  const long n2 = d.n2;
  T dm = in[o] - in0(1);
  out[o] = out0(1) + in[o] - in0(1);
  for (int k = 2; k <= d.jpk; ++k) {
    const long q = o + (long)(k - 1) * n2;
    const T m = msk(k);
    const T dk = in[q] - in0(k);
    out[q] = out0(k) + (T(1) - T(0.5) * m) * dm + T(0.5) * m * dk;
    dm = dk;
  }
}

// h = sum over levels 1..jpkm1 of e3 mask, in level order (domvvl.F90:549-556)
template <class T, class Msk>
__device__ __forceinline__ T vvl_colsum(const Dom<T>& d, const T* e3, long o, Msk msk) {
  T h = e3[o] * msk(1);
  for (int k = 2; k <= d.jpk - 1; ++k) h = h + e3[o + (long)(k - 1) * d.n2] * msk(k);
  return h;
}

// ------------------------------------------------------------- dom_vvl_sf_nxt
// (domvvl.F90:323-327) e3t_a on levels 1..jpkm1 of every column
template <class T>
__global__ void k_vvl_sf_nxt_t(Dom<T> d, VvlArgs<T> a) {
  const ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const long p = (long)c.m * d.n2 + c.ij, o = (long)c.m * d.n3 + c.ij;
  const ColInfo ci = d.ci[c.ij];
  const T ssm = d.ssmask[c.ij];
  const T z_scale = (T(a.ssha[p]) - a.sshb[p]) * ssm / (d.ht_0[c.ij] + a.sshn[p] + T(1) - ssm);
  for (int k = 1; k <= d.jpk - 1; ++k) {
    const long q = o + (long)(k - 1) * d.n2;
    a.e3t_a[q] = a.e3t_b[q] + a.e3t_n[q] * z_scale * tmsk<T>(ci, k);
  }
}

// (domvvl.F90:542-558) e3u_a, e3v_a on every level, hu_a, hv_a and their inverses
template <class T>
__global__ void k_vvl_sf_nxt_uv(Dom<T> d, VvlArgs<T> a) {
  const ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const long p = (long)c.m * d.n2 + c.ij, mo = (long)c.m * d.n3, o = mo + c.ij;
  const ColInfo ci = d.ci[c.ij];
  for (int k = 1; k <= d.jpk; ++k) {
    const long q = o + (long)(k - 1) * d.n2;
    a.e3u_a[q] = vvl_to_u(d, a.e3t_a, ci, c.i, c.j, c.ij, k, mo);
    a.e3v_a[q] = vvl_to_v(d, a.e3t_a, ci, c.i, c.j, c.ij, k, mo);
  }
  const T hu = vvl_colsum(d, a.e3u_a, o, [&](int k) { return umsk<T>(ci, k); });
  const T hv = vvl_colsum(d, a.e3v_a, o, [&](int k) { return vmsk<T>(ci, k); });
  const T su = d.ssumask[c.ij], sv = d.ssvmask[c.ij];
  a.hu_a[p] = hu;
  a.hv_a[p] = hv;
  a.r1_hu_a[p] = su / (hu + T(1) - su);
  a.r1_hv_a[p] = sv / (hv + T(1) - sv);
}

// ----------------------------------------------------------------- tra_nxt_vvl
// tranxt.F90:109 (lbc of tsa), then the Euler swap or tra_nxt_vvl (:240-380) on the
// interior, then the lbc of tsb and tsn; one point per thread as k_tra_nxt.
template <class T>
__global__ void k_tra_nxt_vvl(Dom<T> d, VvlArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const bool edge = !c.interior;
  const long ij = c.q % d.n2;
  const long p = (long)c.m * d.n2 + ij, q3 = (long)c.m * d.n3 + c.q;
  for (int n = 0; n < 2; ++n) {
    const long o = ((long)c.m * 2 + n) * d.n3 + c.q;
    if (edge) a.tsa[o] = T(0);
    if (a.euler) {
      if (c.k <= d.jpk - 1) a.tsn[o] = a.tsa[o];
    } else if (edge) {
      a.tsb[o] = T(0);
      a.tsn[o] = T(0);
    } else if (c.k <= d.jpk - 1) {
      const T e3b = a.e3t_b[q3], e3n = a.e3t_n[q3], e3a = a.e3t_a[q3];
      const T tcb = a.tsb[o] * e3b, tcn = a.tsn[o] * e3n, tca = a.tsa[o] * e3a;
      // FP32: the time laplacians from the two differences (see k_tra_nxt)
      const T e3d = sizeof(T) == 4 ? (e3a - e3n) - (e3n - e3b) : e3a - T(2) * e3n + e3b;
      const T tcd = sizeof(T) == 4 ? (tca - tcn) - (tcn - tcb) : tca - T(2) * tcn + tcb;
      T e3f = e3n + a.atfp * e3d;
      T tcf = tcn + a.atfp * tcd;
      if (c.k == 1) {  // mikt = 1 without ice-shelf cavities (:314-329)
        const long s = ((long)c.m * 2 + n) * d.n2 + ij;
        e3f = e3f - a.zfact2 * (a.emp_b[p] - a.emp[p]);
        tcf = tcf - a.zfact1 * (a.tsc[s] - a.tsc_b[s]);
        if (a.rnf) e3f = e3f - a.zfact2 * (-(a.rnf_b[p] - a.rnf[p]));
      }
      if (a.traqsr && n == 0 && c.k <= a.nksr) tcf = tcf - a.zfact1 * (a.qsr_hc[q3] - a.qsr_hc_b[q3]);  // :333-334
      e3f = T(1) / e3f;
      a.tsb[o] = tcf * e3f;
      a.tsn[o] = a.tsa[o];
    }
  }
}

// --------------------------------------------------------------------- dyn_nxt
// (dynnxt.F90:114-126, :146) the barotropic part of the after velocity replaced by
// the sub-steps' ua_b with the after scale factors, lbc of ua, va; then (:217-226)
// the filter of e3t_b with the forcing removed at the first level, or at the Euler
// step the now scale factors and velocities set to the after ones (:168-186).
template <class T>
__global__ void k_dyn_nxt_vvl_a(Dom<T> d, VvlArgs<T> a) {
  const ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const int jpk = d.jpk;
  const long n2 = d.n2, p = (long)c.m * n2 + c.ij, o = (long)c.m * d.n3 + c.ij;
  const ColInfo ci = d.ci[c.ij];
  const T r1u = a.r1_hu_a[p], r1v = a.r1_hv_a[p];
  const T uab = T(a.ua_b[p]), vab = T(a.va_b[p]);
  T zue = T(0), zve = T(0);
  for (int k = 1; k <= jpk - 1; ++k) {
    const long q = o + (long)(k - 1) * n2;
    zue = zue + a.e3u_a[q] * a.ua[q] * umsk<T>(ci, k);
    zve = zve + a.e3v_a[q] * a.va[q] * vmsk<T>(ci, k);
  }
  for (int k = 1; k <= jpk; ++k) {
    const long q = o + (long)(k - 1) * n2;
    if (!c.interior) {
      a.ua[q] = T(0);
      a.va[q] = T(0);
    } else if (k <= jpk - 1) {
      a.ua[q] = (a.ua[q] - zue * r1u + uab) * umsk<T>(ci, k);
      a.va[q] = (a.va[q] - zve * r1v + vab) * vmsk<T>(ci, k);
    }
  }
  if (a.euler) {
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = o + (long)(k - 1) * n2;
      a.un[q] = a.ua[q];
      a.vn[q] = a.va[q];
      a.e3t_n[q] = a.e3t_a[q];
      a.e3u_n[q] = a.e3u_a[q];
      a.e3v_n[q] = a.e3v_a[q];
    }
  } else {
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = o + (long)(k - 1) * n2;
      const T eb = a.e3t_b[q], en = a.e3t_n[q], ea = a.e3t_a[q];
      a.e3t_b[q] = en + a.atfp * (sizeof(T) == 4 ? (ea - en) - (en - eb) : eb - T(2) * en + ea);
    }
    // zfact2 = atfp rdt / rau0 is dyn_nxt's zcoef
    a.e3t_b[o] = a.e3t_b[o] - a.zfact2 * (a.emp_b[p] - a.emp[p]) * tmsk<T>(ci, 1);
  }
}

// (dynnxt.F90:260-358) e3u_b, e3v_b from the filtered e3t_b, the Asselin filter on
// the velocity (ln_dynadv_vec) or on the thickness-weighted velocity, the before
// velocity returned to the time-split estimate (:312-324), hu_b, hv_b and their
// inverses (:334-343), the now and before barotropic velocities (:345-358).
template <class T>
__global__ void k_dyn_nxt_vvl_b(Dom<T> d, VvlArgs<T> a) {
  const ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const int jpk = d.jpk;
  const long n2 = d.n2, p = (long)c.m * n2 + c.ij, mo = (long)c.m * d.n3, o = mo + c.ij;
  const ColInfo ci = d.ci[c.ij];
  if (!a.euler) {
    T sb = T(0), tb = T(0);
    for (int k = 1; k <= jpk; ++k) {
      const long q = o + (long)(k - 1) * n2;
      const T fu = vvl_to_u(d, a.e3t_b, ci, c.i, c.j, c.ij, k, mo);
      const T fv = vvl_to_v(d, a.e3t_b, ci, c.i, c.j, c.ij, k, mo);
      if (k == jpk) {  // the level below the last: e3 only (vector form)
        if (a.vec) {
          a.e3u_b[q] = fu;
          a.e3v_b[q] = fv;
        }
        break;
      }
      const T ua = a.ua[q], va = a.va[q], un = a.un[q], vn = a.vn[q], ub = a.ub[q], vb = a.vb[q];
      T zuf, zvf;
      if (a.vec) {
        zuf = un + a.atfp * (sizeof(T) == 4 ? (ua - un) - (un - ub) : ub - T(2) * un + ua);
        zvf = vn + a.atfp * (sizeof(T) == 4 ? (va - vn) - (vn - vb) : vb - T(2) * vn + va);
      } else {
        const T zua = a.e3u_a[q] * ua, zva = a.e3v_a[q] * va;
        const T zun = a.e3u_n[q] * un, zvn = a.e3v_n[q] * vn;
        const T zub = a.e3u_b[q] * ub, zvb = a.e3v_b[q] * vb;
        zuf = (zun + a.atfp * (sizeof(T) == 4 ? (zua - zun) - (zun - zub) : zub - T(2) * zun + zua)) / fu;
        zvf = (zvn + a.atfp * (sizeof(T) == 4 ? (zva - zvn) - (zvn - zvb) : zvb - T(2) * zvn + zva)) / fv;
      }
      a.e3u_b[q] = fu;
      a.e3v_b[q] = fv;
      a.ub[q] = zuf;
      a.vb[q] = zvf;
      a.un[q] = ua;
      a.vn[q] = va;
      sb = sb + fu * zuf * umsk<T>(ci, k);
      tb = tb + fv * zvf * vmsk<T>(ci, k);
    }
    const T r1u = a.r1_hu_n[p], r1v = a.r1_hv_n[p], unb = a.un_b[p], vnb = a.vn_b[p];
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = o + (long)(k - 1) * n2;
      a.ub[q] = a.ub[q] - (sb * r1u - unb) * umsk<T>(ci, k);
      a.vb[q] = a.vb[q] - (tb * r1v - vnb) * vmsk<T>(ci, k);
    }
  }
  auto um = [&](int k) { return umsk<T>(ci, k); };
  auto vm = [&](int k) { return vmsk<T>(ci, k); };
  const T hub = vvl_colsum(d, a.e3u_b, o, um), hvb = vvl_colsum(d, a.e3v_b, o, vm);
  const T su = d.ssumask[c.ij], sv = d.ssvmask[c.ij];
  const T r1ub = su / (hub + T(1) - su), r1vb = sv / (hvb + T(1) - sv);
  a.hu_b[p] = hub;
  a.hv_b[p] = hvb;
  a.r1_hu_b[p] = r1ub;
  a.r1_hv_b[p] = r1vb;
  T sun = T(0), sub = T(0), svn = T(0), svb = T(0);
  for (int k = 1; k <= jpk - 1; ++k) {
    const long q = o + (long)(k - 1) * n2;
    sun = sun + a.e3u_a[q] * a.un[q] * um(k);
    sub = sub + a.e3u_b[q] * a.ub[q] * um(k);
    svn = svn + a.e3v_a[q] * a.vn[q] * vm(k);
    svb = svb + a.e3v_b[q] * a.vb[q] * vm(k);
  }
  a.un_b[p] = sun * a.r1_hu_a[p];
  a.vn_b[p] = svn * a.r1_hv_a[p];
  a.ub_b[p] = sub * r1ub;
  a.vb_b[p] = svb * r1vb;
}

// --------------------------------------------------------------------- ssh_swp
// sshwzv.F90:243-262 with the forcing removed from the filtered before ssh
template <class T>
__global__ void k_ssh_swp_vvl(Dom<T> d, VvlArgs<T> a, T* sshb, T* sshn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.jpi || j > d.jpj) return;
  const long ij = (long)(i - 1) + (long)(j - 1) * d.jpi, p = (long)blockIdx.z * d.n2 + ij;
  const T sa = T(a.ssha[p]);
  if (!a.euler) {
    const T sn = sshn[p], sb = sshb[p];
    T b = sn + a.atfp * (sizeof(T) == 4 ? (sa - sn) - (sn - sb) : sb - T(2) * sn + sa);
    T zf = a.emp_b[p] - a.emp[p];
    if (a.rnf) zf = zf - a.rnf_b[p] + a.rnf[p];
    sshb[p] = b - a.zfact2 * zf * d.ssmask[ij];
  }
  sshn[p] = sa;
}

// ------------------------------------------------------------- dom_vvl_sf_swp
// domvvl.F90:617-667 for one column: the before depths, the swap of e3t, e3u, e3v,
// e3f_n from the neighbouring e3u_a (= the new e3u_n), the vertical interpolations,
// the now depths (gde3w with the swapped sshn) and the column depths.
template <class T>
__global__ void k_vvl_sf_swp(Dom<T> d, VvlArgs<T> a) {
  const ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const int jpk = d.jpk;
  const long n2 = d.n2, p = (long)c.m * n2 + c.ij, mo = (long)c.m * d.n3, o = mo + c.ij;
  const ColInfo ci = d.ci[c.ij];
  if (a.gdept_b && a.gdept_n)
    for (int k = 1; k <= jpk; ++k) a.gdept_b[o + (long)(k - 1) * n2] = a.gdept_n[o + (long)(k - 1) * n2];
  if (a.gdepw_b && a.gdepw_n)
    for (int k = 1; k <= jpk; ++k) a.gdepw_b[o + (long)(k - 1) * n2] = a.gdepw_n[o + (long)(k - 1) * n2];
  const ColInfo cn = d.ci[c.j < d.jpj ? c.ij + d.jpi : c.ij];
  for (int k = 1; k <= jpk; ++k) {
    const long q = o + (long)(k - 1) * n2;
    a.e3t_n[q] = a.e3t_a[q];
    a.e3u_n[q] = a.e3u_a[q];
    a.e3v_n[q] = a.e3v_a[q];
    if (a.e3f_n) a.e3f_n[q] = vvl_to_f(d, a.e3u_a, ci, cn, c.i, c.j, c.ij, k, mo);
  }
  const long ij = c.ij;
  vvl_to_w(d, a.e3t_n, a.e3w_n, o, [&](int k) { return d.e3t_n(ij, k, 0); }, [&](int k) { return d.e3w_n(ij, k, 0); },
           [&](int k) { return tmsk<T>(ci, k); });
  if (a.e3w_b)
    vvl_to_w(d, a.e3t_b, a.e3w_b, o, [&](int k) { return d.e3t_n(ij, k, 0); },
             [&](int k) { return d.e3w_n(ij, k, 0); }, [&](int k) { return tmsk<T>(ci, k); });
  auto uw0 = [&](int k) { return a.e3uw_0[o + (long)(k - 1) * n2]; };
  auto vw0 = [&](int k) { return a.e3vw_0[o + (long)(k - 1) * n2]; };
  auto u0 = [&](int k) { return d.e3u_n(ij, k, 0); };
  auto v0 = [&](int k) { return d.e3v_n(ij, k, 0); };
  auto um = [&](int k) { return umsk<T>(ci, k); };
  auto vm = [&](int k) { return vmsk<T>(ci, k); };
  if (a.e3uw_n) vvl_to_w(d, a.e3u_n, a.e3uw_n, o, u0, uw0, um);
  if (a.e3vw_n) vvl_to_w(d, a.e3v_n, a.e3vw_n, o, v0, vw0, vm);
  if (a.e3uw_b) vvl_to_w(d, a.e3u_b, a.e3uw_b, o, u0, uw0, um);
  if (a.e3vw_b) vvl_to_w(d, a.e3v_b, a.e3vw_b, o, v0, vw0, vm);
  if (a.gdept_n && a.gdepw_n) {
    const T sn = a.sshn[p];
    T gt = T(0.5) * a.e3w_n[o], gw = T(0);
    a.gdept_n[o] = gt;
    a.gdepw_n[o] = gw;
    if (a.gde3w_n) a.gde3w_n[o] = gt - sn;
    for (int k = 2; k <= jpk; ++k) {
      const long q = o + (long)(k - 1) * n2;
      const T zcoef = tmsk<T>(ci, k) - wmsk<T>(ci, k);
      gw = gw + a.e3t_n[q - n2];
      gt = zcoef * (gw + T(0.5) * a.e3w_n[q]) + (T(1) - zcoef) * (gt + a.e3w_n[q]);
      a.gdepw_n[q] = gw;
      a.gdept_n[q] = gt;
      if (a.gde3w_n) a.gde3w_n[q] = gt - sn;
    }
  }
  a.hu_n[p] = a.hu_a[p];
  a.r1_hu_n[p] = a.r1_hu_a[p];
  a.hv_n[p] = a.hv_a[p];
  a.r1_hv_n[p] = a.r1_hv_a[p];
  a.ht_n[p] = vvl_colsum(d, a.e3t_n, o, [&](int k) { return tmsk<T>(ci, k); });
}

}  // namespace nemo
