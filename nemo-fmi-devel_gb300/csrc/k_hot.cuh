// k_hot.cuh -- the tracer kernels specialised for the configuration of the hot path:
// horizontally uniform e3 (1-D profiles), constant eddy diffusivity (aht0 * mask),
// no partial steps, standard iso-neutral operator (akz = ah_wslp2), laplacian,
// first pass. Other configurations use the general kernels of k_tra.cuh.
//
// Same arithmetic, in the same order, as the general kernels (and the reference);
// what changes is the bookkeeping around it, which dominated the general kernels'
// instruction count:
//  * the masks of the columns a level reads are carried down the column: each level
//    evaluates only the new level's T / U / V membership, and wmask is the product
//    of two carried T masks;
//  * per-column metrics are loaded once per column, e3 once per level;
//  * 32-bit offsets within one (jpi,jpj,jpk) field, pointers advanced per level.
#pragma once
#include "k_tra.cuh"

namespace nemo {

// true when the context's configuration is the one these kernels assume
template <class T>
inline bool hot_iso_ok(const Dom<T>& d, const LdfArgs<T>& a) {
  auto flat = [](const E3<T>& e) { return e.s == 0 && e.sm == 0; };
  return !a.pahu && !a.pahv && !a.zps && !a.msc && a.lap && a.kpass == 1 && flat(d.e3u_n) && flat(d.e3v_n) &&
         flat(d.e3w_n);
}

template <class T>
__device__ __forceinline__ T t_in(const ColInfo& c, int k) { return (k >= c.tlo && k <= c.thi) ? T(1) : T(0); }
template <class T>
__device__ __forceinline__ T u_in(const ColInfo& c, int k) { return (k >= c.ulo && k <= c.uhi) ? T(1) : T(0); }
template <class T>
__device__ __forceinline__ T v_in(const ColInfo& c, int k) { return (k >= c.vlo && k <= c.vhi) ? T(1) : T(0); }

// Iso-neutral fluxes (traldf_iso.F90:146-357) of one column chunk; see k_iso_flux.
// It also sets akz = ah_wslp2 on the points k_iso_akz_copy_edges covers in general.
template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 6 : 3) k_iso_flux_hot(Dom<T> d, LdfArgs<T> a) {
  const KIdx c = k_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpj = d.jpj, jpk = d.jpk;
  {  // akz = ah_wslp2 where the interior sweep writes neither (traldf_iso.F90:200-201):
     // every level of the edge columns, levels 1 and jpk of the interior columns
    const long base = (long)c.m * d.n3 + c.ij;
    auto copy = [&](int k) {
      const long q = base + (long)(k - 1) * d.n2;
      a.akz[q] = a.ah_wslp2[q];
    };
    if (!c.interior) {
      for (int k = c.k0; k <= c.k1; ++k) copy(k);
    } else {
      if (c.k0 == 1) copy(1);
      if (c.k1 == jpk) copy(jpk);
    }
  }
  if (!(c.i <= jpi - 1 && c.j <= jpj - 1)) return;  // no face owned
  const int n2 = (int)d.n2, ij = (int)c.ij;
  const bool icol = c.interior;
  const ColInfo ci = d.ci[ij], cie = d.ci[ij + 1], cin = d.ci[ij + jpi];
  ColInfo ciw{}, cis{};
  if (icol) {
    ciw = d.ci[ij - 1];
    cis = d.ci[ij - jpi];
  }
  // per-column metrics
  const T e2_e1u = d.e2_e1u[ij], e1_e2v = d.e1_e2v[ij], e2u = d.e2u[ij], e1v = d.e1v[ij];
  const T e2t = icol ? d.e2t[ij] : T(0), e1t = icol ? d.e1t[ij] : T(0);
  const T aht = a.aht_c;
  const T* e3u = d.e3u_n.p.p;
  const T* e3v = d.e3v_n.p.p;
  const long m3 = (long)c.m * d.n3;
  const T* uslp = a.uslp.p + m3 + ij;
  const T* vslp = a.vslp.p + m3 + ij;
  const T* wslpi = a.wslpi.p + m3 + ij;
  const T* wslpj = a.wslpj.p + m3 + ij;
  T* ahw_out = a.ah_wslp2 + m3 + ij;
  T* akz_out = a.akz + m3 + ij;
  constexpr int NT = 2;
  const int k0 = c.k0;
  for (int n0 = 0; n0 < a.kjpt; n0 += NT) {
    const int nt = a.kjpt - n0 < NT ? a.kjpt - n0 : NT;
    const T* tb[NT];
    T *fu[NT], *fv[NT], *fw[NT];
    for (int nn = 0; nn < NT; ++nn) {
      const long mo = ((long)c.m * a.kjpt + n0 + (nn < nt ? nn : 0)) * d.n3 + ij;
      tb[nn] = a.ptb.p + mo;
      fu[nn] = a.zftu + mo;
      fv[nn] = a.zftv + mo;
      fw[nn] = a.ztfw + mo;
    }
    // carried masks: T at k-1, k, k+1 of (i,j), (i+1,j), (i,j+1); U at k-1, k of
    // (i,j), (i-1,j); V at k-1, k of (i,j), (i,j-1)
    T t0m = t_in<T>(ci, k0 - 1), t0 = t_in<T>(ci, k0), t0p = t_in<T>(ci, k0 + 1);
    T tem = t_in<T>(cie, k0 - 1), te_ = t_in<T>(cie, k0), tep = t_in<T>(cie, k0 + 1);
    T tnm = t_in<T>(cin, k0 - 1), tn_ = t_in<T>(cin, k0), tnp = t_in<T>(cin, k0 + 1);
    T u0m = u_in<T>(ci, k0 - 1), u0 = u_in<T>(ci, k0), uwm = u_in<T>(ciw, k0 - 1), uw = u_in<T>(ciw, k0);
    T v0m = v_in<T>(ci, k0 - 1), v0 = v_in<T>(ci, k0), vsm = v_in<T>(cis, k0 - 1), vs = v_in<T>(cis, k0);
    // carried per tracer: tb(k) at (i,j), (i+1,j), (i,j+1); zdk1t(k-1) there; zdit at
    // (i,j), (i-1,j) and zdjt at (i,j), (i,j-1) of level k-1; tb(k-1) at (i,j)
    T t0c[NT] = {}, tec[NT] = {}, tnc[NT] = {}, k10[NT] = {}, k1e[NT] = {}, k1n[NT] = {};
    T di0[NT] = {}, diw[NT] = {}, dj0[NT] = {}, djs[NT] = {}, tup[NT] = {};
    int q = (k0 - 1) * n2;
    for (int k = k0; k <= c.k1; ++k, q += n2) {
      if (k == jpk) {  // interior: ztfw = 0 at jpk
        if (icol)
          for (int nn = 0; nn < nt; ++nn) fw[nn][q] = T(0);
        break;
      }
      // wmask of the three columns at k and k+1
      const T wk = k == 1 ? t0 : msel(t0, t0m), wk1 = msel(t0p, t0);
      const T wke = k == 1 ? te_ : msel(te_, tem), wk1e = msel(tep, te_);
      const T wkn = k == 1 ? tn_ : msel(tn_, tnm), wk1n = msel(tnp, tn_);
      // horizontal fluxes' coefficients (:255-276)
      T pah = msel(aht, u0);
      const T zabe1 = pah * e2_e1u * __ldg(e3u + k - 1);
      const T zmsku_h = rcount4(wke, wk1, wk1e, wk);
      const T zcof1 = -pah * e2u * __ldg(uslp + q) * zmsku_h;
      pah = msel(aht, v0);
      const T zabe2 = pah * e1_e2v * __ldg(e3v + k - 1);
      const T zmskv_h = rcount4(wkn, wk1, wk1n, wk);
      const T zcof2 = -pah * e1v * __ldg(vslp + q) * zmskv_h;
      // vertical flux coefficients and ah_wslp2 = akz (:146-164, :200-201, :291-321).
      // The term (ah_wslp2 - akz) * dk(tb) of :323-332 is an exact 0 here (akz =
      // ah_wslp2) and adding it changes no value, so it is left out.
      const bool vface = icol && k >= 2;
      T zcoef3 = T(0), zcoef4 = T(0);
      if (vface) {
        const T zmsku = msel(rcount4(u0m, uw, uwm, u0), wk);
        const T zmskv = msel(rcount4(v0m, vs, vsm, v0), wk);
        const T zahu_w = (msel(aht, u0m) + msel(aht, uw) + msel(aht, uwm) + msel(aht, u0)) * zmsku;
        const T zahv_w = (msel(aht, v0m) + msel(aht, vs) + msel(aht, vsm) + msel(aht, v0)) * zmskv;
        const T wi = __ldg(wslpi + q), wj = __ldg(wslpj + q);
        const T ahw = zahu_w * wi * wi + zahv_w * wj * wj;
        ahw_out[q] = ahw;
        akz_out[q] = ahw;
        zcoef3 = -zahu_w * e2t * zmsku * wi;
        zcoef4 = -zahv_w * e1t * zmskv * wj;
      }
#pragma unroll
      for (int nn = 0; nn < NT; ++nn) {
        if (nn >= nt) break;
        const T* t = tb[nn];
        if (k == k0) {
          t0c[nn] = __ldg(t + q); tec[nn] = __ldg(t + q + 1); tnc[nn] = __ldg(t + q + jpi);
          if (k > 1) {
            const int qm = q - n2;
            const T a0 = __ldg(t + qm), ae = __ldg(t + qm + 1), an = __ldg(t + qm + jpi);
            k10[nn] = msel(a0 - t0c[nn], wk);
            k1e[nn] = msel(ae - tec[nn], wke);
            k1n[nn] = msel(an - tnc[nn], wkn);
            tup[nn] = a0;
            if (icol) {
              const T aw = __ldg(t + qm - 1), as = __ldg(t + qm - jpi);
              di0[nn] = msel(ae - a0, u0m);
              diw[nn] = msel(a0 - aw, uwm);
              dj0[nn] = msel(an - a0, v0m);
              djs[nn] = msel(a0 - as, vsm);
            }
          }
        }
        const T tc = t0c[nn], te = tec[nn], tn = tnc[nn];
        const T t1 = __ldg(t + q + n2), te1 = __ldg(t + q + 1 + n2), tn1 = __ldg(t + q + jpi + n2);
        // vertical gradients (:250-254)
        const T dk1_0 = msel(tc - t1, wk1), dk1_e = msel(te - te1, wk1e), dk1_n = msel(tn - tn1, wk1n);
        const T dk0_0 = k == 1 ? dk1_0 : k10[nn];
        const T dk0_e = k == 1 ? dk1_e : k1e[nn];
        const T dk0_n = k == 1 ? dk1_n : k1n[nn];
        const T zdi = msel(te - tc, u0);
        const T zdj = msel(tn - tc, v0);
        fu[nn][q] = msel(zabe1 * zdi + zcof1 * (dk0_e + dk1_0 + dk1_e + dk0_0), u0);
        fv[nn][q] = msel(zabe2 * zdj + zcof2 * (dk0_n + dk1_0 + dk1_n + dk0_0), v0);
        if (icol) {
          const T tw = __ldg(t + q - 1), ts = __ldg(t + q - jpi);
          const T zdiw = msel(tc - tw, uw);
          const T zdjs = msel(tc - ts, vs);
          T z = T(0);
          if (vface) {
            const T sdi = di0[nn] + zdiw + diw[nn] + zdi;
            const T sdj = dj0[nn] + zdjs + djs[nn] + zdj;
            z = zcoef3 * sdi + zcoef4 * sdj;
          }
          fw[nn][q] = z;
          di0[nn] = zdi; diw[nn] = zdiw; dj0[nn] = zdj; djs[nn] = zdjs;
        }
        k10[nn] = dk1_0; k1e[nn] = dk1_e; k1n[nn] = dk1_n;
        tup[nn] = tc;
        t0c[nn] = t1; tec[nn] = te1; tnc[nn] = tn1;
      }
      // masks of level k+1 (and k+2 for T)
      t0m = t0; t0 = t0p; t0p = t_in<T>(ci, k + 2);
      tem = te_; te_ = tep; tep = t_in<T>(cie, k + 2);
      tnm = tn_; tn_ = tnp; tnp = t_in<T>(cin, k + 2);
      u0m = u0; u0 = u_in<T>(ci, k + 1); uwm = uw; uw = u_in<T>(ciw, k + 1);
      v0m = v0; v0 = v_in<T>(ci, k + 1); vsm = vs; vs = v_in<T>(cis, k + 1);
    }
  }
}

template <class T>
inline bool hot_fct_ok(const Dom<T>& d, const FctArgs<T>& a) {
  auto flat = [](const E3<T>& e) { return e.s == 0 && e.sm == 0; };
  return a.trp && a.kn_fct_h == 2 && a.kn_fct_v == 2 && !a.pta_in && flat(d.e3t_n) && flat(d.e3t_b) &&
         flat(d.e3t_a) && flat(d.e3u_n) && flat(d.e3v_n);
}

// FCT stage a (traadv_fct.F90:119-280) of one column chunk; see k_fct_a. Tracer nn
// of the member is at offset nn * n3 from tracer 0.
template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 3) k_fct_a_hot(Dom<T> d, FctArgs<T> a) {
  const KIdx c = k_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk, n2 = (int)d.n2, n3 = (int)d.n3, ij = (int)c.ij;
  const long mb = (long)c.m * a.kjpt * d.n3 + ij;
  T* zwi = a.zwi + mb;
  T* ax = a.ax + mb;
  T* ay = a.ay + mb;
  T* az = a.az + mb;
  T* ta = a.pta + mb;
  if (!c.interior) {  // edge columns: every level 0
    for (int k = c.k0; k <= c.k1; ++k)
      for (int n = 0; n < a.kjpt; ++n) {
        const int q = (k - 1) * n2 + n * n3;
        zwi[q] = T(0); ax[q] = T(0); ay[q] = T(0); az[q] = T(0); ta[q] = T(0);
      }
    return;
  }
  const ColInfo ci = d.ci[ij];
  const T e2u0 = d.e2u[ij], e2uw = d.e2u[ij - 1], e1v0 = d.e1v[ij], e1vs = d.e1v[ij - jpi];
  const T e1e2t = d.e1e2t[ij], r1_e1e2t = d.r1_e1e2t[ij];
  const T* e3u = d.e3u_n.p.p;
  const T* e3v = d.e3v_n.p.p;
  const T* e3tn = d.e3t_n.p.p;
  const T* e3tb = d.e3t_b.p.p;
  const T* e3ta = d.e3t_a.p.p;
  const long mv = (long)c.m * d.n3 + ij;
  const T* un = a.pun.p + mv;
  const T* vn = a.pvn.p + mv;
  const T* wn = a.pwn.p + mv;
  const T* tbp_ = a.ptb.p + mb;
  const T* tnp_ = a.ptn.p + mb;
  const T p2dt = a.p2dt;
  const int k0 = c.k0;
  constexpr int NT = 2;
  for (int n0 = 0; n0 < a.kjpt; n0 += NT) {
    const int nt = a.kjpt - n0 < NT ? a.kjpt - n0 : NT;
    const int no = n0 * n3;
    // carried from level k-1: tb(k-1), tn(k-1), the bottom upstream flux of k-1;
    // T masks of the column at k-1, k, k+1
    T tbc[NT] = {}, tnc[NT] = {}, zwzb[NT] = {};
    T tkm = t_in<T>(ci, k0 - 1), tk = t_in<T>(ci, k0), tkp = t_in<T>(ci, k0 + 1);
    T wt = T(0);  // transport through the top face of level k
    int q = (k0 - 1) * n2;
    for (int k = k0; k <= c.k1; ++k, q += n2) {
      if (k == jpk) {  // level jpk: no work, edge values
        for (int nn = 0; nn < nt; ++nn) {
          const int qq = q + no + nn * n3;
          zwi[qq] = T(0); ax[qq] = T(0); ay[qq] = T(0); az[qq] = T(0); ta[qq] = T(0);
        }
        break;
      }
      const bool first = k == k0;
      const T e3uk = __ldg(e3u + k - 1), e3vk = __ldg(e3v + k - 1);
      const T ue = e2u0 * e3uk * __ldg(un + q);
      const T uw = e2uw * e3uk * __ldg(un + q - 1);
      const T vn_ = e1v0 * e3vk * __ldg(vn + q);
      const T vs = e1vs * e3vk * __ldg(vn + q - jpi);
      if (first) wt = e1e2t * __ldg(wn + q);
      const T wb = (k + 1 <= jpk - 1) ? e1e2t * __ldg(wn + q + n2) : T(0);
      const T e3n = __ldg(e3tn + k - 1), e3b = __ldg(e3tb + k - 1), e3a = __ldg(e3ta + k - 1);
      const T r1n = d.r1_e3t[k - 1];  // e3t_n, e3t_b and e3t_a are the one rest-state profile here
      const T tm = tk, wk = k == 1 ? tk : msel(tk, tkm), wk1 = msel(tkp, tk);
#pragma unroll
      for (int nn = 0; nn < NT; ++nn) {
        if (nn >= nt) break;
        const int o = no + nn * n3;
        const T* tb = tbp_ + o;
        const T* tn = tnp_ + o;
        const T tb0 = __ldg(tb + q);
        if (first && k > 1) {  // the carried values of level k-1
          tbc[nn] = __ldg(tb + q - n2);
          tnc[nn] = __ldg(tn + q - n2);
          zwzb[nn] = msel(ups(wt, tb0, tbc[nn]), wk);
        }
        const T zwx_e = ups(ue, tb0, __ldg(tb + q + 1)), zwx_w = ups(uw, __ldg(tb + q - 1), tb0);
        const T zwy_n = ups(vn_, tb0, __ldg(tb + q + jpi)), zwy_s = ups(vs, __ldg(tb + q - jpi), tb0);
        // upstream vertical fluxes at the top (k) and bottom (k+1) faces (:137-156)
        const T zwz_t = (k == 1) ? (a.linssh ? wt * tb0 : T(0)) : zwzb[nn];
        const T zwz_b = (k + 1 <= jpk - 1) ? msel(ups(wb, __ldg(tb + q + n2), tb0), wk1) : T(0);
        const T ztra = -(zwx_e - zwx_w + zwy_n - zwy_s + zwz_t - zwz_b) * r1_e1e2t;
        ta[o + q] = T(0) + msel(divq(ztra, e3n, r1n), tm);
        zwi[o + q] = msel(divq(e3b * tb0 + p2dt * ztra, e3a, r1n), tm);
        // 2nd-order antidiffusive fluxes (:180-190, :255-263)
        const T tn0 = __ldg(tn + q), tne = __ldg(tn + q + 1), tnn = __ldg(tn + q + jpi);
        ax[o + q] = T(0.5) * ue * (tn0 + tne) - zwx_e;
        ay[o + q] = T(0.5) * vn_ * (tn0 + tnn) - zwy_n;
        az[o + q] = k >= 2 ? msel(wt * T(0.5) * (tn0 + tnc[nn]) - zwz_t, wk) : T(0);
        tbc[nn] = tb0;
        tnc[nn] = tn0;
        zwzb[nn] = zwz_b;
      }
      wt = wb;
      tkm = tk; tk = tkp; tkp = t_in<T>(ci, k + 2);
    }
  }
}

// FCT stage b (traadv_fct.F90:361-400) of one column chunk; see k_fct_b.
template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 4) k_fct_b_hot(Dom<T> d, FctArgs<T> a) {
  const KIdx c = k_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk, n2 = (int)d.n2, n3 = (int)d.n3, ij = (int)c.ij;
  const long mb = (long)c.m * a.kjpt * d.n3 + ij;
  T* bu = a.betup + mb;
  T* bd = a.betdo + mb;
  if (!c.interior) {
    for (int k = c.k0; k <= c.k1; ++k)
      for (int n = 0; n < a.kjpt; ++n) {
        const int q = (k - 1) * n2 + n * n3;
        bu[q] = T(0);
        bd[q] = T(0);
      }
    return;
  }
  const T zrtrn = T(1.e-15);
  const ColInfo ci = d.ci[ij], ciw = d.ci[ij - 1], cie = d.ci[ij + 1], cis = d.ci[ij - jpi], cin = d.ci[ij + jpi];
  const T e1e2t = d.e1e2t[ij];
  const T* e3tn = d.e3t_n.p.p;
  const T* tbp_ = a.ptb.p + mb;
  const T* zwip = a.zwi + mb;
  const T* axp = a.ax + mb;
  const T* ayp = a.ay + mb;
  const T* azp = a.az + mb;
  const int k0 = c.k0;
  constexpr int NT = 2;
  for (int n0 = 0; n0 < a.kjpt; n0 += NT) {
    const int nt = a.kjpt - n0 < NT ? a.kjpt - n0 : NT;
    const int no = n0 * n3;
    // carried: masked extrema of the column at level k-1 and k, az(k), zwi(k)
    T upm[NT] = {}, dnm[NT] = {}, up0[NT] = {}, dn0[NT] = {}, azk[NT] = {}, zwik[NT] = {};
    T tkm = t_in<T>(ci, k0 - 1), tk = t_in<T>(ci, k0), tkp = t_in<T>(ci, k0 + 1);
    int q = (k0 - 1) * n2;
    for (int k = k0; k <= c.k1; ++k, q += n2) {
      if (k == jpk) {
        for (int nn = 0; nn < nt; ++nn) {
          bu[q + no + nn * n3] = T(0);
          bd[q + no + nn * n3] = T(0);
        }
        break;
      }
      const bool first = k == k0;
      const int qp = q + n2;
      const T zbt = divq(e1e2t * __ldg(e3tn + k - 1), a.p2dt, a.r1_p2dt);
      const T tw = t_in<T>(ciw, k), te = t_in<T>(cie, k), ts = t_in<T>(cis, k), tn = t_in<T>(cin, k);
#pragma unroll
      for (int nn = 0; nn < NT; ++nn) {
        if (nn >= nt) break;
        const int o = no + nn * n3;
        const T* tb = tbp_ + o;
        const T* zwi = zwip + o;
        const T* ax = axp + o;
        const T* ay = ayp + o;
        const T* az = azp + o;
        if (first) {  // extrema of the column at levels k and k-1, az(k)
          zwik[nn] = __ldg(zwi + q);
          bupdo(__ldg(tb + q), zwik[nn], tk, up0[nn], dn0[nn]);
          if (k > 1) bupdo(__ldg(tb + q - n2), __ldg(zwi + q - n2), tkm, upm[nn], dnm[nn]);
          else { upm[nn] = up0[nn]; dnm[nn] = dn0[nn]; }
          azk[nn] = __ldg(az + q);
        }
        const T zwp = __ldg(zwi + qp);
        T upp, dnp;  // level k+1 of the column
        bupdo(__ldg(tb + qp), zwp, tkp, upp, dnp);
        // the reference's order: centre, west, east, south, north, above, below
        T up = up0[nn], dn = dn0[nn], u2, d2;
        bupdo(__ldg(tb + q - 1), __ldg(zwi + q - 1), tw, u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        bupdo(__ldg(tb + q + 1), __ldg(zwi + q + 1), te, u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        bupdo(__ldg(tb + q - jpi), __ldg(zwi + q - jpi), ts, u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        bupdo(__ldg(tb + q + jpi), __ldg(zwi + q + jpi), tn, u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        up = vmax(up, upm[nn]); dn = vmin(dn, dnm[nn]);
        up = vmax(up, upp); dn = vmin(dn, dnp);
        const T axw = __ldg(ax + q - 1), ax0 = __ldg(ax + q), ays = __ldg(ay + q - jpi), ay0 = __ldg(ay + q);
        const T az0 = azk[nn], azb = __ldg(az + qp);
        const T zpos = pos_part(axw) - neg_part(ax0) + pos_part(ays) - neg_part(ay0) + pos_part(azb) - neg_part(az0);
        const T zneg = pos_part(ax0) - neg_part(axw) + pos_part(ay0) - neg_part(ays) + pos_part(az0) - neg_part(azb);
        const T zw = zwik[nn];
        bu[o + q] = (up - zw) / (zpos + zrtrn) * zbt;
        bd[o + q] = (zw - dn) / (zneg + zrtrn) * zbt;
        upm[nn] = up0[nn]; dnm[nn] = dn0[nn];
        up0[nn] = upp; dn0[nn] = dnp;
        azk[nn] = azb;
        zwik[nn] = zwp;
      }
      tkm = tk; tk = tkp; tkp = t_in<T>(ci, k + 2);
    }
  }
}


// FCT stage c (traadv_fct.F90:404-426, :288-297) with the fused iso-neutral
// divergence (traldf_iso.F90:278-284, :359-366) of one column chunk; see k_fct_c.
// One tracer per pass over the levels, and every value a level reads is loaded
// before any of its arithmetic, so a level costs one memory round trip.
template <class T>
__global__ void __launch_bounds__(128) k_fct_c_hot(Dom<T> d, FctArgs<T> a) {
  const KIdx c = k_index(d);
  if (!c.valid || !c.interior) return;
  const int jpi = d.jpi, jpk = d.jpk, n2 = (int)d.n2, n3 = (int)d.n3, ij = (int)c.ij;
  const long mb = (long)c.m * a.kjpt * d.n3 + ij;
  const T r1_e1e2t = d.r1_e1e2t[ij];
  const T* e3tn = d.e3t_n.p.p;
  const bool w_lim = c.i - 1 >= 2;  // the face i-1 is limited only for i-1 >= 2 (then lbc: 0)
  const bool s_lim = c.j - 1 >= 2;
  const int k1 = c.k1 < jpk - 1 ? c.k1 : jpk - 1;
  const bool iso = a.with_iso;
  const T zsign = a.iso.zsign;
  for (int n = 0; n < a.kjpt; ++n) {
    const int o = n * n3;
    T* ta = a.pta + mb + o;
    const T* ax = a.ax + mb + o;
    const T* ay = a.ay + mb + o;
    const T* az = a.az + mb + o;
    const T* bu = a.betup + mb + o;
    const T* bd = a.betdo + mb + o;
    const T* fu = iso ? a.iso.zftu + mb + o : ax;
    const T* fv = iso ? a.iso.zftv + mb + o : ay;
    const T* fw = iso ? a.iso.ztfw + mb + o : az;
    // carried: limiter coefficients of the column at level k, the limited flux
    // through the top face of level k, the iso-neutral vertical flux of that face
    int q = (c.k0 - 1) * n2;
    T bu0 = __ldg(bu + q), bd0 = __ldg(bd + q);
    T azt = c.k0 >= 2 ? limit(__ldg(az + q), bd0, __ldg(bu + q - n2), bu0, __ldg(bd + q - n2)) : __ldg(az + q);
    T fwt = iso ? __ldg(fw + q) : T(0);
    for (int k = c.k0; k <= k1; ++k, q += n2) {
      const int qp = q + n2;
      // every load of the level first
      const T e3n = __ldg(e3tn + k - 1);
      const T bup = __ldg(bu + qp), bdp = __ldg(bd + qp), azp = __ldg(az + qp);
      const T ax0 = __ldg(ax + q), axw = __ldg(ax + q - 1), ay0 = __ldg(ay + q), ays = __ldg(ay + q - jpi);
      const T bue = __ldg(bu + q + 1), bde = __ldg(bd + q + 1), buw = __ldg(bu + q - 1), bdw = __ldg(bd + q - 1);
      const T bun = __ldg(bu + q + jpi), bdn = __ldg(bd + q + jpi), bus = __ldg(bu + q - jpi), bds = __ldg(bd + q - jpi);
      T fu0 = T(0), fuw = T(0), fv0 = T(0), fvs = T(0), fwb = T(0);
      if (iso) {
        fu0 = __ldg(fu + q); fuw = __ldg(fu + q - 1); fv0 = __ldg(fv + q); fvs = __ldg(fv + q - jpi);
        fwb = __ldg(fw + qp);
      }
      const T ta0 = ta[q];
      // limited fluxes of the six faces (pcc(k+1): the bottom face)
      const T axl = limit(ax0, bd0, bue, bu0, bde);
      const T axlw = w_lim ? limit(axw, bdw, bu0, buw, bd0) : T(0);
      const T ayl = limit(ay0, bd0, bun, bu0, bdn);
      const T ayls = s_lim ? limit(ays, bds, bu0, bus, bd0) : T(0);
      const T azl_b = limit(azp, bdp, bu0, bup, bd0);
      const T r1n = d.r1_e3t[k - 1];
      T tav = ta0 - divq((axl - axlw + ayl - ayls + azt - azl_b) * r1_e1e2t, e3n, r1n);
      if (iso) {
        tav = tav + divq(zsign * (fu0 - fuw + fv0 - fvs) * r1_e1e2t, e3n, r1n);
        tav = tav + divq(zsign * (fwt - fwb) * r1_e1e2t, e3n, r1n);
        fwt = fwb;
      }
      ta[q] = tav;
      bu0 = bup;
      bd0 = bdp;
      azt = azl_b;
    }
  }
}

}  // namespace nemo
