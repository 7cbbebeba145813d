// k_tra.cuh -- tracer kernels: transports, FCT advection (upstream + antidiffusive
// fluxes, Zalesak limiter, final trend), compact 4th-order vertical interpolation,
// laplacian and rotated iso-neutral lateral diffusion, implicit vertical diffusion.
//
// One thread owns one (i,j) column and marches k; i is the fast thread index so
// every 3-D load is coalesced. Indices i, j, k are 1-based as in the Fortran they
// restate, and every expression keeps the reference's association (the FP64
// instantiation is compiled without FMA contraction, so it reproduces the
// reference's FP64 arithmetic operation by operation).
#pragma once
#include "nemo_common.cuh"

namespace nemo {

constexpr int KMAX = 64;  // maximum jpk (checked at context creation)

template <class T>
struct ColIdx {
  int i, j, m;
  long ij;
  bool valid, interior;
};

template <class T>
__device__ __forceinline__ ColIdx<T> col_index(const Dom<T>& d) {
  ColIdx<T> c;
  c.i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  c.j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  c.m = blockIdx.z;
  c.valid = c.i <= d.jpi && c.j <= d.jpj;
  c.interior = c.i >= 2 && c.i <= d.jpi - 1 && c.j >= 2 && c.j <= d.jpj - 1;
  c.ij = (long)(c.i - 1) + (long)(c.j - 1) * d.jpi;
  return c;
}

// --------------------------------------------------------------------------------
// traadv.F90:99-124: zun = e2u*e3u_n*un, zvn = e1v*e3v_n*vn, zwn = e1e2t*wn, 0 at jpk.
template <class T>
__global__ void k_adv_trp(Dom<T> d, const T* __restrict__ un, const T* __restrict__ vn,
                          const T* __restrict__ wn, T* __restrict__ zun, T* __restrict__ zvn,
                          T* __restrict__ zwn) {
  ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const long mo = (long)c.m * d.n3;
  const T e2u = d.e2u[c.ij], e1v = d.e1v[c.ij], e1e2t = d.e1e2t[c.ij];
  for (int k = 1; k <= d.jpk - 1; ++k) {
    long q = mo + c.ij + (long)(k - 1) * d.n2;
    zun[q] = e2u * d.e3u_n(c.ij, k, c.m) * un[q];
    zvn[q] = e1v * d.e3v_n(c.ij, k, c.m) * vn[q];
    zwn[q] = e1e2t * wn[q];
  }
  long q = mo + c.ij + (long)(d.jpk - 1) * d.n2;
  zun[q] = T(0); zvn[q] = T(0); zwn[q] = T(0);
}

// Arguments shared by the three FCT kernels.
template <class T>
struct FctArgs {
  T p2dt;
  const T *pun, *pvn, *pwn;  // transports, or velocities when trp != 0
  int trp;                   // 1: scale velocities to transports on the fly (traadv.F90:110-114)
  const T *ptb, *ptn;        // (jpi,jpj,jpk,kjpt)
  const T* pta_in;           // NULL: the trend starts from tsa = 0 (step.F90:234)
  T* pta;                    // (jpi,jpj,jpk,kjpt)
  T *zwi, *ax, *ay, *az;     // work: monotone guess and antidiffusive fluxes (jpi,jpj,jpk,kjpt)
  T *betup, *betdo;          // work: limiter coefficients (jpi,jpj,jpk,kjpt)
  const T* ztw;              // compact 4th-order tn at w-points (kn_fct_v = 4), or NULL
  int kjpt, kn_fct_h, kn_fct_v, linssh;
};

// Upstream transports at the faces of column (i,j) (traadv_fct.F90:123-145); a face
// value of a neighbouring column is recomputed rather than exchanged.
template <class T>
__device__ __forceinline__ T trp_u(const Dom<T>& d, const FctArgs<T>& a, long ij, long q, int k, int m) {
  T u = a.pun[q];
  return a.trp ? d.e2u[ij] * d.e3u_n(ij, k, m) * u : u;
}
template <class T>
__device__ __forceinline__ T trp_v(const Dom<T>& d, const FctArgs<T>& a, long ij, long q, int k, int m) {
  T v = a.pvn[q];
  return a.trp ? d.e1v[ij] * d.e3v_n(ij, k, m) * v : v;
}
template <class T>
__device__ __forceinline__ T trp_w(const Dom<T>& d, const FctArgs<T>& a, long ij, long q) {
  T w = a.pwn[q];
  return a.trp ? d.e1e2t[ij] * w : w;
}
template <class T>
__device__ __forceinline__ T ups(T u, T tl, T tr) {
  T zfp = u + fabs(u);
  T zfm = u - fabs(u);
  return T(0.5) * (zfp * tl + zfm * tr);
}

// FCT stage a: upstream trend into pta, monotone guess zwi, antidiffusive fluxes
// (traadv_fct.F90:119-278) with the lbc_lnk of :280 folded in (edge values 0).
template <class T>
__global__ void k_fct_a(Dom<T> d, FctArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const T r1_6 = T(1) / T(6);
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;  // tracer-field offset
    const long mv = (long)c.m * n3;                  // velocity-field offset
    const T* tb = a.ptb + mo;
    const T* tn = a.ptn + mo;
    T* ta = a.pta + mo;
    const T* tai = a.pta_in ? a.pta_in + mo : nullptr;
    if (!c.interior) {
      for (int k = 1; k <= jpk; ++k) {
        long q = c.ij + (long)(k - 1) * n2;
        a.zwi[mo + q] = T(0); a.ax[mo + q] = T(0); a.ay[mo + q] = T(0); a.az[mo + q] = T(0);
        if (!tai) ta[q] = T(0);
        else if (tai != ta) ta[q] = tai[q];
      }
      continue;
    }
    const ColInfo ci = d.ci[c.ij];
    const ColInfo ciw = d.ci[c.ij - 1], cie = d.ci[c.ij + 1];
    const ColInfo cis = d.ci[c.ij - jpi], cin = d.ci[c.ij + jpi];
    const T r1_e1e2t = d.r1_e1e2t[c.ij];
    // upstream vertical flux at the top face of level 1 (:146-156)
    T zwz_t = a.linssh ? trp_w(d, a, c.ij, mv + c.ij) * tb[c.ij] : T(0);
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = c.ij + (long)(k - 1) * n2;
      const T tb0 = tb[q], tbe = tb[q + 1], tbw = tb[q - 1], tbn = tb[q + jpi], tbs = tb[q - jpi];
      const T ue = trp_u(d, a, c.ij, mv + q, k, c.m), uw = trp_u(d, a, c.ij - 1, mv + q - 1, k, c.m);
      const T vn_ = trp_v(d, a, c.ij, mv + q, k, c.m), vs = trp_v(d, a, c.ij - jpi, mv + q - jpi, k, c.m);
      const T zwx_e = ups(ue, tb0, tbe), zwx_w = ups(uw, tbw, tb0);
      const T zwy_n = ups(vn_, tb0, tbn), zwy_s = ups(vs, tbs, tb0);
      T zwz_b = T(0);
      T wb = T(0);
      if (k + 1 <= jpk - 1) {
        wb = trp_w(d, a, c.ij, mv + q + n2);
        zwz_b = ups(wb, tb[q + n2], tb0) * wmsk<T>(ci, k + 1);
      }
      const T ztra = -(zwx_e - zwx_w + zwy_n - zwy_s + zwz_t - zwz_b) * r1_e1e2t;
      const T tm = tmsk<T>(ci, k);
      const T tin = tai ? tai[q] : T(0);
      ta[q] = tin + ztra / d.e3t_n(c.ij, k, c.m) * tm;
      a.zwi[mo + q] = (d.e3t_b(c.ij, k, c.m) * tb0 + a.p2dt * ztra) / d.e3t_a(c.ij, k, c.m) * tm;
      // horizontal antidiffusive fluxes (:180-251)
      const T tn0 = tn[q], tne = tn[q + 1], tnn = tn[q + jpi];
      T axv, ayv;
      if (a.kn_fct_h == 2) {
        axv = T(0.5) * ue * (tn0 + tne) - zwx_e;
        ayv = T(0.5) * vn_ * (tn0 + tnn) - zwy_n;
      } else {
        const T tnw = tn[q - 1], tns = tn[q - jpi];
        // ztu(i') = (tn(i'+1) - tn(i')) * umask(i'); zltu(i) = (ztu(i) + ztu(i-1)) / 6
        const T ztu_w = (tn0 - tnw) * umsk<T>(ciw, k);
        const T ztu_0 = (tne - tn0) * umsk<T>(ci, k);
        const T zltu0 = (ztu_0 + ztu_w) * r1_6;
        T zltue = T(0);
        if (c.i + 1 <= jpi - 1) {
          const T ztu_e = (tn[q + 2] - tne) * umsk<T>(cie, k);
          zltue = (ztu_e + ztu_0) * r1_6;
        }
        const T ztv_s = (tn0 - tns) * vmsk<T>(cis, k);
        const T ztv_0 = (tnn - tn0) * vmsk<T>(ci, k);
        const T zltv0 = (ztv_0 + ztv_s) * r1_6;
        T zltvn = T(0);
        if (c.j + 1 <= d.jpj - 1) {
          const T ztv_n = (tn[q + 2 * jpi] - tnn) * vmsk<T>(cin, k);
          zltvn = (ztv_n + ztv_0) * r1_6;
        }
        const T zC2t_u = tn0 + tne;
        const T zC2t_v = tn0 + tnn;
        axv = T(0.5) * ue * (zC2t_u + zltu0 - zltue) - zwx_e;
        ayv = T(0.5) * vn_ * (zC2t_v + zltv0 - zltvn) - zwy_n;
      }
      a.ax[mo + q] = axv;
      a.ay[mo + q] = ayv;
      // vertical antidiffusive flux at the top face of level k (:253-278)
      T azv = T(0);
      if (k >= 2) {
        const T wt = trp_w(d, a, c.ij, mv + q);
        if (a.kn_fct_v == 2)
          azv = (wt * T(0.5) * (tn0 + tn[q - n2]) - zwz_t) * wmsk<T>(ci, k);
        else
          azv = (wt * a.ztw[mo + q] - zwz_t) * wmsk<T>(ci, k);
      }
      a.az[mo + q] = azv;
      zwz_t = zwz_b;
      (void)wb;
    }
    const long q = c.ij + (long)(jpk - 1) * n2;
    a.zwi[mo + q] = T(0); a.ax[mo + q] = T(0); a.ay[mo + q] = T(0); a.az[mo + q] = T(0);
    if (!tai) ta[q] = T(0);
    else if (tai != ta) ta[q] = tai[q];
  }
}

// zbup / zbdo of nonosc (traadv_fct.F90:361-364) at one point.
template <class T>
__device__ __forceinline__ void bupdo(T pbef, T paft, T tm, T& up, T& dn) {
  const T zbig = Big<T>::v;
  up = fmx(pbef * tm - zbig * (T(1) - tm), paft * tm - zbig * (T(1) - tm));
  dn = fmn(pbef * tm + zbig * (T(1) - tm), paft * tm + zbig * (T(1) - tm));
}

// FCT stage b: nonosc extrema and limiter coefficients zbetup / zbetdo
// (traadv_fct.F90:366-400), edge values 0 (lbc_lnk of :400).
template <class T>
__global__ void k_fct_b(Dom<T> d, FctArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const T zrtrn = T(1.e-15);
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    if (!c.interior) {
      for (int k = 1; k <= jpk; ++k) {
        long q = mo + c.ij + (long)(k - 1) * n2;
        a.betup[q] = T(0); a.betdo[q] = T(0);
      }
      continue;
    }
    const T* tb = a.ptb + mo;
    const T* zwi = a.zwi + mo;
    const T* ax = a.ax + mo;
    const T* ay = a.ay + mo;
    const T* az = a.az + mo;
    const ColInfo ci = d.ci[c.ij];
    const ColInfo ciw = d.ci[c.ij - 1], cie = d.ci[c.ij + 1];
    const ColInfo cis = d.ci[c.ij - jpi], cin = d.ci[c.ij + jpi];
    const T e1e2t = d.e1e2t[c.ij];
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = c.ij + (long)(k - 1) * n2;
      const int km1 = k - 1 > 1 ? k - 1 : 1;
      const long qm = c.ij + (long)(km1 - 1) * n2, qp = q + n2;
      T up, dn, u2, d2;
      bupdo(tb[q], zwi[q], tmsk<T>(ci, k), up, dn);
      bupdo(tb[q - 1], zwi[q - 1], tmsk<T>(ciw, k), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
      bupdo(tb[q + 1], zwi[q + 1], tmsk<T>(cie, k), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
      bupdo(tb[q - jpi], zwi[q - jpi], tmsk<T>(cis, k), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
      bupdo(tb[q + jpi], zwi[q + jpi], tmsk<T>(cin, k), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
      bupdo(tb[qm], zwi[qm], tmsk<T>(ci, km1), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
      bupdo(tb[qp], zwi[qp], tmsk<T>(ci, k + 1), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
      const T axw = ax[q - 1], ax0 = ax[q], ays = ay[q - jpi], ay0 = ay[q], az0 = az[q], azb = az[qp];
      const T zpos = fmx(T(0), axw) - fmn(T(0), ax0) + fmx(T(0), ays) - fmn(T(0), ay0) + fmx(T(0), azb) - fmn(T(0), az0);
      const T zneg = fmx(T(0), ax0) - fmn(T(0), axw) + fmx(T(0), ay0) - fmn(T(0), ays) + fmx(T(0), az0) - fmn(T(0), azb);
      const T zbt = e1e2t * d.e3t_n(c.ij, k, c.m) / a.p2dt;
      a.betup[mo + q] = (up - zwi[q]) / (zpos + zrtrn) * zbt;
      a.betdo[mo + q] = (zwi[q] - dn) / (zneg + zrtrn) * zbt;
    }
    const long q = mo + c.ij + (long)(jpk - 1) * n2;
    a.betup[q] = T(0); a.betdo[q] = T(0);
  }
}

// Limited antidiffusive flux (traadv_fct.F90:407-422): f * ( c*a + (1-c)*b ).
template <class T>
__device__ __forceinline__ T limit(T f, T bdo0, T bup1, T bup0, T bdo1) {
  const T za = fmn(T(1), fmn(bdo0, bup1));
  const T zb = fmn(T(1), fmn(bup0, bdo1));
  const T zc = (T(0.5) + sign_nsz(T(0.5), f));
  return f * (zc * za + (T(1) - zc) * zb);
}

// FCT stage c: limit the fluxes (traadv_fct.F90:404-426) and add the divergence of
// the corrected fluxes to pta (:288-297). Interior columns only.
template <class T>
__global__ void k_fct_c(Dom<T> d, FctArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid || !c.interior) return;
  const int jpi = d.jpi, jpj = d.jpj, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const T r1_e1e2t = d.r1_e1e2t[c.ij];
  const bool w_lim = c.i - 1 >= 2;  // the face i-1 is limited only for i-1 >= 2 (then lbc: 0)
  const bool s_lim = c.j - 1 >= 2;
  (void)jpj;
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const T* ax = a.ax + mo;
    const T* ay = a.ay + mo;
    const T* az = a.az + mo;
    const T* bu = a.betup + mo;
    const T* bd = a.betdo + mo;
    T* ta = a.pta + mo;
    T azl_t = az[c.ij];  // level 1: not limited (0 without cavities)
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = c.ij + (long)(k - 1) * n2;
      const T bu0 = bu[q], bd0 = bd[q];
      const T axl = limit(ax[q], bd0, bu[q + 1], bu0, bd[q + 1]);
      const T axlw = w_lim ? limit(ax[q - 1], bd[q - 1], bu0, bu[q - 1], bd0) : T(0);
      const T ayl = limit(ay[q], bd0, bu[q + jpi], bu0, bd[q + jpi]);
      const T ayls = s_lim ? limit(ay[q - jpi], bd[q - jpi], bu0, bu[q - jpi], bd0) : T(0);
      // pcc(k+1) uses zbetdo(k+1), zbetup(k) and zbetup(k+1), zbetdo(k)
      const T azl_b = limit(az[q + n2], bd[q + n2], bu0, bu[q + n2], bd0);
      ta[q] = ta[q] - (axl - axlw + ayl - ayls + azl_t - azl_b) * r1_e1e2t / d.e3t_n(c.ij, k, c.m);
      azl_t = azl_b;
    }
  }
}

// interp_4th_cpt (traadv_fct.F90:517-616): compact 4th-order tn at w-points for the
// interior columns, levels 2..jpkm1, one tridiagonal solve per column.
template <class T>
__global__ void k_interp4(Dom<T> d, const T* __restrict__ ptn, T* __restrict__ ztw, int kjpt) {
  ColIdx<T> c = col_index(d);
  if (!c.valid || !c.interior) return;
  const int jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const ColInfo ci = d.ci[c.ij];
  const int ikt = 2;  // mikt + 1 without ice-shelf cavities
  const int ikb = d.mbkt[c.ij];
  T zwt[KMAX], zws[KMAX], out[KMAX];
  for (int n = 0; n < kjpt; ++n) {
    const long mo = ((long)c.m * kjpt + n) * n3;
    const T* t = ptn + mo;
    auto coef = [&](int k, T& zwd, T& zwi, T& zwsk, T& zwrm) {
      const T tk = t[c.ij + (long)(k - 1) * n2], tkm = t[c.ij + (long)(k - 2) * n2];
      if (k == ikt || k == ikb) {
        zwd = T(1); zwi = T(0); zwsk = T(0);
        zwrm = T(0.5) * (tkm + tk);
      } else {
        const T wm = wmsk<T>(ci, k);
        zwd = T(3) * wm + T(1); zwi = wm; zwsk = wm;
        zwrm = T(3) * wm * (tk + tkm);
      }
    };
    T zwd, zwi, zwrm;
    coef(2, zwd, zwi, zws[2], zwrm);
    zwt[2] = zwd;
    out[2] = zwrm;
    for (int k = 3; k <= jpk - 1; ++k) {
      coef(k, zwd, zwi, zws[k], zwrm);
      zwt[k] = zwd - zwi * zws[k - 1] / zwt[k - 1];
      out[k] = zwrm - zwi / zwt[k - 1] * out[k - 1];
    }
    out[jpk - 1] = out[jpk - 1] / zwt[jpk - 1];
    for (int k = jpk - 2; k >= 2; --k) out[k] = (out[k] - zws[k] * out[k + 1]) / zwt[k];
    for (int k = 2; k <= jpk - 1; ++k) ztw[mo + c.ij + (long)(k - 1) * n2] = out[k];
  }
}

// --------------------------------------------------------------------------------
// Lateral diffusion arguments.
template <class T>
struct LdfArgs {
  const T *pahu, *pahv;      // NULL: aht_c * umask/vmask above jpk (ldftra.F90:292-372)
  T aht_c;
  const T *pgu, *pgv;        // partial-step gradients (jpi,jpj,kjpt) when zps
  int zps;
  const T *ptb, *ptbb;
  T* pta;
  int kjpt, kpass;
  T zsign;
  // iso-neutral
  const T *uslp, *vslp, *wslpi, *wslpj;
  T *ah_wslp2, *akz;
  int lap, blp, msc;
  T z2dt, z1_2dt;
};

template <class T>
__device__ __forceinline__ T ahu(const Dom<T>& d, const LdfArgs<T>& a, const ColInfo& c, long ij, int k, int m) {
  if (a.pahu) return a.pahu[(long)m * d.n3 + ij + (long)(k - 1) * d.n2];
  return k < d.jpk ? a.aht_c * umsk<T>(c, k) : T(0);
}
template <class T>
__device__ __forceinline__ T ahv(const Dom<T>& d, const LdfArgs<T>& a, const ColInfo& c, long ij, int k, int m) {
  if (a.pahv) return a.pahv[(long)m * d.n3 + ij + (long)(k - 1) * d.n2];
  return k < d.jpk ? a.aht_c * vmsk<T>(c, k) : T(0);
}

// tra_ldf_lap (traldf_lap_blp.F90:95-145). Interior columns.
template <class T>
__global__ void k_ldf_lap(Dom<T> d, LdfArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid || !c.interior) return;
  const int jpi = d.jpi, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const ColInfo ci = d.ci[c.ij], ciw = d.ci[c.ij - 1], cis = d.ci[c.ij - jpi];
  const long ijw = c.ij - 1, ijs = c.ij - jpi;
  const T e2_e1u0 = d.e2_e1u[c.ij], e2_e1uw = d.e2_e1u[ijw];
  const T e1_e2v0 = d.e1_e2v[c.ij], e1_e2vs = d.e1_e2v[ijs];
  const T e1e2t = d.e1e2t[c.ij];
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const T* tb = a.ptb + mo;
    T* ta = a.pta + mo;
    const long go = ((long)c.m * a.kjpt + n) * n2;
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = c.ij + (long)(k - 1) * n2;
      const T zu0 = a.zsign * ahu(d, a, ci, c.ij, k, c.m) * e2_e1u0 * d.e3u_n(c.ij, k, c.m);
      const T zuw = a.zsign * ahu(d, a, ciw, ijw, k, c.m) * e2_e1uw * d.e3u_n(ijw, k, c.m);
      const T zv0 = a.zsign * ahv(d, a, ci, c.ij, k, c.m) * e1_e2v0 * d.e3v_n(c.ij, k, c.m);
      const T zvs = a.zsign * ahv(d, a, cis, ijs, k, c.m) * e1_e2vs * d.e3v_n(ijs, k, c.m);
      const T tb0 = tb[q];
      T ztu0 = zu0 * (tb[q + 1] - tb0);
      T ztuw = zuw * (tb0 - tb[q - 1]);
      T ztv0 = zv0 * (tb[q + jpi] - tb0);
      T ztvs = zvs * (tb0 - tb[q - jpi]);
      if (a.zps) {
        if (k == ci.mbku) ztu0 = zu0 * a.pgu[go + c.ij];
        if (k == ciw.mbku) ztuw = zuw * a.pgu[go + ijw];
        if (k == ci.mbkv) ztv0 = zv0 * a.pgv[go + c.ij];
        if (k == cis.mbkv) ztvs = zvs * a.pgv[go + ijs];
      }
      ta[q] = ta[q] + (ztu0 - ztuw + ztv0 - ztvs) / (e1e2t * d.e3t_n(c.ij, k, c.m));
    }
  }
}

// Masked horizontal gradient zdit / zdjt of tra_ldf_iso (traldf_iso.F90:218-241).
template <class T>
__device__ __forceinline__ T dit(const LdfArgs<T>& a, const ColInfo& c, const T* tb, long q, int k, long g) {
  if (a.zps && k == c.mbku) return a.pgu[g];
  return (tb[q + 1] - tb[q]) * umsk<T>(c, k);
}
template <class T>
__device__ __forceinline__ T djt(const LdfArgs<T>& a, const ColInfo& c, const T* tb, long q, int k, long g, int jpi) {
  if (a.zps && k == c.mbkv) return a.pgv[g];
  return (tb[q + jpi] - tb[q]) * vmsk<T>(c, k);
}

// ah_wslp2 (traldf_iso.F90:146-164) and akz (:166-202) at one interior point, level k.
template <class T>
__device__ __forceinline__ void iso_coefs(const Dom<T>& d, const LdfArgs<T>& a, long ij, int k, int m,
                                          const ColInfo& ci, const ColInfo& ciw, const ColInfo& cis) {
  const int jpi = d.jpi;
  const long q = (long)m * d.n3 + ij + (long)(k - 1) * d.n2;
  const T wm = wmsk<T>(ci, k);
  const T zmsku = wm / fmx(umsk<T>(ci, k - 1) + umsk<T>(ciw, k) + umsk<T>(ciw, k - 1) + umsk<T>(ci, k), T(1));
  const T zmskv = wm / fmx(vmsk<T>(ci, k - 1) + vmsk<T>(cis, k) + vmsk<T>(cis, k - 1) + vmsk<T>(ci, k), T(1));
  const T zahu_w = (ahu(d, a, ci, ij, k - 1, m) + ahu(d, a, ciw, ij - 1, k, m) + ahu(d, a, ciw, ij - 1, k - 1, m) +
                    ahu(d, a, ci, ij, k, m)) * zmsku;
  const T zahv_w = (ahv(d, a, ci, ij, k - 1, m) + ahv(d, a, cis, ij - jpi, k, m) + ahv(d, a, cis, ij - jpi, k - 1, m) +
                    ahv(d, a, ci, ij, k, m)) * zmskv;
  const T wi = a.wslpi[q], wj = a.wslpj[q];
  const T ahw = zahu_w * wi * wi + zahv_w * wj * wj;
  a.ah_wslp2[q] = ahw;
  if (a.msc) {
    const T e1u0 = d.e1u[ij], e1uw = d.e1u[ij - 1], e2v0 = d.e2v[ij], e2vs = d.e2v[ij - jpi];
    T akzv = T(0.25) * ((ahu(d, a, ci, ij, k, m) + ahu(d, a, ci, ij, k - 1, m)) / (e1u0 * e1u0) +
                        (ahu(d, a, ciw, ij - 1, k, m) + ahu(d, a, ciw, ij - 1, k - 1, m)) / (e1uw * e1uw) +
                        (ahv(d, a, ci, ij, k, m) + ahv(d, a, ci, ij, k - 1, m)) / (e2v0 * e2v0) +
                        (ahv(d, a, cis, ij - jpi, k, m) + ahv(d, a, cis, ij - jpi, k - 1, m)) / (e2vs * e2vs));
    const T e3w = d.e3w_n(ij, k, m);
    if (a.blp) {
      akzv = T(16) * ahw * (akzv + ahw / (e3w * e3w));
    } else if (a.lap) {
      const T ze3w_2 = e3w * e3w;
      const T zcoef0 = a.z2dt * (akzv + ahw / ze3w_2);
      akzv = fmx(zcoef0 - T(0.5), T(0)) * ze3w_2 * a.z1_2dt;
    }
    a.akz[q] = akzv;
  } else {
    a.akz[q] = ahw;
  }
}

// Edge points of the second MSC loop (traldf_iso.F90:179-197), which runs over
// ji = 1..jpim1, jj = 1..jpjm1 and therefore also updates row 1 and column 1.
template <class T>
__global__ void k_iso_msc_edges(Dom<T> d, LdfArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid || c.interior) return;
  if (c.i > d.jpi - 1 || c.j > d.jpj - 1) return;
  for (int k = 2; k <= d.jpk - 1; ++k) {
    const long q = (long)c.m * d.n3 + c.ij + (long)(k - 1) * d.n2;
    const T e3w = d.e3w_n(c.ij, k, c.m);
    const T ahw = a.ah_wslp2[q];
    T akzv = a.akz[q];
    if (a.blp) {
      akzv = T(16) * ahw * (akzv + ahw / (e3w * e3w));
    } else if (a.lap) {
      const T ze3w_2 = e3w * e3w;
      const T zcoef0 = a.z2dt * (akzv + ahw / ze3w_2);
      akzv = fmx(zcoef0 - T(0.5), T(0)) * ze3w_2 * a.z1_2dt;
    }
    a.akz[q] = akzv;
  }
}

// akz = ah_wslp2 on the whole array (traldf_iso.F90:200-201) for the points the
// interior sweep does not write (edge columns, levels 1 and jpk).
template <class T>
__global__ void k_iso_akz_copy_edges(Dom<T> d, LdfArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  for (int k = 1; k <= d.jpk; ++k) {
    if (c.interior && k >= 2 && k <= d.jpk - 1) continue;
    const long q = (long)c.m * d.n3 + c.ij + (long)(k - 1) * d.n2;
    a.akz[q] = a.ah_wslp2[q];
  }
}

// tra_ldf_iso (traldf_iso.F90:144-366). Interior columns. On kpass = 1 the first
// tracer's sweep also computes ah_wslp2 / akz one level ahead of their use.
template <class T>
__global__ void k_ldf_iso(Dom<T> d, LdfArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid || !c.interior) return;
  const int jpi = d.jpi, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const long ij = c.ij, ijw = ij - 1, ije = ij + 1, ijs = ij - jpi, ijn = ij + jpi;
  const ColInfo ci = d.ci[ij], ciw = d.ci[ijw], cie = d.ci[ije], cis = d.ci[ijs], cin = d.ci[ijn];
  const ColInfo cisw = d.ci[ijs - 1] , cine = d.ci[ijn + 1];
  (void)cisw; (void)cine;
  const ColInfo cise = d.ci[ijs + 1], cinw = d.ci[ijn - 1];
  const T r1_e1e2t = d.r1_e1e2t[ij], e1e2t = d.e1e2t[ij];
  const T e2_e1u0 = d.e2_e1u[ij], e2_e1uw = d.e2_e1u[ijw], e1_e2v0 = d.e1_e2v[ij], e1_e2vs = d.e1_e2v[ijs];
  const T e2u0 = d.e2u[ij], e2uw = d.e2u[ijw], e1v0 = d.e1v[ij], e1vs = d.e1v[ijs];
  const T e2t = d.e2t[ij], e1t = d.e1t[ij];
  const long m3 = (long)c.m * n3;
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const long go = ((long)c.m * a.kjpt + n) * n2;
    const T* tb = a.ptb + mo;
    const T* tbb = a.ptbb + mo;
    T* ta = a.pta + mo;
    const bool coefs = (a.kpass == 1 && n == 0);
    if (coefs && jpk - 1 >= 2) iso_coefs(d, a, ij, 2, c.m, ci, ciw, cis);
    // vertical gradient at a column P, level k: zdk1t = (tb(k)-tb(k+1))*wmask(k+1),
    // zdkt = (tb(k-1)-tb(k))*wmask(k) with zdkt(1) = zdk1t(1) (:250-254)
    auto dk1 = [&](long p, const ColInfo& cp, int k) -> T {
      const long qq = p + (long)(k - 1) * n2;
      return (tb[qq] - tb[qq + n2]) * wmsk<T>(cp, k + 1);
    };
    auto dk0 = [&](long p, const ColInfo& cp, int k) -> T {
      if (k == 1) return dk1(p, cp, 1);
      const long qq = p + (long)(k - 1) * n2;
      return (tb[qq - n2] - tb[qq]) * wmsk<T>(cp, k);
    };
    // horizontal fluxes at the faces (:255-276)
    auto ftu = [&](long p, const ColInfo& cp, const ColInfo& cpe, T e2_e1u, T e2u, int k) -> T {
      const long qq = p + (long)(k - 1) * n2;
      const T pah = ahu(d, a, cp, p, k, c.m);
      const T zabe1 = pah * e2_e1u * d.e3u_n(p, k, c.m);
      const T zmsku = T(1) / fmx(wmsk<T>(cpe, k) + wmsk<T>(cp, k + 1) + wmsk<T>(cpe, k + 1) + wmsk<T>(cp, k), T(1));
      const T zcof1 = -pah * e2u * a.uslp[m3 + qq] * zmsku;
      const T zd = dit(a, cp, tb, qq, k, go + p);
      return (zabe1 * zd + zcof1 * (dk0(p + 1, cpe, k) + dk1(p, cp, k) + dk1(p + 1, cpe, k) + dk0(p, cp, k))) *
             umsk<T>(cp, k);
    };
    auto ftv = [&](long p, const ColInfo& cp, const ColInfo& cpn, T e1_e2v, T e1v, int k) -> T {
      const long qq = p + (long)(k - 1) * n2;
      const T pah = ahv(d, a, cp, p, k, c.m);
      const T zabe2 = pah * e1_e2v * d.e3v_n(p, k, c.m);
      const T zmskv = T(1) / fmx(wmsk<T>(cpn, k) + wmsk<T>(cp, k + 1) + wmsk<T>(cpn, k + 1) + wmsk<T>(cp, k), T(1));
      const T zcof2 = -pah * e1v * a.vslp[m3 + qq] * zmskv;
      const T zd = djt(a, cp, tb, qq, k, go + p, jpi);
      return (zabe2 * zd + zcof2 * (dk0(p + jpi, cpn, k) + dk1(p, cp, k) + dk1(p + jpi, cpn, k) + dk0(p, cp, k))) *
             vmsk<T>(cp, k);
    };
    // vertical flux ztfw at level k >= 2 (:298-357)
    auto tfw = [&](int k) -> T {
      const long qq = ij + (long)(k - 1) * n2;
      const T wm = wmsk<T>(ci, k);
      const T zmsku = wm / fmx(umsk<T>(ci, k - 1) + umsk<T>(ciw, k) + umsk<T>(ciw, k - 1) + umsk<T>(ci, k), T(1));
      const T zmskv = wm / fmx(vmsk<T>(ci, k - 1) + vmsk<T>(cis, k) + vmsk<T>(cis, k - 1) + vmsk<T>(ci, k), T(1));
      const T zahu_w = (ahu(d, a, ci, ij, k - 1, c.m) + ahu(d, a, ciw, ijw, k, c.m) + ahu(d, a, ciw, ijw, k - 1, c.m) +
                        ahu(d, a, ci, ij, k, c.m)) * zmsku;
      const T zahv_w = (ahv(d, a, ci, ij, k - 1, c.m) + ahv(d, a, cis, ijs, k, c.m) + ahv(d, a, cis, ijs, k - 1, c.m) +
                        ahv(d, a, ci, ij, k, c.m)) * zmskv;
      const T zcoef3 = -zahu_w * e2t * zmsku * a.wslpi[m3 + qq];
      const T zcoef4 = -zahv_w * e1t * zmskv * a.wslpj[m3 + qq];
      const long qm = qq - n2;
      const T sdi = dit(a, ci, tb, qm, k - 1, go + ij) + dit(a, ciw, tb, qq - 1, k, go + ijw) +
                    dit(a, ciw, tb, qm - 1, k - 1, go + ijw) + dit(a, ci, tb, qq, k, go + ij);
      const T sdj = djt(a, ci, tb, qm, k - 1, go + ij, jpi) + djt(a, cis, tb, qq - jpi, k, go + ijs, jpi) +
                    djt(a, cis, tb, qm - jpi, k - 1, go + ijs, jpi) + djt(a, ci, tb, qq, k, go + ij, jpi);
      T z = zcoef3 * sdi + zcoef4 * sdj;
      const T e3w = d.e3w_n(ij, k, c.m);
      const T ahw = a.ah_wslp2[m3 + qq], akzv = a.akz[m3 + qq];
      if (a.lap) {
        z = z + e1e2t / e3w * wm * (ahw - akzv) * (tb[qm] - tb[qq]);
      } else if (a.kpass == 1) {
        z = z + ahw * e1e2t * (tb[qm] - tb[qq]) / e3w * wm;
      } else {
        z = z + e1e2t / e3w * wm * (ahw * (tb[qm] - tb[qq]) + akzv * (tbb[qm] - tbb[qq]));
      }
      return z;
    };
    (void)cise; (void)cinw;
    T ztfw_t = T(0);  // ztfw(1) = 0
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = ij + (long)(k - 1) * n2;
      if (coefs && k + 1 <= jpk - 1) iso_coefs(d, a, ij, k + 1, c.m, ci, ciw, cis);
      const T zftu0 = ftu(ij, ci, cie, e2_e1u0, e2u0, k);
      const T zftuw = ftu(ijw, ciw, ci, e2_e1uw, e2uw, k);
      const T zftv0 = ftv(ij, ci, cin, e1_e2v0, e1v0, k);
      const T zftvs = ftv(ijs, cis, ci, e1_e2vs, e1vs, k);
      ta[q] = ta[q] + a.zsign * (zftu0 - zftuw + zftv0 - zftvs) * r1_e1e2t / d.e3t_n(ij, k, c.m);
      const T ztfw_b = (k + 1 <= jpk - 1) ? tfw(k + 1) : T(0);
      ta[q] = ta[q] + a.zsign * (ztfw_t - ztfw_b) * r1_e1e2t / d.e3t_n(ij, k, c.m);
      ztfw_t = ztfw_b;
    }
  }
}

// --------------------------------------------------------------------------------
// tra_zdf_imp (trazdf.F90:143-264) for the interior columns; pta becomes the after
// tracer. With clamp_sal the salinity WHERE( tsa < 0 ) tsa = 0.1 of trazdf.F90:83 is
// applied on the values this kernel writes.
template <class T>
struct ZdfArgs {
  T p2dt;
  const T* ptb;
  T* pta;
  int kjpt;
  const T *avt, *avs, *add;  // add: ah_wslp2 (standard iso), akz (msc) or NULL
  int ddm, is_trc, clamp_sal;
};

template <class T>
__global__ void k_zdf_imp(Dom<T> d, ZdfArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid || !c.interior) return;
  const int jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const ColInfo ci = d.ci[c.ij];
  const long m3 = (long)c.m * n3;
  T zwi[KMAX], zws[KMAX], zwt[KMAX];
  for (int n = 0; n < a.kjpt; ++n) {
    const bool build = (!a.is_trc && (n == 0 || (n == 1 && a.ddm))) || (a.is_trc && n == 0);
    if (build) {
      const T* coef = (!a.is_trc && n == 0) ? a.avt : a.avs;
      // zwt(k) = avt(k) (+ iso-neutral coefficient), zwt(1) = 0 (:153-176)
      auto wt = [&](int k) -> T {
        if (k == 1) return T(0);
        const long q = m3 + c.ij + (long)(k - 1) * n2;
        T v = coef[q];
        if (a.add && k <= jpk - 1) v = v + a.add[q];
        return v;
      };
      T wtk = wt(1);
      T g = T(0);
      for (int k = 1; k <= jpk - 1; ++k) {
        const T wtk1 = wt(k + 1);
        zwi[k] = -a.p2dt * wtk / d.e3w_n(c.ij, k, c.m);
        zws[k] = -a.p2dt * wtk1 / d.e3w_n(c.ij, k + 1, c.m);
        const T e3a = d.e3t_a(c.ij, k, c.m);
        if constexpr (sizeof(T) == 8) {
          // 1st recurrence as written in the reference (trazdf.F90:223-234)
          const T zwd = e3a - zwi[k] - zws[k];
          zwt[k] = (k == 1) ? zwd : zwd - zwi[k] * zws[k - 1] / zwt[k - 1];
        } else {
          // FP32: the same pivots without cancellation. With g(k) = zwt(k) + zws(k),
          // zwt(k) = zwd(k) - zwi(k) zws(k-1)/zwt(k-1) is g(k) - zws(k) where
          // g(k) = e3t_a(k) - zwi(k) g(k-1)/zwt(k-1): a sum of non-negative terms
          // (zwi, zws <= 0), whereas zwd - zwi zws/zwt cancels to O(e3t) from
          // O(p2dt avt/e3w) when the vertical diffusivity is large.
          g = (k == 1) ? e3a - zwi[k] : e3a - zwi[k] * (g / zwt[k - 1]);
          zwt[k] = g - zws[k];
        }
        wtk = wtk1;
      }
    }
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const T* tb = a.ptb + mo;
    T* ta = a.pta + mo;
    const bool clamp = a.clamp_sal && !a.is_trc && n == 1;
    // 2nd recurrence (:238-250), the forward values kept in pta as in the reference
    T prev = T(0);
    for (int k = 1; k <= jpk - 1; ++k) {
      const long q = c.ij + (long)(k - 1) * n2;
      const T zrhs = d.e3t_b(c.ij, k, c.m) * tb[q] + a.p2dt * d.e3t_n(c.ij, k, c.m) * ta[q];
      prev = (k == 1) ? zrhs : zrhs - zwi[k] / zwt[k - 1] * prev;
      ta[q] = prev;
    }
    // 3rd recurrence (:252-264)
    T nxt;
    {
      const int k = jpk - 1;
      const long q = c.ij + (long)(k - 1) * n2;
      nxt = ta[q] / zwt[k] * tmsk<T>(ci, k);
      ta[q] = (clamp && nxt < T(0)) ? T(0.1) : nxt;
    }
    for (int k = jpk - 2; k >= 1; --k) {
      const long q = c.ij + (long)(k - 1) * n2;
      nxt = (ta[q] - zws[k] * nxt) / zwt[k] * tmsk<T>(ci, k);
      ta[q] = (clamp && nxt < T(0)) ? T(0.1) : nxt;
    }
  }
}

// WHERE( x < 0 ) x = 0.1 (trazdf.F90:83) on n values.
template <class T>
__global__ void k_clamp_neg(T* x, long n) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  long s = (long)gridDim.x * blockDim.x;
  for (; i < n; i += s)
    if (x[i] < T(0)) x[i] = T(0.1);
}

}  // namespace nemo
