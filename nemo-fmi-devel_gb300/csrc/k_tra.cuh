// k_tra.cuh -- tracer kernels: transports, FCT advection (upstream + antidiffusive
// fluxes, Zalesak limiter, final trend), compact 4th-order vertical interpolation,
// laplacian and rotated iso-neutral lateral diffusion, implicit vertical diffusion.
//
// Stencil kernels map one thread to one (i,j,k) point: the grid is x = i (32 per
// block, coalesced), y = j, z = (member, level). No state is carried along k, so
// every level of every column is independent and the GPU has ~jpi*jpj*jpk threads
// to hide memory latency with; neighbour values (i+-1, j+-1, k+-1) come from L1/L2.
// A value a reference loop computes once and its neighbours reuse (a face flux, a
// limiter coefficient at k+1) is recomputed by each thread that needs it, with the
// same operands in the same order. Only genuine column recurrences (the compact
// interpolation and the implicit vertical solve) keep one thread per column.
//
// Indices i, j, k are 1-based as in the Fortran they restate, and every expression
// keeps the reference's association (the FP64 instantiation is compiled without
// FMA contraction, so it reproduces the reference's FP64 arithmetic operation by
// operation).
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

// column kernels: grid x = i, y = j, z = member
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

struct PtIdx {
  int i, j, k, m;
  long ij, q;  // column offset, offset within one (jpi,jpj,jpk) field
  bool valid, interior;
};

// point kernels: grid x = i, y = j, z = member * jpk + (k - 1)
template <class T>
__device__ __forceinline__ PtIdx pt_index(const Dom<T>& d) {
  PtIdx c;
  c.i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  c.j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  c.k = (int)(blockIdx.z % (unsigned)d.jpk) + 1;
  c.m = (int)(blockIdx.z / (unsigned)d.jpk);
  c.valid = c.i <= d.jpi && c.j <= d.jpj;
  c.interior = c.i >= 2 && c.i <= d.jpi - 1 && c.j >= 2 && c.j <= d.jpj - 1;
  c.ij = (long)(c.i - 1) + (long)(c.j - 1) * d.jpi;
  c.q = c.ij + (long)(c.k - 1) * d.n2;
  return c;
}

// --------------------------------------------------------------------------------
// traadv.F90:99-124: zun = e2u*e3u_n*un, zvn = e1v*e3v_n*vn, zwn = e1e2t*wn, 0 at jpk.
template <class T>
__global__ void k_adv_trp(Dom<T> d, const T* __restrict__ un, const T* __restrict__ vn,
                          const T* __restrict__ wn, T* __restrict__ zun, T* __restrict__ zvn,
                          T* __restrict__ zwn) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const long q = (long)c.m * d.n3 + c.q;
  if (c.k == d.jpk) {
    zun[q] = T(0); zvn[q] = T(0); zwn[q] = T(0);
    return;
  }
  zun[q] = d.e2u[c.ij] * d.e3u_n(c.ij, c.k, c.m) * un[q];
  zvn[q] = d.e1v[c.ij] * d.e3v_n(c.ij, c.k, c.m) * vn[q];
  zwn[q] = d.e1e2t[c.ij] * wn[q];
}

// Lateral diffusion arguments (also carried by the FCT kernels for the fused
// advection + iso-neutral trend of the hot path).
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
  T *zftu, *zftv, *ztfw;     // work: iso-neutral fluxes (jpi,jpj,jpk,kjpt)
};

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
  int with_iso;              // stage c also adds the iso-neutral trend (kpass 1) of `iso`
  LdfArgs<T> iso;
};

// Upstream transports at the faces of column (i,j) (traadv_fct.F90:123-145).
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
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk, k = c.k;
  const long n2 = d.n2, n3 = d.n3, q = c.q;
  const long mv = (long)c.m * n3;
  const T r1_6 = T(1) / T(6);
  const bool work = c.interior && k <= jpk - 1;
  ColInfo ci{}, ciw{}, cie{}, cis{}, cin{};
  T ue = T(0), uw = T(0), vn_ = T(0), vs = T(0), wt = T(0), wb = T(0), r1_e1e2t = T(0);
  T e3n = T(1), e3b = T(1), e3a = T(1);
  if (work) {
    ci = d.ci[c.ij]; ciw = d.ci[c.ij - 1]; cie = d.ci[c.ij + 1]; cis = d.ci[c.ij - jpi]; cin = d.ci[c.ij + jpi];
    ue = trp_u(d, a, c.ij, mv + q, k, c.m);
    uw = trp_u(d, a, c.ij - 1, mv + q - 1, k, c.m);
    vn_ = trp_v(d, a, c.ij, mv + q, k, c.m);
    vs = trp_v(d, a, c.ij - jpi, mv + q - jpi, k, c.m);
    wt = trp_w(d, a, c.ij, mv + q);
    if (k + 1 <= jpk - 1) wb = trp_w(d, a, c.ij, mv + q + n2);
    r1_e1e2t = d.r1_e1e2t[c.ij];
    e3n = d.e3t_n(c.ij, k, c.m); e3b = d.e3t_b(c.ij, k, c.m); e3a = d.e3t_a(c.ij, k, c.m);
  }
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const T* tb = a.ptb + mo;
    const T* tn = a.ptn + mo;
    T* ta = a.pta + mo;
    const T* tai = a.pta_in ? a.pta_in + mo : nullptr;
    if (!work) {
      a.zwi[mo + q] = T(0); a.ax[mo + q] = T(0); a.ay[mo + q] = T(0); a.az[mo + q] = T(0);
      if (!tai) ta[q] = T(0);
      else if (tai != ta) ta[q] = tai[q];
      continue;
    }
    const T tb0 = tb[q];
    const T zwx_e = ups(ue, tb0, tb[q + 1]), zwx_w = ups(uw, tb[q - 1], tb0);
    const T zwy_n = ups(vn_, tb0, tb[q + jpi]), zwy_s = ups(vs, tb[q - jpi], tb0);
    // upstream vertical fluxes at the top (k) and bottom (k+1) faces (:137-156)
    T zwz_t;
    if (k == 1) zwz_t = a.linssh ? wt * tb0 : T(0);
    else zwz_t = ups(wt, tb0, tb[q - n2]) * wmsk<T>(ci, k);
    const T zwz_b = (k + 1 <= jpk - 1) ? ups(wb, tb[q + n2], tb0) * wmsk<T>(ci, k + 1) : T(0);
    const T ztra = -(zwx_e - zwx_w + zwy_n - zwy_s + zwz_t - zwz_b) * r1_e1e2t;
    const T tm = tmsk<T>(ci, k);
    const T tin = tai ? tai[q] : T(0);
    ta[q] = tin + ztra / e3n * tm;
    a.zwi[mo + q] = (e3b * tb0 + a.p2dt * ztra) / e3a * tm;
    // horizontal antidiffusive fluxes (:180-251)
    const T tn0 = tn[q], tne = tn[q + 1], tnn = tn[q + jpi];
    T axv, ayv;
    if (a.kn_fct_h == 2) {
      axv = T(0.5) * ue * (tn0 + tne) - zwx_e;
      ayv = T(0.5) * vn_ * (tn0 + tnn) - zwy_n;
    } else {
      const T tnw = tn[q - 1], tns = tn[q - jpi];
      const T ztu_w = (tn0 - tnw) * umsk<T>(ciw, k);
      const T ztu_0 = (tne - tn0) * umsk<T>(ci, k);
      const T zltu0 = (ztu_0 + ztu_w) * r1_6;
      T zltue = T(0);
      if (c.i + 1 <= jpi - 1) zltue = ((tn[q + 2] - tne) * umsk<T>(cie, k) + ztu_0) * r1_6;
      const T ztv_s = (tn0 - tns) * vmsk<T>(cis, k);
      const T ztv_0 = (tnn - tn0) * vmsk<T>(ci, k);
      const T zltv0 = (ztv_0 + ztv_s) * r1_6;
      T zltvn = T(0);
      if (c.j + 1 <= d.jpj - 1) zltvn = ((tn[q + 2 * jpi] - tnn) * vmsk<T>(cin, k) + ztv_0) * r1_6;
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
      if (a.kn_fct_v == 2) azv = (wt * T(0.5) * (tn0 + tn[q - n2]) - zwz_t) * wmsk<T>(ci, k);
      else azv = (wt * a.ztw[mo + q] - zwz_t) * wmsk<T>(ci, k);
    }
    a.az[mo + q] = azv;
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
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk, k = c.k;
  const long n2 = d.n2, n3 = d.n3, q = c.q;
  const bool work = c.interior && k <= jpk - 1;
  const T zrtrn = T(1.e-15);
  ColInfo ci{}, ciw{}, cie{}, cis{}, cin{};
  T zbt = T(0);
  if (work) {
    ci = d.ci[c.ij]; ciw = d.ci[c.ij - 1]; cie = d.ci[c.ij + 1]; cis = d.ci[c.ij - jpi]; cin = d.ci[c.ij + jpi];
    zbt = d.e1e2t[c.ij] * d.e3t_n(c.ij, k, c.m) / a.p2dt;
  }
  const int km1 = k - 1 > 1 ? k - 1 : 1;
  const long qm = c.ij + (long)(km1 - 1) * n2, qp = q + n2;
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    if (!work) {
      a.betup[mo + q] = T(0); a.betdo[mo + q] = T(0);
      continue;
    }
    const T* tb = a.ptb + mo;
    const T* zwi = a.zwi + mo;
    const T* ax = a.ax + mo;
    const T* ay = a.ay + mo;
    const T* az = a.az + mo;
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
    a.betup[mo + q] = (up - zwi[q]) / (zpos + zrtrn) * zbt;
    a.betdo[mo + q] = (zwi[q] - dn) / (zneg + zrtrn) * zbt;
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

// tra_ldf_lap (traldf_lap_blp.F90:95-145) at one interior point.
template <class T>
__global__ void k_ldf_lap(Dom<T> d, LdfArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid || !c.interior || c.k > d.jpk - 1) return;
  const int jpi = d.jpi, k = c.k;
  const long n3 = d.n3, n2 = d.n2, q = c.q;
  const ColInfo ci = d.ci[c.ij], ciw = d.ci[c.ij - 1], cis = d.ci[c.ij - jpi];
  const long ijw = c.ij - 1, ijs = c.ij - jpi;
  const T zu0 = a.zsign * ahu(d, a, ci, c.ij, k, c.m) * d.e2_e1u[c.ij] * d.e3u_n(c.ij, k, c.m);
  const T zuw = a.zsign * ahu(d, a, ciw, ijw, k, c.m) * d.e2_e1u[ijw] * d.e3u_n(ijw, k, c.m);
  const T zv0 = a.zsign * ahv(d, a, ci, c.ij, k, c.m) * d.e1_e2v[c.ij] * d.e3v_n(c.ij, k, c.m);
  const T zvs = a.zsign * ahv(d, a, cis, ijs, k, c.m) * d.e1_e2v[ijs] * d.e3v_n(ijs, k, c.m);
  const T den = d.e1e2t[c.ij] * d.e3t_n(c.ij, k, c.m);
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const long go = ((long)c.m * a.kjpt + n) * n2;
    const T* tb = a.ptb + mo;
    T* ta = a.pta + mo;
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
    ta[q] = ta[q] + (ztu0 - ztuw + ztv0 - ztvs) / den;
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

// ah_wslp2 (traldf_iso.F90:146-164) and akz (:166-202) at one interior point, level
// 2 <= k <= jpkm1, first pass.
template <class T>
__device__ __forceinline__ void iso_coefs(const Dom<T>& d, const LdfArgs<T>& a, long ij, int k, int m,
                                          const ColInfo& ci, const ColInfo& ciw, const ColInfo& cis, T& ahw, T& akz) {
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
  ahw = zahu_w * wi * wi + zahv_w * wj * wj;
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
    akz = akzv;
  } else {
    akz = ahw;
  }
}

// Iso-neutral coefficients of interior point (ij, k) for one call: computed on the
// first pass (the point of level k writes them), read on the second.
template <class T>
__device__ __forceinline__ void iso_coefs_at(const Dom<T>& d, const LdfArgs<T>& a, long ij, int k, int m,
                                             const ColInfo& ci, const ColInfo& ciw, const ColInfo& cis, T& ahw,
                                             T& akz) {
  if (a.kpass == 1) {
    iso_coefs(d, a, ij, k, m, ci, ciw, cis, ahw, akz);
  } else {
    const long q = (long)m * d.n3 + ij + (long)(k - 1) * d.n2;
    ahw = a.ah_wslp2[q];
    akz = a.akz[q];
  }
}

// Iso-neutral fluxes of one point (traldf_iso.F90:146-357): on the first pass the
// coefficients ah_wslp2 / akz of the point (levels 2..jpkm1, interior); the
// horizontal fluxes zftu / zftv of the east and north faces (i <= jpim1,
// j <= jpjm1, k <= jpkm1, :255-276); the vertical flux ztfw of the top face
// (interior, levels 2..jpkm1; 0 at levels 1 and jpk, :291-357). Each flux is
// computed once, by the point that owns its face.
template <class T>
__global__ void k_iso_flux(Dom<T> d, LdfArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpj = d.jpj, jpk = d.jpk, k = c.k;
  const long n2 = d.n2, n3 = d.n3;
  const long ij = c.ij, ijw = ij - 1, ijs = ij - jpi;
  const long m3 = (long)c.m * n3;
  const bool hface = c.i <= jpi - 1 && c.j <= jpj - 1 && k <= jpk - 1;
  const bool vface = c.interior && k >= 2 && k <= jpk - 1;
  if (!hface && !(c.interior && (k == 1 || k == jpk))) return;
  const ColInfo ci = d.ci[ij];
  const ColInfo cie = d.ci[ij + (c.i <= jpi - 1 ? 1 : 0)];
  const ColInfo cin = d.ci[ij + (c.j <= jpj - 1 ? jpi : 0)];
  // tracer-independent coefficients, computed once (the flux stores below could
  // alias the metric arrays, so nothing is reloaded between tracers)
  T zabe1 = T(0), zcof1 = T(0), zabe2 = T(0), zcof2 = T(0);
  T umk = T(0), vmk = T(0), wk = T(0), wk1 = T(0), wke = T(0), wk1e = T(0), wkn = T(0), wk1n = T(0);
  if (hface) {
    T pah = ahu(d, a, ci, ij, k, c.m);
    zabe1 = pah * d.e2_e1u[ij] * d.e3u_n(ij, k, c.m);
    const T zmsku = T(1) / fmx(wmsk<T>(cie, k) + wmsk<T>(ci, k + 1) + wmsk<T>(cie, k + 1) + wmsk<T>(ci, k), T(1));
    zcof1 = -pah * d.e2u[ij] * a.uslp[m3 + c.q] * zmsku;
    pah = ahv(d, a, ci, ij, k, c.m);
    zabe2 = pah * d.e1_e2v[ij] * d.e3v_n(ij, k, c.m);
    const T zmskv = T(1) / fmx(wmsk<T>(cin, k) + wmsk<T>(ci, k + 1) + wmsk<T>(cin, k + 1) + wmsk<T>(ci, k), T(1));
    zcof2 = -pah * d.e1v[ij] * a.vslp[m3 + c.q] * zmskv;
    umk = umsk<T>(ci, k); vmk = vmsk<T>(ci, k);
    wk = wmsk<T>(ci, k); wk1 = wmsk<T>(ci, k + 1);
    wke = wmsk<T>(cie, k); wk1e = wmsk<T>(cie, k + 1);
    wkn = wmsk<T>(cin, k); wk1n = wmsk<T>(cin, k + 1);
  }
  T zcoef3 = T(0), zcoef4 = T(0), zvert = T(0), wm = T(0), ahw = T(0), akz = T(0);
  ColInfo ciw{}, cis{};
  if (vface) {
    ciw = d.ci[ijw]; cis = d.ci[ijs];
    iso_coefs_at(d, a, ij, k, c.m, ci, ciw, cis, ahw, akz);
    if (a.kpass == 1) {
      a.ah_wslp2[m3 + c.q] = ahw;
      a.akz[m3 + c.q] = akz;
    }
    wm = wmsk<T>(ci, k);
    const T zmsku = wm / fmx(umsk<T>(ci, k - 1) + umsk<T>(ciw, k) + umsk<T>(ciw, k - 1) + umsk<T>(ci, k), T(1));
    const T zmskv = wm / fmx(vmsk<T>(ci, k - 1) + vmsk<T>(cis, k) + vmsk<T>(cis, k - 1) + vmsk<T>(ci, k), T(1));
    const T zahu_w = (ahu(d, a, ci, ij, k - 1, c.m) + ahu(d, a, ciw, ijw, k, c.m) + ahu(d, a, ciw, ijw, k - 1, c.m) +
                      ahu(d, a, ci, ij, k, c.m)) * zmsku;
    const T zahv_w = (ahv(d, a, ci, ij, k - 1, c.m) + ahv(d, a, cis, ijs, k, c.m) + ahv(d, a, cis, ijs, k - 1, c.m) +
                      ahv(d, a, ci, ij, k, c.m)) * zmskv;
    zcoef3 = -zahu_w * d.e2t[ij] * zmsku * a.wslpi[m3 + c.q];
    zcoef4 = -zahv_w * d.e1t[ij] * zmskv * a.wslpj[m3 + c.q];
    // the laplacian diagonal term of :359-366 without its tracer difference
    if (a.lap) zvert = d.e1e2t[ij] / d.e3w_n(ij, k, c.m) * wm * (ahw - akz);
  }
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const long go = ((long)c.m * a.kjpt + n) * n2;
    const T* tb = a.ptb + mo;
    const T* tbb = a.ptbb + mo;
    const long qq = c.q;
    if (hface) {
      // vertical gradients (:250-254): zdk1t(k) = (tb(k)-tb(k+1))*wmask(k+1),
      // zdkt(k) = (tb(k-1)-tb(k))*wmask(k), zdkt(1) = zdk1t(1)
      const T t0 = tb[qq], t1 = tb[qq + n2], te = tb[qq + 1], te1 = tb[qq + 1 + n2];
      const T tn = tb[qq + jpi], tn1 = tb[qq + jpi + n2];
      const T dk1_0 = (t0 - t1) * wk1, dk1_e = (te - te1) * wk1e, dk1_n = (tn - tn1) * wk1n;
      T dk0_0, dk0_e, dk0_n;
      if (k == 1) {
        dk0_0 = dk1_0; dk0_e = dk1_e; dk0_n = dk1_n;
      } else {
        dk0_0 = (tb[qq - n2] - t0) * wk;
        dk0_e = (tb[qq + 1 - n2] - te) * wke;
        dk0_n = (tb[qq + jpi - n2] - tn) * wkn;
      }
      const T zdi = (a.zps && k == ci.mbku) ? a.pgu[go + ij] : (te - t0) * umk;
      const T zdj = (a.zps && k == ci.mbkv) ? a.pgv[go + ij] : (tn - t0) * vmk;
      a.zftu[mo + qq] = (zabe1 * zdi + zcof1 * (dk0_e + dk1_0 + dk1_e + dk0_0)) * umk;
      a.zftv[mo + qq] = (zabe2 * zdj + zcof2 * (dk0_n + dk1_0 + dk1_n + dk0_0)) * vmk;
    }
    if (c.interior) {
      T z = T(0);
      if (vface) {
        const long qm = qq - n2;
        const T sdi = dit(a, ci, tb, qm, k - 1, go + ij) + dit(a, ciw, tb, qq - 1, k, go + ijw) +
                      dit(a, ciw, tb, qm - 1, k - 1, go + ijw) + dit(a, ci, tb, qq, k, go + ij);
        const T sdj = djt(a, ci, tb, qm, k - 1, go + ij, jpi) + djt(a, cis, tb, qq - jpi, k, go + ijs, jpi) +
                      djt(a, cis, tb, qm - jpi, k - 1, go + ijs, jpi) + djt(a, ci, tb, qq, k, go + ij, jpi);
        z = zcoef3 * sdi + zcoef4 * sdj;
        if (a.lap) {
          z = z + zvert * (tb[qm] - tb[qq]);
        } else {
          const T e1e2t = d.e1e2t[ij];
          const T e3w = d.e3w_n(ij, k, c.m);
          if (a.kpass == 1) z = z + ahw * e1e2t * (tb[qm] - tb[qq]) / e3w * wm;
          else z = z + e1e2t / e3w * wm * (ahw * (tb[qm] - tb[qq]) + akz * (tbb[qm] - tbb[qq]));
        }
      }
      a.ztfw[mo + qq] = z;
    }
  }
}

// Divergence of the iso-neutral fluxes of tracer n at interior point (i,j,k), added
// to tav in the reference's order: horizontal (:278-284), then vertical (:359-366).
template <class T>
__device__ __forceinline__ T iso_div(const Dom<T>& d, const LdfArgs<T>& a, const PtIdx& c, int n, T tav) {
  const long mo = ((long)c.m * a.kjpt + n) * d.n3, q = c.q;
  const T r1 = d.r1_e1e2t[c.ij], e3tn = d.e3t_n(c.ij, c.k, c.m);
  const T* fu = a.zftu + mo;
  const T* fv = a.zftv + mo;
  const T* fw = a.ztfw + mo;
  tav = tav + a.zsign * (fu[q] - fu[q - 1] + fv[q] - fv[q - d.jpi]) * r1 / e3tn;
  tav = tav + a.zsign * (fw[q] - fw[q + d.n2]) * r1 / e3tn;
  return tav;
}

// tra_ldf_iso divergence step at one interior point (k <= jpkm1).
template <class T>
__global__ void k_iso_div(Dom<T> d, LdfArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid || !c.interior || c.k > d.jpk - 1) return;
  for (int n = 0; n < a.kjpt; ++n) {
    T* ta = a.pta + ((long)c.m * a.kjpt + n) * d.n3;
    ta[c.q] = iso_div(d, a, c, n, ta[c.q]);
  }
}

// FCT stage c: limit the fluxes (traadv_fct.F90:404-426) and add the divergence of
// the corrected fluxes to pta (:288-297); with_iso also adds the iso-neutral trend
// divergence of the same point from fluxes k_iso_flux computed (the tra_ldf call
// that follows tra_adv in step.F90:248-252).
template <class T>
__global__ void k_fct_c(Dom<T> d, FctArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid || !c.interior || c.k > d.jpk - 1) return;
  const int jpi = d.jpi, k = c.k;
  const long n2 = d.n2, n3 = d.n3, q = c.q;
  const T r1_e1e2t = d.r1_e1e2t[c.ij];
  const T e3n = d.e3t_n(c.ij, k, c.m);
  const bool w_lim = c.i - 1 >= 2;  // the face i-1 is limited only for i-1 >= 2 (then lbc: 0)
  const bool s_lim = c.j - 1 >= 2;
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const T* ax = a.ax + mo;
    const T* ay = a.ay + mo;
    const T* az = a.az + mo;
    const T* bu = a.betup + mo;
    const T* bd = a.betdo + mo;
    T* ta = a.pta + mo;
    const T bu0 = bu[q], bd0 = bd[q];
    const T axl = limit(ax[q], bd0, bu[q + 1], bu0, bd[q + 1]);
    const T axlw = w_lim ? limit(ax[q - 1], bd[q - 1], bu0, bu[q - 1], bd0) : T(0);
    const T ayl = limit(ay[q], bd0, bu[q + jpi], bu0, bd[q + jpi]);
    const T ayls = s_lim ? limit(ay[q - jpi], bd[q - jpi], bu0, bu[q - jpi], bd0) : T(0);
    // pcc(k) (not limited at k = 1) and pcc(k+1)
    const T azl_t = k >= 2 ? limit(az[q], bd0, bu[q - n2], bu0, bd[q - n2]) : az[q];
    const T azl_b = limit(az[q + n2], bd[q + n2], bu0, bu[q + n2], bd0);
    T tav = ta[q] - (axl - axlw + ayl - ayls + azl_t - azl_b) * r1_e1e2t / e3n;
    if (a.with_iso) tav = iso_div(d, a.iso, c, n, tav);
    ta[q] = tav;
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

// Any jpk <= KMAX, the reference's recurrences with the pivots in local memory; in
// double precision the operations are those of trazdf.F90:218-264 in order.
template <class T>
__global__ void k_zdf_imp(Dom<T> d, ZdfArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid || !c.interior) return;
  const int jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const ColInfo ci = d.ci[c.ij];
  const long m3 = (long)c.m * n3;
  // rat(k) = zwi(k) / zwt(k-1): the tracer-independent factor of the 2nd recurrence
  T rat[KMAX], zws[KMAX], zwt[KMAX];
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
        const T zwi = -a.p2dt * wtk / d.e3w_n(c.ij, k, c.m);
        zws[k] = -a.p2dt * wtk1 / d.e3w_n(c.ij, k + 1, c.m);
        const T e3a = d.e3t_a(c.ij, k, c.m);
        if (k >= 2) rat[k] = zwi / zwt[k - 1];
        if constexpr (sizeof(T) == 8) {
          // 1st recurrence as written in the reference (trazdf.F90:223-234)
          const T zwd = e3a - zwi - zws[k];
          zwt[k] = (k == 1) ? zwd : zwd - zwi * zws[k - 1] / zwt[k - 1];
        } else {
          // FP32: the same pivots without cancellation. With g(k) = zwt(k) + zws(k),
          // zwt(k) = zwd(k) - zwi(k) zws(k-1)/zwt(k-1) is g(k) - zws(k) where
          // g(k) = e3t_a(k) - zwi(k) g(k-1)/zwt(k-1): a sum of non-negative terms
          // (zwi, zws <= 0), whereas zwd - zwi zws/zwt cancels to O(e3t) from
          // O(p2dt avt/e3w) when the vertical diffusivity is large.
          g = (k == 1) ? e3a - zwi : e3a - zwi * (g / zwt[k - 1]);
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
      prev = (k == 1) ? zrhs : zrhs - rat[k] * prev;
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

// FP32, jpk = NK known at compile time: each column is loaded whole into registers
// before it is solved (all its loads in flight at once, no load waiting on a store),
// then stored whole. The same elimination as k_zdf_imp with two register arrays:
// zw(k) = zwi(k) (zws(k) is zwi(k+1): both are -p2dt zwt(k+1) / e3w(k+1)) and the
// reciprocal pivots 1 / zwt(k).
template <int NK>
__global__ void __launch_bounds__(128) k_zdf_imp_reg(Dom<float> d, ZdfArgs<float> a) {
  ColIdx<float> c = col_index(d);
  if (!c.valid || !c.interior) return;
  constexpr int K1 = NK - 1;  // levels solved: 1..jpk-1
  const long n2 = d.n2, n3 = d.n3;
  const ColInfo ci = d.ci[c.ij];
  const long m3 = (long)c.m * n3;
  const float p2dt = a.p2dt;
  float zw[NK + 1], rzwt[NK];
  for (int n = 0; n < a.kjpt; ++n) {
    const bool build = (!a.is_trc && (n == 0 || (n == 1 && a.ddm))) || (a.is_trc && n == 0);
    if (build) {
      const float* coef = (!a.is_trc && n == 0) ? a.avt : a.avs;
      float wt[NK + 1];
#pragma unroll
      for (int k = 2; k <= NK; ++k) {
        const long q = m3 + c.ij + (long)(k - 1) * n2;
        wt[k] = coef[q];
        if (a.add && k <= NK - 1) wt[k] = wt[k] + a.add[q];
      }
      zw[1] = -p2dt * 0.0f / d.e3w_n(c.ij, 1, c.m);
#pragma unroll
      for (int k = 2; k <= NK; ++k) zw[k] = -p2dt * wt[k] / d.e3w_n(c.ij, k, c.m);
      float g = 0.0f;
#pragma unroll
      for (int k = 1; k <= K1; ++k) {
        const float e3a = d.e3t_a(c.ij, k, c.m);
        g = (k == 1) ? e3a - zw[1] : e3a - zw[k] * (g * rzwt[k - 1]);
        rzwt[k] = 1.0f / (g - zw[k + 1]);
      }
    }
    const long mo = ((long)c.m * a.kjpt + n) * n3 + c.ij;
    const float* tb = a.ptb + mo;
    float* ta = a.pta + mo;
    const bool clamp = a.clamp_sal && !a.is_trc && n == 1;
    float x[NK];
#pragma unroll
    for (int k = 1; k <= K1; ++k) x[k] = ta[(long)(k - 1) * n2];
    float prev = 0.0f;
#pragma unroll
    for (int k = 1; k <= K1; ++k) {
      const float zrhs = d.e3t_b(c.ij, k, c.m) * tb[(long)(k - 1) * n2] + p2dt * d.e3t_n(c.ij, k, c.m) * x[k];
      prev = (k == 1) ? zrhs : zrhs - zw[k] * rzwt[k - 1] * prev;
      x[k] = prev;
    }
    float nxt = 0.0f;
#pragma unroll
    for (int k = K1; k >= 1; --k) {
      nxt = (k == K1 ? x[k] : x[k] - zw[k + 1] * nxt) * rzwt[k] * tmsk<float>(ci, k);
      ta[(long)(k - 1) * n2] = (clamp && nxt < 0.0f) ? 0.1f : nxt;
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
