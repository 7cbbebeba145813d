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

// k-march kernels: grid x = i, y = j, z = member * nchunk + chunk. A thread walks
// the levels k0..k1 of one column (KCH levels per chunk), keeping in registers what
// level k+1 shares with level k, so the vertical neighbours are loaded once.
constexpr int KCH = 16;
struct KIdx {
  int i, j, m, k0, k1;
  long ij;
  bool valid, interior;
};
template <class T>
__device__ __forceinline__ KIdx k_index(const Dom<T>& d) {
  const int nch = (d.jpk + KCH - 1) / KCH;
  KIdx c;
  c.i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  c.j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  c.m = (int)(blockIdx.z / (unsigned)nch);
  const int ch = (int)blockIdx.z - c.m * nch;
  c.k0 = ch * KCH + 1;
  c.k1 = c.k0 + KCH - 1 < d.jpk ? c.k0 + KCH - 1 : d.jpk;
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
  RO<T> pahu, pahv;          // NULL: aht_c * umask/vmask above jpk (ldftra.F90:292-372)
  T aht_c;
  RO<T> pgu, pgv;            // partial-step gradients (jpi,jpj,kjpt) when zps
  int zps;
  RO<T> ptb, ptbb;
  T* pta;
  int kjpt, kpass;
  T zsign;
  // iso-neutral
  RO<T> uslp, vslp, wslpi, wslpj;
  T *ah_wslp2, *akz;
  int lap, blp, msc;
  T z2dt, z1_2dt;
  T *zftu, *zftv, *ztfw;     // work: iso-neutral fluxes (jpi,jpj,jpk,kjpt)
  int tma;                   // FP32 hot configuration: stage the tracer planes by TMA
  int* err;                  // device error flag (a timed-out wait of the TMA kernel)
  int polls;                 // bound of each wait on a tensor copy (polls of <= ~1 us)
};

// Arguments shared by the three FCT kernels.
template <class T>
struct FctArgs {
  T p2dt;
  T r1_p2dt;                 // 1 / p2dt, correctly rounded
  RO<T> pun, pvn, pwn;       // transports, or velocities when trp != 0
  int trp;                   // 1: scale velocities to transports on the fly (traadv.F90:110-114)
  RO<T> ptb, ptn;            // (jpi,jpj,jpk,kjpt)
  const T* pta_in;           // NULL: the trend starts from tsa = 0 (step.F90:234)
  T* pta;                    // (jpi,jpj,jpk,kjpt)
  T *zwi, *ax, *ay, *az;     // work: monotone guess and antidiffusive fluxes (jpi,jpj,jpk,kjpt)
  T *betup, *betdo;          // work: limiter coefficients (jpi,jpj,jpk,kjpt)
  RO<T> ztw;                 // compact 4th-order tn at w-points (kn_fct_v = 4), or NULL
  int kjpt, kn_fct_h, kn_fct_v, linssh;
  int with_iso;              // stage c also adds the iso-neutral trend (kpass 1) of `iso`
  LdfArgs<T> iso;
  int tma;                   // FP32 hot configuration: stage the planes by TMA
  int fused;                 // with tma: the three stages as one kernel (k_fct_fused_tma)
  int* err;                  // device error flag (a timed-out wait of a TMA kernel)
  int polls;                 // bound of each wait on a tensor copy (polls of <= ~1 us)
  T* lim;                    // NULL, or where k_fct_c records the limiter multipliers
                             // ((member*kjpt + n)*3 + face)*n3, for the adjoint
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
// ---- value-exact helpers of the FCT and iso-neutral kernels. FP64 runs at 1/64 of
// the FP32 rate on this GPU, and compares, min/max and products by 0/1 masks all
// occupy that pipe; these forms move them to the integer pipe or drop them while
// giving the reference's values (at most the sign of a zero differs, which no later
// operation of these routines can see: zeros are added, multiplied or compared
// with SIGN of key_nosignedzero).

// the sign bit of x is clear (x > 0 or x = +0; -0 counts as negative)
template <class T>
__device__ __forceinline__ bool sgn_pos(T x) {
  if constexpr (sizeof(T) == 8) return __double2hiint(x) >= 0;
  else return __float_as_int(x) >= 0;
}
// integer with the order of the FP64 values (-0 just below +0)
__device__ __forceinline__ long long ord_key(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
// MAX / MIN of two values: FP64 through the integer order of the values, FP32 by
// the min/max instruction
template <class T>
__device__ __forceinline__ T vmax(T a, T b) {
  if constexpr (sizeof(T) == 8) return ord_key(a) > ord_key(b) ? a : b;
  else return fmaxf(a, b);
}
template <class T>
__device__ __forceinline__ T vmin(T a, T b) {
  if constexpr (sizeof(T) == 8) return ord_key(a) < ord_key(b) ? a : b;
  else return fminf(a, b);
}
// MAX(0, x) and MIN(0, x)
template <class T>
__device__ __forceinline__ T pos_part(T x) { return sgn_pos(x) ? x : T(0); }
template <class T>
__device__ __forceinline__ T neg_part(T x) { return sgn_pos(x) ? T(0) : x; }
// x * m for a 0/1 mask m: FP64 selects (no product), FP32 keeps the product
template <class T>
__device__ __forceinline__ T msel(T x, T m) {
  if constexpr (sizeof(T) == 8) return __double2hiint(m) != 0 ? x : T(0);
  else return x * m;
}
// x / y given ry = 1 / y correctly rounded. FP64: Markstein's final correction
// (P. Markstein, IBM J. Res. Dev. 34, 1990): with q0 = x * ry the remainder
// e = x - q0 * y is exact as one fused multiply-add and q0 + e * ry rounds to the
// correctly rounded quotient, i.e. the reference's x / y, in three FP64 operations
// instead of a division. FP32: the division itself.
template <class T>
__device__ __forceinline__ T divq(T x, T y, T ry) {
  if constexpr (sizeof(T) == 8) {
    const double q0 = __dmul_rn(x, ry);
    return __fma_rn(__fma_rn(-q0, y, x), ry, q0);
  } else {
    (void)ry;
    return x / y;
  }
}

// Upstream flux 0.5 * ((u + |u|) * tl + (u - |u|) * tr) (traadv_fct.F90:126-136):
// exactly u * tl for u > 0 and u * tr for u < 0 (the doubled product scales exactly
// and the other term is an exact 0), formed as one product of the selected value.
// The product is rounded on its own (no contraction into the sum that follows), so
// every kernel that forms this flux gets the same value.
template <class T>
__device__ __forceinline__ T rmul(T a, T b) {
  if constexpr (sizeof(T) == 8) return __dmul_rn(a, b);
  else return __fmul_rn(a, b);
}
template <class T>
__device__ __forceinline__ T ups(T u, T tl, T tr) {
  return rmul(u, sgn_pos(u) ? tl : tr);
}

// FCT stage a: upstream trend into pta, monotone guess zwi, antidiffusive fluxes
// (traadv_fct.F90:119-278) with the lbc_lnk of :280 folded in (edge values 0).
// k-march: the upstream flux through the w-face between levels k and k+1 is
// computed once (the bottom flux of k is the top flux of k+1), and tb, tn of
// level k and the transport through that face are carried to level k+1.
template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 3) k_fct_a(Dom<T> d, FctArgs<T> a) {
  const KIdx c = k_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3, ij = c.ij;
  if (!c.interior) {  // edge columns: every level 0 (pta: its input)
    for (int k = c.k0; k <= c.k1; ++k) {
      const long q = ij + (long)(k - 1) * n2;
      for (int n = 0; n < a.kjpt; ++n) {
        const long mo = ((long)c.m * a.kjpt + n) * n3;
        a.zwi[mo + q] = T(0); a.ax[mo + q] = T(0); a.ay[mo + q] = T(0); a.az[mo + q] = T(0);
        T* ta = a.pta + mo;
        const T* tai = a.pta_in ? a.pta_in + mo : nullptr;
        if (!tai) ta[q] = T(0);
        else if (tai != ta) ta[q] = tai[q];
      }
    }
    return;
  }
  const long mv = (long)c.m * n3;
  const ColInfo ci = d.ci[ij], ciw = d.ci[ij - 1], cie = d.ci[ij + 1], cis = d.ci[ij - jpi], cin = d.ci[ij + jpi];
  const T r1_e1e2t = d.r1_e1e2t[ij];
  const T r1_6 = T(1) / T(6);
  constexpr int NT = 2;  // tracers per pass over the levels
  for (int n0 = 0; n0 < a.kjpt; n0 += NT) {
    const int nt = a.kjpt - n0 < NT ? a.kjpt - n0 : NT;
    // carried from level k-1: tb(k-1), tn(k-1), the bottom upstream flux of k-1
    T tbp[NT] = {}, tnp[NT] = {}, zwzb[NT] = {};
    T wt = T(0);  // transport through the top face of level k
    for (int k = c.k0; k <= c.k1; ++k) {
      const long q = ij + (long)(k - 1) * n2;
      if (k == jpk) {  // level jpk: no work, edge values
        for (int nn = 0; nn < nt; ++nn) {
          const long mo = ((long)c.m * a.kjpt + n0 + nn) * n3;
          a.zwi[mo + q] = T(0); a.ax[mo + q] = T(0); a.ay[mo + q] = T(0); a.az[mo + q] = T(0);
          T* ta = a.pta + mo;
          const T* tai = a.pta_in ? a.pta_in + mo : nullptr;
          if (!tai) ta[q] = T(0);
          else if (tai != ta) ta[q] = tai[q];
        }
        continue;
      }
      const bool first = k == c.k0;
      const T ue = trp_u(d, a, ij, mv + q, k, c.m);
      const T uw = trp_u(d, a, ij - 1, mv + q - 1, k, c.m);
      const T vn_ = trp_v(d, a, ij, mv + q, k, c.m);
      const T vs = trp_v(d, a, ij - jpi, mv + q - jpi, k, c.m);
      if (first) wt = trp_w(d, a, ij, mv + q);
      const T wb = (k + 1 <= jpk - 1) ? trp_w(d, a, ij, mv + q + n2) : T(0);
      const T e3n = d.e3t_n(ij, k, c.m), e3b = d.e3t_b(ij, k, c.m), e3a = d.e3t_a(ij, k, c.m);
      const T tm = tmsk<T>(ci, k), wk = wmsk<T>(ci, k), wk1 = wmsk<T>(ci, k + 1);
#pragma unroll
      for (int nn = 0; nn < NT; ++nn) {
        if (nn >= nt) break;
        const long mo = ((long)c.m * a.kjpt + n0 + nn) * n3;
        const RO<T> tb = a.ptb + mo;
        const RO<T> tn = a.ptn + mo;
        T* ta = a.pta + mo;
        const T* tai = a.pta_in ? a.pta_in + mo : nullptr;
        const T tb0 = tb[q];
        if (first && k > 1) {  // the carried values of level k-1
          tbp[nn] = tb[q - n2];
          tnp[nn] = tn[q - n2];
          zwzb[nn] = ups(wt, tb0, tbp[nn]) * wk;
        }
        const T zwx_e = ups(ue, tb0, tb[q + 1]), zwx_w = ups(uw, tb[q - 1], tb0);
        const T zwy_n = ups(vn_, tb0, tb[q + jpi]), zwy_s = ups(vs, tb[q - jpi], tb0);
        // upstream vertical fluxes at the top (k) and bottom (k+1) faces (:137-156)
        const T zwz_t = (k == 1) ? (a.linssh ? wt * tb0 : T(0)) : zwzb[nn];
        const T zwz_b = (k + 1 <= jpk - 1) ? ups(wb, tb[q + n2], tb0) * wk1 : T(0);
        const T ztra = -(zwx_e - zwx_w + zwy_n - zwy_s + zwz_t - zwz_b) * r1_e1e2t;
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
          if (a.kn_fct_v == 2) azv = (wt * T(0.5) * (tn0 + tnp[nn]) - zwz_t) * wk;
          else azv = (wt * a.ztw[mo + q] - zwz_t) * wk;
        }
        a.az[mo + q] = azv;
        tbp[nn] = tb0;
        tnp[nn] = tn0;
        zwzb[nn] = zwz_b;
      }
      wt = wb;
    }
  }
}

// zbup / zbdo of nonosc (traadv_fct.F90:361-364) at one point.
// With tm = 1 the reference's pbef*tm - zbig*(1-tm) is pbef exactly, with tm = 0 it is
// -zbig (pbef, paft finite), so the masked extrema reduce to a select.
template <class T>
__device__ __forceinline__ void bupdo(T pbef, T paft, T tm, T& up, T& dn) {
  const T zbig = Big<T>::v;
  bool wet;
  if constexpr (sizeof(T) == 8) wet = __double2hiint(tm) != 0;  // tm is 0 or 1
  else wet = tm != T(0);
  up = wet ? vmax(pbef, paft) : -zbig;
  dn = wet ? vmin(pbef, paft) : zbig;
}
// FCT stage b: nonosc extrema and limiter coefficients zbetup / zbetdo
// (traadv_fct.F90:366-400), edge values 0 (lbc_lnk of :400). k-march: tb, zwi and
// their masked extrema of levels k and k+1 and az(k+1) are carried down.
template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 4) k_fct_b(Dom<T> d, FctArgs<T> a) {
  const KIdx c = k_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3, ij = c.ij;
  const T zrtrn = T(1.e-15);
  auto zero = [&](int k) {
    const long q = ij + (long)(k - 1) * n2;
    for (int n = 0; n < a.kjpt; ++n) {
      const long mo = ((long)c.m * a.kjpt + n) * n3;
      a.betup[mo + q] = T(0);
      a.betdo[mo + q] = T(0);
    }
  };
  if (!c.interior) {
    for (int k = c.k0; k <= c.k1; ++k) zero(k);
    return;
  }
  const ColInfo ci = d.ci[ij], ciw = d.ci[ij - 1], cie = d.ci[ij + 1], cis = d.ci[ij - jpi], cin = d.ci[ij + jpi];
  const T e1e2t = d.e1e2t[ij];
  constexpr int NT = 2;
  for (int n0 = 0; n0 < a.kjpt; n0 += NT) {
    const int nt = a.kjpt - n0 < NT ? a.kjpt - n0 : NT;
    // carried: masked extrema (up, dn) of the column at level k-1 and k, az(k)
    T upm[NT] = {}, dnm[NT] = {}, up0[NT] = {}, dn0[NT] = {}, azk[NT] = {}, zwik[NT] = {};
    for (int k = c.k0; k <= c.k1; ++k) {
      if (k == jpk) {
        const long q = ij + (long)(k - 1) * n2;
        for (int nn = 0; nn < nt; ++nn) {
          const long mo = ((long)c.m * a.kjpt + n0 + nn) * n3;
          a.betup[mo + q] = T(0);
          a.betdo[mo + q] = T(0);
        }
        continue;
      }
      const bool first = k == c.k0;
      const long q = ij + (long)(k - 1) * n2, qp = q + n2;
      const T zbt = e1e2t * d.e3t_n(ij, k, c.m) / a.p2dt;
#pragma unroll
      for (int nn = 0; nn < NT; ++nn) {
        if (nn >= nt) break;
        const long mo = ((long)c.m * a.kjpt + n0 + nn) * n3;
        const RO<T> tb = a.ptb + mo;
        const RO<T> zwi = a.zwi + mo;
        const RO<T> ax = a.ax + mo;
        const RO<T> ay = a.ay + mo;
        const RO<T> az = a.az + mo;
        if (first) {  // extrema of the column at levels k and k-1, az(k)
          zwik[nn] = zwi[q];
          bupdo(tb[q], zwik[nn], tmsk<T>(ci, k), up0[nn], dn0[nn]);
          if (k > 1) bupdo(tb[q - n2], zwi[q - n2], tmsk<T>(ci, k - 1), upm[nn], dnm[nn]);
          else { upm[nn] = up0[nn]; dnm[nn] = dn0[nn]; }
          azk[nn] = az[q];
        }
        T upp, dnp;  // level k+1 of the column
        bupdo(tb[qp], zwi[qp], tmsk<T>(ci, k + 1), upp, dnp);
        // the reference's order: centre, west, east, south, north, above, below
        T up = up0[nn], dn = dn0[nn], u2, d2;
        bupdo(tb[q - 1], zwi[q - 1], tmsk<T>(ciw, k), u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        bupdo(tb[q + 1], zwi[q + 1], tmsk<T>(cie, k), u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        bupdo(tb[q - jpi], zwi[q - jpi], tmsk<T>(cis, k), u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        bupdo(tb[q + jpi], zwi[q + jpi], tmsk<T>(cin, k), u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        up = vmax(up, upm[nn]); dn = vmin(dn, dnm[nn]);
        up = vmax(up, upp); dn = vmin(dn, dnp);
        const T axw = ax[q - 1], ax0 = ax[q], ays = ay[q - jpi], ay0 = ay[q], az0 = azk[nn], azb = az[qp];
        const T zpos = pos_part(axw) - neg_part(ax0) + pos_part(ays) - neg_part(ay0) + pos_part(azb) - neg_part(az0);
        const T zneg = pos_part(ax0) - neg_part(axw) + pos_part(ay0) - neg_part(ays) + pos_part(az0) - neg_part(azb);
        const T zw = zwik[nn];
        a.betup[mo + q] = (up - zw) / (zpos + zrtrn) * zbt;
        a.betdo[mo + q] = (zw - dn) / (zneg + zrtrn) * zbt;
        upm[nn] = up0[nn]; dnm[nn] = dn0[nn];
        up0[nn] = upp; dn0[nn] = dnp;
        azk[nn] = azb;
        zwik[nn] = zwi[qp];
      }
    }
  }
}

// Limiter multiplier of an antidiffusive flux f (traadv_fct.F90:407-422): c*a + (1-c)*b.
// With zc = 0.5 + SIGN(0.5, f) in {0, 1} the sum is exactly a where f >= 0 and b
// where f < 0 (products by 1 and 0 are exact), so the operands are selected first.
template <class T>
__device__ __forceinline__ T limit_mult(T f, T bdo0, T bup1, T bup0, T bdo1) {
  const bool p = sgn_pos(f);
  return vmin(T(1), vmin(p ? bdo0 : bup0, p ? bup1 : bdo1));
}
// Limited antidiffusive flux: f * ( c*a + (1-c)*b ).
template <class T>
__device__ __forceinline__ T limit(T f, T bdo0, T bup1, T bup0, T bdo1) {
  return rmul(f, limit_mult(f, bdo0, bup1, bup0, bdo1));
}

// interp_4th_cpt (traadv_fct.F90:517-616): compact 4th-order tn at w-points for the
// interior columns, levels 2..jpkm1, one tridiagonal solve per column.
template <class T>
__global__ void k_interp4(Dom<T> d, RO<T> ptn, T* __restrict__ ztw, int kjpt) {
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
    const RO<T> t = ptn + mo;
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
// Eddy diffusivity at a u (v) point: the bound array, else aht_c * umask (vmask)
// above level jpk. W: the caller guarantees k < jpk and a wet point.
template <bool W = false, class T>
__device__ __forceinline__ T ahu(const Dom<T>& d, const LdfArgs<T>& a, const ColInfo& c, long ij, int k, int m) {
  if (a.pahu) return a.pahu[(long)m * d.n3 + ij + (long)(k - 1) * d.n2];
  if constexpr (W) return a.aht_c * T(1);
  else return k < d.jpk ? a.aht_c * umsk<T>(c, k) : T(0);
}
template <bool W = false, class T>
__device__ __forceinline__ T ahv(const Dom<T>& d, const LdfArgs<T>& a, const ColInfo& c, long ij, int k, int m) {
  if (a.pahv) return a.pahv[(long)m * d.n3 + ij + (long)(k - 1) * d.n2];
  if constexpr (W) return a.aht_c * T(1);
  else return k < d.jpk ? a.aht_c * vmsk<T>(c, k) : T(0);
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
    const RO<T> tb = a.ptb + mo;
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
template <bool W = false, class T>
__device__ __forceinline__ T dit(const LdfArgs<T>& a, const ColInfo& c, const RO<T>& tb, long q, int k, long g) {
  if (a.zps && k == c.mbku) return a.pgu[g];
  return (tb[q + 1] - tb[q]) * umk<W, T>(c, k);
}
template <bool W = false, class T>
__device__ __forceinline__ T djt(const LdfArgs<T>& a, const ColInfo& c, const RO<T>& tb, long q, int k, long g, int jpi) {
  if (a.zps && k == c.mbkv) return a.pgv[g];
  return (tb[q + jpi] - tb[q]) * vmk<W, T>(c, k);
}

// w-point mask weights and averaged eddy diffusivities of an interior point, level
// 2 <= k <= jpkm1 (traldf_iso.F90:150-157 and :297-304: the same expressions)
template <class T>
struct IsoW {
  T zmsku, zmskv, zahu_w, zahv_w;
};
template <bool W = false, class T>
__device__ __forceinline__ IsoW<T> iso_w(const Dom<T>& d, const LdfArgs<T>& a, long ij, int k, int m,
                                         const ColInfo& ci, const ColInfo& ciw, const ColInfo& cis) {
  const int jpi = d.jpi;
  const T wm = wmk<W, T>(ci, k);
  IsoW<T> w;
  w.zmsku = wm * rcount(umk<W, T>(ci, k - 1) + umk<W, T>(ciw, k) + umk<W, T>(ciw, k - 1) + umk<W, T>(ci, k));
  w.zmskv = wm * rcount(vmk<W, T>(ci, k - 1) + vmk<W, T>(cis, k) + vmk<W, T>(cis, k - 1) + vmk<W, T>(ci, k));
  w.zahu_w = (ahu<W>(d, a, ci, ij, k - 1, m) + ahu<W>(d, a, ciw, ij - 1, k, m) + ahu<W>(d, a, ciw, ij - 1, k - 1, m) +
              ahu<W>(d, a, ci, ij, k, m)) * w.zmsku;
  w.zahv_w = (ahv<W>(d, a, ci, ij, k - 1, m) + ahv<W>(d, a, cis, ij - jpi, k, m) + ahv<W>(d, a, cis, ij - jpi, k - 1, m) +
              ahv<W>(d, a, ci, ij, k, m)) * w.zmskv;
  return w;
}

// ah_wslp2 (traldf_iso.F90:146-164) and akz (:166-202) at one interior point, level
// 2 <= k <= jpkm1: computed on the first pass, read back on the second.
template <bool W = false, class T>
__device__ __forceinline__ void iso_coefs_at(const Dom<T>& d, const LdfArgs<T>& a, long ij, int k, int m,
                                             const ColInfo& ci, const ColInfo& ciw, const ColInfo& cis,
                                             const IsoW<T>& w, T& ahw, T& akz) {
  const long q = (long)m * d.n3 + ij + (long)(k - 1) * d.n2;
  if (a.kpass != 1) {
    ahw = a.ah_wslp2[q];
    akz = a.akz[q];
    return;
  }
  const int jpi = d.jpi;
  const T wi = a.wslpi[q], wj = a.wslpj[q];
  ahw = w.zahu_w * wi * wi + w.zahv_w * wj * wj;
  if (a.msc) {
    const T e1u0 = d.e1u[ij], e1uw = d.e1u[ij - 1], e2v0 = d.e2v[ij], e2vs = d.e2v[ij - jpi];
    T akzv = T(0.25) * ((ahu<W>(d, a, ci, ij, k, m) + ahu<W>(d, a, ci, ij, k - 1, m)) / (e1u0 * e1u0) +
                        (ahu<W>(d, a, ciw, ij - 1, k, m) + ahu<W>(d, a, ciw, ij - 1, k - 1, m)) / (e1uw * e1uw) +
                        (ahv<W>(d, a, ci, ij, k, m) + ahv<W>(d, a, ci, ij, k - 1, m)) / (e2v0 * e2v0) +
                        (ahv<W>(d, a, cis, ij - jpi, k, m) + ahv<W>(d, a, cis, ij - jpi, k - 1, m)) / (e2vs * e2vs));
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

// Iso-neutral fluxes (traldf_iso.F90:146-357) of one column, k-march: on the first
// pass the coefficients ah_wslp2 / akz (levels 2..jpkm1, interior); the horizontal
// fluxes zftu / zftv of the east and north faces (i <= jpim1, j <= jpjm1,
// k <= jpkm1, :255-276); the vertical flux ztfw of the top face of each level
// (interior; 0 at levels 1 and jpk, :291-357). Each flux is computed once, by the
// column that owns its face. Carried from level k to k+1: tb of the three columns
// whose differences the fluxes take, the vertical gradients zdk1t(k) (= zdkt(k+1))
// and the four horizontal gradients zdit / zdjt that the w-face flux averages.
template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 3) k_iso_flux(Dom<T> d, LdfArgs<T> a) {
  const KIdx c = k_index(d);
  if (!c.valid) return;
  const int jpi = d.jpi, jpj = d.jpj, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3, ij = c.ij, ijw = ij - 1, ijs = ij - jpi;
  const long m3 = (long)c.m * n3;
  if (!(c.i <= jpi - 1 && c.j <= jpj - 1)) return;  // no face owned (interior columns are inside)
  const bool icol = c.interior;
  const ColInfo ci = d.ci[ij], cie = d.ci[ij + 1], cin = d.ci[ij + jpi];
  ColInfo ciw{}, cis{};
  if (icol) {
    ciw = d.ci[ijw];
    cis = d.ci[ijs];
  }
  constexpr int NT = 2;
  for (int n0 = 0; n0 < a.kjpt; n0 += NT) {
    const int nt = a.kjpt - n0 < NT ? a.kjpt - n0 : NT;
    // carried, per tracer: tb(k) at (i,j), (i+1,j), (i,j+1); zdk1t(k-1) there; zdit at
    // (i,j) and (i-1,j) and zdjt at (i,j) and (i,j-1) of level k-1; tb(k-1) at (i,j)
    T t0c[NT] = {}, tec[NT] = {}, tnc[NT] = {}, k10[NT] = {}, k1e[NT] = {}, k1n[NT] = {};
    T di0[NT] = {}, diw[NT] = {}, dj0[NT] = {}, djs[NT] = {}, tup[NT] = {};
    for (int k = c.k0; k <= c.k1; ++k) {
      const long q = ij + (long)(k - 1) * n2;
      if (k == jpk) {  // interior: ztfw = 0 at jpk
        if (icol)
          for (int nn = 0; nn < nt; ++nn) a.ztfw[((long)c.m * a.kjpt + n0 + nn) * n3 + q] = T(0);
        continue;
      }
      const bool first = k == c.k0;
      const bool vface = icol && k >= 2;
      // tracer-independent coefficients of the faces of (i,j,k)
      T pah = ahu(d, a, ci, ij, k, c.m);
      const T zabe1 = pah * d.e2_e1u[ij] * d.e3u_n(ij, k, c.m);
      const T zmsku_h = rcount(wmsk<T>(cie, k) + wmsk<T>(ci, k + 1) + wmsk<T>(cie, k + 1) + wmsk<T>(ci, k));
      const T zcof1 = -pah * d.e2u[ij] * a.uslp[m3 + q] * zmsku_h;
      pah = ahv(d, a, ci, ij, k, c.m);
      const T zabe2 = pah * d.e1_e2v[ij] * d.e3v_n(ij, k, c.m);
      const T zmskv_h = rcount(wmsk<T>(cin, k) + wmsk<T>(ci, k + 1) + wmsk<T>(cin, k + 1) + wmsk<T>(ci, k));
      const T zcof2 = -pah * d.e1v[ij] * a.vslp[m3 + q] * zmskv_h;
      const T um = umsk<T>(ci, k), vm = vmsk<T>(ci, k);
      const T wk = wmsk<T>(ci, k), wk1 = wmsk<T>(ci, k + 1), wke = wmsk<T>(cie, k), wk1e = wmsk<T>(cie, k + 1);
      const T wkn = wmsk<T>(cin, k), wk1n = wmsk<T>(cin, k + 1);
      T zcoef3 = T(0), zcoef4 = T(0), zvert = T(0), ahw = T(0), akz = T(0);
      if (vface) {
        const IsoW<T> w = iso_w(d, a, ij, k, c.m, ci, ciw, cis);
        iso_coefs_at(d, a, ij, k, c.m, ci, ciw, cis, w, ahw, akz);
        if (a.kpass == 1) {
          a.ah_wslp2[m3 + q] = ahw;
          a.akz[m3 + q] = akz;
        }
        zcoef3 = -w.zahu_w * d.e2t[ij] * w.zmsku * a.wslpi[m3 + q];
        zcoef4 = -w.zahv_w * d.e1t[ij] * w.zmskv * a.wslpj[m3 + q];
        // the laplacian diagonal term of :359-366 without its tracer difference
        if (a.lap) zvert = d.e1e2t[ij] / d.e3w_n(ij, k, c.m) * wk * (ahw - akz);
      }
#pragma unroll
      for (int nn = 0; nn < NT; ++nn) {
        if (nn >= nt) break;
        const int n = n0 + nn;
        const long mo = ((long)c.m * a.kjpt + n) * n3;
        const long go = ((long)c.m * a.kjpt + n) * n2;
        const RO<T> tb = a.ptb + mo;
        // masked horizontal gradients zdit / zdjt (:218-241) at column offset o, level kk
        auto zdit = [&](const ColInfo& cc, long o, int kk, T tl, T tr) -> T {
          if (a.zps && kk == cc.mbku) return a.pgu[go + ij + o];
          return (tr - tl) * umsk<T>(cc, kk);
        };
        auto zdjt = [&](const ColInfo& cc, long o, int kk, T tl, T tr) -> T {
          if (a.zps && kk == cc.mbkv) return a.pgv[go + ij + o];
          return (tr - tl) * vmsk<T>(cc, kk);
        };
        if (first) {
          t0c[nn] = tb[q]; tec[nn] = tb[q + 1]; tnc[nn] = tb[q + jpi];
          if (k > 1) {
            const long qm = q - n2;
            const T u0 = tb[qm], ue = tb[qm + 1], un = tb[qm + jpi];
            k10[nn] = (u0 - t0c[nn]) * wk;
            k1e[nn] = (ue - tec[nn]) * wke;
            k1n[nn] = (un - tnc[nn]) * wkn;
            tup[nn] = u0;
            if (icol) {
              const T uw = tb[qm - 1], us = tb[qm - jpi];
              di0[nn] = zdit(ci, 0, k - 1, u0, ue);
              diw[nn] = zdit(ciw, -1, k - 1, uw, u0);
              dj0[nn] = zdjt(ci, 0, k - 1, u0, un);
              djs[nn] = zdjt(cis, -jpi, k - 1, us, u0);
            }
          }
        }
        const T t0 = t0c[nn], te = tec[nn], tn = tnc[nn];
        const T t1 = tb[q + n2], te1 = tb[q + 1 + n2], tn1 = tb[q + jpi + n2];
        // vertical gradients (:250-254): zdk1t(k) = (tb(k)-tb(k+1))*wmask(k+1),
        // zdkt(k) = zdk1t(k-1), zdkt(1) = zdk1t(1)
        const T dk1_0 = (t0 - t1) * wk1, dk1_e = (te - te1) * wk1e, dk1_n = (tn - tn1) * wk1n;
        const T dk0_0 = k == 1 ? dk1_0 : k10[nn];
        const T dk0_e = k == 1 ? dk1_e : k1e[nn];
        const T dk0_n = k == 1 ? dk1_n : k1n[nn];
        const T zdi = zdit(ci, 0, k, t0, te);
        const T zdj = zdjt(ci, 0, k, t0, tn);
        a.zftu[mo + q] = (zabe1 * zdi + zcof1 * (dk0_e + dk1_0 + dk1_e + dk0_0)) * um;
        a.zftv[mo + q] = (zabe2 * zdj + zcof2 * (dk0_n + dk1_0 + dk1_n + dk0_0)) * vm;
        if (icol) {
          const T tw = tb[q - 1], ts = tb[q - jpi];
          const T zdiw = zdit(ciw, -1, k, tw, t0);
          const T zdjs = zdjt(cis, -jpi, k, ts, t0);
          T z = T(0);
          if (vface) {
            const T sdi = di0[nn] + zdiw + diw[nn] + zdi;
            const T sdj = dj0[nn] + zdjs + djs[nn] + zdj;
            z = zcoef3 * sdi + zcoef4 * sdj;
            if (a.lap) {
              z = z + zvert * (tup[nn] - t0);
            } else {
              const RO<T> tbb = a.ptbb + mo;
              const T e1e2t = d.e1e2t[ij];
              const T e3w = d.e3w_n(ij, k, c.m);
              if (a.kpass == 1) z = z + ahw * e1e2t * (tup[nn] - t0) / e3w * wk;
              else z = z + e1e2t / e3w * wk * (ahw * (tup[nn] - t0) + akz * (tbb[q - n2] - tbb[q]));
            }
          }
          a.ztfw[mo + q] = z;
          di0[nn] = zdi; diw[nn] = zdiw; dj0[nn] = zdj; djs[nn] = zdjs;
        }
        k10[nn] = dk1_0; k1e[nn] = dk1_e; k1n[nn] = dk1_n;
        tup[nn] = t0;
        t0c[nn] = t1; tec[nn] = te1; tnc[nn] = tn1;
      }
    }
  }
}

// Divergence of the iso-neutral fluxes of tracer n at interior point (i,j,k), added
// to tav in the reference's order: horizontal (:278-284), then vertical (:359-366).
template <class T>
__device__ __forceinline__ T iso_div(const Dom<T>& d, const LdfArgs<T>& a, const PtIdx& c, int n, T tav) {
  const long mo = ((long)c.m * a.kjpt + n) * d.n3, q = c.q;
  const T r1 = d.r1_e1e2t[c.ij], e3tn = d.e3t_n(c.ij, c.k, c.m);
  const RO<T> fu = a.zftu + mo;
  const RO<T> fv = a.zftv + mo;
  const RO<T> fw = a.ztfw + mo;
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
// divergence of the same point from the fluxes k_iso_flux computed (the tra_ldf
// call that follows tra_adv in step.F90:248-252). k-march: the limited flux through
// the w-face between k and k+1, the coefficients of level k+1 and the iso-neutral
// vertical flux of that face are carried down.
template <class T>
__global__ void __launch_bounds__(128) k_fct_c(Dom<T> d, FctArgs<T> a) {
  const KIdx c = k_index(d);
  if (!c.valid || !c.interior) return;
  const int jpi = d.jpi, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3, ij = c.ij;
  const T r1_e1e2t = d.r1_e1e2t[ij];
  const bool w_lim = c.i - 1 >= 2;  // the face i-1 is limited only for i-1 >= 2 (then lbc: 0)
  const bool s_lim = c.j - 1 >= 2;
  const int k1 = c.k1 < jpk - 1 ? c.k1 : jpk - 1;
  constexpr int NT = 2;
  for (int n0 = 0; n0 < a.kjpt; n0 += NT) {
    const int nt = a.kjpt - n0 < NT ? a.kjpt - n0 : NT;
    // carried: limiter coefficients of the column at level k, the limited flux
    // through the top face of level k, the iso-neutral vertical flux of that face
    T bu0[NT] = {}, bd0[NT] = {}, azt[NT] = {}, fwt[NT] = {};
    for (int k = c.k0; k <= k1; ++k) {
      const bool first = k == c.k0;
      const long q = ij + (long)(k - 1) * n2, qp = q + n2;
      const T e3n = d.e3t_n(ij, k, c.m);
#pragma unroll
      for (int nn = 0; nn < NT; ++nn) {
        if (nn >= nt) break;
        const int n = n0 + nn;
        const long mo = ((long)c.m * a.kjpt + n) * n3;
        const RO<T> ax = a.ax + mo;
        const RO<T> ay = a.ay + mo;
        const RO<T> az = a.az + mo;
        const RO<T> bu = a.betup + mo;
        const RO<T> bd = a.betdo + mo;
        T* ta = a.pta + mo;
        if (first) {
          bu0[nn] = bu[q];
          bd0[nn] = bd[q];
          // pcc(k), not limited at k = 1
          azt[nn] = k >= 2 ? limit(az[q], bd0[nn], bu[q - n2], bu0[nn], bd[q - n2]) : az[q];
          if (a.with_iso) fwt[nn] = RO<T>(a.iso.ztfw + mo)[q];
        }
        const T b_u = bu0[nn], b_d = bd0[nn];
        const T bup = bu[qp], bdp = bd[qp];
        const T axl = limit(ax[q], b_d, bu[q + 1], b_u, bd[q + 1]);
        const T axlw = w_lim ? limit(ax[q - 1], bd[q - 1], b_u, bu[q - 1], b_d) : T(0);
        const T ayl = limit(ay[q], b_d, bu[q + jpi], b_u, bd[q + jpi]);
        const T ayls = s_lim ? limit(ay[q - jpi], bd[q - jpi], b_u, bu[q - jpi], b_d) : T(0);
        // pcc(k+1): the limited flux through the bottom face
        const T azl_b = limit(az[qp], bdp, b_u, bup, b_d);
        if (a.lim) {  // the multipliers of the faces this point owns
          T* L = a.lim + ((long)c.m * a.kjpt + n) * 3 * n3;
          L[q] = limit_mult(ax[q], b_d, bu[q + 1], b_u, bd[q + 1]);
          L[n3 + q] = limit_mult(ay[q], b_d, bu[q + jpi], b_u, bd[q + jpi]);
          L[2 * n3 + qp] = limit_mult(az[qp], bdp, b_u, bup, b_d);
        }
        T tav = ta[q] - (axl - axlw + ayl - ayls + azt[nn] - azl_b) * r1_e1e2t / e3n;
        if (a.with_iso) {
          // iso-neutral divergence: horizontal (traldf_iso.F90:278-284), then
          // vertical (:359-366)
          const RO<T> fu = a.iso.zftu + mo;
          const RO<T> fv = a.iso.zftv + mo;
          const RO<T> fw = a.iso.ztfw + mo;
          const T fwb = fw[qp];
          tav = tav + a.iso.zsign * (fu[q] - fu[q - 1] + fv[q] - fv[q - jpi]) * r1_e1e2t / e3n;
          tav = tav + a.iso.zsign * (fwt[nn] - fwb) * r1_e1e2t / e3n;
          fwt[nn] = fwb;
        }
        ta[q] = tav;
        bu0[nn] = bup;
        bd0[nn] = bdp;
        azt[nn] = azl_b;
      }
    }
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
// interior sweep does not write: levels 1 and jpk of interior columns, every level
// of the edge columns.
template <class T>
__global__ void k_iso_akz_copy_edges(Dom<T> d, LdfArgs<T> a) {
  ColIdx<T> c = col_index(d);
  if (!c.valid) return;
  const long base = (long)c.m * d.n3 + c.ij;
  if (c.interior) {
    const long qt = base + (long)(d.jpk - 1) * d.n2;
    a.akz[base] = a.ah_wslp2[base];
    a.akz[qt] = a.ah_wslp2[qt];
    return;
  }
  for (int k = 1; k <= d.jpk; ++k) {
    const long q = base + (long)(k - 1) * d.n2;
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
  RO<T> ptb;
  T* pta;
  int kjpt;
  RO<T> avt, avs, add;       // add: ah_wslp2 (standard iso), akz (msc) or NULL
  int ddm, is_trc, clamp_sal;
};

// Any jpk <= KMAX, the reference's recurrences with the pivots in local memory; in
// double precision the operations are those of trazdf.F90:218-264 in order, with
// every quotient correctly rounded as the reference's division gives it, but formed
// from a reciprocal (divq): one division per level (1 / zwt(k)) where the reference
// divides six times (zwi, zws, the two pivot quotients of the 1st recurrence and the
// 3rd recurrence of each of T and S); zwi(k+1) is zws(k), the same expression, formed
// once; the divisions by e3w use the rest-state reciprocal profile where e3w is it.
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
  T aux[KMAX];  // FP32: the sub-diagonal zwi, for the increment form; FP64: 1 / zwt
  for (int n = 0; n < a.kjpt; ++n) {
    const bool build = (!a.is_trc && (n == 0 || (n == 1 && a.ddm))) || (a.is_trc && n == 0);
    if (build) {
      const RO<T> coef = (!a.is_trc && n == 0) ? a.avt : a.avs;
      // zwt(k) = avt(k) (+ iso-neutral coefficient), zwt(1) = 0 (:153-176)
      auto wt = [&](int k) -> T {
        if (k == 1) return T(0);
        const long q = m3 + c.ij + (long)(k - 1) * n2;
        T v = coef[q];
        if (a.add && k <= jpk - 1) v = v + a.add[q];
        return v;
      };
      if constexpr (sizeof(T) == 8) {
        // 1st recurrence as written in the reference (trazdf.F90:218-234)
        const bool r3w = d.r1_e3w && d.e3w_n.s == 0;  // e3w is the rest-state profile
        auto over_e3w = [&](T x, int k) {
          const T e = d.e3w_n(c.ij, k, c.m);
          return r3w ? divq(x, e, d.r1_e3w[k - 1]) : x / e;
        };
        T zwi = over_e3w(-a.p2dt * wt(1), 1);
        for (int k = 1; k <= jpk - 1; ++k) {
          zws[k] = over_e3w(-a.p2dt * wt(k + 1), k + 1);
          const T zwd = d.e3t_a(c.ij, k, c.m) - zwi - zws[k];
          if (k == 1) {
            zwt[k] = zwd;
          } else {
            rat[k] = divq(zwi, zwt[k - 1], aux[k - 1]);
            zwt[k] = zwd - divq(zwi * zws[k - 1], zwt[k - 1], aux[k - 1]);
          }
          aux[k] = T(1) / zwt[k];
          zwi = zws[k];
        }
      } else {
      T wtk = wt(1);
      T g = T(0);
      for (int k = 1; k <= jpk - 1; ++k) {
        const T wtk1 = wt(k + 1);
        const T zwi = -a.p2dt * wtk / d.e3w_n(c.ij, k, c.m);
        zws[k] = -a.p2dt * wtk1 / d.e3w_n(c.ij, k + 1, c.m);
        const T e3a = d.e3t_a(c.ij, k, c.m);
        if (k >= 2) rat[k] = zwi / zwt[k - 1];
        aux[k] = zwi;
        {
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
    }
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const RO<T> tb = a.ptb + mo;
    T* ta = a.pta + mo;
    const bool clamp = a.clamp_sal && !a.is_trc && n == 1;
    if constexpr (sizeof(T) == 4) {
      // FP32: the increment form of k_zdf_imp_async (d = x - tb, one rounding of the
      // O(1) values in x = tb + d)
      const int K1 = jpk - 1;
      T prev = T(0);
      for (int k = 1; k <= K1; ++k) {
        const long q = c.ij + (long)(k - 1) * n2;
        const T tbk = tb[q];
        T r = a.p2dt * d.e3t_n(c.ij, k, c.m) * ta[q] + (d.e3t_b(c.ij, k, c.m) - d.e3t_a(c.ij, k, c.m)) * tbk;
        if (k > 1) r = r - aux[k] * (tb[q - n2] - tbk);
        if (k < K1) r = r - zws[k] * (tb[q + n2] - tbk);
        else r = r + zws[k] * tbk;
        prev = (k == 1) ? r : r - rat[k] * prev;
        ta[q] = prev;
      }
      T dnx = T(0);
      for (int k = K1; k >= 1; --k) {
        const long q = c.ij + (long)(k - 1) * n2;
        const T tbk = tb[q];
        const T dk = (k == K1 ? ta[q] : ta[q] - zws[k] * dnx) / zwt[k];
        const T x = (tbk + dk) * tmsk<T>(ci, k);
        dnx = x - tbk;
        ta[q] = (clamp && x < T(0)) ? T(0.1) : x;
      }
    } else {
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
      nxt = divq(ta[q], zwt[k], aux[k]) * tmsk<T>(ci, k);
      ta[q] = (clamp && nxt < T(0)) ? T(0.1) : nxt;
    }
    for (int k = jpk - 2; k >= 1; --k) {
      const long q = c.ij + (long)(k - 1) * n2;
      nxt = divq(ta[q] - zws[k] * nxt, zwt[k], aux[k]) * tmsk<T>(ci, k);
      ta[q] = (clamp && nxt < T(0)) ? T(0.1) : nxt;
    }
    }
  }
}

// Asynchronous 4-byte copy global -> shared (the thread waits for its own copies).
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// FP32, jpk = NK known at compile time: the elimination of k_zdf_imp with two
// arrays, zw(k) = zwi(k) (zws(k) is zwi(k+1): both are -p2dt zwt(k+1) / e3w(k+1))
// and the reciprocal pivots 1 / zwt(k), and everything per column in shared memory: each thread copies the levels of its own column
// (diffusivities, then ta and tb of each tracer) with asynchronous copies, all in
// flight together and without registers, then solves from shared memory (pivots zw
// and 1/zwt there too; the forward values overwrite ta). No block synchronisation:
// a thread reads only what it wrote or copied. Dynamic shared memory:
// 4 * NK * (threads per block) floats.
template <int NK>
__global__ void __launch_bounds__(128, 3) k_zdf_imp_async(Dom<float> d, ZdfArgs<float> a) {
  extern __shared__ float zsm[];
  const int nt = blockDim.x * blockDim.y, t = threadIdx.y * blockDim.x + threadIdx.x;
  float* sx = zsm + t;                // sx[(k-1) * nt]: ta, then the forward values
  float* sb = zsm + NK * nt + t;      // sb[(k-1) * nt]: tb (first: the added coefficient)
  float* zw = zsm + 2 * NK * nt + t;  // zw[(k-1) * nt] = zwi(k), k = 1..NK
  float* rz = zsm + 3 * NK * nt + t;  // rz[(k-1) * nt] = 1 / zwt(k), k = 1..NK-1
  ColIdx<float> c = col_index(d);
  if (!c.valid || !c.interior) return;
  constexpr int K1 = NK - 1;
  const long n2 = d.n2, n3 = d.n3;
  const ColInfo ci = d.ci[c.ij];
  const long m3 = (long)c.m * n3;
  const float p2dt = a.p2dt;
  bool built = false, built_avt = false;
  for (int n = 0; n < a.kjpt; ++n) {
    // zwt = avt (T; S without double diffusion) or avs (S with it, passive tracers)
    const bool use_avt = !a.is_trc && (n == 0 || !a.ddm);
    if (!built || use_avt != built_avt) {
      const float* coef = (use_avt ? a.avt : a.avs).p + m3 + c.ij;
      const float* add = a.add ? a.add.p + m3 + c.ij : nullptr;
      for (int k = 2; k <= NK; ++k) {
        cp_async4(sx + (k - 1) * nt, coef + (long)(k - 1) * n2);
        if (add && k <= NK - 1) cp_async4(sb + (k - 1) * nt, add + (long)(k - 1) * n2);
      }
      cp_async_wait_all();
      zw[0] = -p2dt * 0.0f / d.e3w_n(c.ij, 1, c.m);
#pragma unroll 4
      for (int k = 2; k <= NK; ++k) {
        float wt = sx[(k - 1) * nt];
        if (add && k <= NK - 1) wt = wt + sb[(k - 1) * nt];
        zw[(k - 1) * nt] = -p2dt * wt / d.e3w_n(c.ij, k, c.m);
      }
      float g = 0.0f, rprev = 0.0f;
#pragma unroll 4
      for (int k = 1; k <= K1; ++k) {
        const float e3a = d.e3t_a(c.ij, k, c.m);
        const float zk = zw[(k - 1) * nt];
        g = (k == 1) ? e3a - zk : e3a - zk * (g * rprev);
        rprev = 1.0f / (g - zw[k * nt]);
        rz[(k - 1) * nt] = rprev;
      }
      built = true;
      built_avt = use_avt;
    }
    const long mo = ((long)c.m * a.kjpt + n) * n3 + c.ij;
    const float* tb = a.ptb.p + mo;
    float* ta = a.pta + mo;
    const bool clamp = a.clamp_sal && !a.is_trc && n == 1;
    for (int k = 1; k <= K1; ++k) {
      cp_async4(sx + (k - 1) * nt, ta + (long)(k - 1) * n2);
      cp_async4(sb + (k - 1) * nt, tb + (long)(k - 1) * n2);
    }
    cp_async_wait_all();
    // Increment form: the system is solved for d = x - tb, M d = rhs - M tb, whose
    // right-hand side holds only the trend and differences of tb, so the O(1)
    // tracer values are rounded once, in x = tb + d (the reference's form rounds
    // the full values in both recurrences: ~10 ulps of salinity per step).
    float prev = 0.0f, tbm = 0.0f;
#pragma unroll 4
    for (int k = 1; k <= K1; ++k) {
      const float tbk = sb[(k - 1) * nt];
      float r = p2dt * d.e3t_n(c.ij, k, c.m) * sx[(k - 1) * nt] +
                (d.e3t_b(c.ij, k, c.m) - d.e3t_a(c.ij, k, c.m)) * tbk;
      if (k > 1) r = r - zw[(k - 1) * nt] * (tbm - tbk);    // zwi(k) (tb(k-1) - tb(k))
      if (k < K1) r = r - zw[k * nt] * (sb[k * nt] - tbk);  // zws(k) (tb(k+1) - tb(k))
      else r = r + zw[k * nt] * tbk;                        // last row: no x(k+1)
      prev = (k == 1) ? r : r - zw[(k - 1) * nt] * rz[(k - 2) * nt] * prev;
      sx[(k - 1) * nt] = prev;
      tbm = tbk;
    }
    float dnx = 0.0f;  // x(k+1) - tb(k+1) of the stored (masked) x(k+1)
#pragma unroll 4
    for (int k = K1; k >= 1; --k) {
      const float yk = sx[(k - 1) * nt], tbk = sb[(k - 1) * nt];
      const float dk = (k == K1 ? yk : yk - zw[k * nt] * dnx) * rz[(k - 1) * nt];
      const float x = (tbk + dk) * tmsk<float>(ci, k);
      dnx = x - tbk;
      ta[(long)(k - 1) * n2] = (clamp && x < 0.0f) ? 0.1f : x;
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
