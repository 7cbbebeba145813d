// k_triad.cuh -- the triad (Griffies) iso-neutral operator: ldf_slp_triad's slopes
// of the four i-k and four j-k triads of each T-point (ldfslp.F90:377-617) and
// tra_ldf_triad's fluxes (traldf_triad.F90:50-429).
//
// Every sum the reference accumulates into an array by scattering from its triads
// (wslp2, ah_wslp2, akz, the w-fluxes ztfw) is formed here in gather form: one
// thread per target point adds the contributions of the triads that touch it, in
// the order in which the reference's loop nest adds them, so the FP64 results are
// the reference's roundings and no two threads write one element. The density
// gradients of a triad are evaluated where they are used (a handful of loads from
// the tracer and expansion-ratio columns) instead of being stored.
//
// A triad array is (jpi,jpj,jpk,0:1,0:1) per member: entry (ij, k, a, b) at
// ij + (k-1) n2 + (a + 2 b) n3 of the member's 4 n3 block.
#pragma once
#include "k_tra.cuh"

namespace nemo {

template <class T>
struct TriadArgs {
  LdfArgs<T> l;                        // diffusivities, tracers, trend, ah_wslp2 / akz, flux work
  const T *tsb, *rab;                  // before tracers and their expansion ratios (jpi,jpj,jpk,2)
  const T *gdept, *gdepw;              // now depths of the T- and W-points
  const int* nmln;                     // mixed-layer level (2-D)
  T *tig, *tjg, *ti, *tj;              // the triad slopes
  T* wslp2;                            // null: not formed
  T slpmax, sw, repsln;
  int triad_iso, botmix;
};

template <class T>
__device__ __forceinline__ long tri_at(const Dom<T>& d, int m, long ij, int k, int a, int b) {
  return (long)m * 4 * d.n3 + ij + (long)(k - 1) * d.n2 + (long)(a + 2 * b) * d.n3;
}

template <class T>
__device__ __forceinline__ T sgn(T a, T b) { return b >= T(0) ? fabs(a) : -fabs(a); }
template <class T>
__device__ __forceinline__ T min3(T a, T b, T c) {
  const T m = a < b ? a : b;
  return m < c ? m : c;
}

// i-gradient of the density at T-point ij, level k, across the face ij - ip
// (ldfslp.F90:419-427): the face's T and S differences with the T-point's ratios
template <class T>
__device__ __forceinline__ T tri_dxrho(const Dom<T>& d, const TriadArgs<T>& a, int m, long ij, int k, int ip) {
  const long f = ij - ip, o = (long)m * 2 * d.n3 + (long)(k - 1) * d.n2, s = d.n3;
  const T zdit = a.tsb[o + f + 1] - a.tsb[o + f], zdis = a.tsb[o + s + f + 1] - a.tsb[o + s + f];
  const T r = (-a.rab[o + ij] * zdit + a.rab[o + s + ij] * zdis) * d.r1_e1u[f];
  return sgn(a.repsln > fabs(r) ? a.repsln : fabs(r), r);
}
// j-gradient across the face ij - jp jpi
template <class T>
__device__ __forceinline__ T tri_dyrho(const Dom<T>& d, const TriadArgs<T>& a, int m, long ij, int k, int jp) {
  const long nb = d.jpi, f = ij - jp * nb, o = (long)m * 2 * d.n3 + (long)(k - 1) * d.n2, s = d.n3;
  const T zdjt = a.tsb[o + f + nb] - a.tsb[o + f], zdjs = a.tsb[o + s + f + nb] - a.tsb[o + s + f];
  const T r = (-a.rab[o + ij] * zdjt + a.rab[o + s + ij] * zdjs) * d.r1_e2v[f];
  return sgn(a.repsln > fabs(r) ? a.repsln : fabs(r), r);
}
// vertical gradient at w-level k + kp, at least repsln (:446-463)
template <class T>
__device__ __forceinline__ T tri_dzrho(const Dom<T>& d, const TriadArgs<T>& a, int m, long ij, int k, int kp) {
  const int l = k + kp;
  const long o = (long)m * 2 * d.n3 + ij + (long)(l - 1) * d.n2, s = d.n3;
  T zdkt = T(0), zdks = T(0);
  if (l > 1) {
    zdkt = a.tsb[o - d.n2] - a.tsb[o];
    zdks = a.tsb[o + s - d.n2] - a.tsb[o + s];
  }
  const T r = (-a.rab[o] * zdkt + a.rab[o + s] * zdks) / d.e3w_n(ij, l, m);
  return -(-a.repsln < r ? -a.repsln : r);
}

// the slope of the triad (1 - ip, kp) of T-point ij just below the mixed-layer base
// (:489-506; zti_mlb)
template <class T>
__device__ T tri_mlb_i(const Dom<T>& d, const TriadArgs<T>& a, int m, long ij, int ip, int kp) {
  const int jk = a.nmln[(long)m * d.n2 + ij] + 1;
  if (jk > d.mbkt[ij] || jk - kp < 1) return T(0);  // (a mixed layer of level >= 1 never has jk - kp < 1)
  const long f = ij - ip, g3 = (long)m * d.n3 + (long)(jk - kp - 1) * d.n2;
  const T g = (tri_dxrho(d, a, m, ij, jk - kp, ip) / tri_dzrho(d, a, m, ij, jk - kp, kp) -
               (a.gdept[g3 + f + 1] - a.gdept[g3 + f]) * d.r1_e1u[f]) *
              umsk<T>(d.ci[f], jk);
  const T ze3 = d.e3w_n(ij, jk - kp, m) * d.r1_e1u[f];
  return sgn(min3(a.slpmax, T(5) * ze3, fabs(g)), g);
}
template <class T>
__device__ T tri_mlb_j(const Dom<T>& d, const TriadArgs<T>& a, int m, long ij, int jp, int kp) {
  const int jk = a.nmln[(long)m * d.n2 + ij] + 1;
  if (jk > d.mbkt[ij] || jk - kp < 1) return T(0);  // (a mixed layer of level >= 1 never has jk - kp < 1)
  const long nb = d.jpi, f = ij - jp * nb, g3 = (long)m * d.n3 + (long)(jk - kp - 1) * d.n2;
  const T g = (tri_dyrho(d, a, m, ij, jk - kp, jp) / tri_dzrho(d, a, m, ij, jk - kp, kp) -
               (a.gdept[g3 + f + nb] - a.gdept[g3 + f]) / d.e2v[f]) *
              vmsk<T>(d.ci[f], jk);
  const T ze3 = d.e3w_n(ij, jk - kp, m) / d.e2v[f];
  return sgn(min3(a.slpmax, T(5) * ze3, fabs(g)), g);
}

// ldf_slp_triad (:527-609) at one T-point: its four i-k triads (faces ij and ij - 1)
// and four j-k triads (faces ij and ij - jpi) where the face is inside the
// reference's loops; levels 1 and jpk zeroed elsewhere (:480-483).
template <class T>
__global__ void k_triad_slp(Dom<T> d, TriadArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const int jpk = d.jpk, K = c.k, m = c.m;
  const long ij = c.ij, g3 = (long)m * d.n3 + ij;
  if (K == jpk) {
    for (int s = 0; s < 2; ++s)
      for (int kp = 0; kp < 2; ++kp) {
        const long q = tri_at(d, m, ij, K, s, kp);
        a.tig[q] = T(0); a.tjg[q] = T(0); a.ti[q] = T(0); a.tj[q] = T(0);
      }
    return;
  }
  const int nml = a.nmln[(long)m * d.n2 + ij];
  int kb = (nml < (int)d.mbkt[ij] ? nml : (int)d.mbkt[ij]) + 1;
  kb = kb < 1 ? 1 : kb;  // kept in the column whatever nmln holds
  const T z1_mlbw = T(1) / a.gdepw[g3 + (long)(kb - 1) * d.n2];
  const long gk = g3 + (long)(K - 1) * d.n2;   // (ij, K)
  for (int kp = 0; kp < 2; ++kp) {
    const T znot = (K + kp == 1) ? T(0) : T(1);
    const T zf = (K + kp - 1 >= nml) ? T(1) : T(0);
    const T gw = a.gdepw[gk + (long)kp * d.n2];
    const T e3wk = d.e3w_n(ij, K + kp, m);
    for (int ip = 0; ip < 2; ++ip) {  // i-k triads: face ij - ip
      const long q = tri_at(d, m, ij, K, 1 - ip, kp);
      const int fi = c.i - ip;
      if (fi < 1 || fi > d.jpi - 1 || c.j > d.jpj - 1) {
        if (K == 1) { a.tig[q] = T(0); a.ti[q] = T(0); }
        continue;
      }
      const long f = ij - ip, gf = (long)m * d.n3 + f + (long)(K - 1) * d.n2;
      const T dxr = tri_dxrho(d, a, m, ij, K, ip);
      T raw = dxr / tri_dzrho(d, a, m, ij, K, kp);
      const T coord = znot * (a.gdept[gf + 1] - a.gdept[gf]) * d.r1_e1u[f];
      const T graw = raw - coord;
      const T ze3 = e3wk * d.r1_e1u[f];
      T glim = sgn(min3(a.slpmax, T(5) * ze3, fabs(graw)), graw);
      const T um = umsk<T>(d.ci[f], K + kp);
      glim = (zf * glim + (T(1) - zf) * tri_mlb_i(d, a, m, ij, ip, kp) * gw * z1_mlbw) * um;
      a.tig[q] = glim;
      T lim = (glim + coord) * um;
      if (a.triad_iso) {
        raw = lim * lim / raw;
        raw = sgn(fabs(lim) < fabs(raw) ? fabs(lim) : fabs(raw), raw);
        lim = zf * lim + (T(1) - zf) * raw;
      }
      const T zisw = (T(1) - a.sw) + a.sw * T(2) * fabs(T(0.5) - T(kp) - (T(0.5) - T(ip)) * sgn(T(1), dxr));
      a.ti[q] = lim * zisw;
    }
    for (int jp = 0; jp < 2; ++jp) {  // j-k triads: face ij - jp jpi
      const long q = tri_at(d, m, ij, K, 1 - jp, kp);
      const int fj = c.j - jp;
      if (fj < 1 || fj > d.jpj - 1 || c.i > d.jpi - 1) {
        if (K == 1) { a.tjg[q] = T(0); a.tj[q] = T(0); }
        continue;
      }
      const long nb = d.jpi, f = ij - jp * nb, gf = (long)m * d.n3 + f + (long)(K - 1) * d.n2;
      const T dyr = tri_dyrho(d, a, m, ij, K, jp);
      T raw = dyr / tri_dzrho(d, a, m, ij, K, kp);
      const T coord = znot * (a.gdept[gf + nb] - a.gdept[gf]) * d.r1_e2v[f];
      const T graw = raw - coord;
      const T ze3 = e3wk * d.r1_e2v[f];
      T glim = sgn(min3(a.slpmax, T(5) * ze3, fabs(graw)), graw);
      const T vm = vmsk<T>(d.ci[f], K + kp);
      glim = (zf * glim + (T(1) - zf) * tri_mlb_j(d, a, m, ij, jp, kp) * gw * z1_mlbw) * vm;
      a.tjg[q] = glim;
      T lim = (glim + coord) * vm;
      if (a.triad_iso) {
        raw = lim * lim / raw;
        raw = sgn(fabs(lim) < fabs(raw) ? fabs(lim) : fabs(raw), raw);
        lim = zf * lim + (T(1) - zf) * raw;
      }
      const T zjsw = (T(1) - a.sw) + a.sw * T(2) * fabs(T(0.5) - T(kp) - (T(0.5) - T(jp)) * sgn(T(1), dyr));
      a.tj[q] = lim * zjsw;
    }
  }
}

// wslp2 (:603-613) at one w-point from the triads of its T-point, in the reference's
// order: for kp = 0, 1 (triad level K - kp): i (face ij), j (face ij), then j (face
// ij - jpi), i (face ij - 1); the surface and the closed edges 0.
template <class T>
__global__ void k_triad_wslp2(Dom<T> d, TriadArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const int m = c.m, K = c.k;
  const long ij = c.ij;
  T s = T(0);
  if (K > 1 && c.interior) {
    const T zbt = d.e1e2t[ij] * d.e3w_n(ij, K, m);
    auto ci_ = [&](int ip, int jk, int kp) {
      const int fi = c.i - ip;
      if (fi < 1 || fi > d.jpi - 1 || c.j > d.jpj - 1) return;
      const long f = ij - ip;
      const T zbu = d.e1e2u[f] * d.e3u_n(f, jk, m);
      const T g = a.tig[tri_at(d, m, ij, jk, 1 - ip, kp)];
      s = s + T(0.25) * zbu / zbt * g * g;
    };
    auto cj_ = [&](int jp, int jk, int kp) {
      const int fj = c.j - jp;
      if (fj < 1 || fj > d.jpj - 1 || c.i > d.jpi - 1) return;
      const long f = ij - jp * (long)d.jpi;
      const T zbv = d.e1e2v[f] * d.e3v_n(f, jk, m);
      const T g = a.tjg[tri_at(d, m, ij, jk, 1 - jp, kp)];
      s = s + T(0.25) * zbv / zbt * g * g;
    };
    for (int kp = 0; kp < 2; ++kp) {
      const int jk = K - kp;
      if (jk < 1 || jk > d.jpk - 1) continue;
      ci_(0, jk, kp);
      cj_(0, jk, kp);
      cj_(1, jk, kp);
      ci_(1, jk, kp);
    }
  }
  a.wslp2[(long)m * d.n3 + c.q] = s;
}

// ---------------------------------------------------------------- tra_ldf_triad
// first pass (traldf_triad.F90:135-215): ah_wslp2 and akz at one w-point from the
// triads that touch it (i-k by ip then kp, then j-k), then the stabilising akz
// (ln_traldf_msc) or akz = ah_wslp2.
template <class T>
__global__ void k_triad_coef(Dom<T> d, TriadArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const int m = c.m, K = c.k;
  const long ij = c.ij, w = (long)m * d.n3 + c.q;
  T ah = T(0), ak = T(0);
  const T ze3wr = T(1) / d.e3w_n(ij, K, m);
  for (int ip = 0; ip < 2; ++ip)
    for (int kp = 0; kp < 2; ++kp) {
      const int jk = K - kp, fi = c.i - ip;
      if (jk < 1 || jk > d.jpk - 1 || fi < 1 || fi > d.jpi - 1 || c.j > d.jpj - 1) continue;
      const long f = ij - ip, gf = (long)m * d.n3 + f + (long)(jk - 1) * d.n2;
      const ColInfo cf = d.ci[f];
      const T zbu = d.e1e2u[f] * d.e3u_n(f, jk, m);
      const T zah = T(0.25) * ahu(d, a.l, cf, f, jk, m);
      const T um = umsk<T>(cf, K);
      T s2 = a.tig[tri_at(d, m, ij, jk, 1 - ip, kp)] + (a.gdept[gf + 1] - a.gdept[gf]) * d.r1_e1u[f] * um;
      s2 = s2 * s2;
      ah = ah + zah * zbu * ze3wr * d.r1_e1e2t[ij] * s2;
      ak = ak + zah * d.r1_e1u[f] * d.r1_e1u[f] * um;
    }
  for (int jp = 0; jp < 2; ++jp)
    for (int kp = 0; kp < 2; ++kp) {
      const int jk = K - kp, fj = c.j - jp;
      if (jk < 1 || jk > d.jpk - 1 || fj < 1 || fj > d.jpj - 1 || c.i > d.jpi - 1) continue;
      const long nb = d.jpi, f = ij - jp * nb, gf = (long)m * d.n3 + f + (long)(jk - 1) * d.n2;
      const ColInfo cf = d.ci[f];
      const T zbv = d.e1e2v[f] * d.e3v_n(f, jk, m);
      const T zah = T(0.25) * ahv(d, a.l, cf, f, jk, m);
      const T vm = vmsk<T>(cf, K);
      T s2 = a.tjg[tri_at(d, m, ij, jk, 1 - jp, kp)] + (a.gdept[gf + nb] - a.gdept[gf]) * d.r1_e2v[f] * vm;
      s2 = s2 * s2;
      ah = ah + zah * zbv * ze3wr * d.r1_e1e2t[ij] * s2;
      ak = ak + zah * d.r1_e2v[f] * d.r1_e2v[f] * vm;
    }
  if (a.l.msc) {
    if (K >= 2 && K <= d.jpk - 1 && c.i <= d.jpi - 1 && c.j <= d.jpj - 1) {
      const T e3w = d.e3w_n(ij, K, m);
      if (a.l.blp) {
        ak = T(16) * ah * (ak + ah / (e3w * e3w));
      } else {
        const T ze3w_2 = e3w * e3w;
        const T zcoef0 = a.l.z2dt * (ak + ah / ze3w_2);
        ak = (zcoef0 - T(0.5) > T(0) ? zcoef0 - T(0.5) : T(0)) * ze3w_2 * a.l.z1_2dt;
      }
    }
  } else {
    ak = ah;
  }
  a.l.ah_wslp2[w] = ah;
  a.l.akz[w] = ak;
}

// the before vertical tracer difference of a triad of T-level k (zdkt3d, :265-271)
template <class T>
__device__ __forceinline__ T tri_dk(const Dom<T>& d, const T* tb, long ij, int k, int kp) {
  const long q = ij + (long)(k - 1) * d.n2;
  const ColInfo ci = d.ci[ij];
  if (kp == 1 || k == 1) return (tb[q] - tb[q + d.n2]) * tmsk<T>(ci, k + 1);
  return (tb[q - d.n2] - tb[q]) * tmsk<T>(ci, k);
}

// the i- and j-fluxes zftu, zftv of one face at level k, over the four triads in
// the order ip (jp), kp (:285-350, without eddy-induced velocity)
template <class T>
__global__ void k_triad_flux(Dom<T> d, TriadArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid || c.k > d.jpk - 1) return;
  const int m = c.m, K = c.k;
  const long ij = c.ij, q = c.q, nb = d.jpi;
  const bool in = c.i <= d.jpi - 1 && c.j <= d.jpj - 1;
  const ColInfo ci = d.ci[ij];
  for (int n = 0; n < a.l.kjpt; ++n) {
    const long o = ((long)m * a.l.kjpt + n) * d.n3;
    const T* tb = a.l.ptb.p + o;
    T fu = T(0), fv = T(0);
    if (in) {
      const T ze1ur = d.r1_e1u[ij], ze2vr = d.r1_e2v[ij];
      const T zdxt = (tb[q + 1] - tb[q]) * umsk<T>(ci, K) * ze1ur;
      const T zdyt = (tb[q + nb] - tb[q]) * vmsk<T>(ci, K) * ze2vr;
      const T zbu = T(0.25) * d.e1e2u[ij] * d.e3u_n(ij, K, m);
      const T zbv = T(0.25) * d.e1e2v[ij] * d.e3v_n(ij, K, m);
      const T ahu0 = ahu(d, a.l, ci, ij, K, m), ahv0 = ahv(d, a.l, ci, ij, K, m);
      for (int ip = 0; ip < 2; ++ip)
        for (int kp = 0; kp < 2; ++kp) {
          const long t = ij + ip;
          const T ze3wr = T(1) / d.e3w_n(t, K + kp, m);
          const T zdzt = tri_dk(d, tb, t, K, kp) * ze3wr;
          const T zah = a.botmix ? ahu0 : ahu0 * umsk<T>(ci, K + kp);
          const T zah_slp = zah * a.ti[tri_at(d, m, t, K, 1 - ip, kp)];
          fu = fu - (zah * zdxt + zah_slp * zdzt) * zbu * ze1ur;
        }
      for (int jp = 0; jp < 2; ++jp)
        for (int kp = 0; kp < 2; ++kp) {
          const long t = ij + jp * nb;
          const T ze3wr = T(1) / d.e3w_n(t, K + kp, m);
          const T zdzt = tri_dk(d, tb, t, K, kp) * ze3wr;
          const T zah = a.botmix ? ahv0 : ahv0 * vmsk<T>(ci, K + kp);
          const T zah_slp = zah * a.tj[tri_at(d, m, t, K, 1 - jp, kp)];
          fv = fv - (zah * zdyt + zah_slp * zdzt) * zbv * ze2vr;
        }
    }
    a.l.zftu[o + q] = fu;
    a.l.zftv[o + q] = fv;
  }
}

// ztfw at one w-point: the triad contributions of the levels K - 1 (kp = 1) and K
// (kp = 0), each i-k (ip = 0, 1) then j-k (jp = 0, 1), then the 33 flux (:366-402)
template <class T>
__global__ void k_triad_tfw(Dom<T> d, TriadArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const int m = c.m, K = c.k;
  const long ij = c.ij, q = c.q, nb = d.jpi;
  const T ze3wr = T(1) / d.e3w_n(ij, K, m);
  for (int n = 0; n < a.l.kjpt; ++n) {
    const long o = ((long)m * a.l.kjpt + n) * d.n3;
    const T* tb = a.l.ptb.p + o;
    T t = T(0);
    for (int kp = 1; kp >= 0; --kp) {
      const int jk = K - kp;
      if (jk < 1 || jk > d.jpk - 1) continue;
      for (int ip = 0; ip < 2; ++ip) {
        const int fi = c.i - ip;
        if (fi < 1 || fi > d.jpi - 1 || c.j > d.jpj - 1) continue;
        const long f = ij - ip, qf = f + (long)(jk - 1) * d.n2;
        const ColInfo cf = d.ci[f];
        const T ze1ur = d.r1_e1u[f];
        const T zdxt = (tb[qf + 1] - tb[qf]) * umsk<T>(cf, jk) * ze1ur;
        const T zbu = T(0.25) * d.e1e2u[f] * d.e3u_n(f, jk, m);
        const T a0 = ahu(d, a.l, cf, f, jk, m);
        const T zah = a.botmix ? a0 : a0 * umsk<T>(cf, K);
        const T zah_slp = zah * a.ti[tri_at(d, m, ij, jk, 1 - ip, kp)];
        t = t - (zah_slp + T(0)) * zdxt * zbu * ze3wr;  // + the eddy-induced part (0)
      }
      for (int jp = 0; jp < 2; ++jp) {
        const int fj = c.j - jp;
        if (fj < 1 || fj > d.jpj - 1 || c.i > d.jpi - 1) continue;
        const long f = ij - jp * nb, qf = f + (long)(jk - 1) * d.n2;
        const ColInfo cf = d.ci[f];
        const T ze2vr = d.r1_e2v[f];
        const T zdyt = (tb[qf + nb] - tb[qf]) * vmsk<T>(cf, jk) * ze2vr;
        const T zbv = T(0.25) * d.e1e2v[f] * d.e3v_n(f, jk, m);
        const T a0 = ahv(d, a.l, cf, f, jk, m);
        const T zah = a.botmix ? a0 : a0 * vmsk<T>(cf, K);
        const T zah_slp = zah * a.tj[tri_at(d, m, ij, jk, 1 - jp, kp)];
        t = t - (zah_slp + T(0)) * zdyt * zbv * ze3wr;
      }
    }
    if (K >= 2 && K <= d.jpk - 1 && c.i >= 2 && c.i <= d.jpi - 1 && c.j <= d.jpj - 1) {
      const long w = (long)m * d.n3 + q;
      const T tm = tmsk<T>(d.ci[ij], K);
      const T e3w = d.e3w_n(ij, K, m);
      if (a.l.lap) {
        t = t - d.e1e2t[ij] / e3w * tm * (a.l.ah_wslp2[w] - a.l.akz[w]) * (tb[q - d.n2] - tb[q]);
      } else if (a.l.kpass == 1) {
        t = t - d.e1e2t[ij] / e3w * tm * a.l.ah_wslp2[w] * (tb[q - d.n2] - tb[q]);
      } else {
        const T* tbb = a.l.ptbb.p + o;
        t = t - d.e1e2t[ij] / e3w * tm *
                    (a.l.ah_wslp2[w] * (tb[q - d.n2] - tb[q]) + a.l.akz[w] * (tbb[q - d.n2] - tbb[q]));
      }
    }
    a.l.ztfw[o + q] = t;
  }
}

// the divergence of the fluxes added to pta at one interior point: the horizontal
// part (:354-361), then the vertical part (:404-410)
template <class T>
__global__ void k_triad_div(Dom<T> d, TriadArgs<T> a) {
  const PtIdx c = pt_index(d);
  if (!c.valid || !c.interior || c.k > d.jpk - 1) return;
  const int m = c.m;
  const long q = c.q, nb = d.jpi;
  const T vol = d.e1e2t[c.ij] * d.e3t_n(c.ij, c.k, m);
  for (int n = 0; n < a.l.kjpt; ++n) {
    const long o = ((long)m * a.l.kjpt + n) * d.n3;
    const T* fu = a.l.zftu + o;
    const T* fv = a.l.zftv + o;
    const T* fw = a.l.ztfw + o;
    T x = a.l.pta[o + q];
    x = x + a.l.zsign * (fu[q - 1] - fu[q] + fv[q - nb] - fv[q]) / vol;
    x = x + a.l.zsign * (fw[q + d.n2] - fw[q]) / vol;
    a.l.pta[o + q] = x;
  }
}

}  // namespace nemo
