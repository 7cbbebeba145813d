// k_adj.cuh -- adjoint kernels of the tracer routines (FP64), and tra_nxt.
//
// NEMO has no adjoint of these routines in its tree (its tangent-linear/adjoint,
// NEMOTAM, is a separate project); each kernel here is the transpose of the
// tangent-linear of the forward kernel with respect to the tracer arguments, with
// the coefficients (transports, diffusivities, slopes, scale factors, avt) held
// fixed and, for FCT, the limiter multipliers that the forward recorded.
//
// Gather form: one thread per (i,j,k) point computes the adjoint of the tracer at
// its own point by collecting the terms of every face flux that read it, so no two
// threads write one element and the result does not depend on scheduling. The
// face adjoints that several points share are recomputed by each of them.
// Conventions (those of the host mirror): an adjoint accumulates into the adjoints
// of the inputs (tb_ad += ...); a trend array that the forward only adds to keeps
// its adjoint unchanged.
#pragma once
#include "adj.h"

namespace nemo {

// 1-based point helpers of the gather kernels
struct Pt3 {
  int jpi, jpj, jpk;
  long n2;
  __device__ __forceinline__ long ij(int i, int j) const { return (long)(i - 1) + (long)(j - 1) * jpi; }
  __device__ __forceinline__ long q(int i, int j, int k) const { return ij(i, j) + (long)(k - 1) * n2; }
  // interior cell of a trend loop: 2..jpim1, 2..jpjm1, 1..jpkm1
  __device__ __forceinline__ bool cell(int i, int j, int k) const {
    return i >= 2 && i <= jpi - 1 && j >= 2 && j <= jpj - 1 && k >= 1 && k <= jpk - 1;
  }
  // an east (u) face of a flux loop: 1..jpim1, 1..jpjm1, 1..jpkm1
  __device__ __forceinline__ bool uface(int i, int j, int k) const {
    return i >= 1 && i <= jpi - 1 && j >= 1 && j <= jpj - 1 && k >= 1 && k <= jpk - 1;
  }
  __device__ __forceinline__ bool icol(int i, int j) const { return i >= 2 && i <= jpi - 1 && j >= 2 && j <= jpj - 1; }
};
template <class T>
__device__ __forceinline__ Pt3 pt3(const Dom<T>& d) { return Pt3{d.jpi, d.jpj, d.jpk, d.n2}; }

// ------------------------------------------------------------------ tra_adv_fct
// Adjoint of tra_adv_fct (traadv_fct.F90:54-327) at one point; with kn_fct_h = 4 the
// 4th-order centred horizontal fluxes (:191-227), with kn_fct_v = 4 the compact
// vertical interpolation's part is k_fct_adj_v4's (below). With g = lam r1_e1e2t / e3t_n and h = g tmask on the interior cells (0
// elsewhere), the limited antidiffusive flux of face f has the adjoint
// -(g(f) - g(f+1)); times the recorded multiplier (0 where the forward zeroed the
// flux) it is the adjoint of the flux before limiting, the centred flux of tn minus
// the upstream flux of tb (:182-190, :255-263). The upstream flux gets minus that,
// plus -(h(f) - h(f+1)) from its own trend (:158-170), and passes it to tb
// (:123-156).
__global__ void __launch_bounds__(128) k_fct_adj(Dom<double> d, FctAdj a) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const Pt3 P = pt3(d);
  const int i = c.i, j = c.j, k = c.k, jpi = d.jpi, jpk = d.jpk;
  const long q = c.q, n2 = d.n2, n3 = d.n3, mv = (long)c.m * n3;
  const RO<double> un = a.pun + mv;
  const RO<double> vn = a.pvn + mv;
  const RO<double> wn = a.pwn + mv;
  const bool ic = P.icol(i, j);
  const bool fe = P.uface(i, j, k), fw = P.uface(i - 1, j, k);
  const bool fn = P.uface(i, j, k), fs = P.uface(i, j - 1, k);  // v faces share the u ranges
  // vertical faces of the column: top (level k) and bottom (level k+1), antidiffusive
  // part on interior columns for levels 2..jpkm1, upstream part on every column
  const bool zt = ic && k >= 2 && k <= jpk - 1, zb = ic && k + 1 >= 2 && k + 1 <= jpk - 1;
  const bool ut = k >= 2 && k <= jpk - 1, ub = k + 1 <= jpk - 1;
  const ColInfo ci = d.ci[c.ij];
  const double wmt = wmsk<double>(ci, k), wmb = wmsk<double>(ci, k + 1);
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const RO<double> lam = a.lam + mo;
    const RO<double> tx = a.tape + ((long)c.m * a.kjpt + n) * 3 * n3;
    const RO<double> ty = tx + n3;
    const RO<double> tz = tx + 2 * n3;
    auto g = [&](int ii, int jj, int kk) -> double {
      if (!P.cell(ii, jj, kk)) return 0.0;
      const long o = P.ij(ii, jj);
      return lam[P.q(ii, jj, kk)] * d.r1_e1e2t[o] / d.e3t_n(o, kk, c.m);
    };
    const double gc = g(i, j, k), ge = g(i + 1, j, k), gw = g(i - 1, j, k), gn = g(i, j + 1, k),
                 gs = g(i, j - 1, k), gu = g(i, j, k - 1), gd = g(i, j, k + 1);
    const double tmc = tmsk<double>(ci, k);
    const double hc = gc * tmc;
    const double he = fe ? ge * tmsk<double>(d.ci[c.ij + 1], k) : 0.0;
    const double hw = fw ? gw * tmsk<double>(d.ci[c.ij - 1], k) : 0.0;
    const double hn = fn ? gn * tmsk<double>(d.ci[c.ij + jpi], k) : 0.0;
    const double hs = fs ? gs * tmsk<double>(d.ci[c.ij - jpi], k) : 0.0;
    const double hu = k >= 2 ? gu * tmsk<double>(ci, k - 1) : 0.0;
    const double hd = k + 1 <= jpk ? gd * tmsk<double>(ci, k + 1) : 0.0;
    // limited antidiffusive fluxes -> their adjoints before limiting
    const double axe = fe ? tx[q] * (ge - gc) : 0.0;
    const double axw = fw ? tx[q - 1] * (gc - gw) : 0.0;
    const double ayn = fn ? ty[q] * (gn - gc) : 0.0;
    const double ays = fs ? ty[q - jpi] * (gc - gs) : 0.0;
    const double azt = zt ? tz[q] * (gu - gc) * wmt : 0.0;
    const double azb = zb ? tz[q + n2] * (gc - gd) * wmb : 0.0;
    double tnv = 0.0;
    if (fe) tnv += 0.5 * un[q] * axe;
    if (fw) tnv += 0.5 * un[q - 1] * axw;
    if (fn) tnv += 0.5 * vn[q] * ayn;
    if (fs) tnv += 0.5 * vn[q - jpi] * ays;
    if (a.kv == 2) {
      if (zt) tnv += wn[q] * 0.5 * azt;
      if (zb) tnv += wn[q + n2] * 0.5 * azb;
    }
    if (a.kh == 4) {
      // zltu(m) = (ztu(m) + ztu(m-1)) / 6 enters the flux of u-face m with + and that
      // of face m-1 with -; ztu(m) = (tn(m+1) - tn(m)) umask(m). S: the adjoint of a
      // face's centred bracket; Z: of zltu (interior points only, lbc_lnk zeroes the
      // edges). Likewise in j.
      auto Su = [&](int fi) -> double {
        if (!P.uface(fi, j, k)) return 0.0;
        const long qf = P.q(fi, j, k);
        return 0.5 * un[qf] * (tx[qf] * (g(fi + 1, j, k) - g(fi, j, k)));
      };
      auto Sv = [&](int fj) -> double {
        if (!P.uface(i, fj, k)) return 0.0;
        const long qf = P.q(i, fj, k);
        return 0.5 * vn[qf] * (ty[qf] * (g(i, fj + 1, k) - g(i, fj, k)));
      };
      auto Zu = [&](int mi) -> double { return P.cell(mi, j, k) ? Su(mi) - Su(mi - 1) : 0.0; };
      auto Zv = [&](int mj) -> double { return P.cell(i, mj, k) ? Sv(mj) - Sv(mj - 1) : 0.0; };
      const double zu0 = Zu(i - 1), zu1 = Zu(i), zu2 = Zu(i + 1);
      const double zv0 = Zv(j - 1), zv1 = Zv(j), zv2 = Zv(j + 1);
      const double r1_6 = 1. / 6.;
      if (i >= 2) tnv += r1_6 * (zu0 + zu1) * umsk<double>(d.ci[c.ij - 1], k);
      tnv -= r1_6 * (zu1 + zu2) * umsk<double>(ci, k);
      if (j >= 2) tnv += r1_6 * (zv0 + zv1) * vmsk<double>(d.ci[c.ij - jpi], k);
      tnv -= r1_6 * (zv1 + zv2) * vmsk<double>(ci, k);
    }
    // upstream fluxes: minus the antidiffusive adjoint plus their own trend's
    const double fxe = -axe + (he - hc), fxw = -axw + (hc - hw);
    const double fyn = -ayn + (hn - hc), fys = -ays + (hc - hs);
    const double fzt = -azt + (hu - hc), fzb = -azb + (hc - hd);
    double tbv = 0.0;
    if (fe) { const double u = un[q]; tbv += 0.5 * (u + fabs(u)) * fxe; }
    if (fw) { const double u = un[q - 1]; tbv += 0.5 * (u - fabs(u)) * fxw; }
    if (fn) { const double v = vn[q]; tbv += 0.5 * (v + fabs(v)) * fyn; }
    if (fs) { const double v = vn[q - jpi]; tbv += 0.5 * (v - fabs(v)) * fys; }
    if (ut) { const double w = wn[q]; tbv += (w + fabs(w)) * (0.5 * fzt * wmt); }
    if (ub) { const double w = wn[q + n2]; tbv += (w - fabs(w)) * (0.5 * fzb * wmb); }
    if (k == 1 && a.linssh) tbv += wn[q] * fzt;  // surface flux w tb (:146-156)
    a.tb_ad[mo + q] += tbv;
    a.tn_ad[mo + q] += tnv;
  }
}

// With kn_fct_v = 4 (traadv_fct.F90:253-275): the vertical antidiffusive flux reads
// ztw = M^-1 R tn of interp_4th_cpt (:517-616). One interior column a thread: the
// adjoint V(k) = wn(k) az(k) of ztw(k), k = 2..jpk-1, then tn_ad += R^T M^-T V with
// the forward's rows (special top and bottom rows), pivots zwt, the back
// substitution undone forwards and the elimination backwards (as the oracle's
// ora_interp_4th_cpt_adj). Runs after k_fct_adj, which leaves this part out.
__global__ void k_fct_adj_v4(Dom<double> d, FctAdj a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i < 2 || i > d.jpi - 1 || j < 2 || j > d.jpj - 1) return;
  const int m = blockIdx.z, jpk = d.jpk;
  const Pt3 P = pt3(d);
  const long ij = P.ij(i, j), n2 = d.n2, n3 = d.n3, c3 = (long)m * n3 + ij;
  const ColInfo ci = d.ci[ij];
  const int ikt = 2, ikb = d.mbkt[ij];
  const RO<double> wn = a.pwn + (long)m * n3;
  const double r1 = d.r1_e1e2t[ij];
  auto row = [&](int k, double& dd, double& wi, double& ws, double& w) {
    const double wm = wmsk<double>(ci, k);
    if (k == ikt || k == ikb) { dd = 1.0; wi = 0.0; ws = 0.0; w = 0.5; }
    else { dd = 3.0 * wm + 1.0; wi = wm; ws = wm; w = 3.0 * wm; }
  };
  // the pivots (the same for every tracer)
  {
    double dd, wi, ws, w, wsp;
    row(2, dd, wi, wsp, w);
    a.zwt[c3 + n2] = dd;
    double tp = dd;
    for (int k = 3; k <= jpk - 1; ++k) {
      row(k, dd, wi, ws, w);
      tp = dd - wi * wsp / tp;
      a.zwt[c3 + (long)(k - 1) * n2] = tp;
      wsp = ws;
    }
  }
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)m * a.kjpt + n) * n3;
    const RO<double> lam = a.lam + mo;
    const RO<double> tz = a.tape + ((long)m * a.kjpt + n) * 3 * n3 + 2 * n3;
    auto g = [&](int k) -> double {
      return (k >= 1 && k <= jpk - 1) ? lam[ij + (long)(k - 1) * n2] * r1 / d.e3t_n(ij, k, m) : 0.0;
    };
    // V into za, then the back substitution undone (za: the adjoint of z)
    for (int k = 2; k <= jpk - 1; ++k) {
      const long q = ij + (long)(k - 1) * n2;
      const double az = tz[q] * (g(k - 1) - g(k)) * wmsk<double>(ci, k);
      a.za[c3 + (long)(k - 1) * n2] = wn[q] * az;
    }
    double carry = 0.0;
    for (int k = 2; k <= jpk - 2; ++k) {
      const long o = c3 + (long)(k - 1) * n2;
      double dd, wi, ws, w;
      row(k, dd, wi, ws, w);
      const double x = a.za[o] + carry;
      const double z = x / a.zwt[o];
      a.za[o] = z;
      carry = -ws * z;
    }
    {
      const long o = c3 + (long)(jpk - 2) * n2;
      a.za[o] = (a.za[o] + carry) / a.zwt[o];
    }
    // the elimination undone, then the right-hand side transposed
    double zk = a.za[c3 + (long)(jpk - 2) * n2];
    for (int k = jpk - 1; k >= 2; --k) {
      double dd, wi, ws, w;
      row(k, dd, wi, ws, w);
      const long o = c3 + (long)(k - 1) * n2;
      if (k >= 3) {
        const long om = o - n2;
        const double zm = a.za[om] - wi / a.zwt[om] * zk;
        a.za[om] = zm;
      }
      a.tn_ad[mo + ij + (long)(k - 1) * n2] += w * zk;
      a.tn_ad[mo + ij + (long)(k - 2) * n2] += w * zk;
      if (k >= 3) zk = a.za[o - n2];
    }
  }
}

// ------------------------------------------------------------------ tra_ldf_lap
// Adjoint of tra_ldf_lap (traldf_lap_blp.F90:95-145) at one point: the fluxes of
// the east and north faces of (i-1,j), (i,j), (i,j-1). A partial-step bottom face
// (k = mbku) takes the fixed pgu and passes nothing to tb.
__global__ void __launch_bounds__(128) k_lap_adj(Dom<double> d, LdfArgs<double> a, LdfAdj b) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const Pt3 P = pt3(d);
  const int i = c.i, j = c.j, k = c.k, jpi = d.jpi;
  const long q = c.q, n3 = d.n3;
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const RO<double> lam = b.lam + mo;
    auto g = [&](int ii, int jj) -> double {
      if (!P.cell(ii, jj, k)) return 0.0;
      const long o = P.ij(ii, jj);
      return lam[P.q(ii, jj, k)] / (d.e1e2t[o] * d.e3t_n(o, k, c.m));
    };
    // u face of column (ii,jj): zaheeu * (g(ii,jj) - g(ii+1,jj))
    auto fu = [&](int ii, int jj) -> double {
      if (!P.uface(ii, jj, k)) return 0.0;
      const long o = P.ij(ii, jj);
      const ColInfo cc = d.ci[o];
      if (a.zps && k == cc.mbku) return 0.0;
      const double z = a.zsign * ahu(d, a, cc, o, k, c.m) * d.e2_e1u[o] * d.e3u_n(o, k, c.m);
      return z * (g(ii, jj) - g(ii + 1, jj));
    };
    auto fv = [&](int ii, int jj) -> double {
      if (!P.uface(ii, jj, k)) return 0.0;
      const long o = P.ij(ii, jj);
      const ColInfo cc = d.ci[o];
      if (a.zps && k == cc.mbkv) return 0.0;
      const double z = a.zsign * ahv(d, a, cc, o, k, c.m) * d.e1_e2v[o] * d.e3v_n(o, k, c.m);
      return z * (g(ii, jj) - g(ii, jj + 1));
    };
    (void)jpi;
    b.tb_ad[mo + q] += fu(i - 1, j) - fu(i, j) + fv(i, j - 1) - fv(i, j);
  }
}

// ------------------------------------------------------------------ tra_ldf_iso
// Stage 0: G = zsign lam r1_e1e2t / e3t_n on the interior cells, 0 elsewhere (the
// adjoint weight of a divergence, :278-284 and :359-366).
__global__ void __launch_bounds__(128) k_iso_adj_g(Dom<double> d, LdfArgs<double> a, LdfAdj b) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const Pt3 P = pt3(d);
  for (int n = 0; n < a.kjpt; ++n) {
    const long o = ((long)c.m * a.kjpt + n) * d.n3 + c.q;
    b.G[o] = P.cell(c.i, c.j, c.k) ? a.zsign * b.lam[o] * d.r1_e1e2t[c.ij] / d.e3t_n(c.ij, c.k, c.m) : 0.0;
  }
}

// Coefficients of the iso-neutral fluxes at one face or w-point, as the forward
// kernel forms them (traldf_iso.F90:255-276 horizontal, :297-357 vertical).
struct IsoAdjCoef {
  const Dom<double>& d;
  const LdfArgs<double>& a;
  Pt3 P;
  int m;
  long m3;
  // zcof1 * umask of the u face (ii,jj,kk); zabe1 * umask
  __device__ __forceinline__ double cof1(int ii, int jj, int kk) const {
    const long o = P.ij(ii, jj);
    const ColInfo cc = d.ci[o], ce = d.ci[o + 1];
    const double pah = ahu(d, a, cc, o, kk, m);
    const double zm = rcount(wmsk<double>(ce, kk) + wmsk<double>(cc, kk + 1) + wmsk<double>(ce, kk + 1) +
                             wmsk<double>(cc, kk));
    return -pah * d.e2u[o] * a.uslp[m3 + o + (long)(kk - 1) * P.n2] * zm * umsk<double>(cc, kk);
  }
  __device__ __forceinline__ double cof2(int ii, int jj, int kk) const {
    const long o = P.ij(ii, jj);
    const ColInfo cc = d.ci[o], cn = d.ci[o + P.jpi];
    const double pah = ahv(d, a, cc, o, kk, m);
    const double zm = rcount(wmsk<double>(cn, kk) + wmsk<double>(cc, kk + 1) + wmsk<double>(cn, kk + 1) +
                             wmsk<double>(cc, kk));
    return -pah * d.e1v[o] * a.vslp[m3 + o + (long)(kk - 1) * P.n2] * zm * vmsk<double>(cc, kk);
  }
  __device__ __forceinline__ double abe1(int ii, int jj, int kk) const {
    const long o = P.ij(ii, jj);
    const ColInfo cc = d.ci[o];
    return ahu(d, a, cc, o, kk, m) * d.e2_e1u[o] * d.e3u_n(o, kk, m) * umsk<double>(cc, kk);
  }
  __device__ __forceinline__ double abe2(int ii, int jj, int kk) const {
    const long o = P.ij(ii, jj);
    const ColInfo cc = d.ci[o];
    return ahv(d, a, cc, o, kk, m) * d.e1_e2v[o] * d.e3v_n(o, kk, m) * vmsk<double>(cc, kk);
  }
  // zcoef3 / zcoef4 of the w-point (ii,jj,kk): interior column, 2 <= kk <= jpkm1
  __device__ __forceinline__ void coef34(int ii, int jj, int kk, double& c3, double& c4) const {
    const long o = P.ij(ii, jj);
    const ColInfo cc = d.ci[o], cw = d.ci[o - 1], cs = d.ci[o - P.jpi];
    const IsoW<double> w = iso_w(d, a, o, kk, m, cc, cw, cs);
    const long qq = m3 + o + (long)(kk - 1) * P.n2;
    c3 = -w.zahu_w * d.e2t[o] * w.zmsku * a.wslpi[qq];
    c4 = -w.zahv_w * d.e1t[o] * w.zmskv * a.wslpj[qq];
  }
  // the vertical laplacian coefficients of the w-point on tb and on tbb
  __device__ __forceinline__ void vlap(int ii, int jj, int kk, double& ctb, double& ctbb) const {
    const long o = P.ij(ii, jj);
    const long qq = m3 + o + (long)(kk - 1) * P.n2;
    const double f = d.e1e2t[o] / d.e3w_n(o, kk, m) * wmsk<double>(d.ci[o], kk);
    const double ahw = a.ah_wslp2[qq], akz = a.akz[qq];
    ctbb = 0.0;
    if (a.lap) ctb = f * (ahw - akz);
    else if (a.kpass == 1) ctb = ahw * f;
    else { ctb = ahw * f; ctbb = akz * f; }
  }
};

// Stage 1: adjoints of the masked gradients zdit(i,j,k), zdjt(i,j,k) (u and v faces)
// and of the vertical difference D(k) = (tb(k-1) - tb(k)) wmask(k) of column (i,j),
// k = 2..jpk (zdkt(k) = D(k), zdk1t(k) = D(k+1), zdkt(1) = D(2); :246-254).
__global__ void __launch_bounds__(128) k_iso_adj_grad(Dom<double> d, LdfArgs<double> a, LdfAdj b) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const Pt3 P = pt3(d);
  const int i = c.i, j = c.j, k = c.k, jpk = d.jpk;
  const long n3 = d.n3;
  const IsoAdjCoef C{d, a, P, c.m, (long)c.m * n3};
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const RO<double> G = b.G + mo;
    auto gg = [&](int ii, int jj, int kk) -> double {
      return (ii >= 1 && ii <= P.jpi && jj >= 1 && jj <= P.jpj && kk >= 1 && kk <= jpk) ? G[P.q(ii, jj, kk)] : 0.0;
    };
    // adjoint of the vertical flux ztfw at w-point (ii,jj,kk): G(kk) - G(kk-1)
    auto tfw = [&](int ii, int jj, int kk) -> double {
      if (!P.icol(ii, jj) || kk < 2 || kk > jpk - 1) return 0.0;
      return gg(ii, jj, kk) - gg(ii, jj, kk - 1);
    };
    auto w34 = [&](int ii, int jj, int kk, double& s3, double& s4) {
      const double t = tfw(ii, jj, kk);
      if (t == 0.0) return;
      double c3, c4;
      C.coef34(ii, jj, kk, c3, c4);
      s3 += c3 * t;
      s4 += c4 * t;
    };
    double di = 0.0, dj = 0.0, dk = 0.0;
    if (P.uface(i, j, k)) {
      double s3 = 0.0, s4 = 0.0, t3 = 0.0, t4 = 0.0;
      // zdit(i,j,k) enters ztfw at (i,j,k+1), (i+1,j,k), (i+1,j,k+1), (i,j,k);
      // zdjt(i,j,k) at (i,j,k+1), (i,j+1,k), (i,j+1,k+1), (i,j,k)
      w34(i, j, k + 1, s3, s4);
      w34(i, j, k, s3, s4);
      double x;
      w34(i + 1, j, k, t3, x);
      w34(i + 1, j, k + 1, t3, x);
      w34(i, j + 1, k, x, t4);
      w34(i, j + 1, k + 1, x, t4);
      const ColInfo cc = d.ci[P.ij(i, j)];
      di = C.abe1(i, j, k) * (gg(i, j, k) - gg(i + 1, j, k)) + s3 + t3;
      dj = C.abe2(i, j, k) * (gg(i, j, k) - gg(i, j + 1, k)) + s4 + t4;
      if (a.zps && k == cc.mbku) di = 0.0;
      if (a.zps && k == cc.mbkv) dj = 0.0;
    }
    if (k >= 2) {
      // D(k) is zdkt of level k and zdk1t of level k-1 for the u faces of columns
      // i-1 and i (and the v faces of j-1 and j); at k = 2 also zdkt of level 1
      auto su = [&](int ii, int jj, int kk) -> double {
        return P.uface(ii, jj, kk) ? C.cof1(ii, jj, kk) * (gg(ii, jj, kk) - gg(ii + 1, jj, kk)) : 0.0;
      };
      auto sv = [&](int ii, int jj, int kk) -> double {
        return P.uface(ii, jj, kk) ? C.cof2(ii, jj, kk) * (gg(ii, jj, kk) - gg(ii, jj + 1, kk)) : 0.0;
      };
      double s = su(i, j, k) + su(i - 1, j, k) + su(i, j, k - 1) + su(i - 1, j, k - 1);
      s += sv(i, j, k) + sv(i, j - 1, k) + sv(i, j, k - 1) + sv(i, j - 1, k - 1);
      if (k == 2) s += su(i, j, 1) + su(i - 1, j, 1) + sv(i, j, 1) + sv(i, j - 1, 1);
      const double t = tfw(i, j, k);
      if (t != 0.0) {
        double ctb, ctbb;
        C.vlap(i, j, k, ctb, ctbb);
        s += ctb * t;
      }
      dk = s;
    }
    b.dit[mo + c.q] = di;
    b.djt[mo + c.q] = dj;
    b.dk[mo + c.q] = dk;
  }
}

// Stage 2: tb_ad from the gradient adjoints (zdit = (tb(i+1)-tb(i)) umask, :218-227;
// D(k)), and tbb_ad from the second-pass vertical term (:343-356).
__global__ void __launch_bounds__(128) k_iso_adj_tb(Dom<double> d, LdfArgs<double> a, LdfAdj b) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const Pt3 P = pt3(d);
  const int i = c.i, j = c.j, k = c.k, jpi = d.jpi, jpk = d.jpk;
  const long q = c.q, n2 = d.n2, n3 = d.n3;
  const ColInfo ci = d.ci[c.ij];
  const bool tbb = !a.lap && a.kpass != 1;
  const IsoAdjCoef C{d, a, P, c.m, (long)c.m * n3};
  for (int n = 0; n < a.kjpt; ++n) {
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    const RO<double> di = b.dit + mo;
    const RO<double> dj = b.djt + mo;
    const RO<double> dk = b.dk + mo;
    double v = 0.0;
    if (P.uface(i - 1, j, k)) v += umsk<double>(d.ci[c.ij - 1], k) * di[q - 1];
    if (P.uface(i, j, k)) v -= umsk<double>(ci, k) * di[q];
    if (P.uface(i, j - 1, k)) v += vmsk<double>(d.ci[c.ij - jpi], k) * dj[q - jpi];
    if (P.uface(i, j, k)) v -= vmsk<double>(ci, k) * dj[q];
    if (k + 1 <= jpk) v += wmsk<double>(ci, k + 1) * dk[q + n2];
    if (k >= 2) v -= wmsk<double>(ci, k) * dk[q];
    b.tb_ad[mo + q] += v;
    if (tbb && P.icol(i, j)) {
      const RO<double> G = b.G + mo;
      double u = 0.0, ctb, ctbb;
      if (k + 1 >= 2 && k + 1 <= jpk - 1) {
        C.vlap(i, j, k + 1, ctb, ctbb);
        u += ctbb * (G[q + n2] - G[q]);
      }
      if (k >= 2 && k <= jpk - 1) {
        C.vlap(i, j, k, ctb, ctbb);
        u -= ctbb * (G[q] - G[q - n2]);
      }
      b.tbb_ad[mo + q] += u;
    }
  }
}

// ------------------------------------------------------------------ tra_zdf_imp
// Adjoint of tra_zdf_imp (trazdf.F90:143-264) on one interior column: the
// back-substitution run forwards, then the elimination with its right-hand side
// e3t_b tb + p2dt e3t_n ta run backwards. The matrix is built as k_zdf_imp builds
// it in double precision.
__global__ void k_zdf_adj(Dom<double> d, ZdfArgs<double> a, ZdfAdj b) {
  ColIdx<double> c = col_index(d);
  if (!c.valid || !c.interior) return;
  const int jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const ColInfo ci = d.ci[c.ij];
  const long m3 = (long)c.m * n3;
  double rat[KMAX], zws[KMAX], zwt[KMAX];
  for (int n = 0; n < a.kjpt; ++n) {
    const bool build = (!a.is_trc && (n == 0 || (n == 1 && a.ddm))) || (a.is_trc && n == 0);
    if (build) {
      const RO<double> coef = (!a.is_trc && n == 0) ? a.avt : a.avs;
      auto wt = [&](int k) -> double {
        if (k == 1) return 0.0;
        const long q = m3 + c.ij + (long)(k - 1) * n2;
        double v = coef[q];
        if (a.add && k <= jpk - 1) v = v + a.add[q];
        return v;
      };
      double wtk = wt(1);
      for (int k = 1; k <= jpk - 1; ++k) {
        const double wtk1 = wt(k + 1);
        const double zwi = -a.p2dt * wtk / d.e3w_n(c.ij, k, c.m);
        zws[k] = -a.p2dt * wtk1 / d.e3w_n(c.ij, k + 1, c.m);
        if (k >= 2) rat[k] = zwi / zwt[k - 1];
        const double zwd = d.e3t_a(c.ij, k, c.m) - zwi - zws[k];
        zwt[k] = (k == 1) ? zwd : zwd - zwi * zws[k - 1] / zwt[k - 1];
        wtk = wtk1;
      }
    }
    const long mo = ((long)c.m * a.kjpt + n) * n3;
    double* lam = b.lam + mo;
    double* tb = b.tb_ad + mo;
    // back-substitution (:252-264) run forwards
    double carry = 0.0;  // what level k receives from level k-1
    for (int k = 1; k <= jpk - 2; ++k) {
      const long q = c.ij + (long)(k - 1) * n2;
      const double x = (lam[q] + carry) * tmsk<double>(ci, k) / zwt[k];
      carry = -zws[k] * x;
      lam[q] = x;
    }
    {
      const long q = c.ij + (long)(jpk - 2) * n2;
      lam[q] = (lam[q] + carry) * tmsk<double>(ci, jpk - 1) / zwt[jpk - 1];
    }
    // elimination (:238-250) run backwards
    double up = 0.0;  // what level k receives from level k+1
    for (int k = jpk - 1; k >= 1; --k) {
      const long q = c.ij + (long)(k - 1) * n2;
      const double y = lam[q] + up;
      up = k >= 2 ? -rat[k] * y : 0.0;
      tb[q] += d.e3t_b(c.ij, k, c.m) * y;
      lam[q] = a.p2dt * d.e3t_n(c.ij, k, c.m) * y;
    }
  }
}

// ---------------------------------------------------------------------- tra_nxt
// tra_nxt (tranxt.F90:66-188, tra_nxt_fix :191-237, linear free surface) at one
// point: lbc of tsa, then the Euler swap (first step of an Euler start) or the
// leapfrog with the Asselin filter on the interior, then lbc of tsb, tsn.
template <class T>
__global__ void k_tra_nxt(Dom<T> d, T* tsb, T* tsn, T* tsa, T atfp, int euler) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const bool edge = !c.interior;
  for (int n = 0; n < 2; ++n) {
    const long o = ((long)c.m * 2 + n) * d.n3 + c.q;
    if (edge) tsa[o] = T(0);
    if (euler) {
      if (c.k <= d.jpk - 1) tsn[o] = tsa[o];
    } else if (edge) {
      tsb[o] = T(0);
      tsn[o] = T(0);
    } else if (c.k <= d.jpk - 1) {
      const T ztn = tsn[o];
      // FP32: the time laplacian from the two differences, which round to small
      // values, instead of from the O(1) values (the same sum in exact arithmetic)
      const T ztd = sizeof(T) == 4 ? (tsa[o] - ztn) - (ztn - tsb[o]) : tsa[o] - T(2) * ztn + tsb[o];
      tsb[o] = ztn + atfp * ztd;
      tsn[o] = tsa[o];
    }
  }
}

// Adjoint of k_tra_nxt: on entry the adjoints of the swapped fields, on exit those
// of the fields before the swap.
__global__ void k_tra_nxt_adj(Dom<double> d, double* bb, double* nn, double* aa, double atfp, int euler) {
  const PtIdx c = pt_index(d);
  if (!c.valid) return;
  const bool edge = !c.interior;
  for (int n = 0; n < 2; ++n) {
    const long o = ((long)c.m * 2 + n) * d.n3 + c.q;
    if (euler) {
      double v = aa[o];
      if (c.k <= d.jpk - 1) {
        v += nn[o];
        nn[o] = 0.0;
      }
      aa[o] = edge ? 0.0 : v;
    } else if (edge) {
      bb[o] = 0.0;
      nn[o] = 0.0;
      aa[o] = 0.0;
    } else if (c.k <= d.jpk - 1) {
      const double b = bb[o], v = nn[o];
      aa[o] = aa[o] + (v + atfp * b);
      nn[o] = b - 2.0 * atfp * b;
      bb[o] = atfp * b;
    }
  }
}

}  // namespace nemo
