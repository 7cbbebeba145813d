// k_diag.cuh -- run control and conservation budgets of the model step:
// stp_ctl's test of extrema (stpctl.F90:112-157) and dia_hsb's heat, salt and volume
// budgets (diahsb.F90:60-239), as two-pass device reductions per member (block
// partials, then one block per member), so the step needs no host synchronisation.
//
// dia_hsb's sums are FP64 double-double sums in both precisions (the reference's
// glob_sum with DDPDD, lib_fortran.F90:300-332): each term is formed in FP64 from the
// stored values, accumulated as a compensated (hi, lo) pair per thread, combined
// pairwise across threads and blocks, and rounded to FP64 once.
#pragma once
#include "nemo_common.cuh"

namespace nemo {

constexpr int DG_THREADS = 256;

// ------------------------------------------------------------------ stp_ctl
// Pass 1 (k_ctl_partial) reduces the six maxima (|ssh|, |U|, -S, S, -T, T; NaN-free
// values, in the field's precision: a maximum is exact) and the NaN flags of ssh, U
// and S into one record per block, marching down each water column (S and T over
// its wet levels only). Pass 2 (k_ctl_final, one thread per member) merges the
// records and applies the blow-up test. Only when the test fires does pass 3
// (k_ctl_locate) find the positions the reference prints, MAXLOC(|ssh|),
// MAXLOC(|U|), MINLOC(S), MAXLOC(S), as the first index in Fortran order holding the
// extreme value (a NaN counts as the extreme), and pass 4 (k_ctl_pos) turns them
// into (i, j, k); both return at once otherwise.
constexpr int CTL_REC = 9;
// out[m * 32 + ...]: zmax(1:6) at 0..5, kindic at 6, positions at 7..17, the locate
// request at 18 and the four keys of the extreme values at 19..22
constexpr int CTL_OUT = 32;

template <class T>
__device__ __forceinline__ double ctl_rec_value(T v) {
  return v == -INFINITY ? -1.7976931348623157e308 : (double)v;
}

// grid (nblk, nmem): block records of member blockIdx.y into part[(m * nblk + b) * CTL_REC]
template <class T>
__global__ void __launch_bounds__(DG_THREADS) k_ctl_partial(Dom<T> d, const T* __restrict__ sshn,
                                                            const T* __restrict__ un, const T* __restrict__ ts,
                                                            double* part) {
  const int m = blockIdx.y, nblk = gridDim.x;
  const long n2 = d.n2, n3 = d.n3;
  const long stride = (long)nblk * DG_THREADS;
  T v[6];
  for (int t = 0; t < 6; ++t) v[t] = T(-INFINITY);
  int nan = 0;
  const T* s2 = sshn + m * n2;
  const T* u3 = un + m * n3;
  const T* t3 = ts + m * 2 * n3;
  for (long p = blockIdx.x * (long)DG_THREADS + threadIdx.x; p < n2; p += stride) {
    const T s = fabs(s2[p]);
    v[0] = fmax(v[0], s);
    nan |= s != s ? 1 : 0;
#pragma unroll 4
    for (int k = 1; k <= d.jpk; ++k) {
      const T x = fabs(u3[p + (long)(k - 1) * n2]);
      v[1] = fmax(v[1], x);
      nan |= x != x ? 2 : 0;
    }
    const ColInfo c = d.ci[p];
#pragma unroll 4
    for (int k = c.tlo; k <= c.thi; ++k) {
      const long q = p + (long)(k - 1) * n2;
      const T tv = t3[q], sv = t3[q + n3];
      v[2] = fmax(v[2], -sv);
      v[3] = fmax(v[3], sv);
      nan |= sv != sv ? 4 : 0;
      v[4] = fmax(v[4], -tv);
      v[5] = fmax(v[5], tv);
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    for (int t = 0; t < 6; ++t) v[t] = fmax(v[t], __shfl_down_sync(0xffffffffu, v[t], off));
    nan |= __shfl_down_sync(0xffffffffu, nan, off);
  }
  __shared__ T s_v[DG_THREADS / 32][6];
  __shared__ int s_nan[DG_THREADS / 32];
  if ((threadIdx.x & 31) == 0) {
    for (int t = 0; t < 6; ++t) s_v[threadIdx.x >> 5][t] = v[t];
    s_nan[threadIdx.x >> 5] = nan;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < DG_THREADS / 32; ++w) {
      for (int t = 0; t < 6; ++t) v[t] = fmax(v[t], s_v[w][t]);
      nan |= s_nan[w];
    }
    double* r = part + ((long)m * nblk + blockIdx.x) * CTL_REC;
    for (int t = 0; t < 6; ++t) r[t] = ctl_rec_value(v[t]);
    for (int t = 0; t < 3; ++t) r[6 + t] = (nan >> t) & 1 ? 1.0 : 0.0;
  }
}

// One block (DG_THREADS) per member: the member's records merged, the blow-up test
// (:149-157), its results out[m * CTL_OUT ..] = zmax(1:6), kindic; when it fires the
// locate request, the keys of the extremes, idx = the largest index (to be lowered
// by k_ctl_locate), and flag = 1.
template <class T>
__global__ void __launch_bounds__(DG_THREADS) k_ctl_final(Dom<T> d, const double* part, int nblk, int someoce,
                                                          double* out, unsigned long long* idx, int* flag) {
  const int m = blockIdx.x;
  double z[6];
  for (int t = 0; t < 6; ++t) z[t] = -1.7976931348623157e308;
  int nan = 0;
  for (int b = threadIdx.x; b < nblk; b += DG_THREADS) {
    const double* r = part + ((long)m * nblk + b) * CTL_REC;
    for (int t = 0; t < 6; ++t) z[t] = fmax(z[t], r[t]);
    for (int t = 0; t < 3; ++t) nan |= r[6 + t] != 0.0 ? 1 << t : 0;
  }
  for (int off = 16; off > 0; off >>= 1) {
    for (int t = 0; t < 6; ++t) z[t] = fmax(z[t], __shfl_down_sync(0xffffffffu, z[t], off));
    nan |= __shfl_down_sync(0xffffffffu, nan, off);
  }
  __shared__ double s_z[DG_THREADS / 32][6];
  __shared__ int s_nan[DG_THREADS / 32];
  if ((threadIdx.x & 31) == 0) {
    for (int t = 0; t < 6; ++t) s_z[threadIdx.x >> 5][t] = z[t];
    s_nan[threadIdx.x >> 5] = nan;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < DG_THREADS / 32; ++w) {
    for (int t = 0; t < 6; ++t) z[t] = fmax(z[t], s_z[w][t]);
    nan |= s_nan[w];
  }
  const bool n0 = nan & 1, n1 = (nan >> 1) & 1, n2s = (nan >> 2) & 1;
  double key[4] = {n0 ? INFINITY : z[0], n1 ? INFINITY : z[1], n2s ? -INFINITY : -z[2], n2s ? INFINITY : z[3]};
  if (n0) z[0] = NAN;
  if (n1) z[1] = NAN;
  if (n2s) { z[2] = NAN; z[3] = NAN; }
  const bool trip = someoce && (z[0] > 20.0 || z[1] > 10.0 || z[2] >= 0.0 || z[3] >= 100.0 || z[3] < 0.0 ||
                                isnan(z[0] + z[1] + z[2]));
  double* o = out + (long)m * CTL_OUT;
  for (int t = 0; t < 6; ++t) o[t] = z[t];
  o[6] = trip ? -3.0 : 0.0;
  for (int t = 0; t < 11; ++t) o[7 + t] = 0.0;
  o[18] = trip ? 1.0 : 0.0;
  for (int t = 0; t < 4; ++t) {
    o[19 + t] = key[t];
    idx[m * 4 + t] = 0xffffffffffffffffULL;
  }
  if (trip) atomicExch(flag, 1);
}

// grid (nblk, nmem): the first index in Fortran order of each extreme of a member
// whose test fired (atomicMin into idx); returns at once for the others
template <class T>
__global__ void __launch_bounds__(DG_THREADS) k_ctl_locate(Dom<T> d, const T* __restrict__ sshn,
                                                           const T* __restrict__ un, const T* __restrict__ ts,
                                                           const double* out, unsigned long long* idx) {
  const int m = blockIdx.y;
  const double* o = out + (long)m * CTL_OUT;
  if (o[18] == 0.0) return;
  const double k0 = o[19], k1 = o[20], k2 = o[21], k3 = o[22];
  const long n2 = d.n2, n3 = d.n3;
  const long stride = (long)gridDim.x * DG_THREADS;
  unsigned long long best[4] = {~0ULL, ~0ULL, ~0ULL, ~0ULL};
  const T* s2 = sshn + m * n2;
  const T* u3 = un + m * n3;
  const T* t3 = ts + m * 2 * n3;
  for (long p = blockIdx.x * (long)DG_THREADS + threadIdx.x; p < n2; p += stride) {
    const T s = fabs(s2[p]);
    if ((s != s ? INFINITY : (double)s) == k0 && (unsigned long long)p < best[0]) best[0] = p;
    for (int k = 1; k <= d.jpk; ++k) {
      const long q = p + (long)(k - 1) * n2;
      const T x = fabs(u3[q]);
      if ((x != x ? INFINITY : (double)x) == k1 && (unsigned long long)q < best[1]) best[1] = q;
    }
    const ColInfo c = d.ci[p];
    for (int k = c.tlo; k <= c.thi; ++k) {
      const long q = p + (long)(k - 1) * n2;
      const T sv = t3[q + n3];
      if ((sv != sv ? -INFINITY : (double)sv) == k2 && (unsigned long long)q < best[2]) best[2] = q;
      if ((sv != sv ? INFINITY : (double)sv) == k3 && (unsigned long long)q < best[3]) best[3] = q;
    }
  }
  for (int t = 0; t < 4; ++t) {
    unsigned long long b = best[t];
    for (int off = 16; off > 0; off >>= 1) {
      const unsigned long long o2 = __shfl_down_sync(0xffffffffu, b, off);
      b = o2 < b ? o2 : b;
    }
    if ((threadIdx.x & 31) == 0 && b != ~0ULL) atomicMin(idx + m * 4 + t, b);
  }
}

// One thread per member: the positions (i, j[, k], 1-based) of the located extremes
template <class T>
__global__ void k_ctl_pos(Dom<T> d, double* out, const unsigned long long* idx) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= d.nmem) return;
  double* o = out + (long)m * CTL_OUT;
  if (o[18] == 0.0) return;
  const long long n2 = d.n2, jpi = d.jpi, jpj = d.jpj;
  const unsigned long long* x = idx + m * 4;
  if (x[0] != ~0ULL) { o[7] = (double)(x[0] % jpi + 1); o[8] = (double)(x[0] / jpi + 1); }
  if (x[1] != ~0ULL) {
    o[9] = (double)(x[1] % jpi + 1); o[10] = (double)((x[1] / jpi) % jpj + 1); o[11] = (double)(x[1] / n2 + 1);
  }
  if (x[2] != ~0ULL && x[3] != ~0ULL) {
    o[12] = (double)(x[2] % jpi + 1); o[13] = (double)((x[2] / jpi) % jpj + 1); o[14] = (double)(x[2] / n2 + 1);
    o[15] = (double)(x[3] % jpi + 1); o[16] = (double)((x[3] / jpi) % jpj + 1); o[17] = (double)(x[3] / n2 + 1);
  }
}

// ------------------------------------------------------------------ dia_hsb
constexpr int HSB_NS = 13;  // global sums of one dia_hsb call

// Knuth's two-sum of a double-double (hi, lo) and a double x
__device__ __forceinline__ void dd_acc(double& hi, double& lo, double x) {
  const double s = __dadd_rn(hi, x);
  const double bp = __dadd_rn(s, -hi);
  const double err = __dadd_rn(__dadd_rn(hi, -__dadd_rn(s, -bp)), __dadd_rn(x, -bp));
  hi = s;
  lo = __dadd_rn(lo, err);
}
// (hi, lo) += (bh, bl)
__device__ __forceinline__ void dd_merge(double& hi, double& lo, double bh, double bl) {
  dd_acc(hi, lo, bh);
  lo = __dadd_rn(lo, bl);
}

template <class T>
struct HsbArgs {
  T *tsn, *tsb;                    // masked in place (diahsb.F90:88-89)
  const T *sshn, *emp, *rnf, *tsc, *qsr, *wn;
  E3<T> e3t;                       // e3t_n: bound field or the rest state
  const double *surf;              // e1e2t * tmask_i (2-D, shared by the members)
  double *ssh_ini, *ssh_hc_ini, *ssh_sc_ini;   // (jpi,jpj) per member
  double *e3t_ini, *hc_ini, *sc_ini;           // (jpi,jpj,jpk) per member
  const double* tmask_h;
  double* state;                   // per member: frc_v, frc_t, frc_s, frc_wn_t, frc_wn_s, surf_tot
  double* out;                     // per member NEMO_HSB_N results
  double rdt, r1_rau0, r1_rau0_rcp;
  int linssh, traqsr;
};

// dia_hsb_rst( nit000, 'READ' ) without restart (:283-311): the initial fields
template <class T>
__global__ void k_hsb_init(Dom<T> d, HsbArgs<T> a) {
  const long n2 = d.n2, n3 = d.n3;
  const long tot = (long)d.nmem * n3;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < tot; g += (long)gridDim.x * blockDim.x) {
    const int m = (int)(g / n3);
    const long q = g - m * n3, p = q % n2;
    const int k = (int)(q / n2) + 1;
    const ColInfo c = d.ci[p];
    const double tm = (k >= c.tlo && k <= c.thi) ? 1.0 : 0.0;
    const double e3 = (double)a.e3t(p, k, m);
    const T* ts = a.tsn + (long)m * 2 * n3;
    a.e3t_ini[g] = e3 * tm;
    a.hc_ini[g] = (double)ts[q] * e3 * tm;
    a.sc_ini[g] = (double)ts[q + n3] * e3 * tm;
    if (k == 1) {
      const double s = (double)a.sshn[m * n2 + p];
      a.ssh_ini[m * n2 + p] = s;
      if (a.linssh) {
        a.ssh_hc_ini[m * n2 + p] = (double)ts[q] * s;
        a.ssh_sc_ini[m * n2 + p] = (double)ts[q + n3] * s;
      }
    }
  }
}

// grid (nblk, nmem): the 13 double-double sums of one call, block partials into
// part[((m * nblk + b) * HSB_NS + s) * 2 + hi/lo]:
//  0 -(emp - rnf) * surf, 1 sbc_tsc(T) * surf, 2 sbc_tsc(S) * surf, 3 qsr * surf,
//  4 surf * wn(1) * tsb(1,T), 5 ... (1,S)                      (mask tmask_i, :93-120)
//  6 surf * sshn - surf_ini * ssh_ini, 7/8 surf * (tsn(1) * sshn - ssh_hc/sc_ini)
//  9 (surf e3t_n - surf_ini e3t_ini) tmask, 10/11 heat / salt content variations,
//  12 surf e3t_n tmask                          (mask tmask_h, levels 1..jpk-1, :130-193)
// surf_ini = surf (no ice-sheet coupling).
template <class T>
__global__ void __launch_bounds__(DG_THREADS) k_hsb_partial(Dom<T> d, HsbArgs<T> a, double* part) {
  const int m = blockIdx.y, nblk = gridDim.x;
  const long n2 = d.n2, n3 = d.n3;
  const long stride = (long)nblk * DG_THREADS;
  double hi[HSB_NS], lo[HSB_NS];
  for (int s = 0; s < HSB_NS; ++s) { hi[s] = 0.0; lo[s] = 0.0; }
  T* tsn = a.tsn + (long)m * 2 * n3;
  T* tsb = a.tsb + (long)m * 2 * n3;
  const long m2 = (long)m * n2;
  // masking of tsn, tsb on every level (only where it changes a value) and the 3-D sums
  for (long q = blockIdx.x * (long)DG_THREADS + threadIdx.x; q < n3; q += stride) {
    const long p = q % n2;
    const int k = (int)(q / n2) + 1;
    const ColInfo c = d.ci[p];
    const bool wet = k >= c.tlo && k <= c.thi;
    if (!wet) {
      if (tsn[q] != T(0)) tsn[q] = T(0);
      if (tsn[q + n3] != T(0)) tsn[q + n3] = T(0);
      if (tsb[q] != T(0)) tsb[q] = T(0);
      if (tsb[q + n3] != T(0)) tsb[q + n3] = T(0);
    }
    if (k <= d.jpk - 1) {
      const double tmh = a.tmask_h[p], tm = wet ? 1.0 : 0.0, sf = a.surf[p];
      const double e3 = (double)a.e3t(p, k, m);
      const long g = m * n3 + q;
      const double se3 = sf * e3;
      dd_acc(hi[9], lo[9], (se3 - sf * a.e3t_ini[g]) * tm * tmh);
      dd_acc(hi[10], lo[10], (se3 * (double)tsn[q] - sf * a.hc_ini[g]) * tm * tmh);
      dd_acc(hi[11], lo[11], (se3 * (double)tsn[q + n3] - sf * a.sc_ini[g]) * tm * tmh);
      dd_acc(hi[12], lo[12], se3 * tm * tmh);
    }
  }
  for (long p = blockIdx.x * (long)DG_THREADS + threadIdx.x; p < n2; p += stride) {
    const double tmi = d.tmask_i[p], tmh = a.tmask_h[p], sf = a.surf[p];
    // the surface level is masked by the loop above or is wet; read it masked
    const ColInfo c = d.ci[p];
    const double tm1 = (1 >= c.tlo && 1 <= c.thi) ? 1.0 : 0.0;
    const double rnf = a.rnf ? (double)a.rnf[m2 + p] : 0.0;
    dd_acc(hi[0], lo[0], -((double)a.emp[m2 + p] - rnf + 0.0) * sf * tmi);
    dd_acc(hi[1], lo[1], (double)a.tsc[2 * m2 + p] * sf * tmi);
    dd_acc(hi[2], lo[2], (double)a.tsc[2 * m2 + n2 + p] * sf * tmi);
    if (a.traqsr) dd_acc(hi[3], lo[3], (double)a.qsr[m2 + p] * sf * tmi);
    const double ssh = (double)a.sshn[m2 + p];
    dd_acc(hi[6], lo[6], (sf * ssh - sf * a.ssh_ini[m2 + p]) * tmh);
    if (a.linssh) {
      const double wn1 = (double)a.wn[(long)m * n3 + p];
      dd_acc(hi[4], lo[4], sf * wn1 * ((double)tsb[p] * tm1) * tmi);
      dd_acc(hi[5], lo[5], sf * wn1 * ((double)tsb[p + n3] * tm1) * tmi);
      dd_acc(hi[7], lo[7], sf * ((double)tsn[p] * tm1 * ssh - a.ssh_hc_ini[m2 + p]) * tmh);
      dd_acc(hi[8], lo[8], sf * ((double)tsn[p + n3] * tm1 * ssh - a.ssh_sc_ini[m2 + p]) * tmh);
    }
  }
  // warp and block combination of the pairs
  __shared__ double s_hi[DG_THREADS / 32][HSB_NS], s_lo[DG_THREADS / 32][HSB_NS];
  for (int off = 16; off > 0; off >>= 1)
    for (int s = 0; s < HSB_NS; ++s) {
      const double bh = __shfl_down_sync(0xffffffffu, hi[s], off);
      const double bl = __shfl_down_sync(0xffffffffu, lo[s], off);
      dd_merge(hi[s], lo[s], bh, bl);
    }
  if ((threadIdx.x & 31) == 0)
    for (int s = 0; s < HSB_NS; ++s) { s_hi[threadIdx.x >> 5][s] = hi[s]; s_lo[threadIdx.x >> 5][s] = lo[s]; }
  __syncthreads();
  if (threadIdx.x < HSB_NS) {
    const int s = threadIdx.x;
    double h = s_hi[0][s], l = s_lo[0][s];
    for (int w = 1; w < DG_THREADS / 32; ++w) dd_merge(h, l, s_hi[w][s], s_lo[w][s]);
    double* r = part + (((long)m * nblk + blockIdx.x) * HSB_NS + s) * 2;
    r[0] = h;
    r[1] = l;
  }
}

// One block per member (HSB_NS threads): the sums, the forcing accumulators and the
// drifts (diahsb.F90:93-193).
template <class T>
__global__ void k_hsb_final(Dom<T> d, HsbArgs<T> a, const double* part, int nblk) {
  const int m = blockIdx.x;
  __shared__ double tot[HSB_NS];
  if (threadIdx.x < HSB_NS) {
    const int s = threadIdx.x;
    double h = 0.0, l = 0.0;
    for (int b = 0; b < nblk; ++b) {
      const double* r = part + (((long)m * nblk + b) * HSB_NS + s) * 2;
      dd_merge(h, l, r[0], r[1]);
    }
    tot[s] = __dadd_rn(h, l);
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double* st = a.state + (long)m * 8;
  const double z_frc_trd_v = a.r1_rau0 * tot[0];
  double z_frc_trd_t = tot[1];
  const double z_frc_trd_s = tot[2];
  if (a.traqsr) z_frc_trd_t = z_frc_trd_t + a.r1_rau0_rcp * tot[3];
  st[0] = st[0] + z_frc_trd_v * a.rdt;
  st[1] = st[1] + z_frc_trd_t * a.rdt;
  st[2] = st[2] + z_frc_trd_s * a.rdt;
  if (a.linssh) {
    st[3] = st[3] + (-tot[4]) * a.rdt;
    st[4] = st[4] + (-tot[5]) * a.rdt;
  }
  double zdiff_v1 = tot[6] - st[0];
  double zdiff_v2 = tot[9];
  if (!a.linssh) zdiff_v2 = zdiff_v2 - st[0];
  const double zdiff_hc = tot[10] - st[1], zdiff_sc = tot[11] - st[2];
  double* o = a.out + (long)m * 16;
  o[0] = st[0]; o[1] = st[1]; o[2] = st[2]; o[3] = st[3]; o[4] = st[4];
  o[5] = zdiff_v1; o[6] = zdiff_v2; o[7] = zdiff_hc; o[8] = zdiff_sc;
  if (a.linssh) {
    o[9] = zdiff_hc + tot[7]; o[10] = zdiff_sc + tot[8];
    o[11] = tot[7] - st[3]; o[12] = tot[8] - st[4];
  } else {
    o[9] = o[10] = o[11] = o[12] = 0.0;
  }
  o[13] = tot[12];
  o[14] = st[5];
  o[15] = 0.0;
}

}  // namespace nemo
