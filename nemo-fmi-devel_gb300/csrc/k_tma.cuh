// k_tma.cuh -- tracer stencils with TMA-staged planes (FP32, sm_103a).
//
// A block owns a 32 x 8 tile of columns and marches down a chunk of levels. Each
// level's tracer plane, with a one-point halo on every side, is copied into shared
// memory by one tensor copy (cp.async.bulk.tensor) per tracer, issued by one thread
// several levels ahead into a ring of slots, each slot guarded by an mbarrier that
// the copy completes. The threads read every neighbour from shared memory, so the
// k-march no longer waits on L1/L2 for the halo values of the neighbouring columns,
// and the loads are issued without any per-thread instructions.
//
// TMA rules kept here: the innermost box coordinate starts on a 16-byte boundary (the
// x origin is the tile origin minus 4 floats), the box's inner extent is 160 bytes,
// every slot starts on a 128-byte boundary, out-of-range rows/columns are filled with
// zeros by the copy (loads only; nothing is stored through TMA), and every wait on an
// mbarrier is bounded: after max_polls polls the kernel records an error, waits
// (bounded) for its copies still in flight and returns.
#pragma once
#include <cuda.h>

#include "k_hot.cuh"

namespace nemo {

constexpr int TM_X = 32, TM_Y = 8;                 // tile (threads per block)
constexpr int TM_W = TM_X + 8, TM_H = TM_Y + 2;   // plane box: x from i0-4 (aligned), y from j0-1
constexpr int TM_PLANE = 416;                      // floats per plane slot (TM_W*TM_H = 400, padded to 128 B)
constexpr int TM_NS = 4;                           // ring slots (levels in flight)
constexpr unsigned TM_PLANE_BYTES = TM_W * TM_H * 4;
constexpr int TM_TILE = TM_X * TM_Y;                // floats of a tile box (no halo): the slopes
constexpr unsigned TM_TILE_BYTES = TM_TILE * 4;

// The tensor maps of one launch: the before tracers (plane box with halo) and the four
// iso-neutral slopes (tile box), each a 3-D tensor (jpi, jpj, levels x fields x members).
struct alignas(64) IsoMaps {
  CUtensorMap tb, uslp, vslp, wslpi, wslpj;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// the arrival of the issuing thread, announcing the bytes the copies will deliver
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// the box of the map at (x, y, z) into shared memory
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
// After a failed wait a kernel still waits for every copy it has issued, with this
// bound (independent of the caller's max_polls), before it returns.
constexpr int TM_DRAIN_POLLS = 1 << 16;

// wait for the completion of phase `parity`; false after max_polls polls of at most
// ~1 us each (suspend-time hint), so a wait never lasts longer than ~max_polls us
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int max_polls) {
  for (int it = 0; it < max_polls; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity), "r"(1000u)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Up to NF tensor maps of one launch, each a 3-D tensor of floats (jpi, jpj, levels x
// fields x members) with the plane box {TM_W, TM_H, 1}.
template <int NF>
struct alignas(64) PlaneMaps {
  CUtensorMap m[NF];
};

// A ring of TM_NS slots in shared memory for a k-march: slot s holds up to NF plane
// boxes of one level. Plane g (a running count over the kernel) lives in slot
// g % TM_NS and completes phase (g / TM_NS) & 1 of that slot's mbarrier.
template <class T, int NF>
struct PlaneRing {
  T* base;                   // [TM_NS][NF][TM_PLANE], 128-byte aligned
  unsigned long long* bar;   // [TM_NS]
  __device__ __forceinline__ const T* plane(unsigned g, int f) const {
    return base + ((g % TM_NS) * NF + f) * TM_PLANE;
  }
  __device__ __forceinline__ bool wait(unsigned g, int max_polls) const {
    return mbar_wait(&bar[g % TM_NS], (g / TM_NS) & 1, max_polls);
  }
  // one thread: the nf planes of plane g, field f at (x, y, z(f))
  template <class Z>
  __device__ __forceinline__ void issue(unsigned g, const PlaneMaps<NF>& maps, int nf, int x, int y, Z z) const {
    const unsigned s = g % TM_NS;
    mbar_expect_tx(&bar[s], (unsigned)nf * TM_PLANE_BYTES);
    for (int f = 0; f < nf; ++f) tma_load_3d(base + (s * NF + f) * TM_PLANE, &maps.m[f], x, y, z(f), &bar[s]);
  }
  // after a failure: wait (bounded) for the copies still in flight of the planes issued
  __device__ void drain(unsigned issued, int max_polls) const {
    for (unsigned s = 0; s < TM_NS; ++s) {
      if (issued <= s) continue;
      const unsigned last = s + TM_NS * ((issued - 1 - s) / TM_NS);
      mbar_wait(&bar[s], (last / TM_NS) & 1, max_polls);
    }
  }
};

// Iso-neutral fluxes (traldf_iso.F90:146-357), the configuration of k_iso_flux_hot,
// with the tracer planes and the slopes of every level staged by TMA, so that no
// per-level global load is left in the k-march. The tracer map describes ptb as a
// 3-D tensor (jpi, jpj, jpk * kjpt * nmem), the slope maps each slope field as
// (jpi, jpj, jpk * nmem). Same arithmetic in the same order as
// k_iso_flux_hot; the vertical term (ah_wslp2 - akz) * dk(tb) of :323-332 is exactly 0
// here (akz = ah_wslp2) and is left out.
template <class T>
__global__ void __launch_bounds__(TM_X * TM_Y, 2)
    k_iso_flux_tma(Dom<T> d, LdfArgs<T> a, const __grid_constant__ IsoMaps maps, int* err, int max_polls) {
  static_assert(sizeof(T) == 4, "the TMA kernel is the FP32 form");
  // ring slot: two tracer planes with halo, then the four slope tiles of the level
  __shared__ alignas(128) T pl[TM_NS][2][TM_PLANE];
  __shared__ alignas(128) T sl[TM_NS][4][TM_TILE];
  __shared__ alignas(8) unsigned long long bar[TM_NS];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TM_X + tx;
  const int jpi = d.jpi, jpj = d.jpj, jpk = d.jpk, n2 = (int)d.n2;
  const int nch = (jpk + KCH - 1) / KCH;
  const int m = (int)blockIdx.z / nch, ch = (int)blockIdx.z - m * nch;
  const int k0 = ch * KCH + 1, k1 = k0 + KCH - 1 < jpk ? k0 + KCH - 1 : jpk;
  const int i0 = (int)blockIdx.x * TM_X, j0 = (int)blockIdx.y * TM_Y;  // tile origin (0-based)
  const int i = i0 + tx + 1, j = j0 + ty + 1;
  const bool valid = i <= jpi && j <= jpj;
  const bool icol = i >= 2 && i <= jpi - 1 && j >= 2 && j <= jpj - 1;
  const bool face = i <= jpi - 1 && j <= jpj - 1;
  const int ij = valid ? (i - 1) + (j - 1) * jpi : 0;
  __shared__ int s_abort;  // an earlier failure of this step: skip the work (same for the whole block)
  if (tid == 0) {
    s_abort = *(volatile int*)err != 0;
    for (int s = 0; s < TM_NS; ++s) mbar_init(&bar[s], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (s_abort) return;
  const long m3 = (long)m * d.n3;
  if (valid) {  // akz = ah_wslp2 where the interior sweep writes neither (traldf_iso.F90:200-201)
    auto copy = [&](int k) {
      const long q = m3 + ij + (long)(k - 1) * n2;
      a.akz[q] = a.ah_wslp2[q];
    };
    if (!icol) {
      for (int k = k0; k <= k1; ++k) copy(k);
    } else {
      if (k0 == 1) copy(1);
      if (k1 == jpk) copy(jpk);
    }
  }
  // per-column data of the face-owning threads
  ColInfo ci{}, cie{}, cin{}, ciw{}, cis{};
  T e2_e1u = T(0), e1_e2v = T(0), e2u = T(0), e1v = T(0), e2t = T(0), e1t = T(0);
  if (face) {
    ci = d.ci[ij]; cie = d.ci[ij + 1]; cin = d.ci[ij + jpi];
    e2_e1u = d.e2_e1u[ij]; e1_e2v = d.e1_e2v[ij]; e2u = d.e2u[ij]; e1v = d.e1v[ij];
    if (icol) {
      ciw = d.ci[ij - 1]; cis = d.ci[ij - jpi];
      e2t = d.e2t[ij]; e1t = d.e1t[ij];
    }
  }
  const T aht = a.aht_c;
  const T* e3u = d.e3u_n.p.p;
  const T* e3v = d.e3v_n.p.p;
  T* ahw_out = a.ah_wslp2 + m3 + ij;
  T* akz_out = a.akz + m3 + ij;
  const int o = (ty + 1) * TM_W + tx + 4;  // this column in a plane slot
  const int os = ty * TM_X + tx;           // this column in a slope tile
  unsigned P = 0;       // planes of the finished and current passes: plane g -> slot g % TM_NS, parity (g / TM_NS) & 1
  unsigned issued = 0;  // planes issued (thread 0)
  bool ok = true;
  for (int n0 = 0; n0 < a.kjpt && ok; n0 += 2) {
    const int nt = a.kjpt - n0 < 2 ? a.kjpt - n0 : 2;
    const int np = (k1 + 1 < jpk ? k1 + 1 : jpk) - k0 + 1;  // planes k0 .. min(k1+1, jpk)
    const unsigned pb = P;
    auto issue = [&](int p) {
      const unsigned g = pb + (unsigned)p, s = g % TM_NS;
      issued = g + 1;
      mbar_expect_tx(&bar[s], (unsigned)nt * TM_PLANE_BYTES + 4 * TM_TILE_BYTES);
      for (int nn = 0; nn < nt; ++nn)
        tma_load_3d(&pl[s][nn][0], &maps.tb, i0 - 4, j0 - 1, (m * a.kjpt + n0 + nn) * jpk + (k0 - 1 + p), &bar[s]);
      const int zs = m * jpk + (k0 - 1 + p);
      tma_load_3d(&sl[s][0][0], &maps.uslp, i0, j0, zs, &bar[s]);
      tma_load_3d(&sl[s][1][0], &maps.vslp, i0, j0, zs, &bar[s]);
      tma_load_3d(&sl[s][2][0], &maps.wslpi, i0, j0, zs, &bar[s]);
      tma_load_3d(&sl[s][3][0], &maps.wslpj, i0, j0, zs, &bar[s]);
    };
    if (tid == 0)
      for (int p = 0; p < TM_NS && p < np; ++p) issue(p);
    P += (unsigned)np;
    const T* tbg[2];
    T *fu[2], *fv[2], *fw[2];
    for (int nn = 0; nn < 2; ++nn) {
      const long mo = ((long)m * a.kjpt + n0 + (nn < nt ? nn : 0)) * d.n3 + ij;
      tbg[nn] = a.ptb.p + mo;
      fu[nn] = a.zftu + mo;
      fv[nn] = a.zftv + mo;
      fw[nn] = a.ztfw + mo;
    }
    // carried masks (as k_iso_flux_hot)
    T t0m = t_in<T>(ci, k0 - 1), t0 = t_in<T>(ci, k0), t0p = t_in<T>(ci, k0 + 1);
    T tem = t_in<T>(cie, k0 - 1), te_ = t_in<T>(cie, k0), tep = t_in<T>(cie, k0 + 1);
    T tnm = t_in<T>(cin, k0 - 1), tn_ = t_in<T>(cin, k0), tnp = t_in<T>(cin, k0 + 1);
    T u0m = u_in<T>(ci, k0 - 1), u0 = u_in<T>(ci, k0), uwm = u_in<T>(ciw, k0 - 1), uw = u_in<T>(ciw, k0);
    T v0m = v_in<T>(ci, k0 - 1), v0 = v_in<T>(ci, k0), vsm = v_in<T>(cis, k0 - 1), vs = v_in<T>(cis, k0);
    // carried per tracer: zdk1t(k-1) at (i,j), (i+1,j), (i,j+1); zdit at (i,j), (i-1,j)
    // and zdjt at (i,j), (i,j-1) of level k-1
    T k10[2] = {}, k1e[2] = {}, k1n[2] = {}, di0[2] = {}, diw[2] = {}, dj0[2] = {}, djs[2] = {};
    if (face && k0 > 1)  // level k0-1 from global memory, once per chunk
      for (int nn = 0; nn < nt; ++nn) {
        const T* t = tbg[nn];
        const int qm = (k0 - 2) * n2, q0 = (k0 - 1) * n2;
        const T wk = t0m * t0, wke = tem * te_, wkn = tnm * tn_;
        const T a0 = __ldg(t + qm), ae = __ldg(t + qm + 1), an = __ldg(t + qm + jpi);
        k10[nn] = (a0 - __ldg(t + q0)) * wk;
        k1e[nn] = (ae - __ldg(t + q0 + 1)) * wke;
        k1n[nn] = (an - __ldg(t + q0 + jpi)) * wkn;
        if (icol) {
          const T aw = __ldg(t + qm - 1), as = __ldg(t + qm - jpi);
          di0[nn] = (ae - a0) * u0m;
          diw[nn] = (a0 - aw) * uwm;
          dj0[nn] = (an - a0) * v0m;
          djs[nn] = (a0 - as) * vsm;
        }
      }
    ok = mbar_wait(&bar[pb % TM_NS], (pb / TM_NS) & 1, max_polls);
    int q = (k0 - 1) * n2;
    for (int k = k0; k <= k1; ++k, q += n2) {
      const int p = k - k0;
      if (k == jpk) {  // interior: ztfw = 0 at jpk
        if (icol)
          for (int nn = 0; nn < nt; ++nn) fw[nn][q] = T(0);
        break;
      }
      const unsigned g1 = pb + (unsigned)p + 1;
      ok = mbar_wait(&bar[g1 % TM_NS], (g1 / TM_NS) & 1, max_polls) && ok;
      const T* A0 = &pl[(pb + (unsigned)p) % TM_NS][0][0];
      const T* A1 = &pl[g1 % TM_NS][0][0];
      const T* S0 = &sl[(pb + (unsigned)p) % TM_NS][0][0];
      if (face) {
        const T wk = k == 1 ? t0 : t0m * t0, wk1 = t0 * t0p;
        const T wke = k == 1 ? te_ : tem * te_, wk1e = te_ * tep;
        const T wkn = k == 1 ? tn_ : tnm * tn_, wk1n = tn_ * tnp;
        // horizontal fluxes' coefficients (:255-276)
        T pah = aht * u0;
        const T zabe1 = pah * e2_e1u * __ldg(e3u + k - 1);
        const T zmsku_h = rcount(wke + wk1 + wk1e + wk);
        const T zcof1 = -pah * e2u * S0[os] * zmsku_h;
        pah = aht * v0;
        const T zabe2 = pah * e1_e2v * __ldg(e3v + k - 1);
        const T zmskv_h = rcount(wkn + wk1 + wk1n + wk);
        const T zcof2 = -pah * e1v * S0[TM_TILE + os] * zmskv_h;
        // vertical flux coefficients and ah_wslp2 = akz (:146-164, :200-201, :291-321)
        const bool vface = icol && k >= 2;
        T zcoef3 = T(0), zcoef4 = T(0);
        if (vface) {
          const T zmsku = wk * rcount(u0m + uw + uwm + u0);
          const T zmskv = wk * rcount(v0m + vs + vsm + v0);
          const T zahu_w = (aht * u0m + aht * uw + aht * uwm + aht * u0) * zmsku;
          const T zahv_w = (aht * v0m + aht * vs + aht * vsm + aht * v0) * zmskv;
          const T wi = S0[2 * TM_TILE + os], wj = S0[3 * TM_TILE + os];
          const T ahw = zahu_w * wi * wi + zahv_w * wj * wj;
          ahw_out[q] = ahw;
          akz_out[q] = ahw;
          zcoef3 = -zahu_w * e2t * zmsku * wi;
          zcoef4 = -zahv_w * e1t * zmskv * wj;
        }
#pragma unroll
        for (int nn = 0; nn < 2; ++nn) {
          if (nn >= nt) break;
          const T* B0 = A0 + nn * TM_PLANE;
          const T* B1 = A1 + nn * TM_PLANE;
          const T tc = B0[o], te = B0[o + 1], tn = B0[o + TM_W];
          const T t1 = B1[o], te1 = B1[o + 1], tn1 = B1[o + TM_W];
          // vertical gradients (:250-254)
          const T dk1_0 = (tc - t1) * wk1, dk1_e = (te - te1) * wk1e, dk1_n = (tn - tn1) * wk1n;
          const T dk0_0 = k == 1 ? dk1_0 : k10[nn];
          const T dk0_e = k == 1 ? dk1_e : k1e[nn];
          const T dk0_n = k == 1 ? dk1_n : k1n[nn];
          const T zdi = (te - tc) * u0;
          const T zdj = (tn - tc) * v0;
          fu[nn][q] = (zabe1 * zdi + zcof1 * (dk0_e + dk1_0 + dk1_e + dk0_0)) * u0;
          fv[nn][q] = (zabe2 * zdj + zcof2 * (dk0_n + dk1_0 + dk1_n + dk0_0)) * v0;
          if (icol) {
            const T tw = B0[o - 1], ts = B0[o - TM_W];
            const T zdiw = (tc - tw) * uw;
            const T zdjs = (tc - ts) * vs;
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
        }
      }
      // masks of level k+1 (and k+2 for T)
      t0m = t0; t0 = t0p; t0p = t_in<T>(ci, k + 2);
      tem = te_; te_ = tep; tep = t_in<T>(cie, k + 2);
      tnm = tn_; tn_ = tnp; tnp = t_in<T>(cin, k + 2);
      u0m = u0; u0 = u_in<T>(ci, k + 1); uwm = uw; uw = u_in<T>(ciw, k + 1);
      v0m = v0; v0 = v_in<T>(ci, k + 1); vsm = vs; vs = v_in<T>(cis, k + 1);
      // every thread is done with plane k: its slot takes plane k + TM_NS
      if (!__syncthreads_and(ok)) {
        ok = false;
        break;
      }
      if (tid == 0 && p + TM_NS < np) issue(p + TM_NS);
    }
  }
  if (!ok) {  // a copy did not arrive in time: record it, wait (bounded) for the copies in flight
    if (tid == 0) {
      atomicExch(err, TM_ERR);
      for (unsigned s = 0; s < TM_NS; ++s) {
        if (issued <= s) continue;
        const unsigned last = s + TM_NS * ((issued - 1 - s) / TM_NS);  // last plane issued into slot s
        mbar_wait(&bar[s], (last / TM_NS) & 1, TM_DRAIN_POLLS);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// FCT stages a, b and c fused (traadv_fct.F90:119-297 with nonosc :330-428): no
// intermediate (zwi, the antidiffusive fluxes, the limiter coefficients) goes to HBM.
// A block owns a 32 x 8 tile of columns for the whole column and marches down: step t
// computes stage a at level t on the tile with a 2-point halo (R2), stage b at level
// t-1 with a 1-point halo (R1) and stage c at level t-2 on the tile, each from shared
// memory. The inputs of a level (un, vn, wn and one tracer's tb, tn; one tracer per
// pass) arrive as TMA boxes covering a 3-point halo (x origin aligned to 16 bytes) in
// a ring of FF_NS levels. The halo points are recomputed by neighbouring blocks
// (1.7x stage-a and 1.3x stage-b work) instead of being stored and reloaded.
// Same arithmetic in the same order as k_fct_a_hot, k_fct_b_hot and k_fct_c_hot.
constexpr int FF_BW = 40, FF_BH = 14, FF_PL = 576;  // input box: x from i0-4, y from j0-3 (560 floats, padded)
constexpr unsigned FF_PL_BYTES = FF_BW * FF_BH * 4;
constexpr int FF_NS = 6;                              // input ring: levels t-2 .. t+3
constexpr int FF_NIN = 5;                             // un, vn, wn, tb, tn
constexpr int R2W = TM_X + 4, R2H = TM_Y + 4, R2N = R2W * R2H;  // tile + 2-point halo
constexpr int R1W = TM_X + 2, R1H = TM_Y + 2, R1N = R1W * R1H;  // tile + 1-point halo
// zwi, ax, ay, tmask (3 levels each) and az (2) on R2; betup, betdo (2) on R1; the
// stage-a trend (3) on the tile
constexpr int FF_WORK = 14 * R2N + 4 * R1N + 3 * TM_TILE;
constexpr int FF_SMEM = (FF_NS * FF_NIN * FF_PL + FF_WORK) * 4 + 128;

template <class T>
__global__ void __launch_bounds__(TM_X * TM_Y, 2)
    k_fct_fused_tma(Dom<T> d, FctArgs<T> a, const __grid_constant__ PlaneMaps<FF_NIN> maps, int* err, int max_polls) {
  static_assert(sizeof(T) == 4, "the TMA kernel is the FP32 form");
  extern __shared__ unsigned char ff_smem[];
  __shared__ alignas(8) unsigned long long bar[FF_NS];
  __shared__ int s_abort;
  T* const sm = reinterpret_cast<T*>(ff_smem + ((128u - (smem_u32(ff_smem) & 127u)) & 127u));
  T* const ring = sm;  // [FF_NS][FF_NIN][FF_PL]
  T* const zwis = sm + FF_NS * FF_NIN * FF_PL;
  T* const axs = zwis + 3 * R2N;
  T* const ays = axs + 3 * R2N;
  T* const tms = ays + 3 * R2N;
  T* const azs = tms + 3 * R2N;
  T* const bus = azs + 2 * R2N;
  T* const bds = bus + 2 * R1N;
  T* const tas = bds + 2 * R1N;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TM_X + tx;
  const int jpi = d.jpi, jpj = d.jpj, jpk = d.jpk, n2 = (int)d.n2, n3 = (int)d.n3;
  const int m = (int)blockIdx.z;
  const int i0 = (int)blockIdx.x * TM_X, j0 = (int)blockIdx.y * TM_Y;
  if (tid == 0) {
    s_abort = *(volatile int*)err != 0;
    for (int s = 0; s < FF_NS; ++s) mbar_init(&bar[s], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (s_abort) return;
  auto interior = [&](int i, int j) { return i >= 2 && i <= jpi - 1 && j >= 2 && j <= jpj - 1; };
  auto inside = [&](int i, int j) { return i >= 1 && i <= jpi && j >= 1 && j <= jpj; };
  // ---- per-thread points. Stage a: R2 points tid and tid + 256
  constexpr int NA = (R2N + TM_X * TM_Y - 1) / (TM_X * TM_Y);
  int a_r[NA], a_b[NA], a_tile[NA];
  bool a_in[NA], a_ok[NA];
  ColInfo a_ci[NA];
  T a_e2u[NA], a_e2uw[NA], a_e1v[NA], a_e1vs[NA], a_e1e2t[NA], a_r1[NA];
#pragma unroll
  for (int s = 0; s < NA; ++s) {
    const int r = tid + s * TM_X * TM_Y;
    const int rx = r % R2W, ry = r / R2W;
    const int i = i0 - 2 + rx + 1, j = j0 - 2 + ry + 1;
    a_r[s] = r;
    a_ok[s] = r < R2N;
    a_b[s] = (ry + 1) * FF_BW + rx + 2;
    a_tile[s] = (rx >= 2 && rx < 2 + TM_X && ry >= 2 && ry < 2 + TM_Y) ? (ry - 2) * TM_X + (rx - 2) : -1;
    a_in[s] = a_ok[s] && interior(i, j);
    const bool ins = a_ok[s] && inside(i, j);
    const int ij = ins ? (i - 1) + (j - 1) * jpi : 0;
    a_ci[s] = ins ? d.ci[ij] : ColInfo{};
    a_e2u[s] = a_in[s] ? d.e2u[ij] : T(0);
    a_e2uw[s] = a_in[s] ? d.e2u[ij - 1] : T(0);
    a_e1v[s] = a_in[s] ? d.e1v[ij] : T(0);
    a_e1vs[s] = a_in[s] ? d.e1v[ij - jpi] : T(0);
    a_e1e2t[s] = a_in[s] ? d.e1e2t[ij] : T(0);
    a_r1[s] = a_in[s] ? d.r1_e1e2t[ij] : T(0);
  }
  // stage b: R1 points tid and tid + 256
  constexpr int NB = (R1N + TM_X * TM_Y - 1) / (TM_X * TM_Y);
  int b_r[NB], b_r2[NB], b_b[NB];
  bool b_in[NB], b_ok[NB];
  T b_e1e2t[NB];
#pragma unroll
  for (int s = 0; s < NB; ++s) {
    const int r = tid + s * TM_X * TM_Y;
    const int rx = r % R1W, ry = r / R1W;
    const int i = i0 - 1 + rx + 1, j = j0 - 1 + ry + 1;
    b_r[s] = r;
    b_ok[s] = r < R1N;
    b_r2[s] = (ry + 1) * R2W + rx + 1;
    b_b[s] = (ry + 2) * FF_BW + rx + 3;
    b_in[s] = b_ok[s] && interior(i, j);
    b_e1e2t[s] = b_in[s] ? d.e1e2t[(i - 1) + (j - 1) * jpi] : T(0);
  }
  // stage c: the tile point
  const int ci_ = i0 + tx + 1, cj_ = j0 + ty + 1;
  const bool c_valid = inside(ci_, cj_), c_in = interior(ci_, cj_);
  const int c_ij = c_valid ? (ci_ - 1) + (cj_ - 1) * jpi : 0;
  const int c_r1 = (ty + 1) * R1W + tx + 1, c_r2 = (ty + 2) * R2W + tx + 2;
  const T c_r1e = c_in ? d.r1_e1e2t[c_ij] : T(0);
  const bool w_lim = ci_ - 1 >= 2, s_lim = cj_ - 1 >= 2;
  const bool iso = a.with_iso;
  const T zsign = a.iso.zsign;
  const T zrtrn = T(1.e-15);
  const T p2dt = a.p2dt;
  const T* e3u = d.e3u_n.p.p;
  const T* e3v = d.e3v_n.p.p;
  const T* e3tn = d.e3t_n.p.p;
  const T* e3tb = d.e3t_b.p.p;
  const T* e3ta = d.e3t_a.p.p;
  unsigned issued = 0;
  bool ok = true;
  for (int n = 0; n < a.kjpt && ok; ++n) {
    const unsigned gb = (unsigned)(n * jpk);  // ring plane of level 1 of this pass
    auto slot = [&](int lev) { return ring + ((gb + (unsigned)(lev - 1)) % FF_NS) * (FF_NIN * FF_PL); };
    auto issue = [&](int lev) {
      const unsigned g = gb + (unsigned)(lev - 1), s = g % FF_NS;
      issued = g + 1;
      mbar_expect_tx(&bar[s], FF_NIN * FF_PL_BYTES);
      T* dst = ring + s * (FF_NIN * FF_PL);
      const int zv = m * jpk + lev - 1, zt = (m * a.kjpt + n) * jpk + lev - 1;
      tma_load_3d(dst, &maps.m[0], i0 - 4, j0 - 3, zv, &bar[s]);
      tma_load_3d(dst + FF_PL, &maps.m[1], i0 - 4, j0 - 3, zv, &bar[s]);
      tma_load_3d(dst + 2 * FF_PL, &maps.m[2], i0 - 4, j0 - 3, zv, &bar[s]);
      tma_load_3d(dst + 3 * FF_PL, &maps.m[3], i0 - 4, j0 - 3, zt, &bar[s]);
      tma_load_3d(dst + 4 * FF_PL, &maps.m[4], i0 - 4, j0 - 3, zt, &bar[s]);
    };
    auto wait_level = [&](int lev) {
      const unsigned g = gb + (unsigned)(lev - 1);
      return mbar_wait(&bar[g % FF_NS], (g / FF_NS) & 1, max_polls);
    };
    __syncthreads();  // the previous pass is done with every slot
    // the window of step 1 is levels -1 .. 4: levels 1 .. FF_NS - 2 now, then step t
    // issues level t + FF_NS - 2 into the slot level t - 2 leaves
    if (tid == 0)
      for (int lev = 1; lev <= FF_NS - 2 && lev <= jpk; ++lev) issue(lev);
    T* ta = a.pta + (long)(m * a.kjpt + n) * n3 + c_ij;
    const T* fu = iso ? a.iso.zftu + (long)(m * a.kjpt + n) * n3 + c_ij : nullptr;
    const T* fv = iso ? a.iso.zftv + (long)(m * a.kjpt + n) * n3 + c_ij : nullptr;
    const T* fw = iso ? a.iso.ztfw + (long)(m * a.kjpt + n) * n3 + c_ij : nullptr;
    if (c_valid && !c_in)  // edge columns: the trend is 0 at every level
      for (int k = 1; k <= jpk; ++k) ta[(k - 1) * n2] = T(0);
    T azt = T(0);                                        // limited flux through the top face (level 1: az = 0)
    T fwt = (iso && c_in) ? __ldg(fw) : T(0);            // iso-neutral vertical flux of that face
    ok = wait_level(1) && ok;
    for (int t = 1; t <= jpk + 2; ++t) {
      const int kc = t - 2;  // level of stage c in this step
      T fu0 = T(0), fuw = T(0), fv0 = T(0), fvs = T(0), fwb = T(0);
      if (iso && c_in && kc >= 1 && kc <= jpk - 1) {  // issued early: in flight during stages a and b
        const int q = (kc - 1) * n2;
        fu0 = __ldg(fu + q); fuw = __ldg(fu + q - 1); fv0 = __ldg(fv + q); fvs = __ldg(fv + q - jpi);
        fwb = __ldg(fw + q + n2);
      }
      // ---- stage a at level t (traadv_fct.F90:119-280)
      if (t <= jpk) {
        if (t + 1 <= jpk) ok = wait_level(t + 1) && ok;
        const T* P0 = slot(t);
        const T* Pm = t >= 2 ? slot(t - 1) : P0;
        const T* Pp = t + 1 <= jpk ? slot(t + 1) : P0;
        const int k = t;
        const T e3uk = __ldg(e3u + k - 1), e3vk = __ldg(e3v + k - 1);
        const T e3n = __ldg(e3tn + k - 1), e3b = __ldg(e3tb + k - 1), e3a = __ldg(e3ta + k - 1);
#pragma unroll
        for (int s = 0; s < NA; ++s) {
          if (!a_ok[s]) continue;
          const int r = a_r[s], b = a_b[s];
          const T tk = t_in<T>(a_ci[s], k);
          T zwi_v = T(0), ax_v = T(0), ay_v = T(0), az_v = T(0), ta_v = T(0);
          if (a_in[s] && k < jpk) {
            const T tkm = t_in<T>(a_ci[s], k - 1), tkp = t_in<T>(a_ci[s], k + 1);
            const T* un = P0;
            const T* vn = P0 + FF_PL;
            const T* tb = P0 + 3 * FF_PL;
            const T* tn = P0 + 4 * FF_PL;
            const T ue = a_e2u[s] * e3uk * un[b];
            const T uw = a_e2uw[s] * e3uk * un[b - 1];
            const T vn_ = a_e1v[s] * e3vk * vn[b];
            const T vs = a_e1vs[s] * e3vk * vn[b - FF_BW];
            const T wt = a_e1e2t[s] * P0[2 * FF_PL + b];
            const T wb = (k + 1 <= jpk - 1) ? a_e1e2t[s] * Pp[2 * FF_PL + b] : T(0);
            const T tm = tk, wk = k == 1 ? tk : tkm * tk, wk1 = tk * tkp;
            const T tb0 = tb[b];
            const T zwx_e = ups(ue, tb0, tb[b + 1]), zwx_w = ups(uw, tb[b - 1], tb0);
            const T zwy_n = ups(vn_, tb0, tb[b + FF_BW]), zwy_s = ups(vs, tb[b - FF_BW], tb0);
            const T zwz_t = (k == 1) ? (a.linssh ? wt * tb0 : T(0)) : ups(wt, tb0, Pm[3 * FF_PL + b]) * wk;
            const T zwz_b = (k + 1 <= jpk - 1) ? ups(wb, Pp[3 * FF_PL + b], tb0) * wk1 : T(0);
            const T ztra = -(zwx_e - zwx_w + zwy_n - zwy_s + zwz_t - zwz_b) * a_r1[s];
            ta_v = T(0) + ztra / e3n * tm;
            zwi_v = (e3b * tb0 + p2dt * ztra) / e3a * tm;
            const T tn0 = tn[b];
            ax_v = T(0.5) * ue * (tn0 + tn[b + 1]) - zwx_e;
            ay_v = T(0.5) * vn_ * (tn0 + tn[b + FF_BW]) - zwy_n;
            az_v = k >= 2 ? (wt * T(0.5) * (tn0 + Pm[4 * FF_PL + b]) - zwz_t) * wk : T(0);
          }
          zwis[(k % 3) * R2N + r] = zwi_v;
          axs[(k % 3) * R2N + r] = ax_v;
          ays[(k % 3) * R2N + r] = ay_v;
          tms[(k % 3) * R2N + r] = tk;
          azs[(k % 2) * R2N + r] = az_v;
          if (a_tile[s] >= 0) tas[(k % 3) * TM_TILE + a_tile[s]] = ta_v;
        }
      }
      __syncthreads();
      // ---- stage b at level t-1 (traadv_fct.F90:361-400)
      const int kb = t - 1;
      if (kb >= 1 && kb <= jpk) {
        const T* Q0 = slot(kb) + 3 * FF_PL;
        const T* Qm = kb >= 2 ? slot(kb - 1) + 3 * FF_PL : Q0;
        const T* Qp = kb + 1 <= jpk ? slot(kb + 1) + 3 * FF_PL : Q0;
        const T zbt0 = __ldg(e3tn + kb - 1);
        const T* z0 = zwis + (kb % 3) * R2N;
        const T* zm = zwis + ((kb + 2) % 3) * R2N;
        const T* zp = zwis + ((kb + 1) % 3) * R2N;
        const T* m0 = tms + (kb % 3) * R2N;
        const T* mm = tms + ((kb + 2) % 3) * R2N;
        const T* mp = tms + ((kb + 1) % 3) * R2N;
        const T* x0 = axs + (kb % 3) * R2N;
        const T* y0 = ays + (kb % 3) * R2N;
        const T* a0 = azs + (kb % 2) * R2N;
        const T* ap = azs + ((kb + 1) % 2) * R2N;
#pragma unroll
        for (int s = 0; s < NB; ++s) {
          if (!b_ok[s]) continue;
          T bu = T(0), bd = T(0);
          if (b_in[s] && kb < jpk) {
            const int r2 = b_r2[s], b = b_b[s];
            const T zbt = b_e1e2t[s] * zbt0 / p2dt;
            T up0, dn0, upm, dnm, upp, dnp, u2, d2;
            bupdo(Q0[b], z0[r2], m0[r2], up0, dn0);
            if (kb > 1) bupdo(Qm[b], zm[r2], mm[r2], upm, dnm);
            else { upm = up0; dnm = dn0; }
            bupdo(Qp[b], zp[r2], mp[r2], upp, dnp);
            // the reference's order: centre, west, east, south, north, above, below
            T up = up0, dn = dn0;
            bupdo(Q0[b - 1], z0[r2 - 1], m0[r2 - 1], u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
            bupdo(Q0[b + 1], z0[r2 + 1], m0[r2 + 1], u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
            bupdo(Q0[b - FF_BW], z0[r2 - R2W], m0[r2 - R2W], u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
            bupdo(Q0[b + FF_BW], z0[r2 + R2W], m0[r2 + R2W], u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
            up = vmax(up, upm); dn = vmin(dn, dnm);
            up = vmax(up, upp); dn = vmin(dn, dnp);
            const T axw = x0[r2 - 1], ax0 = x0[r2], ays_ = y0[r2 - R2W], ay0 = y0[r2];
            const T az0 = a0[r2], azb = ap[r2];
            const T zpos = pos_part(axw) - neg_part(ax0) + pos_part(ays_) - neg_part(ay0) + pos_part(azb) - neg_part(az0);
            const T zneg = pos_part(ax0) - neg_part(axw) + pos_part(ay0) - neg_part(ays_) + pos_part(az0) - neg_part(azb);
            const T zw = z0[r2];
            bu = (up - zw) / (zpos + zrtrn) * zbt;
            bd = (zw - dn) / (zneg + zrtrn) * zbt;
          }
          bus[(kb % 2) * R1N + b_r[s]] = bu;
          bds[(kb % 2) * R1N + b_r[s]] = bd;
        }
      }
      // every thread is done with level t-2's inputs: its slot takes level t+4
      if (!__syncthreads_and(ok)) {
        ok = false;
        break;
      }
      if (tid == 0 && t + FF_NS - 2 <= jpk) issue(t + FF_NS - 2);
      // ---- stage c at level t-2 (traadv_fct.F90:404-426, :288-297; traldf_iso.F90:278-284, :359-366)
      if (kc >= 1 && kc <= jpk - 1 && c_in) {
        const int k = kc;
        const T e3n = __ldg(e3tn + k - 1);
        const T* b0 = bus + (k % 2) * R1N;
        const T* d0 = bds + (k % 2) * R1N;
        const T bu0 = b0[c_r1], bd0 = d0[c_r1];
        const T bup = bus[((k + 1) % 2) * R1N + c_r1], bdp = bds[((k + 1) % 2) * R1N + c_r1];
        const T azp = azs[((k + 1) % 2) * R2N + c_r2];
        const T* x0 = axs + (k % 3) * R2N;
        const T* y0 = ays + (k % 3) * R2N;
        const T ax0 = x0[c_r2], axw = x0[c_r2 - 1], ay0 = y0[c_r2], ays_ = y0[c_r2 - R2W];
        const T bue = b0[c_r1 + 1], bde = d0[c_r1 + 1], buw = b0[c_r1 - 1], bdw = d0[c_r1 - 1];
        const T bun = b0[c_r1 + R1W], bdn = d0[c_r1 + R1W], bus_ = b0[c_r1 - R1W], bds_ = d0[c_r1 - R1W];
        const T ta0 = tas[(k % 3) * TM_TILE + tid];
        const T axl = limit(ax0, bd0, bue, bu0, bde);
        const T axlw = w_lim ? limit(axw, bdw, bu0, buw, bd0) : T(0);
        const T ayl = limit(ay0, bd0, bun, bu0, bdn);
        const T ayls = s_lim ? limit(ays_, bds_, bu0, bus_, bd0) : T(0);
        const T azl_b = limit(azp, bdp, bu0, bup, bd0);
        T tav = ta0 - (axl - axlw + ayl - ayls + azt - azl_b) * c_r1e / e3n;
        if (iso) {
          tav = tav + zsign * (fu0 - fuw + fv0 - fvs) * c_r1e / e3n;
          tav = tav + zsign * (fwt - fwb) * c_r1e / e3n;
          fwt = fwb;
        }
        ta[(k - 1) * n2] = tav;
        azt = azl_b;
      }
      if (kc == jpk && c_in) ta[(jpk - 1) * n2] = T(0);  // level jpk: no trend
      __syncthreads();  // stage c is done with the slots the next step's stage a rewrites
    }
  }
  if (!ok) {
    if (tid == 0) {
      atomicExch(err, TM_ERR);
      for (unsigned s = 0; s < FF_NS; ++s) {
        if (issued <= s) continue;
        const unsigned last = s + FF_NS * ((issued - 1 - s) / FF_NS);
        mbar_wait(&bar[s], (last / FF_NS) & 1, TM_DRAIN_POLLS);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// FCT stages a and b of k_fct_a_hot / k_fct_b_hot with every per-level plane staged by
// TMA (box {TM_W, TM_H}: the 32 x 8 tile with a one-point halo) in a ring of TM_NS
// levels; the values of the level above a chunk's first level come from global
// memory, as in the specialised kernels. Same arithmetic in the same order.
constexpr int FA_NF = 7;   // un, vn, wn, tb(2), tn(2)
constexpr int FB_NF = 10;  // tb, zwi, ax, ay, az (x2)
constexpr int FA_SMEM = TM_NS * FA_NF * TM_PLANE * 4 + 128;
constexpr int FB_SMEM = TM_NS * FB_NF * TM_PLANE * 4 + 128;

// shared parts of the two kernels: block geometry, ring set-up, abort check
struct TmaBlock {
  int tx, ty, tid, m, k0, k1, i0, j0, i, j, ij;
  bool valid, icol;
};
template <class T>
__device__ __forceinline__ TmaBlock tma_block(const Dom<T>& d) {
  TmaBlock b;
  b.tx = threadIdx.x; b.ty = threadIdx.y; b.tid = b.ty * TM_X + b.tx;
  const int nch = (d.jpk + KCH - 1) / KCH;
  b.m = (int)blockIdx.z / nch;
  const int ch = (int)blockIdx.z - b.m * nch;
  b.k0 = ch * KCH + 1;
  b.k1 = b.k0 + KCH - 1 < d.jpk ? b.k0 + KCH - 1 : d.jpk;
  b.i0 = (int)blockIdx.x * TM_X; b.j0 = (int)blockIdx.y * TM_Y;
  b.i = b.i0 + b.tx + 1; b.j = b.j0 + b.ty + 1;
  b.valid = b.i <= d.jpi && b.j <= d.jpj;
  b.icol = b.i >= 2 && b.i <= d.jpi - 1 && b.j >= 2 && b.j <= d.jpj - 1;
  b.ij = b.valid ? (b.i - 1) + (b.j - 1) * d.jpi : 0;
  return b;
}

template <class T>
__global__ void __launch_bounds__(TM_X * TM_Y, 3)
    k_fct_a_tma(Dom<T> d, FctArgs<T> a, const __grid_constant__ PlaneMaps<FA_NF> maps, int* err, int max_polls) {
  static_assert(sizeof(T) == 4, "the TMA kernel is the FP32 form");
  extern __shared__ unsigned char fa_smem[];
  __shared__ alignas(8) unsigned long long bar[TM_NS];
  __shared__ int s_abort;
  const PlaneRing<T, FA_NF> ring{
      reinterpret_cast<T*>(fa_smem + ((128u - (smem_u32(fa_smem) & 127u)) & 127u)), bar};
  const TmaBlock c = tma_block(d);
  const int jpi = d.jpi, jpk = d.jpk, n2 = (int)d.n2, n3 = (int)d.n3, ij = c.ij;
  if (c.tid == 0) {
    s_abort = *(volatile int*)err != 0;
    for (int s = 0; s < TM_NS; ++s) mbar_init(&bar[s], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (s_abort) return;
  const long mb = (long)c.m * a.kjpt * d.n3 + ij;
  T* zwi = a.zwi + mb;
  T* ax = a.ax + mb;
  T* ay = a.ay + mb;
  T* az = a.az + mb;
  T* ta = a.pta + mb;
  if (c.valid && !c.icol)  // edge columns: every level 0
    for (int k = c.k0; k <= c.k1; ++k)
      for (int n = 0; n < a.kjpt; ++n) {
        const int q = (k - 1) * n2 + n * n3;
        zwi[q] = T(0); ax[q] = T(0); ay[q] = T(0); az[q] = T(0); ta[q] = T(0);
      }
  const ColInfo ci = c.icol ? d.ci[ij] : ColInfo{};
  const T e2u0 = c.icol ? d.e2u[ij] : T(0), e2uw = c.icol ? d.e2u[ij - 1] : T(0);
  const T e1v0 = c.icol ? d.e1v[ij] : T(0), e1vs = c.icol ? d.e1v[ij - jpi] : T(0);
  const T e1e2t = c.icol ? d.e1e2t[ij] : T(0), r1_e1e2t = c.icol ? d.r1_e1e2t[ij] : T(0);
  const T* e3u = d.e3u_n.p.p;
  const T* e3v = d.e3v_n.p.p;
  const T* e3tn = d.e3t_n.p.p;
  const T* e3tb = d.e3t_b.p.p;
  const T* e3ta = d.e3t_a.p.p;
  const T* tbg = a.ptb.p + mb;
  const T* tng = a.ptn.p + mb;
  const T p2dt = a.p2dt;
  const int k0 = c.k0, o = (c.ty + 1) * TM_W + c.tx + 4;
  const int np = (c.k1 + 1 < jpk ? c.k1 + 1 : jpk) - k0 + 1;  // planes k0 .. min(k1+1, jpk)
  auto issue = [&](int p) {
    const int zv = c.m * jpk + (k0 - 1 + p), zt = c.m * a.kjpt * jpk + (k0 - 1 + p);
    ring.issue((unsigned)p, maps, FA_NF, c.i0 - 4, c.j0 - 1, [&](int f) {
      return f < 3 ? zv : zt + ((f - 3) & 1) * jpk;  // tb0 tb1 tn0 tn1 -> tracer (f-3) & 1
    });
  };
  if (c.tid == 0)
    for (int p = 0; p < TM_NS && p < np; ++p) issue(p);
  unsigned issued = (unsigned)(np < TM_NS ? np : TM_NS);
  // carried from level k-1: tb(k-1), tn(k-1), the bottom upstream flux of k-1
  T tbc[2] = {}, tnc[2] = {}, zwzb[2] = {};
  T tkm = t_in<T>(ci, k0 - 1), tk = t_in<T>(ci, k0), tkp = t_in<T>(ci, k0 + 1);
  T wt = T(0);
  bool ok = ring.wait(0, max_polls);
  int q = (k0 - 1) * n2;
  for (int k = k0; k <= c.k1; ++k, q += n2) {
    const int p = k - k0;
    if (k == jpk) {  // level jpk: no work, edge values
      if (c.icol)
        for (int nn = 0; nn < a.kjpt; ++nn) {
          const int qq = q + nn * n3;
          zwi[qq] = T(0); ax[qq] = T(0); ay[qq] = T(0); az[qq] = T(0); ta[qq] = T(0);
        }
      break;
    }
    ok = ring.wait((unsigned)p + 1, max_polls) && ok;
    if (c.icol) {
      auto L = [&](int f) { return ring.plane((unsigned)p, f); };
      auto L1 = [&](int f) { return ring.plane((unsigned)p + 1, f); };
      const bool first = k == k0;
      const T e3uk = __ldg(e3u + k - 1), e3vk = __ldg(e3v + k - 1);
      const T ue = e2u0 * e3uk * L(0)[o];
      const T uw = e2uw * e3uk * L(0)[o - 1];
      const T vn_ = e1v0 * e3vk * L(1)[o];
      const T vs = e1vs * e3vk * L(1)[o - TM_W];
      if (first) wt = e1e2t * L(2)[o];
      const T wb = (k + 1 <= jpk - 1) ? e1e2t * L1(2)[o] : T(0);
      const T e3n = __ldg(e3tn + k - 1), e3b = __ldg(e3tb + k - 1), e3a = __ldg(e3ta + k - 1);
      const T tm = tk, wk = k == 1 ? tk : tkm * tk, wk1 = tk * tkp;
#pragma unroll
      for (int nn = 0; nn < 2; ++nn) {
        if (nn >= a.kjpt) break;
        const T* TB = L(3 + nn);
        const T* TN = L(5 + nn);
        const int on = nn * n3;
        const T tb0 = TB[o];
        if (first && k > 1) {  // the carried values of level k-1
          tbc[nn] = __ldg(tbg + on + q - n2);
          tnc[nn] = __ldg(tng + on + q - n2);
          zwzb[nn] = ups(wt, tb0, tbc[nn]) * wk;
        }
        const T zwx_e = ups(ue, tb0, TB[o + 1]), zwx_w = ups(uw, TB[o - 1], tb0);
        const T zwy_n = ups(vn_, tb0, TB[o + TM_W]), zwy_s = ups(vs, TB[o - TM_W], tb0);
        // upstream vertical fluxes at the top (k) and bottom (k+1) faces (:137-156)
        const T zwz_t = (k == 1) ? (a.linssh ? wt * tb0 : T(0)) : zwzb[nn];
        const T zwz_b = (k + 1 <= jpk - 1) ? ups(wb, L1(3 + nn)[o], tb0) * wk1 : T(0);
        const T ztra = -(zwx_e - zwx_w + zwy_n - zwy_s + zwz_t - zwz_b) * r1_e1e2t;
        ta[on + q] = T(0) + ztra / e3n * tm;
        zwi[on + q] = (e3b * tb0 + p2dt * ztra) / e3a * tm;
        // 2nd-order antidiffusive fluxes (:180-190, :255-263)
        const T tn0 = TN[o], tne = TN[o + 1], tnn = TN[o + TM_W];
        ax[on + q] = T(0.5) * ue * (tn0 + tne) - zwx_e;
        ay[on + q] = T(0.5) * vn_ * (tn0 + tnn) - zwy_n;
        az[on + q] = k >= 2 ? (wt * T(0.5) * (tn0 + tnc[nn]) - zwz_t) * wk : T(0);
        tbc[nn] = tb0;
        tnc[nn] = tn0;
        zwzb[nn] = zwz_b;
      }
      wt = wb;
    }
    tkm = tk; tk = tkp; tkp = t_in<T>(ci, k + 2);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (c.tid == 0 && p + TM_NS < np) {
      issue(p + TM_NS);
      issued = (unsigned)(p + TM_NS + 1);
    }
  }
  if (!ok) {
    if (c.tid == 0) {
      atomicExch(err, TM_ERR);
      ring.drain(issued, TM_DRAIN_POLLS);
    }
    __syncthreads();
  }
}

template <class T>
__global__ void __launch_bounds__(TM_X * TM_Y, 3)
    k_fct_b_tma(Dom<T> d, FctArgs<T> a, const __grid_constant__ PlaneMaps<FB_NF> maps, int* err, int max_polls) {
  static_assert(sizeof(T) == 4, "the TMA kernel is the FP32 form");
  extern __shared__ unsigned char fb_smem[];
  __shared__ alignas(8) unsigned long long bar[TM_NS];
  __shared__ int s_abort;
  const PlaneRing<T, FB_NF> ring{
      reinterpret_cast<T*>(fb_smem + ((128u - (smem_u32(fb_smem) & 127u)) & 127u)), bar};
  const TmaBlock c = tma_block(d);
  const int jpi = d.jpi, jpk = d.jpk, n2 = (int)d.n2, n3 = (int)d.n3, ij = c.ij;
  if (c.tid == 0) {
    s_abort = *(volatile int*)err != 0;
    for (int s = 0; s < TM_NS; ++s) mbar_init(&bar[s], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (s_abort) return;
  const long mb = (long)c.m * a.kjpt * d.n3 + ij;
  T* bu = a.betup + mb;
  T* bd = a.betdo + mb;
  if (c.valid && !c.icol)
    for (int k = c.k0; k <= c.k1; ++k)
      for (int n = 0; n < a.kjpt; ++n) {
        const int q = (k - 1) * n2 + n * n3;
        bu[q] = T(0);
        bd[q] = T(0);
      }
  const T zrtrn = T(1.e-15);
  ColInfo ci{}, ciw{}, cie{}, cis{}, cin{};
  if (c.icol) { ci = d.ci[ij]; ciw = d.ci[ij - 1]; cie = d.ci[ij + 1]; cis = d.ci[ij - jpi]; cin = d.ci[ij + jpi]; }
  const T e1e2t = c.icol ? d.e1e2t[ij] : T(0);
  const T* e3tn = d.e3t_n.p.p;
  const T* tbg = a.ptb.p + mb;
  const T* zwig = a.zwi + mb;
  const T* azg = a.az + mb;
  const int k0 = c.k0, o = (c.ty + 1) * TM_W + c.tx + 4;
  const int np = (c.k1 + 1 < jpk ? c.k1 + 1 : jpk) - k0 + 1;
  auto issue = [&](int p) {
    const int zt = c.m * a.kjpt * jpk + (k0 - 1 + p);
    ring.issue((unsigned)p, maps, FB_NF, c.i0 - 4, c.j0 - 1, [&](int f) { return zt + (f & 1) * jpk; });
  };
  if (c.tid == 0)
    for (int p = 0; p < TM_NS && p < np; ++p) issue(p);
  unsigned issued = (unsigned)(np < TM_NS ? np : TM_NS);
  // carried: masked extrema of the column at level k-1 and k, az(k), zwi(k)
  T upm[2] = {}, dnm[2] = {}, up0[2] = {}, dn0[2] = {}, azk[2] = {}, zwik[2] = {};
  T tkm = t_in<T>(ci, k0 - 1), tk = t_in<T>(ci, k0), tkp = t_in<T>(ci, k0 + 1);
  bool ok = ring.wait(0, max_polls);
  int q = (k0 - 1) * n2;
  for (int k = k0; k <= c.k1; ++k, q += n2) {
    const int p = k - k0;
    if (k == jpk) {
      if (c.icol)
        for (int nn = 0; nn < a.kjpt; ++nn) {
          bu[q + nn * n3] = T(0);
          bd[q + nn * n3] = T(0);
        }
      break;
    }
    ok = ring.wait((unsigned)p + 1, max_polls) && ok;
    if (c.icol) {
      auto L = [&](int f) { return ring.plane((unsigned)p, f); };
      auto L1 = [&](int f) { return ring.plane((unsigned)p + 1, f); };
      const bool first = k == k0;
      const T zbt = e1e2t * __ldg(e3tn + k - 1) / a.p2dt;
      const T tw = t_in<T>(ciw, k), te = t_in<T>(cie, k), ts = t_in<T>(cis, k), tn = t_in<T>(cin, k);
#pragma unroll
      for (int nn = 0; nn < 2; ++nn) {
        if (nn >= a.kjpt) break;
        // planes of tracer nn: tb 0/1, zwi 2/3, ax 4/5, ay 6/7, az 8/9
        const T* TB = L(nn);
        const T* ZW = L(2 + nn);
        const T* AX = L(4 + nn);
        const T* AY = L(6 + nn);
        const int on = nn * n3;
        if (first) {  // extrema of the column at levels k and k-1, az(k)
          zwik[nn] = ZW[o];
          bupdo(TB[o], zwik[nn], tk, up0[nn], dn0[nn]);
          if (k > 1) bupdo(__ldg(tbg + on + q - n2), __ldg(zwig + on + q - n2), tkm, upm[nn], dnm[nn]);
          else { upm[nn] = up0[nn]; dnm[nn] = dn0[nn]; }
          azk[nn] = L(8 + nn)[o];
        }
        const T zwp = L1(2 + nn)[o];
        T upp, dnp;  // level k+1 of the column
        bupdo(L1(nn)[o], zwp, tkp, upp, dnp);
        // the reference's order: centre, west, east, south, north, above, below
        T up = up0[nn], dn = dn0[nn], u2, d2;
        bupdo(TB[o - 1], ZW[o - 1], tw, u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        bupdo(TB[o + 1], ZW[o + 1], te, u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        bupdo(TB[o - TM_W], ZW[o - TM_W], ts, u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        bupdo(TB[o + TM_W], ZW[o + TM_W], tn, u2, d2); up = vmax(up, u2); dn = vmin(dn, d2);
        up = vmax(up, upm[nn]); dn = vmin(dn, dnm[nn]);
        up = vmax(up, upp); dn = vmin(dn, dnp);
        const T axw = AX[o - 1], ax0 = AX[o], ays = AY[o - TM_W], ay0 = AY[o];
        const T az0 = azk[nn], azb = L1(8 + nn)[o];
        const T zpos = pos_part(axw) - neg_part(ax0) + pos_part(ays) - neg_part(ay0) + pos_part(azb) - neg_part(az0);
        const T zneg = pos_part(ax0) - neg_part(axw) + pos_part(ay0) - neg_part(ays) + pos_part(az0) - neg_part(azb);
        const T zw = zwik[nn];
        bu[on + q] = (up - zw) / (zpos + zrtrn) * zbt;
        bd[on + q] = (zw - dn) / (zneg + zrtrn) * zbt;
        upm[nn] = up0[nn]; dnm[nn] = dn0[nn];
        up0[nn] = upp; dn0[nn] = dnp;
        azk[nn] = azb;
        zwik[nn] = zwp;
      }
      (void)azg;
    }
    tkm = tk; tk = tkp; tkp = t_in<T>(ci, k + 2);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (c.tid == 0 && p + TM_NS < np) {
      issue(p + TM_NS);
      issued = (unsigned)(p + TM_NS + 1);
    }
  }
  if (!ok) {
    if (c.tid == 0) {
      atomicExch(err, TM_ERR);
      ring.drain(issued, TM_DRAIN_POLLS);
    }
    __syncthreads();
  }
}

}  // namespace nemo
