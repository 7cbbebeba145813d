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
        mbar_wait(&bar[s], (last / TM_NS) & 1, max_polls);
      }
    }
    __syncthreads();
  }
}

}  // namespace nemo
