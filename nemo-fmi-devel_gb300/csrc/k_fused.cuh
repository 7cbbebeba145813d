// k_fused.cuh -- the tracer part of one timestep in one kernel: FCT advection
// (upstream fluxes, monotone guess, antidiffusive fluxes, Zalesak limiter, final
// trend; traadv.F90:110-114 + traadv_fct.F90:119-297 + nonosc :330-428) and the
// rotated iso-neutral diffusion (traldf_iso.F90:144-366, kpass = 1) for T and S,
// with no intermediate field in HBM.
//
// A block owns a TX x TY tile of interior columns and marches down k. Each level's
// inputs are staged in shared memory planes with a 3-point halo (the limiter of a
// face needs the limiter coefficients of both neighbours, which need the monotone
// guess of their neighbours, which needs upstream fluxes one point further out),
// and every halo quantity is recomputed locally instead of being exchanged through
// HBM. The k-dependencies form a 3-level pipeline: at step L the kernel loads level
// L, computes the upstream vertical flux at the top of L, the monotone guess and
// antidiffusive fluxes of level L-1, the limiter coefficients of level L-2, and
// finishes level L-3 (limited fluxes, final advective trend, iso-neutral trend).
// Planes are rings indexed by level modulo their depth.
//
// Scope: mixed precision (FP32 bulk), kn_fct_h = kn_fct_v = 2, linear free surface,
// z-coordinate (1-D e3), no partial steps, constant masked eddy diffusivity,
// kjpt = 2 -- the configuration of the GYRE step. Other configurations use the
// per-routine kernels of k_tra.cuh. HBM traffic per cell: read tb, tn (T,S),
// un, vn, wn and the four slopes; write ta (T,S), ah_wslp2 and akz.
#pragma once
#include "k_tra.cuh"

namespace nemo {

constexpr int FTX = 32, FTY = 8, FNT = FTX * FTY;

template <int R>
struct Box {
  static constexpr int W = FTX + 2 * R, H = FTY + 2 * R, N = W * H;
  __device__ static __forceinline__ int ix(int a, int b) { return (a + R) + (b + R) * W; }
};
using B3 = Box<3>;
using B2 = Box<2>;
using B1 = Box<1>;

template <class T>
struct FusedArgs {
  T p2dt;
  const T *un, *vn, *wn;   // velocities; transports are formed on the fly
  const T *tb, *tn;        // (jpi,jpj,jpk,2)
  T* ta;                   // out: advective + iso-neutral trend (tsa starts from 0)
  const T *uslp, *vslp, *wslpi, *wslpj;
  T *ah_wslp2, *akz;
  T aht_c;                 // ahtu = aht_c * umask (ldftra.F90:292-372)
  int lap, msc, linssh;
  T z2dt, z1_2dt;
};

// shared-memory layout (floats), per tracer then common
struct FusedSmem {
  static constexpr int TB = 5, TN = 2, ZWZ = 2, ZWI = 3, AX = 3, AZ = 3, BET = 3, TAU = 3;
  static constexpr int per_tracer = TB * B3::N + TN * B2::N + ZWZ * B2::N + ZWI * B2::N + 2 * AX * B2::N +
                                    AZ * B1::N + 2 * BET * B1::N + TAU * FNT;
  static constexpr int common = 2 * B3::N + 2 * B2::N + 4 * B3::N;  // u, v | w(2) | e2u, e1v, r1_e1e2t, e1e2t
  static constexpr int floats = 2 * per_tracer + common;
  static constexpr size_t bytes = floats * sizeof(float) + B3::N * sizeof(ColInfo);
};

template <class T>
__global__ void __launch_bounds__(FNT, 1) k_tra_fused(Dom<T> d, FusedArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  // ---- carve planes
  T *tbP[2], *tnP[2], *zwzP[2], *zwiP[2], *axP[2], *ayP[2], *azP[2], *buP[2], *bdP[2], *tauP[2];
  {
    T* p = sm;
    for (int n = 0; n < 2; ++n) {
      tbP[n] = p; p += FusedSmem::TB * B3::N;
      tnP[n] = p; p += FusedSmem::TN * B2::N;
      zwzP[n] = p; p += FusedSmem::ZWZ * B2::N;
      zwiP[n] = p; p += FusedSmem::ZWI * B2::N;
      axP[n] = p; p += FusedSmem::AX * B2::N;
      ayP[n] = p; p += FusedSmem::AX * B2::N;
      azP[n] = p; p += FusedSmem::AZ * B1::N;
      buP[n] = p; p += FusedSmem::BET * B1::N;
      bdP[n] = p; p += FusedSmem::BET * B1::N;
      tauP[n] = p; p += FusedSmem::TAU * FNT;
    }
  }
  T* uP = sm + 2 * FusedSmem::per_tracer;
  T* vP = uP + B3::N;
  T* wP = vP + B3::N;             // 2 slots of B2
  T* e2uP = wP + 2 * B2::N;       // B3
  T* e1vP = e2uP + B3::N;         // B3
  T* r1eP = e1vP + B3::N;         // B3: r1_e1e2t
  T* eeP = r1eP + B3::N;          // B3: e1e2t
  ColInfo* ciP = reinterpret_cast<ColInfo*>(sm + FusedSmem::floats);

  const int jpi = d.jpi, jpj = d.jpj, jpk = d.jpk;
  const long n2 = d.n2, n3 = d.n3;
  const int m = blockIdx.z;
  const int i0 = 2 + blockIdx.x * FTX, j0 = 2 + blockIdx.y * FTY;  // first interior column of the tile
  const int tid = threadIdx.x;
  const long mv = (long)m * n3;
  const long mt0 = (long)m * 2 * n3;
  const T zbig = Big<T>::v, zrtrn = T(1.e-15), r1_2 = T(0.5);

  auto gidx = [&](int a, int b, long& ij) -> bool {
    const int gi = i0 + a, gj = j0 + b;
    if (gi < 1 || gi > jpi || gj < 1 || gj > jpj) return false;
    ij = (long)(gi - 1) + (long)(gj - 1) * jpi;
    return true;
  };
  auto interior = [&](int a, int b) -> bool {
    const int gi = i0 + a, gj = j0 + b;
    return gi >= 2 && gi <= jpi - 1 && gj >= 2 && gj <= jpj - 1;
  };
  auto e3t = [&](int k) -> T { return d.e3t_n.p[k - 1]; };

  // ---- static planes: ColInfo and 2-D metrics on the 3-halo box
  for (int t = tid; t < B3::N; t += FNT) {
    const int aa = t % B3::W - 3, bb = t / B3::W - 3;
    long ij;
    if (gidx(aa, bb, ij)) {
      ciP[t] = d.ci[ij];
      e2uP[t] = d.e2u[ij] ;
      e1vP[t] = d.e1v[ij];
      r1eP[t] = d.r1_e1e2t[ij];
      eeP[t] = d.e1e2t[ij];
    } else {
      ciP[t] = ColInfo{1, 0, 1, 0, 1, 0, 1, 1};
      e2uP[t] = T(0); e1vP[t] = T(0); r1eP[t] = T(0); eeP[t] = T(0);
    }
  }

  // per-thread output column
  const int ta_ = tid % FTX, tb_ = tid / FTX;
  long ijT;
  const bool colT = gidx(ta_, tb_, ijT) && interior(ta_, tb_);
  T ztfw_t[2] = {T(0), T(0)};

  for (int L = 1; L <= jpk + 3; ++L) {
    __syncthreads();
    // ================= phase 0: load level L (tb, w), level L-1 (tn, u, v)
    {
      const int sTB = L % FusedSmem::TB, sTN = (L - 1 + 2) % FusedSmem::TN, sW = L % 2;
      for (int t = tid; t < B3::N; t += FNT) {
        const int aa = t % B3::W - 3, bb = t / B3::W - 3;
        long ij;
        const bool in = gidx(aa, bb, ij);
        for (int n = 0; n < 2; ++n) {
          T v = T(0);
          if (in && L <= jpk) v = a.tb[mt0 + n * n3 + (long)(L - 1) * n2 + ij];
          tbP[n][sTB * B3::N + t] = v;
        }
        T u = T(0), vv = T(0);
        if (in && L - 1 >= 1 && L - 1 <= jpk) {
          const long q = mv + (long)(L - 2) * n2 + ij;
          u = a.un[q];
          vv = a.vn[q];
        }
        uP[t] = u;
        vP[t] = vv;
      }
      for (int t = tid; t < B2::N; t += FNT) {
        const int aa = t % B2::W - 2, bb = t / B2::W - 2;
        long ij;
        const bool in = gidx(aa, bb, ij);
        for (int n = 0; n < 2; ++n) {
          T v = T(0);
          if (in && L - 1 >= 1 && L - 1 <= jpk) v = a.tn[mt0 + n * n3 + (long)(L - 2) * n2 + ij];
          tnP[n][sTN * B2::N + t] = v;
        }
        T w = T(0);
        if (in && L <= jpk) w = a.wn[mv + (long)(L - 1) * n2 + ij];
        wP[sW * B2::N + t] = w;
      }
    }
    __syncthreads();
    // ================= phase 1: upstream vertical flux at the top face of level L (on the 2-halo box)
    if (L <= jpk) {
      const int sZ = L % 2, sTB = L % 5, sTBm = (L + 4) % 5, sW = L % 2;
      for (int t = tid; t < B2::N; t += FNT) {
        const int aa = t % B2::W - 2, bb = t / B2::W - 2;
        const int t3 = B3::ix(aa, bb);
        const T w = eeP[t3] * wP[sW * B2::N + t];  // zwn = e1e2t * wn
        for (int n = 0; n < 2; ++n) {
          T z;
          if (L == 1) {
            z = a.linssh ? w * tbP[n][sTB * B3::N + t3] : T(0);
          } else if (L <= jpk - 1) {
            z = ups(w, tbP[n][sTB * B3::N + t3], tbP[n][sTBm * B3::N + t3]) * wmsk<T>(ciP[t3], L);
          } else {
            z = T(0);
          }
          zwzP[n][sZ * B2::N + t] = z;
        }
      }
    }
    __syncthreads();
    // ================= phase 2/3: monotone guess (2-halo), antidiffusive fluxes of level K1 = L-1
    const int K1 = L - 1;
    if (K1 >= 1 && K1 <= jpk) {
      const int sTB = K1 % 5, sZ0 = K1 % 2, sZ1 = L % 2, sI = K1 % 3, sA = K1 % 3, sTN = K1 % 2, sTNm = (K1 + 1) % 2;
      const int sW = K1 % 2;
      const T e3tn = K1 <= jpk - 1 ? e3t(K1) : T(1);
      const T e3tb = K1 <= jpk - 1 ? d.e3t_b.p[K1 - 1] : T(1);
      const T e3ta = K1 <= jpk - 1 ? d.e3t_a.p[K1 - 1] : T(1);
      const T e3u = K1 <= jpk - 1 ? d.e3u_n.p[K1 - 1] : T(0);
      const T e3v = K1 <= jpk - 1 ? d.e3v_n.p[K1 - 1] : T(0);
      for (int t = tid; t < B2::N; t += FNT) {
        const int aa = t % B2::W - 2, bb = t / B2::W - 2;
        const int c3 = B3::ix(aa, bb), w3 = B3::ix(aa - 1, bb), e3_ = B3::ix(aa + 1, bb);
        const int s3 = B3::ix(aa, bb - 1), n3_ = B3::ix(aa, bb + 1);
        const bool inner = interior(aa, bb) && K1 <= jpk - 1;
        // transports at the faces of this point (traadv.F90:110-114)
        const T ue = e2uP[c3] * e3u * uP[c3], uw = e2uP[w3] * e3u * uP[w3];
        const T vn_ = e1vP[c3] * e3v * vP[c3], vs = e1vP[s3] * e3v * vP[s3];
        const ColInfo ci = ciP[c3];
        for (int n = 0; n < 2; ++n) {
          const T* tb = tbP[n] + sTB * B3::N;
          const T tb0 = tb[c3];
          const T zwx_e = ups(ue, tb0, tb[e3_]), zwx_w = ups(uw, tb[w3], tb0);
          const T zwy_n = ups(vn_, tb0, tb[n3_]), zwy_s = ups(vs, tb[s3], tb0);
          T zwi = T(0);
          if (inner) {
            const T ztra = -(zwx_e - zwx_w + zwy_n - zwy_s + zwzP[n][sZ0 * B2::N + t] - zwzP[n][sZ1 * B2::N + t]) *
                           r1eP[c3];
            const T tm = tmsk<T>(ci, K1);
            zwi = (e3tb * tb0 + a.p2dt * ztra) / e3ta * tm;
            if (aa >= 0 && aa < FTX && bb >= 0 && bb < FTY)
              tauP[n][(K1 % 3) * FNT + aa + bb * FTX] = ztra / e3tn * tm;
          }
          zwiP[n][sI * B2::N + t] = zwi;
          // antidiffusive fluxes on the faces of this point (2nd order, :182-190, lbc :280)
          T axv = T(0), ayv = T(0);
          if (inner) {
            const T* tn = tnP[n] + sTN * B2::N;
            const int c2 = t, e2 = B2::ix(aa + 1, bb), n2_ = B2::ix(aa, bb + 1);
            const bool eok = aa + 1 <= FTX + 1, nok = bb + 1 <= FTY + 1;
            // faces at the edge of the 2-halo box feed no limiter in this tile
            if (eok) axv = T(0.5) * ue * (tn[c2] + tn[e2]) - zwx_e;
            if (nok) ayv = T(0.5) * vn_ * (tn[c2] + tn[n2_]) - zwy_n;
          }
          axP[n][sA * B2::N + t] = axv;
          ayP[n][sA * B2::N + t] = ayv;
        }
        // vertical antidiffusive flux at the top face of level K1 (on the 1-halo box)
        if (aa >= -1 && aa <= FTX && bb >= -1 && bb <= FTY) {
          const int t1 = B1::ix(aa, bb);
          for (int n = 0; n < 2; ++n) {
            T azv = T(0);
            if (inner && K1 >= 2) {
              const T w = eeP[c3] * wP[sW * B2::N + t];
              const T* tn0 = tnP[n] + sTN * B2::N;
              const T* tnm = tnP[n] + sTNm * B2::N;
              azv = (w * T(0.5) * (tn0[t] + tnm[t]) - zwzP[n][sZ0 * B2::N + t]) * wmsk<T>(ci, K1);
            }
            azP[n][(K1 % 3) * B1::N + t1] = azv;
          }
        }
      }
    }
    __syncthreads();
    // ================= phase 4: limiter coefficients of level K2 = L-2 (1-halo box)
    const int K2 = L - 2;
    if (K2 >= 1 && K2 <= jpk) {
      const int s0 = K2 % 5, sm1 = ((K2 - 1 > 1 ? K2 - 1 : 1)) % 5, sp1 = (K2 + 1) % 5;
      const int zi0 = K2 % 3, zim = ((K2 - 1 > 1 ? K2 - 1 : 1)) % 3, zip = (K2 + 1) % 3;
      const int km1 = K2 - 1 > 1 ? K2 - 1 : 1;
      const T e3tn = K2 <= jpk - 1 ? e3t(K2) : T(1);
      for (int t = tid; t < B1::N; t += FNT) {
        const int aa = t % B1::W - 1, bb = t / B1::W - 1;
        T bu = T(0), bd = T(0);
        if (interior(aa, bb) && K2 <= jpk - 1) {
          const int c3 = B3::ix(aa, bb);
          const int c2 = B2::ix(aa, bb), w2 = B2::ix(aa - 1, bb), e2 = B2::ix(aa + 1, bb);
          const int s2 = B2::ix(aa, bb - 1), n2_ = B2::ix(aa, bb + 1);
          const int w3 = B3::ix(aa - 1, bb), e3_ = B3::ix(aa + 1, bb), s3 = B3::ix(aa, bb - 1), n3_ = B3::ix(aa, bb + 1);
          const T zbt = eeP[c3] * e3tn / a.p2dt;
          for (int n = 0; n < 2; ++n) {
            const T* tb0 = tbP[n] + s0 * B3::N;
            const T* zw0 = zwiP[n] + zi0 * B2::N;
            T up, dn, u2, d2;
            auto bud = [&](T pb, T pa, T tm, T& uo, T& dno) {
              uo = fmx(pb * tm - zbig * (T(1) - tm), pa * tm - zbig * (T(1) - tm));
              dno = fmn(pb * tm + zbig * (T(1) - tm), pa * tm + zbig * (T(1) - tm));
            };
            bud(tb0[c3], zw0[c2], tmsk<T>(ciP[c3], K2), up, dn);
            bud(tb0[w3], zw0[w2], tmsk<T>(ciP[w3], K2), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
            bud(tb0[e3_], zw0[e2], tmsk<T>(ciP[e3_], K2), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
            bud(tb0[s3], zw0[s2], tmsk<T>(ciP[s3], K2), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
            bud(tb0[n3_], zw0[n2_], tmsk<T>(ciP[n3_], K2), u2, d2); up = fmx(up, u2); dn = fmn(dn, d2);
            bud(tbP[n][sm1 * B3::N + c3], zwiP[n][zim * B2::N + c2], tmsk<T>(ciP[c3], km1), u2, d2);
            up = fmx(up, u2); dn = fmn(dn, d2);
            bud(tbP[n][sp1 * B3::N + c3], zwiP[n][zip * B2::N + c2], tmsk<T>(ciP[c3], K2 + 1), u2, d2);
            up = fmx(up, u2); dn = fmn(dn, d2);
            const T* ax = axP[n] + (K2 % 3) * B2::N;
            const T* ay = ayP[n] + (K2 % 3) * B2::N;
            const T axw = ax[w2], ax0 = ax[c2], ays = ay[s2], ay0 = ay[c2];
            const T az0 = azP[n][(K2 % 3) * B1::N + t], azb = azP[n][((K2 + 1) % 3) * B1::N + t];
            const T zpos = fmx(T(0), axw) - fmn(T(0), ax0) + fmx(T(0), ays) - fmn(T(0), ay0) + fmx(T(0), azb) - fmn(T(0), az0);
            const T zneg = fmx(T(0), ax0) - fmn(T(0), axw) + fmx(T(0), ay0) - fmn(T(0), ays) + fmx(T(0), az0) - fmn(T(0), azb);
            const T paft = zw0[c2];
            bu = (up - paft) / (zpos + zrtrn) * zbt;
            bd = (paft - dn) / (zneg + zrtrn) * zbt;
            buP[n][(K2 % 3) * B1::N + t] = bu;
            bdP[n][(K2 % 3) * B1::N + t] = bd;
          }
        } else {
          for (int n = 0; n < 2; ++n) {
            buP[n][(K2 % 3) * B1::N + t] = T(0);
            bdP[n][(K2 % 3) * B1::N + t] = T(0);
          }
        }
      }
    }
    __syncthreads();
    // ================= phase 5: finish level K = L-3 on the tile's own columns
    const int K = L - 3;
    if (K >= 1 && K <= jpk - 1 && colT) {
      const int c1 = B1::ix(ta_, tb_), w1 = B1::ix(ta_ - 1, tb_), e1 = B1::ix(ta_ + 1, tb_);
      const int s1 = B1::ix(ta_, tb_ - 1), n1 = B1::ix(ta_, tb_ + 1);
      const int c2 = B2::ix(ta_, tb_), w2 = B2::ix(ta_ - 1, tb_), s2 = B2::ix(ta_, tb_ - 1);
      const bool w_lim = i0 + ta_ - 1 >= 2, s_lim = j0 + tb_ - 1 >= 2;
      const T r1e = r1eP[B3::ix(ta_, tb_)];
      const T e3tn = e3t(K);
      const int sk = K % 3, skp = (K + 1) % 3, skm = (K + 2) % 3;  // K, K+1, K-1 in a ring of 3
      // iso-neutral coefficients one level ahead (traldf_iso.F90:146-202)
      const ColInfo ci = ciP[B3::ix(ta_, tb_)];
      const ColInfo ciw = ciP[B3::ix(ta_ - 1, tb_)], cis = ciP[B3::ix(ta_, tb_ - 1)];
      const ColInfo cie = ciP[B3::ix(ta_ + 1, tb_)], cin = ciP[B3::ix(ta_, tb_ + 1)];
      auto ahu = [&](const ColInfo& c, int k) -> T { return k < jpk ? a.aht_c * umsk<T>(c, k) : T(0); };
      auto ahv = [&](const ColInfo& c, int k) -> T { return k < jpk ? a.aht_c * vmsk<T>(c, k) : T(0); };
      T ahw_next = T(0), akz_next = T(0);
      const long q3 = mv + (long)K * n2 + ijT;  // level K+1
      if (K + 1 <= jpk - 1) {
        const int k = K + 1;
        const T wm = wmsk<T>(ci, k);
        const T zmsku = wm / fmx(umsk<T>(ci, k - 1) + umsk<T>(ciw, k) + umsk<T>(ciw, k - 1) + umsk<T>(ci, k), T(1));
        const T zmskv = wm / fmx(vmsk<T>(ci, k - 1) + vmsk<T>(cis, k) + vmsk<T>(cis, k - 1) + vmsk<T>(ci, k), T(1));
        const T zahu_w = (ahu(ci, k - 1) + ahu(ciw, k) + ahu(ciw, k - 1) + ahu(ci, k)) * zmsku;
        const T zahv_w = (ahv(ci, k - 1) + ahv(cis, k) + ahv(cis, k - 1) + ahv(ci, k)) * zmskv;
        const T wi = a.wslpi[q3], wj = a.wslpj[q3];
        ahw_next = zahu_w * wi * wi + zahv_w * wj * wj;
        akz_next = ahw_next;
        if (a.msc) {
          const long ij = ijT;
          const T e1u0 = d.e1u[ij], e1uw = d.e1u[ij - 1], e2v0 = d.e2v[ij], e2vs = d.e2v[ij - jpi];
          T akzv = T(0.25) * ((ahu(ci, k) + ahu(ci, k - 1)) / (e1u0 * e1u0) + (ahu(ciw, k) + ahu(ciw, k - 1)) / (e1uw * e1uw) +
                              (ahv(ci, k) + ahv(ci, k - 1)) / (e2v0 * e2v0) + (ahv(cis, k) + ahv(cis, k - 1)) / (e2vs * e2vs));
          const T e3w = d.e3w_n.p[k - 1];
          const T ze3w_2 = e3w * e3w;
          const T zcoef0 = a.z2dt * (akzv + ahw_next / ze3w_2);
          akz_next = fmx(zcoef0 - T(0.5), T(0)) * ze3w_2 * a.z1_2dt;
        }
        a.ah_wslp2[q3] = ahw_next;
        a.akz[q3] = akz_next;
      }
      const T e2u0 = e2uP[B3::ix(ta_, tb_)], e2uw = e2uP[B3::ix(ta_ - 1, tb_)];
      const T e1v0 = e1vP[B3::ix(ta_, tb_)], e1vs = e1vP[B3::ix(ta_, tb_ - 1)];
      const long ij = ijT;
      const T e2_e1u0 = d.e2_e1u[ij], e2_e1uw = d.e2_e1u[ij - 1], e1_e2v0 = d.e1_e2v[ij], e1_e2vs = d.e1_e2v[ij - jpi];
      const T e3uK = d.e3u_n.p[K - 1], e3vK = d.e3v_n.p[K - 1];
      const T e2t = d.e2t[ij], e1t = d.e1t[ij], e1e2t = d.e1e2t[ij];
      const long qK = mv + (long)(K - 1) * n2 + ij;
      for (int n = 0; n < 2; ++n) {
        // limited fluxes and final advective trend (:404-426, :288-297)
        const T* ax = axP[n] + sk * B2::N;
        const T* ay = ayP[n] + sk * B2::N;
        const T* bu = buP[n] + sk * B1::N;
        const T* bd = bdP[n] + sk * B1::N;
        const T axl = limit(ax[c2], bd[c1], bu[e1], bu[c1], bd[e1]);
        const T axlw = w_lim ? limit(ax[w2], bd[w1], bu[c1], bu[w1], bd[c1]) : T(0);
        const T ayl = limit(ay[c2], bd[c1], bu[n1], bu[c1], bd[n1]);
        const T ayls = s_lim ? limit(ay[s2], bd[s1], bu[c1], bu[s1], bd[c1]) : T(0);
        const T azK = azP[n][sk * B1::N + c1];
        const T azl_t = K >= 2 ? limit(azK, bd[c1], buP[n][skm * B1::N + c1], bu[c1], bdP[n][skm * B1::N + c1]) : azK;
        const T azl_b = limit(azP[n][skp * B1::N + c1], bdP[n][skp * B1::N + c1], bu[c1], buP[n][skp * B1::N + c1], bd[c1]);
        T tav = tauP[n][sk * FNT + ta_ + tb_ * FTX];
        tav = tav - (axl - axlw + ayl - ayls + azl_t - azl_b) * r1e / e3tn;
        // iso-neutral horizontal fluxes (:247-284) from tb(K-1..K+1) on the 1-halo cross
        const T* tbm = tbP[n] + (((K - 1) % 5 + 5) % 5) * B3::N;
        const T* tb0 = tbP[n] + (K % 5) * B3::N;
        const T* tbp = tbP[n] + ((K + 1) % 5) * B3::N;
        auto dk1 = [&](int p3, const ColInfo& cp) -> T { return (tb0[p3] - tbp[p3]) * wmsk<T>(cp, K + 1); };
        auto dk0 = [&](int p3, const ColInfo& cp) -> T {
          if (K == 1) return dk1(p3, cp);
          return (tbm[p3] - tb0[p3]) * wmsk<T>(cp, K);
        };
        const int p0 = B3::ix(ta_, tb_), pw = B3::ix(ta_ - 1, tb_), pe = B3::ix(ta_ + 1, tb_);
        const int ps = B3::ix(ta_, tb_ - 1), pn = B3::ix(ta_, tb_ + 1);
        const int pnw = B3::ix(ta_ - 1, tb_ + 1), pse = B3::ix(ta_ + 1, tb_ - 1);
        (void)pnw; (void)pse;
        auto ftu = [&](int p, int pe_, const ColInfo& cp, const ColInfo& cpe, T e2_e1u, T e2u, T uslp) -> T {
          const T pah = ahu(cp, K);
          const T zabe1 = pah * e2_e1u * e3uK;
          const T zmsku = T(1) / fmx(wmsk<T>(cpe, K) + wmsk<T>(cp, K + 1) + wmsk<T>(cpe, K + 1) + wmsk<T>(cp, K), T(1));
          const T zcof1 = -pah * e2u * uslp * zmsku;
          const T zd = (tb0[pe_] - tb0[p]) * umsk<T>(cp, K);
          return (zabe1 * zd + zcof1 * (dk0(pe_, cpe) + dk1(p, cp) + dk1(pe_, cpe) + dk0(p, cp))) * umsk<T>(cp, K);
        };
        auto ftv = [&](int p, int pn_, const ColInfo& cp, const ColInfo& cpn, T e1_e2v, T e1v, T vslp) -> T {
          const T pah = ahv(cp, K);
          const T zabe2 = pah * e1_e2v * e3vK;
          const T zmskv = T(1) / fmx(wmsk<T>(cpn, K) + wmsk<T>(cp, K + 1) + wmsk<T>(cpn, K + 1) + wmsk<T>(cp, K), T(1));
          const T zcof2 = -pah * e1v * vslp * zmskv;
          const T zd = (tb0[pn_] - tb0[p]) * vmsk<T>(cp, K);
          return (zabe2 * zd + zcof2 * (dk0(pn_, cpn) + dk1(p, cp) + dk1(pn_, cpn) + dk0(p, cp))) * vmsk<T>(cp, K);
        };
        const T zftu0 = ftu(p0, pe, ci, cie, e2_e1u0, e2u0, a.uslp[qK]);
        const T zftuw = ftu(pw, p0, ciw, ci, e2_e1uw, e2uw, a.uslp[qK - 1]);
        const T zftv0 = ftv(p0, pn, ci, cin, e1_e2v0, e1v0, a.vslp[qK]);
        const T zftvs = ftv(ps, p0, cis, ci, e1_e2vs, e1vs, a.vslp[qK - jpi]);
        tav = tav + (zftu0 - zftuw + zftv0 - zftvs) * r1e / e3tn;
        // iso-neutral vertical flux at the bottom face of level K (:298-332)
        T ztfw_b = T(0);
        if (K + 1 <= jpk - 1) {
          const int k = K + 1;
          const T wm = wmsk<T>(ci, k);
          const T zmsku = wm / fmx(umsk<T>(ci, k - 1) + umsk<T>(ciw, k) + umsk<T>(ciw, k - 1) + umsk<T>(ci, k), T(1));
          const T zmskv = wm / fmx(vmsk<T>(ci, k - 1) + vmsk<T>(cis, k) + vmsk<T>(cis, k - 1) + vmsk<T>(ci, k), T(1));
          const T zahu_w = (ahu(ci, k - 1) + ahu(ciw, k) + ahu(ciw, k - 1) + ahu(ci, k)) * zmsku;
          const T zahv_w = (ahv(ci, k - 1) + ahv(cis, k) + ahv(cis, k - 1) + ahv(ci, k)) * zmskv;
          const T zcoef3 = -zahu_w * e2t * zmsku * a.wslpi[q3];
          const T zcoef4 = -zahv_w * e1t * zmskv * a.wslpj[q3];
          // zdit at (i,K), (i-1,K+1), (i-1,K), (i,K+1)
          const T sdi = (tb0[pe] - tb0[p0]) * umsk<T>(ci, K) + (tbp[p0] - tbp[pw]) * umsk<T>(ciw, k) +
                        (tb0[p0] - tb0[pw]) * umsk<T>(ciw, K) + (tbp[pe] - tbp[p0]) * umsk<T>(ci, k);
          const T sdj = (tb0[pn] - tb0[p0]) * vmsk<T>(ci, K) + (tbp[p0] - tbp[ps]) * vmsk<T>(cis, k) +
                        (tb0[p0] - tb0[ps]) * vmsk<T>(cis, K) + (tbp[pn] - tbp[p0]) * vmsk<T>(ci, k);
          T z = zcoef3 * sdi + zcoef4 * sdj;
          const T e3w = d.e3w_n.p[k - 1];
          if (a.lap) z = z + e1e2t / e3w * wm * (ahw_next - akz_next) * (tb0[p0] - tbp[p0]);
          else z = z + ahw_next * e1e2t * (tb0[p0] - tbp[p0]) / e3w * wm;
          ztfw_b = z;
        }
        tav = tav + (ztfw_t[n] - ztfw_b) * r1e / e3tn;
        ztfw_t[n] = ztfw_b;
        a.ta[mt0 + n * n3 + (long)(K - 1) * n2 + ijT] = tav;
      }
      if (K == jpk - 1)
        for (int n = 0; n < 2; ++n) a.ta[mt0 + n * n3 + (long)(jpk - 1) * n2 + ijT] = T(0);
    }
  }
}

}  // namespace nemo
