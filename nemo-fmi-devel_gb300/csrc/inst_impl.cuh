// inst_impl.cuh -- definitions of the launchers declared in launch.h; included by
// inst_fp64.cu and inst_fp32.cu, each of which instantiates one precision.
#pragma once
#include <cudaTypedefs.h>

#include <cstdint>

#include "launch.h"
#include "k_hot.cuh"
#include "k_tma.cuh"

namespace nemo {

constexpr int BX = 32, BY = 4;

// one thread per water column (recurrences along k); ty: block height
template <class T>
static dim3 col_grid(const Dom<T>& d, int ty = BY) {
  return dim3((d.jpi + BX - 1) / BX, (d.jpj + ty - 1) / ty, d.nmem);
}

// one thread per KCH-level chunk of a column: z = member * nchunk + chunk
template <class T>
static dim3 kc_grid(const Dom<T>& d, int ty = BY) {
  return dim3((d.jpi + BX - 1) / BX, (d.jpj + ty - 1) / ty, d.nmem * ((d.jpk + KCH - 1) / KCH));
}

// one thread per (i,j,k) point: z = member * jpk + (k - 1)
template <class T>
static dim3 pt_grid(const Dom<T>& d) {
  return dim3((d.jpi + BX - 1) / BX, (d.jpj + BY - 1) / BY, d.nmem * d.jpk);
}

template <class T>
cudaError_t launch_adv_trp(const Dom<T>& d, const T* un, const T* vn, const T* wn, T* zun, T* zvn, T* zwn,
                           cudaStream_t s) {
  k_adv_trp<T><<<pt_grid(d), dim3(BX, BY), 0, s>>>(d, un, vn, wn, zun, zvn, zwn);
  ktick(NEMO_K_ADV_TRP, s);
  return cudaGetLastError();
}

// cuTensorMapEncodeTiled from the driver, through the runtime (no libcuda link)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)p;
  }();
  return fn;
}

// Tensor map of nf 3-D fields of floats stored one after the other per member, as a
// 3-D tensor (jpi, jpj, jpk * nf * nmem), with a box of bx x by points of one level.
// False (no TMA) when the rows are not a multiple of 16 bytes (jpi % 4 != 0) or the
// base is not 16-byte aligned.
template <class T>
static bool field_tensor_map(const Dom<T>& d, const T* base, int nf, unsigned bx, unsigned by, CUtensorMap* map) {
  const auto fn = tensor_map_encoder();
  if (!fn || sizeof(T) != 4 || d.jpi % 4 != 0 || ((uintptr_t)base & 15) != 0) return false;
  cuuint64_t dims[3] = {(cuuint64_t)d.jpi, (cuuint64_t)d.jpj, (cuuint64_t)d.jpk * nf * d.nmem};
  cuuint64_t strides[2] = {(cuuint64_t)d.jpi * sizeof(T), (cuuint64_t)d.n2 * sizeof(T)};
  cuuint32_t box[3] = {bx, by, 1}, es[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)base, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <class T>
cudaError_t launch_fct(const Dom<T>& d, const FctArgs<T>& a, cudaStream_t s) {
  if (hot_fct_ok(d, a) && !a.lim) {  // the limiter is recorded by k_fct_c only
    if constexpr (sizeof(T) == 4) {
      if (a.tma && a.err && a.kjpt == 2) {  // planes staged by TMA
        if (a.fused) {  // the three stages in one kernel
          PlaneMaps<FF_NIN> maps;
          const bool ok = field_tensor_map(d, a.pun.p, 1, FF_BW, FF_BH, &maps.m[0]) &&
                          field_tensor_map(d, a.pvn.p, 1, FF_BW, FF_BH, &maps.m[1]) &&
                          field_tensor_map(d, a.pwn.p, 1, FF_BW, FF_BH, &maps.m[2]) &&
                          field_tensor_map(d, a.ptb.p, a.kjpt, FF_BW, FF_BH, &maps.m[3]) &&
                          field_tensor_map(d, a.ptn.p, a.kjpt, FF_BW, FF_BH, &maps.m[4]);
          if (ok) {
            static const cudaError_t attr =
                cudaFuncSetAttribute(k_fct_fused_tma<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, FF_SMEM);
            if (attr != cudaSuccess) return attr;
            const dim3 grid((d.jpi + TM_X - 1) / TM_X, (d.jpj + TM_Y - 1) / TM_Y, d.nmem);
            k_fct_fused_tma<T><<<grid, dim3(TM_X, TM_Y), FF_SMEM, s>>>(d, a, maps, a.err, a.polls);
            ktick(NEMO_K_FCT_FUSED, s);
            return cudaGetLastError();
          }
        } else {  // stages a and b with TMA-staged planes, then stage c
          PlaneMaps<FA_NF> ma;
          PlaneMaps<FB_NF> mb;
          bool ok = field_tensor_map(d, a.pun.p, 1, TM_W, TM_H, &ma.m[0]) &&
                    field_tensor_map(d, a.pvn.p, 1, TM_W, TM_H, &ma.m[1]) &&
                    field_tensor_map(d, a.pwn.p, 1, TM_W, TM_H, &ma.m[2]) &&
                    field_tensor_map(d, a.ptb.p, 2, TM_W, TM_H, &ma.m[3]) &&
                    field_tensor_map(d, a.ptn.p, 2, TM_W, TM_H, &ma.m[5]);
          ma.m[4] = ma.m[3];  // tb, tn: one map each, read at the two tracers' levels
          ma.m[6] = ma.m[5];
          const T* fb[5] = {a.ptb.p, a.zwi, a.ax, a.ay, a.az};
          for (int f = 0; f < 5 && ok; ++f) {
            ok = field_tensor_map(d, fb[f], 2, TM_W, TM_H, &mb.m[2 * f]);
            mb.m[2 * f + 1] = mb.m[2 * f];
          }
          if (ok) {
            static const cudaError_t attr_a =
                cudaFuncSetAttribute(k_fct_a_tma<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, FA_SMEM);
            static const cudaError_t attr_b =
                cudaFuncSetAttribute(k_fct_b_tma<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, FB_SMEM);
            if (attr_a != cudaSuccess) return attr_a;
            if (attr_b != cudaSuccess) return attr_b;
            const dim3 grid((d.jpi + TM_X - 1) / TM_X, (d.jpj + TM_Y - 1) / TM_Y, d.nmem * ((d.jpk + KCH - 1) / KCH));
            k_fct_a_tma<T><<<grid, dim3(TM_X, TM_Y), FA_SMEM, s>>>(d, a, ma, a.err, a.polls);
            ktick(NEMO_K_FCT_A_TMA, s);
            k_fct_b_tma<T><<<grid, dim3(TM_X, TM_Y), FB_SMEM, s>>>(d, a, mb, a.err, a.polls);
            ktick(NEMO_K_FCT_B_TMA, s);
            const int tc = kty(NEMO_K_FCT_C);
            k_fct_c_hot<T><<<kc_grid(d, tc), dim3(BX, tc), 0, s>>>(d, a);
            ktick(NEMO_K_FCT_C, s);
            return cudaGetLastError();
          }
        }
      }
    }
    const int ta = kty(NEMO_K_FCT_A), tb = kty(NEMO_K_FCT_B), tc = kty(NEMO_K_FCT_C);
    k_fct_a_hot<T><<<kc_grid(d, ta), dim3(BX, ta), 0, s>>>(d, a);
    ktick(NEMO_K_FCT_A, s);
    k_fct_b_hot<T><<<kc_grid(d, tb), dim3(BX, tb), 0, s>>>(d, a);
    ktick(NEMO_K_FCT_B, s);
    k_fct_c_hot<T><<<kc_grid(d, tc), dim3(BX, tc), 0, s>>>(d, a);
    ktick(NEMO_K_FCT_C, s);
    return cudaGetLastError();
  }
  if (a.kn_fct_v == 4) {
    k_interp4<T><<<col_grid(d), dim3(BX, BY), 0, s>>>(d, a.ptn, const_cast<T*>(a.ztw.p), a.kjpt);
    ktick(NEMO_K_INTERP4, s);
  }
  k_fct_a<T><<<kc_grid(d), dim3(BX, BY), 0, s>>>(d, a);
  ktick(NEMO_K_FCT_A, s);
  k_fct_b<T><<<kc_grid(d), dim3(BX, BY), 0, s>>>(d, a);
  ktick(NEMO_K_FCT_B, s);
  k_fct_c<T><<<kc_grid(d), dim3(BX, BY), 0, s>>>(d, a);
  ktick(NEMO_K_FCT_C, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_ldf_lap(const Dom<T>& d, const LdfArgs<T>& a, cudaStream_t s) {
  k_ldf_lap<T><<<pt_grid(d), dim3(BX, BY), 0, s>>>(d, a);
  ktick(NEMO_K_LDF_LAP, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_ldf_iso(const Dom<T>& d, const LdfArgs<T>& a, int copy_akz_edges, int msc_edges, cudaStream_t s) {
  launch_iso_flux<T>(d, a, s);
  k_iso_div<T><<<pt_grid(d), dim3(BX, BY), 0, s>>>(d, a);
  ktick(NEMO_K_ISO_DIV, s);
  return launch_iso_edges<T>(d, a, copy_akz_edges, msc_edges, s);
}

template <class T>
cudaError_t launch_iso_flux(const Dom<T>& d, const LdfArgs<T>& a, cudaStream_t s) {
  if (hot_iso_ok(d, a)) {
    if constexpr (sizeof(T) == 4) {
      IsoMaps maps;
      if (a.tma && a.err && field_tensor_map(d, a.ptb.p, a.kjpt, TM_W, TM_H, &maps.tb) &&
          field_tensor_map(d, a.uslp.p, 1, TM_X, TM_Y, &maps.uslp) &&
          field_tensor_map(d, a.vslp.p, 1, TM_X, TM_Y, &maps.vslp) &&
          field_tensor_map(d, a.wslpi.p, 1, TM_X, TM_Y, &maps.wslpi) &&
          field_tensor_map(d, a.wslpj.p, 1, TM_X, TM_Y, &maps.wslpj)) {
        const dim3 grid((d.jpi + TM_X - 1) / TM_X, (d.jpj + TM_Y - 1) / TM_Y, d.nmem * ((d.jpk + KCH - 1) / KCH));
        k_iso_flux_tma<T><<<grid, dim3(TM_X, TM_Y), 0, s>>>(d, a, maps, a.err, a.polls);
        ktick(NEMO_K_ISO_FLUX_TMA, s);
        return cudaGetLastError();
      }
    }
    const int ti = kty(NEMO_K_ISO_FLUX);
    k_iso_flux_hot<T><<<kc_grid(d, ti), dim3(BX, ti), 0, s>>>(d, a);
  } else {
    k_iso_flux<T><<<kc_grid(d), dim3(BX, BY), 0, s>>>(d, a);
  }
  ktick(NEMO_K_ISO_FLUX, s);
  return cudaGetLastError();
}

// the points of ah_wslp2 / akz the interior sweep does not write (edge columns,
// levels 1 and jpk; row and column 1 of the MSC correction)
template <class T>
cudaError_t launch_iso_edges(const Dom<T>& d, const LdfArgs<T>& a, int copy_akz_edges, int msc_edges, cudaStream_t s) {
  if (copy_akz_edges && !hot_iso_ok(d, a)) {  // the specialised flux kernel copies them itself
    k_iso_akz_copy_edges<T><<<col_grid(d), dim3(BX, BY), 0, s>>>(d, a);
    ktick(NEMO_K_ISO_AKZ_EDGES, s);
  }
  if (msc_edges) {
    k_iso_msc_edges<T><<<col_grid(d), dim3(BX, BY), 0, s>>>(d, a);
    ktick(NEMO_K_ISO_MSC_EDGES, s);
  }
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_zdf(const Dom<T>& d, const ZdfArgs<T>& a, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (d.jpk == 31) {  // the GYRE levels: columns staged in shared memory
      static bool attr = false;  // dynamic shared memory beyond 48 KB needs the opt-in
      constexpr int smem_max = 4 * 31 * BX * BY * sizeof(float);
      if (!attr) {
        cudaFuncSetAttribute(k_zdf_imp_async<31>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);
        attr = true;
      }
      const int tz = kty(NEMO_K_ZDF_IMP);
      const int smem = 4 * 31 * BX * tz * sizeof(float);
      k_zdf_imp_async<31><<<col_grid(d, tz), dim3(BX, tz), smem, s>>>(d, a);
      ktick(NEMO_K_ZDF_IMP, s);
      return cudaGetLastError();
    }
  }
  const int tz = kty(NEMO_K_ZDF_IMP);
  k_zdf_imp<T><<<col_grid(d, tz), dim3(BX, tz), 0, s>>>(d, a);
  ktick(NEMO_K_ZDF_IMP, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_clamp(T* x, long n, cudaStream_t s) {
  long nb = (n + 255) / 256;
  if (nb > 152L * 16) nb = 152L * 16;
  if (nb < 1) nb = 1;
  k_clamp_neg<T><<<(unsigned)nb, 256, 0, s>>>(x, n);
  ktick(NEMO_K_CLAMP, s);
  return cudaGetLastError();
}

// co-resident blocks per SM of the sub-step kernel, with or without the constant
// cache (dynamic shared memory beyond the 48 KB default needs the opt-in)
template <class T>
int spg_p2_blocks_per_sm(int cache, int vvl) {
  const size_t dyn = cache ? P2_CACHE_BYTES : 0;
  auto kern = vvl ? k_spg_p2<T, true> : k_spg_p2<T, false>;
  if (cache && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, 256, dyn) != cudaSuccess) return 0;
  return nb;
}

// co-resident blocks per SM of the specialised sub-step kernel (mixed form, linear
// free surface, ENE/MIX), with its constant cache
template <class T>
int spg_p2_ene_blocks_per_sm() {
  if constexpr (sizeof(T) != 4) {
    return 0;
  } else {
    if (cudaFuncSetAttribute(k_spg_p2_ene<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)P2H_CACHE_BYTES) != cudaSuccess)
      return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_spg_p2_ene<T>, 256, P2H_CACHE_BYTES) != cudaSuccess)
      return 0;
    return nb;
  }
}

template <class T>
cudaError_t launch_spg(const Dom<T>& d, const SpgArgs<T>& a, const GridBar& bar, int p2_blocks, cudaStream_t s) {
  if (a.vvl) {  // Coriolis factors from the now depths (:241-343)
    k_spg_cor<T><<<col_grid(d), dim3(BX, BY), 0, s>>>(d, a);
    ktick(NEMO_K_SPG_COR, s);
  }
  bool p1a_reg = false;
  if constexpr (sizeof(T) == 4) {
    if (d.jpk == 31) {  // the GYRE levels: columns in registers
      const int t1 = kty(NEMO_K_SPG_P1A);
      k_spg_p1a_reg<31><<<col_grid(d, t1), dim3(BX, t1), 0, s>>>(d, a);
      p1a_reg = true;
    }
  }
  if (!p1a_reg) {
    const int t1 = kty(NEMO_K_SPG_P1A);
    k_spg_p1a<T><<<col_grid(d, t1), dim3(BX, t1), 0, s>>>(d, a);
  }
  ktick(NEMO_K_SPG_P1A, s);
  const int t1b = kty(NEMO_K_SPG_P1B);
  k_spg_p1b<T><<<col_grid(d, t1b), dim3(BX, t1b), 0, s>>>(d, a);
  ktick(NEMO_K_SPG_P1B, s);
  {  // the barrier's arrival counter starts at 0 in every launch
    cudaError_t ez = cudaMemsetAsync(bar.count, 0, sizeof(unsigned int), s);
    if (ez != cudaSuccess) return ez;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p2_blocks);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = a.cache ? P2_CACHE_BYTES : 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e;
  if constexpr (sizeof(T) == 4) {
    if (a.hot) {
      cfg.dynamicSmemBytes = P2H_CACHE_BYTES;
      e = cudaLaunchKernelEx(&cfg, k_spg_p2_ene<T>, d, a, bar);
    } else {
      e = a.vvl ? cudaLaunchKernelEx(&cfg, k_spg_p2<T, true>, d, a, bar)
                : cudaLaunchKernelEx(&cfg, k_spg_p2<T, false>, d, a, bar);
    }
  } else {
    e = a.vvl ? cudaLaunchKernelEx(&cfg, k_spg_p2<T, true>, d, a, bar)
              : cudaLaunchKernelEx(&cfg, k_spg_p2<T, false>, d, a, bar);
  }
  if (e != cudaSuccess) return e;
  ktick(NEMO_K_SPG_P2, s);
  const int t3 = kty(NEMO_K_SPG_P3);
  k_spg_p3<T><<<dim3((d.jpi + BX - 1) / BX, (d.jpj + t3 - 1) / t3, d.nmem * ((d.jpk + KCH3 - 1) / KCH3)),
                 dim3(BX, t3), 0, s>>>(d, a);
  ktick(NEMO_K_SPG_P3, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_lbc(T* p, int jpi, int jpj, long nslab, int is_f, T pval, cudaStream_t s) {
  long per = 2L * jpi + 2L * jpj;
  unsigned gx = (unsigned)((per + 255) / 256);
  unsigned gy = (unsigned)(nslab < 65535 ? nslab : 65535);
  k_lbc_closed<T><<<dim3(gx, gy), 256, 0, s>>>(p, jpi, jpj, nslab, is_f, pval);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_globsum(const T* x, const double* tmask_i, long n2, int nk, int nmem, double* part, int nblk,
                           double* out, cudaStream_t s) {
  k_globsum_partial<T><<<dim3(nblk, nmem), 256, 0, s>>>(x, tmask_i, n2, nk, part);
  k_globsum_final<<<nmem, 256, 0, s>>>(part, nblk, out);
  return cudaGetLastError();
}

#define NEMO_INSTANTIATE(T)                                                                                   \
  template cudaError_t launch_adv_trp<T>(const Dom<T>&, const T*, const T*, const T*, T*, T*, T*, cudaStream_t); \
  template cudaError_t launch_fct<T>(const Dom<T>&, const FctArgs<T>&, cudaStream_t);                        \
  template cudaError_t launch_ldf_lap<T>(const Dom<T>&, const LdfArgs<T>&, cudaStream_t);                    \
  template cudaError_t launch_ldf_iso<T>(const Dom<T>&, const LdfArgs<T>&, int, int, cudaStream_t);          \
  template cudaError_t launch_zdf<T>(const Dom<T>&, const ZdfArgs<T>&, cudaStream_t);                        \
  template cudaError_t launch_iso_edges<T>(const Dom<T>&, const LdfArgs<T>&, int, int, cudaStream_t);        \
  template cudaError_t launch_iso_flux<T>(const Dom<T>&, const LdfArgs<T>&, cudaStream_t);                   \
  template cudaError_t launch_clamp<T>(T*, long, cudaStream_t);                                              \
  template cudaError_t launch_spg<T>(const Dom<T>&, const SpgArgs<T>&, const GridBar&, int, cudaStream_t);   \
  template int spg_p2_blocks_per_sm<T>(int, int);                                                                 \
  template int spg_p2_ene_blocks_per_sm<T>();                                                                 \
  template cudaError_t launch_lbc<T>(T*, int, int, long, int, T, cudaStream_t);                              \
  template cudaError_t launch_globsum<T>(const T*, const double*, long, int, int, double*, int, double*, cudaStream_t);

}  // namespace nemo
