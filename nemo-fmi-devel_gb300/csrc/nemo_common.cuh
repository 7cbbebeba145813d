// nemo_common.cuh -- device-side layout, masks and helpers shared by every kernel.
//
// Layout in HBM: every field keeps NEMO's Fortran order (jpi,jpj,jpk[,kjpt]) with i
// contiguous, so a warp of 32 consecutive i reads 32 consecutive elements. Ensemble
// members are outermost. Kernels map one thread to one (i,j) water column and march
// down k, so 2-D metrics and the per-column level bounds are loaded once per column.
//
// Masks are never read as 3-D arrays: a column's T, U and V masks are contiguous
// level ranges [lo,hi] (dommsk.F90:133-183 builds them from k_top/k_bot and closes
// the domain edges), stored as 8 bytes per column (ColInfo). wmask follows from the
// T range (dommsk.F90:189-194).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace nemo {

struct __align__(8) ColInfo {
  uint8_t tlo, thi, ulo, uhi, vlo, vhi, mbku, mbkv;
};

// A scale-factor field e3(i,j,k[,member]) = p[m*sm + (k-1)*sk + ij*s]. A horizontally
// uniform field (z-coordinate with full steps) is stored as a 1-D profile with
// s = 0, sk = 1, so no 3-D metric traffic is spent on it.
template <class T>
struct E3 {
  const T* p;
  long sk;
  long sm;
  int s;
  __device__ __forceinline__ T operator()(long ij, int k, int m) const {
    return p[m * sm + (long)(k - 1) * sk + ij * (long)s];
  }
};

template <class T>
struct Dom {
  int jpi, jpj, jpk, nmem;
  long n2, n3;  // points per member of a 2-D / 3-D field
  const T *e1t, *e2t, *e1u, *e2u, *e1v, *e2v;
  const T *r1_e1u, *r1_e2u, *r1_e1v, *r1_e2v;
  const T *e1e2t, *r1_e1e2t, *e2_e1u, *e1_e2v, *r1_e1e2u, *r1_e1e2v;
  const T *ht_0, *hu_0, *hv_0, *r1_hu_0, *r1_hv_0;
  const T *ssmask, *ssumask, *ssvmask;
  const T *ff_t, *zwz, *ftne, *ftnw, *ftse, *ftsw;
  const double* tmask_i;
  const ColInfo* ci;
  const uint8_t* mbkt;
  E3<T> e3t_b, e3t_n, e3t_a, e3u_n, e3v_n, e3w_n;
};

__device__ __forceinline__ bool in_range(int k, int lo, int hi) { return k >= lo && k <= hi; }

template <class T>
__device__ __forceinline__ T tmsk(const ColInfo& c, int k) { return in_range(k, c.tlo, c.thi) ? T(1) : T(0); }
template <class T>
__device__ __forceinline__ T umsk(const ColInfo& c, int k) { return in_range(k, c.ulo, c.uhi) ? T(1) : T(0); }
template <class T>
__device__ __forceinline__ T vmsk(const ColInfo& c, int k) { return in_range(k, c.vlo, c.vhi) ? T(1) : T(0); }
template <class T>
__device__ __forceinline__ T wmsk(const ColInfo& c, int k) {
  if (k == 1) return tmsk<T>(c, 1);
  return (in_range(k, c.tlo, c.thi) && in_range(k - 1, c.tlo, c.thi)) ? T(1) : T(0);
}

// SIGN(a,b) with key_nosignedzero (lib_fortran.F90:339-351): b >= 0 gives |a|.
template <class T>
__device__ __forceinline__ T sign_nsz(T a, T b) { return b >= T(0) ? fabs(a) : -fabs(a); }
template <class T>
__device__ __forceinline__ T fmx(T a, T b) { return a > b ? a : b; }
template <class T>
__device__ __forceinline__ T fmn(T a, T b) { return a < b ? a : b; }

// Land sentinel of nonosc (traadv_fct.F90:354). 1e40 overflows FP32; 1e30 keeps the
// same role (far beyond any tracer value) without overflow.
template <class T> struct Big;
template <> struct Big<double> { static constexpr double v = 1.e+40; };
template <> struct Big<float> { static constexpr float v = 1.e+30f; };

// Grid barrier for persistent kernels launched cooperatively (all blocks resident).
// Each wait is bounded: after max_spins polls the block records NEMO_ERR_TIMEOUT in
// *err and returns false; every block checks the flag after each barrier and leaves
// its loop, so the kernel always ends. gen is read before arriving (sense reversal
// by generation counter); the last block to arrive resets the count and bumps gen.
struct GridBar {
  unsigned int* count;
  unsigned int* gen;
  int* err;
  unsigned int nblocks;
  long long max_spins;
};

__device__ __forceinline__ bool grid_barrier(const GridBar& b) {
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
    volatile unsigned int* vgen = b.gen;
    volatile int* verr = b.err;
    unsigned int g = *vgen;
    __threadfence();
    unsigned int arrived = atomicAdd(b.count, 1u);
    if (arrived == b.nblocks - 1) {
      atomicExch(b.count, 0u);
      __threadfence();
      atomicAdd(b.gen, 1u);
    } else {
      long long s = 0;
      while (*vgen == g) {
        if (*verr != 0) break;
        if (++s > b.max_spins) {
          atomicExch(b.err, 5);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *((volatile int*)b.err) == 0;
}

}  // namespace nemo
