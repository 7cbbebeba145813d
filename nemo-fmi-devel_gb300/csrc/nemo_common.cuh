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
#include <cstring>
#include <cuda_runtime.h>

namespace nemo {

struct __align__(8) ColInfo {
  uint8_t tlo, thi, ulo, uhi, vlo, vhi, mbku, mbkv;
};

// Loads through the read-only data path (ld.global.nc). The compiler may move them
// ahead of the kernel's stores, so they are used only for arrays that no thread
// writes while the kernel runs.
template <class T>
__device__ __forceinline__ T ldro(const T* p) { return __ldg(p); }
template <>
__device__ __forceinline__ ColInfo ldro<ColInfo>(const ColInfo* p) {
  const unsigned long long v = __ldg(reinterpret_cast<const unsigned long long*>(p));
  ColInfo c;
  memcpy(&c, &v, sizeof(c));
  return c;
}

// A device array read only through ldro.
template <class T>
struct RO {
  const T* p;
  __host__ __device__ RO(const T* q = nullptr) : p(q) {}
  __device__ __forceinline__ T operator[](long i) const { return ldro(p + i); }
  __host__ __device__ RO operator+(long o) const { return RO(p + o); }
  __host__ __device__ RO operator-(long o) const { return RO(p - o); }
  __host__ __device__ explicit operator bool() const { return p != nullptr; }
};

// A scale-factor field e3(i,j,k[,member]) = p[m*sm + (k-1)*sk + ij*s]. A horizontally
// uniform field (z-coordinate with full steps) is stored as a 1-D profile with
// s = 0, sk = 1, so no 3-D metric traffic is spent on it.
template <class T>
struct E3 {
  RO<T> p;
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
  RO<T> e1t, e2t, e1u, e2u, e1v, e2v;
  RO<T> r1_e1u, r1_e2u, r1_e1v, r1_e2v;
  RO<T> e1e2t, r1_e1e2t, e2_e1u, e1_e2v, r1_e1e2u, r1_e1e2v, e1e2u, e1e2v;
  RO<T> ht_0, hu_0, hv_0, r1_hu_0, r1_hv_0;
  RO<T> ssmask, ssumask, ssvmask;
  RO<T> ff_t, ff_f, zwz, ftne, ftnw, ftse, ftsw;
  RO<double> tmask_i;
  RO<ColInfo> ci;
  RO<uint8_t> mbkt;
  E3<T> e3t_b, e3t_n, e3t_a, e3u_n, e3v_n, e3w_n;
  E3<T> e3f_n;       // now e3 at f-points (the rest state unless NEMO_F_E3F_N is bound)
  RO<T> r1_e1e2f;    // 1 / (e1f e2f)
  // 1 / e3t_0 and 1 / e3w_0 per level (correctly rounded) where the rest-state scale
  // factor is a 1-D profile, else NULL: the divisors of the hot-path tracer kernels
  RO<T> r1_e3t, r1_e3w;
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
// Mask lookups of a kernel body compiled twice: W = true where the caller has
// checked that every mask the body reads is 1 (the wet interior, most points), so
// every multiplication by a mask folds away (x * 1 is exact); W = false reads the
// column's level ranges.
template <bool W, class T>
__device__ __forceinline__ T tmk(const ColInfo& c, int k) {
  if constexpr (W) return T(1); else return tmsk<T>(c, k);
}
template <bool W, class T>
__device__ __forceinline__ T umk(const ColInfo& c, int k) {
  if constexpr (W) return T(1); else return umsk<T>(c, k);
}
template <bool W, class T>
__device__ __forceinline__ T vmk(const ColInfo& c, int k) {
  if constexpr (W) return T(1); else return vmsk<T>(c, k);
}
template <bool W, class T>
__device__ __forceinline__ T wmk(const ColInfo& c, int k) {
  if constexpr (W) return T(1); else return wmsk<T>(c, k);
}
// the T (U, V) range of column c covers levels lo..hi
__device__ __forceinline__ bool t_wet(const ColInfo& c, int lo, int hi) { return c.tlo <= lo && hi <= c.thi; }
__device__ __forceinline__ bool u_wet(const ColInfo& c, int lo, int hi) { return c.ulo <= lo && hi <= c.uhi; }
__device__ __forceinline__ bool v_wet(const ColInfo& c, int lo, int hi) { return c.vlo <= lo && hi <= c.vhi; }

template <class T>
__device__ __forceinline__ T fmx(T a, T b) { return a > b ? a : b; }
template <class T>
__device__ __forceinline__ T fmn(T a, T b) { return a < b ? a : b; }

// 1 / MAX(n, 1) for a sum n of four 0/1 masks (n = 0..4), as the correctly rounded
// quotient the division gives, without dividing: 1, 1, 1/2, 1/3, 1/4.
template <class T> struct Third;
template <> struct Third<double> { static constexpr double v = 0x1.5555555555555p-2; };
template <> struct Third<float> { static constexpr float v = 0x1.555556p-2f; };
template <class T>
__device__ __forceinline__ T rcount(T n) {
  return n <= T(1) ? T(1) : (n == T(2) ? T(0.5) : (n == T(3) ? Third<T>::v : T(0.25)));
}
// rcount of the sum of four 0/1 masks; FP64 counts them on the integer pipe
template <class T>
__device__ __forceinline__ T rcount4(T a, T b, T c, T d) {
  if constexpr (sizeof(T) == 8) {
    const int n = (__double2hiint(a) != 0) + (__double2hiint(b) != 0) + (__double2hiint(c) != 0) +
                  (__double2hiint(d) != 0);
    return n <= 1 ? T(1) : (n == 2 ? T(0.5) : (n == 3 ? Third<T>::v : T(0.25)));
  } else {
    return rcount(a + b + c + d);
  }
}

// Land sentinel of nonosc (traadv_fct.F90:354). 1e40 overflows FP32; 1e30 keeps the
// same role (far beyond any tracer value) without overflow.
// value of the device error flag after a timed-out wait on a tensor copy (a timed-out
// grid barrier of the sub-step kernel writes NEMO_ERR_TIMEOUT)
constexpr int TM_ERR = 2;

template <class T> struct Big;
template <> struct Big<double> { static constexpr double v = 1.e+40; };
// FP32: the masked extrema of a cell whose whole stencil is land are +-zbig, and
// nonosc divides them by zrtrn = 1e-15 and scales by e1e2t e3t / p2dt (up to ~1e11):
// 1e10 keeps that product finite in FP32 (1e30 overflowed to inf, and the limiter's
// 0 * inf gave NaN) while staying far above any tracer value, so wet points are
// limited exactly as with the reference's 1e40.
template <> struct Big<float> { static constexpr float v = 1.e+10f; };

// Grid barrier for persistent kernels launched cooperatively (all blocks resident).
// The arrival counter only grows within a launch (the launcher zeroes it before
// each launch): at its e-th barrier, thread 0 of each block adds 1 with a release
// reduction -- posted, no value returned, so it does not wait for the L2 round trip
// of an atomic -- and polls the counter with acquire loads until it reaches e times
// the block count; the release/acquire pair makes every write before the barrier
// visible after it. No block resets or publishes anything, so the last block to
// arrive is not on the critical path twice. Each wait is bounded: after max_spins
// polls the block records NEMO_ERR_TIMEOUT in *err and returns false; every block
// checks the flag after each barrier and leaves its loop, so the kernel always ends.
struct GridBar {
  unsigned int* count;   // zeroed before each launch
  unsigned int* gen;     // unused
  int* err;
  unsigned int nblocks;
  long long max_spins;
};

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned int atom_add_acq_rel_gpu(unsigned int* p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void st_release_gpu(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void red_add_release_gpu(unsigned int* p, unsigned int v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// epoch: the block's count of barriers passed in this launch (a register, 0 at start)
__device__ __forceinline__ bool grid_barrier(const GridBar& b, unsigned int& epoch) {
  __shared__ int s_err;  // the error flag as thread 0 saw it, for the whole block
  __syncthreads();
  ++epoch;
  if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
    volatile int* verr = b.err;
    const unsigned int target = epoch * b.nblocks;
    red_add_release_gpu(b.count, 1u);
    long long s = 0;
    while ((int)(ld_acquire_gpu(b.count) - target) < 0) {
      if ((++s & 63) == 0 && *verr != 0) break;
      if (s > b.max_spins) {
        atomicExch(b.err, 5);
        break;
      }
    }
    s_err = *verr;
  }
  __syncthreads();
  return s_err == 0;
}

}  // namespace nemo
