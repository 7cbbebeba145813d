// launch.h -- host launchers of the kernels, explicitly instantiated for double (in
// inst_fp64.cu, compiled without FMA contraction) and float (inst_fp32.cu).
#pragma once
#include "k_dyn.cuh"
#include "k_tra.cuh"
#include "../../include/nemo_gpu.h"

namespace nemo {

// Per-kernel timing: while a context times the hot path it installs its clock for
// the calling thread, and every launcher below records an event on the launch
// stream after each kernel it enqueues (ids: enum nemo_kernel_id).
struct KernelClock {
  static constexpr int CAP = 96;
  cudaEvent_t ev[CAP + 1] = {};  // ev[0]: before the first kernel
  int id[CAP] = {};
  int n = 0;
};
extern thread_local KernelClock* t_kclock;

// Block heights of the 32-wide (i, j) launches, per kernel id, chosen by the
// context's autotuner (nemo_gpu_autotune): a context installs its table for the
// calling thread while it runs the hot path; elsewhere the default 4 (32 x 4).
struct LaunchShape {
  unsigned char ty[NEMO_K_COUNT] = {};
};
extern thread_local const LaunchShape* t_shape;
inline int kty(int id) {
  const LaunchShape* s = t_shape;
  return (s && s->ty[id]) ? s->ty[id] : 4;
}
inline void ktick(int id, cudaStream_t s) {
  KernelClock* k = t_kclock;
  if (k && k->n < KernelClock::CAP) {
    cudaEventRecord(k->ev[k->n + 1], s);
    k->id[k->n++] = id;
  }
}

template <class T>
cudaError_t launch_adv_trp(const Dom<T>& d, const T* un, const T* vn, const T* wn, T* zun, T* zvn, T* zwn,
                           cudaStream_t s);
template <class T>
cudaError_t launch_fct(const Dom<T>& d, const FctArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_ldf_lap(const Dom<T>& d, const LdfArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_ldf_iso(const Dom<T>& d, const LdfArgs<T>& a, int copy_akz_edges, int msc_edges, cudaStream_t s);
template <class T>
cudaError_t launch_iso_flux(const Dom<T>& d, const LdfArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_iso_edges(const Dom<T>& d, const LdfArgs<T>& a, int copy_akz_edges, int msc_edges, cudaStream_t s);
template <class T>
cudaError_t launch_zdf(const Dom<T>& d, const ZdfArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_clamp(T* x, long n, cudaStream_t s);
template <class T>
cudaError_t launch_spg(const Dom<T>& d, const SpgArgs<T>& a, const GridBar& bar, int p2_blocks, cudaStream_t s);
template <class T>
int spg_p2_blocks_per_sm(int cache, int vvl);
template <class T>
int spg_p2_ene_blocks_per_sm();
template <class T>
cudaError_t launch_lbc(T* p, int jpi, int jpj, long nslab, int is_f, T pval, cudaStream_t s);
template <class T>
cudaError_t launch_globsum(const T* x, const double* tmask_i, long n2, int nk, int nmem, double* part, int nblk,
                           double* out, cudaStream_t s);

}  // namespace nemo
