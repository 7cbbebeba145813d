// step.h -- host launchers of the rest-of-step kernels (k_step.cuh), defined in
// inst_step.cu for both precisions.
#pragma once
#include "k_tra.cuh"

namespace nemo {

template <class T, class A>
struct NxtArgs {
  T *ua, *va, *un, *vn, *ub, *vb;   // (jpi,jpj,jpk) per member
  T *un_b, *vn_b, *ub_b, *vb_b;     // (jpi,jpj) per member
  const A *ua_b, *va_b;             // after barotropic velocities of dyn_spg_ts
  T atfp;
  int euler;
};

template <class T>
cudaError_t launch_wzv(const Dom<T>& d, const T* un, const T* vn, T* wn, T z1_2dt, cudaStream_t s);
template <class T>
cudaError_t launch_dyn_zdf_step(const Dom<T>& d, const T* ub, const T* vb, T* ua, T* va, T r2dt, cudaStream_t s);
template <class T>
cudaError_t launch_dyn_nxt(const Dom<T>& d, const NxtArgs<T, double>& a, cudaStream_t s);
template <class T>
cudaError_t launch_ssh_swp(const Dom<T>& d, T* sshb, T* sshn, const double* ssha, T atfp, int euler, cudaStream_t s);

}  // namespace nemo
