// adj_fp64.cu -- launchers of the adjoint kernels and of tra_nxt. Compiled with
// --fmad=false like the FP64 forward kernels.
#include "k_adj.cuh"
#include "k_spg_adj.cuh"
#include "k_step_adj.cuh"
#include "launch.h"

namespace nemo {

namespace {
constexpr int AX = 32, AY = 4;
template <class T>
dim3 apt_grid(const Dom<T>& d) {
  return dim3((d.jpi + AX - 1) / AX, (d.jpj + AY - 1) / AY, d.nmem * d.jpk);
}
template <class T>
dim3 acol_grid(const Dom<T>& d) {
  return dim3((d.jpi + AX - 1) / AX, (d.jpj + AY - 1) / AY, d.nmem);
}
}  // namespace

cudaError_t launch_fct_adj(const Dom<double>& d, const FctAdj& a, cudaStream_t s) {
  k_fct_adj<<<apt_grid(d), dim3(AX, AY), 0, s>>>(d, a);
  ktick(NEMO_K_FCT_ADJ, s);
  if (a.kv == 4) {
    k_fct_adj_v4<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, a);
    ktick(NEMO_K_FCT_ADJ, s);
  }
  return cudaGetLastError();
}

cudaError_t launch_lap_adj(const Dom<double>& d, const LdfArgs<double>& a, const LdfAdj& b, cudaStream_t s) {
  k_lap_adj<<<apt_grid(d), dim3(AX, AY), 0, s>>>(d, a, b);
  ktick(NEMO_K_LAP_ADJ, s);
  return cudaGetLastError();
}

cudaError_t launch_iso_adj(const Dom<double>& d, const LdfArgs<double>& a, const LdfAdj& b, cudaStream_t s) {
  k_iso_adj_g<<<apt_grid(d), dim3(AX, AY), 0, s>>>(d, a, b);
  k_iso_adj_grad<<<apt_grid(d), dim3(AX, AY), 0, s>>>(d, a, b);
  k_iso_adj_tb<<<apt_grid(d), dim3(AX, AY), 0, s>>>(d, a, b);
  ktick(NEMO_K_ISO_ADJ, s);
  return cudaGetLastError();
}

cudaError_t launch_zdf_adj(const Dom<double>& d, const ZdfArgs<double>& a, const ZdfAdj& b, cudaStream_t s) {
  k_zdf_adj<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, a, b);
  ktick(NEMO_K_ZDF_ADJ, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_tra_nxt(const Dom<T>& d, T* tsb, T* tsn, T* tsa, T atfp, int euler, cudaStream_t s) {
  k_tra_nxt<T><<<apt_grid(d), dim3(AX, AY), 0, s>>>(d, tsb, tsn, tsa, atfp, euler);
  ktick(NEMO_K_TRA_NXT, s);
  return cudaGetLastError();
}
template cudaError_t launch_tra_nxt<double>(const Dom<double>&, double*, double*, double*, double, int, cudaStream_t);
template cudaError_t launch_tra_nxt<float>(const Dom<float>&, float*, float*, float*, float, int, cudaStream_t);

cudaError_t launch_tra_nxt_adj(const Dom<double>& d, double* tsb_ad, double* tsn_ad, double* tsa_ad, double atfp,
                               int euler, cudaStream_t s) {
  k_tra_nxt_adj<<<apt_grid(d), dim3(AX, AY), 0, s>>>(d, tsb_ad, tsn_ad, tsa_ad, atfp, euler);
  ktick(NEMO_K_TRA_NXT_ADJ, s);
  return cudaGetLastError();
}

cudaError_t launch_spg_adj(const Dom<double>& d, const SpgAdjArgs& a, const SpgAdjStep* steps, int icycle,
                           cudaStream_t s) {
  k_spg_adj_p3<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, a);
  for (int jn = icycle; jn >= 1; --jn) {
    k_spg_adj_s1<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, a, steps[jn - 1]);
    k_spg_adj_s2<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, a, steps[jn - 1]);
    k_spg_adj_s3<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, a, steps[jn - 1]);
  }
  k_spg_adj_p1<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, a);
  ktick(NEMO_K_SPG_ADJ, s);
  return cudaGetLastError();
}

cudaError_t launch_wzv_adj(const Dom<double>& d, double* un_ad, double* vn_ad, double* wn_ad, double* G, cudaStream_t s) {
  k_wzv_adj_g<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, wn_ad, G);
  k_wzv_adj_uv<<<apt_grid(d), dim3(AX, AY), 0, s>>>(d, un_ad, vn_ad, G);
  ktick(NEMO_K_STEP_ADJ, s);
  return cudaGetLastError();
}

cudaError_t launch_dyn_nxt_adj(const Dom<double>& d, const NxtAdjArgs& a, cudaStream_t s) {
  k_dyn_nxt_adj<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, a);
  ktick(NEMO_K_STEP_ADJ, s);
  return cudaGetLastError();
}

cudaError_t launch_ssh_swp_adj(const Dom<double>& d, double* sb, double* sn, double* sa, double atfp, int euler,
                               cudaStream_t s) {
  k_ssh_swp_adj<<<acol_grid(d), dim3(AX, AY), 0, s>>>(d, sb, sn, sa, atfp, euler);
  ktick(NEMO_K_STEP_ADJ, s);
  return cudaGetLastError();
}

}  // namespace nemo
