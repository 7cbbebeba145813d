// inst_step.cu -- launchers of the rest-of-step kernels, both precisions; compiled
// with --fmad=false so the FP64 form rounds as the reference's FP64 CPU build.
#include "k_diag.cuh"
#include "k_step.cuh"
#include "launch.h"

namespace nemo {

namespace {
constexpr int SX = 32, SY = 4;
template <class T>
dim3 s_col(const Dom<T>& d) { return dim3((d.jpi + SX - 1) / SX, (d.jpj + SY - 1) / SY, d.nmem); }
template <class T>
dim3 s_pt(const Dom<T>& d) { return dim3((d.jpi + SX - 1) / SX, (d.jpj + SY - 1) / SY, d.nmem * d.jpk); }
}  // namespace

template <class T>
cudaError_t launch_wzv(const Dom<T>& d, const T* un, const T* vn, T* wn, T z1_2dt, cudaStream_t s) {
  k_wzv<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, un, vn, wn, z1_2dt);
  ktick(NEMO_K_WZV, s);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_dyn_zdf_step(const Dom<T>& d, const T* ub, const T* vb, T* ua, T* va, T r2dt, const T* e3u_b,
                                const T* e3v_b, const T* e3u_a, const T* e3v_a, cudaStream_t s) {
  k_dyn_zdf_step<T><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, ub, vb, ua, va, r2dt, e3u_b, e3v_b, e3u_a, e3v_a);
  ktick(NEMO_K_DYN_ZDF_STEP, s);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_dyn_nxt(const Dom<T>& d, const NxtArgs<T, double>& a, cudaStream_t s) {
  k_dyn_nxt<T, double><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_DYN_NXT, s);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_ssh_swp(const Dom<T>& d, T* sshb, T* sshn, const double* ssha, T atfp, int euler, cudaStream_t s) {
  k_ssh_swp<T, double><<<s_col(d), dim3(SX, SY), 0, s>>>(d, sshb, sshn, ssha, atfp, euler);
  ktick(NEMO_K_SSH_SWP, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vvl_sf_nxt(const Dom<T>& d, const VvlArgs<T>& a, cudaStream_t s) {
  k_vvl_sf_nxt_t<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  k_vvl_sf_nxt_uv<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_VVL_SF, s);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_vvl_sf_swp(const Dom<T>& d, const VvlArgs<T>& a, cudaStream_t s) {
  k_vvl_sf_swp<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_VVL_SF, s);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_tra_nxt_vvl(const Dom<T>& d, const VvlArgs<T>& a, cudaStream_t s) {
  k_tra_nxt_vvl<T><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_VVL_NXT, s);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_dyn_nxt_vvl(const Dom<T>& d, const VvlArgs<T>& a, cudaStream_t s) {
  k_dyn_nxt_vvl_a<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  k_dyn_nxt_vvl_b<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_VVL_NXT, s);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_ssh_swp_vvl(const Dom<T>& d, const VvlArgs<T>& a, T* sshb, T* sshn, cudaStream_t s) {
  k_ssh_swp_vvl<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a, sshb, sshn);
  ktick(NEMO_K_VVL_NXT, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_ldf_slp(const Dom<T>& d, const SlpArgs<T>& a, cudaStream_t s) {
  if (a.gru_b) {  // partial steps: the bottom level's gradients from zps_hde
    k_slp_mxl<T, true><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
    k_slp_pre<T, true><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, a);
  } else {
    k_slp_mxl<T, false><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
    k_slp_pre<T, false><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, a);
  }
  k_slp_filter<T><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_LDF_SLP, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_zps_hde_rd(const Dom<T>& d, const EosArgs<T>& a, const T* prd, T* pgru, T* pgrv, cudaStream_t s) {
  k_zps_hde_rd<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a, prd, pgru, pgrv);
  ktick(NEMO_K_ZPS_HDE, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_zps_hde(const Dom<T>& d, const T* pta, T* pgtu, T* pgtv, int kjpt, cudaStream_t s) {
  k_zps_hde<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, pta, pgtu, pgtv, kjpt);
  ktick(NEMO_K_ZPS_HDE, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_tra_sbc(const Dom<T>& d, const SbcArgs<T>& a, cudaStream_t s) {
  k_tra_sbc<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_TRA_SBC, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_tra_qsr(const Dom<T>& d, const QsrArgs<T>& a, cudaStream_t s) {
  k_tra_qsr<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_TRA_QSR, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_eos(const Dom<T>& d, const EosArgs<T>& a, cudaStream_t s) {
  k_eos<T><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(a.what == 3 ? NEMO_K_BN2 : NEMO_K_EOS, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_dyn_hpg(const Dom<T>& d, const T* rhd, T* ua, T* va, T zcoef0, cudaStream_t s) {
  k_hpg_zco<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, rhd, ua, va, zcoef0);
  ktick(NEMO_K_DYN_HPG, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_zdf_mxl(const Dom<T>& d, const MxlArgs<T>& a, cudaStream_t s) {
  k_zdf_mxl<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_ZDF_MXL, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_dyn_zdf_imp(const Dom<T>& d, const DynZdfArgs<T>& a, cudaStream_t s) {
  k_dyn_zdf_imp<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_DYN_ZDF_STEP, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_usr_sbc_a(const Dom<T>& d, const UsrSbcArgs<T>& a, cudaStream_t s) {
  k_usr_sbc_a<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_USR_SBC, s);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_usr_sbc_b(const Dom<T>& d, const UsrSbcArgs<T>& a, cudaStream_t s) {
  k_usr_sbc_b<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_USR_SBC, s);
  return cudaGetLastError();
}
cudaError_t launch_usr_put(double* dst, const double* v, cudaStream_t s) {
  k_usr_put<<<1, 1, 0, s>>>(dst, v[0], v[1], v[2], v[3], v[4], v[5], v[6]);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_zdf_phy(const Dom<T>& d, const ZphyArgs<T>& a, cudaStream_t s) {
  k_zdf_sh2<T><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_ZDF_PHY, s);
  k_zdf_tke<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, a);
  ktick(NEMO_K_ZDF_PHY, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_dyn_ldf_lap(const Dom<T>& d, const T* ahmt, const T* ahmf, const T* pub, const T* pvb, T* pua, T* pva,
                               T zsign, cudaStream_t s) {
  k_dyn_ldf_lap<T><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, ahmt, ahmf, pub, pvb, pua, pva, zsign);
  ktick(NEMO_K_DYN_LDF, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vor_ene(const Dom<T>& d, int kvor, const T* pun, const T* pvn, T* pua, T* pva, cudaStream_t s) {
  k_vor_ene<T><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, kvor, pun, pvn, pua, pva);
  ktick(NEMO_K_DYN_VOR, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_dyn_keg(const Dom<T>& d, const T* un, const T* vn, T* ua, T* va, cudaStream_t s) {
  k_dyn_keg<T><<<s_pt(d), dim3(SX, SY), 0, s>>>(d, un, vn, ua, va);
  ktick(NEMO_K_DYN_KEG, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_dyn_zad(const Dom<T>& d, const T* un, const T* vn, const T* wn, T* ua, T* va, cudaStream_t s) {
  k_dyn_zad<T><<<s_col(d), dim3(SX, SY), 0, s>>>(d, un, vn, wn, ua, va);
  ktick(NEMO_K_DYN_ZAD, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_stp_ctl(const Dom<T>& d, const T* sshn, const T* un, const T* ts, double* part, int nblk,
                           int someoce, double* out, unsigned long long* idx, int* flag, cudaStream_t s) {
  k_ctl_partial<T><<<dim3(nblk, d.nmem), DG_THREADS, 0, s>>>(d, sshn, un, ts, part);
  ktick(NEMO_K_STP_CTL, s);
  k_ctl_final<T><<<d.nmem, DG_THREADS, 0, s>>>(d, part, nblk, someoce, out, idx, flag);
  ktick(NEMO_K_STP_CTL, s);
  k_ctl_locate<T><<<dim3(nblk, d.nmem), DG_THREADS, 0, s>>>(d, sshn, un, ts, out, idx);
  ktick(NEMO_K_STP_CTL, s);
  k_ctl_pos<T><<<(d.nmem + 31) / 32, 32, 0, s>>>(d, out, idx);
  ktick(NEMO_K_STP_CTL, s);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_hsb_init(const Dom<T>& d, const HsbArgs<T>& a, int nblk, cudaStream_t s) {
  k_hsb_init<T><<<nblk, DG_THREADS, 0, s>>>(d, a);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_dia_hsb(const Dom<T>& d, const HsbArgs<T>& a, double* part, int nblk, cudaStream_t s) {
  k_hsb_partial<T><<<dim3(nblk, d.nmem), DG_THREADS, 0, s>>>(d, a, part);
  k_hsb_final<T><<<d.nmem, 32, 0, s>>>(d, a, part, nblk);
  ktick(NEMO_K_DIA_HSB, s);
  return cudaGetLastError();
}

#define NEMO_STEP_INST(T)                                                                                      \
  template cudaError_t launch_stp_ctl<T>(const Dom<T>&, const T*, const T*, const T*, double*, int, int,       \
                                         double*, unsigned long long*, int*, cudaStream_t);                    \
  template cudaError_t launch_hsb_init<T>(const Dom<T>&, const HsbArgs<T>&, int, cudaStream_t);                \
  template cudaError_t launch_dia_hsb<T>(const Dom<T>&, const HsbArgs<T>&, double*, int, cudaStream_t);         \
  template cudaError_t launch_wzv<T>(const Dom<T>&, const T*, const T*, T*, T, cudaStream_t);                  \
  template cudaError_t launch_dyn_zdf_step<T>(const Dom<T>&, const T*, const T*, T*, T*, T, const T*, const T*, \
                                              const T*, const T*, cudaStream_t);                            \
  template cudaError_t launch_dyn_nxt<T>(const Dom<T>&, const NxtArgs<T, double>&, cudaStream_t);              \
  template cudaError_t launch_ssh_swp<T>(const Dom<T>&, T*, T*, const double*, T, int, cudaStream_t);      \
  template cudaError_t launch_vvl_sf_nxt<T>(const Dom<T>&, const VvlArgs<T>&, cudaStream_t);                \
  template cudaError_t launch_vvl_sf_swp<T>(const Dom<T>&, const VvlArgs<T>&, cudaStream_t);                \
  template cudaError_t launch_tra_nxt_vvl<T>(const Dom<T>&, const VvlArgs<T>&, cudaStream_t);               \
  template cudaError_t launch_dyn_nxt_vvl<T>(const Dom<T>&, const VvlArgs<T>&, cudaStream_t);               \
  template cudaError_t launch_ssh_swp_vvl<T>(const Dom<T>&, const VvlArgs<T>&, T*, T*, cudaStream_t);       \
  template cudaError_t launch_ldf_slp<T>(const Dom<T>&, const SlpArgs<T>&, cudaStream_t);                  \
  template cudaError_t launch_zps_hde_rd<T>(const Dom<T>&, const EosArgs<T>&, const T*, T*, T*, cudaStream_t);  \
  template cudaError_t launch_zps_hde<T>(const Dom<T>&, const T*, T*, T*, int, cudaStream_t);             \
  template cudaError_t launch_tra_sbc<T>(const Dom<T>&, const SbcArgs<T>&, cudaStream_t);                  \
  template cudaError_t launch_tra_qsr<T>(const Dom<T>&, const QsrArgs<T>&, cudaStream_t);                  \
  template cudaError_t launch_eos<T>(const Dom<T>&, const EosArgs<T>&, cudaStream_t);                      \
  template cudaError_t launch_dyn_hpg<T>(const Dom<T>&, const T*, T*, T*, T, cudaStream_t);              \
  template cudaError_t launch_zdf_mxl<T>(const Dom<T>&, const MxlArgs<T>&, cudaStream_t);                  \
  template cudaError_t launch_dyn_zdf_imp<T>(const Dom<T>&, const DynZdfArgs<T>&, cudaStream_t);           \
  template cudaError_t launch_usr_sbc_a<T>(const Dom<T>&, const UsrSbcArgs<T>&, cudaStream_t);              \
  template cudaError_t launch_usr_sbc_b<T>(const Dom<T>&, const UsrSbcArgs<T>&, cudaStream_t);              \
  template cudaError_t launch_zdf_phy<T>(const Dom<T>&, const ZphyArgs<T>&, cudaStream_t);                 \
  template cudaError_t launch_dyn_ldf_lap<T>(const Dom<T>&, const T*, const T*, const T*, const T*, T*, T*, T,   \
                                             cudaStream_t);                                             \
  template cudaError_t launch_vor_ene<T>(const Dom<T>&, int, const T*, const T*, T*, T*, cudaStream_t);       \
  template cudaError_t launch_dyn_keg<T>(const Dom<T>&, const T*, const T*, T*, T*, cudaStream_t);             \
  template cudaError_t launch_dyn_zad<T>(const Dom<T>&, const T*, const T*, const T*, T*, T*, cudaStream_t);
NEMO_STEP_INST(double)
NEMO_STEP_INST(float)

}  // namespace nemo
