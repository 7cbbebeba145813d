// adj.h -- host launchers of the adjoint kernels (FP64) and of tra_nxt, defined in
// adj_fp64.cu (compiled without FMA contraction, like the FP64 forward kernels).
#pragma once
#include "k_tra.cuh"

namespace nemo {

struct FctAdj {
  RO<double> pun, pvn, pwn;  // transports of the forward call (per member)
  RO<double> lam;            // pta_ad (jpi,jpj,jpk,kjpt) per member
  RO<double> tape;           // limiter multipliers, ((m*kjpt + n)*3 + face)*n3, face x,y,z
  double *tb_ad, *tn_ad;
  int kjpt, linssh;
  int kh, kv;              // orders of the forward's antidiffusive fluxes (2 or 4)
  double *zwt, *za;        // kv = 4: work of the transposed vertical interpolation (n3 per member)
};

struct LdfAdj {
  RO<double> lam;           // pta_ad
  double *tb_ad, *tbb_ad;   // tbb_ad: kpass 2 of the bilaplacian iso operator only
  double* G;                // work: zsign lam r1_e1e2t / e3t_n on the interior cells
  double *dit, *djt, *dk;   // work: adjoints of the gradients (jpi,jpj,jpk,kjpt)
};

// the adjoint of dyn_spg_ts (k_spg_adj.cuh)
struct SpgAdjArgs {
  double *ua, *va, *un, *vn;                    // 3-D adjoints (in/out)
  double *ssha, *ua_b, *va_b, *un_adv, *vn_adv; // adjoints of outputs only (read, then zeroed)
  double *ub2_b, *vb2_b, *un_bf, *vn_bf;        // in/out
  double *sshn, *un_b, *vn_b, *ub_b, *vb_b;     // adjoints of inputs only (accumulated)
  const double* rcdu;                           // the forward's bottom drag coefficient
  // work, (jpi,jpj) per member
  double *X, *Y, *uab, *vab;                    // adjoints of the sub-step sums un_adv, vn_adv, ua_b, va_b
  double *Au, *Aub, *Aubb, *Av, *Avb, *Avbb;    // carried adjoints of un_e, ub_e, ubb_e (vn_e ...)
  double *Sn, *Sb, *Sbb;                        // of sshn_e, sshb_e, sshbb_e
  double *Fu, *Fv;                              // of the barotropic forcing zu_frc, zv_frc
  double *gu, *gv, *zhd;                        // per sub-step
  double r1_2dt_b, atfp, rdtbt, grav, sl;
  int euler, sc;
};

// per sub-step constants
struct SpgAdjStep {
  double w1, w2;              // wgtbtp1, wgtbtp2 of the sub-step
  double zb1, zb2, zb3;       // AB3 extrapolation (:724-736)
  double za0, za1, za2, za3;  // AM4 ssh (:904-931)
};

// the adjoint of dyn_nxt (k_step_adj.cuh)
struct NxtAdjArgs {
  double *ua, *va, *un, *vn, *ub, *vb;
  double *un_b, *vn_b, *ub_b, *vb_b;
  double *ua_b, *va_b;
  double atfp;
  int euler;
};

struct ZdfAdj {
  double* lam;     // pta_ad: in, the after tracer's adjoint; out, the trend's
  double* tb_ad;
};


cudaError_t launch_fct_adj(const Dom<double>& d, const FctAdj& a, cudaStream_t s);
cudaError_t launch_lap_adj(const Dom<double>& d, const LdfArgs<double>& a, const LdfAdj& b, cudaStream_t s);
cudaError_t launch_iso_adj(const Dom<double>& d, const LdfArgs<double>& a, const LdfAdj& b, cudaStream_t s);
cudaError_t launch_zdf_adj(const Dom<double>& d, const ZdfArgs<double>& a, const ZdfAdj& b, cudaStream_t s);
template <class T>
cudaError_t launch_tra_nxt(const Dom<T>& d, T* tsb, T* tsn, T* tsa, T atfp, int euler, cudaStream_t s);
cudaError_t launch_tra_nxt_adj(const Dom<double>& d, double* tsb_ad, double* tsn_ad, double* tsa_ad, double atfp,
                               int euler, cudaStream_t s);
// the adjoints of wzv (G: a (jpi,jpj,jpk) work array per member), dyn_nxt, ssh_swp
cudaError_t launch_wzv_adj(const Dom<double>& d, double* un_ad, double* vn_ad, double* wn_ad, double* G, cudaStream_t s);
cudaError_t launch_dyn_nxt_adj(const Dom<double>& d, const NxtAdjArgs& a, cudaStream_t s);
cudaError_t launch_ssh_swp_adj(const Dom<double>& d, double* sb, double* sn, double* sa, double atfp, int euler,
                               cudaStream_t s);
// the adjoint of dyn_spg_ts: steps[jn - 1] holds the constants of sub-step jn
cudaError_t launch_spg_adj(const Dom<double>& d, const SpgAdjArgs& a, const SpgAdjStep* steps, int icycle,
                           cudaStream_t s);

}  // namespace nemo
