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

}  // namespace nemo
