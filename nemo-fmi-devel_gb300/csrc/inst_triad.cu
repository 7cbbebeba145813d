// inst_triad.cu -- launchers of the triad operator's kernels (k_triad.cuh), both
// precisions; compiled with --fmad=false so the FP64 form rounds as the reference's
// FP64 CPU build.
#include "k_triad.cuh"
#include "launch.h"
#include "triad.h"

namespace nemo {

namespace {
constexpr int TX = 32, TY = 4;
template <class T>
dim3 t_pt(const Dom<T>& d) { return dim3((d.jpi + TX - 1) / TX, (d.jpj + TY - 1) / TY, d.nmem * d.jpk); }
}  // namespace

template <class T>
cudaError_t launch_ldf_slp_triad(const Dom<T>& d, const TriadArgs<T>& a, cudaStream_t s) {
  k_triad_slp<T><<<t_pt(d), dim3(TX, TY), 0, s>>>(d, a);
  if (a.wslp2) k_triad_wslp2<T><<<t_pt(d), dim3(TX, TY), 0, s>>>(d, a);
  ktick(NEMO_K_TRIAD, s);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_tra_ldf_triad(const Dom<T>& d, const TriadArgs<T>& a, cudaStream_t s) {
  if (a.l.kpass == 1) k_triad_coef<T><<<t_pt(d), dim3(TX, TY), 0, s>>>(d, a);
  k_triad_flux<T><<<t_pt(d), dim3(TX, TY), 0, s>>>(d, a);
  k_triad_tfw<T><<<t_pt(d), dim3(TX, TY), 0, s>>>(d, a);
  k_triad_div<T><<<t_pt(d), dim3(TX, TY), 0, s>>>(d, a);
  ktick(NEMO_K_TRIAD, s);
  return cudaGetLastError();
}

#define NEMO_TRIAD_INST(T)                                                                 \
  template cudaError_t launch_ldf_slp_triad<T>(const Dom<T>&, const TriadArgs<T>&, cudaStream_t); \
  template cudaError_t launch_tra_ldf_triad<T>(const Dom<T>&, const TriadArgs<T>&, cudaStream_t);
NEMO_TRIAD_INST(double)
NEMO_TRIAD_INST(float)
#undef NEMO_TRIAD_INST

}  // namespace nemo
