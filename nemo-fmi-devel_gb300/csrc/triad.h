// triad.h -- host launchers of the triad operator (k_triad.cuh), defined in
// inst_triad.cu for both precisions.
#pragma once
#include "k_triad.cuh"

namespace nemo {

template <class T>
cudaError_t launch_ldf_slp_triad(const Dom<T>& d, const TriadArgs<T>& a, cudaStream_t s);
template <class T>
cudaError_t launch_tra_ldf_triad(const Dom<T>& d, const TriadArgs<T>& a, cudaStream_t s);

}  // namespace nemo
