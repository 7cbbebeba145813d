// inst_fp64.cu -- FP64 ("plain form") instantiation. Compiled with --fmad=false so
// that every double operation rounds exactly as the reference's FP64 CPU build
// (gfortran without FMA contraction) rounds it.
#include "inst_impl.cuh"
namespace nemo {
NEMO_INSTANTIATE(double)
}
