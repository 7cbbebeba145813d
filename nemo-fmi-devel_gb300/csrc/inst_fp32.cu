// inst_fp32.cu -- FP32-bulk instantiation (mixed precision mode); FMA contraction on.
#include "inst_impl.cuh"
namespace nemo {
NEMO_INSTANTIATE(float)
}
