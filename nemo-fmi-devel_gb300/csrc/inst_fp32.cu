// inst_fp32.cu -- FP32-bulk instantiation (mixed precision mode); FMA contraction on.
#include "inst_impl.cuh"
namespace nemo {
NEMO_INSTANTIATE(float)

cudaError_t launch_tra_fused(const Dom<float>& d, const FusedArgs<float>& a, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_tra_fused<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)FusedSmem::bytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid((d.jpi - 2 + FTX - 1) / FTX, (d.jpj - 2 + FTY - 1) / FTY, d.nmem);
  k_tra_fused<float><<<grid, FNT, FusedSmem::bytes, s>>>(d, a);
  return cudaGetLastError();
}
}
