// noalloc.cu -- the compensated global sum without any device allocation.
//
// Some callers of this library cannot allocate device memory at the point where
// they need a global sum:
//  * host models whose device memory is owned by another runtime -- an OpenACC or
//    CUDA Fortran data region, or the caching allocator of a coupling framework --
//    which must not see allocations made behind its back;
//  * operational set-ups (ensembles packed onto one GPU) that fix the device-memory
//    footprint at start-up and must not fail later on an out-of-memory error.
// They can call nemo_gpu_glob_sum_noalloc: it needs no context, takes the field, the
// mask and the output as device pointers, and keeps its block partial sums in the
// file-scope array g_globsum_scratch below (about 1 MB that every GPU which loads
// the library holds until the process exits). It calls no cudaMalloc, cudaFree or
// other allocating routine.
#include <cstdio>
#include <mutex>

#include "../../include/nemo_gpu.h"
#include "k_dyn.cuh"

namespace {

constexpr int NA_MAX_BLOCKS = 1024;   // partial sums per member
constexpr int NA_MAX_MEMBERS = 64;    // ensemble members per call
constexpr int NA_MAX_DEVICES = 64;

// (hi, lo) partial of every block of every member; nothing carries from one call
// to the next, because each call writes every entry it later reads.
__device__ __align__(256) double g_globsum_scratch[2 * NA_MAX_BLOCKS * NA_MAX_MEMBERS];

struct DeviceSetup {
  double* scratch = nullptr;  // device address of g_globsum_scratch on this device
  int nblk = 0;
};
DeviceSetup g_setup[NA_MAX_DEVICES];
std::mutex g_setup_mutex;

// Once per device, with that device current: the device address of the array (the
// name g_globsum_scratch is only a host-side stand-in) and the partial-sum count.
int setup_current_device(DeviceSetup** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return NEMO_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceSetup& s = g_setup[dev];
  if (!s.scratch) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_globsum_scratch) != cudaSuccess) return NEMO_ERR_CUDA;
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return NEMO_ERR_CUDA;
    s.nblk = 4 * nsm < NA_MAX_BLOCKS ? 4 * nsm : NA_MAX_BLOCKS;
    s.scratch = static_cast<double*>(p);
  }
  *out = &s;
  return NEMO_OK;
}

}  // namespace

extern "C" int nemo_gpu_glob_sum_noalloc(const void* ptab, const double* tmask_i, int jpi, int jpj, int nk,
                                         int nmembers, int is_fp64, void* stream, double* out) {
  if (!ptab || !tmask_i || !out || jpi < 1 || jpj < 1 || nk < 1) return NEMO_ERR_ARG;
  if (nmembers < 1 || nmembers > NA_MAX_MEMBERS) {
    fprintf(stderr, "nemo_gpu_glob_sum_noalloc: nmembers = %d outside 1..%d\n", nmembers, NA_MAX_MEMBERS);
    return NEMO_ERR_ARG;
  }
  DeviceSetup* s = nullptr;
  int st = setup_current_device(&s);
  if (st != NEMO_OK) return st;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const long n2 = (long)jpi * jpj;
  if (is_fp64)
    nemo::k_globsum_partial<double><<<dim3(s->nblk, nmembers), 256, 0, cs>>>(static_cast<const double*>(ptab), tmask_i,
                                                                             n2, nk, s->scratch);
  else
    nemo::k_globsum_partial<float><<<dim3(s->nblk, nmembers), 256, 0, cs>>>(static_cast<const float*>(ptab), tmask_i,
                                                                           n2, nk, s->scratch);
  nemo::k_globsum_final<<<nmembers, 256, 0, cs>>>(s->scratch, s->nblk, out);
  return cudaGetLastError() == cudaSuccess ? NEMO_OK : NEMO_ERR_CUDA;
}
