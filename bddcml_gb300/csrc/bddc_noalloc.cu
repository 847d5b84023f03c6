// Subdomain dot product on device-resident vectors, with all scratch in one
// fixed, statically allocated device array (no device or host allocation per
// call).  Entry point: bddcml_dotprod_subdomain_dev_c (bddc_abi.cpp).
//
// Scratch layout (one array for the whole process and device, 256-byte aligned):
//   [0, 8*NOALLOC_MAX_IFACE)        interface weights w_i of the subdomain (copied per call)
//   [.., +4*NOALLOC_MAX_IFACE)      subdomain dof index of each interface dof (copied per call)
//   [.., +8*NOALLOC_BLOCKS)         per-block partial sums
//   then                            one double result, one unsigned ticket counter
// The ticket counter must be zero when a call starts: each call clears it on
// its stream before the launch (a 4-byte memset, no allocation), so a launch
// that failed part-way cannot leave it stale.  Two calls that overlap in time
// (several host threads, or work on several streams) share the scratch and
// race; callers must not overlap them.
//
// With CUDA's lazy module loading (the default since CUDA 12.2) this file's
// module, and with it the scratch array, is loaded on a device by the first
// call there (at cudaGetSymbolAddress).  That first call is the one that makes
// the device allocation; later calls allocate nothing.
#include <cstdint>
#include <cstring>
#include <string>

#include <cuda_runtime.h>

#include "bddc_internal.hpp"

namespace bddc {

namespace {

constexpr int NOALLOC_BLOCKS = 128;
constexpr int NOALLOC_THREADS = 256;
constexpr size_t OFF_W = 0;
constexpr size_t OFF_IDX = OFF_W + sizeof(double) * NOALLOC_MAX_IFACE;
constexpr size_t OFF_PART = OFF_IDX + sizeof(int) * NOALLOC_MAX_IFACE;
constexpr size_t OFF_RESULT = OFF_PART + sizeof(double) * NOALLOC_BLOCKS;
constexpr size_t OFF_TICKET = OFF_RESULT + sizeof(double);
constexpr size_t SCRATCH_BYTES = OFF_TICKET + 256;

}  // namespace

// The scratch itself: every GPU that loads the library holds this array
// (about 0.8 MB) until the process exits.  Zero-initialised at load.  Host
// code must not pass its name to a kernel (on the host it names a stand-in,
// not device memory); the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_dot_scratch[SCRATCH_BYTES];

namespace {

constexpr int MAX_DEVICES = 64;
unsigned char* g_scratch_ptr[MAX_DEVICES] = {};  // device address of g_dot_scratch, per device

// sum_i v1[i] v2[i] over all ndof dofs, plus sum_j (w_j - 1) v1[idx_j] v2[idx_j]
// over the interface dofs: the weighted product of dd_dotprod_local
// (module_dd.f90:12790-12832).  Partials per block, reduced in block order by
// the last block to arrive, so the result does not depend on scheduling.
__global__ void __launch_bounds__(NOALLOC_THREADS) k_dot_subdomain(const double* __restrict__ v1,
                                                                   const double* __restrict__ v2, int ndof, int nif,
                                                                   unsigned char* __restrict__ scratch) {
  const double* w = reinterpret_cast<const double*>(scratch + OFF_W);
  const int* idx = reinterpret_cast<const int*>(scratch + OFF_IDX);
  double* part = reinterpret_cast<double*>(scratch + OFF_PART);
  double* result = reinterpret_cast<double*>(scratch + OFF_RESULT);
  unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch + OFF_TICKET);
  __shared__ double red[NOALLOC_THREADS / 32];
  __shared__ bool last;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += gridDim.x * blockDim.x) acc += v1[i] * v2[i];
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nif; j += gridDim.x * blockDim.x) {
    const int i = idx[j];
    acc += v1[i] * (w[j] - 1.0) * v2[i];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < NOALLOC_THREADS / 32; ++q) s += red[q];
    part[blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double s = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) s += reinterpret_cast<volatile double*>(part)[b];
    *result = s;
    *ticket = 0u;
  }
}

}  // namespace

bool device_dotprod_noalloc(const int* iface_dofs, const double* weights, int nif, const double* v1,
                            const double* v2, int ndof, double* out, Error& err) {
  auto fail = [&](int code, const std::string& m) {
    err = Error{code, m};
    return false;
  };
  if (nif < 0 || nif > NOALLOC_MAX_IFACE)
    return fail(ERR_ARGUMENT, "subdomain interface has " + std::to_string(nif) +
                                  " dofs; the fixed scratch of this entry point holds at most " +
                                  std::to_string(NOALLOC_MAX_IFACE));
  if (ndof < 0 || (ndof > 0 && (!v1 || !v2)) || !out) return fail(ERR_ARGUMENT, "null vector or result pointer");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= MAX_DEVICES) return fail(ERR_CUDA, "device index out of range");
  if (!g_scratch_ptr[dev]) {  // first call on this device: look up the scratch address
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_dot_scratch);
    if (e != cudaSuccess) return fail(ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  unsigned char* scratch = g_scratch_ptr[dev];
  // legacy default stream: ordered after the caller's work on blocking streams
  const cudaStream_t st = 0;
  if (nif > 0) {
    e = cudaMemcpyAsync(scratch + OFF_W, weights, sizeof(double) * nif, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(scratch + OFF_IDX, iface_dofs, sizeof(int) * nif, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail(ERR_CUDA, std::string("copy to scratch: ") + cudaGetErrorString(e));
  }
  e = cudaMemsetAsync(scratch + OFF_TICKET, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) return fail(ERR_CUDA, std::string("clear the ticket: ") + cudaGetErrorString(e));
  k_dot_subdomain<<<NOALLOC_BLOCKS, NOALLOC_THREADS, 0, st>>>(v1, v2, ndof, nif, scratch);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, scratch + OFF_RESULT, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(ERR_CUDA, std::string("dot product kernel: ") + cudaGetErrorString(e));
  return true;
}

}  // namespace bddc
