// SSF partition weights without any device allocation.
//
// For callers that cannot allocate device memory at the time they need
// weights: a host program whose own pool has already reserved the GPU (the
// usual setup of SCF codes that hand a fixed buffer to their integrator), or
// code that must not trigger allocator synchronization inside a latency-
// critical loop.  The caller passes device pointers for every input and
// output; the work space this kernel needs (point-to-atom distances and the
// inverse inter-atomic distances) lives in the file-scope array below, which
// every GPU that loads this library keeps until the process exits.
//
// Limits and sharing rules:
//   * natoms * npts + natoms * natoms <= kNoAllocScratchDoubles (4 Mi doubles,
//     32 MiB); larger requests are rejected with an error, callers split the
//     points into several calls;
//   * all calls share the one array: calls whose work overlaps on the GPU (two
//     streams, two host threads) race and must be serialized by the caller;
//   * every call looks up the array's device address (cudaGetSymbolAddress)
//     on the current device, so the address stays right after a context
//     reset; the first call on a device also loads this library's device
//     code there and should come before any stream capture;
//   * parent indices must lie in [0, natoms): a point whose parent does not
//     keeps its weight (the call does not synchronize, so it cannot report it).
#include "../host/device_api.hpp"
#include "device_common.cuh"

namespace gb300 {

namespace {

constexpr int64_t kNoAllocScratchDoubles = int64_t(1) << 22;
__device__ __align__(256) double g_ssf_scratch[kNoAllocScratchDoubles];

// Device address of g_ssf_scratch in the current device's context.
double* scratch_address() {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_ssf_scratch);
  if (e != cudaSuccess)
    throw error(std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
  return static_cast<double*>(p);
}

// rab_inv[a * natoms + b] = 1 / |R_a - R_b| (0 on the diagonal)
__global__ void rab_inverse_kernel(int natoms, const double* __restrict__ coords,
                                   double* __restrict__ rab_inv) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)natoms * natoms) return;
  const int a = (int)(i / natoms), b = (int)(i % natoms);
  if (a == b) {
    rab_inv[i] = 0.;
    return;
  }
  const double dx = coords[3 * a] - coords[3 * b];
  const double dy = coords[3 * a + 1] - coords[3 * b + 1];
  const double dz = coords[3 * a + 2] - coords[3 * b + 2];
  rab_inv[i] = 1. / sqrt(dx * dx + dy * dy + dz * dz);
}

}  // namespace

void ssf_weights_noalloc(int64_t npts, int natoms, const double* x, const double* y,
                         const double* z, const int32_t* iparent, const double* dist_nearest,
                         const double* coords, double* weights, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (npts < 0 || natoms <= 0) throw error("invalid sizes");
  if (npts == 0) return;
  const int64_t need = (int64_t)natoms * npts + (int64_t)natoms * natoms;
  if (need > kNoAllocScratchDoubles)
    throw error("request needs " + std::to_string(need) + " scratch doubles; the fixed work "
                "space holds " + std::to_string(kNoAllocScratchDoubles) +
                " (natoms*npts + natoms^2); split the points into smaller calls");
  if (npts > (int64_t)INT32_MAX) throw error("too many points for one call");
  double* scr = scratch_address();
  double* rab_inv = scr;
  double* dist = scr + (int64_t)natoms * natoms;
  const int64_t nn = (int64_t)natoms * natoms;
  rab_inverse_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(natoms, coords, rab_inv);
  GB300_CUDA(cudaGetLastError());
  launch_ssf_weights(npts, natoms, x, y, z, iparent, dist_nearest, coords, rab_inv, natoms, dist,
                     (int)npts, weights, nullptr, s);
}

}  // namespace gb300
