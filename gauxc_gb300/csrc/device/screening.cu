// Shell screening of the task candidates on the device (the Device load
// balancer's collision detection).
//
// Reference: src/load_balancer/device/cuda/cuda_collision_detection.cu:74-121
// (one bit per (task box, shell) from the cube/sphere test, then a scan and a
// position list), with the test of include/gauxc/util/geometry.hpp:36-49.
// Here a CTA takes one candidate box; each warp tests 32 consecutive shells
// and one ballot gives a 32-bit word of the bitset; the host turns the words
// into ascending shell lists.  The test uses explicitly rounded FP64
// multiplies and subtractions (no contraction into FMAs), the same operations
// in the same order as the host's cube_sphere_intersect, so the bits and the
// task lists equal the host load balancer's.
#include "../host/device_api.hpp"
#include "device_common.cuh"

#include <algorithm>

namespace gb300 {

namespace {

__device__ __forceinline__ bool cube_sphere_dev(const double* lo, const double* up, double cx,
                                                double cy, double cz, double rad) {
  double dist = __dmul_rn(rad, rad);
  const double c[3] = {cx, cy, cz};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double r = 0.;
    if (c[i] < lo[i]) r = __dsub_rn(lo[i], c[i]);
    else if (c[i] > up[i]) r = __dsub_rn(c[i], up[i]);
    dist = __dsub_rn(dist, __dmul_rn(r, r));
    if (dist < 0.) return false;
  }
  return true;
}

// boxes[6 i .. 6 i + 5] = lo xyz, up xyz of candidate c0 + i; bits[(i) * nwords + w]
__global__ void collision_kernel(int64_t ncand, int nshells, int nwords,
                                 const double* __restrict__ boxes,
                                 const double* __restrict__ shells,  // x, y, z, radius per shell
                                 uint32_t* __restrict__ bits) {
  const int64_t i = blockIdx.x;
  if (i >= ncand) return;
  const double lo[3] = {boxes[6 * i], boxes[6 * i + 1], boxes[6 * i + 2]};
  const double up[3] = {boxes[6 * i + 3], boxes[6 * i + 4], boxes[6 * i + 5]};
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int w = warp; w < nwords; w += nw) {
    const int s = 32 * w + lane;
    bool hit = false;
    if (s < nshells)
      hit = cube_sphere_dev(lo, up, shells[4 * s], shells[4 * s + 1], shells[4 * s + 2],
                            shells[4 * s + 3]);
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) bits[i * nwords + w] = m;
  }
}

}  // namespace

void screen_boxes_device(const std::vector<double>& boxes, const BasisSet& bs,
                         std::vector<uint32_t>& bits, int& nwords) {
  if (cuda_device_count() == 0) throw error("no CUDA device available for the Device load balancer");
  const int64_t ncand = (int64_t)(boxes.size() / 6);
  const int nsh = (int)bs.shells.size();
  nwords = (nsh + 31) / 32;
  bits.assign((size_t)ncand * nwords, 0u);
  if (ncand == 0 || nsh == 0) return;
  std::vector<double> sh(4 * (size_t)nsh);
  for (int s = 0; s < nsh; ++s) {
    sh[4 * s] = bs.shells[s].O[0];
    sh[4 * s + 1] = bs.shells[s].O[1];
    sh[4 * s + 2] = bs.shells[s].O[2];
    sh[4 * s + 3] = bs.shells[s].cutoff_radius;
  }
  // candidates in chunks whose bitset stays under 256 MB of device memory
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(ncand, (int64_t)(64u << 20) / nwords));
  cudaStream_t st;
  GB300_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double *dsh = nullptr, *dbox = nullptr;
  uint32_t* dbits = nullptr;
  try {
    GB300_CUDA(cudaMalloc(&dsh, sh.size() * sizeof(double)));
    GB300_CUDA(cudaMalloc(&dbox, (size_t)chunk * 6 * sizeof(double)));
    GB300_CUDA(cudaMalloc(&dbits, (size_t)chunk * nwords * sizeof(uint32_t)));
    GB300_CUDA(cudaMemcpyAsync(dsh, sh.data(), sh.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    for (int64_t c0 = 0; c0 < ncand; c0 += chunk) {
      const int64_t n = std::min(chunk, ncand - c0);
      GB300_CUDA(cudaMemcpyAsync(dbox, boxes.data() + 6 * c0, (size_t)n * 6 * sizeof(double),
                                 cudaMemcpyHostToDevice, st));
      collision_kernel<<<(unsigned)n, 256, 0, st>>>(n, nsh, nwords, dbox, dsh, dbits);
      GB300_CUDA(cudaGetLastError());
      GB300_CUDA(cudaMemcpyAsync(bits.data() + (size_t)c0 * nwords, dbits,
                                 (size_t)n * nwords * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    }
    GB300_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    cudaFree(dsh);
    cudaFree(dbox);
    cudaFree(dbits);
    cudaStreamDestroy(st);
    throw;
  }
  cudaFree(dsh);
  cudaFree(dbox);
  cudaFree(dbits);
  GB300_CUDA(cudaStreamDestroy(st));
}

}  // namespace gb300
