// FP64 FMA-pipe throughput probe and device selection.
//
// The DFMA probe gives the measured denominator for the FP64 path's roofline
// (the measured peaks cover HBM copy and BF16 tensor throughput only).
// Every thread runs 8 independent FMA chains; the result is stored only when
// a runtime flag that is never set is non-zero, so nothing is eliminated.
#include "../host/device_api.hpp"
#include "device_common.cuh"
#include "xc_mixed.cuh"

namespace gb300 {

namespace {
__global__ void __launch_bounds__(256) dfma_probe_kernel(int iters, double a, double b, int flag,
                                                         double* out) {
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0.;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  if (flag) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

double measure_fp64_peak() {
  if (cuda_device_count() == 0) throw error("no CUDA device available");
  int dev = 0, sms = 0;
  GB300_CUDA(cudaGetDevice(&dev));
  GB300_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256;
  double* out = nullptr;
  GB300_CUDA(cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  GB300_CUDA(cudaEventCreate(&e0));
  GB300_CUDA(cudaEventCreate(&e1));
  int iters = 256;
  float ms = 0.f;
  for (int rep = 0; rep < 12; ++rep) {
    GB300_CUDA(cudaEventRecord(e0));
    dfma_probe_kernel<<<blocks, threads>>>(iters, 0.999999, 1e-7, 0, out);
    GB300_CUDA(cudaEventRecord(e1));
    GB300_CUDA(cudaEventSynchronize(e1));
    GB300_CUDA(cudaGetLastError());
    GB300_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms > 40.f) break;
    iters *= 2;
  }
  GB300_CUDA(cudaEventDestroy(e0));
  GB300_CUDA(cudaEventDestroy(e1));
  GB300_CUDA(cudaFree(out));
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  return flops / (ms * 1e-3) / 1e12;
}

void set_device(int d) { GB300_CUDA(cudaSetDevice(d)); }

bool host_register(void* p, size_t bytes) {
  const cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterDefault);
  if (e == cudaErrorHostMemoryAlreadyRegistered) {
    cudaGetLastError();
    return false;
  }
  GB300_CUDA(e);
  return true;
}

void host_unregister(void* p) { GB300_CUDA(cudaHostUnregister(p)); }

double tensor_core_selftest(int n, int k) {
  if (cuda_device_count() == 0) throw error("no CUDA device available");
  return ozaki_selftest(n, k);
}

}  // namespace gb300
