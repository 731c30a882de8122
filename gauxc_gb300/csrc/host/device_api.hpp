// Host-visible interface of the device modules (no CUDA types here, so the
// C API layer compiles as plain C++).
#pragma once
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "core.hpp"

namespace gb300 {

struct XCFunctionalDesc;  // functionals.cuh

// Device memory policy: either a caller-provided buffer (bump-allocated, never
// freed) or cudaMalloc bounded by fill_fraction of the free memory.
struct RuntimeEnv {
  bool device = false;
  double fill_fraction = 0.9;
  void* user_mem = nullptr;
  size_t user_bytes = 0;
  size_t user_used = 0;
};

enum class Precision : int { FP64 = 0, Mixed = 1 };

struct PlanStats {
  int64_t ntasks = 0, npts = 0, npts_pad = 0, nbatches = 0;
  double sum_npts_nbe = 0., sum_npts_nbe2 = 0., sum_pad_npts_nbe2 = 0.;
  double scratch_bytes = 0.;
  int64_t gpu_launches = 0;
  double tensor_flops_x = 0., tensor_flops_v = 0.;  // BF16 MMA flops per call (mixed path)
};

class DeviceIntegrator;

struct XCIntegratorHandle {
  std::shared_ptr<LoadBalancer> lb;
  std::shared_ptr<XCFunctionalDesc> func;
  std::shared_ptr<RuntimeEnv> rt;
  Precision prec = Precision::FP64;
  std::shared_ptr<DeviceIntegrator> dev;
  double last_exc = 0., last_nel = 0.;
  bool profiling = false;
};

// eval_exc_vxc for RKS; VXC may be null (EXC only).  Throws gb300::error.
void integrator_eval_exc_vxc(XCIntegratorHandle& h, int64_t m, int64_t n, const double* P,
                             int64_t ldp, double* VXC, int64_t ldvxc, double* EXC);
void integrator_integrate_den(XCIntegratorHandle& h, int64_t m, int64_t n, const double* P,
                              int64_t ldp, double* NEL);
std::map<std::string, double> integrator_timings(const XCIntegratorHandle& h);
PlanStats integrator_plan_stats(XCIntegratorHandle& h);
// Per-kernel-class CUDA-event timing of every launch (collocation, density,
// zmat, vxc, other): {ms, launches} pairs of the last call.
void integrator_set_profiling(XCIntegratorHandle& h, bool on);
std::vector<double> integrator_kernel_times(const XCIntegratorHandle& h);

// FP64 FMA throughput probe (TFLOP/s) on the current device.
double measure_fp64_peak();
// Tensor-core emulated-FP64 GEMM self-test: worst relative error.
double tensor_core_selftest(int n, int k);
void set_device(int dev);

// SSF weights on the device for every task of the load balancer.
void molecular_weights_ssf_device(LoadBalancer& lb, RuntimeEnv& rt);

// SSF weights on caller-owned device arrays with the work space in a fixed
// file-scope device array (no allocation); see ssf_noalloc.cu for the limits.
void ssf_weights_noalloc(int64_t npts, int natoms, const double* x, const double* y,
                         const double* z, const int32_t* iparent, const double* dist_nearest,
                         const double* coords, double* weights, void* stream);

// Stage-level entry points (host arrays in and out, device compute).
void ssf_weights_device(int64_t npts, int natoms, const double* points, const int32_t* iparent,
                        const double* dist_nearest, const double* coords, double* weights);
void collocation_device(const BasisSet& basis, int64_t npts, const double* points, int nshells,
                        const int32_t* shell_list, bool grad, double* phi, double* dphi_x,
                        double* dphi_y, double* dphi_z);

std::shared_ptr<XCFunctionalDesc> make_functional(const std::string& name);
bool functional_is_gga(const XCFunctionalDesc& f);

int cuda_device_count();

}  // namespace gb300
