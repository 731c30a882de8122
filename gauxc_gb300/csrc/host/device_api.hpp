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
  // Algorithmic bytes per call of each kernel class (collocation, density,
  // zmat / Z digits, vxc, other, phi digits, P digits): every operand read
  // once and every result written once, at the sizes the plan runs
  double kbytes[7] = {0, 0, 0, 0, 0, 0, 0};
};

// Tunable parameters of the tensor-core plan (point blocks).
struct PlanParams {
  int pb_max_pts = 384;       // points per point block (multiple of 64, <= 384)
  double nu2_weight = 100.;   // merge-rule cost of one union-basis element squared
                              // (gather / scatter work per block), in tile MACs
  double scratch_bytes = 0.;  // cap of the per-pass work space (0 = from free memory);
                              // a plan that needs more runs in several passes
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
  PlanParams params;
  // bound of the tensor-core pipeline waits (ns) and the error-path check
  // (integrator_set_pipeline_check)
  uint64_t wait_ns = 1000000000ull;
  bool withhold = false;
};

// eval_exc_vxc for RKS; VXC may be null (EXC only).  Throws gb300::error.
void integrator_eval_exc_vxc(XCIntegratorHandle& h, int64_t m, int64_t n, const double* P,
                             int64_t ldp, double* VXC, int64_t ldvxc, double* EXC);
void integrator_integrate_den(XCIntegratorHandle& h, int64_t m, int64_t n, const double* P,
                              int64_t ldp, double* NEL);
// UKS: Ps = P_a + P_b, Pz = P_a - P_b; VXC_s and VXC_z both given, or both null
// (EXC only).  Needs a polarized functional.  Throws gb300::error.
void integrator_eval_exc_vxc_uks(XCIntegratorHandle& h, int64_t m, int64_t n, const double* Ps,
                                 int64_t ldps, const double* Pz, int64_t ldpz, double* VXCs,
                                 int64_t ldvs, double* VXCz, int64_t ldvz, double* EXC);
std::map<std::string, double> integrator_timings(const XCIntegratorHandle& h);
PlanStats integrator_plan_stats(XCIntegratorHandle& h);
// Per-kernel-class CUDA-event timing of every launch (collocation, density,
// zmat, vxc, other): {ms, launches} pairs of the last call.
void integrator_set_profiling(XCIntegratorHandle& h, bool on);
std::vector<double> integrator_kernel_times(const XCIntegratorHandle& h);
// Bound of every tensor-core pipeline wait of the following calls, and the
// check of their error path: with withhold set, the GEMM producers issue no
// copy, each consumer's first wait runs out after wait_ms and the call fails
// with the pipeline error; the context stays usable.
void integrator_set_pipeline_check(XCIntegratorHandle& h, double wait_ms, bool withhold);
// Sets the tensor-core plan parameters; the plan is rebuilt on the next call.
void integrator_set_plan_params(XCIntegratorHandle& h, const PlanParams& p);
// Times one call for each candidate plan (point-block sizes x merge weights)
// on density P and keeps the fastest; returns its compute time in ms and
// writes the chosen parameters to *best.
double integrator_autotune(XCIntegratorHandle& h, const double* P, int64_t ldp, PlanParams* best);

// Many integrators evaluated by one CUDA-graph launch per call.
class IntegratorBatch;
std::shared_ptr<IntegratorBatch> batch_new(const std::vector<XCIntegratorHandle*>& hs);
// EXC[i] for every member; VXC[i] may be null (EXC only).  Host buffers are
// page-locked in place (cudaHostRegister) and stay registered until the
// batch is destroyed or other buffers are passed.
void batch_eval_exc_vxc(IntegratorBatch& b, const double* const* P, const int64_t* ldp,
                        double* const* VXC, const int64_t* ldvxc, double* EXC);
std::map<std::string, double> batch_timings(const IntegratorBatch& b);

// FP64 FMA throughput probe (TFLOP/s) on the current device.
double measure_fp64_peak();
// Page-locks caller host memory in place (cudaHostRegister); false when it
// already is page-locked (nothing done).  host_unregister undoes it.
bool host_register(void* p, size_t bytes);
void host_unregister(void* p);
// Tensor-core emulated-FP64 GEMM self-test: worst relative error.
double tensor_core_selftest(int n, int k);
// Largest relative error of the float-float exp of the collocation over n
// points of [-50, 0] against FP64 exp.
double ff_exp_selftest(int n);
void set_device(int dev);

// Collision bitset of task boxes (6 doubles each: lo xyz, up xyz) against the
// shells' cutoff spheres on the device: bit s % 32 of bits[i * nwords + s / 32]
// is set when shell s survives the cube/sphere test for box i.
void screen_boxes_device(const std::vector<double>& boxes, const BasisSet& bs,
                         std::vector<uint32_t>& bits, int& nwords);

// Stage-level local work driver (lwd.cu): one device-data object over tasks
// [t0, t1) of a weighted load balancer, and the reference's stages on it.
class LWDData;
std::shared_ptr<LWDData> lwd_create(const LoadBalancer& lb, int64_t t0, int64_t t1);
void lwd_eval_collocation(LWDData& d, bool grad);
void lwd_eval_xmat(LWDData& d, double fac, const double* P, int64_t ldp);
void lwd_eval_vvars(LWDData& d, bool gga);
void lwd_eval_uvars(LWDData& d);
void lwd_eval_kern_exc_vxc(LWDData& d, const XCFunctionalDesc& f);
void lwd_inc_exc(LWDData& d);
void lwd_inc_nel(LWDData& d);
void lwd_eval_zmat_vxc(LWDData& d, bool gga);
void lwd_inc_vxc(LWDData& d);
void lwd_symmetrize_vxc(LWDData& d, double* VXC, int64_t ld);
void lwd_results(LWDData& d, double* exc, double* nel);

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

std::shared_ptr<XCFunctionalDesc> make_functional(const std::string& name, bool polarized = false);
bool functional_is_gga(const XCFunctionalDesc& f);

int cuda_device_count();

}  // namespace gb300
