/*
 * gauxc_gb300 -- C ABI of the GB300 device XC integrator.
 *
 * The first part mirrors the reference C API for the device XC-integration
 * path: same type names, handle layout ({header, pointer}), function names,
 * argument order and error behaviour (every call takes a GauXCStatus*; on
 * failure status->code is non-zero and status->message holds a malloc'd
 * string that gauxc_status_delete frees).  A code written against the
 * reference headers (include/gauxc/c/ *.h) links against this library for the
 * functions below.  Each declaration cites the reference declaration it
 * replaces.
 *
 * The second part (gauxc_gb300_*) holds extensions of this library: plan
 * statistics, per-call timings, N_el of the last call, and stage-level entry
 * points (SSF weights, collocation) that the parity tests call directly.
 *
 * Supported: RKS and UKS, LDA/GGA functionals SVWN5, PBE, revPBE, PBE0 (semilocal part),
 * Mura-Knowles radial grids with Lebedev angular grids (unpruned, Robust and
 * Treutler pruning), SSF partition weights on the device, shells with l <= 4.
 */
#ifndef GAUXC_GB300_H
#define GAUXC_GB300_H

#ifdef __cplusplus
#include <cstddef>
#include <cstdint>
extern "C" {
#else
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#endif

/* ------------------------------------------------------------------ types */

/* include/gauxc/c/status.h:24 */
typedef struct GauXCStatus {
  int code;
  char* message;
} GauXCStatus;

/* include/gauxc/c/types.h:26 */
enum GauXC_Type {
  GauXC_Type_Molecule = 1,
  GauXC_Type_BasisSet = 2,
  GauXC_Type_MolGrid = 3,
  GauXC_Type_RuntimeEnvironment = 4,
  GauXC_Type_LoadBalancer = 5,
  GauXC_Type_LoadBalancerFactory = 6,
  GauXC_Type_MolecularWeights = 7,
  GauXC_Type_MolecularWeightsFactory = 8,
  GauXC_Type_Functional = 9,
  GauXC_Type_Integrator = 10,
  /* extension: handle of a batch of integrators (gauxc_gb300_batch_new) */
  GauXC_Type_GB300Batch = 64,
  /* extension: device data of the stage-level work driver (gauxc_gb300_lwd_*) */
  GauXC_Type_GB300DeviceData = 65
};

/* include/gauxc/c/types.h:42 */
typedef struct GauXCHeader {
  enum GauXC_Type type;
} GauXCHeader;

/* include/gauxc/c/enums.h */
enum GauXC_RadialQuad {
  GauXC_RadialQuad_Becke,
  GauXC_RadialQuad_MuraKnowles,
  GauXC_RadialQuad_MurrayHandyLaming,
  GauXC_RadialQuad_TreutlerAhlrichs
};
enum GauXC_AtomicGridSizeDefault {
  GauXC_AtomicGridSizeDefault_FineGrid,
  GauXC_AtomicGridSizeDefault_UltraFineGrid,
  GauXC_AtomicGridSizeDefault_SuperFineGrid,
  GauXC_AtomicGridSizeDefault_GM3,
  GauXC_AtomicGridSizeDefault_GM5
};
enum GauXC_XCWeightAlg {
  GauXC_XCWeightAlg_NOTPARTITIONED,
  GauXC_XCWeightAlg_Becke,
  GauXC_XCWeightAlg_SSF,
  GauXC_XCWeightAlg_LKO
};
enum GauXC_ExecutionSpace { GauXC_ExecutionSpace_Host, GauXC_ExecutionSpace_Device };
enum GauXC_PruningScheme {
  GauXC_PruningScheme_Unpruned,
  GauXC_PruningScheme_Robust,
  GauXC_PruningScheme_Treutler
};

/* include/gauxc/c/functional.h:22-60 (subset; values keep the reference order) */
enum GauXC_Functional {
  GauXC_Functional_SVWN3,
  GauXC_Functional_SVWN5,
  GauXC_Functional_BLYP,
  GauXC_Functional_B3LYP,
  GauXC_Functional_PBE,
  GauXC_Functional_revPBE,
  GauXC_Functional_PBE0
};

/* include/gauxc/c/atom.h:32 */
typedef struct GauXCAtom {
  int64_t Z;
  double x, y, z; /* bohr */
} GauXCAtom;

/* include/gauxc/c/shell.h:30 */
typedef struct GauXCShell {
  int32_t l;
  bool pure;
  int32_t nprim;
  double exponents[32];
  double coefficients[32];
  double origin[3];
  double shell_tolerance;
} GauXCShell;

/* handle types: include/gauxc/c/{molecule,basisset,molgrid,runtime_environment,
   load_balancer,molecular_weights,functional,xc_integrator}.h */
typedef struct GauXCMolecule { GauXCHeader hdr; void* ptr; } GauXCMolecule;
typedef struct GauXCBasisSet { GauXCHeader hdr; void* ptr; } GauXCBasisSet;
typedef struct GauXCMolGrid { GauXCHeader hdr; void* ptr; } GauXCMolGrid;
typedef struct GauXCRuntimeEnvironment { GauXCHeader hdr; void* ptr; void* device_ptr; } GauXCRuntimeEnvironment;
typedef struct GauXCLoadBalancer { GauXCHeader hdr; void* ptr; } GauXCLoadBalancer;
typedef struct GauXCLoadBalancerFactory { GauXCHeader hdr; void* ptr; } GauXCLoadBalancerFactory;
typedef struct GauXCMolecularWeights { GauXCHeader hdr; void* ptr; } GauXCMolecularWeights;
typedef struct GauXCMolecularWeightsFactory { GauXCHeader hdr; void* ptr; } GauXCMolecularWeightsFactory;
typedef struct GauXCFunctional { GauXCHeader hdr; void* ptr; } GauXCFunctional;
typedef struct GauXCIntegrator { GauXCHeader hdr; void* ptr; } GauXCIntegrator;
/* extension: many integrators evaluated by one CUDA-graph launch */
typedef struct GauXCGB300Batch { GauXCHeader hdr; void* ptr; } GauXCGB300Batch;
/* extension: device data of the stage-level work driver */
typedef struct GauXCGB300DeviceData { GauXCHeader hdr; void* ptr; } GauXCGB300DeviceData;

/* include/gauxc/c/molecular_weights.h:34 */
typedef struct GauXCMolecularWeightsSettings {
  enum GauXC_XCWeightAlg weight_alg;
  bool becke_size_adjustment;
} GauXCMolecularWeightsSettings;

/* ------------------------------------------------------------------ reference C API */

void gauxc_status_delete(GauXCStatus* status);                                   /* status.h:33 */
void gauxc_object_delete(GauXCStatus* status, void** handle);                    /* types.h:55 */

GauXCMolecule gauxc_molecule_new(GauXCStatus* status);                           /* molecule.h:45 */
GauXCMolecule gauxc_molecule_new_from_atoms(GauXCStatus* status, const GauXCAtom* atoms,
                                            size_t natoms);                      /* molecule.h:54 */
void gauxc_molecule_delete(GauXCStatus* status, GauXCMolecule* mol);             /* molecule.h:61 */
size_t gauxc_molecule_natoms(GauXCStatus* status, const GauXCMolecule mol);      /* molecule.h:69 */

GauXCBasisSet gauxc_basisset_new(GauXCStatus* status);                           /* basisset.h:45 */
GauXCBasisSet gauxc_basisset_new_from_shells(GauXCStatus* status, const GauXCShell* shells,
                                             size_t nshells, bool normalize);    /* basisset.h:55 */
void gauxc_basisset_delete(GauXCStatus* status, GauXCBasisSet* basis);           /* basisset.h:67 */

GauXCMolGrid gauxc_molgrid_new_default(GauXCStatus* status, const GauXCMolecule mol,
                                       enum GauXC_PruningScheme pruning_scheme,
                                       int64_t batchsize,
                                       enum GauXC_RadialQuad radial_quad,
                                       enum GauXC_AtomicGridSizeDefault grid_size); /* molgrid.h:47 */
void gauxc_molgrid_delete(GauXCStatus* status, GauXCMolGrid* molgrid);           /* molgrid.h:61 */

GauXCRuntimeEnvironment gauxc_runtime_environment_new(GauXCStatus* status);      /* runtime_environment.h:45 */
GauXCRuntimeEnvironment gauxc_device_runtime_environment_new(GauXCStatus* status,
                                                             double fill_fraction); /* runtime_environment.h:89 */
GauXCRuntimeEnvironment gauxc_device_runtime_environment_new_mem(GauXCStatus* status, void* mem,
                                                                 size_t mem_sz); /* runtime_environment.h:103 */
void gauxc_runtime_environment_delete(GauXCStatus* status, GauXCRuntimeEnvironment* env); /* runtime_environment.h:55 */
int gauxc_runtime_environment_comm_rank(GauXCStatus* status, const GauXCRuntimeEnvironment env); /* runtime_environment.h:66 */
int gauxc_runtime_environment_comm_size(GauXCStatus* status, const GauXCRuntimeEnvironment env); /* runtime_environment.h:76 */

GauXCLoadBalancerFactory gauxc_load_balancer_factory_new(GauXCStatus* status,
                                                         enum GauXC_ExecutionSpace ex,
                                                         const char* kernel_name); /* load_balancer.h:69 */
void gauxc_load_balancer_factory_delete(GauXCStatus* status, GauXCLoadBalancerFactory* f); /* load_balancer.h:80 */
GauXCLoadBalancer gauxc_load_balancer_factory_get_instance(
    GauXCStatus* status, const GauXCLoadBalancerFactory factory,
    const GauXCRuntimeEnvironment env, const GauXCMolecule mol, const GauXCMolGrid mg,
    const GauXCBasisSet basis);                                                   /* load_balancer.h:95 */
void gauxc_load_balancer_delete(GauXCStatus* status, GauXCLoadBalancer* lb);     /* load_balancer.h:49 */

GauXCMolecularWeightsFactory gauxc_molecular_weights_factory_new(
    GauXCStatus* status, enum GauXC_ExecutionSpace ex, const char* local_work_kernel_name,
    GauXCMolecularWeightsSettings settings);                                      /* molecular_weights.h:85 */
void gauxc_molecular_weights_factory_delete(GauXCStatus* status,
                                            GauXCMolecularWeightsFactory* factory); /* molecular_weights.h:97 */
GauXCMolecularWeights gauxc_molecular_weights_factory_get_instance(
    GauXCStatus* status, const GauXCMolecularWeightsFactory factory);             /* molecular_weights.h:108 */
void gauxc_molecular_weights_modify_weights(GauXCStatus* status, const GauXCMolecularWeights mw,
                                            const GauXCLoadBalancer lb);          /* molecular_weights.h:63 */
void gauxc_molecular_weights_delete(GauXCStatus* status, GauXCMolecularWeights* mw); /* molecular_weights.h:52 */

GauXCFunctional gauxc_functional_from_string(GauXCStatus* status, const char* functional_spec,
                                             bool polarized);                    /* functional.h:359 */
GauXCFunctional gauxc_functional_from_enum(GauXCStatus* status,
                                           enum GauXC_Functional functional_type,
                                           bool polarized);                      /* functional.h:372 */
void gauxc_functional_delete(GauXCStatus* status, GauXCFunctional* functional);  /* functional.h:383 */

GauXCIntegrator gauxc_integrator_new(GauXCStatus* status, const GauXCFunctional functional,
                                     const GauXCLoadBalancer lb,
                                     enum GauXC_ExecutionSpace execution_space,
                                     const char* integrator_input_type,
                                     const char* integrator_kernel_name,
                                     const char* local_work_kernel_name,
                                     const char* reduction_kernel_name);         /* xc_integrator.h:61 */
void gauxc_integrator_delete(GauXCStatus* status, GauXCIntegrator* integrator);  /* xc_integrator.h:44 */
void gauxc_integrator_integrate_den(GauXCStatus* status, const GauXCIntegrator integrator,
                                    const int64_t m, const int64_t n,
                                    const double* density_matrix, const int64_t ldp,
                                    double* den);                                 /* xc_integrator.h:82 */
void gauxc_integrator_eval_exc_rks(GauXCStatus* status, const GauXCIntegrator integrator,
                                   const int64_t m, const int64_t n,
                                   const double* density_matrix, const int64_t ldp,
                                   double* exc);                                  /* xc_integrator.h:102 */
void gauxc_integrator_eval_exc_vxc_rks(GauXCStatus* status, const GauXCIntegrator integrator,
                                       const int64_t m, const int64_t n,
                                       const double* density_matrix, const int64_t ldp,
                                       double* exc, double* vxc_matrix,
                                       const int64_t vxc_ld);                     /* xc_integrator.h:180 */

/* UKS: density_matrix_s = P_alpha + P_beta, density_matrix_z = P_alpha - P_beta;
   needs a functional made with polarized = true. */
void gauxc_integrator_eval_exc_uks(GauXCStatus* status, const GauXCIntegrator integrator,
                                   const int64_t m, const int64_t n,
                                   const double* density_matrix_s, const int64_t ldp_s,
                                   const double* density_matrix_z, const int64_t ldp_z,
                                   double* exc);                                  /* xc_integrator.h:124 */
void gauxc_integrator_eval_exc_vxc_uks(GauXCStatus* status, const GauXCIntegrator integrator,
                                       const int64_t m, const int64_t n,
                                       const double* density_matrix_s, const int64_t ldp_s,
                                       const double* density_matrix_z, const int64_t ldp_z,
                                       double* exc, double* vxc_matrix_s, const int64_t vxc_ld_s,
                                       double* vxc_matrix_z,
                                       const int64_t vxc_ld_z);                   /* xc_integrator.h:208 */

/* ------------------------------------------------------------------ extensions */

/* Library version string (static storage). */
const char* gauxc_gb300_version(void);
/* Number of CUDA devices visible (0 on a machine without GPU). */
int gauxc_gb300_device_count(void);

size_t gauxc_gb300_basisset_nshells(GauXCStatus* status, const GauXCBasisSet basis);
int32_t gauxc_gb300_basisset_nbf(GauXCStatus* status, const GauXCBasisSet basis);
/* Shell i after normalization; shell_tolerance holds the tolerance, *cutoff the radius. */
void gauxc_gb300_basisset_get_shell(GauXCStatus* status, const GauXCBasisSet basis, size_t i,
                                    GauXCShell* out, double* cutoff_radius);
/* Reset the screening tolerance of every shell (recomputes cutoff radii). */
void gauxc_gb300_basisset_set_tolerance(GauXCStatus* status, GauXCBasisSet basis, double tol);

/* Atomic grid of element Z (origin-centred, batch order). Pass null arrays to query sizes. */
void gauxc_gb300_molgrid_atomic_grid(GauXCStatus* status, const GauXCMolGrid mg, int64_t Z,
                                     int64_t* npts, int64_t* nbatches, double* points,
                                     double* weights, int64_t* batch_ranges);

size_t gauxc_gb300_load_balancer_ntasks(GauXCStatus* status, const GauXCLoadBalancer lb);
/* info = {iParent, npts, nbe, nshells}; *dist_nearest of the task's parent atom. */
void gauxc_gb300_load_balancer_task_info(GauXCStatus* status, const GauXCLoadBalancer lb,
                                         size_t i, int32_t info[4], double* dist_nearest);
/* points (3*npts, xyz interleaved), weights (npts), shell_list (nshells); any may be null. */
void gauxc_gb300_load_balancer_task_data(GauXCStatus* status, const GauXCLoadBalancer lb,
                                         size_t i, double* points, double* weights,
                                         int32_t* shell_list);
bool gauxc_gb300_load_balancer_weights_modified(GauXCStatus* status, const GauXCLoadBalancer lb);
/* A new load balancer over the tasks task_idx[0..n) of lb (in that order):
   same molecule, basis, grid and runtime environment, copies of the tasks with
   their current weights and weights-modified state.  Used to evaluate a
   sample of a large system's tasks (parity checks and CPU timing samples).
   No counterpart in the reference. */
GauXCLoadBalancer gauxc_gb300_load_balancer_subset(GauXCStatus* status, const GauXCLoadBalancer lb,
                                                   const int64_t* task_idx, size_t n);

/* N_el (integral of the total density) of the last eval_exc_vxc call. */
double gauxc_gb300_integrator_last_nel(GauXCStatus* status, const GauXCIntegrator integrator);
/* Timings in ms: {h2d, compute, d2h, wall} of the last call, then the
   device plan's host build {total, merge of tasks into point blocks, layout,
   work lists and uploads} (the plan is built by the first call after the
   load balancer's weights change); returns the count written (<= 8). */
int gauxc_gb300_integrator_timings(GauXCStatus* status, const GauXCIntegrator integrator,
                                   double* out, int nmax);
/* Plan statistics: {ntasks, npts, npts_pad, nbatches, sum npts*nbe, sum npts*nbe^2,
   sum npts_pad*nbe_pad^2, scratch bytes, kernel launches of the last call,
   BF16 tensor FLOPs per call of the density and of the VXC GEMMs (mixed path),
   algorithmic bytes per call of the kernel classes collocation, density,
   zmat (Z digits), vxc, other, phi digits, P digits (each operand read once,
   each result written once)}; returns the count written (at most 18). */
int gauxc_gb300_integrator_plan_stats(GauXCStatus* status, const GauXCIntegrator integrator,
                                      double* out, int nmax);

/* Per-kernel-class CUDA-event timing of each launch of the following calls
   (adds two events per launch on the integrator's stream). */
void gauxc_gb300_integrator_set_profiling(GauXCStatus* status, const GauXCIntegrator integrator,
                                          bool on);
/* {collocation ms, launches, density ms, launches, zmat ms, launches, vxc ms,
   launches, other ms, launches, phi digits ms, launches, P digits ms, launches}
   of the last call (at most nmax values); returns the count written. */
int gauxc_gb300_integrator_kernel_times(GauXCStatus* status, const GauXCIntegrator integrator,
                                        double* out, int nmax);
/* Bound (ms, default 1000) of every wait of the tensor-core pipeline in the
   following calls of a "GB300-Mixed" integrator, and the check of its error
   path: with withhold set, the GEMM producers issue no copy at all, the first
   wait of each consumer runs out after wait_ms with nothing in flight, and the
   call fails with "a tensor-core pipeline wait expired"; the CUDA context stays
   usable and a later call with withhold cleared runs normally.  No counterpart
   in the reference (its device integrator has no bounded waits). */
void gauxc_gb300_integrator_set_pipeline_check(GauXCStatus* status,
                                               const GauXCIntegrator integrator, double wait_ms,
                                               bool withhold);
/* Measured FP64 FMA throughput of the current device in TFLOP/s (about 50 ms probe). */
double gauxc_gb300_measure_fp64_peak(GauXCStatus* status);
/* Page-lock caller host memory in place (P / VXC buffers reused every SCF
   iteration) so that the copies of eval_* run at page-locked bandwidth.
   Returns 1 when it registered the range, 0 when it already was page-locked.
   The memory must stay allocated until gauxc_gb300_host_unregister. */
int gauxc_gb300_host_register(GauXCStatus* status, void* ptr, size_t bytes);
void gauxc_gb300_host_unregister(GauXCStatus* status, void* ptr);
/* Self-test of the tensor-core (split-mantissa BF16) VXC GEMM: the symmetric
   n x n product F Z^T + Z F^T over k points (n multiple of 128, k multiple of
   64, k <= 384) against FP64; returns the worst error relative to the largest
   output element. */
double gauxc_gb300_tensor_core_selftest(GauXCStatus* status, int n, int k);
/* Self-test of the float-float exp of the tensor-core path's collocation:
   the largest relative error against FP64 exp over n points of [-50, 0]. */
double gauxc_gb300_ff_exp_selftest(GauXCStatus* status, int n);
/* cudaSetDevice for the calling thread (one process per GPU). */
void gauxc_gb300_set_device(GauXCStatus* status, int device);

/* Stage entry points (host arrays, computed on the device).
   SSF weights, reference kernel cuda_ssf_1d.cu:24-144 (partition_weights_ssf_1d). */
void gauxc_gb300_ssf_weights(GauXCStatus* status, int64_t npts, int32_t natoms,
                             const double* points, const int32_t* iparent,
                             const double* dist_nearest, const double* coords,
                             double* weights);
/* SSF weights for callers that cannot allocate device memory (a host code whose
   own pool already reserved the GPU, or a loop that must not pay for allocator
   synchronization).  No counterpart in the reference.  Every pointer is a
   device pointer owned by the caller: x, y, z, iparent (values in [0, natoms)),
   dist_nearest and weights hold npts entries, coords 3*natoms (xyz
   interleaved); weights are modified in place, work is queued on `stream`
   (a cudaStream_t; NULL = default stream) and the call returns without
   synchronizing.  The work space is one fixed array of 4 Mi doubles (32 MiB)
   inside the library, kept by every GPU that loads it until exit:
   natoms*npts + natoms*natoms must not exceed 4194304 (larger requests are
   rejected; split the points).  All calls share that array, so calls that
   overlap on the GPU race.  Each call looks the array's address up on the
   current device; the first call on a device also loads the library's device
   code there and should come before any stream capture.  A point whose parent
   index lies outside [0, natoms) keeps its weight.  Nothing is allocated or
   freed. */
void gauxc_gb300_ssf_weights_noalloc(GauXCStatus* status, int64_t npts, int32_t natoms,
                                     const double* x, const double* y, const double* z,
                                     const int32_t* iparent, const double* dist_nearest,
                                     const double* coords, double* weights, void* stream);
/* Collocation of the listed shells, host layout eval[ipt*nbe + ibf]; gradients
   when dphi_* are non-null.  Reference: collocation_device.cu (eval_collocation*). */
void gauxc_gb300_collocation(GauXCStatus* status, const GauXCBasisSet basis, int64_t npts,
                             const double* points, int32_t nshells, const int32_t* shell_list,
                             double* phi, double* dphi_x, double* dphi_y, double* dphi_z);

/* ---- batched evaluation and plan tuning (no counterpart in the reference;
   the per-member work is gauxc_integrator_eval_exc_vxc_rks, xc_integrator.h:180) */

/* Plan parameters: points per point block of a "GB300-Mixed" integrator
   (multiple of 64, 64..384), the weight of a block's union-basis gather and
   scatter work in the block-merge rule, and a cap (GB, 0 = from free memory)
   on the device work space of one pass over the grid; a plan needing more
   runs in several passes.  The plan is rebuilt on the next call. */
void gauxc_gb300_integrator_set_plan_params(GauXCStatus* status, const GauXCIntegrator integrator,
                                            int pb_max_pts, double nu2_weight, double scratch_gb);
/* Autotuner: builds and times one call per candidate plan (point-block sizes
   128/256/384 x merge weights 75/150 for "GB300-Mixed"; the current plan
   otherwise) on density P and keeps the fastest.  Returns its compute time in
   ms and the chosen parameters. */
double gauxc_gb300_integrator_autotune(GauXCStatus* status, const GauXCIntegrator integrator,
                                       int64_t m, int64_t n, const double* P, int64_t ldp,
                                       int* pb_max_pts, double* nu2_weight);
/* A batch over n integrators (any mix of molecules, functionals and
   precisions).  gauxc_gb300_batch_eval_exc_vxc_rks evaluates every member:
   P[i] (nbf_i x nbf_i, ld ldp[i]) in, EXC[i] and VXC[i] (ld ldvxc[i]; NULL =
   EXC only) out.  The first call with a given set of buffers runs the members
   one by one and captures a CUDA graph of all of them (H2D, kernels, D2H on
   one stream per member, forked from and joined into one root stream); later
   calls with the same buffers are a single graph launch.  Members without a
   work-space cap (gauxc_gb300_integrator_set_plan_params) get an equal share
   of the device memory free when the batch is created.  The buffers are
   page-locked in place (cudaHostRegister) until the batch is deleted or other
   buffers are passed; they must stay valid meanwhile.  Members must not be
   evaluated concurrently from other threads. */
GauXCGB300Batch gauxc_gb300_batch_new(GauXCStatus* status, const GauXCIntegrator* integrators,
                                      int32_t n);
void gauxc_gb300_batch_eval_exc_vxc_rks(GauXCStatus* status, const GauXCGB300Batch batch,
                                        const double* const* P, const int64_t* ldp,
                                        double* const* VXC, const int64_t* ldvxc, double* EXC);
/* {compute_ms (graph, CUDA events), wall_ms, graph_launch (0/1), members,
   gpu_launches} of the last call; returns the count written. */
int gauxc_gb300_batch_timings(GauXCStatus* status, const GauXCGB300Batch batch, double* out,
                              int nmax);
void gauxc_gb300_batch_delete(GauXCStatus* status, GauXCGB300Batch* batch);

/* ---- stage-level local work driver
   The stages of the reference's LocalDeviceWorkDriver
   (src/xc_integrator/local_work_driver/device/local_device_work_driver.hpp:62-127)
   on a device-data object (XCDeviceData, xc_device_data.hpp:668-787) that holds
   tasks [task_begin, task_end) of a load balancer with modified weights, all
   in FP64 with every intermediate kept on the device.  One SCF evaluation, in
   the reference integrator's order
   (incore_replicated_xc_device_integrator_exc_vxc.hpp:283-404):
     eval_collocation (gradient for GGA), eval_xmat (fac = 2 for an RKS alpha
     density), eval_vvars (gga), eval_uvars (GGA), eval_kern_exc_vxc, inc_exc,
     inc_nel, eval_zmat_vxc (gga), inc_vxc, symmetrize_vxc, results.
   EXC, N_el and VXC accumulate over the calls until the object is deleted. */
GauXCGB300DeviceData gauxc_gb300_lwd_device_data_new(GauXCStatus* status,
                                                     const GauXCLoadBalancer lb,
                                                     int64_t task_begin, int64_t task_end);
void gauxc_gb300_lwd_device_data_delete(GauXCStatus* status, GauXCGB300DeviceData* data);
void gauxc_gb300_lwd_eval_collocation(GauXCStatus* status, const GauXCGB300DeviceData data,
                                      bool gradient);
/* X = fac * P_sub * phi, P column-major nbf x nbf (host, leading dimension ldp) */
void gauxc_gb300_lwd_eval_xmat(GauXCStatus* status, const GauXCGB300DeviceData data, double fac,
                               const double* P, int64_t ldp);
void gauxc_gb300_lwd_eval_vvars(GauXCStatus* status, const GauXCGB300DeviceData data, bool gga);
void gauxc_gb300_lwd_eval_uvars(GauXCStatus* status, const GauXCGB300DeviceData data);
void gauxc_gb300_lwd_eval_kern_exc_vxc(GauXCStatus* status, const GauXCGB300DeviceData data,
                                       const GauXCFunctional functional);
void gauxc_gb300_lwd_inc_exc(GauXCStatus* status, const GauXCGB300DeviceData data);
void gauxc_gb300_lwd_inc_nel(GauXCStatus* status, const GauXCGB300DeviceData data);
void gauxc_gb300_lwd_eval_zmat_vxc(GauXCStatus* status, const GauXCGB300DeviceData data, bool gga);
void gauxc_gb300_lwd_inc_vxc(GauXCStatus* status, const GauXCGB300DeviceData data);
/* VXC = A + A^T of the accumulated contributions into vxc (host, leading dimension ldvxc) */
void gauxc_gb300_lwd_symmetrize_vxc(GauXCStatus* status, const GauXCGB300DeviceData data,
                                    double* vxc, int64_t ldvxc);
void gauxc_gb300_lwd_results(GauXCStatus* status, const GauXCGB300DeviceData data, double* exc,
                             double* nel);

#ifdef __cplusplus
}
#endif
#endif /* GAUXC_GB300_H */
