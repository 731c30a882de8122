// extern "C" layer: the reference C API for the device XC path
// (src/c-api/*.cxx) plus the gauxc_gb300_* extensions.  Error behaviour
// follows src/c-api/c_status.hpp:12-44: a call first resets the status
// (freeing an old message) and failures set code = 1 and a malloc'd message.
// A caller that passes a null status gets the failure as a C++ exception
// (gb300::error, a std::runtime_error), as the reference throws
// GAUXC_GENERIC_EXCEPTION in that case; with a status, no exception crosses
// the C boundary.
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

#include "../../../include/gauxc_gb300.h"
#include "core.hpp"
#include "device_api.hpp"

using namespace gb300;

namespace {

void status_init(GauXCStatus* st) {
  if (!st) return;
  st->code = 0;
  std::free(st->message);
  st->message = nullptr;
}

void status_fail(GauXCStatus* st, const char* msg) {
  if (!st) throw gb300::error(msg);
  st->code = 1;
  std::free(st->message);
  const size_t n = std::strlen(msg) + 1;
  st->message = static_cast<char*>(std::malloc(n));
  std::memcpy(st->message, msg, n);
}

template <typename F>
void guarded(GauXCStatus* st, F&& f) {
  try {
    f();
  } catch (const std::exception& e) {
    status_fail(st, e.what());
  } catch (...) {
    status_fail(st, "unknown error");
  }
}

template <typename T>
std::shared_ptr<T>& deref(void* p) {
  return *static_cast<std::shared_ptr<T>*>(p);
}

template <typename H>
bool check(GauXCStatus* st, const H& h, GauXC_Type t, const char* what) {
  if (h.ptr == nullptr || h.hdr.type != t) {
    status_fail(st, (std::string("Invalid ") + what + " handle").c_str());
    return false;
  }
  return true;
}

template <typename H, typename T>
H make_handle(GauXC_Type t, std::shared_ptr<T> obj) {
  H h{};
  h.hdr.type = t;
  h.ptr = new std::shared_ptr<T>(std::move(obj));
  return h;
}

template <typename T, typename H>
void destroy(H* h) {
  if (h && h->ptr) {
    delete static_cast<std::shared_ptr<T>*>(h->ptr);
    h->ptr = nullptr;
  }
}

struct LBFactory {
  bool device;
  std::string kernel;
};
// A batch keeps its member integrators alive.
struct BatchHandle {
  std::vector<std::shared_ptr<XCIntegratorHandle>> members;
  std::shared_ptr<IntegratorBatch> batch;
};
struct MWFactory {
  bool device;
  GauXCMolecularWeightsSettings settings;
};
struct MolecularWeights {
  bool device;
  GauXCMolecularWeightsSettings settings;
};

bool iequals(const std::string& a, const char* b) {
  std::string x = a, y = b;
  for (auto& c : x) c = (char)std::toupper(c);
  for (auto& c : y) c = (char)std::toupper(c);
  return x == y;
}

}  // namespace

extern "C" {

void gauxc_status_delete(GauXCStatus* status) {
  if (!status) return;
  std::free(status->message);
  status->message = nullptr;
  status->code = 0;
}

void gauxc_object_delete(GauXCStatus* status, void** handle) {
  status_init(status);
  if (!handle || !*handle) return;
  auto* hdr = static_cast<GauXCHeader*>(*handle);
  switch (hdr->type) {
    case GauXC_Type_Molecule: gauxc_molecule_delete(status, (GauXCMolecule*)*handle); break;
    case GauXC_Type_BasisSet: gauxc_basisset_delete(status, (GauXCBasisSet*)*handle); break;
    case GauXC_Type_MolGrid: gauxc_molgrid_delete(status, (GauXCMolGrid*)*handle); break;
    case GauXC_Type_RuntimeEnvironment:
      gauxc_runtime_environment_delete(status, (GauXCRuntimeEnvironment*)*handle);
      break;
    case GauXC_Type_LoadBalancer: gauxc_load_balancer_delete(status, (GauXCLoadBalancer*)*handle); break;
    case GauXC_Type_LoadBalancerFactory:
      gauxc_load_balancer_factory_delete(status, (GauXCLoadBalancerFactory*)*handle);
      break;
    case GauXC_Type_MolecularWeights:
      gauxc_molecular_weights_delete(status, (GauXCMolecularWeights*)*handle);
      break;
    case GauXC_Type_MolecularWeightsFactory:
      gauxc_molecular_weights_factory_delete(status, (GauXCMolecularWeightsFactory*)*handle);
      break;
    case GauXC_Type_Functional: gauxc_functional_delete(status, (GauXCFunctional*)*handle); break;
    case GauXC_Type_Integrator: gauxc_integrator_delete(status, (GauXCIntegrator*)*handle); break;
    case GauXC_Type_GB300Batch: gauxc_gb300_batch_delete(status, (GauXCGB300Batch*)*handle); break;
    case GauXC_Type_GB300DeviceData:
      gauxc_gb300_lwd_device_data_delete(status, (GauXCGB300DeviceData*)*handle);
      break;
    default: status_fail(status, "unknown handle type");
  }
}

// ---------------------------------------------------------------- molecule
GauXCMolecule gauxc_molecule_new(GauXCStatus* status) {
  status_init(status);
  return make_handle<GauXCMolecule>(GauXC_Type_Molecule, std::make_shared<Molecule>());
}

GauXCMolecule gauxc_molecule_new_from_atoms(GauXCStatus* status, const GauXCAtom* atoms,
                                            size_t natoms) {
  status_init(status);
  GauXCMolecule h{};
  h.hdr.type = GauXC_Type_Molecule;
  if (natoms && !atoms) {
    status_fail(status, "atoms pointer cannot be null");
    return h;
  }
  guarded(status, [&] {
    auto m = std::make_shared<Molecule>();
    for (size_t i = 0; i < natoms; ++i) m->push_back({atoms[i].Z, atoms[i].x, atoms[i].y, atoms[i].z});
    h = make_handle<GauXCMolecule>(GauXC_Type_Molecule, m);
  });
  return h;
}

void gauxc_molecule_delete(GauXCStatus* status, GauXCMolecule* mol) {
  status_init(status);
  destroy<Molecule>(mol);
}

size_t gauxc_molecule_natoms(GauXCStatus* status, const GauXCMolecule mol) {
  status_init(status);
  if (!check(status, mol, GauXC_Type_Molecule, "Molecule")) return 0;
  return deref<Molecule>(mol.ptr)->size();
}

// ---------------------------------------------------------------- basis
GauXCBasisSet gauxc_basisset_new(GauXCStatus* status) {
  status_init(status);
  auto b = std::make_shared<BasisSet>();
  b->finalize();
  return make_handle<GauXCBasisSet>(GauXC_Type_BasisSet, b);
}

GauXCBasisSet gauxc_basisset_new_from_shells(GauXCStatus* status, const GauXCShell* shells,
                                             size_t nshells, bool normalize) {
  status_init(status);
  GauXCBasisSet h{};
  h.hdr.type = GauXC_Type_BasisSet;
  if (nshells && !shells) {
    status_fail(status, "shells pointer cannot be null");
    return h;
  }
  guarded(status, [&] {
    auto b = std::make_shared<BasisSet>();
    for (size_t i = 0; i < nshells; ++i) {
      const GauXCShell& s = shells[i];
      if (s.nprim < 1 || s.nprim > kMaxPrim) throw error("shell nprim out of range [1, 32]");
      if (s.l < 0) throw error("negative angular momentum");
      Shell sh;
      sh.l = s.l;
      sh.pure = s.pure ? 1 : 0;
      sh.nprim = s.nprim;
      for (int k = 0; k < s.nprim; ++k) {
        sh.alpha[k] = s.exponents[k];
        sh.coeff[k] = s.coefficients[k];
      }
      for (int a = 0; a < 3; ++a) sh.O[a] = s.origin[a];
      sh.tol = s.shell_tolerance > 0. ? s.shell_tolerance : kDefaultShellTol;
      if (normalize) sh.normalize();
      sh.compute_cutoff();
      b->shells.push_back(sh);
    }
    b->finalize();
    h = make_handle<GauXCBasisSet>(GauXC_Type_BasisSet, b);
  });
  return h;
}

void gauxc_basisset_delete(GauXCStatus* status, GauXCBasisSet* basis) {
  status_init(status);
  destroy<BasisSet>(basis);
}

// ---------------------------------------------------------------- molgrid
GauXCMolGrid gauxc_molgrid_new_default(GauXCStatus* status, const GauXCMolecule mol,
                                       enum GauXC_PruningScheme pruning_scheme, int64_t batchsize,
                                       enum GauXC_RadialQuad radial_quad,
                                       enum GauXC_AtomicGridSizeDefault grid_size) {
  status_init(status);
  GauXCMolGrid h{};
  h.hdr.type = GauXC_Type_MolGrid;
  if (!check(status, mol, GauXC_Type_Molecule, "Molecule")) return h;
  guarded(status, [&] {
    auto mg = std::make_shared<MolGrid>(make_default_molgrid(
        *deref<Molecule>(mol.ptr), static_cast<PruningScheme>(pruning_scheme), batchsize,
        static_cast<RadialQuad>(radial_quad), (int)grid_size));
    h = make_handle<GauXCMolGrid>(GauXC_Type_MolGrid, mg);
  });
  return h;
}

void gauxc_molgrid_delete(GauXCStatus* status, GauXCMolGrid* molgrid) {
  status_init(status);
  destroy<MolGrid>(molgrid);
}

// ---------------------------------------------------------------- runtime
GauXCRuntimeEnvironment gauxc_runtime_environment_new(GauXCStatus* status) {
  status_init(status);
  auto rt = std::make_shared<RuntimeEnv>();
  GauXCRuntimeEnvironment h{};
  h.hdr.type = GauXC_Type_RuntimeEnvironment;
  h.ptr = new std::shared_ptr<RuntimeEnv>(rt);
  h.device_ptr = nullptr;
  return h;
}

GauXCRuntimeEnvironment gauxc_device_runtime_environment_new(GauXCStatus* status,
                                                             double fill_fraction) {
  status_init(status);
  GauXCRuntimeEnvironment h{};
  h.hdr.type = GauXC_Type_RuntimeEnvironment;
  if (!(fill_fraction > 0. && fill_fraction <= 1.)) {
    status_fail(status, "fill_fraction must be in (0, 1]");
    return h;
  }
  auto rt = std::make_shared<RuntimeEnv>();
  rt->device = true;
  rt->fill_fraction = fill_fraction;
  h.ptr = new std::shared_ptr<RuntimeEnv>(rt);
  h.device_ptr = h.ptr;
  return h;
}

GauXCRuntimeEnvironment gauxc_device_runtime_environment_new_mem(GauXCStatus* status, void* mem,
                                                                 size_t mem_sz) {
  status_init(status);
  GauXCRuntimeEnvironment h{};
  h.hdr.type = GauXC_Type_RuntimeEnvironment;
  if (!mem || !mem_sz) {
    status_fail(status, "device memory buffer must be non-null and non-empty");
    return h;
  }
  auto rt = std::make_shared<RuntimeEnv>();
  rt->device = true;
  rt->user_mem = mem;
  rt->user_bytes = mem_sz;
  h.ptr = new std::shared_ptr<RuntimeEnv>(rt);
  h.device_ptr = h.ptr;
  return h;
}

void gauxc_runtime_environment_delete(GauXCStatus* status, GauXCRuntimeEnvironment* env) {
  status_init(status);
  if (env && env->ptr) {
    delete static_cast<std::shared_ptr<RuntimeEnv>*>(env->ptr);
    env->ptr = nullptr;
    env->device_ptr = nullptr;
  }
}

int gauxc_runtime_environment_comm_rank(GauXCStatus* status, const GauXCRuntimeEnvironment env) {
  status_init(status);
  if (!check(status, env, GauXC_Type_RuntimeEnvironment, "RuntimeEnvironment")) return -1;
  return 0;  // single-process build
}

int gauxc_runtime_environment_comm_size(GauXCStatus* status, const GauXCRuntimeEnvironment env) {
  status_init(status);
  if (!check(status, env, GauXC_Type_RuntimeEnvironment, "RuntimeEnvironment")) return -1;
  return 1;
}

// ---------------------------------------------------------------- load balancer
GauXCLoadBalancerFactory gauxc_load_balancer_factory_new(GauXCStatus* status,
                                                         enum GauXC_ExecutionSpace ex,
                                                         const char* kernel_name) {
  status_init(status);
  GauXCLoadBalancerFactory h{};
  h.hdr.type = GauXC_Type_LoadBalancerFactory;
  if (!kernel_name) {
    status_fail(status, "Load balancer kernel name string cannot be null");
    return h;
  }
  const std::string k = kernel_name;
  if (!(iequals(k, "Default") || iequals(k, "Replicated") || iequals(k, "Replicated-Petite"))) {
    status_fail(status, ("Load balancer kernel not supported: " + k).c_str());
    return h;
  }
  auto f = std::make_shared<LBFactory>(LBFactory{ex == GauXC_ExecutionSpace_Device, k});
  return make_handle<GauXCLoadBalancerFactory>(GauXC_Type_LoadBalancerFactory, f);
}

void gauxc_load_balancer_factory_delete(GauXCStatus* status, GauXCLoadBalancerFactory* f) {
  status_init(status);
  destroy<LBFactory>(f);
}

GauXCLoadBalancer gauxc_load_balancer_factory_get_instance(GauXCStatus* status,
                                                           const GauXCLoadBalancerFactory factory,
                                                           const GauXCRuntimeEnvironment env,
                                                           const GauXCMolecule mol,
                                                           const GauXCMolGrid mg,
                                                           const GauXCBasisSet basis) {
  status_init(status);
  GauXCLoadBalancer h{};
  h.hdr.type = GauXC_Type_LoadBalancer;
  if (!check(status, factory, GauXC_Type_LoadBalancerFactory, "LoadBalancerFactory")) return h;
  if (!check(status, env, GauXC_Type_RuntimeEnvironment, "RuntimeEnvironment")) return h;
  if (!check(status, mol, GauXC_Type_Molecule, "Molecule")) return h;
  if (!check(status, mg, GauXC_Type_MolGrid, "MolGrid")) return h;
  if (!check(status, basis, GauXC_Type_BasisSet, "BasisSet")) return h;
  guarded(status, [&] {
    auto lb = make_load_balancer(deref<Molecule>(mol.ptr), deref<MolGrid>(mg.ptr),
                                 deref<BasisSet>(basis.ptr),
                                 deref<LBFactory>(factory.ptr)->device);
    lb->rt = deref<RuntimeEnv>(env.ptr);
    h = make_handle<GauXCLoadBalancer>(GauXC_Type_LoadBalancer, lb);
  });
  return h;
}

void gauxc_load_balancer_delete(GauXCStatus* status, GauXCLoadBalancer* lb) {
  status_init(status);
  destroy<LoadBalancer>(lb);
}

// ---------------------------------------------------------------- molecular weights
GauXCMolecularWeightsFactory gauxc_molecular_weights_factory_new(
    GauXCStatus* status, enum GauXC_ExecutionSpace ex, const char* local_work_kernel_name,
    GauXCMolecularWeightsSettings settings) {
  status_init(status);
  GauXCMolecularWeightsFactory h{};
  h.hdr.type = GauXC_Type_MolecularWeightsFactory;
  if (!local_work_kernel_name) {
    status_fail(status, "Local work kernel name string cannot be null");
    return h;
  }
  if (ex != GauXC_ExecutionSpace_Device) {
    status_fail(status, "this library computes molecular weights on the device only");
    return h;
  }
  if (settings.weight_alg != GauXC_XCWeightAlg_SSF) {
    status_fail(status, "Only SSF Supported On Device");
    return h;
  }
  auto f = std::make_shared<MWFactory>(MWFactory{true, settings});
  return make_handle<GauXCMolecularWeightsFactory>(GauXC_Type_MolecularWeightsFactory, f);
}

void gauxc_molecular_weights_factory_delete(GauXCStatus* status,
                                            GauXCMolecularWeightsFactory* factory) {
  status_init(status);
  destroy<MWFactory>(factory);
}

GauXCMolecularWeights gauxc_molecular_weights_factory_get_instance(
    GauXCStatus* status, const GauXCMolecularWeightsFactory factory) {
  status_init(status);
  GauXCMolecularWeights h{};
  h.hdr.type = GauXC_Type_MolecularWeights;
  if (!check(status, factory, GauXC_Type_MolecularWeightsFactory, "MolecularWeightsFactory"))
    return h;
  auto& f = deref<MWFactory>(factory.ptr);
  auto mw = std::make_shared<MolecularWeights>(MolecularWeights{f->device, f->settings});
  return make_handle<GauXCMolecularWeights>(GauXC_Type_MolecularWeights, mw);
}

void gauxc_molecular_weights_modify_weights(GauXCStatus* status, const GauXCMolecularWeights mw,
                                            const GauXCLoadBalancer lb) {
  status_init(status);
  if (!check(status, mw, GauXC_Type_MolecularWeights, "MolecularWeights")) return;
  if (!check(status, lb, GauXC_Type_LoadBalancer, "LoadBalancer")) return;
  guarded(status, [&] {
    RuntimeEnv rt;
    molecular_weights_ssf_device(*deref<LoadBalancer>(lb.ptr), rt);
  });
}

void gauxc_molecular_weights_delete(GauXCStatus* status, GauXCMolecularWeights* mw) {
  status_init(status);
  destroy<MolecularWeights>(mw);
}

// ---------------------------------------------------------------- functional
GauXCFunctional gauxc_functional_from_string(GauXCStatus* status, const char* spec,
                                             bool polarized) {
  status_init(status);
  GauXCFunctional h{};
  h.hdr.type = GauXC_Type_Functional;
  if (!spec) {
    status_fail(status, "functional string cannot be null");
    return h;
  }
  guarded(status, [&] {
    h = make_handle<GauXCFunctional>(GauXC_Type_Functional, make_functional(spec, polarized));
  });
  return h;
}

GauXCFunctional gauxc_functional_from_enum(GauXCStatus* status, enum GauXC_Functional f,
                                           bool polarized) {
  const char* name = nullptr;
  switch (f) {
    case GauXC_Functional_SVWN5: name = "SVWN5"; break;
    case GauXC_Functional_PBE: name = "PBE"; break;
    case GauXC_Functional_revPBE: name = "revPBE"; break;
    case GauXC_Functional_PBE0: name = "PBE0"; break;
    default: break;
  }
  if (!name) {
    status_init(status);
    status_fail(status, "functional not supported by this build");
    GauXCFunctional h{};
    h.hdr.type = GauXC_Type_Functional;
    return h;
  }
  return gauxc_functional_from_string(status, name, polarized);
}

void gauxc_functional_delete(GauXCStatus* status, GauXCFunctional* functional) {
  status_init(status);
  destroy<XCFunctionalDesc>(functional);
}

// ---------------------------------------------------------------- integrator
GauXCIntegrator gauxc_integrator_new(GauXCStatus* status, const GauXCFunctional functional,
                                     const GauXCLoadBalancer lb,
                                     enum GauXC_ExecutionSpace execution_space,
                                     const char* integrator_input_type,
                                     const char* integrator_kernel_name,
                                     const char* local_work_kernel_name,
                                     const char* reduction_kernel_name) {
  status_init(status);
  GauXCIntegrator h{};
  h.hdr.type = GauXC_Type_Integrator;
  if (!check(status, functional, GauXC_Type_Functional, "Functional")) return h;
  if (!check(status, lb, GauXC_Type_LoadBalancer, "LoadBalancer")) return h;
  if (!integrator_input_type) {
    status_fail(status, "Integrator input type string cannot be null");
    return h;
  }
  if (!integrator_kernel_name) {
    status_fail(status, "Integrator kernel name string cannot be null");
    return h;
  }
  if (!local_work_kernel_name) {
    status_fail(status, "Local work kernel name string cannot be null");
    return h;
  }
  if (!reduction_kernel_name) {
    status_fail(status, "Reduction kernel name string cannot be null");
    return h;
  }
  guarded(status, [&] {
    if (execution_space != GauXC_ExecutionSpace_Device)
      throw error("this library provides the Device execution space only");
    if (!iequals(integrator_input_type, "Replicated"))
      throw error(std::string("Integrator input type not supported: ") + integrator_input_type);
    const std::string ik = integrator_kernel_name;
    if (!(iequals(ik, "Default") || iequals(ik, "Incore")))
      throw error("Integrator kernel not supported: " + ik);
    const std::string rk = reduction_kernel_name;
    if (!(iequals(rk, "Default") || iequals(rk, "BasicMPI")))
      throw error("Reduction kernel not supported: " + rk);
    const std::string lk = local_work_kernel_name;
    auto ih = std::make_shared<XCIntegratorHandle>();
    if (iequals(lk, "Default") || iequals(lk, "Scheme1") || iequals(lk, "GB300-FP64"))
      ih->prec = Precision::FP64;
    else if (iequals(lk, "GB300-Mixed"))
      ih->prec = Precision::Mixed;
    else
      throw error("Local work kernel not supported: " + lk);
    ih->lb = deref<LoadBalancer>(lb.ptr);
    ih->func = deref<XCFunctionalDesc>(functional.ptr);
    ih->rt = ih->lb->rt ? ih->lb->rt : std::make_shared<RuntimeEnv>();
    h = make_handle<GauXCIntegrator>(GauXC_Type_Integrator, ih);
  });
  return h;
}

void gauxc_integrator_delete(GauXCStatus* status, GauXCIntegrator* integrator) {
  status_init(status);
  destroy<XCIntegratorHandle>(integrator);
}

void gauxc_integrator_integrate_den(GauXCStatus* status, const GauXCIntegrator integrator,
                                    const int64_t m, const int64_t n, const double* P,
                                    const int64_t ldp, double* den) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return;
  if (!P) return status_fail(status, "Density matrix pointer cannot be null");
  if (!den) return status_fail(status, "Density output pointer cannot be null");
  guarded(status, [&] {
    integrator_integrate_den(*deref<XCIntegratorHandle>(integrator.ptr), m, n, P, ldp, den);
  });
}

void gauxc_integrator_eval_exc_rks(GauXCStatus* status, const GauXCIntegrator integrator,
                                   const int64_t m, const int64_t n, const double* P,
                                   const int64_t ldp, double* exc) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return;
  if (!P) return status_fail(status, "Density matrix pointer cannot be null");
  if (!exc) return status_fail(status, "Exc output pointer cannot be null");
  guarded(status, [&] {
    integrator_eval_exc_vxc(*deref<XCIntegratorHandle>(integrator.ptr), m, n, P, ldp, nullptr, 0,
                            exc);
  });
}

void gauxc_integrator_eval_exc_vxc_rks(GauXCStatus* status, const GauXCIntegrator integrator,
                                       const int64_t m, const int64_t n, const double* P,
                                       const int64_t ldp, double* exc, double* vxc,
                                       const int64_t vxc_ld) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return;
  if (!P) return status_fail(status, "Density matrix pointer cannot be null");
  if (!exc) return status_fail(status, "Exc output pointer cannot be null");
  if (!vxc) return status_fail(status, "VXC matrix pointer cannot be null");
  guarded(status, [&] {
    integrator_eval_exc_vxc(*deref<XCIntegratorHandle>(integrator.ptr), m, n, P, ldp, vxc, vxc_ld,
                            exc);
  });
}

void gauxc_integrator_eval_exc_uks(GauXCStatus* status, const GauXCIntegrator integrator,
                                   const int64_t m, const int64_t n, const double* Ps,
                                   const int64_t ldps, const double* Pz, const int64_t ldpz,
                                   double* exc) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return;
  if (!Ps || !Pz) return status_fail(status, "Density matrix pointer cannot be null");
  if (!exc) return status_fail(status, "Exc output pointer cannot be null");
  guarded(status, [&] {
    integrator_eval_exc_vxc_uks(*deref<XCIntegratorHandle>(integrator.ptr), m, n, Ps, ldps, Pz,
                                ldpz, nullptr, 0, nullptr, 0, exc);
  });
}

void gauxc_integrator_eval_exc_vxc_uks(GauXCStatus* status, const GauXCIntegrator integrator,
                                       const int64_t m, const int64_t n, const double* Ps,
                                       const int64_t ldps, const double* Pz, const int64_t ldpz,
                                       double* exc, double* vxcs, const int64_t ldvxcs,
                                       double* vxcz, const int64_t ldvxcz) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return;
  if (!Ps || !Pz) return status_fail(status, "Density matrix pointer cannot be null");
  if (!exc) return status_fail(status, "Exc output pointer cannot be null");
  if (!vxcs || !vxcz) return status_fail(status, "VXC matrix pointer cannot be null");
  guarded(status, [&] {
    integrator_eval_exc_vxc_uks(*deref<XCIntegratorHandle>(integrator.ptr), m, n, Ps, ldps, Pz,
                                ldpz, vxcs, ldvxcs, vxcz, ldvxcz, exc);
  });
}

// ---------------------------------------------------------------- extensions
const char* gauxc_gb300_version(void) { return "gauxc_gb300 0.1.0 (sm_103a)"; }

int gauxc_gb300_device_count(void) { return cuda_device_count(); }

size_t gauxc_gb300_basisset_nshells(GauXCStatus* status, const GauXCBasisSet basis) {
  status_init(status);
  if (!check(status, basis, GauXC_Type_BasisSet, "BasisSet")) return 0;
  return deref<BasisSet>(basis.ptr)->shells.size();
}

int32_t gauxc_gb300_basisset_nbf(GauXCStatus* status, const GauXCBasisSet basis) {
  status_init(status);
  if (!check(status, basis, GauXC_Type_BasisSet, "BasisSet")) return 0;
  return deref<BasisSet>(basis.ptr)->nbf;
}

void gauxc_gb300_basisset_get_shell(GauXCStatus* status, const GauXCBasisSet basis, size_t i,
                                    GauXCShell* out, double* cutoff_radius) {
  status_init(status);
  if (!check(status, basis, GauXC_Type_BasisSet, "BasisSet")) return;
  auto& b = deref<BasisSet>(basis.ptr);
  if (i >= b->shells.size()) return status_fail(status, "shell index out of range");
  const Shell& s = b->shells[i];
  if (out) {
    std::memset(out, 0, sizeof(*out));
    out->l = s.l;
    out->pure = s.pure != 0;
    out->nprim = s.nprim;
    for (int k = 0; k < s.nprim; ++k) {
      out->exponents[k] = s.alpha[k];
      out->coefficients[k] = s.coeff[k];
    }
    for (int a = 0; a < 3; ++a) out->origin[a] = s.O[a];
    out->shell_tolerance = s.tol;
  }
  if (cutoff_radius) *cutoff_radius = s.cutoff_radius;
}

void gauxc_gb300_basisset_set_tolerance(GauXCStatus* status, GauXCBasisSet basis, double tol) {
  status_init(status);
  if (!check(status, basis, GauXC_Type_BasisSet, "BasisSet")) return;
  for (auto& s : deref<BasisSet>(basis.ptr)->shells) s.set_tolerance(tol);
}

void gauxc_gb300_molgrid_atomic_grid(GauXCStatus* status, const GauXCMolGrid mg, int64_t Z,
                                     int64_t* npts, int64_t* nbatches, double* points,
                                     double* weights, int64_t* batch_ranges) {
  status_init(status);
  if (!check(status, mg, GauXC_Type_MolGrid, "MolGrid")) return;
  guarded(status, [&] {
    const AtomicGrid& g = deref<MolGrid>(mg.ptr)->grids.at(Z);
    if (npts) *npts = (int64_t)g.points.size();
    if (nbatches) *nbatches = (int64_t)g.batches.size();
    for (size_t i = 0; i < g.points.size(); ++i) {
      if (points)
        for (int a = 0; a < 3; ++a) points[3 * i + a] = g.points[i][a];
      if (weights) weights[i] = g.weights[i];
    }
    if (batch_ranges)
      for (size_t b = 0; b < g.batches.size(); ++b) {
        batch_ranges[2 * b] = g.batches[b].first;
        batch_ranges[2 * b + 1] = g.batches[b].second;
      }
  });
}

size_t gauxc_gb300_load_balancer_ntasks(GauXCStatus* status, const GauXCLoadBalancer lb) {
  status_init(status);
  if (!check(status, lb, GauXC_Type_LoadBalancer, "LoadBalancer")) return 0;
  return deref<LoadBalancer>(lb.ptr)->tasks.size();
}

void gauxc_gb300_load_balancer_task_info(GauXCStatus* status, const GauXCLoadBalancer lb, size_t i,
                                         int32_t info[4], double* dist_nearest) {
  status_init(status);
  if (!check(status, lb, GauXC_Type_LoadBalancer, "LoadBalancer")) return;
  auto& L = deref<LoadBalancer>(lb.ptr);
  if (i >= L->tasks.size()) return status_fail(status, "task index out of range");
  const XCTask& t = L->tasks[i];
  if (info) {
    info[0] = t.iParent;
    info[1] = t.npts;
    info[2] = t.nbe;
    info[3] = (int32_t)t.shell_list.size();
  }
  if (dist_nearest) *dist_nearest = t.dist_nearest;
}

void gauxc_gb300_load_balancer_task_data(GauXCStatus* status, const GauXCLoadBalancer lb, size_t i,
                                         double* points, double* weights, int32_t* shell_list) {
  status_init(status);
  if (!check(status, lb, GauXC_Type_LoadBalancer, "LoadBalancer")) return;
  auto& L = deref<LoadBalancer>(lb.ptr);
  if (i >= L->tasks.size()) return status_fail(status, "task index out of range");
  const XCTask& t = L->tasks[i];
  if (points) std::memcpy(points, t.points.data(), t.points.size() * sizeof(double));
  if (weights) std::memcpy(weights, t.weights.data(), t.weights.size() * sizeof(double));
  if (shell_list) std::memcpy(shell_list, t.shell_list.data(), t.shell_list.size() * sizeof(int32_t));
}

GauXCLoadBalancer gauxc_gb300_load_balancer_subset(GauXCStatus* status, const GauXCLoadBalancer lb,
                                                   const int64_t* task_idx, size_t n) {
  status_init(status);
  GauXCLoadBalancer h{};
  h.hdr.type = GauXC_Type_LoadBalancer;
  if (!check(status, lb, GauXC_Type_LoadBalancer, "LoadBalancer")) return h;
  if (n > 0 && !task_idx) {
    status_fail(status, "task index array cannot be null");
    return h;
  }
  guarded(status, [&] {
    auto& L = deref<LoadBalancer>(lb.ptr);
    std::vector<int64_t> idx(task_idx, task_idx + n);
    h = make_handle<GauXCLoadBalancer>(GauXC_Type_LoadBalancer, load_balancer_subset(*L, idx));
  });
  return h;
}

bool gauxc_gb300_load_balancer_weights_modified(GauXCStatus* status, const GauXCLoadBalancer lb) {
  status_init(status);
  if (!check(status, lb, GauXC_Type_LoadBalancer, "LoadBalancer")) return false;
  return deref<LoadBalancer>(lb.ptr)->weights_modified;
}

double gauxc_gb300_integrator_last_nel(GauXCStatus* status, const GauXCIntegrator integrator) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return 0.;
  return deref<XCIntegratorHandle>(integrator.ptr)->last_nel;
}

int gauxc_gb300_integrator_timings(GauXCStatus* status, const GauXCIntegrator integrator,
                                   double* out, int nmax) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return 0;
  auto t = integrator_timings(*deref<XCIntegratorHandle>(integrator.ptr));
  const double v[8] = {t["h2d_ms"], t["compute_ms"], t["d2h_ms"], t["wall_ms"],
                       t["plan_ms"], t["plan_merge_ms"], t["plan_layout_ms"], t["plan_lists_ms"]};
  int n = 0;
  for (; n < 8 && n < nmax; ++n) out[n] = v[n];
  return n;
}

int gauxc_gb300_integrator_plan_stats(GauXCStatus* status, const GauXCIntegrator integrator,
                                      double* out, int nmax) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return 0;
  int n = 0;
  guarded(status, [&] {
    PlanStats s = integrator_plan_stats(*deref<XCIntegratorHandle>(integrator.ptr));
    const double v[18] = {(double)s.ntasks, (double)s.npts, (double)s.npts_pad,
                          (double)s.nbatches, s.sum_npts_nbe, s.sum_npts_nbe2,
                          s.sum_pad_npts_nbe2, s.scratch_bytes, (double)s.gpu_launches,
                          s.tensor_flops_x, s.tensor_flops_v, s.kbytes[0], s.kbytes[1],
                          s.kbytes[2], s.kbytes[3], s.kbytes[4], s.kbytes[5], s.kbytes[6]};
    for (; n < 18 && n < nmax; ++n) out[n] = v[n];
  });
  return n;
}

void gauxc_gb300_integrator_set_profiling(GauXCStatus* status, const GauXCIntegrator integrator,
                                          bool on) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return;
  integrator_set_profiling(*deref<XCIntegratorHandle>(integrator.ptr), on);
}

void gauxc_gb300_integrator_set_pipeline_check(GauXCStatus* status,
                                               const GauXCIntegrator integrator, double wait_ms,
                                               bool withhold) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return;
  guarded(status, [&] {
    integrator_set_pipeline_check(*deref<XCIntegratorHandle>(integrator.ptr), wait_ms, withhold);
  });
}

int gauxc_gb300_integrator_kernel_times(GauXCStatus* status, const GauXCIntegrator integrator,
                                        double* out, int nmax) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return 0;
  auto v = integrator_kernel_times(*deref<XCIntegratorHandle>(integrator.ptr));
  int n = 0;
  for (; n < (int)v.size() && n < nmax; ++n) out[n] = v[n];
  return n;
}

void gauxc_gb300_integrator_set_plan_params(GauXCStatus* status, const GauXCIntegrator integrator,
                                            int pb_max_pts, double nu2_weight,
                                            double scratch_gb) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return;
  guarded(status, [&] {
    integrator_set_plan_params(*deref<XCIntegratorHandle>(integrator.ptr),
                               PlanParams{pb_max_pts, nu2_weight, scratch_gb * 1e9});
  });
}

double gauxc_gb300_integrator_autotune(GauXCStatus* status, const GauXCIntegrator integrator,
                                       int64_t m, int64_t n, const double* P, int64_t ldp,
                                       int* pb_max_pts, double* nu2_weight) {
  status_init(status);
  if (!check(status, integrator, GauXC_Type_Integrator, "Integrator")) return 0.;
  if (!P) {
    status_fail(status, "Density matrix pointer cannot be null");
    return 0.;
  }
  double ms = 0.;
  guarded(status, [&] {
    XCIntegratorHandle& h = *deref<XCIntegratorHandle>(integrator.ptr);
    if (m != n || m != h.lb->basis->nbf) throw error("P Must Have Same Dimension as Basis");
    PlanParams best;
    ms = integrator_autotune(h, P, ldp, &best);
    if (pb_max_pts) *pb_max_pts = best.pb_max_pts;
    if (nu2_weight) *nu2_weight = best.nu2_weight;
  });
  return ms;
}

GauXCGB300Batch gauxc_gb300_batch_new(GauXCStatus* status, const GauXCIntegrator* integrators,
                                      int32_t n) {
  status_init(status);
  GauXCGB300Batch b{};
  if (!integrators || n <= 0) {
    status_fail(status, "Batch needs at least one integrator");
    return b;
  }
  for (int32_t i = 0; i < n; ++i)
    if (!check(status, integrators[i], GauXC_Type_Integrator, "Integrator")) return b;
  guarded(status, [&] {
    auto bh = std::make_shared<BatchHandle>();
    std::vector<XCIntegratorHandle*> raw;
    for (int32_t i = 0; i < n; ++i) {
      bh->members.push_back(deref<XCIntegratorHandle>(integrators[i].ptr));
      raw.push_back(bh->members.back().get());
    }
    bh->batch = batch_new(raw);
    b = make_handle<GauXCGB300Batch>(GauXC_Type_GB300Batch, bh);
  });
  return b;
}

void gauxc_gb300_batch_eval_exc_vxc_rks(GauXCStatus* status, const GauXCGB300Batch batch,
                                        const double* const* P, const int64_t* ldp,
                                        double* const* VXC, const int64_t* ldvxc, double* EXC) {
  status_init(status);
  if (!check(status, batch, GauXC_Type_GB300Batch, "Batch")) return;
  if (!P || !ldp || !EXC) return status_fail(status, "P, ldp and EXC arrays cannot be null");
  guarded(status, [&] {
    auto& bh = *deref<BatchHandle>(batch.ptr);
    const size_t n = bh.members.size();
    std::vector<double*> V(n, nullptr);
    std::vector<int64_t> lv(n, 0);
    if (VXC)
      for (size_t i = 0; i < n; ++i) {
        V[i] = VXC[i];
        lv[i] = ldvxc ? ldvxc[i] : 0;
      }
    batch_eval_exc_vxc(*bh.batch, P, ldp, V.data(), lv.data(), EXC);
  });
}

int gauxc_gb300_batch_timings(GauXCStatus* status, const GauXCGB300Batch batch, double* out,
                              int nmax) {
  status_init(status);
  if (!check(status, batch, GauXC_Type_GB300Batch, "Batch")) return 0;
  auto t = batch_timings(*deref<BatchHandle>(batch.ptr)->batch);
  const double v[5] = {t["compute_ms"], t["wall_ms"], t["graph_launch"], t["members"],
                       t["gpu_launches"]};
  int k = 0;
  for (; k < 5 && k < nmax; ++k) out[k] = v[k];
  return k;
}

void gauxc_gb300_batch_delete(GauXCStatus* status, GauXCGB300Batch* batch) {
  status_init(status);
  destroy<BatchHandle>(batch);
}

int gauxc_gb300_host_register(GauXCStatus* status, void* ptr, size_t bytes) {
  status_init(status);
  int r = 0;
  guarded(status, [&] { r = host_register(ptr, bytes) ? 1 : 0; });
  return r;
}

void gauxc_gb300_host_unregister(GauXCStatus* status, void* ptr) {
  status_init(status);
  guarded(status, [&] { host_unregister(ptr); });
}

double gauxc_gb300_measure_fp64_peak(GauXCStatus* status) {
  status_init(status);
  double r = 0.;
  guarded(status, [&] { r = measure_fp64_peak(); });
  return r;
}

double gauxc_gb300_tensor_core_selftest(GauXCStatus* status, int n, int k) {
  status_init(status);
  double r = -1.;
  guarded(status, [&] { r = tensor_core_selftest(n, k); });
  return r;
}

double gauxc_gb300_ff_exp_selftest(GauXCStatus* status, int n) {
  status_init(status);
  double r = -1.;
  guarded(status, [&] {
    if (cuda_device_count() == 0) throw error("no CUDA device available");
    r = ff_exp_selftest(n);
  });
  return r;
}

void gauxc_gb300_set_device(GauXCStatus* status, int device) {
  status_init(status);
  guarded(status, [&] { set_device(device); });
}

void gauxc_gb300_ssf_weights(GauXCStatus* status, int64_t npts, int32_t natoms,
                             const double* points, const int32_t* iparent,
                             const double* dist_nearest, const double* coords, double* weights) {
  status_init(status);
  if (npts < 0 || natoms <= 0) return status_fail(status, "invalid sizes");
  if (npts == 0) return;
  if (!points || !iparent || !dist_nearest || !coords || !weights)
    return status_fail(status, "null array argument");
  for (int64_t i = 0; i < npts; ++i)
    if (iparent[i] < 0 || iparent[i] >= natoms)
      return status_fail(status, "iparent out of range");
  guarded(status, [&] {
    ssf_weights_device(npts, natoms, points, iparent, dist_nearest, coords, weights);
  });
}

void gauxc_gb300_ssf_weights_noalloc(GauXCStatus* status, int64_t npts, int32_t natoms,
                                     const double* x, const double* y, const double* z,
                                     const int32_t* iparent, const double* dist_nearest,
                                     const double* coords, double* weights, void* stream) {
  status_init(status);
  if (npts < 0 || natoms <= 0) return status_fail(status, "invalid sizes");
  if (npts == 0) return;
  if (!x || !y || !z || !iparent || !dist_nearest || !coords || !weights)
    return status_fail(status, "null array argument");
  guarded(status, [&] {
    ssf_weights_noalloc(npts, natoms, x, y, z, iparent, dist_nearest, coords, weights, stream);
  });
}

void gauxc_gb300_collocation(GauXCStatus* status, const GauXCBasisSet basis, int64_t npts,
                             const double* points, int32_t nshells, const int32_t* shell_list,
                             double* phi, double* dphi_x, double* dphi_y, double* dphi_z) {
  status_init(status);
  if (!check(status, basis, GauXC_Type_BasisSet, "BasisSet")) return;
  if (npts <= 0 || nshells <= 0) return status_fail(status, "invalid sizes");
  if (!points || !shell_list || !phi) return status_fail(status, "null array argument");
  auto& b = deref<BasisSet>(basis.ptr);
  for (int i = 0; i < nshells; ++i)
    if (shell_list[i] < 0 || shell_list[i] >= (int)b->shells.size())
      return status_fail(status, "shell index out of range");
  const bool grad = dphi_x || dphi_y || dphi_z;
  if (grad && !(dphi_x && dphi_y && dphi_z))
    return status_fail(status, "gradient outputs must be all null or all non-null");
  guarded(status, [&] {
    collocation_device(*b, npts, points, nshells, shell_list, grad, phi, dphi_x, dphi_y, dphi_z);
  });
}

}  // extern "C"

// ---------------------------------------------------------------- stage-level work driver
namespace {
template <typename F>
void lwd_call(GauXCStatus* status, const GauXCGB300DeviceData& d, F&& f) {
  status_init(status);
  if (!check(status, d, GauXC_Type_GB300DeviceData, "DeviceData")) return;
  guarded(status, [&] { f(*deref<LWDData>(d.ptr)); });
}
}  // namespace

extern "C" {

GauXCGB300DeviceData gauxc_gb300_lwd_device_data_new(GauXCStatus* status,
                                                     const GauXCLoadBalancer lb,
                                                     int64_t task_begin, int64_t task_end) {
  status_init(status);
  GauXCGB300DeviceData h{};
  h.hdr.type = GauXC_Type_GB300DeviceData;
  if (!check(status, lb, GauXC_Type_LoadBalancer, "LoadBalancer")) return h;
  guarded(status, [&] {
    h = make_handle<GauXCGB300DeviceData>(
        GauXC_Type_GB300DeviceData, lwd_create(*deref<LoadBalancer>(lb.ptr), task_begin, task_end));
  });
  return h;
}

void gauxc_gb300_lwd_device_data_delete(GauXCStatus* status, GauXCGB300DeviceData* data) {
  status_init(status);
  destroy<LWDData>(data);
}

void gauxc_gb300_lwd_eval_collocation(GauXCStatus* status, const GauXCGB300DeviceData data,
                                      bool gradient) {
  lwd_call(status, data, [&](LWDData& d) { lwd_eval_collocation(d, gradient); });
}
void gauxc_gb300_lwd_eval_xmat(GauXCStatus* status, const GauXCGB300DeviceData data, double fac,
                               const double* P, int64_t ldp) {
  lwd_call(status, data, [&](LWDData& d) { lwd_eval_xmat(d, fac, P, ldp); });
}
void gauxc_gb300_lwd_eval_vvars(GauXCStatus* status, const GauXCGB300DeviceData data, bool gga) {
  lwd_call(status, data, [&](LWDData& d) { lwd_eval_vvars(d, gga); });
}
void gauxc_gb300_lwd_eval_uvars(GauXCStatus* status, const GauXCGB300DeviceData data) {
  lwd_call(status, data, [&](LWDData& d) { lwd_eval_uvars(d); });
}
void gauxc_gb300_lwd_eval_kern_exc_vxc(GauXCStatus* status, const GauXCGB300DeviceData data,
                                       const GauXCFunctional functional) {
  status_init(status);
  if (!check(status, functional, GauXC_Type_Functional, "Functional")) return;
  lwd_call(status, data, [&](LWDData& d) {
    lwd_eval_kern_exc_vxc(d, *deref<XCFunctionalDesc>(functional.ptr));
  });
}
void gauxc_gb300_lwd_inc_exc(GauXCStatus* status, const GauXCGB300DeviceData data) {
  lwd_call(status, data, [&](LWDData& d) { lwd_inc_exc(d); });
}
void gauxc_gb300_lwd_inc_nel(GauXCStatus* status, const GauXCGB300DeviceData data) {
  lwd_call(status, data, [&](LWDData& d) { lwd_inc_nel(d); });
}
void gauxc_gb300_lwd_eval_zmat_vxc(GauXCStatus* status, const GauXCGB300DeviceData data, bool gga) {
  lwd_call(status, data, [&](LWDData& d) { lwd_eval_zmat_vxc(d, gga); });
}
void gauxc_gb300_lwd_inc_vxc(GauXCStatus* status, const GauXCGB300DeviceData data) {
  lwd_call(status, data, [&](LWDData& d) { lwd_inc_vxc(d); });
}
void gauxc_gb300_lwd_symmetrize_vxc(GauXCStatus* status, const GauXCGB300DeviceData data,
                                    double* vxc, int64_t ldvxc) {
  lwd_call(status, data, [&](LWDData& d) { lwd_symmetrize_vxc(d, vxc, ldvxc); });
}
void gauxc_gb300_lwd_results(GauXCStatus* status, const GauXCGB300DeviceData data, double* exc,
                             double* nel) {
  lwd_call(status, data, [&](LWDData& d) { lwd_results(d, exc, nel); });
}

}  // extern "C"
