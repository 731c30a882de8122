/*
 * gauxc_gb300 -- header-only C++ front end over the C ABI (gauxc_gb300.h).
 *
 * Mirrors the reference C++ API that an SCF code calls for the device XC
 * path, with the same class names, constructor arguments and call shapes:
 *   Molecule, BasisSet<double> / Shell     include/gauxc/molecule.hpp, basisset.hpp, shell.hpp
 *   MolGridFactory::create_default_molgrid include/gauxc/molgrid/defaults.hpp
 *   RuntimeEnvironment / DeviceRuntimeEnvironment
 *                                          include/gauxc/runtime_environment/decl.hpp
 *   LoadBalancerFactory(ex, kernel).get_instance(rt, mol, mg, basis)
 *                                          include/gauxc/load_balancer.hpp
 *   MolecularWeightsFactory(ex, kernel, settings).get_instance().modify_weights(lb)
 *                                          include/gauxc/molecular_weights.hpp
 *   functional_type(spec, polarized)       (ExchCXX::XCFunctional in the reference)
 *   XCIntegratorFactory<MatrixType>(ex, input_type, integrator_kernel,
 *       lwd_kernel, reduction_kernel).get_instance(func, lb)
 *                                          include/gauxc/xc_integrator/integrator_factory.hpp:24-111
 *   XCIntegrator<MatrixType>::eval_exc_vxc(P) -> std::tuple<EXC, VXC>,
 *       eval_exc_vxc(Ps, Pz) -> std::tuple<EXC, VXC_s, VXC_z> (UKS),
 *       eval_exc(P), eval_exc(Ps, Pz), integrate_den(P)
 *                                          include/gauxc/xc_integrator.hpp:30-94
 * The classes live in namespace gauxc_gb300 so that they can sit next to the
 * reference headers; a caller switches with one namespace alias.
 *
 * MatrixType: column-major, with value_type, MatrixType(rows, cols), rows(),
 * cols() and data() (Eigen::MatrixXd qualifies).  Failures throw
 * gauxc_gb300::exception with the C layer's message (the reference throws
 * GauXC::generic_gauxc_exception).  Every object owns its C handle; the C
 * layer keeps what a handle depends on alive, so objects may be destroyed in
 * any order.
 */
#ifndef GAUXC_GB300_HPP
#define GAUXC_GB300_HPP

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "gauxc_gb300.h"

namespace gauxc_gb300 {

enum class ExecutionSpace { Host = GauXC_ExecutionSpace_Host, Device = GauXC_ExecutionSpace_Device };
enum class PruningScheme {
  Unpruned = GauXC_PruningScheme_Unpruned,
  Robust = GauXC_PruningScheme_Robust,
  Treutler = GauXC_PruningScheme_Treutler
};
enum class RadialQuad {
  Becke = GauXC_RadialQuad_Becke,
  MuraKnowles = GauXC_RadialQuad_MuraKnowles,
  MurrayHandyLaming = GauXC_RadialQuad_MurrayHandyLaming,
  TreutlerAhlrichs = GauXC_RadialQuad_TreutlerAhlrichs
};
enum class AtomicGridSizeDefault {
  FineGrid = GauXC_AtomicGridSizeDefault_FineGrid,
  UltraFineGrid = GauXC_AtomicGridSizeDefault_UltraFineGrid,
  SuperFineGrid = GauXC_AtomicGridSizeDefault_SuperFineGrid,
  GM3 = GauXC_AtomicGridSizeDefault_GM3,
  GM5 = GauXC_AtomicGridSizeDefault_GM5
};
enum class XCWeightAlg {
  NOTPARTITIONED = GauXC_XCWeightAlg_NOTPARTITIONED,
  Becke = GauXC_XCWeightAlg_Becke,
  SSF = GauXC_XCWeightAlg_SSF,
  LKO = GauXC_XCWeightAlg_LKO
};

struct exception : std::runtime_error {
  using std::runtime_error::runtime_error;
};

namespace detail {

// Calls fn(&status, args...), turns a failure into an exception.
template <typename F, typename... A>
auto call(F fn, A&&... args) -> decltype(fn(nullptr, std::forward<A>(args)...)) {
  GauXCStatus st{0, nullptr};
  struct Guard {
    GauXCStatus* s;
    ~Guard() { gauxc_status_delete(s); }
  } guard{&st};
  auto check = [&] {
    if (st.code != 0) throw exception(st.message ? st.message : "gauxc_gb300: unknown error");
  };
  if constexpr (std::is_void_v<decltype(fn(nullptr, std::forward<A>(args)...))>) {
    fn(&st, std::forward<A>(args)...);
    check();
  } else {
    auto r = fn(&st, std::forward<A>(args)...);
    check();
    return r;
  }
}

// Shared ownership of one C handle, released by its gauxc_*_delete.
template <typename H, void (*Del)(GauXCStatus*, H*)>
class Owned {
 public:
  Owned() = default;
  explicit Owned(H h)
      : p_(new H(h), [](H* x) {
          GauXCStatus st{0, nullptr};
          Del(&st, x);
          gauxc_status_delete(&st);
          delete x;
        }) {}
  const H& get() const { return *p_; }

 private:
  std::shared_ptr<H> p_;
};

}  // namespace detail

// ------------------------------------------------------------------ molecule / basis
struct Atom {
  int64_t Z;
  double x, y, z;  // bohr
};

class Molecule {
 public:
  explicit Molecule(const std::vector<Atom>& atoms) {
    std::vector<GauXCAtom> a(atoms.size());
    for (size_t i = 0; i < atoms.size(); ++i) a[i] = GauXCAtom{atoms[i].Z, atoms[i].x, atoms[i].y, atoms[i].z};
    h_ = Owned(detail::call(gauxc_molecule_new_from_atoms, a.data(), a.size()));
  }
  size_t natoms() const { return detail::call(gauxc_molecule_natoms, h_.get()); }
  const GauXCMolecule& handle() const { return h_.get(); }

 private:
  using Owned = detail::Owned<GauXCMolecule, gauxc_molecule_delete>;
  Owned h_;
};

struct Shell {
  int l = 0;
  bool pure = true;
  std::vector<double> exponents, coefficients;
  double origin[3] = {0., 0., 0.};
  double tolerance = 1e-10;
};

template <typename T = double>
class BasisSet {
 public:
  explicit BasisSet(const std::vector<Shell>& shells, bool normalize = true) {
    std::vector<GauXCShell> s(shells.size());
    for (size_t i = 0; i < shells.size(); ++i) {
      const Shell& x = shells[i];
      if (x.exponents.size() != x.coefficients.size() || x.exponents.size() > 32)
        throw exception("shell " + std::to_string(i) + ": 1..32 primitives with one coefficient each");
      GauXCShell c{};
      c.l = x.l;
      c.pure = x.pure;
      c.nprim = (int32_t)x.exponents.size();
      for (size_t k = 0; k < x.exponents.size(); ++k) {
        c.exponents[k] = x.exponents[k];
        c.coefficients[k] = x.coefficients[k];
      }
      for (int a = 0; a < 3; ++a) c.origin[a] = x.origin[a];
      c.shell_tolerance = x.tolerance;
      s[i] = c;
    }
    h_ = Owned(detail::call(gauxc_basisset_new_from_shells, s.data(), s.size(), normalize));
  }
  int32_t nbf() const { return detail::call(gauxc_gb300_basisset_nbf, h_.get()); }
  size_t nshells() const { return detail::call(gauxc_gb300_basisset_nshells, h_.get()); }
  const GauXCBasisSet& handle() const { return h_.get(); }

 private:
  using Owned = detail::Owned<GauXCBasisSet, gauxc_basisset_delete>;
  Owned h_;
};

// ------------------------------------------------------------------ grids / runtime
class MolGrid {
 public:
  explicit MolGrid(GauXCMolGrid h) : h_(h) {}
  const GauXCMolGrid& handle() const { return h_.get(); }

 private:
  detail::Owned<GauXCMolGrid, gauxc_molgrid_delete> h_;
};

struct MolGridFactory {
  static MolGrid create_default_molgrid(const Molecule& mol, PruningScheme scheme,
                                        int64_t batch_size, RadialQuad rq,
                                        AtomicGridSizeDefault grid) {
    return MolGrid(detail::call(gauxc_molgrid_new_default, mol.handle(),
                                (enum GauXC_PruningScheme)scheme, batch_size,
                                (enum GauXC_RadialQuad)rq, (enum GauXC_AtomicGridSizeDefault)grid));
  }
};

class RuntimeEnvironment {
 public:
  RuntimeEnvironment() : h_(detail::call(gauxc_runtime_environment_new)) {}
  int comm_rank() const { return detail::call(gauxc_runtime_environment_comm_rank, h_.get()); }
  int comm_size() const { return detail::call(gauxc_runtime_environment_comm_size, h_.get()); }
  const GauXCRuntimeEnvironment& handle() const { return h_.get(); }

 protected:
  explicit RuntimeEnvironment(GauXCRuntimeEnvironment h) : h_(h) {}

 private:
  detail::Owned<GauXCRuntimeEnvironment, gauxc_runtime_environment_delete> h_;
};

// Device memory policy: a fraction of the free memory, or a caller-owned
// device buffer that every plan is carved from (no cudaMalloc afterwards).
class DeviceRuntimeEnvironment : public RuntimeEnvironment {
 public:
  explicit DeviceRuntimeEnvironment(double fill_fraction = 0.9)
      : RuntimeEnvironment(detail::call(gauxc_device_runtime_environment_new, fill_fraction)) {}
  DeviceRuntimeEnvironment(void* mem, size_t bytes)
      : RuntimeEnvironment(detail::call(gauxc_device_runtime_environment_new_mem, mem, bytes)) {}
};

// ------------------------------------------------------------------ load balancer / weights
class LoadBalancer {
 public:
  LoadBalancer(GauXCLoadBalancer h, int64_t nbf) : h_(h), nbf_(nbf) {}
  // basis functions of the basis set the tasks were screened against
  int64_t nbf() const { return nbf_; }
  size_t ntasks() const { return detail::call(gauxc_gb300_load_balancer_ntasks, h_.get()); }
  bool weights_modified() const {
    return detail::call(gauxc_gb300_load_balancer_weights_modified, h_.get());
  }
  const GauXCLoadBalancer& handle() const { return h_.get(); }

 private:
  detail::Owned<GauXCLoadBalancer, gauxc_load_balancer_delete> h_;
  int64_t nbf_;
};

class LoadBalancerFactory {
 public:
  LoadBalancerFactory(ExecutionSpace ex, const std::string& kernel)
      : h_(detail::call(gauxc_load_balancer_factory_new, (enum GauXC_ExecutionSpace)ex,
                        kernel.c_str())) {}
  template <typename T>
  LoadBalancer get_instance(const RuntimeEnvironment& rt, const Molecule& mol, const MolGrid& mg,
                            const BasisSet<T>& basis) const {
    return LoadBalancer(detail::call(gauxc_load_balancer_factory_get_instance, h_.get(),
                                     rt.handle(), mol.handle(), mg.handle(), basis.handle()),
                        (int64_t)basis.nbf());
  }
  template <typename... A>
  std::shared_ptr<LoadBalancer> get_shared_instance(A&&... a) const {
    return std::make_shared<LoadBalancer>(get_instance(std::forward<A>(a)...));
  }

 private:
  detail::Owned<GauXCLoadBalancerFactory, gauxc_load_balancer_factory_delete> h_;
};

struct MolecularWeightsSettings {
  XCWeightAlg weight_alg = XCWeightAlg::SSF;
  bool becke_size_adjustment = false;
};

class MolecularWeights {
 public:
  explicit MolecularWeights(GauXCMolecularWeights h) : h_(h) {}
  void modify_weights(LoadBalancer& lb) const {
    detail::call(gauxc_molecular_weights_modify_weights, h_.get(), lb.handle());
  }

 private:
  detail::Owned<GauXCMolecularWeights, gauxc_molecular_weights_delete> h_;
};

class MolecularWeightsFactory {
 public:
  MolecularWeightsFactory(ExecutionSpace ex, const std::string& kernel,
                          MolecularWeightsSettings s = {})
      : h_(detail::call(gauxc_molecular_weights_factory_new, (enum GauXC_ExecutionSpace)ex,
                        kernel.c_str(),
                        GauXCMolecularWeightsSettings{(enum GauXC_XCWeightAlg)s.weight_alg,
                                                      s.becke_size_adjustment})) {}
  MolecularWeights get_instance() const {
    return MolecularWeights(detail::call(gauxc_molecular_weights_factory_get_instance, h_.get()));
  }

 private:
  detail::Owned<GauXCMolecularWeightsFactory, gauxc_molecular_weights_factory_delete> h_;
};

// ------------------------------------------------------------------ functional / integrator
class functional_type {
 public:
  explicit functional_type(const std::string& spec, bool polarized = false)
      : h_(detail::call(gauxc_functional_from_string, spec.c_str(), polarized)) {}
  const GauXCFunctional& handle() const { return h_.get(); }

 private:
  detail::Owned<GauXCFunctional, gauxc_functional_delete> h_;
};

template <typename MatrixType>
class XCIntegrator {
 public:
  using matrix_type = MatrixType;
  using value_type = typename MatrixType::value_type;
  using exc_vxc_type_rks = std::tuple<value_type, matrix_type>;
  using exc_vxc_type_uks = std::tuple<value_type, matrix_type, matrix_type>;

  explicit XCIntegrator(GauXCIntegrator h, int64_t nbf) : h_(h), nbf_(nbf) {}

  // N_el of the alpha density P (tests/xc_integrator.cxx:190-196)
  value_type integrate_den(const MatrixType& P) {
    value_type n = 0;
    detail::call(gauxc_integrator_integrate_den, h_.get(), (int64_t)P.rows(), (int64_t)P.cols(),
                 P.data(), (int64_t)P.rows(), &n);
    return n;
  }
  value_type eval_exc(const MatrixType& P) {
    value_type e = 0;
    detail::call(gauxc_integrator_eval_exc_rks, h_.get(), (int64_t)P.rows(), (int64_t)P.cols(),
                 P.data(), (int64_t)P.rows(), &e);
    return e;
  }
  exc_vxc_type_rks eval_exc_vxc(const MatrixType& P) {
    MatrixType V(nbf_, nbf_);
    value_type e = 0;
    detail::call(gauxc_integrator_eval_exc_vxc_rks, h_.get(), (int64_t)P.rows(),
                 (int64_t)P.cols(), P.data(), (int64_t)P.rows(), &e, V.data(), (int64_t)nbf_);
    return exc_vxc_type_rks(e, std::move(V));
  }
  // UKS: Ps = P_alpha + P_beta, Pz = P_alpha - P_beta (polarized functional)
  value_type eval_exc(const MatrixType& Ps, const MatrixType& Pz) {
    value_type e = 0;
    detail::call(gauxc_integrator_eval_exc_uks, h_.get(), (int64_t)Ps.rows(), (int64_t)Ps.cols(),
                 Ps.data(), (int64_t)Ps.rows(), Pz.data(), (int64_t)Pz.rows(), &e);
    return e;
  }
  exc_vxc_type_uks eval_exc_vxc(const MatrixType& Ps, const MatrixType& Pz) {
    MatrixType Vs(nbf_, nbf_), Vz(nbf_, nbf_);
    value_type e = 0;
    detail::call(gauxc_integrator_eval_exc_vxc_uks, h_.get(), (int64_t)Ps.rows(),
                 (int64_t)Ps.cols(), Ps.data(), (int64_t)Ps.rows(), Pz.data(), (int64_t)Pz.rows(),
                 &e, Vs.data(), (int64_t)nbf_, Vz.data(), (int64_t)nbf_);
    return exc_vxc_type_uks(e, std::move(Vs), std::move(Vz));
  }
  const GauXCIntegrator& handle() const { return h_.get(); }

 private:
  detail::Owned<GauXCIntegrator, gauxc_integrator_delete> h_;
  int64_t nbf_;
};

template <typename MatrixType>
class XCIntegratorFactory {
 public:
  using integrator_type = XCIntegrator<MatrixType>;

  XCIntegratorFactory(ExecutionSpace ex, std::string integrator_input_type,
                      std::string integrator_kernel_name, std::string local_work_kernel_name,
                      std::string reduction_kernel_name)
      : ex_(ex), input_(std::move(integrator_input_type)), ik_(std::move(integrator_kernel_name)),
        lk_(std::move(local_work_kernel_name)), rk_(std::move(reduction_kernel_name)) {}

  integrator_type get_instance(const functional_type& func, const LoadBalancer& lb) const {
    return integrator_type(detail::call(gauxc_integrator_new, func.handle(), lb.handle(),
                                        (enum GauXC_ExecutionSpace)ex_, input_.c_str(),
                                        ik_.c_str(), lk_.c_str(), rk_.c_str()),
                           lb.nbf());
  }
  std::shared_ptr<integrator_type> get_shared_instance(const functional_type& func,
                                                       const LoadBalancer& lb) const {
    return std::make_shared<integrator_type>(get_instance(func, lb));
  }

 private:
  ExecutionSpace ex_;
  std::string input_, ik_, lk_, rk_;
};

}  // namespace gauxc_gb300

#endif  // GAUXC_GB300_HPP
