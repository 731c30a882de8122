// The header-only C++ front end (include/gauxc_gb300.hpp) used the way an
// SCF code uses the reference's C++ API: build the system, get a load
// balancer and weights, XCIntegratorFactory<MatrixType>(...).get_instance(
// func, lb), then auto [EXC, VXC] = integ.eval_exc_vxc(P).  MatrixType is a
// minimal column-major matrix (what Eigen::MatrixXd provides).  Also checks
// that failures arrive as exceptions, and that a null GauXCStatus* turns a
// C-layer failure into a C++ exception (src/c-api/c_status.hpp:31-44).
// With argument "gpu" it runs on the device and writes nbf, P, VXC, EXC and
// N_el to the file named by the second argument.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gauxc_gb300.hpp"

namespace gx = gauxc_gb300;

struct Matrix {
  using value_type = double;
  Matrix(int64_t r, int64_t c) : r_(r), c_(c), v_((size_t)(r * c), 0.) {}
  int64_t rows() const { return r_; }
  int64_t cols() const { return c_; }
  double* data() { return v_.data(); }
  const double* data() const { return v_.data(); }
  double& operator()(int64_t i, int64_t j) { return v_[(size_t)(i + j * r_)]; }
  int64_t r_, c_;
  std::vector<double> v_;
};

#define EXPECT(c)                                                                \
  do {                                                                           \
    if (!(c)) {                                                                  \
      std::fprintf(stderr, "%s:%d: expectation failed: %s\n", __FILE__, __LINE__, #c); \
      return 1;                                                                  \
    }                                                                            \
  } while (0)

template <typename F>
static bool throws_with(F&& f, const char* text) {
  try {
    f();
  } catch (const std::exception& e) {
    return std::strstr(e.what(), text) != nullptr;
  }
  return false;
}

int main(int argc, char** argv) {
  const bool gpu = argc > 1 && std::string(argv[1]) == "gpu";
  // null status: the C layer throws (C++ callers)
  EXPECT(throws_with([] { gauxc_molecule_natoms(nullptr, GauXCMolecule{{GauXC_Type_Molecule}, nullptr}); },
                     "Invalid Molecule handle"));

  const std::vector<gx::Atom> atoms = {{1, 0.0, 1.579252144093028, 2.174611055780858},
                                       {8, 0.0, 0.0, 0.0},
                                       {1, 0.0, 1.579252144093028, -2.174611055780858}};
  gx::Molecule mol(atoms);
  EXPECT(mol.natoms() == 3);
  std::vector<gx::Shell> shells;
  for (const auto& a : atoms) {
    const int nl[3] = {a.Z == 8 ? 10 : 5, a.Z == 8 ? 6 : 2, a.Z == 8 ? 2 : 0};
    const double a0[3] = {0.08, 0.1, 0.5};
    for (int l = 0; l < 3; ++l)
      for (int k = 0; k < nl[l]; ++k) {
        gx::Shell s;
        s.l = l;
        s.exponents = {a0[l] * std::pow(3.0, k)};
        s.coefficients = {1.0};
        s.origin[0] = a.x;
        s.origin[1] = a.y;
        s.origin[2] = a.z;
        shells.push_back(s);
      }
  }
  gx::BasisSet<double> basis(shells);
  const int64_t nbf = basis.nbf();
  EXPECT(nbf == 60 && basis.nshells() == 32);
  auto mg = gx::MolGridFactory::create_default_molgrid(mol, gx::PruningScheme::Unpruned, 512,
                                                       gx::RadialQuad::MuraKnowles,
                                                       gx::AtomicGridSizeDefault::FineGrid);
  gx::RuntimeEnvironment host_rt;
  EXPECT(host_rt.comm_rank() == 0 && host_rt.comm_size() == 1);
  EXPECT(throws_with([] { gx::DeviceRuntimeEnvironment bad(1.5); }, "fill_fraction"));
  EXPECT(throws_with([] { gx::functional_type f("B3LYP"); }, "not supported"));

  const auto ex = gpu ? gx::ExecutionSpace::Device : gx::ExecutionSpace::Host;
  gx::LoadBalancerFactory lbf(ex, "Default");
  auto lb = gpu ? lbf.get_instance(gx::DeviceRuntimeEnvironment(0.5), mol, mg, basis)
                : lbf.get_instance(host_rt, mol, mg, basis);
  EXPECT(lb.ntasks() > 0 && !lb.weights_modified() && lb.nbf() == nbf);

  gx::functional_type func("PBE");
  gx::XCIntegratorFactory<Matrix> factory(gx::ExecutionSpace::Device, "Replicated", "Default",
                                          "Default", "Default");
  auto integ = factory.get_instance(func, lb);
  EXPECT(throws_with([&] { gx::XCIntegratorFactory<Matrix>(gx::ExecutionSpace::Host, "Replicated",
                                                           "Default", "Default", "Default")
                               .get_instance(func, lb); },
                     "Device execution space only"));

  Matrix P(nbf, nbf);
  {
    Matrix C(nbf, 5);
    uint64_t x = 12345;
    for (int64_t k = 0; k < 5; ++k)
      for (int64_t i = 0; i < nbf; ++i) {
        x = x * 6364136223846793005ULL + 1442695040888963407ULL;
        C(i, k) = ((double)(x >> 11) / 9007199254740992.0 - 0.5) / std::sqrt((double)nbf);
      }
    for (int64_t j = 0; j < nbf; ++j)
      for (int64_t i = 0; i < nbf; ++i) {
        double s = 0.;
        for (int64_t k = 0; k < 5; ++k) s += C(i, k) * C(j, k);
        P(i, j) = s;
      }
  }
  EXPECT(throws_with([&] { integ.eval_exc_vxc(P); }, "Weights Have Not Been Modified"));
  EXPECT(throws_with([&] { integ.eval_exc_vxc(Matrix(nbf - 1, nbf - 1)); },
                     "P Must Have Same Dimension as Basis"));
  if (!gpu) {
    std::printf("host front end ok\n");
    return 0;
  }

  gx::MolecularWeightsFactory(gx::ExecutionSpace::Device, "Default",
                              gx::MolecularWeightsSettings{})
      .get_instance()
      .modify_weights(lb);
  EXPECT(lb.weights_modified());
  auto [EXC, VXC] = integ.eval_exc_vxc(P);
  const double exc_only = integ.eval_exc(P);
  const double den = integ.integrate_den(P);
  EXPECT(std::fabs(exc_only - EXC) <= 1e-12);
  if (argc > 2) {
    FILE* f = std::fopen(argv[2], "wb");
    EXPECT(f != nullptr);
    std::fwrite(&nbf, sizeof(int64_t), 1, f);
    std::fwrite(P.data(), sizeof(double), (size_t)(nbf * nbf), f);
    std::fwrite(VXC.data(), sizeof(double), (size_t)(nbf * nbf), f);
    std::fwrite(&EXC, sizeof(double), 1, f);
    std::fwrite(&exc_only, sizeof(double), 1, f);
    std::fwrite(&den, sizeof(double), 1, f);
    std::fclose(f);
  }
  std::printf("EXC %.15f N_el %.15f\ndevice front end ok\n", EXC, den);
  return 0;
}
