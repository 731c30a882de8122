// Host-side data model of the GB300 XC integrator: molecule, basis, grid,
// load balancer (task generation + shell screening) and the integrator
// object that owns the device-resident plan.
//
// Reference interfaces mirrored here:
//   Atom / Molecule           include/gauxc/atom.hpp, include/gauxc/molecule.hpp
//   Shell (normalize, cutoff) include/gauxc/shell.hpp:48-229
//   BasisSetMap (shell->ao)   include/gauxc/basisset_map.hpp:185-194
//   MolMeta (R_AB, nearest)   src/molmeta.cxx:28-60
//   XCTask                    include/gauxc/xc_task.hpp:25-119
//   LoadBalancer              src/load_balancer/host/replicated_host_load_balancer.cxx:22-193
#pragma once
#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace gb300 {

struct error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct Atom {
  int64_t Z;
  double x, y, z;
};
using Molecule = std::vector<Atom>;

constexpr int kMaxPrim = 32;
constexpr double kDefaultShellTol = 1e-10;

struct Shell {
  double alpha[kMaxPrim] = {};
  double coeff[kMaxPrim] = {};
  double O[3] = {};
  int32_t nprim = 0, l = 0, pure = 1;
  double cutoff_radius = 0.;
  double tol = kDefaultShellTol;

  int size() const { return pure ? 2 * l + 1 : (l + 1) * (l + 2) / 2; }
  // Primitive + contraction normalization (include/gauxc/shell.hpp:72-109).
  void normalize();
  // Radial cutoff walk (include/gauxc/util/gau_rad_eval.hpp:32-71).
  void compute_cutoff();
  void set_tolerance(double t) {
    tol = t;
    compute_cutoff();
  }
};

struct BasisSet {
  std::vector<Shell> shells;
  std::vector<int32_t> shell_offs;  // first AO of each shell
  int32_t nbf = 0;
  int max_l = 0;
  void finalize();
};

struct MolMeta {
  size_t natoms = 0;
  std::vector<double> rab;           // natoms x natoms, symmetric
  std::vector<double> dist_nearest;  // per atom
  explicit MolMeta(const Molecule& mol);
  MolMeta() = default;
};

// ---------------------------------------------------------------- grids
enum class RadialQuad { Becke = 0, MuraKnowles = 1, MurrayHandyLaming = 2, TreutlerAhlrichs = 3 };
enum class PruningScheme { Unpruned = 0, Robust = 1, Treutler = 2 };

// One atomic grid centred at the origin, already split into batches.  The
// batcher reorders points so that every batch is a contiguous range.
struct AtomicGrid {
  std::vector<std::array<double, 3>> points;
  std::vector<double> weights;
  std::vector<std::pair<int64_t, int64_t>> batches;  // [begin, end)
  int64_t max_batch = 512;
};

struct MolGrid {
  std::map<int64_t, AtomicGrid> grids;  // by atomic number
  int64_t batch_size = 512;
};

// Lebedev rule with `npts` points (throws if no rule has that size).
void lebedev_rule(int npts, std::vector<std::array<double, 3>>& pts,
                  std::vector<double>& w);
int lebedev_npts_by_order(int order);
int lebedev_order_by_npts(int npts);
int lebedev_next_order(int order);

MolGrid make_default_molgrid(const Molecule& mol, PruningScheme prune,
                             int64_t batch_size, RadialQuad rq,
                             int grid_size_enum);

// ---------------------------------------------------------------- tasks
struct XCTask {
  int32_t iParent = -1;
  std::vector<double> points;   // 3 * npts, xyz interleaved
  std::vector<double> weights;  // npts
  int32_t npts = 0;
  double dist_nearest = 0.;
  std::vector<int32_t> shell_list;
  int32_t nbe = 0;
};

struct RuntimeEnv;  // device_api.hpp

struct LoadBalancer {
  std::shared_ptr<RuntimeEnv> rt;  // device memory policy of the integrators built on it
  std::shared_ptr<const Molecule> mol;
  std::shared_ptr<const BasisSet> basis;
  std::shared_ptr<const MolGrid> molgrid;
  std::shared_ptr<MolMeta> meta;
  std::vector<XCTask> tasks;
  bool weights_modified = false;
  bool device_screening = false;
  uint64_t generation = 0;  // bumped whenever tasks/weights change
};

std::shared_ptr<LoadBalancer> make_load_balancer(
    std::shared_ptr<const Molecule> mol, std::shared_ptr<const MolGrid> mg,
    std::shared_ptr<const BasisSet> basis, bool device);

// A load balancer over tasks `idx` of `lb` (in that order, each index in
// range): same molecule, basis, grid and runtime, copies of the tasks with
// their current weights and the weights-modified state.
std::shared_ptr<LoadBalancer> load_balancer_subset(const LoadBalancer& lb,
                                                   const std::vector<int64_t>& idx);

// cube/sphere test (include/gauxc/util/geometry.hpp:36-49)
inline bool cube_sphere_intersect(const double* lo, const double* up,
                                  const double* c, double rad) {
  double dist = rad * rad;
  for (int i = 0; i < 3; ++i) {
    double r = 0.;
    if (c[i] < lo[i]) r = lo[i] - c[i];
    else if (c[i] > up[i]) r = c[i] - up[i];
    dist -= r * r;
    if (dist < 0.) return false;
  }
  return true;
}

}  // namespace gb300
