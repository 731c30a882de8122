// Atomic quadratures (radial x Lebedev), pruning schemes and the point batcher.
//
// Reference behaviour followed:
//   default grid sizes           src/molgrid_defaults.cxx:144-202
//   Mura-Knowles scale factors   src/molgrid_defaults.cxx:52-70
//   Treutler / Robust pruning    src/grid_factory.cxx:158-222
//   pruned grid assembly         src/grid_factory.cxx:72-86 (RadialGridPartition)
// The radial rule and the Lebedev sets come from their published definitions
// (Mura & Knowles, JCP 104, 9848 (1996); Lebedev & Laikov, Dokl. Math. 59,
// 477 (1999)); the orbit table is generated by gen_lebedev.py.
//
// Batching: the reference delegates to a third-party batcher that is not part
// of its source tree.  This build partitions every atomic grid with its own
// octree: the cube [-rmax, rmax]^3 is split at its geometric centre into eight
// octants (octant bit a set when coordinate a >= the split value), recursively,
// until a cell holds at most `batch_size` points.  The partition is stable
// (points keep quadrature order inside a batch) and empty cells are dropped.
#include "core.hpp"

#include <algorithm>
#include <cmath>
#include <functional>
#include <set>

namespace gb300 {

#include "lebedev_orbits.inc"

namespace {
constexpr int kNumRules = sizeof(kLebedevRules) / sizeof(kLebedevRules[0]);

const int* find_rule_by_npts(int npts) {
  for (int i = 0; i < kNumRules; ++i)
    if (kLebedevRules[i][1] == npts) return kLebedevRules[i];
  return nullptr;
}
}  // namespace

int lebedev_npts_by_order(int order) {
  for (int i = 0; i < kNumRules; ++i)
    if (kLebedevRules[i][0] == order) return kLebedevRules[i][1];
  return -1;
}
int lebedev_order_by_npts(int npts) {
  const int* r = find_rule_by_npts(npts);
  return r ? r[0] : -1;
}
int lebedev_next_order(int order) {
  for (int i = 0; i < kNumRules; ++i)
    if (kLebedevRules[i][0] >= order) return kLebedevRules[i][0];
  return -1;
}

// Expand every orbit representative (|c0|>=|c1|>=|c2|) into all distinct
// coordinate permutations and sign choices.
void lebedev_rule(int npts, std::vector<std::array<double, 3>>& pts,
                  std::vector<double>& w) {
  const int* rule = find_rule_by_npts(npts);
  if (!rule) throw error("no Lebedev rule with " + std::to_string(npts) + " points");
  pts.clear();
  w.clear();
  static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2},
                                  {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  for (int o = 0; o < rule[2]; ++o) {
    const double* d = kLebedevOrbitData[rule[3] + o];
    const int size = (int)d[4];
    std::set<std::array<double, 3>> seen;
    for (int p = 0; p < 6; ++p)
      for (int s = 0; s < 8; ++s) {
        std::array<double, 3> v;
        for (int a = 0; a < 3; ++a) {
          const double c = d[perms[p][a]];
          v[a] = ((s >> a) & 1) ? -c : c;
          if (v[a] == 0.) v[a] = 0.;  // fold -0 into +0
        }
        if (seen.insert(v).second) {
          pts.push_back(v);
          w.push_back(d[3]);
        }
      }
    if ((int)seen.size() != size) throw error("Lebedev orbit expansion mismatch");
  }
}

namespace {

// Mura-Knowles radial rule (m = 3): x_i = i/(N+1),
// r_i = -alpha ln(1 - x_i^3), w_i = 3 alpha x_i^2 / ((1-x_i^3)(N+1)) * r_i^2.
void mura_knowles(int n, double alpha, std::vector<double>& r, std::vector<double>& w) {
  r.resize(n);
  w.resize(n);
  const double inv = 1. / (n + 1);
  for (int i = 0; i < n; ++i) {
    const double x = (i + 1) * inv;
    const double x3 = x * x * x;
    const double ri = -alpha * std::log(1. - x3);
    r[i] = ri;
    w[i] = 3. * alpha * x * x / (1. - x3) * inv * ri * ri;
  }
}

double mk_scale(int64_t Z) {
  switch (Z) {
    case 3: case 4: case 11: case 12: case 19: case 20:
    case 37: case 38: case 55: case 56: case 87: case 88:
      return 7.0;
    default:
      return 5.0;
  }
}

struct Region {
  int r_begin, r_end, nang;
};

void default_sizes(int64_t Z, int grid, int& nrad, int& nang) {
  switch (grid) {
    case 0: nrad = 75; nang = 302; return;                 // Fine
    case 1: nrad = 99; nang = 590; return;                 // UltraFine
    case 2: nrad = (Z <= 2) ? 175 : 250; nang = 974; return;  // SuperFine
    case 3: nrad = 35; nang = 110; return;                 // GM3
    case 4: nrad = 50; nang = 302; return;                 // GM5
    default: throw error("grid size default not supported in this build");
  }
}

std::vector<Region> pruning_regions(PruningScheme s, int nrad, int nang) {
  if (s == PruningScheme::Unpruned) return {{0, nrad, nang}};
  const int low = lebedev_npts_by_order(7);
  if (s == PruningScheme::Treutler) {
    const int med = lebedev_npts_by_order(11);
    const int r3 = nrad / 3 + 1, r2 = nrad / 2 + 1;
    return {{0, r3, low}, {r3, r2, med}, {r2, nrad, nang}};
  }
  // Robust (Psi4) scheme
  const int base = lebedev_order_by_npts(nang);
  if (base < 0) throw error("invalid base angular grid");
  const int med_order = lebedev_next_order(base > 6 ? base - 6 : base);
  const int med = lebedev_npts_by_order(med_order);
  const int r4 = nrad / 4 + 1, r2 = nrad / 2 + 1;
  return {{0, r4, low}, {r4, r2, med}, {r2, nrad, nang}};
}

void octree_batches(AtomicGrid& g) {
  const int64_t n = (int64_t)g.points.size();
  double rmax = 0.;
  for (auto& p : g.points)
    for (int a = 0; a < 3; ++a) rmax = std::max(rmax, std::abs(p[a]));
  std::vector<int64_t> idx(n);
  for (int64_t i = 0; i < n; ++i) idx[i] = i;
  std::vector<int64_t> order;
  order.reserve(n);
  std::vector<std::pair<int64_t, int64_t>> batches;

  std::function<void(std::vector<int64_t>&, std::array<double, 3>, std::array<double, 3>)> rec =
      [&](std::vector<int64_t>& ids, std::array<double, 3> lo, std::array<double, 3> up) {
        if ((int64_t)ids.size() <= g.max_batch) {
          if (!ids.empty()) {
            batches.push_back({(int64_t)order.size(), (int64_t)(order.size() + ids.size())});
            order.insert(order.end(), ids.begin(), ids.end());
          }
          return;
        }
        std::array<double, 3> mid;
        for (int a = 0; a < 3; ++a) mid[a] = 0.5 * (lo[a] + up[a]);
        std::vector<int64_t> oct[8];
        for (int64_t i : ids) {
          int k = 0;
          for (int a = 0; a < 3; ++a)
            if (g.points[i][a] >= mid[a]) k |= (1 << a);
          oct[k].push_back(i);
        }
        for (int k = 0; k < 8; ++k) {
          std::array<double, 3> l2 = lo, u2 = up;
          for (int a = 0; a < 3; ++a) {
            if ((k >> a) & 1) l2[a] = mid[a];
            else u2[a] = mid[a];
          }
          rec(oct[k], l2, u2);
        }
      };
  rec(idx, {-rmax, -rmax, -rmax}, {rmax, rmax, rmax});

  std::vector<std::array<double, 3>> p2(n);
  std::vector<double> w2(n);
  for (int64_t i = 0; i < n; ++i) {
    p2[i] = g.points[order[i]];
    w2[i] = g.weights[order[i]];
  }
  g.points.swap(p2);
  g.weights.swap(w2);
  g.batches.swap(batches);
}

AtomicGrid make_atomic_grid(int64_t Z, PruningScheme prune, RadialQuad rq,
                            int grid, int64_t batch) {
  if (rq != RadialQuad::MuraKnowles)
    throw error("only the Mura-Knowles radial quadrature is built in this library");
  int nrad, nang;
  default_sizes(Z, grid, nrad, nang);
  std::vector<double> r, wr;
  mura_knowles(nrad, mk_scale(Z), r, wr);
  AtomicGrid g;
  g.max_batch = batch;
  for (const auto& reg : pruning_regions(prune, nrad, nang)) {
    std::vector<std::array<double, 3>> ang;
    std::vector<double> wa;
    lebedev_rule(reg.nang, ang, wa);
    for (int i = reg.r_begin; i < reg.r_end; ++i)
      for (size_t j = 0; j < ang.size(); ++j) {
        g.points.push_back({r[i] * ang[j][0], r[i] * ang[j][1], r[i] * ang[j][2]});
        g.weights.push_back(wr[i] * wa[j]);
      }
  }
  octree_batches(g);
  return g;
}

}  // namespace

MolGrid make_default_molgrid(const Molecule& mol, PruningScheme prune,
                             int64_t batch_size, RadialQuad rq, int grid_size_enum) {
  if (batch_size <= 0) throw error("batch size must be positive");
  MolGrid mg;
  mg.batch_size = batch_size;
  for (const auto& a : mol)
    if (!mg.grids.count(a.Z))
      mg.grids.emplace(a.Z, make_atomic_grid(a.Z, prune, rq, grid_size_enum, batch_size));
  return mg;
}

}  // namespace gb300
