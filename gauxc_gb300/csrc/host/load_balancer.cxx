// Task generation with micro-batch shell screening and task merging.
//
// Follows src/load_balancer/host/replicated_host_load_balancer.cxx:22-193 and
// the "petite" screen of petite_replicated_load_balancer.cxx:31-65:
//   * for every atom, every batch of its (recentred) atomic grid gives one
//     task candidate whose box is the bounding box of its points;
//   * a shell is kept iff its cutoff sphere intersects the box;
//   * candidates with no shells are dropped;
//   * tasks are sorted by (iParent, shell_list) and tasks with identical
//     (iParent, shell_list) are merged by concatenating their points.
// Single-process build: every task is local (the reference's rank assignment
// by XCTask::cost is the identity for one rank).  The Device load balancer
// screens the candidate boxes on the GPU (screening.cu) and gives the same
// task list.
#include "core.hpp"
#include "device_api.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <exception>
#include <limits>
#include <thread>

namespace gb300 {

namespace {

std::vector<int32_t> screen_box(const BasisSet& bs, const double* lo, const double* up,
                                int32_t& nbe) {
  std::vector<int32_t> list;
  nbe = 0;
  for (size_t s = 0; s < bs.shells.size(); ++s) {
    const Shell& sh = bs.shells[s];
    if (cube_sphere_intersect(lo, up, sh.O, sh.cutoff_radius)) {
      list.push_back((int32_t)s);
      nbe += sh.size();
    }
  }
  return list;
}

}  // namespace

std::shared_ptr<LoadBalancer> make_load_balancer(std::shared_ptr<const Molecule> mol,
                                                 std::shared_ptr<const MolGrid> mg,
                                                 std::shared_ptr<const BasisSet> basis,
                                                 bool device) {
  auto lb = std::make_shared<LoadBalancer>();
  lb->mol = mol;
  lb->molgrid = mg;
  lb->basis = basis;
  lb->meta = std::make_shared<MolMeta>(*mol);
  lb->device_screening = device;

  // Task candidates of every atom (points, weights, the batch's bounding box),
  // atoms spread over host threads; the lists are joined in atom order, so
  // the result does not depend on the threads.  The host screens each box as
  // it goes; the Device load balancer screens all boxes in one kernel.
  const size_t nat = mol->size();
  std::vector<std::vector<XCTask>> per_atom(nat);
  std::vector<std::vector<double>> per_atom_box(nat);
  auto parallel_atoms = [&](auto&& fn) {
    const size_t nth = std::min<size_t>(nat, std::max(1u, std::thread::hardware_concurrency()));
    std::atomic<size_t> next{0};
    std::exception_ptr failure;
    std::atomic<bool> failed{false};
    auto worker = [&]() {
      for (size_t i; !failed && (i = next++) < nat;) {
        try {
          fn(i);
        } catch (...) {
          if (!failed.exchange(true)) failure = std::current_exception();
        }
      }
    };
    std::vector<std::thread> pool;
    for (size_t k = 1; k < nth; ++k) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
    if (failure) std::rethrow_exception(failure);
  };
  parallel_atoms([&](size_t iat) {
    const Atom& at = (*mol)[iat];
    const double c[3] = {at.x, at.y, at.z};
    const AtomicGrid& g = mg->grids.at(at.Z);
    for (const auto& b : g.batches) {
      const int64_t n = b.second - b.first;
      if (n == 0) continue;
      XCTask t;
      t.iParent = (int32_t)iat;
      t.npts = (int32_t)n;
      t.points.resize(3 * n);
      t.weights.resize(n);
      double lo[3] = {std::numeric_limits<double>::infinity(),
                      std::numeric_limits<double>::infinity(),
                      std::numeric_limits<double>::infinity()};
      double up[3] = {-lo[0], -lo[1], -lo[2]};
      for (int64_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) {
          const double v = g.points[b.first + i][a] + c[a];
          t.points[3 * i + a] = v;
          lo[a] = std::min(lo[a], v);
          up[a] = std::max(up[a], v);
        }
        t.weights[i] = g.weights[b.first + i];
      }
      if (device) {
        per_atom_box[iat].insert(per_atom_box[iat].end(), {lo[0], lo[1], lo[2], up[0], up[1], up[2]});
      } else {
        t.shell_list = screen_box(*basis, lo, up, t.nbe);
        if (t.shell_list.empty()) continue;
      }
      t.dist_nearest = lb->meta->dist_nearest[iat];
      per_atom[iat].push_back(std::move(t));
    }
  });
  if (device) {
    // collision bitset of every candidate box on the device, decoded per atom
    std::vector<size_t> first(nat + 1, 0);
    for (size_t i = 0; i < nat; ++i) first[i + 1] = first[i] + per_atom[i].size();
    std::vector<double> boxes;
    boxes.reserve(6 * first[nat]);
    for (const auto& v : per_atom_box) boxes.insert(boxes.end(), v.begin(), v.end());
    std::vector<uint32_t> bits;
    int nwords = 0;
    screen_boxes_device(boxes, *basis, bits, nwords);
    parallel_atoms([&](size_t iat) {
      std::vector<XCTask> kept;
      for (size_t k = 0; k < per_atom[iat].size(); ++k) {
        XCTask& t = per_atom[iat][k];
        const uint32_t* w = bits.data() + (first[iat] + k) * (size_t)nwords;
        t.nbe = 0;
        for (int q = 0; q < nwords; ++q)
          for (uint32_t m = w[q]; m; m &= m - 1) {
            const int sh = 32 * q + __builtin_ctz(m);
            t.shell_list.push_back(sh);
            t.nbe += basis->shells[sh].size();
          }
        if (!t.shell_list.empty()) kept.push_back(std::move(t));
      }
      per_atom[iat].swap(kept);
    });
  }
  // Sort each atom's tasks by shell list and merge equal lists (their points
  // joined in batch order), atoms in parallel: every task of a list has one
  // parent, so this is the global stable sort by (iParent, shell_list) and
  // merge of the Default load balancer, done per parent.
  parallel_atoms([&](size_t iat) {
    std::vector<XCTask>& v = per_atom[iat];
    std::stable_sort(v.begin(), v.end(), [](const XCTask& a, const XCTask& b) {
      return a.shell_list < b.shell_list;
    });
    std::vector<XCTask> merged;
    for (auto& t : v) {
      if (!merged.empty() && merged.back().shell_list == t.shell_list) {
        XCTask& m = merged.back();
        m.points.insert(m.points.end(), t.points.begin(), t.points.end());
        m.weights.insert(m.weights.end(), t.weights.begin(), t.weights.end());
        m.npts += t.npts;
      } else {
        merged.push_back(std::move(t));
      }
    }
    v.swap(merged);
  });
  size_t ntask = 0;
  for (const auto& v : per_atom) ntask += v.size();
  std::vector<XCTask> merged;
  merged.reserve(ntask);
  for (auto& v : per_atom)
    for (auto& t : v) merged.push_back(std::move(t));
  lb->tasks = std::move(merged);
  lb->generation++;
  return lb;
}

std::shared_ptr<LoadBalancer> load_balancer_subset(const LoadBalancer& lb,
                                                   const std::vector<int64_t>& idx) {
  auto sub = std::make_shared<LoadBalancer>();
  sub->rt = lb.rt;
  sub->mol = lb.mol;
  sub->basis = lb.basis;
  sub->molgrid = lb.molgrid;
  sub->meta = lb.meta;
  sub->device_screening = lb.device_screening;
  sub->weights_modified = lb.weights_modified;
  sub->tasks.reserve(idx.size());
  for (int64_t i : idx) {
    if (i < 0 || i >= (int64_t)lb.tasks.size()) throw error("task index out of range");
    sub->tasks.push_back(lb.tasks[i]);
  }
  sub->generation = lb.generation + 1;
  return sub;
}

}  // namespace gb300
