// Device-resident plan and the per-iteration stage loop of eval_exc_vxc.
//
// Reference driver: IncoreReplicatedXCDeviceIntegrator::eval_exc_vxc_ /
// exc_vxc_local_work_ (src/xc_integrator/replicated/device/
// incore_replicated_xc_device_integrator_exc_vxc.hpp:46-412):
//   * dims checked (m == n == nbf, ld >= nbf), weights must be modified,
//   * tasks sorted by npts * nbe (descending),
//   * P sent to the device, EXC / N_el / VXC zeroed,
//   * per task batch: collocation, X, vvars/uvars, functional, EXC/N_el,
//     Z, VXC increment,
//   * symmetrize, copy EXC / VXC back.
// Differences by design: the plan (tasks, points, weights, shell->column maps,
// work lists) is built once per load-balancer state and stays resident across
// SCF iterations, so a call moves only P in and VXC out; every stage is a
// single launch over all tasks of a batch, driven by precomputed work lists.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <iterator>
#include <thread>

#include "../host/device_api.hpp"
#include "device_common.cuh"
#include "functionals.cuh"
#include "xc_kernels.cuh"
#include "xc_mixed.cuh"

namespace gb300 {

int cuda_device_count() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

namespace {

int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// Device allocation from a caller buffer (bump) or cudaMalloc.
class Arena {
 public:
  explicit Arena(RuntimeEnv* rt) : rt_(rt) {}
  ~Arena() {
    for (void* p : owned_) cudaFree(p);
  }
  template <typename T>
  T* alloc(size_t n) {
    const size_t bytes = std::max<size_t>(n * sizeof(T), 256);
    if (rt_ && rt_->user_mem) {
      const size_t off = (rt_->user_used + 255) / 256 * 256;
      if (off + bytes > rt_->user_bytes)
        throw error("device memory buffer given to the runtime environment is too small");
      rt_->user_used = off + bytes;
      return reinterpret_cast<T*>(static_cast<char*>(rt_->user_mem) + off);
    }
    void* p = nullptr;
    GB300_CUDA(cudaMalloc(&p, bytes));
    owned_.push_back(p);
    return static_cast<T*>(p);
  }
  template <typename T>
  T* upload(const std::vector<T>& v, cudaStream_t s) {
    T* d = alloc<T>(v.size());
    if (!v.empty())
      GB300_CUDA(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return d;
  }

 private:
  RuntimeEnv* rt_;
  std::vector<void*> owned_;
};

struct Batch {
  int t_begin, t_end;
  int coll_begin, coll_end;
  int dens_begin, dens_end;
  int vxc_begin, vxc_end;
  int64_t g0 = 0, g1 = 0;  // padded point range of the batch's tasks
};

// One batch of point blocks of the mixed path.
struct MBatch {
  int b0, b1;                // point blocks
  int coll_begin, coll_end;  // collocation items
  int x_begin, x_end;        // density GEMM tiles
  int v_begin, v_end;        // VXC GEMM tiles
  int64_t g0, g1;            // point range
  int max_nu_pad;
  int partial_base;
  int x_sched, x_ncl;        // persistent-launch schedules (offsets into sched_, clusters)
  int v_sched, v_ncl;
};

}  // namespace

class DeviceIntegrator {
 public:
  DeviceIntegrator(const LoadBalancer& lb, const XCFunctionalDesc& f, Precision prec,
                   RuntimeEnv& rt, const PlanParams& pp)
      : func_(f), prec_(prec), params_(pp), arena_(&rt), rt_(&rt) {
    if (cuda_device_count() == 0) throw error("no CUDA device available for the device integrator");
    GB300_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    {
      // the device can address pageable host memory (coherent host link):
      // P and VXC move by kernels reading / writing the caller's buffers
      int dev = 0, pma = 0;
      GB300_CUDA(cudaGetDevice(&dev));
      GB300_CUDA(cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev));
      host_direct_ = pma != 0;
    }
    for (auto& e : ev_) GB300_CUDA(cudaEventCreate(&e));
    build(lb);
  }
  ~DeviceIntegrator() {
    for (auto& e : pev_) cudaEventDestroy(e);
    for (auto& e : ev_) cudaEventDestroy(e);
    if (stream_) cudaStreamDestroy(stream_);
  }

  uint64_t generation = 0;
  PlanStats stats;
  std::map<std::string, double> timings;
  bool profiling = false;
  // tensor-core pipeline: bound of every wait, and the error-path check
  // (producers issue no copy; see OzSchedule)
  uint64_t wait_ns = kOzWaitNs;
  bool withhold = false;
  // per kernel class: accumulated ms and launch count of the last call
  // collocation, density, zmat, vxc, other, phi digits (+ point scales), P digits
  double kclass_ms[7] = {0, 0, 0, 0, 0, 0, 0};
  int64_t kclass_n[7] = {0, 0, 0, 0, 0, 0, 0};

  void eval(const double* P, int64_t ldp, double* VXC, int64_t ldvxc, double* EXC, double* NEL,
            bool den_only);
  // UKS: Ps = P_a + P_b, Pz = P_a - P_b in, VXC_s / VXC_z out (both null: EXC only).
  void eval_uks(const double* Ps, int64_t ldps, const double* Pz, int64_t ldpz, double* VXCs,
                int64_t ldvs, double* VXCz, int64_t ldvz, double* EXC, double* NEL);
  // All device work of one call on this integrator's stream, without waiting:
  // P (host, ld ldp) in, VXC (host, ld ldvxc) out when do_vxc, {EXC, N_el}
  // into en_host and the pipeline error flag into err_host.  Host buffers must
  // be page-locked when the call is captured into a CUDA graph.  Returns the
  // number of kernel launches.
  int64_t enqueue(const double* P, int64_t ldp, double* VXC, int64_t ldvxc, double* en_host,
                  int* err_host, bool do_vxc, bool events);
  cudaStream_t stream() const { return stream_; }
  int nbf() const { return nbf_; }

 private:
  void build(const LoadBalancer& lb);
  void build_mixed(const LoadBalancer& lb);
  int64_t eval_mixed_batches(bool do_vxc);
  int64_t eval_mixed_batches_uks(bool do_vxc);
  int64_t enqueue_uks(const double* Ps, int64_t ldps, const double* Pz, int64_t ldpz,
                      double* VXCs, int64_t ldvs, double* VXCz, int64_t ldvz, double* en_host,
                      int* err_host, bool do_vxc);
  // brings a caller density matrix in as c P (c a power of two), in the
  // device AO order; `stage` (n x n) receives the caller's matrix first when
  // that order is a permutation
  int64_t load_density(const double* P, int64_t ldp, double* dst, double c, double* stage);
  // VXC = A + A^T, in the caller's AO order, into V (device or host memory the
  // device addresses)
  void symmetrize_out(const double* A, double* V, int64_t ld);
  // VXC = A + A^T out to the caller (host_direct_: straight; otherwise staged)
  int64_t store_vxc(const double* A, double* stage, double* VXC, int64_t ldvxc);
  void ensure_uks();

  XCFunctionalDesc func_;
  Precision prec_;
  PlanParams params_;
  Arena arena_;
  RuntimeEnv* rt_;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev_[4];

  int nbf_ = 0;
  bool gga_ = false;
  ShellsDev sh_{};
  TasksDev tk_{};
  std::vector<Batch> batches_;
  int2* coll_items_ = nullptr;
  int2* dens_items_ = nullptr;
  int4* vxc_items_ = nullptr;
  int ndens_ = 0;
  double* scr_ = nullptr;
  double4* zcoef_ = nullptr;
  double2* partials_ = nullptr;
  bool host_direct_ = false;  // P / VXC moved by kernels (pageable memory access)
  double* P_ = nullptr;
  double* A_ = nullptr;
  double* V_ = nullptr;
  double* out_ = nullptr;
  // mixed path: P_ and A_ are held in a permuted AO order (perm_: position ->
  // caller's AO index, iperm_ its inverse); null on the FP64 path
  int* perm_ = nullptr;
  int* iperm_ = nullptr;
  int64_t npts_plan_ = 0;
  // UKS work space (first polarized call): the z density, its VXC
  // accumulator (and staging), (rho, grad rho) of both densities, Z_z
  // coefficients, P_z row scales, functional partials of the FP64 path
  bool uks_ready_ = false;
  double* Pz_ = nullptr;
  double* Az_ = nullptr;
  double* Vz_ = nullptr;
  double* rho4s_ = nullptr;
  double* rho4z_ = nullptr;
  double4* zcoefz_ = nullptr;
  double* prsz_ = nullptr;
  double2* partials_pol_ = nullptr;
  int npol_ = 0;
  // mixed path (point blocks)
  PBMaskDev mk_{};
  MixedPBDev mp_{};
  std::vector<MBatch> mbatches_;
  OzItem* slots_ = nullptr;
  std::vector<int> zoff_h_;   // host copy of MixedPBDev::zoff  // GEMM slots of every launch (kCluster tiles each)
  int* sched_ = nullptr;
  double* f64_ = nullptr;
  __nv_bfloat16* dig_ = nullptr;
  double* rho4_ = nullptr;
  double* prs_ = nullptr;  // row scales of P
  int* err_ = nullptr;
  std::vector<cudaEvent_t> pev_;
  std::vector<int> pev_class_;
  size_t pev_used_ = 0;
  // bracket one launch of kernel class k with events when profiling
  template <typename F>
  int64_t timed(int k, F&& launch) {
    if (!profiling) return launch();
    while (pev_.size() < pev_used_ + 2) {
      cudaEvent_t e;
      GB300_CUDA(cudaEventCreate(&e));
      pev_.push_back(e);
      pev_class_.push_back(0);
    }
    GB300_CUDA(cudaEventRecord(pev_[pev_used_], stream_));
    const int64_t n = launch();
    GB300_CUDA(cudaEventRecord(pev_[pev_used_ + 1], stream_));
    pev_class_[pev_used_] = k;
    pev_class_[pev_used_ + 1] = (int)n;
    pev_used_ += 2;
    return n;
  }
};

void DeviceIntegrator::build(const LoadBalancer& lb) {
  const BasisSet& bs = *lb.basis;
  nbf_ = bs.nbf;
  gga_ = func_.is_gga != 0;
  cudaStream_t s = stream_;

  // ---- shells
  {
    std::vector<double> a, c, o;
    std::vector<int> off{0}, l, pure;
    for (const auto& sh : bs.shells) {
      if (sh.l > 4) throw error("device collocation supports l <= 4");
      for (int k = 0; k < sh.nprim; ++k) {
        a.push_back(sh.alpha[k]);
        c.push_back(sh.coeff[k]);
      }
      off.push_back((int)a.size());
      o.insert(o.end(), sh.O, sh.O + 3);
      l.push_back(sh.l);
      pure.push_back(sh.pure);
    }
    sh_.nshells = (int)bs.shells.size();
    sh_.alpha = arena_.upload(a, s);
    sh_.coeff = arena_.upload(c, s);
    sh_.prim_off = arena_.upload(off, s);
    sh_.origin = arena_.upload(o, s);
    sh_.l = arena_.upload(l, s);
    sh_.pure = arena_.upload(pure, s);
    sh_.exp2_tab = arena_.upload(exp2_table(), s);
  }

  P_ = arena_.alloc<double>((size_t)nbf_ * nbf_);
  A_ = arena_.alloc<double>((size_t)nbf_ * nbf_);
  if (!host_direct_) V_ = arena_.alloc<double>((size_t)nbf_ * nbf_);  // staging for the copy out
  out_ = arena_.alloc<double>(2);
  err_ = arena_.alloc<int>(1);
  GB300_CUDA(cudaMemsetAsync(err_, 0, sizeof(int), s));
  if (prec_ == Precision::Mixed) {
    const auto t0 = std::chrono::steady_clock::now();
    build_mixed(lb);
    if (func_.polarized) ensure_uks();
    GB300_CUDA(cudaStreamSynchronize(s));
    timings["plan_ms"] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    generation = lb.generation;
    return;
  }

  // ---- task order: npts * nbe descending (stable)
  const auto& tasks = lb.tasks;
  std::vector<int> order(tasks.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (int64_t)tasks[a].npts * tasks[a].nbe > (int64_t)tasks[b].npts * tasks[b].nbe;
  });

  const int nt = (int)tasks.size();
  std::vector<int64_t> pt_off(nt), bf_off(nt), sh_off(nt), scr_off(nt);
  std::vector<int> npts_pad(nt), nbe(nt), nbe_pad(nt), nsh(nt);
  std::vector<int> bf_list, sh_list, sh_col;
  std::vector<double> X, Y, Z, W;
  const int nblk = gga_ ? 5 : 2;
  stats = PlanStats{};
  int64_t pts = 0;
  for (int i = 0; i < nt; ++i) {
    const XCTask& t = tasks[order[i]];
    pt_off[i] = pts;
    npts_pad[i] = (int)round_up(t.npts, kPtBlock);
    for (int p = 0; p < npts_pad[i]; ++p) {
      const int q = p < t.npts ? p : 0;
      X.push_back(t.points[3 * q + 0]);
      Y.push_back(t.points[3 * q + 1]);
      Z.push_back(t.points[3 * q + 2]);
      W.push_back(p < t.npts ? t.weights[p] : 0.);
    }
    pts += npts_pad[i];
    bf_off[i] = (int64_t)bf_list.size();
    sh_off[i] = (int64_t)sh_list.size();
    int col = 0;
    for (int s_ : t.shell_list) {
      sh_list.push_back(s_);
      sh_col.push_back(col);
      const int sz = bs.shells[s_].size();
      for (int k = 0; k < sz; ++k) bf_list.push_back(bs.shell_offs[s_] + k);
      col += sz;
    }
    nsh[i] = (int)t.shell_list.size();
    nbe[i] = col;
    if (col != t.nbe) throw error("task nbe does not match its shell list");
    nbe_pad[i] = (int)round_up(col, kBfBlock);
    for (int k = col; k < nbe_pad[i]; ++k) bf_list.push_back(-1);
    stats.npts += t.npts;
    stats.sum_npts_nbe += (double)t.npts * t.nbe;
    stats.sum_npts_nbe2 += (double)t.npts * t.nbe * t.nbe;
    stats.sum_pad_npts_nbe2 += (double)npts_pad[i] * nbe_pad[i] * nbe_pad[i];
    {
      // algorithmic bytes: phi (and grad phi) written by the collocation and
      // read by density, zmat (Z written) and vxc; P_sub read by the density
      // kernel, the task's VXC block read-modify-written once
      const double pe = (double)t.npts * t.nbe * 8.;
      const double nq = gga_ ? 4. : 1.;
      stats.kbytes[0] += nq * pe;
      stats.kbytes[1] += nq * pe + 8. * t.nbe * t.nbe + 32. * t.npts;
      stats.kbytes[2] += nq * pe + pe + 32. * t.npts;
      stats.kbytes[3] += 2. * pe + 16. * t.nbe * t.nbe;
    }
  }
  stats.ntasks = nt;
  stats.npts_pad = pts;

  // ---- batches under the scratch budget
  size_t free_b = 0, total_b = 0;
  GB300_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const double nbf2 = (double)nbf_ * nbf_ * 8.;
  double static_bytes = 3 * nbf2 + pts * (4 * 8. + 32.) + bf_list.size() * 4. + 1e6;
  if (func_.polarized) static_bytes += 3 * nbf2 + pts * (2 * 32. + 32.);  // ensure_uks
  double budget;
  if (rt_->user_mem)
    budget = (double)rt_->user_bytes - rt_->user_used - static_bytes - 64e6;
  else
    budget = rt_->fill_fraction * (double)free_b - static_bytes;
  if (const char* cap = std::getenv("GAUXC_GB300_SCRATCH_GB")) budget = std::min(budget, atof(cap) * 1e9);
  if (params_.scratch_bytes > 0.) budget = std::min(budget, params_.scratch_bytes);
  budget = std::min(budget, 128e9);
  std::vector<int2> coll, dens;
  std::vector<int4> vx;
  double used = 0., max_used = 0.;
  Batch cur{0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < nt; ++i) {
    const double need = (double)nblk * npts_pad[i] * nbe_pad[i] * 8.;
    if (need > budget) throw error("insufficient device memory for one task's scratch");
    if (used + need > budget && i > cur.t_begin) {
      cur.t_end = i;
      cur.coll_end = (int)coll.size();
      cur.dens_end = (int)dens.size();
      cur.vxc_end = (int)vx.size();
      batches_.push_back(cur);
      cur = Batch{i, i, (int)coll.size(), 0, (int)dens.size(), 0, (int)vx.size(), 0};
      used = 0.;
    }
    scr_off[i] = (int64_t)(used / 8.);
    used += need;
    max_used = std::max(max_used, used);
    for (int b = 0; b < (npts_pad[i] + 127) / 128; ++b) coll.push_back(make_int2(i, b));
    for (int b = 0; b < npts_pad[i] / kPtBlock; ++b) dens.push_back(make_int2(i, b));
    const int nb = nbe_pad[i] / kBfBlock;
    for (int I = 0; I < nb; ++I)
      for (int J = 0; J < nb; ++J) vx.push_back(make_int4(i, I, J, 0));
  }
  cur.t_end = nt;
  cur.coll_end = (int)coll.size();
  cur.dens_end = (int)dens.size();
  cur.vxc_end = (int)vx.size();
  if (nt > 0) batches_.push_back(cur);
  for (Batch& b : batches_) {
    b.g0 = pt_off[b.t_begin];
    b.g1 = pt_off[b.t_end - 1] + npts_pad[b.t_end - 1];
  }
  npts_plan_ = pts;
  stats.nbatches = (int64_t)batches_.size();
  stats.scratch_bytes = max_used;

  tk_.ntasks = nt;
  tk_.pt_off = arena_.upload(pt_off, s);
  tk_.npts_pad = arena_.upload(npts_pad, s);
  tk_.nbe = arena_.upload(nbe, s);
  tk_.nbe_pad = arena_.upload(nbe_pad, s);
  tk_.bf_off = arena_.upload(bf_off, s);
  tk_.bf_list = arena_.upload(bf_list, s);
  tk_.sh_off = arena_.upload(sh_off, s);
  tk_.nsh = arena_.upload(nsh, s);
  tk_.sh_list = arena_.upload(sh_list, s);
  tk_.sh_col = arena_.upload(sh_col, s);
  tk_.scr_off = arena_.upload(scr_off, s);
  tk_.x = arena_.upload(X, s);
  tk_.y = arena_.upload(Y, s);
  tk_.z = arena_.upload(Z, s);
  tk_.w = arena_.upload(W, s);
  coll_items_ = arena_.upload(coll, s);
  dens_items_ = arena_.upload(dens, s);
  vxc_items_ = arena_.upload(vx, s);
  ndens_ = (int)dens.size();
  scr_ = arena_.alloc<double>((size_t)(max_used / 8.) + 1);
  zcoef_ = arena_.alloc<double4>(std::max<int64_t>(pts, 1));
  partials_ = arena_.alloc<double2>(std::max(ndens_, 1));
  if (func_.polarized) ensure_uks();
  GB300_CUDA(cudaStreamSynchronize(s));
  generation = lb.generation;
}

void DeviceIntegrator::ensure_uks() {
  if (uks_ready_) return;
  const size_t n2 = (size_t)nbf_ * nbf_;
  const size_t np = (size_t)std::max<int64_t>(npts_plan_, 1);
  Pz_ = arena_.alloc<double>(n2);
  Az_ = arena_.alloc<double>(n2);
  if (!host_direct_) Vz_ = arena_.alloc<double>(n2);
  rho4s_ = prec_ == Precision::Mixed ? rho4_ : arena_.alloc<double>(4 * np);
  rho4z_ = arena_.alloc<double>(4 * np);
  zcoefz_ = arena_.alloc<double4>(np);
  const int nb = prec_ == Precision::Mixed ? (int)mbatches_.size() : (int)batches_.size();
  npol_ = std::max(nb, 1) * functional_partial_blocks();
  if (prec_ == Precision::Mixed) {
    prsz_ = arena_.alloc<double>((size_t)nbf_);
    partials_pol_ = partials_;  // one block of partials per batch, as the RKS pass
  } else {
    partials_pol_ = arena_.alloc<double2>((size_t)npol_);
  }
  uks_ready_ = true;
}

// Padded tensor-core work of one point block: density GEMM (M = basis rows
// padded to kMTile, N = points padded to kNTile, K = basis padded to kBK)
// plus the symmetric VXC GEMM (about half the M x N basis tiles, K = 2 points
// padded to kBK).
static double pb_cost(int npts, int nu, double nu2_weight) {
  const double np = (double)round_up(npts, kNTile), nk = (double)round_up(npts, kBK);
  const double m = (double)round_up(nu, kMTile), n = (double)round_up(nu, kNTile),
               k = (double)round_up(nu, kBK);
  return m * np * k + m * n * nk + nu2_weight * m * n;
}

// Point blocks for the tensor-core path: consecutive tasks (in the spatial
// order below) are merged while the block holds at most
// kPBMaxPts points and the padded GEMM work of the merged block plus the
// union-size term does not exceed that of its parts kept apart; a task larger
// than kPBMaxPts points is split.  Padded extents: PBDims.
void DeviceIntegrator::build_mixed(const LoadBalancer& lb) {
  const auto t_plan0 = std::chrono::steady_clock::now();
  auto ms_since = [](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  };
  const BasisSet& bs = *lb.basis;
  cudaStream_t s = stream_;
  const auto& tasks = lb.tasks;
  struct Seg {
    int task, p0, p1;
  };
  struct PB {
    std::vector<Seg> segs;
    std::vector<int> shells;  // union, in device AO order
    int nu = 0, npts = 0;
  };
  const int maxp = std::max(kNTile, std::min(kPBMaxPts, params_.pb_max_pts / kNTile * kNTile));
  const double w2 = std::max(0., params_.nu2_weight);
  // Device AO order.  A block's union basis holds, for every cutoff radius,
  // the shells of that radius whose centres lie within reach of its points:
  // in the caller's order (atom by atom) that is a patchwork of short shell
  // runs.  Here the shells are ordered by cutoff radius (largest first), then
  // by the Morton code of their centre, so a block's union becomes a few long
  // runs per radius, and the P gather and the VXC atomics touch fewer DRAM
  // sectors.  P_ and A_ live in this order; P comes in and VXC goes out
  // through permuting copies.
  const int nsh_all = (int)bs.shells.size();
  std::vector<int> shell_pos(nsh_all), new_off(nsh_all), shell_at(nsh_all);
  {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (const auto& sh : bs.shells)
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], sh.O[k]);
        hi[k] = std::max(hi[k], sh.O[k]);
      }
    auto morton = [&](const double* O) {
      uint64_t code = 0;
      for (int k = 0; k < 3; ++k) {
        const double span = hi[k] - lo[k];
        const uint64_t q = span > 0. ? (uint64_t)std::min(1023., (O[k] - lo[k]) / span * 1023.) : 0;
        for (int bit = 0; bit < 10; ++bit) code |= ((q >> bit) & 1ull) << (3 * bit + k);
      }
      return code;
    };
    std::vector<uint64_t> mc(nsh_all);
    for (int x = 0; x < nsh_all; ++x) mc[x] = morton(bs.shells[x].O);
    std::vector<int> ord(nsh_all);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
      const Shell &sa = bs.shells[a], &sb = bs.shells[b];
      if (sa.cutoff_radius != sb.cutoff_radius) return sa.cutoff_radius > sb.cutoff_radius;
      if (sa.l != sb.l) return sa.l < sb.l;
      return mc[a] < mc[b];
    });
    std::vector<int> perm(nbf_), iperm(nbf_);
    int o = 0;
    for (int k = 0; k < nsh_all; ++k) {
      const int x = ord[k];
      shell_pos[x] = k;
      shell_at[k] = x;
      new_off[x] = o;
      for (int f = 0; f < bs.shells[x].size(); ++f) {
        perm[o + f] = bs.shell_offs[x] + f;
        iperm[bs.shell_offs[x] + f] = o + f;
      }
      o += bs.shells[x].size();
    }
    perm_ = arena_.upload(perm, s);
    iperm_ = arena_.upload(iperm, s);
  }
  // Task order of the merge: along a Morton curve of the tasks' centroids
  // (0.5 bohr cells, coarser when the molecule spans more than 511 bohr), so
  // that consecutive tasks are spatial neighbours and merged blocks stay
  // compact; tasks of different parent atoms may share a block (each point
  // keeps its own task's shell screening through the collocation mask).  On
  // 256 waters (CPU model of the merge): 48.6k blocks and 1.07e11 sum nu^2
  // against 74.5k and 1.72e11 in load-balancer order, for 1 % less tensor
  // work.
  std::vector<int> torder(tasks.size());
  {
    std::vector<double> cen(3 * tasks.size(), 0.);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (size_t t = 0; t < tasks.size(); ++t) {
      const XCTask& tt = tasks[t];
      for (int p = 0; p < tt.npts; ++p)
        for (int k = 0; k < 3; ++k) cen[3 * t + k] += tt.points[3 * p + k];
      for (int k = 0; k < 3; ++k) {
        if (tt.npts > 0) cen[3 * t + k] /= tt.npts;
        lo[k] = std::min(lo[k], cen[3 * t + k]);
        hi[k] = std::max(hi[k], cen[3 * t + k]);
      }
    }
    double span = 0.;
    for (int k = 0; k < 3; ++k) span = std::max(span, hi[k] - lo[k]);
    const double cell = std::max(0.5, span / 1023.);
    std::vector<uint64_t> key(tasks.size(), 0);
    for (size_t t = 0; t < tasks.size(); ++t)
      for (int k = 0; k < 3; ++k) {
        const uint64_t u = (uint64_t)std::min(1023., std::max(0., std::floor((cen[3 * t + k] - lo[k]) / cell)));
        for (int bit = 0; bit < 10; ++bit) key[t] |= ((u >> bit) & 1ull) << (3 * bit + k);
      }
    std::iota(torder.begin(), torder.end(), 0);
    std::stable_sort(torder.begin(), torder.end(), [&](int x, int y) { return key[x] < key[y]; });
  }
  // Merge: each task (piece) joins the cheapest of the last kMergeWindow
  // blocks with room for its points, if that does not raise the cost, else
  // it opens a block.  The open blocks' shell sets are bitsets over the
  // device AO order (so a closed block lists its shells in that order); the
  // union's basis size is nu(b) + nbe(t) - nbe(b & t), the intersection
  // counted per shell size class with popcounts.  On 256 waters (CPU model)
  // the window of 8 gives 40k blocks and 35 % less sum nu^2 than joining only
  // the last block, for 3 % less tensor work.
  constexpr int kMergeWindow = 8;
  const int nw = (nsh_all + 63) / 64;
  std::vector<int> csize;                     // distinct shell sizes
  std::vector<std::vector<uint64_t>> cmask;   // shells of each size, as bitsets
  for (int x = 0; x < nsh_all; ++x) {
    const int sz = bs.shells[x].size(), q = shell_pos[x];
    size_t c = 0;
    while (c < csize.size() && csize[c] != sz) ++c;
    if (c == csize.size()) {
      csize.push_back(sz);
      cmask.emplace_back(nw, 0ull);
    }
    cmask[c][q >> 6] |= 1ull << (q & 63);
  }
  // basis functions of a block's shell set (bits a) shared with the current
  // task, whose nonzero words tw hold its shells split by size class (tcb,
  // csize.size() words per entry of tw)
  std::vector<int> tw;
  std::vector<uint64_t> tcb;
  auto common_nbe = [&](const std::vector<uint64_t>& a) {
    const size_t ncs = csize.size();
    int n = 0;
    for (size_t j = 0; j < tw.size(); ++j) {
      const uint64_t m = a[tw[j]];
      for (size_t c = 0; c < ncs; ++c) n += __builtin_popcountll(m & tcb[j * ncs + c]) * csize[c];
    }
    return n;
  };
  struct OpenPB {
    int pb;
    std::vector<uint64_t> bits;
  };
  std::vector<PB> pbs;
  std::vector<OpenPB> win;  // the last kMergeWindow blocks, oldest first
  auto close_oldest = [&]() {
    PB& b = pbs[win.front().pb];
    b.shells.clear();
    for (int i = 0; i < nw; ++i)
      for (uint64_t w = win.front().bits[i]; w; w &= w - 1)
        b.shells.push_back(shell_at[i * 64 + __builtin_ctzll(w)]);
    win.erase(win.begin());
  };
  std::vector<uint64_t> tb(nw);
  for (int t : torder) {
    const XCTask& tt = tasks[t];
    std::fill(tb.begin(), tb.end(), 0ull);
    for (int x : tt.shell_list) tb[shell_pos[x] >> 6] |= 1ull << (shell_pos[x] & 63);
    tw.clear();
    tcb.clear();
    for (int i = 0; i < nw; ++i)
      if (tb[i]) {
        tw.push_back(i);
        for (size_t c = 0; c < csize.size(); ++c) tcb.push_back(tb[i] & cmask[c][i]);
      }
    for (int p0 = 0; p0 < tt.npts; p0 += maxp) {
      const int p1 = std::min(tt.npts, p0 + maxp), n = p1 - p0;
      int best = -1, best_nu = 0;
      double best_d = 0.;
      for (int w = (int)win.size() - 1; w >= 0; --w) {
        const PB& b = pbs[win[w].pb];
        if (b.npts + n > maxp) continue;
        const int nu = b.nu + tt.nbe - common_nbe(win[w].bits);
        const double d = pb_cost(b.npts + n, nu, w2) - pb_cost(b.npts, b.nu, w2) - pb_cost(n, tt.nbe, w2);
        if (d <= best_d) {
          best = w;
          best_d = d;
          best_nu = nu;
        }
      }
      if (best >= 0) {
        PB& b = pbs[win[best].pb];
        for (int i : tw) win[best].bits[i] |= tb[i];
        b.nu = best_nu;
        b.npts += n;
        b.segs.push_back({t, p0, p1});
      } else {
        PB b;
        b.segs.push_back({t, p0, p1});
        b.nu = tt.nbe;
        b.npts = n;
        pbs.push_back(std::move(b));
        win.push_back(OpenPB{(int)pbs.size() - 1, tb});
        if ((int)win.size() > kMergeWindow) close_oldest();
      }
    }
  }
  while (!win.empty()) close_oldest();
  // Blocks stay in the merge's spatial order: the VXC updates of neighbouring
  // blocks then hit the same rows and columns of the nbf x nbf accumulator
  // while they are resident in L2, and P's rows are gathered from L2 likewise.
  std::vector<int> order(pbs.size());
  std::iota(order.begin(), order.end(), 0);

  timings["plan_merge_ms"] = ms_since(t_plan0);
  const auto t_layout0 = std::chrono::steady_clock::now();

  const int npb = (int)pbs.size();
  std::vector<int64_t> pt_off(npb), bf_off(npb), sh_off(npb), f64_off(npb), dig_off(npb),
      mask_off(npb);
  std::vector<int> npts_pad(npb), nk(npb), nu(npb), nu_pad(npb), nsh(npb), bf_list, sh_list,
      sh_col, member;
  std::vector<uint8_t> mask;
  std::vector<double> X, Y, Z, W;
  stats = PlanStats{};
  // pass 1 (sequential): sizes and offsets of every block's lists
  int64_t pts = 0, nsh_tot = 0, nbf_tot = 0, nmask = 0;
  for (int i = 0; i < npb; ++i) {
    const PB& b = pbs[order[i]];
    pt_off[i] = pts;
    npts_pad[i] = (int)round_up(b.npts, kNTile);
    nk[i] = (int)round_up(b.npts, kBK);  // the VXC GEMM's points: real ones, K granularity
    nu[i] = b.nu;
    nu_pad[i] = (int)round_up(b.nu, kMTile);
    nsh[i] = (int)b.shells.size();
    {
      int nu_shells = 0;  // the merge's running union size against the closed shell list
      for (int x : b.shells) nu_shells += bs.shells[x].size();
      if (nu_shells != b.nu) throw error("plan: point-block basis size disagrees with its shells");
    }
    sh_off[i] = nsh_tot;
    bf_off[i] = nbf_tot;
    mask_off[i] = nmask;
    nsh_tot += nsh[i];
    nbf_tot += nu_pad[i];
    nmask += (int64_t)b.segs.size() * nsh[i];
    pts += npts_pad[i];
    stats.npts += b.npts;
    stats.sum_pad_npts_nbe2 += (double)npts_pad[i] * nu_pad[i] * nu_pad[i];
    {
      // algorithmic bytes of each kernel at this plan's sizes: phi as
      // float-float pairs (8 B), digit operands 6 BF16 planes (12 B)
      const PBDims d(npts_pad[i], nu[i], nk[i]);
      const double nq = gga_ ? 4. : 1.;
      const double phi = 8. * d.np * d.nu128;
      stats.kbytes[0] += nq * phi;                                          // collocation
      stats.kbytes[5] += phi + 12. * ((double)d.nu128 * d.nk + (double)d.nun * d.nk +
                                      (double)d.np * d.nu16);               // phi digits
      stats.kbytes[6] += 8. * d.nu * d.nu + 12. * d.nu128 * d.nu16;         // P digits
      stats.kbytes[1] += 12. * ((double)d.nu128 * d.nu16 + (double)d.np * d.nu16) + nq * phi +
                         32. * d.np;                                        // density GEMM
      stats.kbytes[2] += nq * phi + 32. * d.np + 12. * (double)(d.nu128 + d.nun) * d.nk;  // Z digits
      stats.kbytes[3] += 12. * (double)(d.nu128 + d.nun) * 2. * d.nk + 8. * d.nu * d.nu;  // VXC GEMM
    }
  }
  npts_plan_ = pts;
  sh_list.resize(nsh_tot);
  sh_col.resize(nsh_tot);
  bf_list.resize(nbf_tot);
  mask.resize(nmask);
  X.resize(pts);
  Y.resize(pts);
  Z.resize(pts);
  W.resize(pts);
  member.resize(pts);
  // pass 2 (host threads over blocks): the union's columns in device AO
  // order (shell data stays indexed by the caller's shell index), each
  // member task's shell mask over the union, and the points (padded with
  // zero-weight copies of the block's first point)
  auto fill = [&](int i0, int i1) {
    std::vector<uint64_t> mbits(nw, 0ull);  // a member task's shells (cleared after use)
    for (int i = i0; i < i1; ++i) {
      const PB& b = pbs[order[i]];
      const std::vector<int>& ushells = b.shells;
      int64_t so = sh_off[i], bo = bf_off[i];
      int col = 0;
      for (int x : ushells) {
        sh_list[so] = x;
        sh_col[so++] = col;
        for (int k = 0; k < bs.shells[x].size(); ++k) bf_list[bo++] = new_off[x] + k;
        col += bs.shells[x].size();
      }
      for (int k = col; k < nu_pad[i]; ++k) bf_list[bo++] = -1;
      int64_t mo = mask_off[i];
      for (size_t m = 0; m < b.segs.size(); ++m) {
        const XCTask& tt = tasks[b.segs[m].task];
        for (int x : tt.shell_list) mbits[x >> 6] |= 1ull << (x & 63);
        for (int x : ushells) mask[mo++] = (uint8_t)((mbits[x >> 6] >> (x & 63)) & 1ull);
        for (int x : tt.shell_list) mbits[x >> 6] = 0ull;
      }
      int64_t g = pt_off[i];
      for (size_t m = 0; m < b.segs.size(); ++m) {
        const Seg& sg = b.segs[m];
        const XCTask& tt = tasks[sg.task];
        for (int p = sg.p0; p < sg.p1; ++p, ++g) {
          X[g] = tt.points[3 * p];
          Y[g] = tt.points[3 * p + 1];
          Z[g] = tt.points[3 * p + 2];
          W[g] = tt.weights[p];
          member[g] = (int)m;
        }
      }
      for (const int64_t g0 = pt_off[i]; g < pt_off[i] + npts_pad[i]; ++g) {
        X[g] = X[g0];
        Y[g] = Y[g0];
        Z[g] = Z[g0];
        W[g] = 0.;
        member[g] = 0;
      }
    }
  };
  {
    const int nthr = std::max(1, std::min<int>(32, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int k = 0; k < nthr; ++k)
      pool.emplace_back(fill, (int)((int64_t)npb * k / nthr), (int)((int64_t)npb * (k + 1) / nthr));
    for (auto& th : pool) th.join();
  }
  for (const auto& t : tasks) {
    stats.sum_npts_nbe += (double)t.npts * t.nbe;
    stats.sum_npts_nbe2 += (double)t.npts * t.nbe * t.nbe;
  }
  stats.ntasks = (int64_t)tasks.size();
  stats.npts_pad = pts;

  timings["plan_layout_ms"] = ms_since(t_layout0);
  const auto t_lists0 = std::chrono::steady_clock::now();
  // ---- batches under the workspace budget
  size_t free_b = 0, total_b = 0;
  GB300_CUDA(cudaMemGetInfo(&free_b, &total_b));
  double static_bytes = pts * (3 * 8. + 8. + 32. + 32. + 4.) + bf_list.size() * 4. +
                        mask.size() + 8. * nbf_ + 64e6;
  if (func_.polarized)  // ensure_uks
    static_bytes += 3. * nbf_ * nbf_ * 8. + pts * (32. + 32.) + nbf_ * 8.;
  double budget = rt_->user_mem ? (double)rt_->user_bytes - rt_->user_used - static_bytes
                                : rt_->fill_fraction * (double)free_b - static_bytes;
  if (const char* cap = std::getenv("GAUXC_GB300_SCRATCH_GB")) budget = std::min(budget, atof(cap) * 1e9);
  if (params_.scratch_bytes > 0.) budget = std::min(budget, params_.scratch_bytes);
  budget = std::min(budget, 96e9);
  std::vector<int2> coll;
  std::vector<OzItem> xi, vi;
  double f64_used = 0., dig_used = 0., max_f64 = 0., max_dig = 0.;
  const int nfb = functional_partial_blocks();
  MBatch cur{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  auto close_batch = [&](int i) {
    cur.b1 = i;
    cur.coll_end = (int)coll.size();
    cur.x_end = (int)xi.size();
    cur.v_end = (int)vi.size();
    cur.g1 = i > 0 ? pt_off[i - 1] + npts_pad[i - 1] : 0;
    mbatches_.push_back(cur);
  };
  for (int i = 0; i < npb; ++i) {
    const double nf = (double)mixed_f64_doubles(npts_pad[i], nu[i], gga_) * 8.;
    const double nd = (double)mixed_dig_elems(npts_pad[i], nu[i], nk[i]) * 2.;
    if (nf + nd > budget) throw error("insufficient device memory for one point block");
    if (f64_used + dig_used + nf + nd > budget && i > cur.b0) {
      close_batch(i);
      cur = MBatch{i, i, (int)coll.size(), 0, (int)xi.size(), 0, (int)vi.size(), 0, pt_off[i], 0,
                   0, (int)mbatches_.size() * nfb, 0, 0, 0, 0};
      f64_used = dig_used = 0.;
    }
    f64_off[i] = (int64_t)(f64_used / 8.);
    dig_off[i] = (int64_t)(dig_used / 2.);
    f64_used += std::ceil(nf / 256.) * 256.;
    dig_used += std::ceil(nd / 256.) * 256.;
    max_f64 = std::max(max_f64, f64_used);
    max_dig = std::max(max_dig, dig_used);
    cur.max_nu_pad = std::max(cur.max_nu_pad, nu_pad[i]);
    for (int b = 0; b < (npts_pad[i] + 127) / 128; ++b) coll.push_back(make_int2(i, b));
    const PBDims d(npts_pad[i], nu[i], nk[i]);
    // Density tiles in cluster-slot order: the (m0, n0) tiles ("chains") in
    // row-major order, four per block (the last block of a point block
    // padded with empty entries); a block runs its chains' K chunks in
    // consecutive slots, so each CTA sums a tile's chunks before the phi
    // contraction and the chains of one row block share their A blocks.
    {
      const int nchunk = (d.nu16 + kMaxK - 1) / kMaxK;
      std::vector<std::pair<int, int>> ch;
      for (int m0 = 0; m0 < d.nu128; m0 += kMTile)
        for (int n0 = 0; n0 < d.np; n0 += kNTile) ch.push_back({m0, n0});
      for (size_t c0 = 0; c0 < ch.size(); c0 += kCluster)
        for (int c = 0; c < nchunk; ++c)
          for (int r = 0; r < kCluster; ++r) {
            if (c0 + r >= ch.size()) {
              xi.push_back(OzItem{-1, 0, 0, 0, 0, 0, 0});
              continue;
            }
            xi.push_back(OzItem{i, ch[c0 + r].first, ch[c0 + r].second, c * kMaxK,
                                std::min((c + 1) * kMaxK, d.nu16), 0, 0});
            oz_set_operands(xi.back(), d, dig_off[i], false);
          }
    }
    // symmetric VXC: tiles reaching the upper triangle, K = phi | Z
    for (int m0 = 0; m0 < d.nu128; m0 += kMTile)
      for (int n0 = 0; n0 < d.nun; n0 += kNTile)
        if (m0 < n0 + kNTile) {
          vi.push_back(OzItem{i, m0, n0, 0, 2 * d.nk, 0, 0});
          oz_set_operands(vi.back(), d, dig_off[i], true);
        }
  }
  if (npb > 0) close_batch(npb);
  {
    int npairs = 0;
    for (int lev = 2; lev <= kLevels; ++lev)
      for (int i = 1; i <= kSlices; ++i)
        if (lev - i >= 1 && lev - i <= kSlices) ++npairs;
    for (const OzItem& q : xi)
      if (q.pb >= 0) stats.tensor_flops_x += 2.0 * kMTile * kNTile * (q.k1 - q.k0) * npairs;
    for (const OzItem& q : vi) stats.tensor_flops_v += 2.0 * kMTile * kNTile * (q.k1 - q.k0) * npairs;
  }
  // per-cluster slot lists of every persistent GEMM launch
  const int ncl = ozaki_clusters();
  std::vector<int> sched;
  std::vector<OzItem> slots;
  for (MBatch& mb : mbatches_) {
    mb.x_sched = (int)sched.size();
    mb.x_ncl = ozaki_schedule(xi, mb.x_begin, mb.x_end, ncl, slots, sched);
    mb.v_sched = (int)sched.size();
    mb.v_ncl = ozaki_schedule(vi, mb.v_begin, mb.v_end, ncl, slots, sched);
  }
  stats.nbatches = (int64_t)mbatches_.size();
  stats.scratch_bytes = max_f64 + max_dig;

  tk_.ntasks = npb;
  tk_.pt_off = arena_.upload(pt_off, s);
  tk_.npts_pad = arena_.upload(npts_pad, s);
  tk_.nbe = arena_.upload(nu, s);
  tk_.nbe_pad = arena_.upload(nu_pad, s);
  tk_.bf_off = arena_.upload(bf_off, s);
  tk_.bf_list = arena_.upload(bf_list, s);
  tk_.sh_off = arena_.upload(sh_off, s);
  tk_.nsh = arena_.upload(nsh, s);
  tk_.sh_list = arena_.upload(sh_list, s);
  tk_.sh_col = arena_.upload(sh_col, s);
  tk_.scr_off = arena_.upload(f64_off, s);
  tk_.x = arena_.upload(X, s);
  tk_.y = arena_.upload(Y, s);
  tk_.z = arena_.upload(Z, s);
  tk_.w = arena_.upload(W, s);
  mk_.member = arena_.upload(member, s);
  mk_.mask_off = arena_.upload(mask_off, s);
  mk_.mask = arena_.upload(mask, s);
  mp_.f64_off = tk_.scr_off;
  mp_.dig_off = arena_.upload(dig_off, s);
  // z_digits CTAs: nu128 nk / 2048 per block (256 threads, 8 points each)
  zoff_h_.assign(npb + 1, 0);
  for (int i = 0; i < npb; ++i) {
    const PBDims d(npts_pad[i], nu[i], nk[i]);
    zoff_h_[i + 1] = zoff_h_[i] + d.nu128 * d.nk / 2048;
  }
  mp_.nk = arena_.upload(nk, s);
  mp_.zoff = arena_.upload(zoff_h_, s);
  coll_items_ = arena_.upload(coll, s);
  slots_ = arena_.upload(slots, s);
  sched_ = arena_.upload(sched, s);
  f64_ = arena_.alloc<double>((size_t)(max_f64 / 8.) + 32);
  dig_ = arena_.alloc<__nv_bfloat16>((size_t)(max_dig / 2.) + 128);
  rho4_ = arena_.alloc<double>((size_t)std::max<int64_t>(pts, 1) * 4);
  prs_ = arena_.alloc<double>((size_t)nbf_);
  zcoef_ = arena_.alloc<double4>(std::max<int64_t>(pts, 1));
  ndens_ = (int)mbatches_.size() * nfb;
  partials_ = arena_.alloc<double2>(std::max(ndens_, 1));
  timings["plan_lists_ms"] = ms_since(t_lists0);
}

int64_t DeviceIntegrator::eval_mixed_batches(bool do_vxc) {
  cudaStream_t s = stream_;
  int64_t launches = 0;
  launches += timed(4, [&] {
    launch_p_row_scales(P_, nbf_, prs_, s);
    return (int64_t)1;
  });
  for (const MBatch& b : mbatches_) {
    GB300_CUDA(cudaMemsetAsync(rho4_ + 4 * b.g0, 0, (size_t)(b.g1 - b.g0) * 4 * sizeof(double), s));
    launches += timed(0, [&] {
      launch_collocation_masked(sh_, tk_, mk_, coll_items_ + b.coll_begin,
                                b.coll_end - b.coll_begin, f64_, gga_, s);
      return (int64_t)1;
    });
    launches += timed(5, [&] {
      launch_phi_digits(tk_, mp_, b.b0, b.b1, gga_, f64_, dig_, s);
      return (int64_t)1;
    });
    launches += timed(6, [&] {
      launch_p_digits(tk_, mp_, b.b0, b.b1, b.max_nu_pad, gga_, P_, prs_, nbf_, f64_, dig_, s);
      return (int64_t)1;
    });
    launches += timed(1, [&] {
      launch_ozaki_x(tk_, mp_, OzSchedule{slots_, sched_ + b.x_sched, b.x_ncl, wait_ns, withhold ? 1 : 0}, f64_, dig_, gga_,
                     rho4_, err_, s);
      return (int64_t)1;
    });
    launches += timed(4, [&] {
      launch_functional(b.g0, b.g1, tk_.w, rho4_, func_, zcoef_, partials_ + b.partial_base, s);
      return (int64_t)1;
    });
    if (!do_vxc) continue;
    launches += timed(2, [&] {
      launch_z_digits(tk_, mp_, b.b0, b.b1, zoff_h_[b.b0], zoff_h_[b.b1], gga_, zcoef_, f64_, dig_, s);
      return (int64_t)2;
    });
    launches += timed(3, [&] {
      launch_ozaki_v(tk_, mp_, OzSchedule{slots_, sched_ + b.v_sched, b.v_ncl, wait_ns, withhold ? 1 : 0}, f64_, dig_, gga_,
                     A_, nbf_, err_, s);
      return (int64_t)1;
    });
  }
  return launches;
}

int64_t DeviceIntegrator::enqueue(const double* P, int64_t ldp, double* VXC, int64_t ldvxc,
                                  double* en_host, int* err_host, bool do_vxc, bool events) {
  cudaStream_t s = stream_;
  const size_t row = (size_t)nbf_ * sizeof(double);
  // the error flag of this call's pipeline waits starts clear
  GB300_CUDA(cudaMemsetAsync(err_, 0, sizeof(int), s));
  if (events) GB300_CUDA(cudaEventRecord(ev_[0], s));
  // A_ (cleared next) stages the caller's P when the device order differs
  int64_t launches = load_density(P, ldp, P_, 1., A_);
  if (events) GB300_CUDA(cudaEventRecord(ev_[1], s));
  if (do_vxc) GB300_CUDA(cudaMemsetAsync(A_, 0, (size_t)nbf_ * nbf_ * sizeof(double), s));
  pev_used_ = 0;
  if (prec_ == Precision::Mixed) launches += eval_mixed_batches(do_vxc);
  for (const Batch& b : batches_) {
    const int nt = b.t_end - b.t_begin;
    launches += timed(0, [&] {
      launch_collocation(sh_, tk_, coll_items_ + b.coll_begin, b.coll_end - b.coll_begin, scr_,
                         gga_, s);
      return (int64_t)1;
    });
    launches += timed(1, [&] {
      launch_density_fp64(tk_, dens_items_ + b.dens_begin, b.dens_end - b.dens_begin, scr_, P_,
                          nbf_, func_, zcoef_, partials_ + b.dens_begin, s);
      return (int64_t)1;
    });
    if (do_vxc) {
      launches += timed(2, [&] {
        launch_zmat(tk_, b.t_begin, nt, zcoef_, scr_, gga_, s);
        return (int64_t)1;
      });
      launches += timed(3, [&] {
        launch_vxc_fp64(tk_, vxc_items_ + b.vxc_begin, b.vxc_end - b.vxc_begin, scr_, A_, nbf_,
                        gga_, s);
        return (int64_t)1;
      });
    }
  }
  if (do_vxc && !host_direct_)
    launches += timed(4, [&] {
      symmetrize_out(A_, V_, nbf_);
      return (int64_t)1;
    });
  launches += timed(4, [&] {
    launch_reduce_partials(partials_, ndens_, out_, s);
    return (int64_t)1;
  });
  if (events) GB300_CUDA(cudaEventRecord(ev_[2], s));
  if (do_vxc) {
    if (host_direct_) {
      // VXC = A + A^T written straight into the caller's buffer
      symmetrize_out(A_, VXC, ldvxc);
      ++launches;
    } else if (ldvxc == nbf_) {
      GB300_CUDA(cudaMemcpyAsync(VXC, V_, row * nbf_, cudaMemcpyDeviceToHost, s));
    } else {
      GB300_CUDA(cudaMemcpy2DAsync(VXC, (size_t)ldvxc * sizeof(double), V_, row, row, nbf_,
                                   cudaMemcpyDeviceToHost, s));
    }
  }
  GB300_CUDA(cudaMemcpyAsync(en_host, out_, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB300_CUDA(cudaMemcpyAsync(err_host, err_, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (events) GB300_CUDA(cudaEventRecord(ev_[3], s));
  stats.gpu_launches = launches;
  return launches;
}

int64_t DeviceIntegrator::load_density(const double* P, int64_t ldp, double* dst, double c,
                                       double* stage) {
  cudaStream_t s = stream_;
  const size_t row = (size_t)nbf_ * sizeof(double);
  // the caller's matrix lands coalesced (in `stage` when it is permuted next)
  double* land = perm_ ? stage : dst;
  int64_t n = 0;
  if (host_direct_) {
    // the device reads the caller's (pageable or page-locked) P itself
    launch_copy_matrix(P, ldp, land, nbf_, nbf_, s);
    ++n;
  } else if (ldp == nbf_) {
    GB300_CUDA(cudaMemcpyAsync(land, P, row * nbf_, cudaMemcpyHostToDevice, s));
  } else {
    GB300_CUDA(cudaMemcpy2DAsync(land, row, P, (size_t)ldp * sizeof(double), row, nbf_,
                                 cudaMemcpyHostToDevice, s));
  }
  if (perm_) {
    launch_permute_matrix(land, nbf_, perm_, c, dst, s);
    ++n;
  } else if (c != 1.) {
    launch_scale(dst, (int64_t)nbf_ * nbf_, c, s);
    ++n;
  }
  return n;
}

void DeviceIntegrator::symmetrize_out(const double* A, double* V, int64_t ld) {
  if (iperm_)
    launch_symmetrize_perm(A, nbf_, iperm_, V, ld, stream_);
  else
    launch_symmetrize(A, nbf_, V, ld, stream_);
}

int64_t DeviceIntegrator::store_vxc(const double* A, double* stage, double* VXC, int64_t ldvxc) {
  cudaStream_t s = stream_;
  const size_t row = (size_t)nbf_ * sizeof(double);
  if (host_direct_) {
    symmetrize_out(A, VXC, ldvxc);
    return 1;
  }
  symmetrize_out(A, stage, nbf_);
  if (ldvxc == nbf_)
    GB300_CUDA(cudaMemcpyAsync(VXC, stage, row * nbf_, cudaMemcpyDeviceToHost, s));
  else
    GB300_CUDA(cudaMemcpy2DAsync(VXC, (size_t)ldvxc * sizeof(double), stage, row, row, nbf_,
                                 cudaMemcpyDeviceToHost, s));
  return 1;
}

int64_t DeviceIntegrator::eval_mixed_batches_uks(bool do_vxc) {
  cudaStream_t s = stream_;
  int64_t launches = 0;
  launches += timed(4, [&] {
    launch_p_row_scales(P_, nbf_, prs_, s);
    launch_p_row_scales(Pz_, nbf_, prsz_, s);
    return (int64_t)2;
  });
  for (const MBatch& b : mbatches_) {
    const size_t bytes = (size_t)(b.g1 - b.g0) * 4 * sizeof(double);
    GB300_CUDA(cudaMemsetAsync(rho4s_ + 4 * b.g0, 0, bytes, s));
    GB300_CUDA(cudaMemsetAsync(rho4z_ + 4 * b.g0, 0, bytes, s));
    launches += timed(0, [&] {
      launch_collocation_masked(sh_, tk_, mk_, coll_items_ + b.coll_begin,
                                b.coll_end - b.coll_begin, f64_, gga_, s);
      return (int64_t)1;
    });
    launches += timed(5, [&] {
      launch_phi_digits(tk_, mp_, b.b0, b.b1, gga_, f64_, dig_, s);
      return (int64_t)1;
    });
    const OzSchedule xs{slots_, sched_ + b.x_sched, b.x_ncl, wait_ns, withhold ? 1 : 0};
    // the two densities in turn through the same P digit space
    for (int d = 0; d < 2; ++d) {
      launches += timed(6, [&] {
        launch_p_digits(tk_, mp_, b.b0, b.b1, b.max_nu_pad, gga_, d ? Pz_ : P_, d ? prsz_ : prs_,
                        nbf_, f64_, dig_, s);
        return (int64_t)1;
      });
      launches += timed(1, [&] {
        launch_ozaki_x(tk_, mp_, xs, f64_, dig_, gga_, d ? rho4z_ : rho4s_, err_, s);
        return (int64_t)1;
      });
    }
    launches += timed(4, [&] {
      launch_functional_pol(b.g0, b.g1, tk_.w, rho4s_, rho4z_, func_, zcoef_, zcoefz_,
                            partials_pol_ + b.partial_base, true, s);
      return (int64_t)1;
    });
    if (!do_vxc) continue;
    const OzSchedule vs{slots_, sched_ + b.v_sched, b.v_ncl, wait_ns, withhold ? 1 : 0};
    for (int d = 0; d < 2; ++d) {
      launches += timed(2, [&] {
        launch_z_digits(tk_, mp_, b.b0, b.b1, zoff_h_[b.b0], zoff_h_[b.b1], gga_,
                        d ? zcoefz_ : zcoef_, f64_, dig_, s);
        return (int64_t)2;
      });
      launches += timed(3, [&] {
        launch_ozaki_v(tk_, mp_, vs, f64_, dig_, gga_, d ? Az_ : A_, nbf_, err_, s);
        return (int64_t)1;
      });
    }
  }
  return launches;
}

int64_t DeviceIntegrator::enqueue_uks(const double* Ps, int64_t ldps, const double* Pz,
                                      int64_t ldpz, double* VXCs, int64_t ldvs, double* VXCz,
                                      int64_t ldvz, double* en_host, int* err_host, bool do_vxc) {
  ensure_uks();
  cudaStream_t s = stream_;
  GB300_CUDA(cudaMemsetAsync(err_, 0, sizeof(int), s));
  GB300_CUDA(cudaEventRecord(ev_[0], s));
  // P_s / 2 and P_z / 2: the RKS passes (X = 2 P phi) then give X = P phi
  // A_ and Az_ (cleared next) stage the caller's matrices when the device
  // order differs
  int64_t launches = load_density(Ps, ldps, P_, 0.5, A_) + load_density(Pz, ldpz, Pz_, 0.5, Az_);
  GB300_CUDA(cudaEventRecord(ev_[1], s));
  if (do_vxc) {
    GB300_CUDA(cudaMemsetAsync(A_, 0, (size_t)nbf_ * nbf_ * sizeof(double), s));
    GB300_CUDA(cudaMemsetAsync(Az_, 0, (size_t)nbf_ * nbf_ * sizeof(double), s));
  }
  pev_used_ = 0;
  if (prec_ == Precision::Mixed) {
    launches += eval_mixed_batches_uks(do_vxc);
  } else {
    const int nfb = functional_partial_blocks();
    for (size_t ib = 0; ib < batches_.size(); ++ib) {
      const Batch& b = batches_[ib];
      const int nt = b.t_end - b.t_begin;
      launches += timed(0, [&] {
        launch_collocation(sh_, tk_, coll_items_ + b.coll_begin, b.coll_end - b.coll_begin, scr_,
                           gga_, s);
        return (int64_t)1;
      });
      launches += timed(1, [&] {
        launch_density_fp64_rho(tk_, dens_items_ + b.dens_begin, b.dens_end - b.dens_begin, scr_,
                                P_, nbf_, gga_, reinterpret_cast<double4*>(rho4s_), s);
        launch_density_fp64_rho(tk_, dens_items_ + b.dens_begin, b.dens_end - b.dens_begin, scr_,
                                Pz_, nbf_, gga_, reinterpret_cast<double4*>(rho4z_), s);
        return (int64_t)2;
      });
      launches += timed(4, [&] {
        launch_functional_pol(b.g0, b.g1, tk_.w, rho4s_, rho4z_, func_, zcoef_, zcoefz_,
                              partials_pol_ + ib * nfb, false, s);
        return (int64_t)1;
      });
      if (!do_vxc) continue;
      for (int d = 0; d < 2; ++d) {
        launches += timed(2, [&] {
          launch_zmat(tk_, b.t_begin, nt, d ? zcoefz_ : zcoef_, scr_, gga_, s);
          return (int64_t)1;
        });
        launches += timed(3, [&] {
          launch_vxc_fp64(tk_, vxc_items_ + b.vxc_begin, b.vxc_end - b.vxc_begin, scr_,
                          d ? Az_ : A_, nbf_, gga_, s);
          return (int64_t)1;
        });
      }
    }
  }
  launches += timed(4, [&] {
    launch_reduce_partials(partials_pol_, npol_, out_, s);
    return (int64_t)1;
  });
  GB300_CUDA(cudaEventRecord(ev_[2], s));
  if (do_vxc) {
    launches += store_vxc(A_, V_, VXCs, ldvs);
    launches += store_vxc(Az_, Vz_, VXCz, ldvz);
  }
  GB300_CUDA(cudaMemcpyAsync(en_host, out_, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB300_CUDA(cudaMemcpyAsync(err_host, err_, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB300_CUDA(cudaEventRecord(ev_[3], s));
  stats.gpu_launches = launches;
  return launches;
}

void DeviceIntegrator::eval_uks(const double* Ps, int64_t ldps, const double* Pz, int64_t ldpz,
                                double* VXCs, int64_t ldvs, double* VXCz, int64_t ldvz,
                                double* EXC, double* NEL) {
  auto t_host0 = std::chrono::steady_clock::now();
  const bool do_vxc = VXCs != nullptr && VXCz != nullptr;
  double en[2] = {0., 0.};
  int herr = 0;
  const int64_t launches =
      enqueue_uks(Ps, ldps, Pz, ldpz, VXCs, ldvs, VXCz, ldvz, en, &herr, do_vxc);
  GB300_CUDA(cudaStreamSynchronize(stream_));
  if (herr)
    throw error("a tensor-core pipeline wait expired on the device (error code " +
                std::to_string(herr) + ")");
  auto t_host1 = std::chrono::steady_clock::now();
  if (EXC) *EXC = en[0];
  if (NEL) *NEL = en[1];
  float h2d, comp, d2h;
  GB300_CUDA(cudaEventElapsedTime(&h2d, ev_[0], ev_[1]));
  GB300_CUDA(cudaEventElapsedTime(&comp, ev_[1], ev_[2]));
  GB300_CUDA(cudaEventElapsedTime(&d2h, ev_[2], ev_[3]));
  timings["h2d_ms"] = h2d;
  timings["compute_ms"] = comp;
  timings["d2h_ms"] = d2h;
  timings["wall_ms"] = std::chrono::duration<double, std::milli>(t_host1 - t_host0).count();
  timings["gpu_launches"] = (double)launches;
  for (int k = 0; k < 7; ++k) {
    kclass_ms[k] = 0.;
    kclass_n[k] = 0;
  }
  for (size_t i = 0; i < pev_used_; i += 2) {
    float ms = 0.f;
    GB300_CUDA(cudaEventElapsedTime(&ms, pev_[i], pev_[i + 1]));
    kclass_ms[pev_class_[i]] += ms;
    kclass_n[pev_class_[i]] += pev_class_[i + 1];
  }
}

void DeviceIntegrator::eval(const double* P, int64_t ldp, double* VXC, int64_t ldvxc, double* EXC,
                            double* NEL, bool den_only) {
  auto t_host0 = std::chrono::steady_clock::now();
  const bool do_vxc = (VXC != nullptr) && !den_only;
  double en[2] = {0., 0.};
  int herr = 0;
  const int64_t launches = enqueue(P, ldp, VXC, ldvxc, en, &herr, do_vxc, true);
  GB300_CUDA(cudaStreamSynchronize(stream_));
  if (herr)
    throw error("a tensor-core pipeline wait expired on the device (error code " +
                std::to_string(herr) + ")");
  auto t_host1 = std::chrono::steady_clock::now();
  if (EXC) *EXC = en[0];
  if (NEL) *NEL = en[1];
  float h2d, comp, d2h;
  GB300_CUDA(cudaEventElapsedTime(&h2d, ev_[0], ev_[1]));
  GB300_CUDA(cudaEventElapsedTime(&comp, ev_[1], ev_[2]));
  GB300_CUDA(cudaEventElapsedTime(&d2h, ev_[2], ev_[3]));
  timings["h2d_ms"] = h2d;
  timings["compute_ms"] = comp;
  timings["d2h_ms"] = d2h;
  timings["wall_ms"] = std::chrono::duration<double, std::milli>(t_host1 - t_host0).count();
  timings["gpu_launches"] = (double)launches;
  for (int k = 0; k < 7; ++k) {
    kclass_ms[k] = 0.;
    kclass_n[k] = 0;
  }
  for (size_t i = 0; i < pev_used_; i += 2) {
    float ms = 0.f;
    GB300_CUDA(cudaEventElapsedTime(&ms, pev_[i], pev_[i + 1]));
    kclass_ms[pev_class_[i]] += ms;
    kclass_n[pev_class_[i]] += pev_class_[i + 1];
  }
}

// ---------------------------------------------------------------- API glue

namespace {
void ensure_plan(XCIntegratorHandle& h) {
  if (!h.lb) throw error("integrator has no load balancer");
  if (!h.lb->weights_modified) throw error("Weights Have Not Been Modified");
  if (!h.dev || h.dev->generation != h.lb->generation) {
    h.dev.reset();
    if (h.rt && h.rt->user_mem) h.rt->user_used = 0;
    h.dev = std::make_shared<DeviceIntegrator>(*h.lb, *h.func, h.prec, *h.rt, h.params);
  }
  h.dev->profiling = h.profiling;
  h.dev->wait_ns = h.wait_ns;
  h.dev->withhold = h.withhold;
}
void check_dims(const XCIntegratorHandle& h, int64_t m, int64_t n, int64_t ldp) {
  const int64_t nbf = h.lb->basis->nbf;
  if (m != n) throw error("P Must Be Square");
  if (m != nbf) throw error("P Must Have Same Dimension as Basis");
  if (ldp < nbf) throw error("Invalid LDP");
}
}  // namespace

void integrator_eval_exc_vxc(XCIntegratorHandle& h, int64_t m, int64_t n, const double* P,
                             int64_t ldp, double* VXC, int64_t ldvxc, double* EXC) {
  if (!P) throw error("null density matrix");
  if (h.func->polarized) throw error("RKS evaluation requires an unpolarized functional");
  check_dims(h, m, n, ldp);
  if (VXC && ldvxc < h.lb->basis->nbf) throw error("Invalid LDVXC");
  ensure_plan(h);
  double nel = 0.;
  h.dev->eval(P, ldp, VXC, ldvxc, EXC, &nel, false);
  h.last_exc = EXC ? *EXC : 0.;
  h.last_nel = nel;
}

void integrator_eval_exc_vxc_uks(XCIntegratorHandle& h, int64_t m, int64_t n, const double* Ps,
                                 int64_t ldps, const double* Pz, int64_t ldpz, double* VXCs,
                                 int64_t ldvs, double* VXCz, int64_t ldvz, double* EXC) {
  if (!Ps || !Pz) throw error("null density matrix");
  if (!h.func->polarized) throw error("UKS evaluation requires a polarized functional");
  check_dims(h, m, n, ldps);
  check_dims(h, m, n, ldpz);
  if ((VXCs == nullptr) != (VXCz == nullptr))
    throw error("VXC_s and VXC_z must both be given (or both be null for EXC only)");
  const int64_t nbf = h.lb->basis->nbf;
  if (VXCs && (ldvs < nbf || ldvz < nbf)) throw error("Invalid LDVXC");
  ensure_plan(h);
  double nel = 0.;
  h.dev->eval_uks(Ps, ldps, Pz, ldpz, VXCs, ldvs, VXCz, ldvz, EXC, &nel);
  h.last_exc = EXC ? *EXC : 0.;
  h.last_nel = nel;
}

void integrator_integrate_den(XCIntegratorHandle& h, int64_t m, int64_t n, const double* P,
                              int64_t ldp, double* NEL) {
  if (!P) throw error("null density matrix");
  check_dims(h, m, n, ldp);
  ensure_plan(h);
  double exc = 0., nel2 = 0.;
  h.dev->eval(P, ldp, nullptr, 0, &exc, &nel2, true);
  // the plan evaluates rho = 2 phi^T P phi (RKS, X factor 2); integrate_den
  // integrates phi^T P phi (X factor 1, incore_..._integrate_den.hpp:133)
  *NEL = 0.5 * nel2;
  h.last_nel = *NEL;
}

std::map<std::string, double> integrator_timings(const XCIntegratorHandle& h) {
  return h.dev ? h.dev->timings : std::map<std::string, double>{};
}

void integrator_set_profiling(XCIntegratorHandle& h, bool on) {
  h.profiling = on;
  if (h.dev) h.dev->profiling = on;
}

void integrator_set_pipeline_check(XCIntegratorHandle& h, double wait_ms, bool withhold) {
  if (!(wait_ms > 0.) || wait_ms > 60000.) throw error("pipeline wait bound must lie in (0, 60000] ms");
  h.wait_ns = (uint64_t)(wait_ms * 1e6);
  h.withhold = withhold;
  if (h.dev) {
    h.dev->wait_ns = h.wait_ns;
    h.dev->withhold = withhold;
  }
}

std::vector<double> integrator_kernel_times(const XCIntegratorHandle& h) {
  std::vector<double> v(14, 0.);
  if (!h.dev) return v;
  for (int k = 0; k < 7; ++k) {
    v[2 * k] = h.dev->kclass_ms[k];
    v[2 * k + 1] = (double)h.dev->kclass_n[k];
  }
  return v;
}

PlanStats integrator_plan_stats(XCIntegratorHandle& h) {
  ensure_plan(h);
  return h.dev->stats;
}

void integrator_set_plan_params(XCIntegratorHandle& h, const PlanParams& p) {
  if (!(p.scratch_bytes >= 0.)) throw error("scratch cap must be non-negative");
  if (p.pb_max_pts < kNTile || p.pb_max_pts > kPBMaxPts)
    throw error("point-block size must lie in [" + std::to_string(kNTile) + ", " +
                std::to_string(kPBMaxPts) + "]");
  if (!(p.nu2_weight >= 0.)) throw error("merge weight must be non-negative");
  h.params = p;
  h.dev.reset();  // rebuilt with the new parameters on the next call
}

// Candidate plans: point-block sizes x weights of the per-block gather and
// scatter work (union basis squared) in the merge rule.  Each candidate is
// built and timed on one warm call; the fastest stays in place.
double integrator_autotune(XCIntegratorHandle& h, const double* P, int64_t ldp, PlanParams* best) {
  if (!P) throw error("null density matrix");
  const int64_t nbf = h.lb->basis->nbf;
  check_dims(h, nbf, nbf, ldp);
  std::vector<double> V((size_t)nbf * nbf);
  std::vector<PlanParams> cands;
  if (h.prec == Precision::Mixed) {
    for (int pts : {128, 256, 384})
      for (double w : {75., 150.}) cands.push_back(PlanParams{pts, w, h.params.scratch_bytes});
  } else {
    cands.push_back(h.params);
  }
  double best_ms = -1.;
  PlanParams bp = h.params;
  for (const PlanParams& c : cands) {
    h.params = c;
    h.dev.reset();
    ensure_plan(h);
    double exc = 0., nel = 0.;
    h.dev->eval(P, ldp, V.data(), nbf, &exc, &nel, false);
    h.dev->eval(P, ldp, V.data(), nbf, &exc, &nel, false);
    const double ms = h.dev->timings["compute_ms"];
    if (best_ms < 0. || ms < best_ms) {
      best_ms = ms;
      bp = c;
    }
  }
  if (h.params.pb_max_pts != bp.pb_max_pts || h.params.nu2_weight != bp.nu2_weight ||
      h.params.scratch_bytes != bp.scratch_bytes) {
    h.params = bp;
    h.dev.reset();
    ensure_plan(h);
  }
  if (best) *best = bp;
  return best_ms;
}

// ---------------------------------------------------------------- batches
// One CUDA graph per set of caller buffers: the root stream forks into every
// member integrator's stream, each member enqueues its whole call (P in,
// kernels, VXC / EXC / error flag out) and the root joins them.  Replaying
// the graph is then a single launch per SCF iteration, and the members'
// branches run concurrently on the GPU.
class IntegratorBatch {
 public:
  explicit IntegratorBatch(const std::vector<XCIntegratorHandle*>& hs) : hs_(hs) {
    if (hs_.empty()) throw error("empty integrator batch");
    for (auto* h : hs_) {
      if (!h) throw error("null integrator in batch");
      if (h->func && h->func->polarized)
        throw error("batched evaluation takes RKS members (unpolarized functionals) only");
    }
    // Members share the device: each one without its own work-space cap gets
    // an equal share of the memory free now (plus what its current plan holds).
    size_t free_b = 0, total_b = 0;
    GB300_CUDA(cudaMemGetInfo(&free_b, &total_b));
    int uncapped = 0;
    for (auto* h : hs_)
      if (h->params.scratch_bytes <= 0.) ++uncapped;
    if (uncapped) {
      double held = 0.;
      for (auto* h : hs_)
        if (h->params.scratch_bytes <= 0. && h->dev) held += h->dev->stats.scratch_bytes;
      const double share = 0.8 * ((double)free_b + held) / uncapped;
      for (auto* h : hs_)
        if (h->params.scratch_bytes <= 0.) {
          h->params.scratch_bytes = std::max(share, 256e6);
          h->dev.reset();
        }
    }
    GB300_CUDA(cudaStreamCreateWithFlags(&root_, cudaStreamNonBlocking));
    GB300_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
    GB300_CUDA(cudaEventCreate(&t0_));
    GB300_CUDA(cudaEventCreate(&t1_));
    joins_.resize(hs_.size());
    for (auto& e : joins_) GB300_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    GB300_CUDA(cudaMallocHost(&en_, 2 * hs_.size() * sizeof(double)));
    GB300_CUDA(cudaMallocHost(&err_, hs_.size() * sizeof(int)));
  }
  ~IntegratorBatch() {
    release_graph();
    unregister_all();
    for (auto& e : joins_) cudaEventDestroy(e);
    cudaEventDestroy(fork_);
    cudaEventDestroy(t0_);
    cudaEventDestroy(t1_);
    cudaStreamDestroy(root_);
    cudaFreeHost(en_);
    cudaFreeHost(err_);
  }

  void eval(const double* const* P, const int64_t* ldp, double* const* VXC, const int64_t* ldvxc,
            double* EXC) {
    const size_t n = hs_.size();
    auto t_host0 = std::chrono::steady_clock::now();
    bool same = exec_ != nullptr && cap_dev_.size() == n;
    for (size_t i = 0; i < n; ++i) {
      XCIntegratorHandle& h = *hs_[i];
      if (!P[i]) throw error("null density matrix in batch member " + std::to_string(i));
      const int64_t nbf = h.lb->basis->nbf;
      check_dims(h, nbf, nbf, ldp[i]);
      if (VXC[i] && ldvxc[i] < nbf) throw error("Invalid LDVXC");
      ensure_plan(h);
      if (same && (cap_dev_[i] != h.dev.get() || cap_P_[i] != P[i] || cap_V_[i] != VXC[i] ||
                   cap_ldp_[i] != ldp[i] || cap_ldv_[i] != (VXC[i] ? ldvxc[i] : 0)))
        same = false;
    }
    if (!same) {
      // First call with these buffers: plain calls (which also set up every
      // kernel), then capture the graph for the next calls.
      for (size_t i = 0; i < n; ++i) {
        XCIntegratorHandle& h = *hs_[i];
        double nel = 0.;
        h.dev->eval(P[i], ldp[i], VXC[i], VXC[i] ? ldvxc[i] : 0, &EXC[i], &nel, false);
        h.last_exc = EXC[i];
        h.last_nel = nel;
      }
      capture(P, ldp, VXC, ldvxc);
      timings_["graph_launch"] = 0.;
      timings_["wall_ms"] =
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_host0).count();
      return;
    }
    GB300_CUDA(cudaEventRecord(t0_, root_));
    GB300_CUDA(cudaGraphLaunch(exec_, root_));
    GB300_CUDA(cudaEventRecord(t1_, root_));
    GB300_CUDA(cudaStreamSynchronize(root_));
    for (size_t i = 0; i < n; ++i) {
      if (err_[i])
        throw error("a tensor-core pipeline wait expired on the device (batch member " +
                    std::to_string(i) + ", error code " + std::to_string(err_[i]) + ")");
      EXC[i] = en_[2 * i];
      hs_[i]->last_exc = en_[2 * i];
      hs_[i]->last_nel = en_[2 * i + 1];
    }
    float ms = 0.f;
    GB300_CUDA(cudaEventElapsedTime(&ms, t0_, t1_));
    timings_["graph_launch"] = 1.;
    timings_["compute_ms"] = ms;  // whole graph: H2D, kernels, D2H of every member
    timings_["wall_ms"] =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_host0).count();
    timings_["members"] = (double)n;
    timings_["gpu_launches"] = (double)launches_;
  }

  const std::map<std::string, double>& timings() const { return timings_; }

 private:
  void release_graph() {
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
  }
  void unregister_all() {
    for (void* p : registered_) cudaHostUnregister(p);
    registered_.clear();
  }
  // Page-locks [p, p + bytes) in place unless it already is.
  void pin(const void* p, size_t bytes) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess &&
        (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice ||
         a.type == cudaMemoryTypeManaged))
      return;
    cudaGetLastError();
    const cudaError_t e = cudaHostRegister(const_cast<void*>(p), bytes, cudaHostRegisterDefault);
    if (e == cudaErrorHostMemoryAlreadyRegistered) {
      cudaGetLastError();
      return;
    }
    GB300_CUDA(e);
    registered_.push_back(const_cast<void*>(p));
  }
  void capture(const double* const* P, const int64_t* ldp, double* const* VXC,
               const int64_t* ldvxc) {
    const size_t n = hs_.size();
    release_graph();
    unregister_all();
    cap_dev_.assign(n, nullptr);
    cap_P_.assign(n, nullptr);
    cap_V_.assign(n, nullptr);
    cap_ldp_.assign(n, 0);
    cap_ldv_.assign(n, 0);
    for (size_t i = 0; i < n; ++i) {
      const int64_t nbf = hs_[i]->lb->basis->nbf;
      pin(P[i], (size_t)((nbf - 1) * ldp[i] + nbf) * sizeof(double));
      if (VXC[i]) pin(VXC[i], (size_t)((nbf - 1) * ldvxc[i] + nbf) * sizeof(double));
    }
    std::vector<bool> prof(n);
    for (size_t i = 0; i < n; ++i) {
      prof[i] = hs_[i]->dev->profiling;
      hs_[i]->dev->profiling = false;  // no event records inside the graph
    }
    launches_ = 0;
    GB300_CUDA(cudaStreamBeginCapture(root_, cudaStreamCaptureModeThreadLocal));
    bool ok = false;
    try {
      GB300_CUDA(cudaEventRecord(fork_, root_));
      for (size_t i = 0; i < n; ++i) {
        DeviceIntegrator& d = *hs_[i]->dev;
        GB300_CUDA(cudaStreamWaitEvent(d.stream(), fork_, 0));
        launches_ += d.enqueue(P[i], ldp[i], VXC[i], VXC[i] ? ldvxc[i] : 0, en_ + 2 * i, err_ + i,
                               VXC[i] != nullptr, false);
        GB300_CUDA(cudaEventRecord(joins_[i], d.stream()));
        GB300_CUDA(cudaStreamWaitEvent(root_, joins_[i], 0));
      }
      ok = true;
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(root_, &g);
      if (g) cudaGraphDestroy(g);
      for (size_t i = 0; i < n; ++i) hs_[i]->dev->profiling = prof[i];
      throw;
    }
    GB300_CUDA(cudaStreamEndCapture(root_, &graph_));
    for (size_t i = 0; i < n; ++i) hs_[i]->dev->profiling = prof[i];
    if (!ok || !graph_) throw error("graph capture failed");
    GB300_CUDA(cudaGraphInstantiate(&exec_, graph_, 0));
    for (size_t i = 0; i < n; ++i) {
      cap_dev_[i] = hs_[i]->dev.get();
      cap_P_[i] = P[i];
      cap_V_[i] = VXC[i];
      cap_ldp_[i] = ldp[i];
      cap_ldv_[i] = VXC[i] ? ldvxc[i] : 0;
    }
  }

  std::vector<XCIntegratorHandle*> hs_;
  cudaStream_t root_ = nullptr;
  cudaEvent_t fork_ = nullptr, t0_ = nullptr, t1_ = nullptr;
  std::vector<cudaEvent_t> joins_;
  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t exec_ = nullptr;
  double* en_ = nullptr;
  int* err_ = nullptr;
  int64_t launches_ = 0;
  std::vector<DeviceIntegrator*> cap_dev_;
  std::vector<const double*> cap_P_;
  std::vector<double*> cap_V_;
  std::vector<int64_t> cap_ldp_, cap_ldv_;
  std::vector<void*> registered_;
  std::map<std::string, double> timings_;
};

std::shared_ptr<IntegratorBatch> batch_new(const std::vector<XCIntegratorHandle*>& hs) {
  return std::make_shared<IntegratorBatch>(hs);
}

void batch_eval_exc_vxc(IntegratorBatch& b, const double* const* P, const int64_t* ldp,
                        double* const* VXC, const int64_t* ldvxc, double* EXC) {
  b.eval(P, ldp, VXC, ldvxc, EXC);
}

std::map<std::string, double> batch_timings(const IntegratorBatch& b) { return b.timings(); }

}  // namespace gb300
