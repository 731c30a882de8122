// Molecular-weights module and stage-level entry points.
//
// MolecularWeights (device, SSF): src/molecular_weights/device/
// device_molecular_weights.cxx:18-88 -- gathers every task's points, applies
// the SSF kernel in point batches sized to the device, writes the weights back
// into the tasks and marks the load balancer as weighted.  R_AB enters the
// kernel inverted (send_static_data_weights, xc_device_stack_data.cxx:322-348).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "../host/device_api.hpp"
#include "device_common.cuh"
#include "functionals.cuh"

namespace gb300 {

namespace {

template <typename T>
struct DevBuf {
  T* p = nullptr;
  explicit DevBuf(size_t n) { GB300_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T))); }
  ~DevBuf() { cudaFree(p); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

// Runs the SSF kernel over npts points.  Up to kSSFScreenedMaxAtoms atoms:
// the screened kernel in batches of up to 2^24 points, with the FP32 inputs
// of its factor classification (atom coordinates relative to their centroid
// o, and the margin on mu); larger molecules: the reference-order kernel in
// batches bounded by its distance table.
void ssf_batched(int64_t npts, int natoms, const double* x, const double* y, const double* z,
                 const int32_t* ip, const double* dn, const double* coords,
                 const std::vector<double>& rab_inv, double* w) {
  if (cuda_device_count() == 0) throw error("no CUDA device available for SSF weights");
  cudaStream_t s;
  GB300_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const bool screened = natoms <= kSSFScreenedMaxAtoms;
  const int64_t max_scr_doubles = (int64_t)1 << 29;  // 4 GiB of distances per batch
  const int64_t cap = screened ? ((int64_t)1 << 24) : max_scr_doubles / std::max(natoms, 1);
  const int64_t bsz = std::max<int64_t>(1, std::min<int64_t>(npts, cap));
  DevBuf<double> dx(bsz), dy(bsz), dz(bsz), dw(bsz), ddn(bsz), dc(3 * natoms),
      drab((size_t)natoms * natoms), dscr(screened ? 1 : (size_t)bsz * natoms);
  DevBuf<int32_t> dip(bsz), dstat(1);
  DevBuf<float4> dcf(screened ? natoms : 1);
  double o[3] = {0., 0., 0.};
  float margin = 0.f;
  if (screened) {
    // |mu_f - mu| <= 2 (28 E 2^-24 / R_min + 2^-20): E the largest |x - o| of
    // atoms and points, R_min the smallest interatomic distance (FP32
    // rounding of the coordinates, of differences, squares and roots, and
    // rsqrtf's 2 ulp), with a factor 2 to spare
    for (int a = 0; a < natoms; ++a)
      for (int k = 0; k < 3; ++k) o[k] += coords[3 * a + k] / natoms;
    double e2 = 0.;
    for (int a = 0; a < natoms; ++a) {
      const double u = coords[3 * a] - o[0], v = coords[3 * a + 1] - o[1], t = coords[3 * a + 2] - o[2];
      e2 = std::max(e2, u * u + v * v + t * t);
    }
    for (int64_t i = 0; i < npts; ++i) {
      const double u = x[i] - o[0], v = y[i] - o[1], t = z[i] - o[2];
      e2 = std::max(e2, u * u + v * v + t * t);
    }
    double rinv_max = 0.;
    for (double r : rab_inv) rinv_max = std::max(rinv_max, r);
    const double E = std::sqrt(e2) * (1. + 1e-6);
    const double m = 2. * (28. * E * std::ldexp(1., -24) * rinv_max + std::ldexp(1., -20));
    margin = (float)std::max(m, 1e-5);
    std::vector<float4> cf(natoms);
    for (int a = 0; a < natoms; ++a)
      cf[a] = make_float4((float)(coords[3 * a] - o[0]), (float)(coords[3 * a + 1] - o[1]),
                          (float)(coords[3 * a + 2] - o[2]), 0.f);
    GB300_CUDA(cudaMemcpyAsync(dcf.p, cf.data(), natoms * sizeof(float4), cudaMemcpyHostToDevice, s));
    GB300_CUDA(cudaStreamSynchronize(s));
  }
  GB300_CUDA(cudaMemsetAsync(dstat.p, 0, sizeof(int), s));
  GB300_CUDA(cudaMemcpyAsync(dc.p, coords, 3 * natoms * sizeof(double), cudaMemcpyHostToDevice, s));
  GB300_CUDA(cudaMemcpyAsync(drab.p, rab_inv.data(), rab_inv.size() * sizeof(double),
                             cudaMemcpyHostToDevice, s));
  for (int64_t b = 0; b < npts; b += bsz) {
    const int64_t n = std::min(bsz, npts - b);
    const size_t nd = n * sizeof(double);
    GB300_CUDA(cudaMemcpyAsync(dx.p, x + b, nd, cudaMemcpyHostToDevice, s));
    GB300_CUDA(cudaMemcpyAsync(dy.p, y + b, nd, cudaMemcpyHostToDevice, s));
    GB300_CUDA(cudaMemcpyAsync(dz.p, z + b, nd, cudaMemcpyHostToDevice, s));
    GB300_CUDA(cudaMemcpyAsync(dw.p, w + b, nd, cudaMemcpyHostToDevice, s));
    GB300_CUDA(cudaMemcpyAsync(ddn.p, dn + b, nd, cudaMemcpyHostToDevice, s));
    GB300_CUDA(cudaMemcpyAsync(dip.p, ip + b, n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    if (screened)
      launch_ssf_weights_screened(n, natoms, dx.p, dy.p, dz.p, dip.p, ddn.p, dc.p, dcf.p, o[0],
                                  o[1], o[2], margin, drab.p, natoms, dw.p, dstat.p, s);
    else
      launch_ssf_weights(n, natoms, dx.p, dy.p, dz.p, dip.p, ddn.p, dc.p, drab.p, natoms, dscr.p,
                         (int)n, dw.p, dstat.p, s);
    GB300_CUDA(cudaMemcpyAsync(w + b, dw.p, nd, cudaMemcpyDeviceToHost, s));
    GB300_CUDA(cudaStreamSynchronize(s));
  }
  int bad = 0;
  GB300_CUDA(cudaMemcpy(&bad, dstat.p, sizeof(int), cudaMemcpyDeviceToHost));
  GB300_CUDA(cudaStreamDestroy(s));
  if (bad) throw error("SSF weights: a parent atom index lies outside the molecule");
}

std::vector<double> rab_inverse(int natoms, const double* coords) {
  std::vector<double> r((size_t)natoms * natoms, 0.);
  for (int i = 0; i < natoms; ++i)
    for (int j = 0; j < natoms; ++j) {
      if (i == j) continue;
      const double dx = coords[3 * i] - coords[3 * j];
      const double dy = coords[3 * i + 1] - coords[3 * j + 1];
      const double dz = coords[3 * i + 2] - coords[3 * j + 2];
      r[(size_t)i * natoms + j] = 1. / std::sqrt(dx * dx + dy * dy + dz * dz);
    }
  return r;
}

}  // namespace

void molecular_weights_ssf_device(LoadBalancer& lb, RuntimeEnv&) {
  if (lb.weights_modified) return;
  const Molecule& mol = *lb.mol;
  const int natoms = (int)mol.size();
  std::vector<double> coords(3 * natoms);
  for (int i = 0; i < natoms; ++i) {
    coords[3 * i] = mol[i].x;
    coords[3 * i + 1] = mol[i].y;
    coords[3 * i + 2] = mol[i].z;
  }
  int64_t npts = 0;
  for (const auto& t : lb.tasks) npts += t.npts;
  std::vector<double> x(npts), y(npts), z(npts), w(npts), dn(npts);
  std::vector<int32_t> ip(npts);
  int64_t o = 0;
  for (const auto& t : lb.tasks)
    for (int p = 0; p < t.npts; ++p, ++o) {
      x[o] = t.points[3 * p];
      y[o] = t.points[3 * p + 1];
      z[o] = t.points[3 * p + 2];
      w[o] = t.weights[p];
      dn[o] = t.dist_nearest;
      ip[o] = t.iParent;
    }
  ssf_batched(npts, natoms, x.data(), y.data(), z.data(), ip.data(), dn.data(), coords.data(),
              rab_inverse(natoms, coords.data()), w.data());
  o = 0;
  for (auto& t : lb.tasks)
    for (int p = 0; p < t.npts; ++p, ++o) t.weights[p] = w[o];
  lb.weights_modified = true;
  lb.generation++;
}

void ssf_weights_device(int64_t npts, int natoms, const double* points, const int32_t* iparent,
                        const double* dist_nearest, const double* coords, double* weights) {
  std::vector<double> x(npts), y(npts), z(npts);
  for (int64_t i = 0; i < npts; ++i) {
    x[i] = points[3 * i];
    y[i] = points[3 * i + 1];
    z[i] = points[3 * i + 2];
  }
  ssf_batched(npts, natoms, x.data(), y.data(), z.data(), iparent, dist_nearest, coords,
              rab_inverse(natoms, coords), weights);
}

// One task made of `npts` points and the listed shells; outputs in the
// reference's host layout eval[ipt * nbe + ibf].
void collocation_device(const BasisSet& bs, int64_t npts, const double* points, int nshells,
                        const int32_t* shell_list, bool grad, double* phi, double* dphi_x,
                        double* dphi_y, double* dphi_z) {
  if (cuda_device_count() == 0) throw error("no CUDA device available for collocation");
  std::vector<double> a, c, o;
  std::vector<int> off{0}, l, pure, sh_col;
  int nbe = 0;
  for (int i = 0; i < nshells; ++i) {
    const Shell& sh = bs.shells.at(shell_list[i]);
    if (sh.l > 4) throw error("device collocation supports l <= 4");
    for (int k = 0; k < sh.nprim; ++k) {
      a.push_back(sh.alpha[k]);
      c.push_back(sh.coeff[k]);
    }
    off.push_back((int)a.size());
    o.insert(o.end(), sh.O, sh.O + 3);
    l.push_back(sh.l);
    pure.push_back(sh.pure);
    sh_col.push_back(nbe);
    nbe += sh.size();
  }
  const int np_pad = (int)((npts + kPtBlock - 1) / kPtBlock * kPtBlock);
  const int nbe_pad = (nbe + kBfBlock - 1) / kBfBlock * kBfBlock;
  std::vector<double> X(np_pad), Y(np_pad), Z(np_pad), W(np_pad, 0.);
  for (int p = 0; p < np_pad; ++p) {
    const int q = p < npts ? p : 0;
    X[p] = points[3 * q];
    Y[p] = points[3 * q + 1];
    Z[p] = points[3 * q + 2];
  }
  std::vector<int> shl(nshells);
  for (int i = 0; i < nshells; ++i) shl[i] = i;
  const int64_t blk = (int64_t)np_pad * nbe_pad;
  DevBuf<double> da(a.size()), dc(c.size()), dorig(o.size()), dX(np_pad), dY(np_pad), dZ(np_pad),
      dW(np_pad), dscr(4 * blk);
  DevBuf<int> doff(off.size()), dl(l.size()), dpure(pure.size()), dshl(nshells), dcol(nshells),
      dnp(1), dnbe(1), dnbep(1), dnsh(1);
  DevBuf<int64_t> dptoff(1), dshoff(1), dscroff(1);
  DevBuf<int2> ditems((np_pad + 127) / 128);
  auto up = [](void* d, const void* h, size_t b) {
    if (b) GB300_CUDA(cudaMemcpy(d, h, b, cudaMemcpyHostToDevice));
  };
  up(da.p, a.data(), a.size() * 8);
  up(dc.p, c.data(), c.size() * 8);
  up(dorig.p, o.data(), o.size() * 8);
  up(doff.p, off.data(), off.size() * 4);
  up(dl.p, l.data(), l.size() * 4);
  up(dpure.p, pure.data(), pure.size() * 4);
  up(dshl.p, shl.data(), shl.size() * 4);
  up(dcol.p, sh_col.data(), sh_col.size() * 4);
  up(dX.p, X.data(), np_pad * 8);
  up(dY.p, Y.data(), np_pad * 8);
  up(dZ.p, Z.data(), np_pad * 8);
  up(dW.p, W.data(), np_pad * 8);
  const int64_t zero64 = 0;
  up(dnp.p, &np_pad, 4);
  up(dnbe.p, &nbe, 4);
  up(dnbep.p, &nbe_pad, 4);
  up(dnsh.p, &nshells, 4);
  up(dptoff.p, &zero64, 8);
  up(dshoff.p, &zero64, 8);
  up(dscroff.p, &zero64, 8);
  std::vector<int2> items((np_pad + 127) / 128);
  for (size_t b = 0; b < items.size(); ++b) items[b] = make_int2(0, (int)b);
  up(ditems.p, items.data(), items.size() * sizeof(int2));
  ShellsDev sh{nshells, da.p, dc.p, doff.p, dorig.p, dl.p, dpure.p};
  TasksDev tk{};
  tk.ntasks = 1;
  tk.pt_off = dptoff.p;
  tk.npts_pad = dnp.p;
  tk.nbe = dnbe.p;
  tk.nbe_pad = dnbep.p;
  tk.sh_off = dshoff.p;
  tk.nsh = dnsh.p;
  tk.sh_list = dshl.p;
  tk.sh_col = dcol.p;
  tk.scr_off = dscroff.p;
  tk.x = dX.p;
  tk.y = dY.p;
  tk.z = dZ.p;
  tk.w = dW.p;
  launch_collocation(sh, tk, ditems.p, (int)items.size(), dscr.p, grad, 0);
  GB300_CUDA(cudaDeviceSynchronize());
  std::vector<double> h((grad ? 4 : 1) * blk);
  GB300_CUDA(cudaMemcpy(h.data(), dscr.p, h.size() * 8, cudaMemcpyDeviceToHost));
  double* outs[4] = {phi, dphi_x, dphi_y, dphi_z};
  for (int q = 0; q < (grad ? 4 : 1); ++q) {
    if (!outs[q]) continue;
    for (int64_t p = 0; p < npts; ++p)
      for (int b = 0; b < nbe; ++b) outs[q][p * nbe + b] = h[q * blk + (int64_t)b * np_pad + p];
  }
}

// ---------------------------------------------------------------- functionals
std::shared_ptr<XCFunctionalDesc> make_functional(const std::string& name0, bool polarized) {
  std::string name = name0;
  for (auto& ch : name) ch = (char)toupper(ch);
  auto f = std::make_shared<XCFunctionalDesc>();
  f->x_scale = 1.;
  f->c_scale = 1.;
  f->kappa = 0.804;
  f->mu = 0.2195149727645171;
  if (name == "SVWN5") {
    f->kind = kXC_SVWN5;
    f->is_gga = 0;
  } else if (name == "PBE") {
    f->kind = kXC_PBE;
    f->is_gga = 1;
  } else if (name == "REVPBE") {
    f->kind = kXC_PBE;
    f->is_gga = 1;
    f->kappa = 1.245;
  } else if (name == "PBE0") {
    f->kind = kXC_PBE;
    f->is_gga = 1;
    f->x_scale = 0.75;
  } else {
    throw error("functional not supported by this build: " + name0);
  }
  f->polarized = polarized ? 1 : 0;
  return f;
}

bool functional_is_gga(const XCFunctionalDesc& f) { return f.is_gga != 0; }

}  // namespace gb300
