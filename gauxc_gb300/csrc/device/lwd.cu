// Stage-level local work driver: the reference's LocalDeviceWorkDriver
// stages as separate device steps over one device-data object.
//
// Reference interface: src/xc_integrator/local_work_driver/device/
// local_device_work_driver.hpp:62-127 (stages over XCDeviceData,
// xc_device_data.hpp:668-787), driven in the order of
// incore_replicated_xc_device_integrator_exc_vxc.hpp:283-404:
//   create_device_data + pack tasks   -> LWDData(lb, task range)
//   eval_collocation(_gradient)       -> launch_collocation (collocation.cu)
//   eval_xmat(fac, P)                 -> xmat_kernel: X = fac P_sub phi (stored)
//   eval_vvars_{lda,gga}              -> vvars_kernel: rho, grad rho = 2 grad(phi) . X
//   eval_uvars_gga                    -> uvars_kernel: sigma = |grad rho|^2
//   eval_kern_exc_vxc_{lda,gga}       -> kern_kernel: eps, vrho, vsigma, all times w
//                                        (scale_{lda,gga}_output, scheme1_base.cxx:1303-1331)
//   inc_exc / inc_nel                 -> dot_kernel + fixed-order reduction
//   eval_zmat_{lda,gga}_vxc           -> zcoef_kernel + zmat_kernel (xc_fp64.cu)
//   inc_vxc                           -> vxc_fp64_kernel (xc_fp64.cu)
//   symmetrize_vxc                    -> symmetrize_kernel (xc_common.cu)
// Everything is FP64 and every intermediate stays in device memory, as in the
// reference's stage decomposition; the integrator (integrator.cu) runs the
// same arithmetic fused into fewer kernels.  The tasks of the range stay in
// load-balancer order and must fit in device memory together.
#include <algorithm>
#include <memory>
#include <vector>

#include "../host/device_api.hpp"
#include "device_common.cuh"
#include "functionals.cuh"
#include "xc_kernels.cuh"

namespace gb300 {

namespace {

constexpr int TM = 64, TN = 64, KT = 16, NT = 256;

// X[mu][p] = fac sum_nu P[bf(nu), bf(mu)] phi[nu][p] for one 64 x 64 tile.
__global__ void __launch_bounds__(NT) xmat_kernel(TasksDev tk, const int4* __restrict__ items,
                                                  const double* __restrict__ scr,
                                                  const double* __restrict__ P, int nbf, double fac,
                                                  double* __restrict__ X,
                                                  const int64_t* __restrict__ xoff) {
  __shared__ double As[KT][TM + 1];
  __shared__ double Bs[KT][TN + 1];
  const int4 it = items[blockIdx.x];
  const int t = it.x, m0 = it.y * TM, p0 = it.z * TN;
  const int np = tk.npts_pad[t], nbe_pad = tk.nbe_pad[t];
  const double* phi = scr + tk.scr_off[t];
  const int* bf = tk.bf_list + tk.bf_off[t];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < nbe_pad; k0 += KT) {
#pragma unroll
    for (int r = 0; r < (KT * TM) / NT; ++r) {
      const int e = tid + r * NT;
      const int k = e / TM, c = e % TM;
      const int gk = bf[k0 + k], gm = bf[m0 + c];
      As[k][c] = (gk >= 0 && gm >= 0) ? P[(int64_t)gm * nbf + gk] : 0.;
      Bs[k][c] = phi[(int64_t)(k0 + k) * np + p0 + c];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  double* x = X + xoff[t];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      x[(int64_t)(m0 + ty + 16 * i) * np + p0 + tx + 16 * j] = fac * acc[i][j];
}

// rho_p = sum_mu phi[mu][p] X[mu][p]; grad rho_p = 2 sum_mu grad phi[mu][p] X[mu][p]
template <bool GGA>
__global__ void vvars_kernel(TasksDev tk, const double* __restrict__ scr,
                             const double* __restrict__ X, const int64_t* __restrict__ xoff,
                             double4* __restrict__ den) {
  const int t = blockIdx.y;
  const int np = tk.npts_pad[t];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const int nbe_pad = tk.nbe_pad[t];
  const int64_t blk = (int64_t)np * nbe_pad;
  const double* phi = scr + tk.scr_off[t];
  const double* x = X + xoff[t];
  double r = 0., gx = 0., gy = 0., gz = 0.;
  for (int mu = 0; mu < nbe_pad; ++mu) {
    const int64_t o = (int64_t)mu * np + p;
    const double xv = x[o];
    r = fma(phi[o], xv, r);
    if (GGA) {
      gx = fma(phi[o + blk], xv, gx);
      gy = fma(phi[o + 2 * blk], xv, gy);
      gz = fma(phi[o + 3 * blk], xv, gz);
    }
  }
  den[tk.pt_off[t] + p] = make_double4(r, 2. * gx, 2. * gy, 2. * gz);
}

__global__ void uvars_kernel(int64_t n, const double4* __restrict__ den, double* __restrict__ gamma) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const double4 d = den[g];
    gamma[g] = d.y * d.y + d.z * d.z + d.w * d.w;
  }
}

// eps, vrho, vsigma at every point, each multiplied by the point's weight
__global__ void kern_kernel(int64_t n, const double4* __restrict__ den,
                            const double* __restrict__ gamma, const double* __restrict__ w,
                            XCFunctionalDesc f, double* __restrict__ eps, double* __restrict__ vrho,
                            double* __restrict__ vsigma) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    double e, vr, vs;
    xc_eval_unpol(f, den[g].x, f.is_gga ? gamma[g] : 0., e, vr, vs);
    const double wg = w[g];
    eps[g] = wg * e;
    vrho[g] = wg * vr;
    vsigma[g] = wg * vs;
  }
}

// Z coefficients (zmat_kernel): 0.5 vrho, and 2 vsigma grad rho for GGA
__global__ void zcoef_kernel(int64_t n, const double4* __restrict__ den,
                             const double* __restrict__ vrho, const double* __restrict__ vsigma,
                             int gga, double4* __restrict__ zc) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const double4 d = den[g];
    const double gf = gga ? 2. * vsigma[g] : 0.;
    zc[g] = make_double4(0.5 * vrho[g], gf * d.y, gf * d.z, gf * d.w);
  }
}

// partials[block] = (sum a[g] rho[g], 0) over a grid-stride share
__global__ void dot_kernel(int64_t n, const double* __restrict__ a,
                           const double4* __restrict__ den, double2* __restrict__ partials) {
  __shared__ double red[256];
  double s = 0.;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x)
    s = fma(a[g], den[g].x, s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = make_double2(red[0], 0.);
}

__global__ void accumulate_kernel(const double* __restrict__ v, double* __restrict__ acc) {
  *acc += v[0];
}

template <typename T>
struct Buf {
  T* p = nullptr;
  Buf() = default;
  explicit Buf(size_t n) { GB300_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T))); }
  ~Buf() {
    if (p) cudaFree(p);
  }
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  Buf(Buf&& o) noexcept : p(o.p) { o.p = nullptr; }
  Buf& operator=(Buf&& o) noexcept {
    std::swap(p, o.p);
    return *this;
  }
};

template <typename T>
Buf<T> upload(const std::vector<T>& v, cudaStream_t s) {
  Buf<T> b(v.size());
  if (!v.empty())
    GB300_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return b;
}

constexpr int kDotBlocks = 256;

}  // namespace

class LWDData {
 public:
  LWDData(const LoadBalancer& lb, int64_t t0, int64_t t1) {
    if (cuda_device_count() == 0) throw error("no CUDA device available for the local work driver");
    if (!lb.weights_modified) throw error("Weights Have Not Been Modified");
    if (t0 < 0 || t1 > (int64_t)lb.tasks.size() || t0 > t1) throw error("task range out of bounds");
    GB300_CUDA(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
    const BasisSet& bs = *lb.basis;
    nbf_ = bs.nbf;
    // shells
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
    sh_alpha_ = upload(a, s_);
    sh_coeff_ = upload(c, s_);
    sh_off_ = upload(off, s_);
    sh_origin_ = upload(o, s_);
    sh_l_ = upload(l, s_);
    sh_pure_ = upload(pure, s_);
    sh_ = ShellsDev{(int)bs.shells.size(), sh_alpha_.p, sh_coeff_.p, sh_off_.p, sh_origin_.p,
                    sh_l_.p, sh_pure_.p};
    // tasks [t0, t1) in load-balancer order, padded as the FP64 integrator pads them
    const int nt = (int)(t1 - t0);
    std::vector<int64_t> pt_off(nt), bf_off(nt), sh_offv(nt), scr_off(nt), xoff(nt);
    std::vector<int> npts_pad(nt), nbe(nt), nbe_pad(nt), nsh(nt), bf_list, sh_list, sh_col;
    std::vector<double> X, Y, Z, W;
    std::vector<int2> coll;
    std::vector<int4> xm, vx;
    int64_t pts = 0, scr = 0, xs = 0;
    maxnp_ = 0;
    for (int i = 0; i < nt; ++i) {
      const XCTask& tt = lb.tasks[t0 + i];
      pt_off[i] = pts;
      npts_pad[i] = (tt.npts + kPtBlock - 1) / kPtBlock * kPtBlock;
      maxnp_ = std::max(maxnp_, npts_pad[i]);
      for (int p = 0; p < npts_pad[i]; ++p) {
        const int q = p < tt.npts ? p : 0;
        X.push_back(tt.points[3 * q]);
        Y.push_back(tt.points[3 * q + 1]);
        Z.push_back(tt.points[3 * q + 2]);
        W.push_back(p < tt.npts ? tt.weights[p] : 0.);
      }
      pts += npts_pad[i];
      bf_off[i] = (int64_t)bf_list.size();
      sh_offv[i] = (int64_t)sh_list.size();
      int col = 0;
      for (int sl : tt.shell_list) {
        sh_list.push_back(sl);
        sh_col.push_back(col);
        for (int k = 0; k < bs.shells[sl].size(); ++k) bf_list.push_back(bs.shell_offs[sl] + k);
        col += bs.shells[sl].size();
      }
      nsh[i] = (int)tt.shell_list.size();
      nbe[i] = col;
      nbe_pad[i] = (col + kBfBlock - 1) / kBfBlock * kBfBlock;
      for (int k = col; k < nbe_pad[i]; ++k) bf_list.push_back(-1);
      const int64_t blk = (int64_t)npts_pad[i] * nbe_pad[i];
      scr_off[i] = scr;
      scr += 5 * blk;  // phi, grad phi (3), Z
      xoff[i] = xs;
      xs += blk;
      for (int b = 0; b < (npts_pad[i] + 127) / 128; ++b) coll.push_back(make_int2(i, b));
      for (int m = 0; m < nbe_pad[i] / TM; ++m)
        for (int p = 0; p < npts_pad[i] / TN; ++p) xm.push_back(make_int4(i, m, p, 0));
      for (int I = 0; I < nbe_pad[i] / kBfBlock; ++I)
        for (int J = 0; J < nbe_pad[i] / kBfBlock; ++J) vx.push_back(make_int4(i, I, J, 0));
    }
    npts_ = pts;
    t_pt_off_ = upload(pt_off, s_);
    t_npts_ = upload(npts_pad, s_);
    t_nbe_ = upload(nbe, s_);
    t_nbe_pad_ = upload(nbe_pad, s_);
    t_bf_off_ = upload(bf_off, s_);
    t_bf_ = upload(bf_list, s_);
    t_sh_off_ = upload(sh_offv, s_);
    t_nsh_ = upload(nsh, s_);
    t_sh_ = upload(sh_list, s_);
    t_sh_col_ = upload(sh_col, s_);
    t_scr_off_ = upload(scr_off, s_);
    t_x_ = upload(X, s_);
    t_y_ = upload(Y, s_);
    t_z_ = upload(Z, s_);
    t_w_ = upload(W, s_);
    tk_ = TasksDev{nt, t_pt_off_.p, t_npts_.p, t_nbe_.p, t_nbe_pad_.p, t_bf_off_.p, t_bf_.p,
                   t_sh_off_.p, t_nsh_.p, t_sh_.p, t_sh_col_.p, t_scr_off_.p, t_x_.p, t_y_.p,
                   t_z_.p, t_w_.p};
    xoff_ = upload(xoff, s_);
    coll_ = upload(coll, s_);
    ncoll_ = (int)coll.size();
    xm_ = upload(xm, s_);
    nxm_ = (int)xm.size();
    vx_ = upload(vx, s_);
    nvx_ = (int)vx.size();
    scr_ = Buf<double>((size_t)scr);
    X_ = Buf<double>((size_t)xs);
    den_ = Buf<double4>((size_t)pts);
    gamma_ = Buf<double>((size_t)pts);
    eps_ = Buf<double>((size_t)pts);
    vrho_ = Buf<double>((size_t)pts);
    vsig_ = Buf<double>((size_t)pts);
    zc_ = Buf<double4>((size_t)pts);
    partials_ = Buf<double2>(kDotBlocks);
    red_ = Buf<double>(2);
    acc_ = Buf<double>(2);
    P_ = Buf<double>((size_t)nbf_ * nbf_);
    A_ = Buf<double>((size_t)nbf_ * nbf_);
    GB300_CUDA(cudaMemsetAsync(gamma_.p, 0, (size_t)std::max<int64_t>(pts, 1) * sizeof(double), s_));
    GB300_CUDA(cudaMemsetAsync(acc_.p, 0, 2 * sizeof(double), s_));
    GB300_CUDA(cudaMemsetAsync(A_.p, 0, (size_t)nbf_ * nbf_ * sizeof(double), s_));
    GB300_CUDA(cudaStreamSynchronize(s_));
  }
  ~LWDData() {
    if (s_) cudaStreamDestroy(s_);
  }

  void eval_collocation(bool grad) {
    launch_collocation(sh_, tk_, coll_.p, ncoll_, scr_.p, grad, s_);
    grad_ = grad;
  }
  void eval_xmat(double fac, const double* P, int64_t ldp) {
    const size_t row = (size_t)nbf_ * sizeof(double);
    GB300_CUDA(cudaMemcpy2DAsync(P_.p, row, P, (size_t)ldp * sizeof(double), row, nbf_,
                                 cudaMemcpyHostToDevice, s_));
    if (nxm_) xmat_kernel<<<nxm_, NT, 0, s_>>>(tk_, xm_.p, scr_.p, P_.p, nbf_, fac, X_.p, xoff_.p);
    GB300_CUDA(cudaGetLastError());
  }
  void eval_vvars(bool gga) {
    if (gga && !grad_) throw error("eval_vvars_gga needs eval_collocation_gradient first");
    if (!tk_.ntasks) return;
    // one CTA row per 128 points of the largest task; shorter tasks exit early
    dim3 g((maxnp_ + 127) / 128, tk_.ntasks);
    if (gga)
      vvars_kernel<true><<<g, 128, 0, s_>>>(tk_, scr_.p, X_.p, xoff_.p, den_.p);
    else
      vvars_kernel<false><<<g, 128, 0, s_>>>(tk_, scr_.p, X_.p, xoff_.p, den_.p);
    GB300_CUDA(cudaGetLastError());
  }
  void eval_uvars() {
    uvars_kernel<<<1216, 256, 0, s_>>>(npts_, den_.p, gamma_.p);
    GB300_CUDA(cudaGetLastError());
  }
  void eval_kern(const XCFunctionalDesc& f) {
    if (f.polarized) throw error("the local work driver takes unpolarized (RKS) functionals");
    kern_kernel<<<1216, 256, 0, s_>>>(npts_, den_.p, gamma_.p, tk_.w, f, eps_.p, vrho_.p, vsig_.p);
    GB300_CUDA(cudaGetLastError());
  }
  // which = 0: EXC += sum eps_w rho; 1: N_el += sum w rho
  void inc(int which) {
    dot_kernel<<<kDotBlocks, 256, 0, s_>>>(npts_, which ? tk_.w : eps_.p, den_.p, partials_.p);
    launch_reduce_partials(partials_.p, kDotBlocks, red_.p, s_);
    accumulate_kernel<<<1, 1, 0, s_>>>(red_.p, acc_.p + which);
    GB300_CUDA(cudaGetLastError());
  }
  void eval_zmat(bool gga) {
    if (gga && !grad_) throw error("eval_zmat_gga_vxc needs eval_collocation_gradient first");
    zcoef_kernel<<<1216, 256, 0, s_>>>(npts_, den_.p, vrho_.p, vsig_.p, gga ? 1 : 0, zc_.p);
    GB300_CUDA(cudaGetLastError());
    launch_zmat(tk_, 0, tk_.ntasks, zc_.p, scr_.p, gga, s_);
    zgga_ = gga;
  }
  void inc_vxc() { launch_vxc_fp64(tk_, vx_.p, nvx_, scr_.p, A_.p, nbf_, zgga_, s_); }
  void symmetrize(double* VXC, int64_t ld) {
    Buf<double> V((size_t)nbf_ * nbf_);
    launch_symmetrize(A_.p, nbf_, V.p, nbf_, s_);
    const size_t row = (size_t)nbf_ * sizeof(double);
    GB300_CUDA(cudaMemcpy2DAsync(VXC, (size_t)ld * sizeof(double), V.p, row, row, nbf_,
                                 cudaMemcpyDeviceToHost, s_));
    GB300_CUDA(cudaStreamSynchronize(s_));
  }
  void results(double* exc, double* nel) {
    double h[2];
    GB300_CUDA(cudaMemcpyAsync(h, acc_.p, sizeof(h), cudaMemcpyDeviceToHost, s_));
    GB300_CUDA(cudaStreamSynchronize(s_));
    if (exc) *exc = h[0];
    if (nel) *nel = h[1];
  }
  int nbf() const { return nbf_; }

 private:
  cudaStream_t s_ = nullptr;
  int nbf_ = 0, maxnp_ = 0;
  int64_t npts_ = 0;
  bool grad_ = false, zgga_ = false;
  Buf<double> sh_alpha_, sh_coeff_, sh_origin_;
  Buf<int> sh_off_, sh_l_, sh_pure_;
  ShellsDev sh_{};
  Buf<int64_t> t_pt_off_, t_bf_off_, t_sh_off_, t_scr_off_, xoff_;
  Buf<int> t_npts_, t_nbe_, t_nbe_pad_, t_bf_, t_nsh_, t_sh_, t_sh_col_;
  Buf<double> t_x_, t_y_, t_z_, t_w_;
  TasksDev tk_{};
  Buf<int2> coll_;
  Buf<int4> xm_, vx_;
  int ncoll_ = 0, nxm_ = 0, nvx_ = 0;
  Buf<double> scr_, X_, gamma_, eps_, vrho_, vsig_, red_, acc_, P_, A_;
  Buf<double4> den_, zc_;
  Buf<double2> partials_;
};

std::shared_ptr<LWDData> lwd_create(const LoadBalancer& lb, int64_t t0, int64_t t1) {
  return std::make_shared<LWDData>(lb, t0, t1);
}
void lwd_eval_collocation(LWDData& d, bool grad) { d.eval_collocation(grad); }
void lwd_eval_xmat(LWDData& d, double fac, const double* P, int64_t ldp) {
  if (!P) throw error("null density matrix");
  if (ldp < d.nbf()) throw error("Invalid LDP");
  d.eval_xmat(fac, P, ldp);
}
void lwd_eval_vvars(LWDData& d, bool gga) { d.eval_vvars(gga); }
void lwd_eval_uvars(LWDData& d) { d.eval_uvars(); }
void lwd_eval_kern_exc_vxc(LWDData& d, const XCFunctionalDesc& f) { d.eval_kern(f); }
void lwd_inc_exc(LWDData& d) { d.inc(0); }
void lwd_inc_nel(LWDData& d) { d.inc(1); }
void lwd_eval_zmat_vxc(LWDData& d, bool gga) { d.eval_zmat(gga); }
void lwd_inc_vxc(LWDData& d) { d.inc_vxc(); }
void lwd_symmetrize_vxc(LWDData& d, double* VXC, int64_t ld) {
  if (!VXC) throw error("VXC matrix pointer cannot be null");
  if (ld < d.nbf()) throw error("Invalid LDVXC");
  d.symmetrize(VXC, ld);
}
void lwd_results(LWDData& d, double* exc, double* nel) { d.results(exc, nel); }

}  // namespace gb300
