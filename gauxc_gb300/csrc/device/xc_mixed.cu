// Mixed-precision path, element-wise kernels: power-of-two scales, digit
// (slice) generation for P, phi and Z, and the per-point functional.
//
// Layouts per point block (np points, nu_pad basis rows, see xc_mixed.cuh):
//   FP64 region (at f64_off): phi[mu][p] (+ d/dx, d/dy, d/dz) in FP64,
//     r[nu_pad], sp[np], cz[nu_pad], then phi (+ grad) as float-float pairs
//   digits (bf16, at dig_off): Pd[s][nu][mu], Fd[s][p][mu], FdT[s][mu][p],
//     Zd[s][nu][p]   (K index contiguous in every GEMM operand)
// Scales are powers of two taken from IEEE exponent bits and digits come from
// integer arithmetic on the fixed-point value (ffmath.cuh), so these kernels
// issue almost no FP64 instructions.
#include <cuda_bf16.h>

#include <cfloat>

#include "ffmath.cuh"
#include "functionals.cuh"
#include "xc_mixed.cuh"

namespace gb300 {

namespace {

__device__ __forceinline__ int exp_of_pow2(double p) {
  return (int)(((unsigned long long)__double_as_longlong(p) >> 52) & 0x7FF) - 1023;
}

// digits of v (|v| < 2^es) written as kSlices bf16 values, `stride` apart
__device__ __forceinline__ void write_digits(double v, int es, __nv_bfloat16* out, int64_t stride) {
  ff::digits<kSlices>(ff::fixed42(v, es),
                      [&](int i, float x) { out[i * stride] = __float2bfloat16_rn(x); });
}

struct PBView {
  int np, nu, nu_pad;
  int64_t blk;
  const double* phi;
  double *r, *sp, *cz;
  float2* phi2;  // float-float copies of phi (+ grad)
  __nv_bfloat16 *Pd, *Fd, *FdT, *Zd;
};

__device__ __forceinline__ PBView view(const TasksDev& tk, const MixedPBDev& mp, int b, bool gga,
                                       const double* f64c, const __nv_bfloat16* digc) {
  double* f64 = const_cast<double*>(f64c);
  __nv_bfloat16* dig = const_cast<__nv_bfloat16*>(digc);
  PBView v;
  v.np = tk.npts_pad[b];
  v.nu = tk.nbe[b];
  v.nu_pad = tk.nbe_pad[b];
  v.blk = (int64_t)v.np * v.nu_pad;
  double* base = f64 + mp.f64_off[b];
  v.phi = base;
  v.r = base + (gga ? 4 : 1) * v.blk;
  v.sp = v.r + v.nu_pad;
  v.cz = v.sp + v.np;
  v.phi2 = reinterpret_cast<float2*>(v.cz + v.nu_pad);
  const int64_t S = kSlices;
  __nv_bfloat16* d = dig + mp.dig_off[b];
  v.Pd = d;
  v.Fd = d + S * v.nu_pad * v.nu_pad;
  v.FdT = v.Fd + S * v.blk;
  v.Zd = v.FdT + S * v.blk;
  return v;
}

// ---------------------------------------------------------------- point scales
__global__ void point_scale_kernel(TasksDev tk, MixedPBDev mp, int b0, double* f64, int gga) {
  const int b = b0 + blockIdx.y;
  PBView v = view(tk, mp, b, gga, f64, nullptr);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < v.np; p += gridDim.x * blockDim.x) {
    unsigned long long m = 0;
    for (int mu = 0; mu < v.nu; ++mu) m = max(m, ff::abs_key(v.phi[(int64_t)mu * v.np + p]));
    v.sp[p] = ff::pow2(ff::scale_exponent(m));
  }
}

// ---------------------------------------------------------------- phi digits
// 32 x 32 tiles (mu x p): FdT written along p, Fd written along mu through
// smem; float-float copies of phi (+ grad) for the density epilogue.
__global__ void phi_digits_kernel(TasksDev tk, MixedPBDev mp, int b0, const double* f64,
                                  __nv_bfloat16* dig, int gga) {
  __shared__ __nv_bfloat16 t[kSlices][32][34];
  const int b = b0 + blockIdx.y;
  PBView v = view(tk, mp, b, gga, f64, dig);
  const int tmu = v.nu_pad / 32, tp = v.np / 32;
  const int nq = gga ? 4 : 1;
  for (int tile = blockIdx.x; tile < tmu * tp; tile += gridDim.x) {
    const int mu0 = (tile / tp) * 32, p0 = (tile % tp) * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
      const int mu = mu0 + r, p = p0 + threadIdx.x;
      const int64_t o = (int64_t)mu * v.np + p;
      const double x = v.phi[o];
      const int es = exp_of_pow2(v.sp[p]);
      ff::digits<kSlices>(ff::fixed42(x, es), [&](int i, float d) {
        const __nv_bfloat16 h = __float2bfloat16_rn(d);
        v.FdT[i * v.blk + o] = h;
        t[i][r][threadIdx.x] = h;
      });
      for (int q = 0; q < nq; ++q) v.phi2[q * v.blk + o] = ff::split(v.phi[q * v.blk + o]);
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
      const int p = p0 + r, mu = mu0 + threadIdx.x;
#pragma unroll
      for (int i = 0; i < kSlices; ++i)
        v.Fd[i * v.blk + (int64_t)p * v.nu_pad + mu] = t[i][threadIdx.x][r];
    }
    __syncthreads();
  }
}

// Maximum of a 64-bit key over the CTA (blockDim.x a multiple of 32, <= 1024).
__device__ __forceinline__ unsigned long long block_max(unsigned long long m,
                                                        unsigned long long* red) {
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned long long x = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0ULL;
    for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(0xffffffffu, x, o));
    if (threadIdx.x == 0) red[0] = x;
  }
  __syncthreads();
  return red[0];
}

// ---------------------------------------------------------------- P digits
// One CTA per (row nu, block): gathers P[U_nu, U_mu], row scale, digits.
__global__ void p_digits_kernel(TasksDev tk, MixedPBDev mp, int b0, const double* __restrict__ P,
                                int nbf, double* f64, __nv_bfloat16* dig, int gga) {
  __shared__ unsigned long long red[32];
  const int b = b0 + blockIdx.y;
  PBView v = view(tk, mp, b, gga, f64, dig);
  const int row = blockIdx.x;
  if (row >= v.nu_pad) return;
  const int* bf = tk.bf_list + tk.bf_off[b];
  const int gr = bf[row];
  unsigned long long m = 0;
  if (gr >= 0)
    for (int mu = threadIdx.x; mu < v.nu; mu += blockDim.x) {
      const int gc = bf[mu];
      if (gc >= 0) m = max(m, ff::abs_key(P[(int64_t)gr * nbf + gc]));
    }
  const int es = ff::scale_exponent(block_max(m, red));
  if (threadIdx.x == 0) v.r[row] = ff::pow2(es);
  const int64_t ps = (int64_t)v.nu_pad * v.nu_pad;
  for (int mu = threadIdx.x; mu < v.nu_pad; mu += blockDim.x) {
    const int gc = mu < v.nu ? bf[mu] : -1;
    const double x = (gr >= 0 && gc >= 0) ? P[(int64_t)gr * nbf + gc] : 0.;
    write_digits(x, es, v.Pd + (int64_t)row * v.nu_pad + mu, ps);
  }
}

// ---------------------------------------------------------------- Z digits
// Zt[nu][p] = sp[p] (zc.x phi + zc.y dphi_x + zc.z dphi_y + zc.w dphi_z),
// column scale cz[nu] over the block's points, digits Zd[s][nu][p].
__global__ void z_digits_kernel(TasksDev tk, MixedPBDev mp, int b0, const double4* __restrict__ zc,
                                double* f64, __nv_bfloat16* dig, int gga) {
  __shared__ unsigned long long red[32];
  const int b = b0 + blockIdx.y;
  PBView v = view(tk, mp, b, gga, f64, dig);
  const int row = blockIdx.x;
  if (row >= v.nu_pad) return;
  const double4* z = zc + tk.pt_off[b];
  const double* f = v.phi + (int64_t)row * v.np;
  auto zval = [&](int p) {
    const double4 c = z[p];
    double val = c.x * f[p];
    if (gga) val += c.y * f[p + v.blk] + c.z * f[p + 2 * v.blk] + c.w * f[p + 3 * v.blk];
    return v.sp[p] * val;
  };
  unsigned long long m = 0;
  for (int p = threadIdx.x; p < v.np; p += blockDim.x) m = max(m, ff::abs_key(zval(p)));
  const int es = ff::scale_exponent(block_max(m, red));
  if (threadIdx.x == 0) v.cz[row] = ff::pow2(es);
  for (int p = threadIdx.x; p < v.np; p += blockDim.x)
    write_digits(zval(p), es, v.Zd + (int64_t)row * v.np + p, v.blk);
}

// ---------------------------------------------------------------- functional
__global__ void functional_kernel(int64_t g0, int64_t g1, const double* __restrict__ w,
                                  const double* __restrict__ rho4, XCFunctionalDesc func,
                                  double4* __restrict__ zcoef, double2* __restrict__ partials) {
  __shared__ double se[256], sn[256];
  double e = 0., n = 0.;
  for (int64_t g = g0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < g1;
       g += (int64_t)gridDim.x * blockDim.x) {
    const double r = rho4[4 * g];
    const double dx = rho4[4 * g + 1], dy = rho4[4 * g + 2], dz = rho4[4 * g + 3];
    const double sigma = func.is_gga ? dx * dx + dy * dy + dz * dz : 0.;
    double eps, vr, vs;
    xc_eval_unpol(func, r, sigma, eps, vr, vs);
    const double wg = w[g];
    e += (wg * eps) * r;
    n += wg * r;
    const double gf = 2. * wg * vs;
    zcoef[g] = func.is_gga ? make_double4(0.5 * wg * vr, gf * dx, gf * dy, gf * dz)
                           : make_double4(0.5 * wg * vr, 0., 0., 0.);
  }
  se[threadIdx.x] = e;
  sn[threadIdx.x] = n;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      se[threadIdx.x] += se[threadIdx.x + o];
      sn[threadIdx.x] += sn[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = make_double2(se[0], sn[0]);
}

}  // namespace

void launch_point_scales(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, bool gga,
                         double* f64, cudaStream_t s) {
  if (b1 <= b0) return;
  point_scale_kernel<<<dim3(kPBMaxPts / 128, b1 - b0), 128, 0, s>>>(tk, mp, b0, f64, gga);
  GB300_CUDA(cudaGetLastError());
}

void launch_phi_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, bool gga,
                       const double* f64, __nv_bfloat16* dig, cudaStream_t s) {
  if (b1 <= b0) return;
  phi_digits_kernel<<<dim3(128, b1 - b0), dim3(32, 8), 0, s>>>(tk, mp, b0, f64, dig, gga);
  GB300_CUDA(cudaGetLastError());
}

void launch_p_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, int max_nu_pad,
                     bool gga, const double* P, int nbf, double* f64, __nv_bfloat16* dig,
                     cudaStream_t s) {
  if (b1 <= b0) return;
  p_digits_kernel<<<dim3(max_nu_pad, b1 - b0), 256, 0, s>>>(tk, mp, b0, P, nbf, f64, dig, gga);
  GB300_CUDA(cudaGetLastError());
}

void launch_z_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, int max_nu_pad,
                     bool gga, const double4* zcoef, double* f64, __nv_bfloat16* dig,
                     cudaStream_t s) {
  if (b1 <= b0) return;
  z_digits_kernel<<<dim3(max_nu_pad, b1 - b0), 128, 0, s>>>(tk, mp, b0, zcoef, f64, dig, gga);
  GB300_CUDA(cudaGetLastError());
}

int functional_partial_blocks() { return 512; }

void launch_functional(int64_t g0, int64_t g1, const double* w, const double* rho4,
                       const XCFunctionalDesc& f, double4* zcoef, double2* partials,
                       cudaStream_t s) {
  if (g1 <= g0) return;
  functional_kernel<<<functional_partial_blocks(), 256, 0, s>>>(g0, g1, w, rho4, f, zcoef,
                                                                partials);
  GB300_CUDA(cudaGetLastError());
}

}  // namespace gb300
