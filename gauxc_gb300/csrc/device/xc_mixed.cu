// Mixed-precision path, element-wise kernels: power-of-two scales, digit
// (slice) generation for P, phi and Z, and the per-point functional.
//
// Layouts per point block (PBDims d: np points, nu basis functions):
//   FP64 region (at f64_off): PBF64 (phi, scales)
//   digits (bf16, at dig_off): Pd, Fd, Va, Vb in the tiled operand layout of
//     xc_mixed.cuh (oz_offset); every thread writes 8 consecutive K entries
//     of one row, i.e. one 16-byte row of a core matrix per digit plane
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

// Digits of 8 values x[e] (|x[e]| < 2^es[e]; double or float-float) stored as
// kSlices 16-byte rows: plane i at out + i * plane.
// Digit planes of 8 values as BF16 pairs: w[i][k] holds digit i of x[2k]
// (low half) and x[2k + 1] (high half).
template <typename T>
__device__ __forceinline__ void digits8(const T (&x)[8], const int (&es)[8],
                                        uint32_t (&w)[kSlices][4]) {
#pragma unroll
  for (int e = 0; e < 8; e += 2) {
    float a[kSlices];
    ff::digits_f32<kSlices>(ff::fixed42(x[e], es[e]), [&](int i, float v) { a[i] = v; });
    ff::digits_f32<kSlices>(ff::fixed42(x[e + 1], es[e + 1]),
                            [&](int i, float v) { w[i][e >> 1] = ff::pack_bf16x2(a[i], v); });
  }
}

__device__ __forceinline__ void store_planes(const uint32_t (&w)[kSlices][4], __nv_bfloat16* out,
                                             int64_t plane) {
#pragma unroll
  for (int i = 0; i < kSlices; ++i)
    __stcs(reinterpret_cast<uint4*>(out + i * plane), make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]));
}

template <typename T>
__device__ __forceinline__ void store_digits8(const T (&x)[8], const int (&es)[8],
                                              __nv_bfloat16* out, int64_t plane) {
  uint32_t w[kSlices][4];
  digits8(x, es, w);
  store_planes(w, out, plane);
}

using ff::ffl;

// float-float scaled by 2^e (exact in the float range)
__device__ __forceinline__ ffl scale2(ffl v, int e) {
  const float s = ff::pow2f(e);
  return ffl(v.hi * s, v.lo * s);
}

__device__ __forceinline__ unsigned abs_key_f(ffl v) { return __float_as_uint(v.hi) & 0x7FFFFFFFu; }

struct PBView {
  PBDims d;
  PBF64 o;
  const ffl* phi;            // [q][mu][p], float-float (collocation of the point blocks)
  double *r, *sp, *cz;
  unsigned* gkey;            // largest |grad phi| of each point, as float magnitude bits
  __nv_bfloat16 *Pd, *Fd, *Va, *Vb;
  __device__ PBView(const TasksDev& tk, const MixedPBDev& mp, int b, bool gga, const double* f64c,
                    const __nv_bfloat16* digc)
      : d(tk.npts_pad[b], tk.nbe[b], mp.nk[b]), o(d, gga ? 4 : 1) {
    double* base = const_cast<double*>(f64c) + mp.f64_off[b];
    phi = reinterpret_cast<const ffl*>(base);
    r = base + o.r;
    sp = base + o.sp;
    gkey = reinterpret_cast<unsigned*>(base + o.gp);
    cz = base + o.cz;
    __nv_bfloat16* dg = digc ? const_cast<__nv_bfloat16*>(digc) + mp.dig_off[b] : nullptr;
    Pd = dg + d.pd();
    Fd = dg + d.fd();
    Va = dg + d.va();
    Vb = dg + d.vb();
  }
};

// Maximum of a 64-bit key over the threads of a CTA that share (tid & 7),
// i.e. over one of 8 rows handled by the CTA (blockDim.x = 256).
__device__ __forceinline__ unsigned long long row8_max(unsigned long long m,
                                                       unsigned long long* red) {
  m = max(m, __shfl_xor_sync(0xffffffffu, m, 8));
  m = max(m, __shfl_xor_sync(0xffffffffu, m, 16));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < 8) red[w * 8 + lane] = m;
  __syncthreads();
  unsigned long long x = 0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) x = max(x, red[k * 8 + (threadIdx.x & 7)]);
  __syncthreads();
  return x;
}

// ---------------------------------------------------------------- phi digits
// Va[mu][p] (K < nk) and Vb[mu][nk + p] (rows mu < nun): one thread per
// (mu, 8 points), consecutive threads on consecutive mu.  Fd (rows p, K = mu):
// the CTA's threads walk (point, group of 8 rows) items of the CTA's share of
// the basis.  The point scales sp come from the collocation kernel.
__global__ void phi_digits_kernel(TasksDev tk, MixedPBDev mp, int b0, const double* f64,
                                  __nv_bfloat16* dig, int gga) {
  const int b = b0 + blockIdx.y;
  PBView v(tk, mp, b, gga, f64, dig);
  const PBDims& d = v.d;
  const int k2 = 2 * d.nk;
  const int stride = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  for (int u = t0; u < d.nu128 * (d.nk / 8); u += stride) {
    const int mu = u % d.nu128, p0 = (u / d.nu128) * 8;
    ffl x[8];
    int es[8];
    const float4* src = reinterpret_cast<const float4*>(v.phi + (int64_t)mu * d.np + p0);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float4 t = src[e];
      x[2 * e] = ffl(t.x, t.y);
      x[2 * e + 1] = ffl(t.z, t.w);
    }
#pragma unroll
    for (int e = 0; e < 8; ++e) es[e] = exp_of_pow2(v.sp[p0 + e]);
    uint32_t w[kSlices][4];  // one split for both operands
    digits8(x, es, w);
    store_planes(w, v.Va + oz_offset(0, mu, p0, kMTile, k2), kMTile * kBK);
    if (mu < d.nun) store_planes(w, v.Vb + oz_offset(0, mu, d.nk + p0, kNTile, k2), kNTile * kBK);
  }
  // Fd: items (point p, group of 8 rows) of this CTA's share of the row
  // groups, consecutive threads on consecutive points
  const int ng = d.nu16 / 8;
  const int per = (ng + gridDim.x - 1) / gridDim.x;
  const int g0 = blockIdx.x * per, g1 = min(ng, g0 + per);
  const int nitems = d.np * max(g1 - g0, 0);
  for (int item = threadIdx.x; item < nitems; item += blockDim.x) {
    const int p = item % d.np, mu0 = (g0 + item / d.np) * 8;
    int es[8];
    const int e0 = exp_of_pow2(v.sp[p]);
#pragma unroll
    for (int e = 0; e < 8; ++e) es[e] = e0;
    ffl x[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) x[e] = v.phi[(int64_t)(mu0 + e) * d.np + p];
    store_digits8(x, es, v.Fd + oz_offset(0, p, mu0, kNTile, d.nu16), kNTile * kBK);
  }
}

// ---------------------------------------------------------------- P digits
// Row scales of the whole density matrix, once per evaluation: rs[i] is the
// power of two above max_j |P[i][j]| (one warp per row).
__global__ void p_row_scales_kernel(const double* __restrict__ P, int nbf, double* __restrict__ rs) {
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= nbf) return;
  unsigned long long m = 0;
  for (int c = lane; c < nbf; c += 32) m = max(m, ff::abs_key(P[(int64_t)row * nbf + c]));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) rs[row] = ff::pow2(ff::scale_exponent(m));
}

// Pd (rows nu, K = mu) in one pass.  A warp owns 8 rows: it loads them 32
// columns at a time, one coalesced row load per instruction (P[U_nu, U_mu]
// is contiguous along a shell), transposes through shared memory so that lane
// (row l & 7, column group l >> 3) holds 8 consecutive entries of one row,
// and splits them with the row's global scale r[nu] = rs[row of nu].  One
// store instruction then writes four whole 128-byte core matrices of a plane.
__global__ void p_digits_kernel(TasksDev tk, MixedPBDev mp, int b0, const double* __restrict__ P,
                                const double* __restrict__ rs, int nbf, double* f64,
                                __nv_bfloat16* dig, int gga) {
  __shared__ double tile[8][8][33];
  const int b = b0 + blockIdx.y;
  PBView v(tk, mp, b, gga, f64, dig);
  const PBDims& d = v.d;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = (blockIdx.x * 8 + warp) * 8;
  if (row0 >= d.nu128) return;
  const int* bf = tk.bf_list + tk.bf_off[b];
  const int r = lane & 7, j = lane >> 3;
  const int gmy = bf[row0 + r];
  const double rr = gmy >= 0 ? rs[gmy] : ff::pow2(-1022);
  if (j == 0) v.r[row0 + r] = rr;
  int es[8];
  {
    const int e0 = exp_of_pow2(rr);
#pragma unroll
    for (int e = 0; e < 8; ++e) es[e] = e0;
  }
  double(*t)[33] = tile[warp];
  for (int c0 = 0; c0 < d.nu16; c0 += 32) {
    const int mu = c0 + lane;
    const int gc = mu < d.nu ? bf[mu] : -1;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int gr = bf[row0 + q];
      t[q][lane] = (gr >= 0 && gc >= 0) ? P[(int64_t)gr * nbf + gc] : 0.;
    }
    __syncwarp();
    if (c0 + 8 * j < d.nu16) {
      double x[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) x[e] = t[r][8 * j + e];
      store_digits8(x, es, v.Pd + oz_offset(0, row0 + r, c0 + 8 * j, kMTile, d.nu16),
                    kMTile * kBK);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- Z digits
// Zt[nu][p] = sp[p] (zc.x phi + zc.y dphi_x + zc.z dphi_y + zc.w dphi_z),
// in float-float, with one scale cz for the whole block: 2^e above the bound
//   |Zt| <= sp (|zc.x| sp + (|zc.y| + |zc.z| + |zc.w|) max|grad phi|)
// taken from exponents only (z_scale_kernel, one CTA per block).  Digits go
// to Vb[nu][p] (rows nu < nun) and Va[nu][np + p] (rows nu < nu128).
__global__ void z_scale_kernel(TasksDev tk, MixedPBDev mp, int b0, const double4* __restrict__ zc,
                               double* f64, int gga) {
  __shared__ int red[32];
  const int b = b0 + blockIdx.x;
  PBView v(tk, mp, b, gga, f64, nullptr);
  const PBDims& d = v.d;
  // coefficients of point p: zf[4 p + k], float-float (functional_kernel)
  const ffl* zf = reinterpret_cast<const ffl*>(zc + tk.pt_off[b]);
  int eb = -1000;
  for (int p = threadIdx.x; p < d.np; p += blockDim.x) {
    const int esp = exp_of_pow2(v.sp[p]);
    int t = ff::scale_exponent_f(abs_key_f(zf[4 * p])) + esp;
    if (gga) {
      const int eg = ff::scale_exponent_f(v.gkey[p]);
      t = max(t, ff::scale_exponent_f(abs_key_f(zf[4 * p + 1])) + eg);
      t = max(t, ff::scale_exponent_f(abs_key_f(zf[4 * p + 2])) + eg);
      t = max(t, ff::scale_exponent_f(abs_key_f(zf[4 * p + 3])) + eg);
      t += 2;
    }
    eb = max(eb, t + esp);
  }
  for (int o = 16; o > 0; o >>= 1) eb = max(eb, __shfl_xor_sync(0xffffffffu, eb, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = eb;
  __syncthreads();
  int es_z = -1000;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) es_z = max(es_z, red[k]);
  es_z = min(max(es_z, -1000), 1000);
  const double cz = ff::pow2(es_z);
  for (int row = threadIdx.x; row < d.nu128; row += blockDim.x) v.cz[row] = cz;
  // the point scale sp (a power of two) folds exactly into the coefficients
  ffl* zw = reinterpret_cast<ffl*>(const_cast<double4*>(zc) + tk.pt_off[b]);
  for (int p = threadIdx.x; p < d.np; p += blockDim.x) {
    const int esp = exp_of_pow2(v.sp[p]);
#pragma unroll
    for (int k = 0; k < 4; ++k) zw[4 * p + k] = scale2(zf[4 * p + k], esp);
  }
}

// One thread per (row nu, 8-point group of the nk VXC points): CTA c of the
// launch covers pairs 256 (c - zoff[b]) .. +255 of block b (zoff: CTA
// offsets of the blocks, nu128 nk / 2048 each), rows in groups of 8 with the
// point group next, so that 8 lanes write one 128-byte core matrix.
__global__ void __launch_bounds__(256, 4) z_digits_kernel(TasksDev tk, MixedPBDev mp, int b0, int b1, int c0,
                                const double4* __restrict__ zc, double* f64, __nv_bfloat16* dig,
                                int gga) {
  const int c = c0 + blockIdx.x;
  int lo = b0, hi = b1 - 1;  // last block with zoff[b] <= c
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mp.zoff[mid] <= c) lo = mid; else hi = mid - 1;
  }
  const int b = lo;
  PBView v(tk, mp, b, gga, f64, dig);
  const PBDims& d = v.d;
  const int ng = d.nk / 8;
  const int t = (c - mp.zoff[b]) * blockDim.x + threadIdx.x;
  const int row = (t / (8 * ng)) * 8 + (t & 7), g = (t % (8 * ng)) >> 3;
  if (row >= d.nu128) return;
  // coefficients already scaled by sp (z_scale_kernel): 4 float-float per point
  const float4* zf4 = reinterpret_cast<const float4*>(zc + tk.pt_off[b]) + 2 * (g * 8);
  const int es_z = exp_of_pow2(v.cz[0]);
  const int k2 = 2 * d.nk;
  // Zt in float-float, 16-byte loads: phi of 8 points is 4 float4 per value q
  const float4* f4 = reinterpret_cast<const float4*>(v.phi + (int64_t)row * d.np + g * 8);
  const int64_t qs = v.o.blk / 2;  // one value plane, in float4
  ffl x[8];
#pragma unroll
  for (int e2 = 0; e2 < 4; ++e2) {
    const float4 c0 = zf4[4 * e2], c1 = zf4[4 * e2 + 1], c2 = zf4[4 * e2 + 2], c3 = zf4[4 * e2 + 3];
    const float4 ph = f4[e2];
    ffl v0 = ffl(c0.x, c0.y) * ffl(ph.x, ph.y);
    ffl v1 = ffl(c2.x, c2.y) * ffl(ph.z, ph.w);
    if (gga) {
      const float4 gx = f4[qs + e2], gy = f4[2 * qs + e2], gz = f4[3 * qs + e2];
      v0 = v0 + ffl(c0.z, c0.w) * ffl(gx.x, gx.y) + ffl(c1.x, c1.y) * ffl(gy.x, gy.y) +
           ffl(c1.z, c1.w) * ffl(gz.x, gz.y);
      v1 = v1 + ffl(c2.z, c2.w) * ffl(gx.z, gx.w) + ffl(c3.x, c3.y) * ffl(gy.z, gy.w) +
           ffl(c3.z, c3.w) * ffl(gz.z, gz.w);
    }
    x[2 * e2] = v0;
    x[2 * e2 + 1] = v1;
  }
  int es[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) es[e] = es_z;
  uint32_t w[kSlices][4];  // one split for both operands
  digits8(x, es, w);
  store_planes(w, v.Va + oz_offset(0, row, d.nk + g * 8, kMTile, k2), kMTile * kBK);
  if (row < d.nun) store_planes(w, v.Vb + oz_offset(0, row, g * 8, kNTile, k2), kNTile * kBK);
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
    // Z coefficients for z_digits_kernel as four float-float pairs in the
    // point's 32-byte slot
    const double c0 = 0.5 * wg * vr, c1 = func.is_gga ? gf * dx : 0.,
                 c2 = func.is_gga ? gf * dy : 0., c3 = func.is_gga ? gf * dz : 0.;
    const float2 a = ff::split(c0), b = ff::split(c1), c = ff::split(c2), e = ff::split(c3);
    float4* zq = reinterpret_cast<float4*>(zcoef + g);
    zq[0] = make_float4(a.x, a.y, b.x, b.y);
    zq[1] = make_float4(c.x, c.y, e.x, e.y);
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

void launch_phi_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, bool gga,
                       const double* f64, __nv_bfloat16* dig, cudaStream_t s) {
  if (b1 <= b0) return;
  phi_digits_kernel<<<dim3(64, b1 - b0), 256, 0, s>>>(tk, mp, b0, f64, dig, gga);
  GB300_CUDA(cudaGetLastError());
}

void launch_p_row_scales(const double* P, int nbf, double* rs, cudaStream_t s) {
  if (nbf <= 0) return;
  p_row_scales_kernel<<<(nbf + 7) / 8, 256, 0, s>>>(P, nbf, rs);
  GB300_CUDA(cudaGetLastError());
}

void launch_p_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, int max_nu_pad,
                     bool gga, const double* P, const double* rs, int nbf, double* f64,
                     __nv_bfloat16* dig, cudaStream_t s) {
  if (b1 <= b0) return;
  p_digits_kernel<<<dim3(max_nu_pad / 64, b1 - b0), 256, 0, s>>>(tk, mp, b0, P, rs, nbf, f64, dig,
                                                                  gga);
  GB300_CUDA(cudaGetLastError());
}

void launch_z_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, int zc0, int zc1,
                     bool gga, const double4* zcoef, double* f64, __nv_bfloat16* dig,
                     cudaStream_t s) {
  if (b1 <= b0 || zc1 <= zc0) return;
  z_scale_kernel<<<b1 - b0, 256, 0, s>>>(tk, mp, b0, zcoef, f64, gga);
  GB300_CUDA(cudaGetLastError());
  z_digits_kernel<<<zc1 - zc0, 256, 0, s>>>(tk, mp, b0, b1, zc0, zcoef, f64, dig, gga);
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
