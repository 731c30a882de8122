// Collocation of basis functions (and their gradients) on the task grids.
//
// phi_mu(r_p) = R(|r_p - O|) * S_mu(r_p - O), R(r) = sum_k c_k exp(-a_k r^2),
// grad phi = (r_p - O) R1 S + R grad S,  R1 = -2 sum_k a_k c_k exp(-a_k r^2)
// (reference: collocation_device_masked_combined_kernel,
//  kernels/collocation_masked_combined_kernels.hpp:26-92, and the gradient
//  shell-to-task kernels kernels/collocation/collocation_shell_to_task_kernels_*).
//
// Output layout per task (batch scratch at scr + scr_off[t]): column-major
// phi[col * npts_pad + p] (points fastest), followed by d/dx, d/dy, d/dz
// blocks when gradients are requested.  Padding columns are written as zero.
// One thread owns one point and walks the task's shell list, so every store
// of a warp covers 32 consecutive points of one column.
//
// The value type is double for the FP64 path and a float-float pair (ff::ffl,
// same 8-byte slots) for the point blocks of the tensor-core path, where the
// digits need about 44 significant bits: FP32 instructions then replace the
// FP64 ones of exp and of the angular polynomials, GB300's FP64 pipe being
// about 64 times slower than its FP32 pipe.
#include <cmath>
#include <cstring>
#include <type_traits>

#include "device_common.cuh"
#include "ffmath.cuh"
#include "xc_mixed.cuh"
#include "collocation_angular.inc"

namespace gb300 {

namespace {

// Value sink for the generated angular code: stores a float-float value and
// keeps the largest |hi| seen, as IEEE magnitude bits, in *m.
struct MaxSink {
  ff::ffl* p;
  unsigned* m;
  struct Ref {
    ff::ffl* q;
    unsigned* m;
    __device__ __forceinline__ void operator=(ff::ffl v) const {
      *q = v;
      *m = max(*m, __float_as_uint(v.hi) & 0x7FFFFFFFu);
    }
  };
  __device__ __forceinline__ Ref operator[](int64_t i) const { return Ref{p + i, m}; }
};

template <bool GRAD, typename V, typename O>
__device__ __forceinline__ void eval_shell(int l, int pure, V x, V y, V z, V R, V R1, O f, O fx,
                                           O fy, O fz, int64_t s) {
  if (GRAD) {
    if (pure) {
      switch (l) {
        case 0: ang_grad_p_0(x, y, z, R, R1, f, fx, fy, fz, s); break;
        case 1: ang_grad_p_1(x, y, z, R, R1, f, fx, fy, fz, s); break;
        case 2: ang_grad_p_2(x, y, z, R, R1, f, fx, fy, fz, s); break;
        case 3: ang_grad_p_3(x, y, z, R, R1, f, fx, fy, fz, s); break;
        default: ang_grad_p_4(x, y, z, R, R1, f, fx, fy, fz, s); break;
      }
    } else {
      switch (l) {
        case 0: ang_grad_c_0(x, y, z, R, R1, f, fx, fy, fz, s); break;
        case 1: ang_grad_c_1(x, y, z, R, R1, f, fx, fy, fz, s); break;
        case 2: ang_grad_c_2(x, y, z, R, R1, f, fx, fy, fz, s); break;
        case 3: ang_grad_c_3(x, y, z, R, R1, f, fx, fy, fz, s); break;
        default: ang_grad_c_4(x, y, z, R, R1, f, fx, fy, fz, s); break;
      }
    }
  } else {
    if (pure) {
      switch (l) {
        case 0: ang_eval_p_0(x, y, z, R, f, s); break;
        case 1: ang_eval_p_1(x, y, z, R, f, s); break;
        case 2: ang_eval_p_2(x, y, z, R, f, s); break;
        case 3: ang_eval_p_3(x, y, z, R, f, s); break;
        default: ang_eval_p_4(x, y, z, R, f, s); break;
      }
    } else {
      switch (l) {
        case 0: ang_eval_c_0(x, y, z, R, f, s); break;
        case 1: ang_eval_c_1(x, y, z, R, f, s); break;
        case 2: ang_eval_c_2(x, y, z, R, f, s); break;
        case 3: ang_eval_c_3(x, y, z, R, f, s); break;
        default: ang_eval_c_4(x, y, z, R, f, s); break;
      }
    }
  }
}

// With MASK, a block of merged tasks is evaluated on its union shell list and
// a shell outside the point's own task list contributes exact zeros, so the
// merged block reproduces the per-task screening of the reference.
// exp(-a r2) in the value type's arithmetic
__device__ __forceinline__ double exp_neg_v(double x, const float2*) { return exp(x); }
__device__ __forceinline__ ff::ffl exp_neg_v(ff::ffl x, const float2* tab) {
  return ff::exp_neg(x, tab);
}

template <bool GRAD, bool MASK, typename V>
__global__ void __launch_bounds__(128) collocation_kernel(ShellsDev sh, TasksDev tk, PBMaskDev mk,
                                                          const int2* __restrict__ items,
                                                          double* __restrict__ scr) {
  // float-float path: the table of 2^(j/32) in shared memory
  __shared__ float2 tab[32];
  if constexpr (!std::is_same<V, double>::value) {
    if (threadIdx.x < 32) tab[threadIdx.x] = sh.exp2_tab[threadIdx.x];
    __syncthreads();
  }
  const int2 it = items[blockIdx.x];
  const int t = it.x;
  const int p = it.y * blockDim.x + threadIdx.x;
  const int np = tk.npts_pad[t];
  if (p >= np) return;
  const int64_t g = tk.pt_off[t] + p;
  const V px = V(tk.x[g]), py = V(tk.y[g]), pz = V(tk.z[g]);
  const int64_t ld = np;
  const int64_t blk = (int64_t)np * tk.nbe_pad[t];
  V* f = reinterpret_cast<V*>(scr + tk.scr_off[t]);
  V* fx = f + blk;
  V* fy = fx + blk;
  V* fz = fy + blk;
  const V zero = V(0);
  const int64_t s0 = tk.sh_off[t];
  const int ns = tk.nsh[t];
  const uint8_t* active = nullptr;
  if (MASK) active = mk.mask + mk.mask_off[t] + (int64_t)mk.member[g] * ns;
  unsigned mval = 0, mgrad = 0;  // largest |phi|, |grad phi| of the point (mixed path)
  for (int i = 0; i < ns; ++i) {
    const int s = tk.sh_list[s0 + i];
    const int col = tk.sh_col[s0 + i];
    if (MASK && !active[i]) {
      const int sz = sh.pure[s] ? 2 * sh.l[s] + 1 : (sh.l[s] + 1) * (sh.l[s] + 2) / 2;
      for (int m = 0; m < sz; ++m) {
        const int64_t o = (int64_t)(col + m) * ld + p;
        f[o] = zero;
        if (GRAD) {
          fx[o] = zero;
          fy[o] = zero;
          fz[o] = zero;
        }
      }
      continue;
    }
    const V dx = px - V(sh.origin[3 * s + 0]);
    const V dy = py - V(sh.origin[3 * s + 1]);
    const V dz = pz - V(sh.origin[3 * s + 2]);
    const V r2 = dx * dx + dy * dy + dz * dz;
    V R = zero, R1 = zero;
    for (int k = sh.prim_off[s]; k < sh.prim_off[s + 1]; ++k) {
      const V a = V(sh.alpha[k]);
      const V e = V(sh.coeff[k]) * exp_neg_v(-(a * r2), tab);
      R = R + e;
      if (GRAD) R1 = R1 + a * e;
    }
    R1 = R1 * V(-2);
    const int64_t o = (int64_t)col * ld + p;
    if constexpr (MASK) {
      eval_shell<GRAD>(sh.l[s], sh.pure[s], dx, dy, dz, R, R1, MaxSink{f + o, &mval},
                       MaxSink{fx + o, &mgrad}, MaxSink{fy + o, &mgrad}, MaxSink{fz + o, &mgrad}, ld);
    } else {
      eval_shell<GRAD>(sh.l[s], sh.pure[s], dx, dy, dz, R, R1, f + o, fx + o, fy + o, fz + o, ld);
    }
  }
  for (int c = tk.nbe[t]; c < tk.nbe_pad[t]; ++c) {
    const int64_t o = (int64_t)c * ld + p;
    f[o] = zero;
    if (GRAD) {
      fx[o] = zero;
      fy[o] = zero;
      fz[o] = zero;
    }
  }
  if constexpr (MASK) {
    // the point's scale sp (power of two above max |phi|) and the key of
    // max |grad phi|, in the block's FP64 region (PBF64)
    const PBF64 o(PBDims(np, tk.nbe[t]), GRAD ? 4 : 1);
    double* base = scr + tk.scr_off[t];
    base[o.sp + p] = ff::pow2(ff::scale_exponent_f(mval));
    reinterpret_cast<unsigned*>(base + o.gp)[p] = GRAD ? mgrad : 0u;
  }
}

}  // namespace

void launch_collocation(const ShellsDev& sh, const TasksDev& tk, const int2* items, int nitems,
                        double* scr, bool grad, cudaStream_t s) {
  if (nitems == 0) return;
  const PBMaskDev none{};
  if (grad)
    collocation_kernel<true, false, double><<<nitems, 128, 0, s>>>(sh, tk, none, items, scr);
  else
    collocation_kernel<false, false, double><<<nitems, 128, 0, s>>>(sh, tk, none, items, scr);
  GB300_CUDA(cudaGetLastError());
}

std::vector<float2> exp2_table() {
  std::vector<float2> t(32);
  for (int j = 0; j < 32; ++j) {
    const double v = std::exp2(j / 32.);
    const float hi = (float)v;
    t[j] = make_float2(hi, (float)(v - (double)hi));
  }
  return t;
}

namespace {
// exp_neg against FP64 exp on n points spread over [-50, 0]: largest relative
// error, as the bits of a non-negative double (atomicMax on the bit pattern)
__global__ void exp_neg_selftest_kernel(int n, const float2* __restrict__ gtab,
                                        unsigned long long* __restrict__ worst) {
  __shared__ float2 tab[32];
  if (threadIdx.x < 32) tab[threadIdx.x] = gtab[threadIdx.x];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double x = -50. * (double)i / (double)(n - 1) - 1e-3 * (double)(i % 7);
    const ff::ffl xf(x);
    const ff::ffl y = ff::exp_neg(xf, tab);
    const double ref = exp((double)xf.hi + (double)xf.lo);
    const double err = fabs(((double)y.hi + (double)y.lo) - ref) / ref;
    atomicMax(worst, (unsigned long long)__double_as_longlong(err));
  }
}
}  // namespace

double ff_exp_selftest(int n) {
  if (n < 2) throw std::runtime_error("ff_exp_selftest: n < 2");
  const std::vector<float2> t = exp2_table();
  float2* dtab = nullptr;
  unsigned long long* dw = nullptr;
  GB300_CUDA(cudaMalloc(&dtab, 32 * sizeof(float2)));
  GB300_CUDA(cudaMalloc(&dw, sizeof(unsigned long long)));
  GB300_CUDA(cudaMemcpy(dtab, t.data(), 32 * sizeof(float2), cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemset(dw, 0, sizeof(unsigned long long)));
  exp_neg_selftest_kernel<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256>>>(n, dtab, dw);
  GB300_CUDA(cudaGetLastError());
  unsigned long long w = 0;
  GB300_CUDA(cudaMemcpy(&w, dw, sizeof(w), cudaMemcpyDeviceToHost));
  cudaFree(dtab);
  cudaFree(dw);
  double r;
  std::memcpy(&r, &w, sizeof(r));
  return r;
}

void launch_collocation_masked(const ShellsDev& sh, const TasksDev& tk, const PBMaskDev& mk,
                               const int2* items, int nitems, double* scr, bool grad,
                               cudaStream_t s) {
  if (nitems == 0) return;
  if (grad)
    collocation_kernel<true, true, ff::ffl><<<nitems, 128, 0, s>>>(sh, tk, mk, items, scr);
  else
    collocation_kernel<false, true, ff::ffl><<<nitems, 128, 0, s>>>(sh, tk, mk, items, scr);
  GB300_CUDA(cudaGetLastError());
}

}  // namespace gb300
