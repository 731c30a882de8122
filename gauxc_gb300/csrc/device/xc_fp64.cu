// Plain FP64 path of the per-iteration XC integration: density (with the
// X = phi * P_sub contraction fused in), functional, Z matrix, VXC
// contraction with the scatter-add, symmetrization and the EXC / N_el sums.
//
// Reference stages (src/xc_integrator/local_work_driver/device/scheme1_base.cxx):
//   eval_xmat (fac = 2) + sym_pack_submat        :1603-1664, kernels/pack_submat.cu
//   eval_vvars_{lda,gga}, eval_uvars_gga          :613-860, kernels/uvvars_{lda,gga}.hpp
//   eval_kern_exc_vxc_* + scale by weights        :1303-1431
//   inc_exc / inc_nel                             :558-610
//   eval_zmat_{lda,gga}_vxc                       :250-315, kernels/zmat_vxc.cu:20-47,148-187
//   inc_vxc (syr2k + atomic scatter)              :1711-1766, kernels/cuda_inc_potential.cu
//   symmetrize_vxc                                :1787-1818
//
// GB300 structure: one CTA owns 64 points of one task and streams the whole
// basis through registers, so X never touches memory and rho / grad rho are
// reduced deterministically inside the CTA; the functional is evaluated in
// the same CTA.  The VXC contraction computes full (not triangular) tiles of
// A_t = phi_t^T Z_t and scatters them into one nbf x nbf accumulator A;
// VXC = A + A^T at the end (equal to the reference's syr2k + lower-to-upper
// symmetrization, same flop count).  FP64 on GB300 is a throttled pipe, so
// these kernels are DFMA-issue bound and need only modest register tiling.
#include "device_common.cuh"
#include "functionals.cuh"
#include "xc_kernels.cuh"

namespace gb300 {

namespace {

constexpr int TM = 64, TN = 64, KT = 16, NT = 256;

// ---------------------------------------------------------------- density
// RHO: write (rho, grad rho) of each point to rho_out instead of evaluating
// the functional (the two densities of a UKS call, whose polarized
// functional runs afterwards on both).
template <bool GGA, bool RHO>
__global__ void __launch_bounds__(NT) density_fp64_kernel(TasksDev tk, const int2* __restrict__ items,
                                                          const double* __restrict__ scr,
                                                          const double* __restrict__ P, int nbf,
                                                          XCFunctionalDesc func,
                                                          double4* __restrict__ zcoef,
                                                          double2* __restrict__ partials,
                                                          double4* __restrict__ rho_out) {
  __shared__ double As[KT][TM + 1];
  __shared__ double Bs[KT][TN + 1];
  __shared__ double red[2][NT / 16];

  const int2 it = items[blockIdx.x];
  const int t = it.x;
  const int p0 = it.y * TM;
  const int np = tk.npts_pad[t];
  const int nbe_pad = tk.nbe_pad[t];
  const int64_t blk = (int64_t)np * nbe_pad;
  const double* phi = scr + tk.scr_off[t];
  const double* phx = phi + blk;
  const double* phy = phx + blk;
  const double* phz = phy + blk;
  const int* bf = tk.bf_list + tk.bf_off[t];

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;

  double rho[4] = {0, 0, 0, 0}, gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0}, gz[4] = {0, 0, 0, 0};

  for (int n0 = 0; n0 < nbe_pad; n0 += TN) {
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.;

    for (int k0 = 0; k0 < nbe_pad; k0 += KT) {
      // A tile: phi[k0+k][p0+p]; B tile: P[bf(n0+n), bf(k0+k)] (P symmetric)
#pragma unroll
      for (int r = 0; r < (KT * TM) / NT; ++r) {
        const int e = tid + r * NT;
        const int k = e / TM, p = e % TM;
        As[k][p] = phi[(int64_t)(k0 + k) * np + p0 + p];
        const int gk = bf[k0 + k], gn = bf[n0 + p];
        Bs[k][p] = (gk >= 0 && gn >= 0) ? P[(int64_t)gk * nbf + gn] : 0.;
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
    // contract the X tile with phi (and grad phi) of the same columns
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t col = (int64_t)(n0 + tx + 16 * j) * np + p0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t o = col + ty + 16 * i;
        rho[i] = fma(phi[o], acc[i][j], rho[i]);
        if (GGA) {
          gx[i] = fma(phx[o], acc[i][j], gx[i]);
          gy[i] = fma(phy[o], acc[i][j], gy[i]);
          gz[i] = fma(phz[o], acc[i][j], gz[i]);
        }
      }
    }
  }

  // reduce across the 16 column threads of each point row
#pragma unroll
  for (int off = 8; off > 0; off >>= 1) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      rho[i] += __shfl_xor_sync(0xffffffffu, rho[i], off);
      if (GGA) {
        gx[i] += __shfl_xor_sync(0xffffffffu, gx[i], off);
        gy[i] += __shfl_xor_sync(0xffffffffu, gy[i], off);
        gz[i] += __shfl_xor_sync(0xffffffffu, gz[i], off);
      }
    }
  }

  if (RHO) {
    if (tx == 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t g = tk.pt_off[t] + p0 + ty + 16 * i;
        rho_out[g] = GGA ? make_double4(2. * rho[i], 4. * gx[i], 4. * gy[i], 4. * gz[i])
                         : make_double4(2. * rho[i], 0., 0., 0.);
      }
    }
    return;
  }
  double exc_loc = 0., nel_loc = 0.;
  if (tx == 0) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int p = p0 + ty + 16 * i;
      const int64_t g = tk.pt_off[t] + p;
      const double w = tk.w[g];
      const double r = 2. * rho[i];  // X = 2 P phi  (RKS, P = alpha density)
      double dx = 0., dy = 0., dz = 0., sigma = 0.;
      if (GGA) {
        dx = 4. * gx[i];
        dy = 4. * gy[i];
        dz = 4. * gz[i];
        sigma = dx * dx + dy * dy + dz * dz;
      }
      double eps, vrho, vsigma;
      xc_eval_unpol(func, r, sigma, eps, vrho, vsigma);
      exc_loc += (w * eps) * r;
      nel_loc += w * r;
      const double gf = 2. * w * vsigma;
      zcoef[g] = make_double4(0.5 * w * vrho, gf * dx, gf * dy, gf * dz);
    }
    red[0][ty] = exc_loc;
    red[1][ty] = nel_loc;
  }
  __syncthreads();
  if (tid == 0) {
    double e = 0., n = 0.;
    for (int i = 0; i < NT / 16; ++i) {
      e += red[0][i];
      n += red[1][i];
    }
    partials[blockIdx.x] = make_double2(e, n);
  }
}

// ---------------------------------------------------------------- Z matrix
// Z[col][p] = zc.x * phi + zc.y * dphi_x + zc.z * dphi_y + zc.w * dphi_z
template <bool GGA>
__global__ void zmat_kernel(TasksDev tk, int t_begin, const double4* __restrict__ zcoef,
                            double* __restrict__ scr) {
  const int t = t_begin + blockIdx.y;
  const int np = tk.npts_pad[t];
  const int64_t blk = (int64_t)np * tk.nbe_pad[t];
  const double* phi = scr + tk.scr_off[t];
  double* Z = const_cast<double*>(phi) + (GGA ? 4 : 1) * blk;
  const double4* zc = zcoef + tk.pt_off[t];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < blk;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(e % np);
    const double4 c = zc[p];
    double v = c.x * phi[e];
    if (GGA) v += c.y * phi[e + blk] + c.z * phi[e + 2 * blk] + c.w * phi[e + 3 * blk];
    Z[e] = v;
  }
}

// ---------------------------------------------------------------- VXC
// A[bf(I), bf(J)] += sum_p phi[I][p] Z[J][p]  for one 64 x 64 tile of a task.
template <bool GGA>
__global__ void __launch_bounds__(NT) vxc_fp64_kernel(TasksDev tk, const int4* __restrict__ items,
                                                      const double* __restrict__ scr,
                                                      double* __restrict__ A, int nbf) {
  __shared__ double As[KT][TM + 1];
  __shared__ double Bs[KT][TN + 1];
  const int4 it = items[blockIdx.x];
  const int t = it.x;
  const int I0 = it.y * TM, J0 = it.z * TN;
  const int np = tk.npts_pad[t];
  const int64_t blk = (int64_t)np * tk.nbe_pad[t];
  const double* phi = scr + tk.scr_off[t];
  const double* Z = phi + (GGA ? 4 : 1) * blk;
  const int* bf = tk.bf_list + tk.bf_off[t];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.;

  for (int k0 = 0; k0 < np; k0 += KT) {
#pragma unroll
    for (int r = 0; r < (KT * TM) / NT; ++r) {
      const int e = tid + r * NT;
      const int row = e / KT, k = e % KT;
      As[k][row] = phi[(int64_t)(I0 + row) * np + k0 + k];
      Bs[k][row] = Z[(int64_t)(J0 + row) * np + k0 + k];
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
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gi = bf[I0 + ty + 16 * i];
    if (gi < 0) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gj = bf[J0 + tx + 16 * j];
      // accumulates A^T (row gi, column gj of A^T is contiguous in gj);
      // only A + A^T is ever used
      if (gj >= 0) atomicAdd(&A[(int64_t)gi * nbf + gj], acc[i][j]);
    }
  }
}

}  // namespace

void launch_density_fp64(const TasksDev& tk, const int2* items, int nitems, const double* scr,
                         const double* P, int nbf, const XCFunctionalDesc& f, double4* zcoef,
                         double2* partials, cudaStream_t s) {
  if (!nitems) return;
  if (f.is_gga)
    density_fp64_kernel<true, false>
        <<<nitems, NT, 0, s>>>(tk, items, scr, P, nbf, f, zcoef, partials, nullptr);
  else
    density_fp64_kernel<false, false>
        <<<nitems, NT, 0, s>>>(tk, items, scr, P, nbf, f, zcoef, partials, nullptr);
  GB300_CUDA(cudaGetLastError());
}

void launch_density_fp64_rho(const TasksDev& tk, const int2* items, int nitems, const double* scr,
                             const double* P, int nbf, bool gga, double4* rho4, cudaStream_t s) {
  if (!nitems) return;
  XCFunctionalDesc f{};
  if (gga)
    density_fp64_kernel<true, true>
        <<<nitems, NT, 0, s>>>(tk, items, scr, P, nbf, f, nullptr, nullptr, rho4);
  else
    density_fp64_kernel<false, true>
        <<<nitems, NT, 0, s>>>(tk, items, scr, P, nbf, f, nullptr, nullptr, rho4);
  GB300_CUDA(cudaGetLastError());
}

void launch_zmat(const TasksDev& tk, int t_begin, int ntasks, const double4* zcoef, double* scr,
                 bool gga, cudaStream_t s) {
  if (!ntasks) return;
  dim3 g(64, ntasks);
  if (gga)
    zmat_kernel<true><<<g, 256, 0, s>>>(tk, t_begin, zcoef, scr);
  else
    zmat_kernel<false><<<g, 256, 0, s>>>(tk, t_begin, zcoef, scr);
  GB300_CUDA(cudaGetLastError());
}

void launch_vxc_fp64(const TasksDev& tk, const int4* items, int nitems, const double* scr,
                     double* A, int nbf, bool gga, cudaStream_t s) {
  if (!nitems) return;
  if (gga)
    vxc_fp64_kernel<true><<<nitems, NT, 0, s>>>(tk, items, scr, A, nbf);
  else
    vxc_fp64_kernel<false><<<nitems, NT, 0, s>>>(tk, items, scr, A, nbf);
  GB300_CUDA(cudaGetLastError());
}

}  // namespace gb300
