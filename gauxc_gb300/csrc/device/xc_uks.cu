// UKS (spin-polarized) stage of the XC pass: the polarized functional on the
// (rho, grad rho) of the scalar and z densities, giving the Z coefficients of
// Z_s and Z_z, and the EXC / N_el partials.
//
// Reference (host driver, restated by the oracle):
//   rho_+- = (rho_s +- rho_z) / 2; grad n, grad M from X_s = P_s phi,
//   X_z = P_z phi; sigma_aa, sigma_ab, sigma_bb of eval_uvvar_gga_uks
//   (reference_local_host_work_driver.cxx:270-327; device uvvars_gga.hpp
//   UKS kernels); vrho, vsigma scaled by the weights
//   (reference_replicated_xc_host_integrator_exc_vxc.hpp:453-475);
//   Z_s = ((fp + fm) / 2) phi + (g1 grad n + g2 grad M) . grad phi,
//   Z_z = ((fp - fm) / 2) phi + (g3 grad M + g2 grad n) . grad phi with
//   fp = w vrho_a / 2, fm = w vrho_b / 2, g1 = w (v_aa + v_ab + v_bb) / 2,
//   g2 = w (v_aa - v_bb) / 2, g3 = w (v_aa - v_ab + v_bb) / 2
//   (eval_zmat_{lda,gga}_vxc_uks, :607-631, :715-770; device zmat_vxc.cu:62-94,
//   197-275).
// The two density passes run the RKS kernels on P_s / 2 and P_z / 2 (an exact
// power-of-two scaling), whose X = 2 P phi then equals the reference's
// X = P phi of each density; Z_s and Z_z go through the RKS Z and VXC kernels.
#include "ffmath.cuh"
#include "functionals_pol.cuh"
#include "xc_kernels.cuh"
#include "xc_mixed.cuh"

namespace gb300 {

namespace {

template <bool FF>
__global__ void functional_pol_kernel(int64_t g0, int64_t g1, const double* __restrict__ w,
                                      const double* __restrict__ rs,
                                      const double* __restrict__ rz, XCFunctionalDesc func,
                                      double4* __restrict__ zs, double4* __restrict__ zz,
                                      double2* __restrict__ partials) {
  __shared__ double se[256], sn[256];
  double e = 0., n = 0.;
  for (int64_t g = g0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < g1;
       g += (int64_t)gridDim.x * blockDim.x) {
    const double rho_s = rs[4 * g], rho_z = rz[4 * g];
    const double ra = 0.5 * (rho_s + rho_z), rb = 0.5 * (rho_s - rho_z);
    double gn[3] = {0., 0., 0.}, gm[3] = {0., 0., 0.};
    if (func.is_gga)
      for (int a = 0; a < 3; ++a) {
        gn[a] = rs[4 * g + 1 + a];
        gm[a] = rz[4 * g + 1 + a];
      }
    const double nn = gn[0] * gn[0] + gn[1] * gn[1] + gn[2] * gn[2];
    const double mm = gm[0] * gm[0] + gm[1] * gm[1] + gm[2] * gm[2];
    const double nm = gn[0] * gm[0] + gn[1] * gm[1] + gn[2] * gm[2];
    const double saa = 0.25 * (nn + mm) + 0.5 * nm, sab = 0.25 * (nn - mm),
                 sbb = 0.25 * (nn + mm) - 0.5 * nm;
    double eps, vr[2], vs[3];
    xc_eval_pol(func, ra, rb, saa, sab, sbb, eps, vr, vs);
    const double wg = w[g];
    e += (wg * eps) * (ra + rb);
    n += wg * (ra + rb);
    const double fp = 0.5 * wg * vr[0], fm = 0.5 * wg * vr[1];
    const double g1c = 0.5 * wg * (vs[0] + vs[1] + vs[2]), g2c = 0.5 * wg * (vs[0] - vs[2]),
                 g3c = 0.5 * wg * (vs[0] - vs[1] + vs[2]);
    double cs[4] = {0.5 * (fp + fm), 0., 0., 0.}, cz[4] = {0.5 * (fp - fm), 0., 0., 0.};
    if (func.is_gga)
      for (int a = 0; a < 3; ++a) {
        cs[1 + a] = g1c * gn[a] + g2c * gm[a];
        cz[1 + a] = g3c * gm[a] + g2c * gn[a];
      }
    if (FF) {
      // float-float pairs in the point's 32-byte slot (as functional_kernel)
      float4* qs = reinterpret_cast<float4*>(zs + g);
      float4* qz = reinterpret_cast<float4*>(zz + g);
      float2 p[4], q[4];
      for (int k = 0; k < 4; ++k) {
        p[k] = ff::split(cs[k]);
        q[k] = ff::split(cz[k]);
      }
      qs[0] = make_float4(p[0].x, p[0].y, p[1].x, p[1].y);
      qs[1] = make_float4(p[2].x, p[2].y, p[3].x, p[3].y);
      qz[0] = make_float4(q[0].x, q[0].y, q[1].x, q[1].y);
      qz[1] = make_float4(q[2].x, q[2].y, q[3].x, q[3].y);
    } else {
      zs[g] = make_double4(cs[0], cs[1], cs[2], cs[3]);
      zz[g] = make_double4(cz[0], cz[1], cz[2], cz[3]);
    }
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

__global__ void scale_kernel(double* __restrict__ x, int64_t n, double c) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= c;
}

}  // namespace

void launch_functional_pol(int64_t g0, int64_t g1, const double* w, const double* rho4s,
                           const double* rho4z, const XCFunctionalDesc& f, double4* zs,
                           double4* zz, double2* partials, bool ff, cudaStream_t s) {
  const int nb = functional_partial_blocks();
  if (g1 <= g0) {
    GB300_CUDA(cudaMemsetAsync(partials, 0, (size_t)nb * sizeof(double2), s));
    return;
  }
  if (ff)
    functional_pol_kernel<true><<<nb, 256, 0, s>>>(g0, g1, w, rho4s, rho4z, f, zs, zz, partials);
  else
    functional_pol_kernel<false><<<nb, 256, 0, s>>>(g0, g1, w, rho4s, rho4z, f, zs, zz, partials);
  GB300_CUDA(cudaGetLastError());
}

void launch_scale(double* x, int64_t n, double c, cudaStream_t s) {
  if (n <= 0) return;
  scale_kernel<<<1216, 256, 0, s>>>(x, n, c);
  GB300_CUDA(cudaGetLastError());
}

}  // namespace gb300
