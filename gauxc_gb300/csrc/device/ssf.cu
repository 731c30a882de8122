// Stratmann-Scuseria-Frisch partition weights on the device.
//
// Algorithm of the reference device kernel
// (src/xc_integrator/local_work_driver/device/cuda/kernels/cuda_ssf_1d.cu:24-131,
// distances from grid_to_center.cu:18-71):
//   w_p <- w_p * P_parent(p) / sum_A P_A(p),
//   P_A = prod_{B != A} s(mu_AB),  mu_AB = (r_A - r_B) / R_AB,
//   s(mu) = 1/2 - (1/32)(35 x - 35 x^3 + 21 x^5 - 5 x^7), x = mu / 0.64  for |mu| < 0.64,
//   s = 0 for mu >= 0.64 and 1 for mu <= -0.64.
// Points closer to their parent than (1 - 0.64)/2 of the parent's nearest
// neighbour distance keep their weight; a product stops once it falls to
// 1e-13 or below; a parent product below machine epsilon zeroes the weight.
//
// Layout: distances are stored atom-major (dist[a * ld + p]) so that the
// per-point loops read consecutive addresses across a warp.
#include "device_common.cuh"

#include <cfloat>

namespace gb300 {

namespace {
constexpr double kSSFa = 0.64;
constexpr double kSSFTol = 1e-13;

__global__ void grid_to_center_kernel(int64_t npts, int natoms, const double* __restrict__ x,
                                      const double* __restrict__ y, const double* __restrict__ z,
                                      const double* __restrict__ coords, double* __restrict__ dist,
                                      int ld) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const double px = x[p], py = y[p], pz = z[p];
  for (int a = blockIdx.y; a < natoms; a += gridDim.y) {
    const double dx = px - coords[3 * a + 0];
    const double dy = py - coords[3 * a + 1];
    const double dz = pz - coords[3 * a + 2];
    dist[(int64_t)a * ld + p] = sqrt(dx * dx + dy * dy + dz * dz);
  }
}

__device__ __forceinline__ double ssf_s(double mu) {
  if (fabs(mu) < kSSFa) {
    const double s = mu * 1.5625;  // mu / 0.64
    const double s2 = s * s, s3 = s * s2, s5 = s3 * s2, s7 = s5 * s2;
    return 0.5 - (0.5 / 16.) * (35. * (s - s3) + 21. * s5 - 5. * s7);
  }
  return mu >= kSSFa ? 0. : 1.;
}

__device__ __forceinline__ double cell_product(int A, int natoms, int64_t p, const double* dist,
                                               int ld, const double* __restrict__ rab_inv,
                                               int ld_rab) {
  const double rA = dist[(int64_t)A * ld + p];
  const double* rinv = rab_inv + (int64_t)A * ld_rab;
  double ps = 1.;
  for (int B = 0; B < natoms; ++B) {
    if (ps <= kSSFTol) break;
    if (B == A) continue;
    ps *= ssf_s((rA - dist[(int64_t)B * ld + p]) * rinv[B]);
  }
  return ps;
}

__global__ void ssf_weights_kernel(int64_t npts, int natoms, const int32_t* __restrict__ iparent,
                                   const double* __restrict__ dist_nearest,
                                   const double* __restrict__ rab_inv, int ld_rab,
                                   const double* __restrict__ dist, int ld,
                                   double* __restrict__ weights, int* __restrict__ status) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int ip = iparent[p];
  if (ip < 0 || ip >= natoms) {
    // a parent index outside the molecule: the point keeps its weight and
    // the call reports the error (when the caller passed a status word)
    if (status) atomicExch(status, 1);
    return;
  }
  const double cutoff = 0.5 * (1. - kSSFa) * dist_nearest[p];
  if (dist[(int64_t)ip * ld + p] < cutoff) return;
  const double parent = cell_product(ip, natoms, p, dist, ld, rab_inv, ld_rab);
  if (parent < DBL_EPSILON) {
    weights[p] = 0.;
    return;
  }
  double sum = parent;
  for (int A = 0; A < natoms; ++A) {
    if (A == ip) continue;
    sum += cell_product(A, natoms, p, dist, ld, rab_inv, ld_rab);
  }
  weights[p] *= parent / sum;
}
}  // namespace

void launch_ssf_weights(int64_t npts, int natoms, const double* x, const double* y,
                        const double* z, const int32_t* iparent, const double* dist_nearest,
                        const double* coords, const double* rab_inv, int ld_rab,
                        double* dist_scr, int ld_dist, double* weights, int* status,
                        cudaStream_t s) {
  if (npts == 0) return;
  const int threads = 256;
  dim3 g1((unsigned)((npts + threads - 1) / threads), (unsigned)std::min(natoms, 64));
  grid_to_center_kernel<<<g1, threads, 0, s>>>(npts, natoms, x, y, z, coords, dist_scr, ld_dist);
  dim3 g2((unsigned)((npts + threads - 1) / threads));
  ssf_weights_kernel<<<g2, threads, 0, s>>>(npts, natoms, iparent, dist_nearest, rab_inv, ld_rab,
                                            dist_scr, ld_dist, weights, status);
  GB300_CUDA(cudaGetLastError());
}

}  // namespace gb300
