// Launchers of the per-iteration XC kernels (FP64 and mixed precision).
#pragma once
#include "device_common.cuh"
#include "functionals.cuh"

namespace gb300 {

void launch_density_fp64(const TasksDev& tk, const int2* items, int nitems, const double* scr,
                         const double* P, int nbf, const XCFunctionalDesc& f, double4* zcoef,
                         double2* partials, cudaStream_t s);
// (rho, grad rho) of every point of the items into rho4 (no functional): the
// per-density pass of a UKS call.
void launch_density_fp64_rho(const TasksDev& tk, const int2* items, int nitems, const double* scr,
                             const double* P, int nbf, bool gga, double4* rho4, cudaStream_t s);
// Polarized functional on points [g0, g1) from the (rho, grad rho) of the
// scalar density Ps and the z density Pz (rho4s, rho4z, 4 doubles a point):
// the Z coefficients of Z_s and Z_z (FP64 double4, or float-float pairs for
// the tensor-core path when ff) and functional_partial_blocks() EXC / N_el
// partials.
void launch_functional_pol(int64_t g0, int64_t g1, const double* w, const double* rho4s,
                           const double* rho4z, const XCFunctionalDesc& f, double4* zs,
                           double4* zz, double2* partials, bool ff, cudaStream_t s);
// x[i] *= c for n doubles (device memory).
void launch_scale(double* x, int64_t n, double c, cudaStream_t s);

void launch_zmat(const TasksDev& tk, int t_begin, int ntasks, const double4* zcoef, double* scr,
                 bool gga, cudaStream_t s);
void launch_vxc_fp64(const TasksDev& tk, const int4* items, int nitems, const double* scr,
                     double* A, int nbf, bool gga, cudaStream_t s);

// VXC(i,j) = A(i,j) + A(j,i), written with leading dimension ld.
void launch_symmetrize(const double* A, int nbf, double* vxc, int64_t ld, cudaStream_t s);
// VXC = A + A^T in the caller's AO order from an accumulator held in a
// permuted order (iperm: caller's AO index -> position in A)
void launch_symmetrize_perm(const double* A, int nbf, const int* iperm, double* vxc, int64_t ld,
                            cudaStream_t s);
// dst = scale P(perm, perm) (perm: position -> caller's AO index), n x n, ld n
void launch_permute_matrix(const double* src, int nbf, const int* perm, double scale, double* dst,
                           cudaStream_t s);
// dst = src for n x n column-major matrices; either may be device-addressable host memory.
void launch_copy_matrix(const double* src, int64_t lds, double* dst, int64_t ldd, int n,
                        cudaStream_t s);
// out[0] = sum of partials[i].x, out[1] = sum of partials[i].y (compensated,
// fixed order, single CTA)
void launch_reduce_partials(const double2* partials, int64_t n, double* out, cudaStream_t s);

}  // namespace gb300
