// Launchers of the per-iteration XC kernels (FP64 and mixed precision).
#pragma once
#include "device_common.cuh"
#include "functionals.cuh"

namespace gb300 {

void launch_density_fp64(const TasksDev& tk, const int2* items, int nitems, const double* scr,
                         const double* P, int nbf, const XCFunctionalDesc& f, double4* zcoef,
                         double2* partials, cudaStream_t s);
void launch_zmat(const TasksDev& tk, int t_begin, int ntasks, const double4* zcoef, double* scr,
                 bool gga, cudaStream_t s);
void launch_vxc_fp64(const TasksDev& tk, const int4* items, int nitems, const double* scr,
                     double* A, int nbf, bool gga, cudaStream_t s);

// VXC(i,j) = A(i,j) + A(j,i), written with leading dimension ld.
void launch_symmetrize(const double* A, int nbf, double* vxc, int64_t ld, cudaStream_t s);
// dst = src for n x n column-major matrices; either may be device-addressable host memory.
void launch_copy_matrix(const double* src, int64_t lds, double* dst, int64_t ldd, int n,
                        cudaStream_t s);
// out[0] = sum of partials[i].x, out[1] = sum of partials[i].y (compensated,
// fixed order, single CTA)
void launch_reduce_partials(const double2* partials, int64_t n, double* out, cudaStream_t s);

}  // namespace gb300
