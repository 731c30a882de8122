// Mixed-precision path: split-mantissa FP64 emulation of the two contractions
// on BF16 tensor cores (tcgen05.mma, FP32 accumulation in TMEM).
//
// Every FP64 operand x is scaled by a power of two 2^e (per row of P, per grid
// point of phi, per basis column of Z) so that |x| <= 1 and split into
// kSlices signed digits of 7 bits:  x = 2^e sum_i d_i 2^(-7 i), |d_1| <= 128,
// |d_i| <= 64 (i > 1).  Digit i is stored in BF16 as d_i 2^(-7 (i - 1)), which
// is exact.  A product is the sum over slice pairs (i, j) with i + j <= kLevels
// of BF16 GEMMs; pairs of equal i + j share one TMEM accumulator so each of the
// four leading levels is an exact integer sum in FP32 (the K extent of one GEMM
// is at most 512: 512 * 2^15 < 2^24); the remaining pairs (relative weight
// below 2^-28) share a fifth accumulator.  The epilogue adds the levels in FP64.
#pragma once
#include <functional>
#include <vector>

#include <cuda_bf16.h>

#include "device_common.cuh"
#include "functionals.cuh"

namespace gb300 {

constexpr int kSlices = 6;      // digits per operand
constexpr int kLevels = 7;      // keep pairs with i + j <= kLevels
constexpr int kMaxK = 512;      // K extent of one tensor-core GEMM (exactness bound)
constexpr int kMTile = 128;     // rows of a GEMM tile (basis functions)
constexpr int kNTile = 64;      // columns of a GEMM tile
constexpr int kPBMaxPts = 512;  // points per point block

// Point blocks (merged tasks of one atom) reuse TasksDev; these extra arrays
// give the per-point member task and the member x shell activity mask.
struct PBMaskDev {
  const int* member;        // per padded point: member task index within its block
  const int64_t* mask_off;  // per block: offset into mask
  const uint8_t* mask;      // [nmember][nsh] 1 = shell in the member's list
};

// Per point-block workspace offsets (batch relative).
struct MixedPBDev {
  const int64_t* f64_off;   // doubles: phi (+ grad) blocks, then r[nu_pad], sp[np], cz[nu_pad]
  const int64_t* dig_off;   // bf16 elements: Pd, Fd, FdT, Zd
};

// One tensor-core GEMM tile: output rows [m0, m0+128) x cols [n0, n0+64),
// K range [k0, k1) of point block pb.
struct OzItem {
  int pb, m0, n0, k0, k1;
};

void launch_collocation_masked(const ShellsDev& sh, const TasksDev& tk, const PBMaskDev& mk,
                               const int2* items, int nitems, double* scr, bool grad,
                               cudaStream_t s);

// Digits / scales.  All launchers take the batch's point-block range [b0, b1).
void launch_point_scales(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, bool gga,
                         double* f64, cudaStream_t s);
void launch_phi_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, bool gga,
                       const double* f64, __nv_bfloat16* dig, cudaStream_t s);
void launch_p_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, int max_nu_pad,
                     bool gga, const double* P, int nbf, double* f64, __nv_bfloat16* dig,
                     cudaStream_t s);
void launch_z_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, int max_nu_pad,
                     bool gga, const double4* zcoef, double* f64, __nv_bfloat16* dig,
                     cudaStream_t s);
// Functional on points [g0, g1): zcoef and functional_partial_blocks() EXC/N_el partials.
int functional_partial_blocks();
void launch_functional(int64_t g0, int64_t g1, const double* w, const double* rho4,
                       const XCFunctionalDesc& f, double4* zcoef, double2* partials,
                       cudaStream_t s);

// Tensor-core GEMMs.  err: device int set non-zero when a bounded wait expired.
void launch_ozaki_x(const TasksDev& tk, const MixedPBDev& mp, const OzItem* items, int nitems,
                    const double* f64, const __nv_bfloat16* dig, bool gga, double* rho4,
                    int* err, cudaStream_t s);
void launch_ozaki_v(const TasksDev& tk, const MixedPBDev& mp, const OzItem* items, int nitems,
                    const double* f64, const __nv_bfloat16* dig, bool gga, double* A, int nbf,
                    int* err, cudaStream_t s);

size_t ozaki_smem_bytes();
// Tensor-core GEMM self-test (n x n output, K = k); worst relative error.
double ozaki_selftest(int n, int k);

// Host helpers: workspace sizes of one point block.  The FP64 region holds
// phi (+ grad) in FP64, the scales r[nu_pad], sp[np], cz[nu_pad], then the same
// phi (+ grad) as float-float pairs (float2, one double's worth each).
inline int64_t mixed_f64_doubles(int np, int nu_pad, bool gga) {
  return 2LL * (gga ? 4 : 1) * np * nu_pad + 2 * nu_pad + np;
}
inline int64_t mixed_dig_elems(int np, int nu_pad) {
  return (int64_t)kSlices * ((int64_t)nu_pad * nu_pad + 3LL * np * nu_pad);
}

}  // namespace gb300
