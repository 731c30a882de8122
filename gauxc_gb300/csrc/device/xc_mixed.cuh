// Mixed-precision path: split-mantissa FP64 emulation of the two contractions
// on BF16 tensor cores (tcgen05.mma, FP32 accumulation in TMEM).
//
// Every FP64 operand x is scaled by a power of two 2^e (per row of the whole
// density matrix, per grid point of phi, per point block for Z) so that |x| <= 1 and split into
// kSlices signed digits of 7 bits:  x = 2^e sum_i d_i 2^(-7 i), |d_1| <= 128,
// |d_i| <= 64 (i > 1).  Digit i is stored in BF16 as d_i 2^(-7 (i - 1)), which
// is exact.  A product is the sum over slice pairs (i, j) with i + j <= kLevels
// of BF16 GEMMs (21 pairs); pairs of equal i + j share one TMEM accumulator,
// levels 0-2 exact integer sums in FP32 for a K extent of at most 768
// (kMaxK; levels 3-5, 2^-21 of the result and below, may round).  The
// epilogue adds the six levels in float-float arithmetic (the three
// smallest first in FP32).
//
// GEMM operands live in HBM already in the tensor core's shared-memory image:
// tiles of TR rows (128 for the M operand, 64 for the N operand) by kBK
// columns of K, all kSlices digit planes of one tile adjacent, each plane in
// the K-major no-swizzle layout of 8-row x 16-byte core matrices (oz_offset).
// One pipeline stage of the GEMM kernel is then two contiguous bulk copies.
#pragma once
#include <functional>
#include <vector>

#include <cuda_bf16.h>

#include "device_common.cuh"
#include "functionals.cuh"

namespace gb300 {

constexpr int kSlices = 6;      // digits per operand
constexpr int kLevels = 7;      // keep pairs with i + j <= kLevels
// K extent of one tensor-core GEMM (a density chunk; the VXC GEMM's 2 nk).
// Level L sums K (L + 1) digit products, at most 2^13 each with the leading
// digit (|d_0| <= 128) and 2^12 otherwise: levels 0-2 stay below 20480 K,
// exact in FP32 for K <= 819.  Levels 3-5 may round beyond K = 512, by 2^-24
// of values below 2^-21 of the result (2^-45, under the 2^-42 of the digits
// themselves).
constexpr int kMaxK = 768;
constexpr int kMTile = 128;     // rows of a GEMM tile (M operand)
constexpr int kNTile = 64;      // columns of a GEMM tile (N operand rows)
constexpr int kBK = 16;         // K extent of one operand tile (one MMA)
constexpr int kPBMaxPts = 384;  // points per point block (2 x 384 = kMaxK for the VXC GEMM)

__host__ __device__ constexpr int oz_round(int x, int m) { return (x + m - 1) / m * m; }

// Element offset of digit plane s of entry (r, k) of an operand stored as
// tiles of TR rows; kpad = padded K extent (a multiple of kBK).
__host__ __device__ inline int64_t oz_offset(int s, int r, int k, int TR, int kpad) {
  const int64_t chunk = ((int64_t)(r / TR) * (kpad / kBK) + k / kBK) * kSlices + s;
  const int rr = r % TR, kk = k % kBK;
  return chunk * TR * kBK + ((rr >> 3) * (kBK / 8) + (kk >> 3)) * 64 + (rr & 7) * 8 + (kk & 7);
}

// Padded extents of one point block: np points (multiple of kNTile: the
// density GEMM's N tiles and the phi planes), nk <= np points of the VXC
// GEMM's K extent (the block's real points rounded up to kBK; nk = np when
// not given), nu basis functions in the union.
struct PBDims {
  int np, nu, nu16, nun, nu128, nk;
  __host__ __device__ PBDims(int np_, int nu_, int nk_ = 0)
      : np(np_), nu(nu_), nu16(oz_round(nu_, kBK)), nun(oz_round(nu_, kNTile)),
        nu128(oz_round(nu_, kMTile)), nk(nk_ > 0 ? nk_ : np_) {}
  // digit operands (bf16 element offsets within the block's region)
  //   Pd [nu128 rows, TR 128] x [K = mu, nu16]   density GEMM, M operand
  //   Fd [np rows,    TR  64] x [K = mu, nu16]   density GEMM, N operand
  //   Va [nu128 rows, TR 128] x [K = 2 nk]       VXC GEMM, M operand: phi | Z
  //   Vb [nun rows,   TR  64] x [K = 2 nk]       VXC GEMM, N operand: Z | phi
  // so that Va Vb^T = phi^T Z + Z^T phi, the symmetric VXC contribution.
  __host__ __device__ int64_t pd() const { return 0; }
  __host__ __device__ int64_t fd() const { return (int64_t)kSlices * nu128 * nu16; }
  __host__ __device__ int64_t va() const { return fd() + (int64_t)kSlices * np * nu16; }
  __host__ __device__ int64_t vb() const { return va() + (int64_t)kSlices * nu128 * 2 * nk; }
  __host__ __device__ int64_t dig_elems() const { return vb() + (int64_t)kSlices * nun * 2 * nk; }
};

// FP64 region of a point block (offsets in doubles): phi[q][mu][p] (q = value,
// d/dx, d/dy, d/dz; nu128 rows), r[nu128] (row scales of P), sp[np] (point
// scales of phi), gp[np] (largest |grad phi| of a point, as an IEEE magnitude
// key), cz[nu128] (scale of Z, one value per block).  phi entries are
// float-float pairs (one double's worth each); sp and gp are written by the
// collocation kernel.
struct PBF64 {
  int64_t blk, r, sp, gp, cz, total;
  __host__ __device__ PBF64(const PBDims& d, int nq)
      : blk((int64_t)d.np * d.nu128), r(nq * blk), sp(r + d.nu128), gp(sp + d.np),
        cz(gp + d.np), total(cz + d.nu128) {}
};

// Point blocks (merged tasks of one atom) reuse TasksDev (npts_pad = np,
// nbe = nu, nbe_pad = nu128); these extra arrays give the per-point member
// task and the member x shell activity mask.
struct PBMaskDev {
  const int* member;        // per padded point: member task index within its block
  const int64_t* mask_off;  // per block: offset into mask
  const uint8_t* mask;      // [nmember][nsh] 1 = shell in the member's list
};

// Per point-block workspace offsets (batch relative).
struct MixedPBDev {
  const int64_t* f64_off;   // doubles: PBF64 layout
  const int64_t* dig_off;   // bf16 elements: PBDims layout
  const int* zoff;          // first z_digits CTA of each block (nu128 nk / 2048 per block)
  const int* nk;            // VXC K extent of each block (PBDims::nk)
};

// One tensor-core GEMM tile: output rows [m0, m0+128) x cols [n0, n0+64),
// K range [k0, k1) of point block pb; a / b: bf16 element offsets in the
// digit work space of K block k0 of the tile's A row block and B row block
// (oz_set_operands).
struct OzItem {
  int pb, m0, n0, k0, k1;
  int64_t a, b;
};

// Fills it.a / it.b for a density (vxc false) or VXC (vxc true) tile of a
// point block with dimensions d whose digits start at element dig_off.
inline void oz_set_operands(OzItem& it, const PBDims& d, int64_t dig_off, bool vxc) {
  const int64_t nkb = (vxc ? 2 * d.nk : d.nu16) / kBK;
  const int64_t kb0 = it.k0 / kBK;
  it.a = dig_off + (vxc ? d.va() : d.pd()) +
         ((int64_t)(it.m0 / kMTile) * nkb + kb0) * (kSlices * kMTile * kBK);
  it.b = dig_off + (vxc ? d.vb() : d.fd()) +
         ((int64_t)(it.n0 / kNTile) * nkb + kb0) * (kSlices * kNTile * kBK);
}

// Work list of one persistent GEMM launch on clusters of kCluster CTAs:
// cluster c processes slots slot_off[c] .. slot_off[c + 1] - 1 in order; CTA
// r of the cluster takes items[kCluster * slot + r] (pb < 0: none).
// wait_ns bounds every pipeline wait of the launch (a wait that runs longer
// records an error code and the CTAs leave).  withhold != 0 makes every
// producer issue no copy at all, so that the first wait on a stage runs out
// with nothing in flight: the check of the error path (the error status
// reaches the host and the next call runs normally).
constexpr int kCluster = 4;
constexpr uint64_t kOzWaitNs = 1000000000ull;  // 1 s
struct OzSchedule {
  const OzItem* items;
  const int* slot_off;
  int nclusters;
  uint64_t wait_ns = kOzWaitNs;
  int withhold = 0;
};

void launch_collocation_masked(const ShellsDev& sh, const TasksDev& tk, const PBMaskDev& mk,
                               const int2* items, int nitems, double* scr, bool grad,
                               cudaStream_t s);

// Digits / scales.  All launchers take the batch's point-block range [b0, b1).
void launch_phi_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, bool gga,
                       const double* f64, __nv_bfloat16* dig, cudaStream_t s);
// rs[i]: power of two above max_j |P[i][j]| (launch_p_row_scales, once per call)
void launch_p_row_scales(const double* P, int nbf, double* rs, cudaStream_t s);
void launch_p_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, int max_nu_pad,
                     bool gga, const double* P, const double* rs, int nbf, double* f64,
                     __nv_bfloat16* dig, cudaStream_t s);
// Z digits of blocks [b0, b1), whose z_digits CTAs are [zc0, zc1) (MixedPBDev::zoff).
void launch_z_digits(const TasksDev& tk, const MixedPBDev& mp, int b0, int b1, int zc0, int zc1,
                     bool gga, const double4* zcoef, double* f64, __nv_bfloat16* dig,
                     cudaStream_t s);
// Functional on points [g0, g1): zcoef and functional_partial_blocks() EXC/N_el partials.
int functional_partial_blocks();
void launch_functional(int64_t g0, int64_t g1, const double* w, const double* rho4,
                       const XCFunctionalDesc& f, double4* zcoef, double2* partials,
                       cudaStream_t s);

// Tensor-core GEMMs.  err: device int set non-zero when a bounded wait expired.
void launch_ozaki_x(const TasksDev& tk, const MixedPBDev& mp, const OzSchedule& sched,
                    const double* f64, const __nv_bfloat16* dig, bool gga, double* rho4,
                    int* err, cudaStream_t s);
void launch_ozaki_v(const TasksDev& tk, const MixedPBDev& mp, const OzSchedule& sched,
                    const double* f64, const __nv_bfloat16* dig, bool gga, double* A, int nbf,
                    int* err, cudaStream_t s);

// Host: group items[begin, end) into slots of kCluster tiles (list order;
// tiles sharing an A operand should be adjacent) and distribute the slots
// over up to `nclusters` clusters.  Appends the slots to `slots` and ncl + 1
// absolute slot offsets to slot_off; returns ncl, the clusters to launch.
int ozaki_schedule(const std::vector<OzItem>& items, size_t begin, size_t end, int nclusters,
                   std::vector<OzItem>& slots, std::vector<int>& slot_off);
// Clusters of the GEMM kernels that can be resident at once on this device.
int ozaki_clusters();

size_t ozaki_smem_bytes();
// Self-test of the symmetric VXC GEMM (n x n output, k points); worst error
// relative to the largest output element.
double ozaki_selftest(int n, int k);

// Host helpers: workspace sizes of one point block.
inline int64_t mixed_f64_doubles(int np, int nu, bool gga) {
  return PBF64(PBDims(np, nu), gga ? 4 : 1).total;
}
inline int64_t mixed_dig_elems(int np, int nu, int nk) { return PBDims(np, nu, nk).dig_elems(); }

}  // namespace gb300
