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
// per-point loops read consecutive addresses across a warp.  Every point-atom
// distance, in the table or computed on the fly, is the same FP64 expression
// (dist64), so the two kernels below see identical distances.
#include "device_common.cuh"

#include <algorithm>
#include <cfloat>

namespace gb300 {

namespace {
constexpr double kSSFa = 0.64;
constexpr double kSSFTol = 1e-13;

// |p - c| in FP64 with every rounding spelled out (no contraction choices
// left to the compiler): sqrt(fma(dz, dz, fma(dy, dy, dx * dx))).
__device__ __forceinline__ double dist64(double px, double py, double pz,
                                         const double* __restrict__ c) {
  const double dx = __dsub_rn(px, c[0]), dy = __dsub_rn(py, c[1]), dz = __dsub_rn(pz, c[2]);
  return __dsqrt_rn(__fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx))));
}

__global__ void grid_to_center_kernel(int64_t npts, int natoms, const double* __restrict__ x,
                                      const double* __restrict__ y, const double* __restrict__ z,
                                      const double* __restrict__ coords, double* __restrict__ dist,
                                      int ld) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const double px = x[p], py = y[p], pz = z[p];
  for (int a = blockIdx.y; a < natoms; a += gridDim.y)
    dist[(int64_t)a * ld + p] = dist64(px, py, pz, coords + 3 * a);
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
// ---------------------------------------------------------------- screened kernel
// Same weights, far fewer and far cheaper cell-product factors.  A warp
// takes 32 consecutive points (a chunk; the points of one task are close
// together) and
//   * sorts the atoms by their distance d_B to the centre of the chunk's
//     bounding box (bitonic sort of 32-bit (d_B, B) keys in shared memory), h being
//     the chunk's radius, so that every point has r_B in [d_B - h, d_B + h];
//   * drops, for the whole chunk, every atom A that one of the four atoms
//     nearest to the centre kills at every point:
//     ((d_A - h) - (d_B + h)) / R_AB >= a gives s(mu_AB) = 0, so P_A = 0;
//   * evaluates each remaining cell product over the atoms in distance
//     order: the nearest atoms (the likely zero factors) come first, and the
//     loop ends at the first atom with d_B - h >= r_A (1 + a) / (1 - a):
//     from there on R_AB <= r_A + r_B gives mu_AB <= -a, a factor of exactly
//     1 for every later atom;
//   * classifies every factor first in FP32 (distances and R_AB from FP32
//     coordinates relative to an origin o): mu_f <= -a - m means mu <= -a
//     (factor exactly 1, skipped) and mu_f >= a + m means mu >= a (factor
//     exactly 0), where the margin m bounds |mu_f - mu| (the caller derives
//     it from the largest |x - o| of atoms and points and the smallest R_AB:
//     FP32 rounding of coordinates, differences, squares and roots).  Only
//     factors inside the switching band take the FP64 path: distances from
//     dist64, mu = (r_A - r_B) / R_AB and s(mu) exactly as the reference.
// The cell products follow the reference's rules: a zero factor ends the
// product, and so does a product at or below 1e-13 (kept as it is).  Only
// the order of the factors differs from cuda_ssf_1d.cu (nearest first instead
// of atom index order); atoms dropped for the chunk contribute exactly 0.
// Margins of 1e-9 on mu and of 1e-12 relative / 1e-10 bohr on h keep every
// bound valid under FP64 rounding.  No distance table is needed.
constexpr int kSSFWarps = 4;
constexpr double kSSFFar = (1. + kSSFa) / (1. - kSSFa);

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Sort keys of the chunk's atoms: the float bits of d_B rounded down with the
// low 11 mantissa bits replaced by the atom index (natoms <= 2048), so that
// the key orders by distance and the key with the index bits cleared is a
// lower bound of d_B.
constexpr uint32_t kSSFIndexMask = 0x7FFu;
__device__ __forceinline__ float key_dist(uint32_t key) {
  return __uint_as_float(key & ~kSSFIndexMask);
}

// Factors inside the switching band are not evaluated where the FP32 pass
// finds them (a lane at a time, the other lanes of the warp idle on the
// throttled FP64 pipe): each lane queues them, kSSFSlots at most, and the
// warp evaluates every queued factor with all 32 lanes at once, then each
// lane applies its own values in order.
constexpr int kSSFSlots = 16;
constexpr uint16_t kSSFZero = 0xFFFFu;  // queued factor that is exactly 0
struct SSFWarpScratch {
  double px[32], py[32], pz[32], rA[32];  // each lane's point and r_A of its cell
  double s[32][kSSFSlots];                // values of the queued factors
  int A[32], off[32];                     // each lane's cell atom, queue offsets
  uint16_t b[32][kSSFSlots];              // queued atoms B (kSSFZero: factor 0)
};

// Evaluates every queued factor (all lanes), then lane by lane multiplies
// its own in queue order into ps, applying the reference's stops: a product
// at or below 1e-13 ends the cell (`done`), as does a zero factor.
__device__ __forceinline__ void ssf_flush(SSFWarpScratch& ws, int lane, int& cnt, double& ps,
                                          bool& done, const double* __restrict__ coords,
                                          const double* __restrict__ rab_inv, int ld_rab) {
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  ws.off[lane] = incl - cnt;
  __syncwarp();
  for (int e = lane; e < total; e += 32) {
    int lo = 0, hi = 31;  // the last lane whose queue starts at or before e
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (ws.off[mid] <= e) lo = mid; else hi = mid - 1;
    }
    const int L = lo, slot = e - ws.off[L];
    const int B = ws.b[L][slot];
    double v = 0.;
    if (B != kSSFZero) {
      const double mu = (ws.rA[L] - dist64(ws.px[L], ws.py[L], ws.pz[L], coords + 3 * B)) *
                        rab_inv[(int64_t)ws.A[L] * ld_rab + B];
      v = mu >= kSSFa ? 0. : (mu > -kSSFa ? ssf_s(mu) : 1.);
    }
    ws.s[L][slot] = v;
  }
  __syncwarp();
  if (cnt > 0) {
    // the factors are <= 1, so the product only decreases: when the whole
    // queue leaves it above 1e-13 no stop was passed on the way
    double q = ps;
    for (int j = 0; j < cnt; ++j) q *= ws.s[lane][j];
    if (q > kSSFTol) {
      ps = q;
    } else {
      for (int j = 0; j < cnt; ++j) {
        ps *= ws.s[lane][j];
        if (ps <= kSSFTol) break;
      }
      done = true;
    }
  }
  cnt = 0;
  __syncwarp();
}

// Cell products P_A at the warp's points (warp-collective: every lane calls
// it; `act` false leaves a lane out), the atoms in the chunk's distance order,
// rA = dist64 of the lane's point to its A.
__device__ __forceinline__ double cell_warp(bool act, int A, double rA, int natoms, double h,
                                            const uint32_t* __restrict__ keys, float qx, float qy,
                                            float qz, SSFWarpScratch& ws, int lane,
                                            const double* __restrict__ coords,
                                            const float4* __restrict__ cf,
                                            const double* __restrict__ rab_inv, int ld_rab,
                                            float margin) {
  ws.A[lane] = A;
  ws.rA[lane] = rA;
  const float4 gA = cf[A];
  const float rAf = (float)rA;
  // atoms with d_B >= lim have r_B >= kSSFFar r_A (1 + 1e-9): factor 1
  const float limf = __double2float_ru(kSSFFar * rA * (1. + 1e-9) + h);
  const float lo = -(float)kSSFa - margin, hi = (float)kSSFa + margin;
  double ps = 1.;
  bool done = !act;
  int cnt = 0;
  for (int k = 0; k < natoms; ++k) {
    if (!done) {
      const uint32_t key = keys[k];
      if (key_dist(key) >= limf) {
        done = true;
      } else {
        const int B = (int)(key & kSSFIndexMask);
        if (B != A) {
          const float4 gB = cf[B];
          const float dx = qx - gB.x, dy = qy - gB.y, dz = qz - gB.z;
          const float rBf = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
          const float ex = gA.x - gB.x, ey = gA.y - gB.y, ez = gA.z - gB.z;
          const float muf = (rAf - rBf) * rsqrtf(fmaf(ez, ez, fmaf(ey, ey, ex * ex)));
          if (muf >= hi) {  // mu >= a: factor exactly 0
            ws.b[lane][cnt++] = kSSFZero;
            done = true;
          } else if (!(muf <= lo)) {  // inside the band (mu <= -a: factor 1, skipped)
            ws.b[lane][cnt++] = (uint16_t)B;
          }
        }
      }
    }
    const bool all_done = __all_sync(0xffffffffu, done);
    if (all_done || __any_sync(0xffffffffu, cnt == kSSFSlots)) {
      ssf_flush(ws, lane, cnt, ps, done, coords, rab_inv, ld_rab);
      if (all_done || __all_sync(0xffffffffu, done)) return ps;
    }
  }
  ssf_flush(ws, lane, cnt, ps, done, coords, rab_inv, ld_rab);
  return ps;
}

__global__ void __launch_bounds__(kSSFWarps * 32)
    ssf_screened_kernel(int64_t npts, int natoms, int nsort, const double* __restrict__ x,
                        const double* __restrict__ y, const double* __restrict__ z,
                        const int32_t* __restrict__ iparent,
                        const double* __restrict__ dist_nearest,
                        const double* __restrict__ coords, const float4* __restrict__ cf,
                        double ox, double oy, double oz, float margin,
                        const double* __restrict__ rab_inv, int ld_rab,
                        double* __restrict__ weights, int* __restrict__ status) {
  extern __shared__ uint32_t ssf_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // per warp: nsort sort keys, then up to nsort candidate atoms (uint16)
  uint32_t* keys = ssf_smem + (size_t)warp * (nsort + nsort / 2);
  uint16_t* cand = reinterpret_cast<uint16_t*>(keys + nsort);
  const int64_t p0 = ((int64_t)blockIdx.x * kSSFWarps + warp) * 32;
  if (p0 >= npts) return;  // the whole warp
  const int64_t p = p0 + lane;
  const bool act = p < npts;
  const int64_t pq = act ? p : p0;
  const double px = x[pq], py = y[pq], pz = z[pq];
  const double cx = 0.5 * (warp_min(px) + warp_max(px));
  const double cy = 0.5 * (warp_min(py) + warp_max(py));
  const double cz = 0.5 * (warp_min(pz) + warp_max(pz));
  double h = sqrt((px - cx) * (px - cx) + (py - cy) * (py - cy) + (pz - cz) * (pz - cz));
  h = warp_max(h) * (1. + 1e-12) + 1e-10;

  // ---- atoms in distance order (keys: d_B as float rounded down, atom index)
  for (int b = lane; b < nsort; b += 32) {
    uint32_t k = ~0u;
    if (b < natoms) {
      const double dx = cx - coords[3 * b], dy = cy - coords[3 * b + 1], dz = cz - coords[3 * b + 2];
      const float df = __double2float_rd(sqrt(dx * dx + dy * dy + dz * dz));
      k = (__float_as_uint(df) & ~kSSFIndexMask) | (uint32_t)b;
    }
    keys[b] = k;
  }
  __syncwarp();
  for (int kk = 2; kk <= nsort; kk <<= 1)
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < nsort; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const uint32_t u = keys[i], v = keys[ixj];
          if ((u > v) == ((i & kk) == 0)) {
            keys[i] = v;
            keys[ixj] = u;
          }
        }
      }
      __syncwarp();
    }

  // ---- atoms not killed at every point of the chunk by one of the four nearest
  int kb[4];
  double kd[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    kb[q] = q < natoms ? (int)(keys[q] & kSSFIndexMask) : -1;
    if (kb[q] >= 0) {
      const double dx = cx - coords[3 * kb[q]], dy = cy - coords[3 * kb[q] + 1],
                   dz = cz - coords[3 * kb[q] + 2];
      kd[q] = sqrt(dx * dx + dy * dy + dz * dz) + h;  // upper bound of r_B
    }
  }
  int ncand = 0;
  for (int a0 = 0; a0 < natoms; a0 += 32) {
    const int A = a0 + lane;
    bool keep = A < natoms;
    if (keep) {
      const double dx = cx - coords[3 * A], dy = cy - coords[3 * A + 1], dz = cz - coords[3 * A + 2];
      const double dlo = sqrt(dx * dx + dy * dy + dz * dz) - h;  // lower bound of r_A
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (kb[q] >= 0 && kb[q] != A &&
            (dlo - kd[q]) * rab_inv[(int64_t)A * ld_rab + kb[q]] >= kSSFa + 1e-9)
          keep = false;
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) cand[ncand + __popc(m & ((1u << lane) - 1))] = (uint16_t)A;
    ncand += __popc(m);
  }
  __syncwarp();

  // ---- the lanes' points (reference rules, cuda_ssf_1d.cu:61-128); every
  // lane stays in the warp-collective cell evaluations, `live` marks the
  // points still being weighted
  SSFWarpScratch& ws = reinterpret_cast<SSFWarpScratch*>(
      ssf_smem + (size_t)kSSFWarps * (nsort + nsort / 2))[warp];
  int ip = act ? iparent[p] : 0;
  bool live = act;
  if (act && (ip < 0 || ip >= natoms)) {
    if (status) atomicExch(status, 1);
    live = false;
    ip = 0;
  }
  ws.px[lane] = px;
  ws.py[lane] = py;
  ws.pz[lane] = pz;
  const float qx = (float)(px - ox), qy = (float)(py - oy), qz = (float)(pz - oz);
  const double rip = dist64(px, py, pz, coords + 3 * ip);
  if (live && rip < 0.5 * (1. - kSSFa) * dist_nearest[p]) live = false;
  const double parent = cell_warp(live, ip, rip, natoms, h, keys, qx, qy, qz, ws, lane, coords,
                                  cf, rab_inv, ld_rab, margin);
  if (live && parent < DBL_EPSILON) {
    weights[p] = 0.;
    live = false;
  }
  double sum = parent;
  for (int c = 0; c < ncand; ++c) {
    const int A = cand[c];
    const bool use = live && A != ip;
    if (!__any_sync(0xffffffffu, use)) continue;
    const double v = cell_warp(use, A, dist64(px, py, pz, coords + 3 * A), natoms, h, keys, qx, qy,
                               qz, ws, lane, coords, cf, rab_inv, ld_rab, margin);
    if (use) sum += v;
  }
  if (live) weights[p] *= parent / sum;
}

}  // namespace

void launch_ssf_weights_screened(int64_t npts, int natoms, const double* x, const double* y,
                                 const double* z, const int32_t* iparent,
                                 const double* dist_nearest, const double* coords,
                                 const float4* coords_f, double ox, double oy, double oz,
                                 float margin, const double* rab_inv, int ld_rab, double* weights,
                                 int* status, cudaStream_t s) {
  if (npts == 0) return;
  if (natoms > kSSFScreenedMaxAtoms) throw std::runtime_error("screened SSF: more atoms than its sort keys can index");
  int nsort = 32;
  while (nsort < natoms) nsort <<= 1;
  // per warp: nsort keys and nsort / 2 words of candidates (nsort >= 32, so
  // 8-byte aligned), then the per-warp factor queues (SSFWarpScratch)
  const size_t smem = (size_t)kSSFWarps * ((nsort + nsort / 2) * sizeof(uint32_t) +
                                           sizeof(SSFWarpScratch));
  static bool attr = false;
  if (!attr) {
    GB300_CUDA(cudaFuncSetAttribute(
        ssf_screened_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)((size_t)kSSFWarps * ((kSSFScreenedMaxAtoms + kSSFScreenedMaxAtoms / 2) *
                                       sizeof(uint32_t) + sizeof(SSFWarpScratch)))));
    attr = true;
  }
  const int64_t chunks = (npts + 31) / 32;
  const unsigned blocks = (unsigned)((chunks + kSSFWarps - 1) / kSSFWarps);
  ssf_screened_kernel<<<blocks, kSSFWarps * 32, smem, s>>>(
      npts, natoms, nsort, x, y, z, iparent, dist_nearest, coords, coords_f, ox, oy, oz, margin,
      rab_inv, ld_rab, weights, status);
  GB300_CUDA(cudaGetLastError());
}

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
