// Tensor-core GEMMs of the mixed-precision path (tcgen05.mma, BF16 digits,
// FP32 level accumulators in TMEM) with two fused epilogues:
//
//  X tile (density): D[nu, p] = sum_mu Pd[nu, mu] Fd[p, mu], K chunks of
//    <= 768 (kMaxK) run back to back on one CTA and are summed in float-float
//    registers; X'[nu, p] = 2 * 2^-14 * D * r_nu * s_p is then contracted
//    with phi[nu, p] (rho) and 2 grad phi[nu, p] (grad rho); the sums over
//    the tile's 128 basis rows (TMEM lanes) run as warp reduce-scatters in
//    float-float arithmetic and each warp adds its per-point partials to
//    rho4.
//  V tile (VXC): D[mu, nu] = sum_k Va[mu, k] Vb[nu, k] over K = 2 np, i.e.
//    (phi^T Z + Z^T phi)[mu, nu] / cz; only tiles reaching the upper triangle
//    run, and A[mu, nu] += 2^-14 cz D for mu < nu (half of it for mu = nu),
//    scattered with coalesced FP64 atomics.
//
// Persistent, warp-specialised CTAs (one per SM) in clusters of kCluster.  A
// cluster walks a list of slots; a slot holds one tile (128 x 64 outputs) per
// CTA of the cluster, or none.  Tiles of a slot with the same A operand
// (point block, row block, K range) form a sharing group: each of its CTAs
// loads 1/n of every A block and multicasts it to all n, so the group reads A
// from memory once.  All CTAs of a cluster step through the same sequence of
// stage uses (as many per slot as the slot's longest tile has K blocks) and
// each MMA commit is multicast to the `empty` barrier of every CTA in the
// cluster, so a producer refills a stage only when every CTA it writes to has
// released it.
//   warp 0    producer: per K block its share of A (multicast) and its own B
//             tile as bulk copies (the operands are stored in HBM as
//             shared-memory images, xc_mixed.cuh) into a kStages ring,
//             completion counted on the stage's `full` mbarrier;
//   warp 1    one lane issues the MMAs of a K block and commits them to the
//             stage's `empty` mbarriers; after a tile's last block it commits
//             to `tfull`.  Each level i + j (0..5) of the slice-pair
//             products has its own exact FP32 accumulator of 64 TMEM columns,
//             placed so that digit plane i of A times adjacent B planes
//             j0 .. j1 is a single MMA of N = 64 (j1 - j0 + 1) <= 256 writing
//             levels i + j0 .. i + j1: 8 MMAs per K block instead of 21, so A
//             is read from shared memory 8 times instead of 21;
//   warps 2-9 epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, columns
//             32 ((w - 2) / 4) .. +31 of each level.  The six levels of a
//             column are summed into a float-float value right away, TMEM is
//             handed back (`tempty`) and the rest of the epilogue runs from
//             registers while the next tile's MMAs proceed;
//   warps 10-11 (density only) process the chunks that warps 5 and 9, which
//             share the MMA warp's SM sub-partition, drain and hand over.
// Every mbarrier wait is bounded.  On expiry the CTA records an error code,
// each role leaves its loop, the producer waits (bounded) until the cluster
// has released the stages it filled, the MMA lane for its MMAs, TMEM is
// released and the CTAs of the cluster leave together.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <queue>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ffmath.cuh"
#include "umma.cuh"
#include "xc_mixed.cuh"

namespace gb300 {

namespace {

constexpr int kStages = 5;
constexpr int kEpiWarps = 8;  // two per TMEM lane quarter, 32 columns each
constexpr int kHelpWarps = 2;  // process the chunks drained by the quarter-1 warps
constexpr int kThreads = 64 + 32 * (kEpiWarps + kHelpWarps);
constexpr int kAccs = kLevels - 1;  // exact level accumulators (i + j = 0..5)
constexpr int kAPlane = kMTile * kBK * 2;  // bytes of one digit plane of an A tile (4 KB)
constexpr int kBPlane = kNTile * kBK * 2;  // bytes of one digit plane of a B tile (2 KB)
constexpr int kABytes = kSlices * kAPlane;
constexpr int kBBytes = kSlices * kBPlane;
constexpr int kStageBytes = kABytes + kBBytes;
constexpr uint32_t kTmemCols = 512;  // six levels x 64 columns (384) rounded up
constexpr int kChunkBytes = 32 * 16 * 8;  // one unit's data: 32 rows x 16 columns, 8 bytes each
constexpr int kWorkWarps = kEpiWarps - 2;  // draining warps that also process (not quarter 1)
constexpr int kRedOffset = kStages * kStageBytes;  // per working warp: a parked chunk
constexpr int kHandOffset = kRedOffset + kWorkWarps * kChunkBytes;
constexpr int kBarOffset = kHandOffset + 4 * kChunkBytes;  // the four quarter-1 chunks
constexpr uint16_t kClusterMask = (1u << kCluster) - 1;
static_assert(kBK == 16, "one MMA (K = 16) per operand tile");
static_assert(kABytes % (16 * 12) == 0, "A shares of 1/2, 1/3, 1/4 are 16-byte multiples");
static_assert(kNTile == 64 && kAccs * kNTile <= (int)kTmemCols, "six levels of 64 columns");
static_assert(kSlices == 6 && kLevels == 7, "MMA grouping below assumes 6 digits, levels <= 7");

enum { EPI_X = 0, EPI_V = 1 };
// error codes: which wait expired
enum { ERR_EMPTY = 1, ERR_TEMPTY = 2, ERR_FULL = 3, ERR_TFULL = 4, ERR_HAND = 5 };

struct Bars {
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t tfull;
  uint64_t tempty;
  uint64_t hfull;   // quarter-1 chunks handed over (2 arrivals)
  uint64_t hempty;  // and processed (kHelpWarps arrivals)
  uint64_t done;
  uint32_t tmem_slot;
  int fail;
};

__device__ __forceinline__ int exp_of_pow2(double p) {
  return (int)(((unsigned long long)__double_as_longlong(p) >> 52) & 0x7FF) - 1023;
}

__device__ __forceinline__ void set_fail(Bars* B, int code) { atomicCAS(&B->fail, 0, code); }

// Failure flag as seen by lane 0, the same in every lane of the warp.
__device__ __forceinline__ bool warp_failed(const Bars* B) {
  const int f = *reinterpret_cast<const volatile int*>(&B->fail);
  return __shfl_sync(0xffffffffu, f, 0) != 0;
}

// Bounded wait (limit_ns) whose outcome is the same in every lane of the warp.
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  const bool ok = umma::mbar_wait(bar, parity, limit_ns);
  return __all_sync(0xffffffffu, ok);
}

// The MMAs of one K block.  Digit plane i of A times B planes j0..j1 (adjacent
// in shared memory, so one operand of 64 (j1 - j0 + 1) rows) accumulates into
// levels i + j0 .. i + j1 (TMEM columns 64 (i + j0) ..), all pairs with
// i + j <= 5.  On a tile's first block the two plane-0 MMAs, which cover all
// six levels, overwrite instead of accumulating.  da / db: descriptors of
// the stage's A and B tiles; a plane further on is a constant added to the
// descriptor's address field (bytes / 16, no carry out of the field).
__device__ __forceinline__ void issue_block(uint32_t d0, uint64_t da, uint64_t db, bool acc_prev) {
  auto mma = [&](int i, int j0, int nplanes, bool first) {
    umma::mma_bf16(d0 + (i + j0) * kNTile, da + (uint64_t)((i * kAPlane) >> 4),
                   db + (uint64_t)((j0 * kBPlane) >> 4), umma::idesc_bf16_f32(kMTile, kNTile * nplanes),
                   (acc_prev || !first) ? 1u : 0u);
  };
  mma(0, 0, 4, true);   // levels 0-3
  mma(0, 4, 2, true);   // levels 4-5
  mma(1, 0, 4, false);  // levels 1-4
  mma(1, 4, 1, false);  // level 5
  mma(2, 0, 4, false);  // levels 2-5
  mma(3, 0, 3, false);  // levels 3-5
  mma(4, 0, 2, false);  // levels 4-5
  mma(5, 0, 1, false);  // level 5
}

// Sum over the 32 lanes of 16 float-float values per lane (reduce-scatter):
// on return lanes 2k and 2k+1 both hold, in h[0] + l[0], the total of value
// index 8 b4 + 4 b3 + 2 b2 + b1 (bk = bit k of the lane index).
__device__ __forceinline__ void reduce16(float (&h)[16], float (&l)[16], int lane) {
#pragma unroll
  for (int step = 0; step < 4; ++step) {
    const int o = 16 >> step;
    const int half = 8 >> step;
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float sh = up ? h[i] : h[i + half], sl = up ? l[i] : l[i + half];
      const float kh = up ? h[i + half] : h[i], kl = up ? l[i + half] : l[i];
      const float rh = __shfl_xor_sync(0xffffffffu, sh, o);
      const float rl = __shfl_xor_sync(0xffffffffu, sl, o);
      const float2 t = ff::add(make_float2(kh, kl), make_float2(rh, rl));
      h[i] = t.x;
      l[i] = t.y;
    }
  }
  const float rh = __shfl_xor_sync(0xffffffffu, h[0], 1);
  const float rl = __shfl_xor_sync(0xffffffffu, l[0], 1);
  const float2 t = ff::add(make_float2(h[0], l[0]), make_float2(rh, rl));
  h[0] = t.x;
  l[0] = t.y;
}

// This thread's lane of TMEM columns [col, col + 16) of the six levels as
// float-float values hi + lo; ACC: added to hi + lo (the earlier K chunks of
// the tile).  Levels 0-2 (and the running sum) enter through exact two-sums;
// levels 3-5 (below 2^-21 of the products' magnitude) are summed in FP32 and
// added to lo with the two-sums' error terms, whose rounding (2^-24 of level
// 3) stays under the error of the 42-bit digits; a final fast two-sum
// normalises hi + lo.
template <bool ACC>
__device__ __forceinline__ void drain_levels(uint32_t tb, uint32_t col, float (&hi)[16],
                                             float (&lo)[16]) {
  float v[3][16];
  umma::tmem_ld16x3(tb + 3 * kNTile + col, tb + 4 * kNTile + col, tb + 5 * kNTile + col, v);
  float t[16];
#pragma unroll
  for (int n = 0; n < 16; ++n) t[n] = v[0][n] + (v[1][n] + v[2][n]);
  umma::tmem_ld16x3(tb + col, tb + kNTile + col, tb + 2 * kNTile + col, v);
#pragma unroll
  for (int n = 0; n < 16; ++n) {
    float s, e, u, d;
    if (ACC) {
      ff::two_sum(hi[n], v[0][n], s, e);
      e += lo[n];
    } else {
      s = v[0][n];
      e = 0.f;
    }
    ff::two_sum(s, v[1][n], u, d);
    e += d;
    ff::two_sum(u, v[2][n], s, d);
    const ff::ffl r = ff::fast_two_sum(s, e + (d + t[n]));  // |lo| <= ulp(hi) / 2
    hi[n] = r.hi;
    lo[n] = r.lo;
  }
}

// A slot as seen by one CTA of the cluster: its tile (pb < 0: none), the
// number of stage uses of the slot (K blocks of its longest tile), and the
// CTAs sharing this CTA's A operand (mask; this CTA loads share `part` of
// `nparts`).
struct SlotView {
  OzItem it;
  int nkb, uses, part, nparts;
  uint16_t mask;
};

struct SlotItems {
  OzItem q[kCluster];
};

__device__ __forceinline__ void load_slot(const OzItem* items, int slot, SlotItems& s) {
#pragma unroll
  for (int r = 0; r < kCluster; ++r) s.q[r] = items[(int64_t)slot * kCluster + r];
}

__device__ __forceinline__ bool same_a(const OzItem& a, const OzItem& b) {
  return a.pb == b.pb && a.m0 == b.m0 && a.k0 == b.k0 && a.k1 == b.k1;
}

__device__ __forceinline__ SlotView view_of(const SlotItems& s, int rank) {
  SlotView v;
#pragma unroll
  for (int r = 0; r < kCluster; ++r)
    if (r == rank) v.it = s.q[r];
  v.nkb = v.it.pb >= 0 ? (v.it.k1 - v.it.k0) / kBK : 0;
  v.uses = 0;
  v.mask = 0;
#pragma unroll
  for (int r = 0; r < kCluster; ++r) {
    if (s.q[r].pb < 0) continue;
    v.uses = max(v.uses, (s.q[r].k1 - s.q[r].k0) / kBK);
    if (v.it.pb >= 0 && same_a(s.q[r], v.it))
      v.mask |= (uint16_t)(1u << r);
  }
  v.part = __popc(v.mask & ((1u << rank) - 1));
  v.nparts = __popc(v.mask);
  return v;
}

template <int EPI>
__global__ void __launch_bounds__(kThreads, 1)
    ozaki_kernel(TasksDev tk, MixedPBDev mp, OzSchedule sched, const double* __restrict__ f64,
                 const __nv_bfloat16* __restrict__ dig, int gga, double* __restrict__ out, int nbf,
                 int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  Bars* B = reinterpret_cast<Bars*>(smem + kBarOffset);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rank = (int)umma::cluster_ctarank();
  const int cl = blockIdx.x / kCluster;
  int beg = sched.slot_off[cl];
  const int end = sched.slot_off[cl + 1];
  const uint64_t wl = sched.wait_ns;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      umma::mbar_init(&B->full[s], 1);
      umma::mbar_init(&B->empty[s], kCluster);  // one MMA commit from every CTA
    }
    umma::mbar_init(&B->tfull, 1);
    umma::mbar_init(&B->tempty, kEpiWarps);
    umma::mbar_init(&B->hfull, 2);
    umma::mbar_init(&B->hempty, kHelpWarps);
    umma::mbar_init(&B->done, 1);
    B->fail = 0;
    umma::fence_barrier_init();
  }
  if (warp == 0) umma::tmem_alloc(&B->tmem_slot, kTmemCols);
  umma::fence_before_sync();
  __syncthreads();
  // the barriers of every CTA are initialised before any peer copies or arrives
  umma::cluster_sync();
  umma::fence_after_sync();
  const uint32_t tmem = B->tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    const uint64_t pol = umma::l2_evict_first_policy();
    uint32_t g = 0;
    SlotItems cur, nxt;
    if (beg < end) load_slot(sched.items, beg, cur);
    nxt = cur;
    // withheld copies: no stage is ever filled, the consumers' first waits
    // run out and nothing is in flight when the CTAs leave
    const int pend = sched.withhold ? beg : end;
    for (int sl = beg; sl < pend; ++sl) {
      if (warp_failed(B)) break;
      // the next slot's entries load while this slot's copies are issued
      if (sl + 1 < end) load_slot(sched.items, sl + 1, nxt);
      const SlotView v = view_of(cur, rank);
      const uint8_t* A = reinterpret_cast<const uint8_t*>(dig + v.it.a);
      const uint8_t* Bm = reinterpret_cast<const uint8_t*>(dig + v.it.b);
      const uint32_t a_lo = (uint32_t)(v.part * kABytes / max(v.nparts, 1));
      const uint32_t a_hi = (uint32_t)((v.part + 1) * kABytes / max(v.nparts, 1));
      bool ok = true;
      for (int u = 0; u < v.uses; ++u, ++g) {
        const int st = (int)(g % kStages);
        // every CTA this one writes to has released the stage
        if (g >= (uint32_t)kStages && !warp_wait(&B->empty[st], ((g / kStages) - 1) & 1, wl)) {
          if (lane == 0) set_fail(B, ERR_EMPTY);
          ok = false;
          break;
        }
        if (lane == 0) {
          if (u < v.nkb) {
            // the whole stage lands here: the A shares of the group and own B
            umma::mbar_arrive_expect_tx(&B->full[st], kStageBytes);
            uint8_t* sa = smem + st * kStageBytes;
            const uint8_t* ga = A + (int64_t)u * kABytes;
            if (EPI == EPI_V) {
              // operands leave L2 before the lines of the VXC accumulator
              // that the epilogue's atomics keep updating
              if (v.nparts > 1)
                umma::bulk_g2s_multicast_hint(sa + a_lo, ga + a_lo, a_hi - a_lo, &B->full[st],
                                              v.mask, pol);
              else
                umma::bulk_g2s_hint(sa, ga, kABytes, &B->full[st], pol);
              umma::bulk_g2s_hint(sa + kABytes, Bm + (int64_t)u * kBBytes, kBBytes, &B->full[st], pol);
            } else {
              if (v.nparts > 1)
                umma::bulk_g2s_multicast(sa + a_lo, ga + a_lo, a_hi - a_lo, &B->full[st], v.mask);
              else
                umma::bulk_g2s(sa, ga, kABytes, &B->full[st]);
              umma::bulk_g2s(sa + kABytes, Bm + (int64_t)u * kBBytes, kBBytes, &B->full[st]);
            }
          } else {
            umma::mbar_arrive(&B->full[st]);  // no tile (or a shorter one): empty use
          }
        }
        __syncwarp();
      }
      if (!ok) break;
      cur = nxt;
    }
    // Every stage use filled here has been released by all CTAs of the
    // cluster: the copies this CTA multicast have landed and the MMA commits
    // aimed at this CTA have arrived.
    for (uint32_t x = g > (uint32_t)kStages ? g - kStages : 0; x < g; ++x)
      warp_wait(&B->empty[x % kStages], (x / kStages) & 1, wl);
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issue
    // descriptors of stage 0; stage st is st * kStageBytes / 16 further
    const uint64_t da0 = umma::smem_desc(umma::smem_u32(smem), 128, (kBK / 8) * 128);
    const uint64_t db0 = umma::smem_desc(umma::smem_u32(smem) + kABytes, 128, (kBK / 8) * 128);
    uint32_t g = 0, st = 0, ph = 0;  // stage use, its stage and phase parity
    int li = 0;
    SlotItems cur, nxt;
    if (beg < end) load_slot(sched.items, beg, cur);
    nxt = cur;
    for (int sl = beg; sl < end; ++sl) {
      if (warp_failed(B)) break;
      if (sl + 1 < end) load_slot(sched.items, sl + 1, nxt);
      const SlotView v = view_of(cur, rank);
      // the epilogue has drained the previous tile's accumulators
      if (v.nkb > 0 && li >= 1 && !warp_wait(&B->tempty, (li - 1) & 1, wl)) {
        if (lane == 0) set_fail(B, ERR_TEMPTY);
        break;
      }
      umma::fence_after_sync();
      bool ok = true;
      for (int u = 0; u < v.uses; ++u, ++g) {
        if (!warp_wait(&B->full[st], ph, wl)) {
          if (lane == 0) set_fail(B, ERR_FULL);
          ok = false;
          break;
        }
        umma::fence_after_sync();
        if (lane == 0) {
          if (u < v.nkb) {
            const uint64_t so = (uint64_t)((st * kStageBytes) >> 4);
            issue_block(tmem, da0 + so, db0 + so, u > 0);
          }
          umma::mma_commit_multicast(&B->empty[st], kClusterMask);
        }
        __syncwarp();
        if (++st == kStages) {
          st = 0;
          ph ^= 1;
        }
      }
      if (!ok) break;
      if (v.nkb > 0) {
        if (lane == 0) umma::mma_commit(&B->tfull);
        __syncwarp();
        ++li;
      }
      cur = nxt;
    }
    // every MMA issued above has completed before TMEM is released
    if (lane == 0) umma::mma_commit(&B->done);
    __syncwarp();
    warp_wait(&B->done, 0, wl);
  } else {
    // ------------------------------------------------------------ epilogue
    // Work comes in units (TMEM lane quarter qq, 16-column chunk c).  Warps
    // 2-9 drain: warp w quarter w % 4, chunks c0 and c0 + 1 (columns
    // 32 ((w - 2) / 4) .. +31).  In the density GEMM, whose units are heavy,
    // the two quarter-1 warps, which share their SM sub-partition with the
    // MMA warp, only drain and hand their chunks over in shared memory to
    // warps 10 (chunks 0, 1) and 11 (chunks 2, 3) on other sub-partitions, so
    // that the MMA warp keeps its issue slots.  The VXC units are light:
    // every draining warp processes its own and warps 10-11 stay idle.
    const bool relays = EPI == EPI_X;
    const bool helper = warp >= 2 + kEpiWarps;
    const int q4 = warp & 3;  // TMEM lane quarter this warp may access (draining warps)
    const int c0 = helper ? (warp - 2 - kEpiWarps) * 2 : ((warp - 2) >> 2) * 2;
    const bool relay = relays && !helper && q4 == 1;
    const uint32_t lane_base = tmem + ((uint32_t)(q4 * 32) << 16);
    // one chunk of 32 x 16 values: (hi, lo) floats or doubles, in a layout
    // of 16 words per row whose column is XOR-swizzled by the row
    float2* hand = reinterpret_cast<float2*>(smem + kHandOffset);
    float2* mine = helper || relay ? nullptr
                   : q4 == 1       ? hand + ((warp - 2) >> 2) * (kChunkBytes / 8)
                                   : reinterpret_cast<float2*>(smem + kRedOffset) +
                                         ((warp - 2) - (warp >= 6 ? 1 : 0)) * (kChunkBytes / 8);
    if (helper && !relays) beg = end;  // nothing to do
    const int nq = gga ? 4 : 1;
    int li = 0, hn = 0;
    // D of the tile in hand (float-float), summed over its K chunks when the
    // next entry continues the same tile (density); zero after each use
    float hi[2][16], lo[2][16];
    bool acc = false;  // hi + lo hold the earlier K chunks of the tile
#pragma unroll
    for (int n = 0; n < 16; ++n) hi[0][n] = lo[0][n] = hi[1][n] = lo[1][n] = 0.f;
    OzItem nit = beg < end ? sched.items[(int64_t)beg * kCluster + rank] : OzItem{};
    for (int sl = beg; sl < end; ++sl) {
      if (warp_failed(B)) break;
      const OzItem it = nit;
      // the next tile's entry loads while this one is processed
      if (sl + 1 < end) nit = sched.items[(int64_t)(sl + 1) * kCluster + rank];
      if (it.pb < 0) continue;
      const int lc = li++;
      const bool last = EPI == EPI_V || sl + 1 == end || nit.pb != it.pb || nit.m0 != it.m0 ||
                        nit.n0 != it.n0 || nit.k0 != it.k1;
      // Tile prologue, before the accumulators are ready: block metadata.
      const int b = it.pb;
      const PBDims d(tk.npts_pad[b], tk.nbe[b]);
      const PBF64 o(d, nq);
      const double* base = f64 + mp.f64_off[b];
      int64_t gpt = 0;
      const int* bfl = nullptr;
      int ecz = 0;
      if (EPI == EPI_X) {
        gpt = tk.pt_off[b] + it.n0;
      } else {
        bfl = tk.bf_list + tk.bf_off[b];
        ecz = exp_of_pow2(base[o.cz]);
      }
      if (!helper) {
        if (!warp_wait(&B->tfull, lc & 1, wl)) {
          if (lane == 0) set_fail(B, ERR_TFULL);
          break;
        }
        umma::fence_after_sync();
        // levels -> float-float in registers, then TMEM goes back to the MMAs
        if (acc) {
          drain_levels<true>(lane_base, c0 * 16, hi[0], lo[0]);
          drain_levels<true>(lane_base, c0 * 16 + 16, hi[1], lo[1]);
        } else {
          drain_levels<false>(lane_base, c0 * 16, hi[0], lo[0]);
          drain_levels<false>(lane_base, c0 * 16 + 16, hi[1], lo[1]);
        }
        umma::fence_before_sync();
        __syncwarp();
        if (lane == 0) umma::mbar_arrive(&B->tempty);
      }
      acc = EPI == EPI_X && !last;
      if (!last) continue;
      const int hc = hn++;
      auto put = [&](float2* buf, const float (&h0)[16], const float (&l0)[16]) {
#pragma unroll
        for (int n = 0; n < 16; ++n) buf[lane * 16 + (n ^ (lane & 15))] = make_float2(h0[n], l0[n]);
      };
      auto get = [&](const float2* buf, float (&h0)[16], float (&l0)[16]) {
#pragma unroll
        for (int n = 0; n < 16; ++n) {
          const float2 v = buf[lane * 16 + (n ^ (lane & 15))];
          h0[n] = v.x;
          l0[n] = v.y;
        }
      };
      auto clear = [&](float (&h0)[16], float (&l0)[16]) {
#pragma unroll
        for (int n = 0; n < 16; ++n) h0[n] = l0[n] = 0.f;
      };
      if (relay) {
        // hand both chunks over once the helpers are done with the previous ones
        if (hc >= 1 && !warp_wait(&B->hempty, (hc - 1) & 1, wl)) {
          if (lane == 0) set_fail(B, ERR_HAND);
          break;
        }
        put(hand + (c0 + 0) * (kChunkBytes / 8), hi[0], lo[0]);
        put(hand + (c0 + 1) * (kChunkBytes / 8), hi[1], lo[1]);
        __syncwarp();
        if (lane == 0) umma::mbar_arrive(&B->hfull);
        clear(hi[0], lo[0]);
        clear(hi[1], lo[1]);
        continue;
      }
      if (helper && !warp_wait(&B->hfull, hc & 1, wl)) {
        if (lane == 0) set_fail(B, ERR_HAND);
        break;
      }
      // density: the second chunk waits in shared memory while the first is
      // processed (registers); VXC keeps it in registers
      if (!helper && EPI == EPI_X) put(mine, hi[1], lo[1]);
      for (int k = 0; k < 2; ++k) {
        const int c = c0 + k;
        const int qq = helper ? 1 : q4;
        if (helper) {
          get(hand + c * (kChunkBytes / 8), hi[0], lo[0]);
        } else if (k == 1) {
          if (EPI == EPI_X) {
            get(mine, hi[0], lo[0]);
          } else {
#pragma unroll
            for (int n = 0; n < 16; ++n) {
              hi[0][n] = hi[1][n];
              lo[0][n] = lo[1][n];
            }
          }
        }
        __syncwarp();
        // one unit: rows of quarter qq, columns jc .. jc + 15, values hi[0] + lo[0]
        const int i = it.m0 + qq * 32 + lane;  // tile row (basis function nu / mu)
        const int jc = it.n0 + c * 16;
        if (EPI == EPI_X) {
          // X'[nu, p] = 2^(er + esp - 13) D, a power of two times D
          const int e_row = exp_of_pow2(base[o.r + i]);
          const int e_col = exp_of_pow2(base[o.sp + jc + (lane & 15)]);
          // phi[q][nu = i][jc .. jc + 15]: 128 contiguous bytes per lane
          const float4* ph = reinterpret_cast<const float4*>(base + (int64_t)i * d.np + jc);
          const int64_t qs = o.blk / 2;  // one value plane, in float4
          float2 pf[16];  // phi[nu = i][p] of the pass in hand, float-float
#pragma unroll
          for (int n = 0; n < 8; ++n) {
            const float4 t = ph[n];
            pf[2 * n] = make_float2(t.x, t.y);
            pf[2 * n + 1] = make_float2(t.z, t.w);
          }
#pragma unroll
          for (int n = 0; n < 16; ++n) {
            const float sc = ff::pow2f(e_row + __shfl_sync(0xffffffffu, e_col, n) - 13);
            hi[0][n] *= sc;
            lo[0][n] *= sc;
          }
          // passes q: phi, then 2 grad phi
          for (int q = 0; q < nq; ++q) {
            float h[16], l[16];
#pragma unroll
            for (int n = 0; n < 16; ++n) {
              float2 fv = pf[n];
              if (q) fv = make_float2(2.f * fv.x, 2.f * fv.y);
              const float2 t = ff::mul(make_float2(hi[0][n], lo[0][n]), fv);
              h[n] = t.x;
              l[n] = t.y;
            }
            // the next pass's phi values load while this pass is reduced
            if (q + 1 < nq) {
#pragma unroll
              for (int n = 0; n < 8; ++n) {
                const float4 t = ph[(q + 1) * qs + n];
                pf[2 * n] = make_float2(t.x, t.y);
                pf[2 * n + 1] = make_float2(t.z, t.w);
              }
            }
            reduce16(h, l, lane);
            if ((lane & 1) == 0) {
              const int n = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 +
                            ((lane >> 1) & 1);
              double* dst = &out[4 * (gpt + c * 16 + n) + q];
              atomicAdd(dst, ff::f2d_scaled(h[0], 0));
              atomicAdd(dst, ff::f2d_scaled(l[0], 0));
            }
          }
        } else {
          // S[i][j] = (phi^T Z + Z^T phi)[i][j] = 2^(ecz - 14) D: the strict
          // upper triangle (i < j, union indices) and the diagonal as
          // S[i][i] / 2 go to the accumulator, so that A + A^T is the block's
          // VXC contribution.  Either triangle of A may hold an entry, so
          // S[i][j] goes to A[bf(j)][bf(i)]: for a fixed column j the 32
          // lanes (consecutive rows i) write consecutive addresses, and no
          // transposition is needed.  hi and lo enter A as two exact
          // doubles, each built from the float's fields with a few integer
          // operations (f2d_scaled), with one FP64 atomic each: measured
          // faster than one atomic of the rounded double of hi + lo, whose
          // integer construction costs more than the second atomic (GB300's
          // FP64 pipe is throttled, so no FP64 arithmetic is used here).
          const int gm = bfl[i];
          const int gn_l = bfl[jc + (lane & 15)];
#pragma unroll
          for (int n = 0; n < 16; ++n) {
            const int gn = __shfl_sync(0xffffffffu, gn_l, n);
            if (i <= jc + n && gm >= 0 && gn >= 0) {
              const int e2 = ecz - 14 - (i == jc + n ? 1 : 0);
              double* dst = &out[(int64_t)gn * nbf + gm];
              atomicAdd(dst, ff::f2d_scaled(hi[0][n], e2));
              atomicAdd(dst, ff::f2d_scaled(lo[0][n], e2));
            }
          }
        }
        clear(hi[0], lo[0]);
      }
      clear(hi[1], lo[1]);
      if (helper) {
        __syncwarp();
        if (lane == 0) umma::mbar_arrive(&B->hempty);
      }
    }
  }

  umma::fence_before_sync();
  __syncthreads();
  if (tid == 0 && B->fail) atomicExch(err, B->fail);
  umma::fence_after_sync();
  if (warp == 0) umma::tmem_dealloc(tmem, kTmemCols);
  // no CTA leaves while a peer of the cluster may still address its barriers
  umma::cluster_sync();
}

template <int EPI>
void set_smem_attr() {
  static bool done = false;
  if (!done) {
    GB300_CUDA(cudaFuncSetAttribute(ozaki_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)ozaki_smem_bytes()));
    done = true;
  }
}

template <int EPI>
void launch(const TasksDev& tk, const MixedPBDev& mp, const OzSchedule& sched, const double* f64,
            const __nv_bfloat16* dig, bool gga, double* out, int nbf, int* err, cudaStream_t s) {
  if (sched.nclusters <= 0) return;
  set_smem_attr<EPI>();
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(sched.nclusters * kCluster);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = ozaki_smem_bytes();
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kCluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  GB300_CUDA(cudaLaunchKernelEx(&cfg, ozaki_kernel<EPI>, tk, mp, sched, f64, dig, gga ? 1 : 0, out,
                                nbf, err));
}

}  // namespace

size_t ozaki_smem_bytes() { return (size_t)kBarOffset + sizeof(Bars) + 1024; }

int ozaki_clusters() {
  static int n = 0;
  if (n == 0) {
    set_smem_attr<EPI_X>();
    set_smem_attr<EPI_V>();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kCluster);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = ozaki_smem_bytes();
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kCluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nx = 0, nv = 0;
    GB300_CUDA(cudaOccupancyMaxActiveClusters(&nx, ozaki_kernel<EPI_X>, &cfg));
    GB300_CUDA(cudaOccupancyMaxActiveClusters(&nv, ozaki_kernel<EPI_V>, &cfg));
    n = std::min(nx, nv);
    if (n <= 0) throw std::runtime_error("tensor-core GEMM: no cluster of 4 CTAs fits the device");
  }
  return n;
}

int ozaki_schedule(const std::vector<OzItem>& items, size_t begin, size_t end, int nclusters,
                   std::vector<OzItem>& slots, std::vector<int>& slot_off) {
  // Slots: kCluster entries taken in list order; the last slot is padded
  // with empty entries (pb = -1).
  std::vector<OzItem> v;
  for (size_t i = begin; i < end; ++i) v.push_back(items[i]);
  const size_t nslot = (v.size() + kCluster - 1) / kCluster;
  while (v.size() < nslot * kCluster) v.push_back(OzItem{-1, 0, 0, 0, 0, 0, 0});
  // Units: runs of slots in which every CTA continues the K range of the
  // same tile (the K chunks of a chain) stay together on one cluster.
  auto continues = [](const OzItem& a, const OzItem& b) {
    if (a.pb < 0 || b.pb < 0) return a.pb < 0 && b.pb < 0;
    return a.pb == b.pb && a.m0 == b.m0 && a.n0 == b.n0 && b.k0 == a.k1;
  };
  // A slot costs its longest tile (all CTAs of a cluster step through the
  // same stage uses) plus the epilogue.
  auto cost = [&](size_t s) {
    int kb = 0;
    for (int r = 0; r < kCluster; ++r) {
      const OzItem& q = v[s * kCluster + r];
      if (q.pb >= 0) kb = std::max(kb, (q.k1 - q.k0) / kBK);
    }
    return (long long)kb + 2;
  };
  std::vector<size_t> ustart;
  for (size_t s = 0; s < nslot; ++s) {
    bool cont = s > 0;
    for (int r = 0; r < kCluster && cont; ++r)
      cont = continues(v[(s - 1) * kCluster + r], v[s * kCluster + r]);
    if (!cont) ustart.push_back(s);
  }
  ustart.push_back(nslot);
  const size_t nunit = ustart.size() - 1;
  const int ncl = (int)std::min<size_t>((size_t)std::max(nclusters, 1), nunit);
  if (ncl == 0) {
    slot_off.push_back((int)(slots.size() / kCluster));
    return 0;
  }
  // Units go, in list order (point blocks in atom order), to the least
  // loaded cluster.
  using Load = std::pair<long long, int>;
  std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
  for (int c = 0; c < ncl; ++c) heap.push({0LL, c});
  std::vector<std::vector<size_t>> lists(ncl);
  for (size_t u = 0; u < nunit; ++u) {
    Load l = heap.top();
    heap.pop();
    for (size_t s = ustart[u]; s < ustart[u + 1]; ++s) {
      lists[l.second].push_back(s);
      l.first += cost(s);
    }
    heap.push(l);
  }
  for (int c = 0; c < ncl; ++c) {
    slot_off.push_back((int)(slots.size() / kCluster));
    for (size_t s : lists[c])
      for (int r = 0; r < kCluster; ++r) slots.push_back(v[s * kCluster + r]);
  }
  slot_off.push_back((int)(slots.size() / kCluster));
  return ncl;
}

// Self-test of the symmetric VXC GEMM: S = F Z^T + Z F^T (n x n) over k
// points for seeded random F in (-1, 1) and Z with row magnitudes spanning
// 2^-10..2^10 (one power-of-two scale for all of Z), digits built on the host
// in the tiled operand layout.  The kernel leaves S[i][j] (i < j) and
// S[i][i] / 2 in A; returns the largest error against an FP64 S relative to
// max |S|.
double ozaki_selftest(int n, int k) {
  if (n % kMTile || k % kNTile || 2 * k > kMaxK) throw std::runtime_error("selftest sizes");
  const PBDims d(k, n);
  const int np = k, k2 = 2 * k;
  const PBF64 o(d, 1);
  uint64_t st = 12345;
  auto rnd = [&]() {
    st = st * 6364136223846793005ULL + 1442695040888963407ULL;
    return ((st >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
  };
  std::vector<double> F((size_t)n * np), Z((size_t)n * np);
  for (auto& x : F) x = rnd() * 0.999;
  double zmax = 0.;
  for (int r = 0; r < n; ++r) {
    const double sc = std::ldexp(1.0, (int)(rnd() * 10));
    for (int p = 0; p < np; ++p) {
      Z[(size_t)r * np + p] = rnd() * sc;
      zmax = std::max(zmax, std::fabs(Z[(size_t)r * np + p]));
    }
  }
  int ez;
  std::frexp(zmax, &ez);
  const double cz = std::ldexp(1.0, ez);
  std::vector<__nv_bfloat16> dig(d.dig_elems(), __float2bfloat16_rn(0.f));
  auto digits = [&](double x, int64_t at, int64_t plane) {
    double r = x, up = 128.0, keep = 1.0;
    for (int i = 0; i < kSlices; ++i) {
      const double dd = std::rint(r * up);
      dig[at + i * plane] = __float2bfloat16_rn((float)(dd * keep));
      r -= dd / up;
      up *= 128.0;
      keep /= 128.0;
    }
  };
  for (int r = 0; r < n; ++r)
    for (int p = 0; p < np; ++p) {
      const double f = F[(size_t)r * np + p], z = Z[(size_t)r * np + p] / cz;
      digits(f, d.va() + oz_offset(0, r, p, kMTile, k2), kMTile * kBK);
      digits(z, d.va() + oz_offset(0, r, np + p, kMTile, k2), kMTile * kBK);
      digits(z, d.vb() + oz_offset(0, r, p, kNTile, k2), kNTile * kBK);
      digits(f, d.vb() + oz_offset(0, r, np + p, kNTile, k2), kNTile * kBK);
    }
  std::vector<double> f64(o.total, 0.);
  for (int r = 0; r < d.nu128; ++r) f64[o.cz + r] = cz;
  std::vector<int> bf(d.nu128);
  for (int i = 0; i < d.nu128; ++i) bf[i] = i;
  std::vector<OzItem> items;
  for (int m0 = 0; m0 < d.nu128; m0 += kMTile)
    for (int n0 = 0; n0 < d.nun; n0 += kNTile)
      if (m0 < n0 + kNTile) {
        items.push_back(OzItem{0, m0, n0, 0, k2, 0, 0});
        oz_set_operands(items.back(), d, 0, true);
      }
  std::vector<OzItem> slots;
  std::vector<int> slot_off;
  const int ncl = ozaki_schedule(items, 0, items.size(), ozaki_clusters(), slots, slot_off);
  int zero_i = 0;
  int64_t zero_l = 0;
  __nv_bfloat16* ddig;
  double *df64, *dA;
  int *dbf, *dnp, *dnu, *derr, *doffs;
  int64_t *doff, *dz;
  OzItem* ditems;
  GB300_CUDA(cudaMalloc(&ddig, dig.size() * 2));
  GB300_CUDA(cudaMalloc(&df64, f64.size() * 8));
  GB300_CUDA(cudaMalloc(&dA, (size_t)n * n * 8));
  GB300_CUDA(cudaMalloc(&dbf, d.nu128 * 4));
  GB300_CUDA(cudaMalloc(&dnp, 4));
  GB300_CUDA(cudaMalloc(&dnu, 4));
  GB300_CUDA(cudaMalloc(&derr, 4));
  GB300_CUDA(cudaMalloc(&doffs, slot_off.size() * 4));
  GB300_CUDA(cudaMalloc(&doff, 8));
  GB300_CUDA(cudaMalloc(&dz, 8));
  GB300_CUDA(cudaMalloc(&ditems, slots.size() * sizeof(OzItem)));
  GB300_CUDA(cudaMemcpy(ddig, dig.data(), dig.size() * 2, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(df64, f64.data(), f64.size() * 8, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemset(dA, 0, (size_t)n * n * 8));
  GB300_CUDA(cudaMemcpy(dbf, bf.data(), d.nu128 * 4, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(dnp, &np, 4, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(dnu, &n, 4, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(derr, &zero_i, 4, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(doffs, slot_off.data(), slot_off.size() * 4, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(doff, &zero_l, 8, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(dz, &zero_l, 8, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(ditems, slots.data(), slots.size() * sizeof(OzItem), cudaMemcpyHostToDevice));
  TasksDev tk{};
  tk.npts_pad = dnp;
  tk.nbe_pad = dnu;
  tk.nbe = dnu;
  tk.bf_off = dz;
  tk.bf_list = dbf;
  tk.pt_off = dz;
  MixedPBDev mp{doff, doff};
  launch<EPI_V>(tk, mp, OzSchedule{ditems, doffs, ncl}, df64, ddig, false, dA, n, derr, 0);
  GB300_CUDA(cudaDeviceSynchronize());
  std::vector<double> C((size_t)n * n);
  int herr = 0;
  GB300_CUDA(cudaMemcpy(C.data(), dA, C.size() * 8, cudaMemcpyDeviceToHost));
  GB300_CUDA(cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost));
  cudaFree(ddig); cudaFree(df64); cudaFree(dA); cudaFree(dbf); cudaFree(dnp); cudaFree(dnu);
  cudaFree(derr); cudaFree(doffs); cudaFree(doff); cudaFree(dz); cudaFree(ditems);
  if (herr)
    throw std::runtime_error("selftest: a pipeline wait expired (code " + std::to_string(herr) + ")");
  std::vector<double> S((size_t)n * n);
  double smax = 0.;
  for (int a = 0; a < n; ++a)
    for (int b = a; b < n; ++b) {
      double acc = 0.;
      for (int p = 0; p < np; ++p)
        acc += F[(size_t)a * np + p] * Z[(size_t)b * np + p] + Z[(size_t)a * np + p] * F[(size_t)b * np + p];
      S[(size_t)a * n + b] = acc;
      smax = std::max(smax, std::fabs(acc));
    }
  // the accumulator may hold an entry in either triangle: compare A + A^T
  // with the symmetric product
  double worst = 0.;
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b) {
      const double ref = S[(size_t)std::min(a, b) * n + std::max(a, b)];
      const double got = C[(size_t)a * n + b] + C[(size_t)b * n + a];
      worst = std::max(worst, std::fabs(got - ref) / std::max(smax, 1e-300));
    }
  return worst;
}

void launch_ozaki_x(const TasksDev& tk, const MixedPBDev& mp, const OzSchedule& sched,
                    const double* f64, const __nv_bfloat16* dig, bool gga, double* rho4, int* err,
                    cudaStream_t s) {
  launch<EPI_X>(tk, mp, sched, f64, dig, gga, rho4, 0, err, s);
}

void launch_ozaki_v(const TasksDev& tk, const MixedPBDev& mp, const OzSchedule& sched,
                    const double* f64, const __nv_bfloat16* dig, bool gga, double* A, int nbf,
                    int* err, cudaStream_t s) {
  launch<EPI_V>(tk, mp, sched, f64, dig, gga, A, nbf, err, s);
}

}  // namespace gb300
