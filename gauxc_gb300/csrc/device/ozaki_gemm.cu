// Tensor-core GEMMs of the mixed-precision path (tcgen05.mma, BF16 digits,
// FP32 level accumulators in TMEM) with two fused epilogues:
//
//  X tile (density): D[nu, p] = sum_mu Pd[nu, mu] Fd[p, mu] over one K chunk;
//    X'[nu, p] = 2 * 2^-14 * D * r_nu * s_p is contracted on the spot with
//    phi[nu, p] (rho) and 2 grad phi[nu, p] (grad rho) and reduced over the
//    tile's 128 basis rows; the four per-point partial sums are added to rho4.
//    rho is linear in X, so K chunks never need to be summed in X itself.
//  V tile (VXC): D[mu, nu] = sum_p FdT[mu, p] Zd[nu, p];
//    A[mu, nu] += 2^-14 * D * cz_nu, scattered with coalesced FP64 atomics.
//
// CTA = 128 threads.  All threads stage operand tiles with cp.async into a
// 3-deep ring of K blocks (BK = 32, kSlices digit tiles of A and B per block);
// thread 0 issues the MMAs of a block and commits them to the block's
// mbarrier, which frees the stage for the next load.  The 128 x 64 accumulators
// of the five levels occupy 320 TMEM columns (512 allocated).  Every mbarrier
// wait is bounded; on expiry the CTA records an error and leaves after its
// copies drained and TMEM is released.
#include <cuda_bf16.h>

#include <cmath>
#include <stdexcept>
#include <vector>

#include "ffmath.cuh"
#include "umma.cuh"
#include "xc_mixed.cuh"

namespace gb300 {

namespace {

constexpr int BK = 32;
constexpr int NT = 128;
constexpr int kStages = 3;
constexpr int kATile = kMTile * BK * 2;   // bytes of one A digit tile (8 KB)
constexpr int kBTile = kNTile * BK * 2;   // bytes of one B digit tile (4 KB)
constexpr int kStageBytes = kSlices * (kATile + kBTile);
constexpr int kAccs = 5;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t kIdesc = umma::idesc_bf16_f32(kMTile, kNTile);
constexpr double kDigitScale = 1.0 / 16384.0;  // 2^-14

struct Pair {
  int8_t i, j, acc;
};
// slice pairs (0-based digits) with i + j + 2 <= kLevels, grouped by level
__constant__ Pair c_pairs[32];
__constant__ int c_npairs;

enum { EPI_X = 0, EPI_V = 1 };

template <int EPI>
__global__ void __launch_bounds__(NT, 1)
    ozaki_kernel(TasksDev tk, MixedPBDev mp, const OzItem* __restrict__ items,
                 const double* __restrict__ f64, const __nv_bfloat16* __restrict__ dig, int gga,
                 double* __restrict__ out, int nbf, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kStages);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const OzItem it = items[blockIdx.x];
  const int b = it.pb;
  const int np = tk.npts_pad[b];
  const int nu_pad = tk.nbe_pad[b];
  const int64_t S = kSlices;
  const __nv_bfloat16* base = dig + mp.dig_off[b];
  const __nv_bfloat16 *A, *B;
  int64_t lda, ldb, a_slice, b_slice;
  if (EPI == EPI_X) {
    A = base;
    lda = nu_pad;
    a_slice = (int64_t)nu_pad * nu_pad;
    B = base + S * nu_pad * nu_pad;
    ldb = nu_pad;
    b_slice = (int64_t)np * nu_pad;
  } else {
    A = base + S * nu_pad * nu_pad + S * (int64_t)np * nu_pad;
    lda = np;
    a_slice = (int64_t)nu_pad * np;
    B = A + S * (int64_t)nu_pad * np;
    ldb = np;
    b_slice = (int64_t)nu_pad * np;
  }
  const int nkb = (it.k1 - it.k0) / BK;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) umma::mbar_init(&bars[s], 1);
    umma::fence_barrier_init();
  }
  if (warp == 0) umma::tmem_alloc(tmem_slot, kTmemCols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  auto load_block = [&](int kb) {
    uint8_t* st = smem + (kb % kStages) * kStageBytes;
    const int kg = it.k0 + kb * BK;
    for (int c = tid; c < kSlices * kMTile * (BK / 8); c += NT) {
      const int s = c / (kMTile * (BK / 8)), rem = c % (kMTile * (BK / 8));
      const int row = rem / (BK / 8), kc = rem % (BK / 8);
      umma::cp_async16(st + s * kATile + umma::tile_offset<BK>(row, kc * 8),
                       A + s * a_slice + (int64_t)(it.m0 + row) * lda + kg + kc * 8);
    }
    uint8_t* stb = st + kSlices * kATile;
    for (int c = tid; c < kSlices * kNTile * (BK / 8); c += NT) {
      const int s = c / (kNTile * (BK / 8)), rem = c % (kNTile * (BK / 8));
      const int row = rem / (BK / 8), kc = rem % (BK / 8);
      umma::cp_async16(stb + s * kBTile + umma::tile_offset<BK>(row, kc * 8),
                       B + s * b_slice + (int64_t)(it.n0 + row) * ldb + kg + kc * 8);
    }
  };

  bool failed = false;
  uint32_t acc_init = 0;  // bit a set once accumulator a received its first MMA
  for (int kb = 0; kb < 2; ++kb) {
    if (kb < nkb) load_block(kb);
    umma::cp_async_commit();
  }
  for (int kb = 0; kb < nkb; ++kb) {
    const int nb = kb + 2;
    bool ok = true;
    if (nb < nkb) {
      if (nb >= kStages) ok = umma::mbar_wait(&bars[nb % kStages], ((nb - kStages) / kStages) & 1,
                                              kWaitLimit);
      if (ok) load_block(nb);
    }
    umma::cp_async_commit();
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    umma::cp_async_wait<2>();
    umma::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      umma::fence_after_sync();
      const uint8_t* st = smem + (kb % kStages) * kStageBytes;
      const uint32_t a0 = umma::smem_u32(st), b0 = umma::smem_u32(st + kSlices * kATile);
      for (int q = 0; q < c_npairs; ++q) {
        const Pair pr = c_pairs[q];
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
          const uint64_t ad = umma::smem_desc(a0 + pr.i * kATile + kk * 256, 128, (BK / 8) * 128);
          const uint64_t bd = umma::smem_desc(b0 + pr.j * kBTile + kk * 256, 128, (BK / 8) * 128);
          const uint32_t accum = (acc_init >> pr.acc) & 1u;
          umma::mma_bf16(tmem + pr.acc * kNTile, ad, bd, kIdesc, accum);
          acc_init |= 1u << pr.acc;
        }
      }
      umma::mma_commit(&bars[kb % kStages]);
    }
  }
  // all MMAs done once the last block's commit arrived
  if (!failed && nkb > 0) {
    const int last = nkb - 1;
    const bool ok = umma::mbar_wait(&bars[last % kStages], (last / kStages) & 1, kWaitLimit);
    if (__syncthreads_or(!ok)) failed = true;
  }
  umma::cp_async_wait_all();
  __syncthreads();
  umma::fence_after_sync();

  if (!failed && nkb > 0) {
    const int row = warp * 32 + lane;  // TMEM lane == tile row
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    const double* phi = f64 + mp.f64_off[b];
    const int64_t blk = (int64_t)np * nu_pad;
    const int nq = gga ? 4 : 1;
    const double* rvec = phi + nq * blk;
    const double* spv = rvec + nu_pad;
    const double* czv = spv + np;
    const float2* phi2 = reinterpret_cast<const float2*>(czv + nu_pad);
    const int* bfl = tk.bf_list + tk.bf_off[b];
    for (int c = 0; c < kNTile / 16; ++c) {
      // exact float-float sum of the level accumulators
      float hi[16], lo[16];
#pragma unroll
      for (int n = 0; n < 16; ++n) hi[n] = lo[n] = 0.f;
#pragma unroll
      for (int a = 0; a < kAccs; ++a) {
        float v[16];
        umma::tmem_ld16(lane_addr + a * kNTile + c * 16, v);
#pragma unroll
        for (int n = 0; n < 16; ++n) {
          float s, e;
          ff::two_sum(hi[n], v[n], s, e);
          hi[n] = s;
          lo[n] += e;
        }
      }
      if (EPI == EPI_X) {
        // X'[nu, p] = 2 * 2^-14 * r_nu * s_p * D: a power of two times D
        float* redf = reinterpret_cast<float*>(smem);  // [q*16+n][2][kMTile+1]
        const int nu = it.m0 + row;
        const int er = (int)((((unsigned long long)__double_as_longlong(rvec[nu])) >> 52) & 0x7FF) - 1023;
        for (int n = 0; n < 16; ++n) {
          const int p = it.n0 + c * 16 + n;
          const int esp = (int)((((unsigned long long)__double_as_longlong(spv[p])) >> 52) & 0x7FF) - 1023;
          const int e = er + esp - 13;
          const float sc = (e >= -126 && e <= 127) ? __uint_as_float((unsigned)(e + 127) << 23) : 0.f;
          const float2 X = make_float2(hi[n] * sc, lo[n] * sc);
          for (int q = 0; q < nq; ++q) {
            float2 f = phi2[q * blk + (int64_t)nu * np + p];
            if (q) f = make_float2(2.f * f.x, 2.f * f.y);
            const float2 t = ff::mul(X, f);
            redf[((q * 16 + n) * 2 + 0) * (kMTile + 1) + row] = t.x;
            redf[((q * 16 + n) * 2 + 1) * (kMTile + 1) + row] = t.y;
          }
        }
        __syncthreads();
        for (int e = tid; e < nq * 16; e += NT) {
          const float* ph = redf + (e * 2 + 0) * (kMTile + 1);
          const float* pl = redf + (e * 2 + 1) * (kMTile + 1);
          float S = 0.f, E = 0.f;
          for (int m = 0; m < kMTile; ++m) {
            float s2, e2;
            ff::two_sum(S, ph[m], s2, e2);
            S = s2;
            E += e2 + pl[m];
          }
          const int q = e / 16, n = e % 16;
          const int64_t g = tk.pt_off[b] + it.n0 + c * 16 + n;
          atomicAdd(&out[4 * g + q], (double)S + (double)E);
        }
        __syncthreads();
      } else {
        double* red = reinterpret_cast<double*>(smem);
#pragma unroll
        for (int n = 0; n < 16; ++n) {
          const int nu = it.n0 + c * 16 + n;
          red[row * 17 + n] = ((double)hi[n] + (double)lo[n]) * (kDigitScale * czv[nu]);
        }
        __syncthreads();
        for (int e = tid; e < kMTile * 16; e += NT) {
          const int m = e / 16, n = e % 16;
          const int gm = bfl[it.m0 + m], gn = bfl[it.n0 + c * 16 + n];
          if (gm >= 0 && gn >= 0) atomicAdd(&out[(int64_t)gm * nbf + gn], red[m * 17 + n]);
        }
        __syncthreads();
      }
    }
  }
  if (failed && tid == 0) atomicExch(err, 1);
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, kTmemCols);
}

bool g_pairs_ready = false;

void upload_pairs() {
  if (g_pairs_ready) return;
  Pair h[32];
  int n = 0;
  for (int lev = 2; lev <= kLevels; ++lev)
    for (int i = 1; i <= kSlices; ++i) {
      const int j = lev - i;
      if (j < 1 || j > kSlices) continue;
      h[n++] = Pair{(int8_t)(i - 1), (int8_t)(j - 1), (int8_t)(lev - 2 < kAccs - 1 ? lev - 2 : kAccs - 1)};
    }
  GB300_CUDA(cudaMemcpyToSymbol(c_pairs, h, sizeof(Pair) * n));
  GB300_CUDA(cudaMemcpyToSymbol(c_npairs, &n, sizeof(int)));
  g_pairs_ready = true;
}

template <int EPI>
void launch(const TasksDev& tk, const MixedPBDev& mp, const OzItem* items, int nitems,
            const double* f64, const __nv_bfloat16* dig, bool gga, double* out, int nbf, int* err,
            cudaStream_t s) {
  if (!nitems) return;
  upload_pairs();
  const size_t smem = ozaki_smem_bytes();
  static bool attr[2] = {false, false};
  if (!attr[EPI]) {
    GB300_CUDA(cudaFuncSetAttribute(ozaki_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
    attr[EPI] = true;
  }
  ozaki_kernel<EPI><<<nitems, NT, smem, s>>>(tk, mp, items, f64, dig, gga ? 1 : 0, out, nbf, err);
  GB300_CUDA(cudaGetLastError());
}

}  // namespace

size_t ozaki_smem_bytes() { return (size_t)kStages * kStageBytes + 128 + 1024; }

// Self-test of the VXC-tile GEMM: C[mu][nu] = sum_p F[mu][p] Z[nu][p] for
// seeded random F in (-1, 1) and Z with row scales spanning 2^-20..2^20,
// digits built on the host, compared against an FP64 product.  Returns the
// largest |C - C_ref| / max|C_ref row|.
double ozaki_selftest(int n, int k) {
  if (n % kMTile || k % kNTile || k > kMaxK) throw std::runtime_error("selftest sizes");
  const int nu_pad = n, np = k;
  const int64_t S = kSlices, blk = (int64_t)np * nu_pad;
  uint64_t st = 12345;
  auto rnd = [&]() {
    st = st * 6364136223846793005ULL + 1442695040888963407ULL;
    return ((st >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
  };
  std::vector<double> F(blk), Z(blk), cz(nu_pad);
  for (auto& x : F) x = rnd() * 0.999;
  for (int r = 0; r < nu_pad; ++r) {
    const double sc = std::ldexp(1.0, (int)(rnd() * 20));
    double m = 0.;
    for (int p = 0; p < np; ++p) {
      Z[(int64_t)r * np + p] = rnd() * sc;
      m = std::max(m, std::fabs(Z[(int64_t)r * np + p]));
    }
    int e;
    std::frexp(m, &e);
    cz[r] = std::ldexp(1.0, e);
  }
  auto digits = [&](double x, std::vector<__nv_bfloat16>& out, int64_t at, int64_t stride) {
    double r = x, up = 128.0, keep = 1.0;
    for (int i = 0; i < kSlices; ++i) {
      const double d = std::rint(r * up);
      out[at + i * stride] = __float2bfloat16_rn((float)(d * keep));
      r -= d / up;
      up *= 128.0;
      keep /= 128.0;
    }
  };
  const int64_t off_fdt = S * nu_pad * nu_pad + S * blk, off_zd = off_fdt + S * blk;
  std::vector<__nv_bfloat16> dig(off_zd + S * blk, __float2bfloat16_rn(0.f));
  for (int r = 0; r < nu_pad; ++r)
    for (int p = 0; p < np; ++p) {
      digits(F[(int64_t)r * np + p], dig, off_fdt + (int64_t)r * np + p, blk);
      digits(Z[(int64_t)r * np + p] / cz[r], dig, off_zd + (int64_t)r * np + p, blk);
    }
  std::vector<double> f64(blk + 2 * nu_pad + np, 0.);
  for (int r = 0; r < nu_pad; ++r) f64[blk + nu_pad + np + r] = cz[r];
  std::vector<int> bf(nu_pad);
  for (int i = 0; i < nu_pad; ++i) bf[i] = i;
  std::vector<OzItem> items;
  for (int m0 = 0; m0 < nu_pad; m0 += kMTile)
    for (int n0 = 0; n0 < nu_pad; n0 += kNTile) items.push_back(OzItem{0, m0, n0, 0, np});
  int zero_i = 0;
  int64_t zero_l = 0;
  __nv_bfloat16* ddig;
  double *df64, *dA;
  int *dbf, *dnp, *dnu, *derr;
  int64_t *doff, *dz;
  OzItem* ditems;
  GB300_CUDA(cudaMalloc(&ddig, dig.size() * 2));
  GB300_CUDA(cudaMalloc(&df64, f64.size() * 8));
  GB300_CUDA(cudaMalloc(&dA, (size_t)n * n * 8));
  GB300_CUDA(cudaMalloc(&dbf, nu_pad * 4));
  GB300_CUDA(cudaMalloc(&dnp, 4));
  GB300_CUDA(cudaMalloc(&dnu, 4));
  GB300_CUDA(cudaMalloc(&derr, 4));
  GB300_CUDA(cudaMalloc(&doff, 8));
  GB300_CUDA(cudaMalloc(&dz, 8));
  GB300_CUDA(cudaMalloc(&ditems, items.size() * sizeof(OzItem)));
  GB300_CUDA(cudaMemcpy(ddig, dig.data(), dig.size() * 2, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(df64, f64.data(), f64.size() * 8, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemset(dA, 0, (size_t)n * n * 8));
  GB300_CUDA(cudaMemcpy(dbf, bf.data(), nu_pad * 4, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(dnp, &np, 4, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(dnu, &nu_pad, 4, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(derr, &zero_i, 4, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(doff, &zero_l, 8, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(dz, &zero_l, 8, cudaMemcpyHostToDevice));
  GB300_CUDA(cudaMemcpy(ditems, items.data(), items.size() * sizeof(OzItem), cudaMemcpyHostToDevice));
  TasksDev tk{};
  tk.npts_pad = dnp;
  tk.nbe_pad = dnu;
  tk.nbe = dnu;
  tk.bf_off = dz;
  tk.bf_list = dbf;
  tk.pt_off = dz;
  MixedPBDev mp{doff, doff};
  launch<EPI_V>(tk, mp, ditems, (int)items.size(), df64, ddig, false, dA, n, derr, 0);
  GB300_CUDA(cudaDeviceSynchronize());
  std::vector<double> C((size_t)n * n);
  int herr = 0;
  GB300_CUDA(cudaMemcpy(C.data(), dA, C.size() * 8, cudaMemcpyDeviceToHost));
  GB300_CUDA(cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost));
  cudaFree(ddig); cudaFree(df64); cudaFree(dA); cudaFree(dbf); cudaFree(dnp); cudaFree(dnu);
  cudaFree(derr); cudaFree(doff); cudaFree(dz); cudaFree(ditems);
  if (herr) throw std::runtime_error("selftest: pipeline wait expired");
  double worst = 0.;
  for (int mu = 0; mu < n; ++mu) {
    std::vector<double> ref(n);
    double rmax = 0.;
    for (int nu = 0; nu < n; ++nu) {
      double acc = 0.;
      for (int p = 0; p < np; ++p) acc += F[(int64_t)mu * np + p] * Z[(int64_t)nu * np + p];
      ref[nu] = acc;
      rmax = std::max(rmax, std::fabs(acc) / cz[nu]);
    }
    for (int nu = 0; nu < n; ++nu)
      worst = std::max(worst, std::fabs(C[(size_t)mu * n + nu] - ref[nu]) / cz[nu] / std::max(rmax, 1e-300));
  }
  return worst;
}

void launch_ozaki_x(const TasksDev& tk, const MixedPBDev& mp, const OzItem* items, int nitems,
                    const double* f64, const __nv_bfloat16* dig, bool gga, double* rho4, int* err,
                    cudaStream_t s) {
  launch<EPI_X>(tk, mp, items, nitems, f64, dig, gga, rho4, 0, err, s);
}

void launch_ozaki_v(const TasksDev& tk, const MixedPBDev& mp, const OzItem* items, int nitems,
                    const double* f64, const __nv_bfloat16* dig, bool gga, double* A, int nbf,
                    int* err, cudaStream_t s) {
  launch<EPI_V>(tk, mp, items, nitems, f64, dig, gga, A, nbf, err, s);
}

}  // namespace gb300
