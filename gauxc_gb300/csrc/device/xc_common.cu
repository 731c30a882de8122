// Symmetrization of the VXC accumulator and the EXC / N_el reduction.
//
// Reference: symmetrize_matrix_device (kernels/symmetrize_mat.cu:18-48) copies
// the lower triangle to the upper one; here the accumulator holds A with
// VXC = A + A^T, formed with a shared-memory tile transpose.  The reference
// sums EXC / N_el with cublasDdot per batch (kernels/cublas_extensions.cu:
// 86-112, plain FP64); this build reduces per-CTA partials in a fixed order
// with Neumaier compensation, so the result is bit-reproducible.
#include <algorithm>

#include "xc_kernels.cuh"

namespace gb300 {

namespace {

__global__ void symmetrize_kernel(const double* __restrict__ A, int n, double* __restrict__ V,
                                  int64_t ld) {
  // output block: rows [r0, r0+32), columns [c0, c0+32) of V (column-major)
  __shared__ double T[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tx = threadIdx.x;
  // T[y][x] = A(c0 + x, r0 + y): coalesced along x
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int row = c0 + tx, col = r0 + y;
    if (row < n && col < n) T[y][tx] = A[(int64_t)col * n + row];
  }
  __syncthreads();
  // V(r0 + tx, c0 + y) = A(r0 + tx, c0 + y) + A(c0 + y, r0 + tx)
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int row = r0 + tx, col = c0 + y;
    if (row < n && col < n)
      V[(int64_t)col * ld + row] = A[(int64_t)col * n + row] + T[tx][y];
  }
}

// VXC(r, c) = A(ip[r], ip[c]) + A(ip[c], ip[r]): the accumulator A is held in
// a permuted AO order (ip: caller's AO index -> position in A), VXC comes out
// in the caller's order.  Both reads gather within one column of A; the
// writes are coalesced along r.
__global__ void symmetrize_perm_kernel(const double* __restrict__ A, int n,
                                       const int* __restrict__ ip, double* __restrict__ V,
                                       int64_t ld) {
  __shared__ double T[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tx = threadIdx.x;
  const int pr = r0 + tx < n ? ip[r0 + tx] : 0;
  const int pc = c0 + tx < n ? ip[c0 + tx] : 0;
  // T[y][x] = A(ip[c0 + x], ip[r0 + y])
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int prow = __shfl_sync(0xffffffffu, pr, y);
    if (r0 + y < n && c0 + tx < n) T[y][tx] = A[(int64_t)prow * n + pc];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int col = c0 + y;
    const int pcol = __shfl_sync(0xffffffffu, pc, y);
    if (r0 + tx < n && col < n) V[(int64_t)col * ld + r0 + tx] = A[(int64_t)pcol * n + pr] + T[tx][y];
  }
}

// dst(r, c) = scale src(perm[r], perm[c]) for n x n matrices (leading
// dimension n): the symmetric AO permutation (perm: position -> caller's AO
// index).  A CTA row walks columns; its threads gather within one column.
__global__ void permute_matrix_kernel(const double* __restrict__ src, int n,
                                      const int* __restrict__ perm, double scale,
                                      double* __restrict__ dst) {
  for (int c = blockIdx.y; c < n; c += gridDim.y) {
    const double* sc = src + (int64_t)perm[c] * n;
    double* dc = dst + (int64_t)c * n;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
      dc[r] = scale * sc[perm[r]];
  }
}

struct Neu {
  double s = 0., c = 0.;
  __device__ void add(double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  __device__ double value() const { return s + c; }
};

__global__ void reduce_partials_kernel(const double2* __restrict__ p, int64_t n, double* out) {
  __shared__ double se[256], ce[256], sn[256], cn[256];
  Neu e, q;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 v = p[i];
    e.add(v.x);
    q.add(v.y);
  }
  se[threadIdx.x] = e.s; ce[threadIdx.x] = e.c;
  sn[threadIdx.x] = q.s; cn[threadIdx.x] = q.c;
  __syncthreads();
  if (threadIdx.x == 0) {
    Neu E, N;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      E.add(se[i]); E.add(ce[i]);
      N.add(sn[i]); N.add(cn[i]);
    }
    out[0] = E.value();
    out[1] = N.value();
  }
}

}  // namespace

void launch_symmetrize(const double* A, int nbf, double* vxc, int64_t ld, cudaStream_t s) {
  dim3 g((nbf + 31) / 32, (nbf + 31) / 32), b(32, 8);
  symmetrize_kernel<<<g, b, 0, s>>>(A, nbf, vxc, ld);
  GB300_CUDA(cudaGetLastError());
}

void launch_symmetrize_perm(const double* A, int nbf, const int* iperm, double* vxc, int64_t ld,
                            cudaStream_t s) {
  if (nbf <= 0) return;
  dim3 g((nbf + 31) / 32, (nbf + 31) / 32), b(32, 8);
  symmetrize_perm_kernel<<<g, b, 0, s>>>(A, nbf, iperm, vxc, ld);
  GB300_CUDA(cudaGetLastError());
}

void launch_permute_matrix(const double* src, int nbf, const int* perm, double scale, double* dst,
                           cudaStream_t s) {
  if (nbf <= 0) return;
  const int gx = std::min((nbf + 255) / 256, 16);
  dim3 g(gx, std::min(nbf, std::max(1, 4864 / gx)));
  permute_matrix_kernel<<<g, 256, 0, s>>>(src, nbf, perm, scale, dst);
  GB300_CUDA(cudaGetLastError());
}

// dst(:, c) = src(:, c) for the n x n column-major matrices (leading
// dimensions lds, ldd); either side may be host memory the device can
// address (pageable memory access).
__global__ void copy_matrix_kernel(const double* __restrict__ src, int64_t lds,
                                   double* __restrict__ dst, int64_t ldd, int n) {
  const int64_t total = (int64_t)n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = i / n, r = i - c * n;
    dst[c * ldd + r] = src[c * lds + r];
  }
}

void launch_copy_matrix(const double* src, int64_t lds, double* dst, int64_t ldd, int n,
                        cudaStream_t s) {
  if (n <= 0) return;
  copy_matrix_kernel<<<1216, 256, 0, s>>>(src, lds, dst, ldd, n);
  GB300_CUDA(cudaGetLastError());
}

void launch_reduce_partials(const double2* partials, int64_t n, double* out, cudaStream_t s) {
  reduce_partials_kernel<<<1, 256, 0, s>>>(partials, n, out);
  GB300_CUDA(cudaGetLastError());
}

}  // namespace gb300
