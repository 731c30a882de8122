// Shared definitions for the GB300 device kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#ifndef GB300_HD
#define GB300_HD __host__ __device__
#endif

namespace gb300 {

#define GB300_CUDA(call)                                                          \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + \
                               " at " + __FILE__ + ":" + std::to_string(__LINE__));  \
  } while (0)

// Shells in structure-of-arrays form (device pointers).
struct ShellsDev {
  int nshells;
  const double* alpha;    // packed primitives
  const double* coeff;    // packed, normalized contraction coefficients
  const int* prim_off;    // [nshells+1]
  const double* origin;   // [3*nshells]
  const int* l;           // angular momentum
  const int* pure;        // 1 = spherical
  // 2^(j/32), j = 0..31, as float-float pairs (exp2_table; the float-float
  // collocation of the tensor-core path only)
  const float2* exp2_tab = nullptr;
};

// The 32 values 2^(j/32) as float-float pairs (hi = the float nearest the
// double, lo = the float nearest the remainder), for ff::exp_neg.
std::vector<float2> exp2_table();

// Per-task layout of the device-resident plan (all device pointers).
// Points of task t live at [pt_off[t], pt_off[t] + npts_pad[t]); tasks are
// padded to a multiple of kPtBlock points with zero-weight copies of their
// first point.  Basis columns are padded to a multiple of kBfBlock with zero
// columns whose global AO index is -1.
struct TasksDev {
  int ntasks;
  const int64_t* pt_off;
  const int* npts_pad;
  const int* nbe;
  const int* nbe_pad;
  const int64_t* bf_off;   // into bf_list
  const int* bf_list;      // global AO index of each local column (-1 = padding)
  const int64_t* sh_off;   // into sh_list / sh_col
  const int* nsh;
  const int* sh_list;      // global shell index
  const int* sh_col;       // first local column of the shell
  const int64_t* scr_off;  // offset (doubles) of the task's scratch block, batch-relative
  const double* x;
  const double* y;
  const double* z;
  const double* w;
};

constexpr int kPtBlock = 64;   // point padding / density tile rows
constexpr int kBfBlock = 64;   // basis padding / tile columns

// ---------------------------------------------------------------- launchers
// SSF weights of npts points (reference algorithm, cuda_ssf_1d.cu:24-131);
// status (may be null) is set to 1 when a parent index lies outside
// [0, natoms), and that point keeps its weight.
void launch_ssf_weights(int64_t npts, int natoms, const double* x, const double* y,
                        const double* z, const int32_t* iparent, const double* dist_nearest,
                        const double* coords, const double* rab_inv, int ld_rab,
                        double* dist_scr, int ld_dist, double* weights, int* status,
                        cudaStream_t s);

// The same weights with the cell products screened per chunk of 32 points
// and every factor classified in FP32 first (ssf.cu); natoms <=
// kSSFScreenedMaxAtoms.  coords_f: (x - o, y - o, z - o, 0) of every atom in
// FP32 for the origin o; margin: a bound on the FP32 error of mu (ssf.cu).
constexpr int kSSFScreenedMaxAtoms = 2048;
void launch_ssf_weights_screened(int64_t npts, int natoms, const double* x, const double* y,
                                 const double* z, const int32_t* iparent,
                                 const double* dist_nearest, const double* coords,
                                 const float4* coords_f, double ox, double oy, double oz,
                                 float margin, const double* rab_inv, int ld_rab, double* weights,
                                 int* status, cudaStream_t s);

void launch_collocation(const ShellsDev& sh, const TasksDev& tk, const int2* items, int nitems,
                        double* scr, bool grad, cudaStream_t s);

}  // namespace gb300
