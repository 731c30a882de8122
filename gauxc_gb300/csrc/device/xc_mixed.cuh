// Mixed-precision (split-mantissa FP64 emulation) contractions.
#pragma once
#include <functional>
#include <vector>

#include "device_common.cuh"
#include "functionals.cuh"

namespace gb300 {

struct MixedWorkspace {
  char* base = nullptr;
  size_t bytes = 0;
};

MixedWorkspace mixed_workspace_create(int ntasks, const std::vector<int>& npts_pad,
                                      const std::vector<int>& nbe_pad,
                                      const std::vector<int64_t>& scr_off,
                                      const std::function<char*(size_t)>& alloc);

// Return the number of kernel launches issued.
int launch_density_mixed(MixedWorkspace& ws, const TasksDev& tk, int t_begin, int t_end,
                         const int2* items, int nitems, const double* scr, const double* P,
                         int nbf, const XCFunctionalDesc& f, double4* zcoef, double2* partials,
                         cudaStream_t s);
int launch_vxc_mixed(MixedWorkspace& ws, const TasksDev& tk, int t_begin, int t_end,
                     const int4* items, int nitems, const double* scr, double* A, int nbf,
                     bool gga, cudaStream_t s);

}  // namespace gb300
