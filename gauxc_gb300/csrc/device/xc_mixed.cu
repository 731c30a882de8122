// Mixed-precision contractions: not built yet in this revision; selecting the
// "GB300-Mixed" local work driver raises an error instead of silently running
// another path.
#include "xc_mixed.cuh"

namespace gb300 {

MixedWorkspace mixed_workspace_create(int, const std::vector<int>&, const std::vector<int>&,
                                      const std::vector<int64_t>&,
                                      const std::function<char*(size_t)>&) {
  throw std::runtime_error("GB300-Mixed local work driver is not available in this build");
}
int launch_density_mixed(MixedWorkspace&, const TasksDev&, int, int, const int2*, int,
                         const double*, const double*, int, const XCFunctionalDesc&, double4*,
                         double2*, cudaStream_t) {
  throw std::runtime_error("GB300-Mixed local work driver is not available in this build");
}
int launch_vxc_mixed(MixedWorkspace&, const TasksDev&, int, int, const int4*, int, const double*,
                     double*, int, bool, cudaStream_t) {
  throw std::runtime_error("GB300-Mixed local work driver is not available in this build");
}

}  // namespace gb300
