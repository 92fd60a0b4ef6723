// Instantiations of the Tabbed delay-and-sum kernels (generic and TMA-staged) and
// of the staging plan for f32 channel data.  Split per storage type so the
// library's files compile in parallel.
#include "das_staged.cuh"

namespace pgb {

cudaError_t launch_das_tabbed_f32(const DasArgs &a, int interp, int sum, bool census, cudaStream_t s) {
    return launch_das_geom_type<GEOM_TABBED, float>(a, interp, sum, census, s);
}

cudaError_t launch_plan_f32(const DasArgs &a, int interp, int *plan, cudaStream_t s) {
    return launch_plan_type<float>(a, interp, plan, s);
}

cudaError_t launch_staged_f32(const DasArgs &a, int interp, int sum, const int *plan, int *status,
                               cudaStream_t s) {
    return launch_staged_type<float>(a, interp, sum, plan, status, s);
}

cudaError_t launch_staged_adj_f32(const DasArgs &a, int sum, const int *plan, cudaStream_t s) {
    return launch_staged_adj<float>(a, sum, plan, s);
}

}  // namespace pgb
