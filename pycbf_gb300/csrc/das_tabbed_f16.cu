// Instantiations of the delay-and-sum kernels: tabbed geometry, f16 channel data.
// (Split per geometry and storage type so the library's files compile in parallel.)
#include "das_impl.cuh"

namespace pgb {

cudaError_t launch_das_tabbed_f16(const DasArgs &a, int interp, int sum, bool census, cudaStream_t s) {
    return launch_das_geom_type<GEOM_TABBED, __half>(a, interp, sum, census, s);
}

}  // namespace pgb
