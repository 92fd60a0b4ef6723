// Instantiations of the delay-and-sum kernels: synth geometry, f32 channel data.
// (Split per geometry and storage type so the library's files compile in parallel.)
#include "das_impl.cuh"

namespace pgb {

cudaError_t launch_das_synth_f32(const DasArgs &a, int interp, int sum, bool census, cudaStream_t s) {
    return launch_das_geom_type<GEOM_SYNTH, float>(a, interp, sum, census, s);
}

}  // namespace pgb
