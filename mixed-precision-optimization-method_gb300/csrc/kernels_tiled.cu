// kernels_tiled.cu -- z-marching shared-memory velocity / stress kernels (in progress).
#include "behf_internal.cuh"

namespace behf {

template <class S> bool tiled_supported(const Geom&) { return false; }
template <class S> cudaError_t launch_tiled(const Geom&, const DevPtrs&, bool, cudaStream_t) {
    return cudaErrorNotSupported;
}

template bool tiled_supported<double>(const Geom&);
template bool tiled_supported<float>(const Geom&);
template bool tiled_supported<__half>(const Geom&);
template bool tiled_supported<__nv_bfloat16>(const Geom&);
template cudaError_t launch_tiled<double>(const Geom&, const DevPtrs&, bool, cudaStream_t);
template cudaError_t launch_tiled<float>(const Geom&, const DevPtrs&, bool, cudaStream_t);
template cudaError_t launch_tiled<__half>(const Geom&, const DevPtrs&, bool, cudaStream_t);
template cudaError_t launch_tiled<__nv_bfloat16>(const Geom&, const DevPtrs&, bool, cudaStream_t);

}  // namespace behf
