// kernels_tiled_f64.cu -- FP64 has no tiled kernel (the FP64 kind is the GPU oracle run, on the plain kernels).
#include "behf_internal.cuh"

namespace behf {
template <>
bool tiled_supported<double>(const Geom&) {
    return false;
}
template <>
cudaError_t tiled_build_maps<double>(const Geom&, const DevPtrs&, void*, void*) {
    return cudaErrorNotSupported;
}
template <>
cudaError_t tiled_field_maps<double>(const Geom&, void* const*, void* const*, void*, void*) {
    return cudaErrorNotSupported;
}
template <>
cudaError_t tiled_field_maps_rows4<double>(const Geom&, void* const*, void* const*, void*, void*) {
    return cudaErrorNotSupported;
}
template <>
cudaError_t launch_tiled<double>(const Geom&, const DevPtrs&, const void*, bool, cudaStream_t) {
    return cudaErrorNotSupported;
}
template <>
bool tiled_supported_rows4<double>(const Geom&) {
    return false;
}
template <>
cudaError_t tiled_build_maps_rows4<double>(const Geom&, const DevPtrs&, void*, void*) {
    return cudaErrorNotSupported;
}
template <>
cudaError_t launch_tiled_rows4<double>(const Geom&, const DevPtrs&, const void*, bool, cudaStream_t) {
    return cudaErrorNotSupported;
}
}  // namespace behf
