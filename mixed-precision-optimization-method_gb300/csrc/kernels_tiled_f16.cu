// kernels_tiled_f16.cu -- __half instantiation of the z-marching velocity/stress kernels (kernels_tiled_impl.cuh).
#include "kernels_tiled_impl.cuh"

namespace behf {
BEHF_TILED_INSTANTIATE(__half)
}  // namespace behf
