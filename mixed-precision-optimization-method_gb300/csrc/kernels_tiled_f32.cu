// kernels_tiled_f32.cu -- float instantiation of the z-marching velocity/stress kernels (kernels_tiled_impl.cuh).
#include "kernels_tiled_impl.cuh"

namespace behf {
BEHF_TILED_INSTANTIATE(float)
}  // namespace behf
