// kernels_tiled_bf16.cu -- __nv_bfloat16 instantiation of the z-marching velocity/stress kernels (kernels_tiled_impl.cuh).
#include "kernels_tiled_impl.cuh"

namespace behf {
BEHF_TILED_INSTANTIATE(__nv_bfloat16)
}  // namespace behf
