// kernels_tiled_f16_rows4.cu -- __half instantiation of the z-marching kernels with 4-row tiles (kernels_tiled_impl.cuh):
// four compute warps and a producer warp per CTA, up to four CTAs per SM, entry points suffixed _rows4.
#define BEHF_TILED_TY 4
#define BEHF_TILED_NAMESPACE tiled4
#define BEHF_TILED_FN(name) name##_rows4
#define BEHF_WS_MINB16 4
#define BEHF_TILED_MINB16 6
#define BEHF_TILED_MINB16_T 6
#include "kernels_tiled_impl.cuh"

namespace behf {
BEHF_TILED_INSTANTIATE(__half)
}  // namespace behf
