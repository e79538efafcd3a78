// behf_medium.cuh -- device medium generator (kernels_medium.cu).
#pragma once
#include "behf_internal.cuh"

namespace behf {
// mod[9]: outputs (N floats each); work: 5*N floats when the spec has a perturbation.
cudaError_t generate_medium(const behf_medium_spec& s, int nx, int ny, int nz, float* const mod[kNMod], float* work,
                            cudaStream_t st, int nblk);
}  // namespace behf
