// behf_aux.cuh -- declarations of the set-up / per-step helper kernels (kernels_aux.cu).
#pragma once
#include "behf_internal.cuh"

namespace behf {

struct CoefArgs {
    const float* mod[kNMod];   // cell-centred moduli, [nz][ny][nx] (unpitched)
    int nx, ny, nz;
    long long px, plane;       // pitch of the outputs
    double dt;
    double ratio[kNCoef];      // scale ratios x 1/h applied to the physical coefficient
    double inv[kNCoef];        // 2^-e per array (storage multiplier inverse)
    void* out[kNCoef];
    unsigned long long* maxbits;  // pass 0: per-array max |ratio * coef| as double bits
    int pass;
    int dither;                // 16-bit coefficients: 0 round to nearest, 1 unbiased hash-dithered rounding
};

struct RecScales {
    double s[kNField];
};

int aux_grid_blocks();
template <class S> cudaError_t aux_build_coefs(const CoefArgs& a, cudaStream_t st);
cudaError_t aux_med_stats(const float* rho, const float* hh, const float* c1, long long N, unsigned long long* out,
                          cudaStream_t st);
template <class S>
cudaError_t aux_source(const DevPtrs& p, long long o, int kind, const float* w, int nw, const int* d_it, int s_off,
                       double fac, cudaStream_t st);
template <class S>
cudaError_t aux_record(const DevPtrs& p, const long long* off, const int* comp, int nrec, double* seis, int cap,
                       const int* d_it, int s_off, const RecScales& sc, cudaStream_t st);
cudaError_t aux_tick(int* d_it, int n, cudaStream_t st);
cudaError_t aux_wait_selftest(int* err, cudaStream_t st);
template <class S>
cudaError_t aux_health(const void* f, int nx, int ny, int nz, long long px, long long plane, double limit,
                       double* part, int nblk, int* flag, double* out, cudaStream_t st);
template <class S>
cudaError_t aux_get(const void* f, float* out, int nx, int ny, int nz, long long px, long long plane, double scale,
                    cudaStream_t st);
template <class S>
cudaError_t aux_set(void* f, const float* in, int nx, int ny, int nz, long long px, long long plane, double scale,
                    cudaStream_t st);

}  // namespace behf
