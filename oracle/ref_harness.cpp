// ref_harness.cpp -- runs the reference's own FD kernels on the CPU to pin the oracle.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build.py extracts the bodies of Source, FD_Vbottom and
// FD_Tbottom (kernel.cu:130-142, 317-401, 585-675) together with the d_C* scale macros from the
// read-only reference tree into oracle/_ref/ref_kernels.inc (never committed), and compiles them
// here as host functions.  Each CUDA "thread" becomes one call with blockIdx = the cell, so the
// kernels run unchanged on a single domain (partIndex = 0, nzt = nz - 1), exactly the setting of
// the reference's bottom part.  The output is the golden data the oracle is checked against.
#include <cstdint>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace refshim {
// Host stand-in for cuda_fp16's __half as the kernels use it: float in, float out,
// double assignment rounds once (as __half::operator=(double) does).
struct half16 {
    _Float16 v;
    half16& operator=(float f) {
        v = (_Float16)f;
        return *this;
    }
    half16& operator=(double d) {
        v = (_Float16)d;
        return *this;
    }
    operator float() const { return (float)v; }
};
struct dim3u {
    unsigned x, y, z;
};
static thread_local dim3u threadIdx = {0, 0, 0};
static thread_local dim3u blockIdx = {0, 0, 0};
static thread_local dim3u blockDim = {1, 1, 1};
typedef half16 data_t;
#define __global__ static
#include "ref_kernels.inc"
#undef __global__
}  // namespace refshim

using refshim::data_t;

// The reference's medium builder (outputfunc.cpp:153-222), linked from its own source file.
void create_model_all(float*** vp, float*** vs, float*** rhos, float*** vf, float*** vfg, float*** rho,
                      float*** rhof, float*** M, float*** C, float*** C1, float*** C2, float*** HH,
                      float*** H2u, float*** mu, int nr, int ny, int nc);
float*** space3d(int nr, int ny, int nc);
void free_space3d(float*** a, int nr, int ny);

// out[9] in the oracle's moduli order: rho, rhof, mu, M, C, HH, H2u, C1, C2; each [nz][ny][nx].
extern "C" int ref_medium(int nz, int ny, int nx, float* const out[9]) {
    float*** a[14];
    for (int i = 0; i < 14; i++) a[i] = space3d(nz, ny, nx);
    // argument order of create_model_all: vp vs rhos vf vfg rho rhof M C C1 C2 HH H2u mu
    create_model_all(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13],
                     nz, ny, nx);
    const int pick[9] = {5, 6, 13, 7, 8, 11, 12, 9, 10};
    for (int q = 0; q < 9; q++)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                std::memcpy(out[q] + ((size_t)k * ny + j) * nx, a[pick[q]][k][j], sizeof(float) * nx);
    for (int i = 0; i < 14; i++) free_space3d(a[i], nz, ny);
    return 0;
}

extern "C" int ref_run(int nx, int ny, int nz, float DT, int nt, int sn, const float* wavelet,
                       uint16_t* const st[16], const uint16_t* const cf[23], const uint16_t* const pr[12],
                       uint16_t* const ax[48], int nrec, const int* rec_lin, const int* rec_comp, float* seis) {
    static_assert(sizeof(data_t) == 2, "half stand-in must be 2 bytes");
    auto S = [&](int i) { return reinterpret_cast<data_t*>(st[i]); };
    auto K = [&](int i) { return reinterpret_cast<data_t*>(const_cast<uint16_t*>(cf[i])); };
    auto P = [&](int i) { return reinterpret_cast<data_t*>(const_cast<uint16_t*>(pr[i])); };
    auto A = [&](int i) { return reinterpret_cast<data_t*>(ax[i]); };
    data_t *vux = S(0), *vuy = S(1), *vuz = S(2), *vwx = S(3), *vwy = S(4), *vwz = S(5);
    data_t *txx = S(6), *tyy = S(7), *tzz = S(8), *txy = S(9), *txz = S(10), *tyz = S(11), *ss = S(12);
    data_t *vwx2 = S(13), *vwy2 = S(14), *vwz2 = S(15);
    data_t *dxi = P(0), *dxi2 = P(1), *e_dxi = P(2), *e_dxi2 = P(3);
    data_t *dyj = P(4), *dyj2 = P(5), *e_dyj = P(6), *e_dyj2 = P(7);
    data_t *dzk = P(8), *dzk2 = P(9), *e_dzk = P(10), *e_dzk2 = P(11);
    const int nzt = nz - 1;
    for (int it = 0; it < nt; it++) {
        {
            refshim::blockIdx = {(unsigned)(sn % nx), (unsigned)((sn / nx) % ny), (unsigned)(sn / (nx * ny))};
            refshim::Source(txx, tyy, tzz, wavelet[it], sn, nx, ny, nz);
        }
#pragma omp parallel for collapse(2) schedule(static)
        for (int iz = 0; iz < nzt; iz++)
            for (int iy = 0; iy < ny; iy++)
                for (int ix = 0; ix < nx; ix++) {
                    refshim::blockIdx = {(unsigned)ix, (unsigned)iy, (unsigned)iz};
                    refshim::FD_Vbottom(vux, vuy, vuz, txx, tyy, tzz, txz, txy, tyz,
                                        A(0), A(1), A(2), A(3), A(4), A(5), A(6), A(7), A(8),
                                        A(12), A(13), A(14), A(15), A(16), A(17), A(18), A(19), A(20),
                                        e_dxi, dxi, e_dxi2, dxi2, e_dyj, dyj, e_dyj2, dyj2, e_dzk, dzk, dzk2, e_dzk2,
                                        ss, vwx, vwy, vwz, vwx2, vwy2, vwz2, A(21), A(22), A(23), A(9), A(10), A(11),
                                        K(0), K(1), K(2), K(3), K(4), K(5), K(6), K(7), K(8),
                                        K(9), K(10), K(11), K(12), K(13), K(14), DT, nx, ny, nzt, 0);
                }
#pragma omp parallel for collapse(2) schedule(static)
        for (int iz = 0; iz < nzt; iz++)
            for (int iy = 0; iy < ny; iy++)
                for (int ix = 0; ix < nx; ix++) {
                    refshim::blockIdx = {(unsigned)ix, (unsigned)iy, (unsigned)iz};
                    refshim::FD_Tbottom(vux, vuy, vuz, txx, tzz, tyy, txz, txy, tyz,
                                        A(24), A(25), A(26), A(27), A(28), A(29), A(30), A(31), A(32),
                                        A(36), A(37), A(38), A(39), A(40), A(41), A(42), A(43), A(44),
                                        e_dxi, dxi, e_dxi2, dxi2, e_dyj2, dyj2, e_dyj, dyj, dzk2, e_dzk2, e_dzk, dzk,
                                        A(45), A(46), A(47), vwx, vwy, vwz, ss, A(33), A(34), A(35),
                                        K(15), K(16), K(17), K(18), K(19), K(20), K(21), K(22), DT, nx, ny, nzt, 0);
                }
        for (int r = 0; r < nrec; r++) seis[(size_t)r * nt + it] = (float)S(rec_comp[r])[rec_lin[r]];
    }
    return 0;
}
