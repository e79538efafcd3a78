// kernels_aux.cu -- set-up and per-step helper kernels (compiled with -fmad=false so that the
// double-precision coefficient build rounds exactly like a host computation of the same formulas).
//
//   k_coef        staggered averaging (main.cpp:322-359) + BEHF coefficients (main.cpp:431-494)
//   k_med_stats   medium extrema for the automatic storage scales
//   k_source      source injection at one cell (kernel.cu:130-142, one thread instead of a full grid)
//   k_record      receiver gather into the FP64 seismogram buffer (replaces kernel.cu:2197-2243)
//   k_tick        advances the device step counter read by k_source / k_record
//   k_health_*    FP64 energy norms + non-finite/saturation detector
//   k_get/k_set   one field in physical units <-> storage units
#include <cfloat>

#include "behf_aux.cuh"
#include "kernels_tiled.cuh"

namespace behf {

namespace {

__device__ __forceinline__ void atomic_max_pos(unsigned long long* a, double v) {
    atomicMax(a, (unsigned long long)__double_as_longlong(v));  // v >= 0: bit order == value order
}
__device__ __forceinline__ void atomic_min_pos(unsigned long long* a, double v) {
    atomicMin(a, (unsigned long long)__double_as_longlong(v));
}

// Physical coefficients of cell (i,j,k), double; zero on the outer planes (main.cpp loops 1..n-2).
__device__ void cell_coefs(const CoefArgs& a, int i, int j, int k, double out[kNCoef]) {
#pragma unroll
    for (int q = 0; q < kNCoef; q++) out[q] = 0.0;
    if (i < 1 || j < 1 || k < 1 || i > a.nx - 2 || j > a.ny - 2 || k > a.nz - 2) return;
    const long long sy = a.nx, sz = (long long)a.nx * a.ny;
    const long long c = k * sz + j * sy + i;
    auto m = [&](int q, long long o) { return (double)a.mod[q][o]; };
    auto harm4 = [&](long long p0, long long p1, long long p2, long long p3) {
        const double v0 = m(BEHF_MU, p0), v1 = m(BEHF_MU, p1), v2 = m(BEHF_MU, p2), v3 = m(BEHF_MU, p3);
        if (v0 == 0 || v1 == 0 || v2 == 0 || v3 == 0) return 0.0;
        return 1.0 / (0.25 * (1 / v0 + 1 / v1 + 1 / v2 + 1 / v3));
    };
    const double muxz = harm4(c, c + 1, c + sz, c + sz + 1);
    const double muyz = harm4(c, c + sy, c + sz, c + sz + sy);
    const double muxy = harm4(c, c + 1, c + sy, c + sy + 1);
    const long long nb[3] = {c + 1, c + sy, c + sz};
    double rho[3], rhof[3], b[3], mm[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        rho[d] = 0.5 * (m(BEHF_RHO, c) + m(BEHF_RHO, nb[d]));
        rhof[d] = 0.5 * (m(BEHF_RHOF, c) + m(BEHF_RHOF, nb[d]));
        b[d] = 0.5 * (m(BEHF_C1, c) + m(BEHF_C1, nb[d]));
        mm[d] = 0.5 * (m(BEHF_C2, c) + m(BEHF_C2, nb[d]));
    }
    const double dt = a.dt;
    if (!(b[0] == 0 || b[1] == 0 || b[2] == 0)) {  // any fluid neighbour zeroes the Darcy update
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const double mp = mm[d] - rhof[d] * rhof[d] / rho[d];
            const double D = mp + 0.5 * dt * b[d];
            out[VW1X + d] = (mp - 0.5 * dt * b[d]) / D;
            out[VW2X + d] = dt * (rhof[d] / rho[d]) / D;
            out[VW3X + d] = dt / D;
        }
    }
    if (!(rho[0] == 0 || rho[1] == 0 || rho[2] == 0)) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            out[VU1X + d] = dt / rho[d];
            out[VU2X + d] = rhof[d] / rho[d];
        }
    }
    out[P1] = m(BEHF_C, c) * dt;
    out[P2] = m(BEHF_M, c) * dt;
    out[S1] = m(BEHF_H2U, c) * dt;
    out[S2] = m(BEHF_HH, c) * dt;
    out[S3] = m(BEHF_C, c) * dt;
    out[SXYC] = muxy * dt;
    out[SXZC] = muxz * dt;
    out[SYZC] = muyz * dt;
}

// Unbiased rounding of a coefficient to FP16: the two FP16 neighbours a <= s <= b are chosen with
// probabilities (b - s)/(b - a) and (s - a)/(b - a), decided by a hash of (cell, array), so the rounding errors
// of a homogeneous region average to zero over a wavelength instead of biasing the wave speed.
__device__ __half dither_half(double s, long long cell, int q) {
    const __half a = __float2half_rn((float)s);
    const double da = (double)__half2float(a);
    if (da == s) return a;
    unsigned short ab = __half_as_ushort(a), bb;
    if ((ab & 0x7fffu) == 0) bb = s > 0 ? 0x0001 : 0x8001;
    else bb = ((da < s) == !(ab & 0x8000u)) ? (unsigned short)(ab + 1) : (unsigned short)(ab - 1);
    const __half b = __ushort_as_half(bb);
    const double db = (double)__half2float(b);
    const double pb = (s - da) / (db - da);  // in (0, 1/2]
    unsigned long long h = (unsigned long long)cell * 0x9E3779B97F4A7C15ull + (unsigned long long)(q + 1) * 0xD1B54A32D192ED03ull;
    h ^= h >> 30;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 27;
    h *= 0x94D049BB133111EBull;
    h ^= h >> 31;
    const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
    return u < pb ? b : a;
}

template <class K, class W>
__global__ void k_coef(CoefArgs a, int pass) {
    double mx[kNCoef];
#pragma unroll
    for (int q = 0; q < kNCoef; q++) mx[q] = 0.0;
    const long long N = (long long)a.nx * a.ny * a.nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % a.nx);
        const int j = (int)((c / a.nx) % a.ny);
        const int k = (int)(c / ((long long)a.nx * a.ny));
        double v[kNCoef];
        cell_coefs(a, i, j, k, v);
        const long long o = k * a.plane + j * a.px + i;
        if (pass == 0) {
#pragma unroll
            for (int q = 3; q < kNCoef; q++) mx[q] = fmax(mx[q], fabs(v[q] * a.ratio[q]));
        } else {
#pragma unroll
            for (int q = 0; q < 3; q++) reinterpret_cast<W*>(a.out[q])[o] = (W)v[q];
#pragma unroll
            for (int q = 3; q < kNCoef; q++) {
                const double s = v[q] * a.ratio[q] * a.inv[q];
                if constexpr (sizeof(K) == 2)
                    reinterpret_cast<K*>(a.out[q])[o] = a.dither ? dither_half(s, c, q) : __float2half_rn((float)s);
                else reinterpret_cast<K*>(a.out[q])[o] = (K)s;
            }
        }
    }
    if (pass == 0) {
        __shared__ double red[kNCoef][8];
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
        for (int q = 3; q < kNCoef; q++) {
            double v = mx[q];
            for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
            if (lane == 0) red[q][wid] = v;
        }
        __syncthreads();
        if (threadIdx.x < kNCoef && threadIdx.x >= 3) {
            double v = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) v = fmax(v, red[threadIdx.x][w]);
            atomic_max_pos(a.maxbits + threadIdx.x, v);
        }
    }
}

// Medium extrema: [0] max sqrt(rho*H), [1] max rho, [2] min C1 over C1 > 0.
__global__ void k_med_stats(const float* rho, const float* hh, const float* c1, long long N, unsigned long long* out) {
    double zmax = 0, rmax = 0, bmin = DBL_MAX;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        const double r = fmax((double)rho[c], 0.0), h = fmax((double)hh[c], 0.0), b = c1[c];
        zmax = fmax(zmax, sqrt(r * h));
        rmax = fmax(rmax, r);
        if (b > 0) bmin = fmin(bmin, b);
    }
    for (int o = 16; o > 0; o >>= 1) {
        zmax = fmax(zmax, __shfl_xor_sync(0xffffffffu, zmax, o));
        rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        bmin = fmin(bmin, __shfl_xor_sync(0xffffffffu, bmin, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_pos(out + 0, zmax);
        atomic_max_pos(out + 1, rmax);
        atomic_min_pos(out + 2, bmin);
    }
}

template <class S>
__global__ void k_source(DevPtrs p, long long o, int kind, const float* w, int nw, const int* d_it, int s_off,
                         double fac) {
    typedef Traits<S> T;
    typedef typename T::C C;
    const int it = *d_it + s_off;
    if (it >= nw) return;
    const C val = (C)((double)w[it] * fac);
    auto add = [&](int q) {
        S* f = reinterpret_cast<S*>(p.f[q]) + o;
        *f = T::st(T::ld(*f) + val);
    };
    if (kind == BEHF_SRC_EXPLOSIVE) {
        add(BEHF_SXX);
        add(BEHF_SYY);
        add(BEHF_SZZ);
    } else if (kind == BEHF_SRC_PRESSURE) {
        add(BEHF_P);
    } else {
        add(BEHF_VZ);
    }
}

template <class S>
__global__ void k_record(DevPtrs p, const long long* off, const int* comp, int nrec, double* seis, int cap,
                         const int* d_it, int s_off, RecScales sc) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const int it = *d_it + s_off;
    if (it >= cap) return;
    const int q = comp[r];
    seis[(long long)r * cap + it] = (double)Traits<S>::ld(reinterpret_cast<const S*>(p.f[q])[off[r]]) / sc.s[q];
}

__global__ void k_tick(int* d_it, int n) { *d_it += n; }

// Sum of squares of one field per block (storage units, FP64) + non-finite / saturation flag.
template <class S>
__global__ void k_health_part(const void* f, int nx, int ny, int nz, long long px, long long plane, double limit,
                              double* part, int* flag) {
    double acc = 0.0;
    int bad = 0;
    const long long N = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % nx);
        const long long r = c / nx;
        const int j = (int)(r % ny), k = (int)(r / ny);
        const double v = (double)Traits<S>::ld(reinterpret_cast<const S*>(f)[k * plane + j * px + i]);
        if (!(fabs(v) < limit)) bad = 1;  // NaN, Inf or at the top of the storage range
        else acc += v * v;
    }
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
        part[blockIdx.x] = s;
    }
    if (bad) atomicOr(flag, 1);
}

// Deterministic final sum of the block partials (fixed order, one warp).
__global__ void k_health_final(const double* part, int nblk, double* out) {
    double s = 0;
    for (int b = threadIdx.x; b < nblk; b += 32) s += part[b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) *out = s;
}

template <class S>
__global__ void k_get(const void* f, float* out, int nx, int ny, int nz, long long px, long long plane, double scale) {
    const long long N = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % nx);
        const long long r = c / nx;
        const int j = (int)(r % ny), k = (int)(r / ny);
        out[c] = (float)((double)Traits<S>::ld(reinterpret_cast<const S*>(f)[k * plane + j * px + i]) / scale);
    }
}
template <class S>
__global__ void k_set(void* f, const float* in, int nx, int ny, int nz, long long px, long long plane, double scale) {
    const long long N = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % nx);
        const long long r = c / nx;
        const int j = (int)(r % ny), k = (int)(r / ny);
        reinterpret_cast<S*>(f)[k * plane + j * px + i] =
            Traits<S>::st((typename Traits<S>::C)((double)in[c] * scale));
    }
}

}  // namespace

int aux_grid_blocks() {
    return device_sms() * 8;
}

template <class S>
cudaError_t aux_build_coefs(const CoefArgs& a, cudaStream_t st) {
    typedef typename Traits<S>::K K;
    typedef typename Traits<S>::W W;
    k_coef<K, W><<<aux_grid_blocks(), 256, 0, st>>>(a, a.pass);
    return cudaGetLastError();
}

cudaError_t aux_med_stats(const float* rho, const float* hh, const float* c1, long long N, unsigned long long* out,
                          cudaStream_t st) {
    k_med_stats<<<aux_grid_blocks(), 256, 0, st>>>(rho, hh, c1, N, out);
    return cudaGetLastError();
}

template <class S>
cudaError_t aux_source(const DevPtrs& p, long long o, int kind, const float* w, int nw, const int* d_it, int s_off,
                       double fac, cudaStream_t st) {
    k_source<S><<<1, 1, 0, st>>>(p, o, kind, w, nw, d_it, s_off, fac);
    return cudaGetLastError();
}

template <class S>
cudaError_t aux_record(const DevPtrs& p, const long long* off, const int* comp, int nrec, double* seis, int cap,
                       const int* d_it, int s_off, const RecScales& sc, cudaStream_t st) {
    if (nrec <= 0) return cudaSuccess;
    k_record<S><<<(nrec + 255) / 256, 256, 0, st>>>(p, off, comp, nrec, seis, cap, d_it, s_off, sc);
    return cudaGetLastError();
}

cudaError_t aux_tick(int* d_it, int n, cudaStream_t st) {
    k_tick<<<1, 1, 0, st>>>(d_it, n);
    return cudaGetLastError();
}

// Self-test of the pipelines' bounded wait: every thread waits (tiled::mbar_wait, the wait of the TMA pipelines)
// on an mbarrier that nothing arrives at; the wait gives up after its cycle limit and the block reports through
// the context's error word, exactly as a pipeline kernel whose copies never land.
__global__ void k_wait_selftest(int* err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        tiled::mbar_init(&bar, 1);
        tiled::fence_init();
    }
    __syncthreads();
    const bool ok = tiled::mbar_wait(&bar, 0u);
    if (!__all_sync(0xffffffffu, ok) && threadIdx.x == 0) atomicExch(err, 1);
}
cudaError_t aux_wait_selftest(int* err, cudaStream_t st) {
    k_wait_selftest<<<1, 32, 0, st>>>(err);
    return cudaGetLastError();
}

template <class S>
cudaError_t aux_health(const void* f, int nx, int ny, int nz, long long px, long long plane, double limit,
                       double* part, int nblk, int* flag, double* out, cudaStream_t st) {
    k_health_part<S><<<nblk, 256, 0, st>>>(f, nx, ny, nz, px, plane, limit, part, flag);
    k_health_final<<<1, 32, 0, st>>>(part, nblk, out);
    return cudaGetLastError();
}

template <class S>
cudaError_t aux_get(const void* f, float* out, int nx, int ny, int nz, long long px, long long plane, double scale,
                    cudaStream_t st) {
    k_get<S><<<aux_grid_blocks(), 256, 0, st>>>(f, out, nx, ny, nz, px, plane, scale);
    return cudaGetLastError();
}
template <class S>
cudaError_t aux_set(void* f, const float* in, int nx, int ny, int nz, long long px, long long plane, double scale,
                    cudaStream_t st) {
    k_set<S><<<aux_grid_blocks(), 256, 0, st>>>(f, in, nx, ny, nz, px, plane, scale);
    return cudaGetLastError();
}

#define BEHF_AUX_INST(S)                                                                                          \
    template cudaError_t aux_build_coefs<S>(const CoefArgs&, cudaStream_t);                                    \
    template cudaError_t aux_source<S>(const DevPtrs&, long long, int, const float*, int, const int*, int, double, \
                                       cudaStream_t);                                                            \
    template cudaError_t aux_record<S>(const DevPtrs&, const long long*, const int*, int, double*, int, const int*, \
                                       int, const RecScales&, cudaStream_t);                                     \
    template cudaError_t aux_health<S>(const void*, int, int, int, long long, long long, double, double*, int, int*, \
                                       double*, cudaStream_t);                                                   \
    template cudaError_t aux_get<S>(const void*, float*, int, int, int, long long, long long, double, cudaStream_t); \
    template cudaError_t aux_set<S>(void*, const float*, int, int, int, long long, long long, double, cudaStream_t);
BEHF_AUX_INST(double)
BEHF_AUX_INST(float)
BEHF_AUX_INST(__half)
BEHF_AUX_INST(__nv_bfloat16)

}  // namespace behf
