// behf_internal.cuh -- types shared by the libbehf translation units.
//
// Data layout in HBM (one context):
//   * 13 wavefields, one array each, x fastest with a row pitch px (multiple of 16 elements) and
//     plane stride px*ny; storage type S = double | float | __half | __nv_bfloat16, values scaled by
//     the per-field storage scales (s_v for v, s_q for q, s_sigma for the stresses, s_p for p).
//   * 23 per-cell coefficient arrays (same pitch): the three Darcy factors VW1 in W (float, or double
//     for FP64) and 20 more in K (half for the 16-bit kinds, else S) multiplied by a power of two
//     kmul[j] so that each array's largest magnitude sits just below 1.
//   * CPML memory only inside the boundary slabs: for each axis 8 derivatives x {psi, previous
//     derivative} in W, 2L+1 slab cells ([0,L) and [n-1-L, n)) at slab indices 0..2L, layouts
//     x: [nz][ny][W], y: [nz][W][nx], z: [W][ny][nx] with W = 2L+1 rounded up to a multiple of 4 (16-byte
//     rows of FP32 for the tensor-memory kernels' TMA boxes of x-slab memory; the padding is never
//     touched).  The reference keeps 24+24 full-volume FP16 arrays instead (common.h:27-30).
//   * 1-D damping profiles per axis (A = e, B = -dt d / 2, and the half-shifted A2, B2).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "behf.h"

namespace behf {

constexpr int kNField = 13;
constexpr int kNCoef = 23;
constexpr int kNMod = 9;

// Coefficient indices (reference names VelocityWParameter*, VelocityUParameter*, PressParameter*,
// StressParameter*: main.cpp:431-494).
enum {
    VW1X = 0, VW1Y, VW1Z, VW2X, VW2Y, VW2Z, VW3X, VW3Y, VW3Z, VU1X, VU1Y, VU1Z, VU2X, VU2Y, VU2Z,
    P1, P2, S1, S2, S3, SXYC, SXZC, SYZC
};

// Storage traits: S stored, C arithmetic, K coefficient storage, W CPML memory / Darcy factor.
template <class S> struct Traits;
template <> struct Traits<double> {
    typedef double C;
    typedef double K;
    typedef double W;
    static __device__ __forceinline__ C ld(double v) { return v; }
    static __device__ __forceinline__ double st(C v) { return v; }
    static __device__ __forceinline__ C ldk(double v) { return v; }
    static constexpr int prec = BEHF_FP64;
};
template <> struct Traits<float> {
    typedef float C;
    typedef float K;
    typedef float W;
    static __device__ __forceinline__ C ld(float v) { return v; }
    static __device__ __forceinline__ float st(C v) { return v; }
    static __device__ __forceinline__ C ldk(float v) { return v; }
    static constexpr int prec = BEHF_FP32;
};
template <> struct Traits<__half> {
    typedef float C;
    typedef __half K;
    typedef float W;
    static __device__ __forceinline__ C ld(__half v) { return __half2float(v); }
    static __device__ __forceinline__ __half st(C v) { return __float2half_rn(v); }
    static __device__ __forceinline__ C ldk(__half v) { return __half2float(v); }
    static constexpr int prec = BEHF_FP16;
};
template <> struct Traits<__nv_bfloat16> {
    typedef float C;
    typedef __half K;
    typedef float W;
    static __device__ __forceinline__ C ld(__nv_bfloat16 v) { return __bfloat162float(v); }
    static __device__ __forceinline__ __nv_bfloat16 st(C v) { return __float2bfloat16_rn(v); }
    static __device__ __forceinline__ C ldk(__half v) { return __half2float(v); }
    static constexpr int prec = BEHF_BF16;
};

// Largest finite value of each storage format: the health checks flag a stored value whose magnitude reaches it
// (saturated by a rounding that overflowed into it, or past it as Inf).  BF16 keeps FP32's exponent range but only
// 8 significand bits, so its top is (2 - 2^-7) 2^127, below FLT_MAX.
inline double storage_max(int precision) {
    switch (precision) {
        case BEHF_FP16: return 65504.0;
        case BEHF_BF16: return 3.3895313892515355e38;
        case BEHF_FP32: return 3.4028234663852886e38;
        default: return 1.7976931348623157e308;
    }
}

// Staggered first-derivative weights of order 2R: D(i+1/2) = sum_m w_m (f[i+m] - f[i-m+1]) / h.
template <int R>
__host__ __device__ constexpr double stencil_w(int m) {
    return R == 1 ? 1.0
         : R == 2 ? (m == 1 ? 9.0 / 8.0 : -1.0 / 24.0)
         : R == 3 ? (m == 1 ? 75.0 / 64.0 : m == 2 ? -25.0 / 384.0 : 3.0 / 640.0)
                  : (m == 1 ? 1225.0 / 1024.0 : m == 2 ? -245.0 / 3072.0 : m == 3 ? 49.0 / 5120.0 : -5.0 / 7168.0);
}

// Type-erased device pointers of one context (cast inside the kernels).
struct DevPtrs {
    void* f[kNField];
    void* k[kNCoef];       // k[0..2]: VW1 in W; k[3..22]: K
    void* psi[3][8];       // CPML memory per axis, 4 V derivatives then 4 T derivatives
    void* prv[3][8];
    void* pa[3];           // per-axis profiles in C: e, -dt d/2 (integer points), and half-shifted
    void* pb[3];
    void* pa2[3];
    void* pb2[3];
};

struct Geom {
    int nx, ny, nz;
    int R, L, W;           // stencil half-width, CPML width, slab pitch (2L+1 rounded up to 4; 0 without CPML)
    int xs_bw;             // tensor-memory kernels: width of the TMA box of x-slab CPML memory (0: none)
    int slab_pf;           // tensor-memory kernels: 1 when the y/z-slab tensor maps exist (L2 prefetch of slab memory)
    long long px, plane;   // row pitch and plane stride in elements
    int bug;               // reference vz/VW3y compatibility
    int* err;              // device error word: set to 1 by a kernel whose bounded wait timed out
    int zchunk_req;        // tiled kernels: z planes per CTA (0 = automatic)
    int ws;                // tiled kernels: 0 = classic, 1 = warp-specialised (every read through TMA), 2 = the same
                           // with the z derivatives accumulated in tensor memory
    int sr;                // 16-bit kinds, tiled kernels: stochastic rounding of the stored fields
    const int* step;       // device step counter (seeds the stochastic rounding)
    int step_off;          // step offset of this launch within a graph chunk
    float kmulf[kNCoef];   // power-of-two multipliers of the stored coefficients
    double kmuld[kNCoef];
    // Exact identities the tiled kernels use instead of reading two more arrays (effective, scaled values):
    //   VW2 = VU2 * VW3 * c_vw2   (dt rho_f/rho / D = (rho_f/rho) (dt / D)),  c_vw2 = s_p s_q / (s_v s_sigma)
    //   S3  = P1 * c_s3           (both C dt),                                 c_s3  = s_sigma s_v / (s_p s_q)
    float c_vw2, c_s3;
};

__host__ __device__ __forceinline__ int slab_index(int i, int n, int L) {
    return i < L ? i : (i >= n - 1 - L ? L + (i - (n - 1 - L)) : -1);
}

// Per-device state is kept in arrays indexed by the CUDA device ordinal (at most kMaxDevices devices).
constexpr int kMaxDevices = 64;
inline int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
    return dev;
}

// SMs of the current device, read once per device (thread-safe; 148 if the query fails).
inline int device_sms() {
    static std::once_flag once[kMaxDevices];
    static int sms[kMaxDevices];
    const int dev = current_device();
    std::call_once(once[dev], [&] {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        sms[dev] = n > 0 ? n : 148;
    });
    return sms[dev];
}

// A set-up step that must run once on every device a kernel is launched on (a kernel's shared-memory opt-in:
// cudaFuncSetAttribute applies to the current device only).  run_once runs f once per device, with that device
// current, also when several host threads launch at the same time; every caller gets f's status on its device.
struct PerDevice {
    std::once_flag flag[kMaxDevices];
    cudaError_t status[kMaxDevices] = {};
};
template <class F>
inline cudaError_t run_once(PerDevice& pd, F&& f) {
    const int dev = current_device();
    std::call_once(pd.flag[dev], [&] { pd.status[dev] = f(); });
    return pd.status[dev];
}

// Makes a context's device current for the duration of an entry point and restores the caller's device after.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess) prev = cur;
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};

// z planes per CTA of a z-marching launch over nxy tiles and `planes` planes with `slots` CTAs resident per
// wave: the chunk length in [minz, maxz] minimising (waves, rounded up) x (chunk + halo), so that the last wave
// is not left mostly empty (a wave's time is set by its longest CTA) and short chunks do not repeat the halo
// planes' warm-up too often; among the chunk lengths that give at least minw waves, or as many CTAs as the
// shortest chunk gives when that is fewer (more, shorter CTAs even out tiles of unequal cost).  Ties go to the
// longer chunk.
inline int wave_zchunk(int nxy, int planes, int slots, int minz, int maxz, int halo, int minw = 1) {
    if (planes <= 0) return 1;
    if (minz < 1) minz = 1;
    if (maxz < minz) maxz = minz;
    const int cmax = planes / minz > 1 ? planes / minz : 1;
    const long long nmax = (planes + (planes + cmax - 1) / cmax - 1) / ((planes + cmax - 1) / cmax);
    const long long floor_ctas = std::min((long long)minw * slots, (long long)nxy * nmax);
    int best = planes < maxz ? planes : maxz;
    long long bestcost = -1;
    for (int nch = 1; nch <= cmax; nch++) {
        const int zc = (planes + nch - 1) / nch;
        if (zc > maxz) continue;
        const long long n = (planes + zc - 1) / zc;
        if ((long long)nxy * n < floor_ctas) continue;
        const long long waves = ((long long)nxy * n + slots - 1) / slots;
        const long long cost = waves * (zc + halo);
        if (bestcost < 0 || cost < bestcost) {
            bestcost = cost;
            best = zc;
        }
    }
    return best;
}

// Launchers (defined per translation unit).
template <class S> cudaError_t launch_plain(const Geom& g, const DevPtrs& p, bool vel, cudaStream_t st);
// maps: the context's tiled::VMaps (vel) or tiled::TMaps (stress), host memory, 64-byte aligned.
template <class S> cudaError_t launch_tiled(const Geom& g, const DevPtrs& p, const void* maps, bool vel, cudaStream_t st);
template <class S> bool tiled_supported(const Geom& g);
template <class S> cudaError_t tiled_build_maps(const Geom& g, const DevPtrs& p, void* vmaps, void* tmaps);
// Re-encode only the field maps of built maps: vf the 13 arrays the velocity kernel reads, tf the stress kernel's.
template <class S> cudaError_t tiled_field_maps(const Geom& g, void* const* vf, void* const* tf, void* vmaps, void* tmaps);
// The same with 4-row tiles (kernels_tiled_<type>_rows4.cu).
template <class S> cudaError_t launch_tiled_rows4(const Geom& g, const DevPtrs& p, const void* maps, bool vel, cudaStream_t st);
template <class S> bool tiled_supported_rows4(const Geom& g);
template <class S> cudaError_t tiled_build_maps_rows4(const Geom& g, const DevPtrs& p, void* vmaps, void* tmaps);
template <class S> cudaError_t tiled_field_maps_rows4(const Geom& g, void* const* vf, void* const* tf, void* vmaps,
                                                      void* tmaps);

}  // namespace behf
