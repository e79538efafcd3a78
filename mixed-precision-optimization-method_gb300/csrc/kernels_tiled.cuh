// kernels_tiled.cuh -- z-marching velocity / stress kernels for sm_103a (FP16, BF16, FP32 storage).
//
// One CTA owns an xy tile of TXC x TY cells (64 x 8; 256 threads, each thread a pair of adjacent x cells,
// one warp per tile row) and marches it through a range of z planes, one plane per iteration:
//   * thread 0 issues TMA copies (cp.async.bulk.tensor.3d) for plane k + 1 while plane k is computed: the
//     xy-halo boxes of the fields with x/y derivatives into a two-stage shared-memory ring, and the next plane
//     of each field with a z derivative into a z ring of 2R + 2 planes (the reference re-reads every
//     neighbour from HBM, kernel.cu:172-185); full/empty mbarriers pipeline the stages.  Halo boxes start on
//     16-byte x boundaries (x0 - 16 B) and TMA zero-fills outside the grid, which provides the ghost zeros of
//     the domain faces;
//   * the cell's own fields and coefficients are coalesced pair loads from global memory (each is read by one
//     thread only), issued where they hide best: before the waits (stress) or after the stencils (velocity);
//   * x/y/z stencils are evaluated on cell pairs with packed FP32 arithmetic (fma.rn.f32x2);
//   * CPML memory is touched only on slab cells (z: block-uniform, y: warp-uniform, x: per cell).
// Every mbarrier wait is bounded: on timeout the CTA sets the context's error word, drains its
// outstanding copies (bounded again) and exits, so the host sees BEHF_ERR_TIMEOUT instead of a hang.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "behf_internal.cuh"

// The tiled kernels are compiled twice: with 8-row tiles in behf::tiled (kernels_tiled_<type>.cu) and with 4-row
// tiles in behf::tiled4, entry points suffixed _rows4 (kernels_tiled_<type>_rows4.cu).  A translation unit sets the
// tile height, the namespace and the entry-point names before including this header.
#ifndef BEHF_TILED_NAMESPACE
#define BEHF_TILED_NAMESPACE tiled
#endif
#ifndef BEHF_TILED_FN
#define BEHF_TILED_FN(name) name
#endif

namespace behf {
namespace BEHF_TILED_NAMESPACE {

#ifndef BEHF_TILED_TY
#define BEHF_TILED_TY 8
#endif
constexpr int TXC = 64;            // cells per tile row (x)
constexpr int TY = BEHF_TILED_TY;  // tile rows (y), one warp each
constexpr int NTH = 32 * TY;       // threads per CTA
constexpr long long kSpinLimit = 4000000000LL;  // clock64 cycles (~2 s) before a wait gives up

template <class S> struct Pair;
template <> struct Pair<__half> {
    typedef __half2 T;
    static __device__ __forceinline__ float2 f2(T v) { return __half22float2(v); }
    static __device__ __forceinline__ T pack(float2 v) { return __float22half2_rn(v); }
    static __device__ __forceinline__ __half one(float v) { return __float2half_rn(v); }
};
template <> struct Pair<__nv_bfloat16> {
    typedef __nv_bfloat162 T;
    static __device__ __forceinline__ float2 f2(T v) { return __bfloat1622float2(v); }
    static __device__ __forceinline__ T pack(float2 v) { return __float22bfloat162_rn(v); }
    static __device__ __forceinline__ __nv_bfloat16 one(float v) { return __float2bfloat16_rn(v); }
};
template <> struct Pair<float> {
    typedef float2 T;
    static __device__ __forceinline__ float2 f2(T v) { return v; }
    static __device__ __forceinline__ T pack(float2 v) { return v; }
    static __device__ __forceinline__ float one(float v) { return v; }
};

// Stochastic rounding of a float pair to the 16-bit storage types, from 32 random bits r (16 per value for
// BF16, 13 per value for FP16): a value between two representable neighbours goes to the upper one with
// probability equal to its distance from the lower one, so rounding errors average out over the steps instead
// of dropping increments smaller than half a unit in the last place.  Adding the random bits below the kept
// mantissa bits and truncating does exactly that for normal numbers; FP16 subnormals (|x| < 2^-14) and
// non-finite values are rounded to nearest.
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float sr_trunc(float x, uint32_t r, int drop) {
    const uint32_t u = __float_as_uint(x), mask = (1u << drop) - 1u;
    return __uint_as_float((u + (r & mask)) & ~mask);
}
template <class S> struct SR;
template <> struct SR<__half> {
    static __device__ __forceinline__ __half2 pack(float2 v, uint32_t r) {
        const float a = fabsf(v.x) >= 6.103515625e-05f && fabsf(v.x) < 65504.f ? sr_trunc(v.x, r, 13) : v.x;
        const float b = fabsf(v.y) >= 6.103515625e-05f && fabsf(v.y) < 65504.f ? sr_trunc(v.y, r >> 16, 13) : v.y;
        return __floats2half2_rn(a, b);
    }
};
template <> struct SR<__nv_bfloat16> {
    static __device__ __forceinline__ __nv_bfloat162 pack(float2 v, uint32_t r) {
        const float a = isfinite(v.x) ? sr_trunc(v.x, r, 16) : v.x;
        const float b = isfinite(v.y) ? sr_trunc(v.y, r >> 16, 16) : v.y;
        return __floats2bfloat162_rn(a, b);
    }
};
template <> struct SR<float> {
    static __device__ __forceinline__ float2 pack(float2 v, uint32_t) { return v; }
};

// Box geometry in elements.  X boxes carry an x halo of HX = 16 bytes each side, Y boxes a y halo of R
// rows, XY boxes both; own-cell boxes are TXC x TY.
template <class S, int R>
struct Geo {
    static constexpr int HX = 16 / (int)sizeof(S);
    static constexpr int BW = TXC + 2 * HX;
    static constexpr int BH = TY + 2 * R;
    static constexpr int X_B = BW * TY * (int)sizeof(S);
    static constexpr int Y_B = TXC * BH * (int)sizeof(S);
    static constexpr int XY_B = BW * BH * (int)sizeof(S);
    static constexpr int OWN_B = TXC * TY * (int)sizeof(S);
    static constexpr int KOWN_B = TXC * TY * (int)sizeof(typename Traits<S>::K);
    static constexpr int WOWN_B = TXC * TY * 4;  // FP32 Darcy factor
};

constexpr int al128(int b) { return (b + 127) & ~127; }

struct VMaps {
    CUtensorMap halo[6];  // txx(X) tyy(Y) txy(XY) txz(X) tyz(Y) p(XY)
    CUtensorMap zlead[4]; // tzz txz tyz p: own-cell boxes for the z ring
    // own-cell boxes of the warp-specialised kernel: vx vy vz qx qy qz, VW1 x y z (FP32), then VW3, VU1, VU2
    // (x y z each)
    CUtensorMap own[18];
    CUtensorMap xs[8];    // x-slab CPML memory of slots 0..3 (psi 0..3, then prev 0..3): boxes xs_bw x TY x 1
    CUtensorMap xp[4];    // x damping profiles A, B, A2, B2: 1-D boxes of TXC
    CUtensorMap ys[8], zs[8];  // y- and z-slab CPML memory of slots 0..3 (L2 prefetch): boxes TXC x TY x 1
};
struct TMaps {
    CUtensorMap halo[5];  // vx vy vz (XY) qx (X) qy (Y)
    CUtensorMap zlead[4]; // vx vy vz qz: own-cell boxes for the z ring
    CUtensorMap own[14];  // sxx syy szz sxy sxz syz p, then P1 P2 S1 S2 Sxy Sxz Syz
    CUtensorMap xs[8];    // x-slab CPML memory of slots 4..7 (psi, then prev)
    CUtensorMap xp[4];    // x damping profiles A, B, A2, B2
    CUtensorMap ys[8], zs[8];  // y- and z-slab CPML memory of slots 4..7 (L2 prefetch)
};

// ------------------------------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// try_wait with a suspend-time hint: the hardware parks the waiting warp (up to `ns` nanoseconds) instead of
// letting it spin, so waiting warps do not take issue slots from the warps that compute.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity, uint32_t ns) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
        : "memory");
    return ok != 0;
}
// Bounded wait: false once kSpinLimit cycles have passed (the clock is read every 256 polls).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity, 1000000u)) return true;
    const long long t0 = clock64();
    for (unsigned n = 1;; n++) {
        if (mbar_try_wait(bar, parity, 1000000u)) return true;
        if ((n & 255u) == 0 && clock64() - t0 > kSpinLimit) return false;
    }
}
__device__ __forceinline__ void tma3(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}
// L2 prefetch of one box (no shared memory, no barrier; out-of-range parts are skipped).
__device__ __forceinline__ void tma3_prefetch(const CUtensorMap* map, int x, int y, int z) {
    asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(z)
                 : "memory");
}
__device__ __forceinline__ void tma1(void* dst, const CUtensorMap* map, uint64_t* bar, int x) {
    asm volatile(
        "cp.async.bulk.tensor.1d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3}], [%2];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x)
        : "memory");
}
__device__ __forceinline__ void fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// ------------------------------------------------------------------------------------- pair math
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

template <int R>
__device__ __forceinline__ float wgt(int m) {
    return (float)stencil_w<R>(m);
}

// Window of 2*RA+2 values around the pair (x, x+1), RA = R rounded up to even: w[d + RA] = f[x + d].
template <class S, int R>
struct XWin {
    static constexpr int RA = (R + 1) & ~1;
    float w[2 * RA + 2];
    __device__ __forceinline__ void load(const S* rowp) {  // rowp points at f[x] in smem (x even)
        typedef typename Pair<S>::T P;
#pragma unroll
        for (int u = 0; u <= RA; u++) {
            const float2 v = Pair<S>::f2(*reinterpret_cast<const P*>(rowp - RA + 2 * u));
            w[2 * u] = v.x;
            w[2 * u + 1] = v.y;
        }
    }
    // forward (at x+1/2): sum_m c_m (f[x+m] - f[x-m+1]) for both cells
    __device__ __forceinline__ float2 fwd() const {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int m = 1; m <= R; m++) {
            const float c = wgt<R>(m);
            acc = fma2(f2(c, c), f2(w[RA + m], w[RA + m + 1]), acc);
            acc = fma2(f2(-c, -c), f2(w[RA - m + 1], w[RA - m + 2]), acc);
        }
        return acc;
    }
    // backward (at x): sum_m c_m (f[x+m-1] - f[x-m])
    __device__ __forceinline__ float2 bwd() const {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int m = 1; m <= R; m++) {
            const float c = wgt<R>(m);
            acc = fma2(f2(c, c), f2(w[RA + m - 1], w[RA + m]), acc);
            acc = fma2(f2(-c, -c), f2(w[RA - m], w[RA - m + 1]), acc);
        }
        return acc;
    }
};

// Column of 2R+1 pairs: v[R + d] = pair at offset d (rows in y, or planes in z).
template <int R>
__device__ __forceinline__ float2 col_fwd(const float2* v) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int m = 1; m <= R; m++) {
        const float c = wgt<R>(m);
        acc = fma2(f2(c, c), v[R + m], acc);
        acc = fma2(f2(-c, -c), v[R - m + 1], acc);
    }
    return acc;
}
template <int R>
__device__ __forceinline__ float2 col_bwd(const float2* v) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int m = 1; m <= R; m++) {
        const float c = wgt<R>(m);
        acc = fma2(f2(c, c), v[R + m - 1], acc);
        acc = fma2(f2(-c, -c), v[R - m], acc);
    }
    return acc;
}

template <class S, int R>
__device__ __forceinline__ void load_col(float2* v, const S* p, int stride) {  // p at row/plane 0 of the pair
    typedef typename Pair<S>::T P;
#pragma unroll
    for (int d = -R; d <= R; d++) v[R + d] = Pair<S>::f2(*reinterpret_cast<const P*>(p + d * stride));
}

// ------------------------------------------------------------------------------------- tensor maps (host)
inline PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

template <class T> inline CUtensorMapDataType dtype_of();
template <> inline CUtensorMapDataType dtype_of<__half>() { return CU_TENSOR_MAP_DATA_TYPE_FLOAT16; }
template <> inline CUtensorMapDataType dtype_of<__nv_bfloat16>() { return CU_TENSOR_MAP_DATA_TYPE_BFLOAT16; }
template <> inline CUtensorMapDataType dtype_of<float>() { return CU_TENSOR_MAP_DATA_TYPE_FLOAT32; }
template <> inline CUtensorMapDataType dtype_of<double>() { return CU_TENSOR_MAP_DATA_TYPE_FLOAT64; }

// 3-D map over a pitched [nz][ny][px] array of T (logical extent nx), box bw x bh x 1.
template <class T>
inline bool encode(CUtensorMap* m, const Geom& g, void* base, int bw, int bh) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)(g.px * sizeof(T)), (cuuint64_t)(g.plane * sizeof(T))};
    const cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(m, dtype_of<T>(), 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 3-D map over one x-slab CPML memory array ([nz][ny][W] FP32, W a multiple of 4), box bw x TY x 1.
inline bool encode_xslab(CUtensorMap* m, const Geom& g, void* base, int bw) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.W, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)g.W * 4, (cuuint64_t)g.W * g.ny * 4};
    const cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)TY, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 3-D map over an FP32 array of dims (d0, d1, d2) (innermost first; d0 a multiple of 4), box TXC x TY x 1: the y-
// ([nz][W][nx]: nx, W, nz) and z-slab ([W][ny][nx]: nx, ny, W) CPML memory, for L2 prefetches of a tile's rows.
inline bool encode_slab(CUtensorMap* m, void* base, int d0, int d1, int d2) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
    const cuuint64_t strides[2] = {(cuuint64_t)d0 * 4, (cuuint64_t)d0 * d1 * 4};
    const cuuint32_t box[3] = {(cuuint32_t)TXC, (cuuint32_t)TY, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 1-D map over an FP32 array of n values (a damping profile), boxes of TXC; beyond n the box reads zeros.
inline bool encode_prof(CUtensorMap* m, int n, void* base) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[1] = {(cuuint64_t)n};
    const cuuint64_t strides[1] = {4};  // unused for rank 1
    const cuuint32_t box[1] = {(cuuint32_t)TXC};
    const cuuint32_t es[1] = {1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 1, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The tile's box of x-slab CPML memory (tensor-memory kernels): the first slab index it starts at, or -1 when the
// tile updates no x-slab cell, updates cells of both slabs, or its slab cells do not fit a box of g.xs_bw
// starting at a multiple of 4 (16 bytes, the TMA rule for the innermost coordinate).  CTA-uniform.
__host__ __device__ __forceinline__ int xs_tile_base(const Geom& g, int x0) {
    if (g.xs_bw <= 0 || g.W <= 0) return -1;
    const int lo = x0 > g.R ? x0 : g.R;
    const int hi = x0 + TXC < g.nx - g.R ? x0 + TXC : g.nx - g.R;  // updated cells [lo, hi)
    if (lo >= hi) return -1;
    const int r0 = g.nx - 1 - g.L;  // first cell of the upper slab (slab index L)
    const bool left = lo < g.L, right = hi > r0;
    if (left == right) return -1;
    const int s_lo = left ? lo : g.L + ((lo > r0 ? lo : r0) - r0);
    const int s_hi = left ? (hi < g.L ? hi : g.L) : g.L + (hi - r0);
    const int base = s_lo & ~3;
    return s_hi - base <= g.xs_bw ? base : -1;
}

// Trapezoidal CPML memory update of one cell: psi = A psi + B (A prev + D); prev = D; returns D + psi.
__device__ __forceinline__ float pml1(float D, float* psi, float* prv, float A, float B) {
    const float pn = A * (*psi) + B * (A * (*prv) + D);
    *psi = pn;
    *prv = D;
    return D + pn;
}

}  // namespace BEHF_TILED_NAMESPACE
}  // namespace behf
