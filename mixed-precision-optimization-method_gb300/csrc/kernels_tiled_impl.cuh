// kernels_tiled_impl.cuh -- bodies of the z-marching kernels (included once per storage precision by
// kernels_tiled_{f16,bf16,f32}.cu so the three instantiations compile in parallel).
#pragma once
#include "kernels_tiled.cuh"

namespace behf {
namespace BEHF_TILED_NAMESPACE {

// Pipeline depth: NS stages in the shared-memory ring (NS - 1 planes in flight while one is computed), and
// the CTAs per SM the launch bounds aim for (registers capped at 65536 / (256 MINB)).
#ifndef BEHF_TILED_NS16
#define BEHF_TILED_NS16 2
#endif
// 16-bit kinds run 3 CTAs per SM (80 registers: 6 warps per scheduler instead of 4; measured at 1024^3 FP16
// stress 17.5 -> 16.2 ms, velocity 18.35 -> 17.8 ms with its own-cell loads issued after the stencils).
#ifndef BEHF_TILED_MINB16_T
#define BEHF_TILED_MINB16_T 3
#endif
#ifndef BEHF_TILED_MINB16
#define BEHF_TILED_MINB16 3
#endif
#ifndef BEHF_TILED_NS32
#define BEHF_TILED_NS32 2
#endif
#ifndef BEHF_TILED_MINB32
#define BEHF_TILED_MINB32 1
#endif
// Velocity kernel, 16-bit kinds: the groups of the cell's own loads issued before the pipeline waits (their latency
// overlaps the waits, but their registers stay live through the stencils), the rest after the stencils: a mask of
// 1 = v and q, 2 = VW1 (FP32), 4 = VW3, VU1, VU2.  0 (all after) fits 80 registers; 7 spills at 3 CTAs per SM.
// Measured at 1024^3 FP16 on one GPU: 0 17.79 ms, 1 19.52, 2 18.56, 4 18.42.  FP32 (1 CTA per SM) always issues
// them early.
#ifndef BEHF_TILED_VLOAD_EARLY16
#define BEHF_TILED_VLOAD_EARLY16 0
#endif
// Stress kernel, 16-bit kinds: the cell's own stresses/pressure and coefficients are loaded 0 before the pipeline
// waits, 1 after the stencils, 2 fields before and coefficients after (1024^3 FP16, one GPU: 16.18, 17.67 and
// 17.85 ms; all three at 80 registers without spills).  FP32 always loads them early.
#ifndef BEHF_TILED_SLOAD16
#define BEHF_TILED_SLOAD16 0
#endif
// At least this many waves of resident CTAs where 16-plane z ranges allow it.
#ifndef BEHF_TILED_MINW
#define BEHF_TILED_MINW 4
#endif
// Longest z range a CTA marches by default (BEHF_OPT_ZCHUNK overrides it).
#ifndef BEHF_TILED_ZCHUNK
#define BEHF_TILED_ZCHUNK 64
#endif
template <class S> struct Depth {
    static constexpr int NS = sizeof(S) == 2 ? BEHF_TILED_NS16 : BEHF_TILED_NS32;
    static constexpr int MINB = sizeof(S) == 2 ? BEHF_TILED_MINB16 : BEHF_TILED_MINB32;
    static constexpr int MINB_T = sizeof(S) == 2 ? BEHF_TILED_MINB16_T : BEHF_TILED_MINB32;
};
constexpr int NWARP = NTH / 32;

// Shared-memory map of one CTA.  NS stages holding the halo boxes of plane k, then the z ring: for each of
// the four fields with a z-derivative, ZS = 2R + NS own-cell boxes holding plane z at slot z % ZS (the window
// k-R..k+R of the plane being computed plus the planes the producer has already requested).  A cell's own
// fields and coefficients are read by its thread straight from global memory (coalesced pair loads issued
// before the stencil work), so only data shared between threads goes through shared memory.
//   velocity stage: txx(X) tyy(Y) txy(XY) txz(X) tyz(Y) p(XY);  ring: tzz txz tyz p
//   stress stage:   vx vy vz (XY) qx (X) qy (Y);                ring: vx vy vz qz
template <class S, int R, bool VEL>
struct Map {
    typedef Geo<S, R> G;
    static constexpr int NS = Depth<S>::NS;
    static constexpr int ZS = 2 * R + NS;
    static constexpr int X = al128(G::X_B), Y = al128(G::Y_B), XY = al128(G::XY_B), OW = al128(G::OWN_B);
    __host__ __device__ static constexpr int halo(int i) {
        return VEL ? (i == 0 ? 0 : i == 1 ? X : i == 2 ? X + Y : i == 3 ? X + Y + XY : i == 4 ? 2 * X + Y + XY
                                                                                       : 2 * X + 2 * Y + XY)
                   : (i < 3 ? i * XY : i == 3 ? 3 * XY : 3 * XY + X);
    }
    static constexpr int stage = VEL ? 2 * X + 2 * Y + 2 * XY : 3 * XY + X + Y;
    static constexpr int ring = NS * stage;            // z ring: [field][slot] boxes of OW bytes
    static constexpr int bytes = ring + 4 * ZS * OW;
    static constexpr uint32_t stage_tx = VEL ? 2 * (G::X_B + G::Y_B + G::XY_B) : 3 * G::XY_B + G::X_B + G::Y_B;
};

__device__ __forceinline__ float comp(float2 v, int c) { return c ? v.y : v.x; }
__device__ __forceinline__ void setc(float2& v, int c, float x) {
    if (c) v.y = x;
    else v.x = x;
}
__device__ __forceinline__ float prof(const void* a, int i) { return reinterpret_cast<const float*>(a)[i]; }


// CPML of the four derivatives of one axis for one cell: all eight loads first, then the updates, then the
// eight stores (the arrays cannot alias, but the compiler cannot know; batching keeps one memory latency).
__device__ __forceinline__ void pml4(const DevPtrs& p, int ax, int slot0, long long so, float A, float B, float A2,
                                     float B2, float& d0, float& d1, float& d2, float& d3, bool half0, bool half1,
                                     bool half2, bool half3) {
    float* ps[4];
    float* pv[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        ps[j] = reinterpret_cast<float*>(p.psi[ax][slot0 + j]) + so;
        pv[j] = reinterpret_cast<float*>(p.prv[ax][slot0 + j]) + so;
    }
    float s[4], v[4];
    // read-only-path loads: a slab element is read once, before the same thread writes it, in a launch, so the
    // non-coherent path is exact, and it lets the compiler start the next cell's loads before this cell's stores
#pragma unroll
    for (int j = 0; j < 4; j++) {
        s[j] = __ldg(ps[j]);
        v[j] = __ldg(pv[j]);
    }
    float* d[4] = {&d0, &d1, &d2, &d3};
    const bool h[4] = {half0, half1, half2, half3};
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float a = h[j] ? A2 : A, b = h[j] ? B2 : B;
        const float D = *d[j];
        const float pn = a * s[j] + b * (a * v[j] + D);  // psi = A psi + B (A prev + D)
        s[j] = pn;
        v[j] = D;
        *d[j] = D + pn;
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        *ps[j] = s[j];
        *pv[j] = v[j];
    }
}

// CPML for the pair: x per cell, y per row (warp-uniform), z per plane (CTA-uniform).  Slots 0..3 of the
// velocity kernel / 4..7 of the stress kernel; `half` flags mark forward (half-shifted) derivatives.  PAIRED: the
// two cells' memory loads of an axis batched (pml4x2: one memory latency per axis); else cell by cell (pml4: fewer
// live registers, for kernels at their register limit); XS (cell by cell only): the x-slab memory and the x
// profiles read from shared memory, xrow being this warp's row of a TMA box that starts at slab index xbase (arrays
// xplane floats apart) and xprof the pair's entry in the tile's profile boxes (A, B, A2, B2, TXC floats apart).
// All forms give the same bits.
// The same with the cell's memory already in shared memory (psi of the four slots, then prev, sp floats apart):
// one derivative at a time, since a shared-memory load needs no batching, so that few registers stay live.
__device__ __forceinline__ void pml4_sm(const DevPtrs& p, int ax, int slot0, long long so, const float* sm, int sp,
                                        float A, float B, float A2, float B2, float& d0, float& d1, float& d2,
                                        float& d3, bool half0, bool half1, bool half2, bool half3) {
    float* d[4] = {&d0, &d1, &d2, &d3};
    const bool h[4] = {half0, half1, half2, half3};
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float a = h[j] ? A2 : A, b = h[j] ? B2 : B;
        const float D = *d[j];
        const float pn = a * sm[j * sp] + b * (a * sm[(4 + j) * sp] + D);  // psi = A psi + B (A prev + D)
        reinterpret_cast<float*>(p.psi[ax][slot0 + j])[so] = pn;
        reinterpret_cast<float*>(p.prv[ax][slot0 + j])[so] = D;
        *d[j] = D + pn;
    }
}

// CPML of the four derivatives of one axis for both cells of a pair (in[c]: cell c lies in the slab, at element
// so[c] of the axis' memory arrays): all sixteen loads first, then the updates, then the stores.  The arrays cannot
// alias, but the compiler cannot know; batching the pair's loads keeps one memory latency per axis instead of one
// per cell.
__device__ __forceinline__ void pml4x2(const DevPtrs& p, int ax, int slot0, const long long (&so)[2],
                                       const bool (&in)[2], float2 A, float2 B, float2 A2, float2 B2, float2& d0,
                                       float2& d1, float2& d2, float2& d3, bool half0, bool half1, bool half2,
                                       bool half3) {
    float s[2][4], v[2][4];
#pragma unroll
    for (int c = 0; c < 2; c++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            s[c][j] = in[c] ? reinterpret_cast<const float*>(p.psi[ax][slot0 + j])[so[c]] : 0.f;
            v[c][j] = in[c] ? reinterpret_cast<const float*>(p.prv[ax][slot0 + j])[so[c]] : 0.f;
        }
    float2* d[4] = {&d0, &d1, &d2, &d3};
    const bool h[4] = {half0, half1, half2, half3};
#pragma unroll
    for (int c = 0; c < 2; c++) {
        if (!in[c]) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float a = h[j] ? comp(A2, c) : comp(A, c), b = h[j] ? comp(B2, c) : comp(B, c);
            const float D = comp(*d[j], c);
            const float pn = a * s[c][j] + b * (a * v[c][j] + D);  // psi = A psi + B (A prev + D)
            s[c][j] = pn;
            v[c][j] = D;
            setc(*d[j], c, D + pn);
        }
    }
#pragma unroll
    for (int c = 0; c < 2; c++) {
        if (!in[c]) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            reinterpret_cast<float*>(p.psi[ax][slot0 + j])[so[c]] = s[c][j];
            reinterpret_cast<float*>(p.prv[ax][slot0 + j])[so[c]] = v[c][j];
        }
    }
}
// CPML for the pair: x per cell, y per row (warp-uniform), z per plane (CTA-uniform).  Slots 0..3 of the
// velocity kernel / 4..7 of the stress kernel; `half` flags mark forward (half-shifted) derivatives.  PAIRED: the
// x slab's two cells batched (pml4x2: one memory latency instead of two); else cell by cell (pml4: fewer live
// registers), or XS: the x-slab memory and the x profiles read from shared memory, xrow being this warp's row of a
// TMA box that starts at slab index xbase (arrays xplane floats apart) and xprof the pair's entry in the tile's
// profile boxes (A, B, A2, B2, TXC floats apart).  PAIRYZ: the y and z slabs' two cells batched likewise.  All
// forms give the same bits.
template <int SLOT0, bool PAIRED, bool XS = false, bool PAIRYZ = PAIRED>
__device__ __forceinline__ void pml_pair(const Geom& g, const DevPtrs& p, int x, int y, int k, bool a0, bool a1,
                                         float2& dx0, float2& dx1, float2& dx2, float2& dx3, const bool hx[4],
                                         float2& dy0, float2& dy1, float2& dy2, float2& dy3, const bool hy[4],
                                         float2& dz0, float2& dz1, float2& dz2, float2& dz3, const bool hz[4],
                                         const float* xrow = nullptr, int xbase = 0, int xplane = 0,
                                         const float* xprof = nullptr) {
    if constexpr (PAIRED) {
        const int si0 = a0 ? slab_index(x, g.nx, g.L) : -1, si1 = a1 ? slab_index(x + 1, g.nx, g.L) : -1;
        if (si0 >= 0 || si1 >= 0) {
            const bool in[2] = {si0 >= 0, si1 >= 0};
            const long long row = ((long long)k * g.ny + y) * g.W;
            const long long so[2] = {row + si0, row + si1};
            auto pr = [&](void* const* t) {
                return f2(in[0] ? prof(t[0], x) : 0.f, in[1] ? prof(t[0], x + 1) : 0.f);
            };
            pml4x2(p, 0, SLOT0, so, in, pr(p.pa), pr(p.pb), pr(p.pa2), pr(p.pb2), dx0, dx1, dx2, dx3, hx[0], hx[1],
                   hx[2], hx[3]);
        }
    } else {
#pragma unroll
        for (int c = 0; c < 2; c++) {
            const int xc = x + c;
            const int si = (c ? a1 : a0) ? slab_index(xc, g.nx, g.L) : -1;
            if (si >= 0) {
                const long long so = ((long long)k * g.ny + y) * g.W + si;
                float a = comp(dx0, c), b = comp(dx1, c), d = comp(dx2, c), e = comp(dx3, c);
                if constexpr (XS)
                    pml4_sm(p, 0, SLOT0, so, xrow + (si - xbase), xplane, xprof[c], xprof[TXC + c],
                            xprof[2 * TXC + c], xprof[3 * TXC + c], a, b, d, e, hx[0], hx[1], hx[2], hx[3]);
                else
                    pml4(p, 0, SLOT0, so, prof(p.pa[0], xc), prof(p.pb[0], xc), prof(p.pa2[0], xc), prof(p.pb2[0], xc),
                         a, b, d, e, hx[0], hx[1], hx[2], hx[3]);
                setc(dx0, c, a);
                setc(dx1, c, b);
                setc(dx2, c, d);
                setc(dx3, c, e);
            }
        }
    }
    // y (slab index sj, memory [nz][W][nx]) and z (sk, [W][ny][nx]): both cells share the profiles
    auto yz = [&](int ax, long long base, float2& e0, float2& e1, float2& e2, float2& e3, const bool hh[4]) {
        const int pos = ax == 1 ? y : k;
        const float A = prof(p.pa[ax], pos), B = prof(p.pb[ax], pos), A2 = prof(p.pa2[ax], pos),
                    B2 = prof(p.pb2[ax], pos);
        if constexpr (PAIRYZ) {
            const bool in[2] = {a0, a1};
            const long long so[2] = {base, base + 1};
            pml4x2(p, ax, SLOT0, so, in, f2(A, A), f2(B, B), f2(A2, A2), f2(B2, B2), e0, e1, e2, e3, hh[0], hh[1],
                   hh[2], hh[3]);
        } else {
#pragma unroll
            for (int c = 0; c < 2; c++) {
                if (!(c ? a1 : a0)) continue;
                float a = comp(e0, c), b = comp(e1, c), d = comp(e2, c), e = comp(e3, c);
                pml4(p, ax, SLOT0, base + c, A, B, A2, B2, a, b, d, e, hh[0], hh[1], hh[2], hh[3]);
                setc(e0, c, a);
                setc(e1, c, b);
                setc(e2, c, d);
                setc(e3, c, e);
            }
        }
    };
    const int sj = slab_index(y, g.ny, g.L);
    if (sj >= 0) yz(1, ((long long)k * g.W + sj) * g.nx + x, dy0, dy1, dy2, dy3, hy);
    const int sk = slab_index(k, g.nz, g.L);
    if (sk >= 0) yz(2, ((long long)sk * g.ny + y) * g.nx + x, dz0, dz1, dz2, dz3, hz);
}

// Store a pair, or the one active cell of it.
template <class S>
__device__ __forceinline__ void store_pair(S* dst, typename Pair<S>::T v, bool a0, bool a1) {
    if (a0 && a1) {
        *reinterpret_cast<typename Pair<S>::T*>(dst) = v;
    } else {
        const float2 f = Pair<S>::f2(v);
        if (a0) dst[0] = Pair<S>::one(f.x);
        if (a1) dst[1] = Pair<S>::one(f.y);
    }
}

// Single-producer pipeline: thread 0 issues every TMA; each warp releases a stage after reading it (one
// arrival per warp on empty[s]); the producer refills a stage only after all eight warps released it.
// Waits are bounded; phase bits track the parity of each barrier's next completion.
template <int NS>
struct Pipe {
    uint64_t* full;
    uint64_t* empty;
    uint32_t fph = 0, eph = 0;
    int pend[NS];  // producer: issued but not yet consumed by thread 0 (for the drain on error)
};

template <class M, class Issue>
__device__ __forceinline__ bool producer_step(Pipe<M::NS>& pp, int it, int k, int kb, int ke, Issue&& issue) {
    constexpr int NS = M::NS;
    if (k + NS - 1 >= ke) return true;
    const int sp = (it + NS - 1) % NS;
    if (it >= 1) {  // the stage was used by step it-1: wait until every warp released it
        if (!mbar_wait(&pp.empty[sp], (pp.eph >> sp) & 1u)) return false;
        pp.eph ^= 1u << sp;
    }
    fence_async();
    issue(sp, k + NS - 1, k + NS - 1 == kb);  // the first plane also brings the z-ring warm-up
    pp.pend[sp]++;
    return true;
}

template <class M>
__device__ __forceinline__ void producer_drain(Pipe<M::NS>& pp) {
#pragma unroll
    for (int s = 0; s < M::NS; s++)
        for (int n = 0; n < pp.pend[s]; n++) {
            mbar_wait(&pp.full[s], (pp.fph >> s) & 1u);
            pp.fph ^= 1u << s;
        }
}

// Byte offsets of the z-ring slots of planes k-R .. k+R (shared by the four fields).
template <class M, int R>
__device__ __forceinline__ void ring_slots(int k, int* off) {
    int s = (k - R) % M::ZS;
#pragma unroll
    for (int d = 0; d <= 2 * R; d++) {
        off[d] = s * M::OW;
        s = (s + 1 == M::ZS) ? 0 : s + 1;
    }
}

// ----------------------------------------------------------------------------------------- velocity
template <class S, int R>
__global__ void __launch_bounds__(NTH, Depth<S>::MINB)
    k_vel(const __grid_constant__ VMaps maps, const Geom g, const DevPtrs p, const int zchunk) {
    typedef Pair<S> PS;
    typedef typename PS::T P;
    typedef typename Traits<S>::K K;
    typedef typename Pair<K>::T KP;
    typedef Geo<S, R> G;
    typedef Map<S, R, true> M;
    constexpr int NS = M::NS;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bfull[NS], bempty[NS];
    // TMA destinations start on 128-byte boundaries: round the dynamic base up (128 B are reserved for it)
    unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);

    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int x0 = blockIdx.x * TXC, y0 = blockIdx.y * TY;
    const int kb = R + blockIdx.z * zchunk;
    const int ke = min(kb + zchunk, g.nz - R);
    if (kb >= ke) return;
    const int xl = 2 * tx, x = x0 + xl, y = y0 + ty;
    const bool a0 = x >= R && x < g.nx - R, a1 = x + 1 >= R && x + 1 < g.nx - R;
    const bool live = (y >= R && y < g.ny - R) && (a0 || a1);
    const long long col = (long long)y * g.px + x;
    const int oe = ty * TXC + xl;  // element offset of the pair in an own-cell box
    // stochastic-rounding seed of this step (velocity and stress draw different bits)
    const uint32_t seed = g.sr ? mix32((uint32_t)(*g.step + g.step_off) * 0x9e3779b9u + 0x2545f491u) : 0u;

    if (tid == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&bfull[s], 1);
            mbar_init(&bempty[s], NWARP);
        }
        fence_init();
    }
    __syncthreads();

    // z ring fields: tzz (forward), txz (backward), tyz (backward), p (forward)
    auto issue = [&](int st, int k, bool warm) {
        unsigned char* b = smem + st * M::stage;
        uint64_t* br = &bfull[st];
        mbar_expect_tx(br, M::stage_tx + 4 * G::OWN_B * (warm ? 2 * R + 1 : 1));
        tma3(b + M::halo(0), &maps.halo[0], br, x0 - G::HX, y0, k);      // txx  (x halo)
        tma3(b + M::halo(1), &maps.halo[1], br, x0, y0 - R, k);          // tyy  (y halo)
        tma3(b + M::halo(2), &maps.halo[2], br, x0 - G::HX, y0 - R, k);  // txy  (x, y halo)
        tma3(b + M::halo(3), &maps.halo[3], br, x0 - G::HX, y0, k);      // txz  (x halo)
        tma3(b + M::halo(4), &maps.halo[4], br, x0, y0 - R, k);          // tyz  (y halo)
        tma3(b + M::halo(5), &maps.halo[5], br, x0 - G::HX, y0 - R, k);  // p    (x, y halo)
        const int z0 = warm ? k - R : k + R;
        for (int z = z0; z <= k + R; z++)
#pragma unroll
            for (int f = 0; f < 4; f++)
                tma3(smem + M::ring + (f * M::ZS + z % M::ZS) * M::OW, &maps.zlead[f], br, x0, y0, z);
    };

    Pipe<NS> pp{bfull, bempty};
    for (int s = 0; s < NS; s++) pp.pend[s] = 0;
    if (tid == 0)
        for (int j = 0; j < NS - 1 && kb + j < ke; j++) {
            issue(j, kb + j, j == 0);
            pp.pend[j]++;
        }
    bool failed = false;
    for (int k = kb, it = 0; k < ke; k++, it++) {
        const int st = it % NS;
        // the cell's own data of plane k (v, q, VW1 in FP32, VW3, VU1, VU2) does not go through the pipeline: its
        // coalesced pair loads are issued before the waits (FP32) or after the stencils (16-bit kinds)
        const long long go = (long long)k * g.plane + col;
        P vo_s[3], qo_s[3];
        float2 vw1[3];
        KP kw3[3], ku1[3], ku2[3];
        // groups: 1 = v, q; 2 = VW1; 4 = VW3, VU1, VU2
        auto load_own = [&](int groups) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (groups & 1) {
                    vo_s[a] = *reinterpret_cast<const P*>(reinterpret_cast<const S*>(p.f[BEHF_VX + a]) + go);
                    qo_s[a] = *reinterpret_cast<const P*>(reinterpret_cast<const S*>(p.f[BEHF_QX + a]) + go);
                }
                if (groups & 2)
                    vw1[a] = *reinterpret_cast<const float2*>(reinterpret_cast<const float*>(p.k[VW1X + a]) + go);
                if (groups & 4) {
                    kw3[a] = *reinterpret_cast<const KP*>(reinterpret_cast<const K*>(p.k[VW3X + a]) + go);
                    ku1[a] = *reinterpret_cast<const KP*>(reinterpret_cast<const K*>(p.k[VU1X + a]) + go);
                    ku2[a] = *reinterpret_cast<const KP*>(reinterpret_cast<const K*>(p.k[VU2X + a]) + go);
                }
            }
        };
        constexpr int early = sizeof(S) == 4 ? 7 : BEHF_TILED_VLOAD_EARLY16;
        if (early && live) load_own(early);
        bool ok = true;
        if (tid == 0) ok = producer_step<M>(pp, it, k, kb, ke, issue);
        if (ok) ok = mbar_wait(&bfull[st], (pp.fph >> st) & 1u);
        if (!__all_sync(0xffffffffu, ok)) {  // warp-uniform exit: every lane leaves together
            failed = true;
            break;
        }
        pp.fph ^= 1u << st;
        if (tid == 0) pp.pend[st]--;
        const unsigned char* b = smem + st * M::stage;
        if (live) {
            const S* txx = reinterpret_cast<const S*>(b + M::halo(0));
            const S* tyy = reinterpret_cast<const S*>(b + M::halo(1));
            const S* txy = reinterpret_cast<const S*>(b + M::halo(2));
            const S* txz = reinterpret_cast<const S*>(b + M::halo(3));
            const S* tyz = reinterpret_cast<const S*>(b + M::halo(4));
            const S* pp_ = reinterpret_cast<const S*>(b + M::halo(5));
            const int rX = ty * G::BW + G::HX + xl;          // X box: row ty
            const int rXY = (ty + R) * G::BW + G::HX + xl;   // XY box: row ty + R
            const int rY = (ty + R) * TXC + xl;              // Y box: row ty + R
            XWin<S, R> w;
            w.load(txx + rX);
            float2 x1 = w.fwd();
            w.load(pp_ + rXY);
            float2 s1 = w.fwd();
            w.load(txy + rXY);
            float2 y2 = w.bwd();
            w.load(txz + rX);
            float2 z2 = w.bwd();
            float2 cv[2 * R + 1];
            load_col<S, R>(cv, tyy + rY, TXC);
            float2 y1 = col_fwd<R>(cv);
            load_col<S, R>(cv, pp_ + rXY, G::BW);
            float2 s2 = col_fwd<R>(cv);
            load_col<S, R>(cv, txy + rXY, G::BW);
            float2 x2 = col_bwd<R>(cv);
            load_col<S, R>(cv, tyz + rY, TXC);
            float2 z3 = col_bwd<R>(cv);
            int zo[2 * R + 1];
            ring_slots<M, R>(k, zo);
            auto zcol = [&](int f) {
                const unsigned char* rb = smem + M::ring + f * M::ZS * M::OW + oe * sizeof(S);
#pragma unroll
                for (int d = 0; d <= 2 * R; d++) cv[d] = PS::f2(*reinterpret_cast<const P*>(rb + zo[d]));
            };
            zcol(0);
            float2 z1 = col_fwd<R>(cv);
            zcol(3);
            float2 s3 = col_fwd<R>(cv);
            zcol(1);
            float2 x3 = col_bwd<R>(cv);
            zcol(2);
            float2 y3 = col_bwd<R>(cv);

            if (g.W > 0) {
                // x: x1 (fwd), s1 (fwd), y2 (bwd), z2 (bwd); y: y1, s2 (fwd), x2, z3 (bwd);
                // z: z1, s3 (fwd), x3, y3 (bwd)
                const bool hf[4] = {true, true, false, false};
                pml_pair<0, sizeof(S) == 4>(g, p, x, y, k, a0, a1, x1, s1, y2, z2, hf, y1, s2, x2, z3, hf, z1, s3, x3, y3, hf);
            }
            const float2 sum[3] = {add2(add2(x1, x2), x3), add2(add2(y1, y2), y3), add2(add2(z1, z2), z3)};
            const float2 dp[3] = {s1, s2, s3};
            if (early != 7) load_own(7 & ~early);
            auto km = [&](KP kv, int j) { return mul2(Pair<K>::f2(kv), f2(g.kmulf[j], g.kmulf[j])); };
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float2 vw3 = km(kw3[a], VW3X + a);
                const float2 vu1 = km(ku1[a], VU1X + a), vu2 = km(ku2[a], VU2X + a);
                const float2 vw2 = mul2(mul2(vu2, vw3), f2(g.c_vw2, g.c_vw2));
                const float2 vw3p = (a == 2 && g.bug) ? km(kw3[1], VW3Y) : vw3;  // reference: vz uses VW3y
                const float2 qo = PS::f2(qo_s[a]);
                // q' = VW1 q - VW2 sum(d sigma) - VW3 d p
                const float2 t = fma2(vw2, sum[a], mul2(vw3p, dp[a]));
                const float2 qn = fma2(vw1[a], qo, make_float2(-t.x, -t.y));
                const P qs = g.sr ? SR<S>::pack(qn, mix32(seed ^ (uint32_t)go ^ (0x3c6ef372u * (uint32_t)(a + 1))))
                                  : PS::pack(qn);
                store_pair<S>(reinterpret_cast<S*>(p.f[BEHF_QX + a]) + go, qs, a0, a1);
                // v' = v + VU1 sum(d sigma) - VU2 (q' - q)
                const float2 dq = sub2(PS::f2(qs), qo);
                const float2 vn = fma2(vu1, sum[a], fma2(make_float2(-vu2.x, -vu2.y), dq, PS::f2(vo_s[a])));
                const P vs = g.sr ? SR<S>::pack(vn, mix32(seed ^ (uint32_t)go ^ (0x1b873593u * (uint32_t)(a + 1))))
                                  : PS::pack(vn);
                store_pair<S>(reinterpret_cast<S*>(p.f[BEHF_VX + a]) + go, vs, a0, a1);
            }
        }
        __syncwarp();
        if (tx == 0) mbar_arrive(&bempty[st]);
    }
    if (failed) atomicExch(g.err, 1);
    if (tid == 0) producer_drain<M>(pp);
}

// ----------------------------------------------------------------------------------------- stress
template <class S, int R>
__global__ void __launch_bounds__(NTH, Depth<S>::MINB_T)
    k_str(const __grid_constant__ TMaps maps, const Geom g, const DevPtrs p, const int zchunk) {
    typedef Pair<S> PS;
    typedef typename PS::T P;
    typedef typename Traits<S>::K K;
    typedef typename Pair<K>::T KP;
    typedef Geo<S, R> G;
    typedef Map<S, R, false> M;
    constexpr int NS = M::NS;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bfull[NS], bempty[NS];
    unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);

    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int x0 = blockIdx.x * TXC, y0 = blockIdx.y * TY;
    const int kb = R + blockIdx.z * zchunk;
    const int ke = min(kb + zchunk, g.nz - R);
    if (kb >= ke) return;
    const int xl = 2 * tx, x = x0 + xl, y = y0 + ty;
    const bool a0 = x >= R && x < g.nx - R, a1 = x + 1 >= R && x + 1 < g.nx - R;
    const bool live = (y >= R && y < g.ny - R) && (a0 || a1);
    const long long col = (long long)y * g.px + x;
    const int oe = ty * TXC + xl;
    const uint32_t seed = g.sr ? mix32((uint32_t)(*g.step + g.step_off) * 0x9e3779b9u + 0x6a09e667u) : 0u;

    if (tid == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&bfull[s], 1);
            mbar_init(&bempty[s], NWARP);
        }
        fence_init();
    }
    __syncthreads();

    // z ring fields: vx (forward), vy (forward), vz (backward), qz (backward)
    auto issue = [&](int st, int k, bool warm) {
        unsigned char* b = smem + st * M::stage;
        uint64_t* br = &bfull[st];
        mbar_expect_tx(br, M::stage_tx + 4 * G::OWN_B * (warm ? 2 * R + 1 : 1));
        tma3(b + M::halo(0), &maps.halo[0], br, x0 - G::HX, y0 - R, k);  // vx (x, y halo)
        tma3(b + M::halo(1), &maps.halo[1], br, x0 - G::HX, y0 - R, k);  // vy
        tma3(b + M::halo(2), &maps.halo[2], br, x0 - G::HX, y0 - R, k);  // vz
        tma3(b + M::halo(3), &maps.halo[3], br, x0 - G::HX, y0, k);      // qx (x halo)
        tma3(b + M::halo(4), &maps.halo[4], br, x0, y0 - R, k);          // qy (y halo)
        const int z0 = warm ? k - R : k + R;
        for (int z = z0; z <= k + R; z++)
#pragma unroll
            for (int f = 0; f < 4; f++)
                tma3(smem + M::ring + (f * M::ZS + z % M::ZS) * M::OW, &maps.zlead[f], br, x0, y0, z);
    };

    Pipe<NS> pp{bfull, bempty};
    for (int s = 0; s < NS; s++) pp.pend[s] = 0;
    if (tid == 0)
        for (int j = 0; j < NS - 1 && kb + j < ke; j++) {
            issue(j, kb + j, j == 0);
            pp.pend[j]++;
        }
    bool failed = false;
    for (int k = kb, it = 0; k < ke; k++, it++) {
        const int st = it % NS;
        // the cell's own data of plane k (seven stresses/pressure, P1 P2 S1 S2 Sxy Sxz Syz; S3 = P1 c_s3) does not
        // go through the pipeline: its loads are issued before the waits
        const long long go = (long long)k * g.plane + col;
        P so_s[7];
        KP kk[7];
        constexpr int smode = sizeof(S) == 4 ? 0 : BEHF_TILED_SLOAD16;
        auto load_fields = [&]() {
#pragma unroll
            for (int q = 0; q < 7; q++)
                so_s[q] = *reinterpret_cast<const P*>(reinterpret_cast<const S*>(p.f[BEHF_SXX + q]) + go);
        };
        auto load_coefs = [&]() {
#pragma unroll
            for (int q = 0; q < 7; q++) {
                const int j = q < 4 ? P1 + q : P1 + q + 1;
                kk[q] = *reinterpret_cast<const KP*>(reinterpret_cast<const K*>(p.k[j]) + go);
            }
        };
        if (live) {
            if (smode != 1) load_fields();
            if (smode == 0) load_coefs();
        }
        bool ok = true;
        if (tid == 0) ok = producer_step<M>(pp, it, k, kb, ke, issue);
        if (ok) ok = mbar_wait(&bfull[st], (pp.fph >> st) & 1u);
        if (!__all_sync(0xffffffffu, ok)) {  // warp-uniform exit: every lane leaves together
            failed = true;
            break;
        }
        pp.fph ^= 1u << st;
        if (tid == 0) pp.pend[st]--;
        const unsigned char* b = smem + st * M::stage;
        if (live) {
            const S* vx = reinterpret_cast<const S*>(b + M::halo(0));
            const S* vy = reinterpret_cast<const S*>(b + M::halo(1));
            const S* vz = reinterpret_cast<const S*>(b + M::halo(2));
            const S* qx = reinterpret_cast<const S*>(b + M::halo(3));
            const S* qy = reinterpret_cast<const S*>(b + M::halo(4));
            const int rX = ty * G::BW + G::HX + xl;
            const int rXY = (ty + R) * G::BW + G::HX + xl;
            const int rY = (ty + R) * TXC + xl;
            XWin<S, R> w;
            w.load(vx + rXY);
            float2 uxx = w.bwd();
            w.load(vy + rXY);
            float2 uyx = w.fwd();
            w.load(vz + rXY);
            float2 uzx = w.fwd();
            w.load(qx + rX);
            float2 wx = w.bwd();
            float2 cv[2 * R + 1];
            load_col<S, R>(cv, vy + rXY, G::BW);
            float2 uyy = col_bwd<R>(cv);
            load_col<S, R>(cv, vx + rXY, G::BW);
            float2 uxy = col_fwd<R>(cv);
            load_col<S, R>(cv, vz + rXY, G::BW);
            float2 uzy = col_fwd<R>(cv);
            load_col<S, R>(cv, qy + rY, TXC);
            float2 wy = col_bwd<R>(cv);
            int zo[2 * R + 1];
            ring_slots<M, R>(k, zo);
            auto zcol = [&](int f) {
                const unsigned char* rb = smem + M::ring + f * M::ZS * M::OW + oe * sizeof(S);
#pragma unroll
                for (int d = 0; d <= 2 * R; d++) cv[d] = PS::f2(*reinterpret_cast<const P*>(rb + zo[d]));
            };
            zcol(2);
            float2 uzz = col_bwd<R>(cv);
            zcol(3);
            float2 wz = col_bwd<R>(cv);
            zcol(0);
            float2 uxz = col_fwd<R>(cv);
            zcol(1);
            float2 uyz = col_fwd<R>(cv);

            if (g.W > 0) {
                // x: uxx, wx (bwd), uyx, uzx (fwd); y: uyy, wy (bwd), uxy, uzy (fwd); z: uzz, wz (bwd), uxz, uyz (fwd)
                const bool hf[4] = {false, false, true, true};
                pml_pair<4, sizeof(S) == 4>(g, p, x, y, k, a0, a1, uxx, wx, uyx, uzx, hf, uyy, wy, uxy, uzy, hf, uzz, wz, uxz, uyz, hf);
            }
            if (smode == 1) load_fields();
            if (smode != 0) load_coefs();
            const float2 dv = add2(add2(uxx, uyy), uzz);
            const float2 dq = add2(add2(wx, wy), wz);
            auto kc = [&](int q) {
                const int j = q < 4 ? P1 + q : P1 + q + 1;
                return mul2(Pair<K>::f2(kk[q]), f2(g.kmulf[j], g.kmulf[j]));
            };
            auto own = [&](int q) { return PS::f2(so_s[q]); };
            auto put = [&](int field, float2 v) {
                const P sv = g.sr ? SR<S>::pack(v, mix32(seed ^ (uint32_t)go ^ (0x85ebca6bu * (uint32_t)(field + 1))))
                                  : PS::pack(v);
                store_pair<S>(reinterpret_cast<S*>(p.f[field]) + go, sv, a0, a1);
            };
            const float2 p1 = kc(0), p2 = kc(1), g1 = kc(2), g2 = kc(3);
            const float2 g3dq = mul2(mul2(p1, f2(g.c_s3, g.c_s3)), dq);  // S3 = P1 c_s3
            // p' = p - P1 div v - P2 div q
            put(BEHF_P, sub2(own(6), fma2(p1, dv, mul2(p2, dq))));
            // s_ii' = s_ii + S1 (d_jj + d_kk) + S2 d_ii + S3 div q
            put(BEHF_SXX, add2(own(0), fma2(g1, add2(uyy, uzz), fma2(g2, uxx, g3dq))));
            put(BEHF_SYY, add2(own(1), fma2(g1, add2(uxx, uzz), fma2(g2, uyy, g3dq))));
            put(BEHF_SZZ, add2(own(2), fma2(g1, add2(uxx, uyy), fma2(g2, uzz, g3dq))));
            // s_ij' = s_ij + S_ij (d_j v_i + d_i v_j)
            put(BEHF_SXY, fma2(kc(4), add2(uxy, uyx), own(3)));
            put(BEHF_SXZ, fma2(kc(5), add2(uxz, uzx), own(4)));
            put(BEHF_SYZ, fma2(kc(6), add2(uyz, uzy), own(5)));
        }
        __syncwarp();
        if (tx == 0) mbar_arrive(&bempty[st]);
    }
    if (failed) atomicExch(g.err, 1);
    if (tid == 0) producer_drain<M>(pp);
}

}  // namespace BEHF_TILED_NAMESPACE
}  // namespace behf

#include "kernels_tiled_ws.cuh"
#include "kernels_tiled_zq.cuh"

namespace behf {
namespace BEHF_TILED_NAMESPACE {

// ----------------------------------------------------------------------------------------- host side
// The field tensor maps: vf the arrays the velocity kernel reads (stresses and pressure in halo and z-lead boxes,
// its own velocities and Darcy velocities), tf the arrays the stress kernel reads.  Both are the context's fields
// for an in-place step; the gradient's recompute passes snapshot slots instead and steps out of place (the
// warp-specialised and tensor-memory kernels read fields only through these maps and store through DevPtrs::f).
template <class S, int R>
bool field_maps_r(const Geom& g, void* const* vf, void* const* tf, VMaps* vm, TMaps* tm) {
    typedef Geo<S, R> G;
    bool ok = true;
    // velocity
    ok &= encode<S>(&vm->halo[0], g, vf[BEHF_SXX], G::BW, TY);
    ok &= encode<S>(&vm->halo[1], g, vf[BEHF_SYY], TXC, G::BH);
    ok &= encode<S>(&vm->halo[2], g, vf[BEHF_SXY], G::BW, G::BH);
    ok &= encode<S>(&vm->halo[3], g, vf[BEHF_SXZ], G::BW, TY);
    ok &= encode<S>(&vm->halo[4], g, vf[BEHF_SYZ], TXC, G::BH);
    ok &= encode<S>(&vm->halo[5], g, vf[BEHF_P], G::BW, G::BH);
    ok &= encode<S>(&vm->zlead[0], g, vf[BEHF_SZZ], TXC, TY);
    ok &= encode<S>(&vm->zlead[1], g, vf[BEHF_SXZ], TXC, TY);
    ok &= encode<S>(&vm->zlead[2], g, vf[BEHF_SYZ], TXC, TY);
    ok &= encode<S>(&vm->zlead[3], g, vf[BEHF_P], TXC, TY);
    for (int a = 0; a < 3; a++) {
        ok &= encode<S>(&vm->own[a], g, vf[BEHF_VX + a], TXC, TY);
        ok &= encode<S>(&vm->own[3 + a], g, vf[BEHF_QX + a], TXC, TY);
    }
    // stress
    ok &= encode<S>(&tm->halo[0], g, tf[BEHF_VX], G::BW, G::BH);
    ok &= encode<S>(&tm->halo[1], g, tf[BEHF_VY], G::BW, G::BH);
    ok &= encode<S>(&tm->halo[2], g, tf[BEHF_VZ], G::BW, G::BH);
    ok &= encode<S>(&tm->halo[3], g, tf[BEHF_QX], G::BW, TY);
    ok &= encode<S>(&tm->halo[4], g, tf[BEHF_QY], TXC, G::BH);
    ok &= encode<S>(&tm->zlead[0], g, tf[BEHF_VX], TXC, TY);
    ok &= encode<S>(&tm->zlead[1], g, tf[BEHF_VY], TXC, TY);
    ok &= encode<S>(&tm->zlead[2], g, tf[BEHF_VZ], TXC, TY);
    ok &= encode<S>(&tm->zlead[3], g, tf[BEHF_QZ], TXC, TY);
    for (int q = 0; q < 7; q++) ok &= encode<S>(&tm->own[q], g, tf[BEHF_SXX + q], TXC, TY);
    return ok;
}

template <class S, int R>
bool build_maps_r(const Geom& g, const DevPtrs& p, VMaps* vm, TMaps* tm) {
    bool ok = field_maps_r<S, R>(g, p.f, p.f, vm, tm);
    // own-cell boxes (warp-specialised kernels)
    typedef typename Traits<S>::K K;
    typedef typename Traits<S>::W Wt;
    for (int a = 0; a < 3; a++) {
        ok &= encode<Wt>(&vm->own[6 + a], g, p.k[VW1X + a], TXC, TY);
        ok &= encode<K>(&vm->own[9 + a], g, p.k[VW3X + a], TXC, TY);
        ok &= encode<K>(&vm->own[12 + a], g, p.k[VU1X + a], TXC, TY);
        ok &= encode<K>(&vm->own[15 + a], g, p.k[VU2X + a], TXC, TY);
    }
    for (int q = 0; q < 7; q++) ok &= encode<K>(&tm->own[7 + q], g, p.k[q < 4 ? P1 + q : P1 + q + 1], TXC, TY);
    // x-slab CPML memory and x profiles, staged by the tensor-memory kernels (FP32 memory)
    if (g.W > 0 && g.xs_bw > 0 && sizeof(Wt) == 4) {
        for (int j = 0; j < 4; j++) {
            ok &= encode_xslab(&vm->xs[j], g, p.psi[0][j], g.xs_bw);
            ok &= encode_xslab(&vm->xs[4 + j], g, p.prv[0][j], g.xs_bw);
            ok &= encode_xslab(&tm->xs[j], g, p.psi[0][4 + j], g.xs_bw);
            ok &= encode_xslab(&tm->xs[4 + j], g, p.prv[0][4 + j], g.xs_bw);
        }
        void* const prof[4] = {p.pa[0], p.pb[0], p.pa2[0], p.pb2[0]};
        for (int j = 0; j < 4; j++) {
            ok &= encode_prof(&vm->xp[j], g.nx, prof[j]);
            ok &= encode_prof(&tm->xp[j], g.nx, prof[j]);
        }
    }
    // y- and z-slab CPML memory (L2 prefetch boxes; their rows are 16-byte multiples only when nx is a multiple of 4)
    if (g.slab_pf)
        for (int j = 0; j < 8; j++) {
            void* const vy = j < 4 ? p.psi[1][j] : p.prv[1][j - 4];
            void* const vz = j < 4 ? p.psi[2][j] : p.prv[2][j - 4];
            void* const ty = j < 4 ? p.psi[1][4 + j] : p.prv[1][j];
            void* const tz = j < 4 ? p.psi[2][4 + j] : p.prv[2][j];
            ok &= encode_slab(&vm->ys[j], vy, g.nx, g.W, g.nz);
            ok &= encode_slab(&vm->zs[j], vz, g.nx, g.ny, g.W);
            ok &= encode_slab(&tm->ys[j], ty, g.nx, g.W, g.nz);
            ok &= encode_slab(&tm->zs[j], tz, g.nx, g.ny, g.W);
        }
    return ok;
}

template <class S, int R>
cudaError_t launch_r(const Geom& g, const DevPtrs& p, const void* maps, bool vel, cudaStream_t st) {
    const int nbx = (g.nx - R + TXC - 1) / TXC, nby = (g.ny - R + TY - 1) / TY;
    const int planes = g.nz - 2 * R;
    // z chunks of at most BEHF_TILED_ZCHUNK planes: short z ranges keep the CTAs that share halo rows marching the
    // same planes at the same time, so the rows one CTA brings into L2 are still there when its neighbours read
    // them (measured at 1024^3 FP16: 64-plane chunks 34.7 ms per step against 40.2 ms for whole columns); within
    // that, a chunk count that fills the last wave of resident CTAs (MINB per SM) with at least four waves where
    // 16-plane chunks allow it (the autotuner's choice at 128^3-256^3: 0.79 ms per step at 256^3 against 0.89 ms
    // for two waves of 36-plane chunks)
    const bool ws = g.ws != 0, zq = g.ws >= 2;
    const int minb = ws ? WDepth<S>::MINB : vel ? Depth<S>::MINB : Depth<S>::MINB_T;
    const int slots = minb * device_sms();
    int zchunk = wave_zchunk(nbx * nby, planes, slots, 16, BEHF_TILED_ZCHUNK, R, BEHF_TILED_MINW);
    if (g.zchunk_req > 0) zchunk = g.zchunk_req < planes ? g.zchunk_req : planes;
    const dim3 grid(nbx, nby, (planes + zchunk - 1) / zchunk);
    const VMaps& vm = *reinterpret_cast<const VMaps*>(maps);
    const TMaps& tm = *reinterpret_cast<const TMaps*>(maps);
    // each kernel's shared-memory opt-in, once per device
    auto optin = [](PerDevice& once, const void* fn, int smem) {
        return run_once(once, [&] {
            return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        });
    };
    cudaError_t e = cudaSuccess;
    if (zq) {
        // stochastic rounding (16-bit kinds) and the x-slab staging (variant 4, when every x-edge tile's box fits)
        // select the instantiation; each has its own opt-in flags
        const bool sr = g.sr && sizeof(S) == 2;
        const bool xs = g.ws == 3 &&
                        (vel ? xs_grid_ok<ZMap<S, R, true>>(g, nbx) : xs_grid_ok<ZMap<S, R, false>>(g, nbx));
        auto go = [&](auto srnd, auto xst) -> cudaError_t {
            constexpr bool SR_ = decltype(srnd)::value, XS_ = decltype(xst)::value;
            static PerDevice once_v, once_t;
            if (vel) {
                const int smem = ZMap<S, R, true>::bytes + 128;
                cudaError_t r = optin(once_v, (const void*)k_vel_zq<S, R, SR_, XS_>, smem);
                if (r != cudaSuccess) return r;
                k_vel_zq<S, R, SR_, XS_><<<grid, NTH_WS, smem, st>>>(vm, g, p, zchunk);
            } else {
                const int smem = ZMap<S, R, false>::bytes + 128;
                cudaError_t r = optin(once_t, (const void*)k_str_zq<S, R, SR_, XS_>, smem);
                if (r != cudaSuccess) return r;
                k_str_zq<S, R, SR_, XS_><<<grid, NTH_WS, smem, st>>>(tm, g, p, zchunk);
            }
            return cudaSuccess;
        };
        using T_ = std::true_type;
        using F_ = std::false_type;
        e = sr ? (xs ? go(T_{}, T_{}) : go(T_{}, F_{})) : (xs ? go(F_{}, T_{}) : go(F_{}, F_{}));
        if (e != cudaSuccess) return e;
    } else if (ws && vel) {
        static PerDevice once;
        const int smem = WMap<S, R, true>::bytes + 128;
        if ((e = optin(once, (const void*)k_vel_ws<S, R>, smem)) != cudaSuccess) return e;
        k_vel_ws<S, R><<<grid, NTH_WS, smem, st>>>(vm, g, p, zchunk);
    } else if (ws) {
        static PerDevice once;
        const int smem = WMap<S, R, false>::bytes + 128;
        if ((e = optin(once, (const void*)k_str_ws<S, R>, smem)) != cudaSuccess) return e;
        k_str_ws<S, R><<<grid, NTH_WS, smem, st>>>(tm, g, p, zchunk);
    } else if (vel) {
        static PerDevice once;
        const int smem = Map<S, R, true>::bytes + 128;
        if ((e = optin(once, (const void*)k_vel<S, R>, smem)) != cudaSuccess) return e;
        k_vel<S, R><<<grid, NTH, smem, st>>>(vm, g, p, zchunk);
    } else {
        static PerDevice once;
        const int smem = Map<S, R, false>::bytes + 128;
        if ((e = optin(once, (const void*)k_str<S, R>, smem)) != cudaSuccess) return e;
        k_str<S, R><<<grid, NTH, smem, st>>>(tm, g, p, zchunk);
    }
    return cudaGetLastError();
}

}  // namespace BEHF_TILED_NAMESPACE

#define BEHF_TILED_INSTANTIATE(S)                                                                           \
    template <>                                                                                            \
    bool BEHF_TILED_FN(tiled_supported)<S>(const Geom& g) {                                                               \
        return g.R >= 1 && g.R <= 4 && BEHF_TILED_NAMESPACE::encoder() != nullptr && g.nz > 2 * g.R;                      \
    }                                                                                                      \
    template <>                                                                                            \
    cudaError_t BEHF_TILED_FN(tiled_build_maps)<S>(const Geom& g, const DevPtrs& p, void* vm, void* tm) {                 \
        bool ok = false;                                                                                   \
        auto* v = reinterpret_cast<BEHF_TILED_NAMESPACE::VMaps*>(vm);                                                     \
        auto* t = reinterpret_cast<BEHF_TILED_NAMESPACE::TMaps*>(tm);                                                     \
        switch (g.R) {                                                                                     \
            case 1: ok = BEHF_TILED_NAMESPACE::build_maps_r<S, 1>(g, p, v, t); break;                                      \
            case 2: ok = BEHF_TILED_NAMESPACE::build_maps_r<S, 2>(g, p, v, t); break;                                      \
            case 3: ok = BEHF_TILED_NAMESPACE::build_maps_r<S, 3>(g, p, v, t); break;                                      \
            case 4: ok = BEHF_TILED_NAMESPACE::build_maps_r<S, 4>(g, p, v, t); break;                                      \
        }                                                                                                  \
        return ok ? cudaSuccess : cudaErrorInvalidValue;                                                   \
    }                                                                                                      \
    template <>                                                                                            \
    cudaError_t BEHF_TILED_FN(tiled_field_maps)<S>(const Geom& g, void* const* vf, void* const* tf, void* vm,    \
                                                   void* tm) {                                             \
        bool ok = false;                                                                                   \
        auto* v = reinterpret_cast<BEHF_TILED_NAMESPACE::VMaps*>(vm);                                      \
        auto* t = reinterpret_cast<BEHF_TILED_NAMESPACE::TMaps*>(tm);                                      \
        switch (g.R) {                                                                                     \
            case 1: ok = BEHF_TILED_NAMESPACE::field_maps_r<S, 1>(g, vf, tf, v, t); break;                 \
            case 2: ok = BEHF_TILED_NAMESPACE::field_maps_r<S, 2>(g, vf, tf, v, t); break;                 \
            case 3: ok = BEHF_TILED_NAMESPACE::field_maps_r<S, 3>(g, vf, tf, v, t); break;                 \
            case 4: ok = BEHF_TILED_NAMESPACE::field_maps_r<S, 4>(g, vf, tf, v, t); break;                 \
        }                                                                                                  \
        return ok ? cudaSuccess : cudaErrorInvalidValue;                                                   \
    }                                                                                                      \
    template <>                                                                                            \
    cudaError_t BEHF_TILED_FN(launch_tiled)<S>(const Geom& g, const DevPtrs& p, const void* maps, bool vel, cudaStream_t st) { \
        switch (g.R) {                                                                                     \
            case 1: return BEHF_TILED_NAMESPACE::launch_r<S, 1>(g, p, maps, vel, st);                                      \
            case 2: return BEHF_TILED_NAMESPACE::launch_r<S, 2>(g, p, maps, vel, st);                                      \
            case 3: return BEHF_TILED_NAMESPACE::launch_r<S, 3>(g, p, maps, vel, st);                                      \
            case 4: return BEHF_TILED_NAMESPACE::launch_r<S, 4>(g, p, maps, vel, st);                                      \
        }                                                                                                  \
        return cudaErrorInvalidValue;                                                                      \
    }

}  // namespace behf
