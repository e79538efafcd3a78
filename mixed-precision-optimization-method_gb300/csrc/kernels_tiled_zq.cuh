// kernels_tiled_zq.cuh -- warp-specialised z-marching kernels whose z derivatives accumulate in tensor memory
// (included by kernels_tiled_impl.cuh).
//
// The x / y stencils, the producer warp and the TMA stages are those of kernels_tiled_ws.cuh.  The z stencils are
// evaluated differently: a thread's z column is private to it, so instead of re-reading 2R + 1 planes of a shared-
// memory ring for every plane (and converting each 16-bit value again), each plane that arrives is converted once
// and added, with its 2R stencil weights, into the partial sums of the 2R output planes it contributes to.  Those
// partial sums (2R pairs per field, four fields) live in TMEM, the per-SM tensor memory that tcgen05.ld / .st move
// to and from registers 16 columns at a time: per plane and field one load, 2R packed FMAs and one store, instead
// of 2R + 1 shared-memory loads, 4R + 2 conversions and 2R packed FMAs.  The partial sums add the taps in plane
// order, so the derivative is the same FP32 stencil as the other kernels' but not bit for bit.
//   fwd  D(k) = sum_m c_m (f(k+m) - f(k-m+1)):  f(z) adds +c_{R-j} (j < R) / -c_{j-R+1} (j >= R) to D(z-R+j),
//        j = 0..2R-1; D(z-R) is then complete.
//   bwd  D(k) = sum_m c_m (f(k+m-1) - f(k-m)):  D(z-R) is complete before f(z) arrives; f(z) adds
//        +c_{R-j+1} (j <= R) / -c_{j-R} (j > R) to D(z-R+j), j = 1..2R.
// Each CTA allocates 128 TMEM columns (warps w and w + 4 share a 32-lane quarter, 64 columns each: 4 fields x 16);
// the register limit keeps at most two 8-row CTAs (or four 4-row CTAs of 64 columns) on an SM, 256 of the 512
// columns, so an allocation never waits.
// The first 2R planes of a z range arrive in a one-shot warm-up area, whose partial sums are formed in registers;
// once every compute warp has read it, the tiles at the x edges receive there, with each plane, the CPML memory of
// their x-slab cells (TMA boxes), so that their slab updates read it from shared memory instead of waiting on
// global loads.  Every wait is bounded; on any exit path the compute warps meet at a named barrier and warp 0 frees
// the TMEM.
#pragma once
#include <type_traits>

namespace behf {
namespace BEHF_TILED_NAMESPACE {

#ifndef BEHF_ZQ_NS
#define BEHF_ZQ_NS 2
#endif
// Plane-loop unrolling.  Unrolled by the stage count, each copy's stage (and its shared-memory offsets) is fixed, but
// the loop's code doubles and competes for the instruction cache (instruction-fetch stalls were the second stall):
// not unrolled, 1024^3 FP16 runs at 39.2 Gpt/s against 37.9 unrolled by two (BF16 36.3 against 35.4).
#ifndef BEHF_ZQ_UNROLL
#define BEHF_ZQ_UNROLL 1
#endif
constexpr int kZqUnroll = BEHF_ZQ_UNROLL;
// y- and z-slab CPML memory of a cell pair loaded in one batch (one memory latency instead of two)
#ifndef BEHF_ZQ_PAIRYZ
#define BEHF_ZQ_PAIRYZ true
#endif
constexpr uint32_t kZqCols = 16 * TY;  // TMEM columns per CTA: 64 per lane quarter's warps (TY / 4 of them)

// Store a cell pair; FULL: both cells are known to be updated (no per-cell guard).
template <class S, bool FULL>
__device__ __forceinline__ void store_cells(S* dst, typename Pair<S>::T v, bool a0, bool a1) {
    if constexpr (FULL) *reinterpret_cast<typename Pair<S>::T*>(dst) = v;
    else store_pair<S>(dst, v, a0, a1);
}
__device__ __forceinline__ void tm_alloc(uint32_t* dst) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(kZqCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tm_dealloc(uint32_t taddr) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kZqCols) : "memory");
}
__device__ __forceinline__ void tm_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tm_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// 16 columns of this thread's lane (one field's partial sums): load and wait for the load.  The caller waits for its
// earlier stores once per plane (tm_wait_st) before the first load; the four fields' columns are disjoint.
__device__ __forceinline__ void tm_ld16(uint32_t ta, float (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]), "=f"(r[7]), "=f"(r[8]),
          "=f"(r[9]), "=f"(r[10]), "=f"(r[11]), "=f"(r[12]), "=f"(r[13]), "=f"(r[14]), "=f"(r[15])
        : "r"(ta)
        : "memory");
}
__device__ __forceinline__ void tm_st16(uint32_t ta, const float (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(ta),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
        "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
        : "memory");
}
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void bar_compute() {  // the eight compute warps only (the producer warp has left)
    asm volatile("bar.sync 1, %0;" ::"n"(NTH) : "memory");
}

// One plane f(z) (a cell pair v) into the partial sums s[0..4R) of one field (pair j in s[2j], s[2j+1]); writes the
// shifted sums for the next plane to t[0..16) and returns the completed derivative pair of plane z - R.
template <int R, bool FWD>
__device__ __forceinline__ float2 zq_math(const float* s, float2 v, float* t) {
    float2 out;
    if (FWD) {
        float a[4 * R];
#pragma unroll
        for (int j = 0; j < 2 * R; j++) {
            const float w = j < R ? wgt<R>(R - j) : -wgt<R>(j - R + 1);
            const float2 r = fma2(f2(w, w), v, f2(s[2 * j], s[2 * j + 1]));
            a[2 * j] = r.x;
            a[2 * j + 1] = r.y;
        }
        out = f2(a[0], a[1]);
#pragma unroll
        for (int i = 0; i < 4 * R - 2; i++) t[i] = a[i + 2];
        t[4 * R - 2] = 0.f;
        t[4 * R - 1] = 0.f;
    } else {
        out = f2(s[0], s[1]);
#pragma unroll
        for (int j = 1; j <= 2 * R; j++) {
            const float w = j <= R ? wgt<R>(R - j + 1) : -wgt<R>(j - R);
            const float2 base = j < 2 * R ? f2(s[2 * j], s[2 * j + 1]) : f2(0.f, 0.f);
            const float2 r = fma2(f2(w, w), v, base);
            t[2 * j - 2] = r.x;
            t[2 * j - 1] = r.y;
        }
    }
#pragma unroll
    for (int i = 4 * R; i < 16; i++) t[i] = 0.f;
    return out;
}

// One field (columns ta .. ta + 15) advanced by one plane: load, the sums, store.
template <int R, bool FWD>
__device__ __forceinline__ float2 zq_one(uint32_t ta, float2 v) {
    float s[16], t[16];
    tm_ld16(ta, s);
    const float2 d = zq_math<R, FWD>(s, v, t);
    tm_st16(ta, t);
    return d;
}

// Weight of plane offset d = z - k in the derivative of output plane k (0 outside the stencil).
template <int R, bool FWD>
__host__ __device__ constexpr float zq_w(int d) {
    return FWD ? (d >= 1 && d <= R ? (float)stencil_w<R>(d) : d >= 1 - R && d <= 0 ? -(float)stencil_w<R>(1 - d) : 0.f)
               : (d >= 0 && d <= R - 1 ? (float)stencil_w<R>(d + 1) : d >= -R && d <= -1 ? -(float)stencil_w<R>(-d) : 0.f);
}

// The partial sums after the 2R warm-up planes z_w = kb - R + w (w = 0..2R-1), in registers: entry j (output plane
// kb + j) is the sum over w of zq_w(z_w - kb - j) v_w, taken in plane order as the plane-by-plane updates would,
// then stored once.  v: the field's 2R warm-up values of this thread's cell pair.
template <int R, bool FWD>
__device__ __forceinline__ void zq_warm(uint32_t ta, const float2 (&v)[2 * R]) {
    float t[16];
#pragma unroll
    for (int j = 0; j < 2 * R; j++) {
        float2 acc = f2(0.f, 0.f);
#pragma unroll
        for (int w = 0; w < 2 * R; w++) {
            const float c = zq_w<R, FWD>(w - R - j);
            if (c != 0.f) acc = fma2(f2(c, c), v[w], acc);
        }
        t[2 * j] = acc.x;
        t[2 * j + 1] = acc.y;
    }
#pragma unroll
    for (int i = 4 * R; i < 16; i++) t[i] = 0.f;
    tm_st16(ta, t);
}

// Shared-memory map: NS stages of [halo | own fields | own FP32 Darcy | own coefficients | z-lead plane (4 fields)],
// then the warm-up area (2R planes of the 4 z fields).
template <class S, int R, bool VEL>
struct ZMap {
    typedef Geo<S, R> G;
    typedef WMap<S, R, VEL> W;
    static constexpr int NS = BEHF_ZQ_NS;
    static constexpr int OW = W::OW, OK = W::OK, OWW = W::OWW;
    static constexpr int NF = W::NF, NW = W::NW, NK = W::NK;
    __host__ __device__ static constexpr int halo(int i) { return Map<S, R, VEL>::halo(i); }
    static constexpr int own_f = W::own_f, own_w = W::own_w, own_k = W::own_k;
    static constexpr int zl = own_k + NK * OK;
    static constexpr int stage = zl + 4 * OW;
    static constexpr int warm = NS * stage;
    static constexpr int bytes = warm + 4 * 2 * R * OW;
    static constexpr uint32_t stage_tx = W::stage_tx + 4 * G::OWN_B;
    static constexpr uint32_t warm_tx = 4 * 2 * R * G::OWN_B;
};

// x-slab CPML memory staged by TMA: the tiles at the x edges bring, with each plane, the memory of their x-slab cells
// (eight FP32 arrays, boxes of xs_bw x TY) into the warm-up area, which is idle once the warm-up planes are read
// (one set per stage).  Bytes of one set, and whether this CTA stages (CTA-uniform; xbase from xs_tile_base).
// After the sets, the tile's four x profiles (TXC values each), brought once with the first plane.
constexpr int kXsProfBytes = 4 * TXC * 4;
// Each array's box starts on a 128-byte boundary (the TMA rule for a shared-memory destination): with 8-row tiles
// xs_bw x 8 x 4 bytes already is a multiple of 128, with 4-row tiles it is padded.  xs_set_tx: the bytes the eight
// boxes bring (the stage's expected transaction count).
__host__ __device__ __forceinline__ int xs_box_bytes(const Geom& g) { return al128(g.xs_bw * TY * 4); }
__host__ __device__ __forceinline__ int xs_set_bytes(const Geom& g) { return 8 * xs_box_bytes(g); }
__host__ __device__ __forceinline__ int xs_set_tx(const Geom& g) { return 8 * g.xs_bw * TY * 4; }
template <class M>
__device__ __forceinline__ bool xs_staged(const Geom& g, int xbase) {
    return xbase >= 0 && M::NS * xs_set_bytes(g) + kXsProfBytes <= M::bytes - M::warm;
}
// L2 prefetch, by the producer, of the y- and z-slab CPML memory (and the x-slab memory where it is not staged)
// that plane k's slab cells will load: a few tensor prefetches per plane instead of the compute warps' global loads
// missing L2.  ybox: the first slab row index of the tile's y-slab box, or -1 (no y-slab rows); xbox likewise for
// an x-slab box read by the compute threads.
template <class Maps>
__device__ __forceinline__ void slab_prefetch(const Geom& g, const Maps& maps, int x0, int y0, int k, int ybox,
                                              int xbox) {
    if (!g.slab_pf) return;
    const int sk = slab_index(k, g.nz, g.L);
    if (sk >= 0)
        for (int j = 0; j < 8; j++) tma3_prefetch(&maps.zs[j], x0, y0, sk);
    if (ybox >= 0)
        for (int j = 0; j < 8; j++) tma3_prefetch(&maps.ys[j], x0, ybox, k);
    if (xbox >= 0)
        for (int j = 0; j < 8; j++) tma3_prefetch(&maps.xs[j], xbox, y0, k);
}
// The tile's y-slab box start (the slab index of its first updated slab row), or -1.
__device__ __forceinline__ int ys_tile_box(const Geom& g, int y0) {
    if (g.W <= 0) return -1;
    for (int r = 0; r < TY; r++) {
        const int y = y0 + r;
        if (y >= g.R && y < g.ny - g.R && slab_index(y, g.ny, g.L) >= 0) return slab_index(y, g.ny, g.L);
    }
    return -1;
}

// Host: whether every tile of the grid that updates x-slab cells can stage them; the launcher then runs the XS
// instantiation, whose x-slab path reads shared memory only.
template <class M>
inline bool xs_grid_ok(const Geom& g, int nbx) {
    if (g.xs_bw <= 0 || g.W <= 0 || M::NS * xs_set_bytes(g) + kXsProfBytes > M::bytes - M::warm) return false;
    for (int bx = 0; bx < nbx; bx++) {
        const int x0 = bx * TXC;
        const int lo = x0 > g.R ? x0 : g.R, hi = x0 + TXC < g.nx - g.R ? x0 + TXC : g.nx - g.R;
        if (lo >= hi) continue;
        if ((lo < g.L || hi > g.nx - 1 - g.L) && xs_tile_base(g, x0) < 0) return false;
    }
    return true;
}

// Producer of a ZQ kernel: the warm-up planes kb-R .. kb+R-1 of the z fields on `warm`, then the stages.  With
// xs: each stage's x-slab boxes (issue_x) and, with the first plane, the x profiles (issue_p), counted in the
// stages' expected bytes by `issue`; those of the first stages only after every compute warp has read the warm-up
// area (`wfree`).
template <class M, int R, class Issue, class IssueX, class IssueP>
__device__ __forceinline__ void zq_produce(unsigned char* smem, uint64_t* full, uint64_t* empty, uint64_t* warm,
                                           uint64_t* wfree, const CUtensorMap* zlead, int x0, int y0, int kb, int ke,
                                           int* err, bool xs, Issue&& issue, IssueX&& issue_x, IssueP&& issue_p) {
    mbar_expect_tx(warm, M::warm_tx);
    for (int w = 0; w < 2 * R; w++)
#pragma unroll
        for (int f = 0; f < 4; f++) tma3(smem + M::warm + (f * 2 * R + w) * M::OW, &zlead[f], warm, x0, y0, kb - R + w);
    const int nfirst = ke - kb < M::NS ? ke - kb : M::NS;
    bool xok = xs;
    ws_produce<M::NS>(full, empty, kb, ke, err, [&](int st, int k, bool) {
        issue(st, k);
        if (!xok) return;
        const int it = k - kb;
        if (it >= M::NS) {
            issue_x(st, k);
        } else if (it == nfirst - 1) {
            if (!mbar_wait(wfree, 0)) {  // the compute warps never finished the warm-up: their waits run out too
                xok = false;
                atomicExch(err, 1);
                return;
            }
            issue_p();
            for (int i = 0; i < nfirst; i++) issue_x(i % M::NS, kb + i);
        }
    });
    mbar_wait(warm, 0);
}

// ----------------------------------------------------------------------------------------- velocity
template <class S, int R, bool SRND, bool XS>
__global__ void __launch_bounds__(NTH_WS, WDepth<S>::MINB)
    k_vel_zq(const __grid_constant__ VMaps maps, const Geom g, const DevPtrs p, const int zchunk) {
    typedef Pair<S> PS;
    typedef typename PS::T P;
    typedef typename Traits<S>::K K;
    typedef typename Pair<K>::T KP;
    typedef Geo<S, R> G;
    typedef ZMap<S, R, true> M;
    constexpr int NS = M::NS;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bfull[NS], bempty[NS], bwarm, bwfree;
    __shared__ uint32_t tbase;
    unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);

    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int x0 = blockIdx.x * TXC, y0 = blockIdx.y * TY;
    const int kb = R + blockIdx.z * zchunk;
    const int ke = min(kb + zchunk, g.nz - R);
    if (kb >= ke) return;
    if (tid == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&bfull[s], 1);
            mbar_init(&bempty[s], NWARP);
        }
        mbar_init(&bwarm, 1);
        mbar_init(&bwfree, NWARP);
        fence_init();
    }
    if (ty == 0) tm_alloc(&tbase);
    tm_fence_before();
    __syncthreads();
    tm_fence_after();

    if (ty == NWARP) {  // producer warp
        if (tx == 0) {
            const int xbase = xs_tile_base(g, x0);
            const bool xs = XS && xs_staged<M>(g, xbase);
            const int xsb = xs_set_bytes(g);
            // L2 prefetch of the slab memory in the instantiation without x staging (measured: BF16 +2.0 %; with the
            // staging it cost FP16 1.4 %, so that instantiation has none)
            const int ybox = XS ? -1 : ys_tile_box(g, y0), xbox = XS ? -1 : xbase;
            if (!XS)
                for (int k = kb; k < ke && k < kb + NS; k++) slab_prefetch(g, maps, x0, y0, k, ybox, xbox);
            auto issue = [&](int st, int k) {
                unsigned char* b = smem + st * M::stage;
                uint64_t* br = &bfull[st];
                mbar_expect_tx(br, M::stage_tx + (xs ? (uint32_t)(xs_set_tx(g) + (k == kb ? kXsProfBytes : 0)) : 0u));
                tma3(b + M::halo(0), &maps.halo[0], br, x0 - G::HX, y0, k);      // txx  (x halo)
                tma3(b + M::halo(1), &maps.halo[1], br, x0, y0 - R, k);          // tyy  (y halo)
                tma3(b + M::halo(2), &maps.halo[2], br, x0 - G::HX, y0 - R, k);  // txy  (x, y halo)
                tma3(b + M::halo(3), &maps.halo[3], br, x0 - G::HX, y0, k);      // txz  (x halo)
                tma3(b + M::halo(4), &maps.halo[4], br, x0, y0 - R, k);          // tyz  (y halo)
                tma3(b + M::halo(5), &maps.halo[5], br, x0 - G::HX, y0 - R, k);  // p    (x, y halo)
#pragma unroll
                for (int f = 0; f < 6; f++) tma3(b + M::own_f + f * M::OW, &maps.own[f], br, x0, y0, k);
#pragma unroll
                for (int a = 0; a < 3; a++) tma3(b + M::own_w + a * M::OWW, &maps.own[6 + a], br, x0, y0, k);
#pragma unroll
                for (int j = 0; j < 9; j++) tma3(b + M::own_k + j * M::OK, &maps.own[9 + j], br, x0, y0, k);
#pragma unroll
                for (int f = 0; f < 4; f++) tma3(b + M::zl + f * M::OW, &maps.zlead[f], br, x0, y0, k + R);
                if (!XS && k + NS < ke) slab_prefetch(g, maps, x0, y0, k + NS, ybox, xbox);  // the plane NS ahead
            };
            auto issue_x = [&](int st, int k) {
                unsigned char* xb = smem + M::warm + st * xsb;
#pragma unroll
                for (int j = 0; j < 8; j++) tma3(xb + j * xs_box_bytes(g), &maps.xs[j], &bfull[st], xbase, y0, k);
            };
            auto issue_p = [&]() {  // on the first plane's stage (stage 0)
                unsigned char* pb = smem + M::warm + NS * xsb;
#pragma unroll
                for (int j = 0; j < 4; j++) tma1(pb + j * (kXsProfBytes / 4), &maps.xp[j], &bfull[0], x0);
            };
            zq_produce<M, R>(smem, bfull, bempty, &bwarm, &bwfree, maps.zlead, x0, y0, kb, ke, g.err, xs, issue,
                             issue_x, issue_p);
        }
        return;
    }

    const int xl = 2 * tx, x = x0 + xl, y = y0 + ty;
    const bool a0 = x >= R && x < g.nx - R, a1 = x + 1 >= R && x + 1 < g.nx - R;
    const bool live = (y >= R && y < g.ny - R) && (a0 || a1);
    const long long col = (long long)y * g.px + x;
    const int oe = ty * TXC + xl;
    const uint32_t seed = SRND ? mix32((uint32_t)(*g.step + g.step_off) * 0x9e3779b9u + 0x2545f491u) : 0u;
    // every lane of the warp updates both of its cells (the interior of the grid): stores need no per-cell guard
    const bool wfull = __all_sync(0xffffffffu, live && a0 && a1);
    const uint32_t ta = tbase + ((uint32_t)(32 * (ty & 3)) << 16) + (uint32_t)(ty >> 2) * 64u;
    // x and y of a thread are fixed: whether its cells lie in an x or y slab is decided once, z per plane
    const bool xy_slab = g.W > 0 && live && ((a0 && slab_index(x, g.nx, g.L) >= 0) ||
                                             (a1 && slab_index(x + 1, g.nx, g.L) >= 0) || slab_index(y, g.ny, g.L) >= 0);
    // z fields: tzz (fwd), txz (bwd), tyz (bwd), p (fwd); box(f) gives field f's plane of cell pairs
    auto zsteps = [&](auto box, float2& d0, float2& d1, float2& d2, float2& d3) {
        auto val = [&](int f) { return PS::f2(*reinterpret_cast<const P*>(box(f) + oe * sizeof(S))); };
        tm_wait_st();  // the previous plane's stores
        d0 = zq_one<R, true>(ta, val(0));
        d1 = zq_one<R, false>(ta + 16, val(1));
        d2 = zq_one<R, false>(ta + 32, val(2));
        d3 = zq_one<R, true>(ta + 48, val(3));
    };
    constexpr bool FWD0 = true, FWD1 = false, FWD2 = false, FWD3 = true;  // tzz, txz, tyz, p
    bool failed = !__all_sync(0xffffffffu, mbar_wait(&bwarm, 0));
    if (!failed) {
        auto warm = [&](int f, float2 (&v)[2 * R]) {
#pragma unroll
            for (int w = 0; w < 2 * R; w++)
                v[w] = PS::f2(*reinterpret_cast<const P*>(smem + M::warm + (f * 2 * R + w) * M::OW + oe * sizeof(S)));
        };
        float2 v[2 * R];
        warm(0, v);
        zq_warm<R, FWD0>(ta, v);
        warm(1, v);
        zq_warm<R, FWD1>(ta + 16, v);
        warm(2, v);
        zq_warm<R, FWD2>(ta + 32, v);
        warm(3, v);
        zq_warm<R, FWD3>(ta + 48, v);
    }
    __syncwarp();
    if (tx == 0) mbar_arrive(&bwfree);  // the warm-up area is read: the producer may stage x-slab memory there

#pragma unroll kZqUnroll
    for (int k = kb, it = 0; k < ke && !failed; k++, it++) {
        const int st = it % NS;
        const bool ok = mbar_wait(&bfull[st], (it / NS) & 1);
        if (!__all_sync(0xffffffffu, ok)) {
            failed = true;
            break;
        }
        const unsigned char* b = smem + st * M::stage;
        // every lane of the warp takes part in the tensor-memory steps
        float2 z1, x3, y3, s3;
        zsteps([&](int f) { return b + M::zl + f * M::OW; }, z1, x3, y3, s3);
        float2 x1 = f2(0.f, 0.f), s1 = x1, y2 = x1, z2 = x1, y1 = x1, s2 = x1, x2 = x1, z3 = x1;
        if (live) {
            const S* txx = reinterpret_cast<const S*>(b + M::halo(0));
            const S* tyy = reinterpret_cast<const S*>(b + M::halo(1));
            const S* txy = reinterpret_cast<const S*>(b + M::halo(2));
            const S* txz = reinterpret_cast<const S*>(b + M::halo(3));
            const S* tyz = reinterpret_cast<const S*>(b + M::halo(4));
            const S* pp_ = reinterpret_cast<const S*>(b + M::halo(5));
            const int rX = ty * G::BW + G::HX + xl;
            const int rXY = (ty + R) * G::BW + G::HX + xl;
            const int rY = (ty + R) * TXC + xl;
            XWin<S, R> w;
            w.load(txx + rX);
            x1 = w.fwd();
            w.load(pp_ + rXY);
            s1 = w.fwd();
            w.load(txy + rXY);
            y2 = w.bwd();
            w.load(txz + rX);
            z2 = w.bwd();
            float2 cv[2 * R + 1];
            load_col<S, R>(cv, tyy + rY, TXC);
            y1 = col_fwd<R>(cv);
            load_col<S, R>(cv, pp_ + rXY, G::BW);
            s2 = col_fwd<R>(cv);
            load_col<S, R>(cv, txy + rXY, G::BW);
            x2 = col_bwd<R>(cv);
            load_col<S, R>(cv, tyz + rY, TXC);
            z3 = col_bwd<R>(cv);
        }
        if (live) {
            const long long go = (long long)k * g.plane + col;
            if (xy_slab || (g.W > 0 && slab_index(k, g.nz, g.L) >= 0)) {
                // XS: the x-slab memory staged in the warm-up area (formed here: nothing extra stays live in the loop)
                const int xbase = XS ? xs_tile_base(g, x0) : 0;
                const float* xrow =
                    XS ? reinterpret_cast<const float*>(smem + M::warm + st * xs_set_bytes(g)) + ty * g.xs_bw : nullptr;
                const float* xprof =
                    XS ? reinterpret_cast<const float*>(smem + M::warm + NS * xs_set_bytes(g)) + xl : nullptr;
                const bool hf[4] = {true, true, false, false};
                pml_pair<0, false, XS, BEHF_ZQ_PAIRYZ>(g, p, x, y, k, a0, a1, x1, s1, y2, z2, hf, y1, s2, x2, z3, hf, z1, s3, x3, y3, hf,
                                       xrow, xbase, xs_box_bytes(g) / 4, xprof);
            }
            const float2 sum[3] = {add2(add2(x1, x2), x3), add2(add2(y1, y2), y3), add2(add2(z1, z2), z3)};
            const float2 dp[3] = {s1, s2, s3};
            auto own = [&](int f) { return PS::f2(*reinterpret_cast<const P*>(b + M::own_f + f * M::OW + oe * sizeof(S))); };
            auto coef = [&](int j, int kidx) {
                const KP kv = *reinterpret_cast<const KP*>(b + M::own_k + j * M::OK + oe * sizeof(K));
                return mul2(Pair<K>::f2(kv), f2(g.kmulf[kidx], g.kmulf[kidx]));
            };
            // two copies of the update: warps whose cells are all inside the updated region store unguarded
            auto update = [&](auto full) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float2 vw1 = *reinterpret_cast<const float2*>(b + M::own_w + a * M::OWW + oe * 4);
                const float2 vw3 = coef(a, VW3X + a);
                const float2 vu1 = coef(3 + a, VU1X + a), vu2 = coef(6 + a, VU2X + a);
                const float2 vw2 = mul2(mul2(vu2, vw3), f2(g.c_vw2, g.c_vw2));
                const float2 vw3p = (a == 2 && g.bug) ? coef(1, VW3Y) : vw3;  // reference: vz uses VW3y
                const float2 qo = own(3 + a);
                // q' = VW1 q - VW2 sum(d sigma) - VW3 d p
                const float2 t = fma2(vw2, sum[a], mul2(vw3p, dp[a]));
                const float2 qn = fma2(vw1, qo, make_float2(-t.x, -t.y));
                const P qs = SRND ? SR<S>::pack(qn, mix32(seed ^ (uint32_t)go ^ (0x3c6ef372u * (uint32_t)(a + 1))))
                                  : PS::pack(qn);
                store_cells<S, decltype(full)::value>(reinterpret_cast<S*>(p.f[BEHF_QX + a]) + go, qs, a0, a1);
                // v' = v + VU1 sum(d sigma) - VU2 (q' - q)
                const float2 dq = sub2(PS::f2(qs), qo);
                const float2 vn = fma2(vu1, sum[a], fma2(make_float2(-vu2.x, -vu2.y), dq, own(a)));
                const P vs = SRND ? SR<S>::pack(vn, mix32(seed ^ (uint32_t)go ^ (0x1b873593u * (uint32_t)(a + 1))))
                                  : PS::pack(vn);
                store_cells<S, decltype(full)::value>(reinterpret_cast<S*>(p.f[BEHF_VX + a]) + go, vs, a0, a1);
            }
            };
            if (wfull) update(std::true_type{});
            else update(std::false_type{});
        }
        __syncwarp();
        if (tx == 0) mbar_arrive(&bempty[st]);
    }
    if (failed) atomicExch(g.err, 1);
    tm_fence_before();
    bar_compute();
    if (ty == 0) {
        tm_fence_after();
        tm_dealloc(tbase);
    }
}

// ----------------------------------------------------------------------------------------- stress
template <class S, int R, bool SRND, bool XS>
__global__ void __launch_bounds__(NTH_WS, WDepth<S>::MINB)
    k_str_zq(const __grid_constant__ TMaps maps, const Geom g, const DevPtrs p, const int zchunk) {
    typedef Pair<S> PS;
    typedef typename PS::T P;
    typedef typename Traits<S>::K K;
    typedef typename Pair<K>::T KP;
    typedef Geo<S, R> G;
    typedef ZMap<S, R, false> M;
    constexpr int NS = M::NS;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bfull[NS], bempty[NS], bwarm, bwfree;
    __shared__ uint32_t tbase;
    unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);

    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int x0 = blockIdx.x * TXC, y0 = blockIdx.y * TY;
    const int kb = R + blockIdx.z * zchunk;
    const int ke = min(kb + zchunk, g.nz - R);
    if (kb >= ke) return;
    if (tid == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&bfull[s], 1);
            mbar_init(&bempty[s], NWARP);
        }
        mbar_init(&bwarm, 1);
        mbar_init(&bwfree, NWARP);
        fence_init();
    }
    if (ty == 0) tm_alloc(&tbase);
    tm_fence_before();
    __syncthreads();
    tm_fence_after();

    if (ty == NWARP) {  // producer warp
        if (tx == 0) {
            const int xbase = xs_tile_base(g, x0);
            const bool xs = XS && xs_staged<M>(g, xbase);
            const int xsb = xs_set_bytes(g);
            // L2 prefetch of the slab memory in the instantiation without x staging (measured: BF16 +2.0 %; with the
            // staging it cost FP16 1.4 %, so that instantiation has none)
            const int ybox = XS ? -1 : ys_tile_box(g, y0), xbox = XS ? -1 : xbase;
            if (!XS)
                for (int k = kb; k < ke && k < kb + NS; k++) slab_prefetch(g, maps, x0, y0, k, ybox, xbox);
            auto issue = [&](int st, int k) {
                unsigned char* b = smem + st * M::stage;
                uint64_t* br = &bfull[st];
                mbar_expect_tx(br, M::stage_tx + (xs ? (uint32_t)(xs_set_tx(g) + (k == kb ? kXsProfBytes : 0)) : 0u));
                tma3(b + M::halo(0), &maps.halo[0], br, x0 - G::HX, y0 - R, k);  // vx (x, y halo)
                tma3(b + M::halo(1), &maps.halo[1], br, x0 - G::HX, y0 - R, k);  // vy
                tma3(b + M::halo(2), &maps.halo[2], br, x0 - G::HX, y0 - R, k);  // vz
                tma3(b + M::halo(3), &maps.halo[3], br, x0 - G::HX, y0, k);      // qx (x halo)
                tma3(b + M::halo(4), &maps.halo[4], br, x0, y0 - R, k);          // qy (y halo)
#pragma unroll
                for (int f = 0; f < 7; f++) tma3(b + M::own_f + f * M::OW, &maps.own[f], br, x0, y0, k);
#pragma unroll
                for (int j = 0; j < 7; j++) tma3(b + M::own_k + j * M::OK, &maps.own[7 + j], br, x0, y0, k);
#pragma unroll
                for (int f = 0; f < 4; f++) tma3(b + M::zl + f * M::OW, &maps.zlead[f], br, x0, y0, k + R);
                if (!XS && k + NS < ke) slab_prefetch(g, maps, x0, y0, k + NS, ybox, xbox);  // the plane NS ahead
            };
            auto issue_x = [&](int st, int k) {
                unsigned char* xb = smem + M::warm + st * xsb;
#pragma unroll
                for (int j = 0; j < 8; j++) tma3(xb + j * xs_box_bytes(g), &maps.xs[j], &bfull[st], xbase, y0, k);
            };
            auto issue_p = [&]() {  // on the first plane's stage (stage 0)
                unsigned char* pb = smem + M::warm + NS * xsb;
#pragma unroll
                for (int j = 0; j < 4; j++) tma1(pb + j * (kXsProfBytes / 4), &maps.xp[j], &bfull[0], x0);
            };
            zq_produce<M, R>(smem, bfull, bempty, &bwarm, &bwfree, maps.zlead, x0, y0, kb, ke, g.err, xs, issue,
                             issue_x, issue_p);
        }
        return;
    }

    const int xl = 2 * tx, x = x0 + xl, y = y0 + ty;
    const bool a0 = x >= R && x < g.nx - R, a1 = x + 1 >= R && x + 1 < g.nx - R;
    const bool live = (y >= R && y < g.ny - R) && (a0 || a1);
    const long long col = (long long)y * g.px + x;
    const int oe = ty * TXC + xl;
    const uint32_t seed = SRND ? mix32((uint32_t)(*g.step + g.step_off) * 0x9e3779b9u + 0x6a09e667u) : 0u;
    const bool wfull = __all_sync(0xffffffffu, live && a0 && a1);
    const uint32_t ta = tbase + ((uint32_t)(32 * (ty & 3)) << 16) + (uint32_t)(ty >> 2) * 64u;
    const bool xy_slab = g.W > 0 && live && ((a0 && slab_index(x, g.nx, g.L) >= 0) ||
                                             (a1 && slab_index(x + 1, g.nx, g.L) >= 0) || slab_index(y, g.ny, g.L) >= 0);
    // z fields: vx (fwd), vy (fwd), vz (bwd), qz (bwd); box(f) gives field f's plane of cell pairs
    auto zsteps = [&](auto box, float2& d0, float2& d1, float2& d2, float2& d3) {
        auto val = [&](int f) { return PS::f2(*reinterpret_cast<const P*>(box(f) + oe * sizeof(S))); };
        tm_wait_st();  // the previous plane's stores
        d0 = zq_one<R, true>(ta, val(0));
        d1 = zq_one<R, true>(ta + 16, val(1));
        d2 = zq_one<R, false>(ta + 32, val(2));
        d3 = zq_one<R, false>(ta + 48, val(3));
    };
    constexpr bool FWD0 = true, FWD1 = true, FWD2 = false, FWD3 = false;  // vx, vy, vz, qz
    bool failed = !__all_sync(0xffffffffu, mbar_wait(&bwarm, 0));
    if (!failed) {
        auto warm = [&](int f, float2 (&v)[2 * R]) {
#pragma unroll
            for (int w = 0; w < 2 * R; w++)
                v[w] = PS::f2(*reinterpret_cast<const P*>(smem + M::warm + (f * 2 * R + w) * M::OW + oe * sizeof(S)));
        };
        float2 v[2 * R];
        warm(0, v);
        zq_warm<R, FWD0>(ta, v);
        warm(1, v);
        zq_warm<R, FWD1>(ta + 16, v);
        warm(2, v);
        zq_warm<R, FWD2>(ta + 32, v);
        warm(3, v);
        zq_warm<R, FWD3>(ta + 48, v);
    }
    __syncwarp();
    if (tx == 0) mbar_arrive(&bwfree);  // the warm-up area is read: the producer may stage x-slab memory there

#pragma unroll kZqUnroll
    for (int k = kb, it = 0; k < ke && !failed; k++, it++) {
        const int st = it % NS;
        const bool ok = mbar_wait(&bfull[st], (it / NS) & 1);
        if (!__all_sync(0xffffffffu, ok)) {
            failed = true;
            break;
        }
        const unsigned char* b = smem + st * M::stage;
        // every lane of the warp takes part in the tensor-memory steps
        float2 uxz, uyz, uzz, wz;
        zsteps([&](int f) { return b + M::zl + f * M::OW; }, uxz, uyz, uzz, wz);
        float2 uxx = f2(0.f, 0.f), uyx = uxx, uzx = uxx, wx = uxx, uyy = uxx, uxy = uxx, uzy = uxx, wy = uxx;
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
            uxx = w.bwd();
            w.load(vy + rXY);
            uyx = w.fwd();
            w.load(vz + rXY);
            uzx = w.fwd();
            w.load(qx + rX);
            wx = w.bwd();
            float2 cv[2 * R + 1];
            load_col<S, R>(cv, vy + rXY, G::BW);
            uyy = col_bwd<R>(cv);
            load_col<S, R>(cv, vx + rXY, G::BW);
            uxy = col_fwd<R>(cv);
            load_col<S, R>(cv, vz + rXY, G::BW);
            uzy = col_fwd<R>(cv);
            load_col<S, R>(cv, qy + rY, TXC);
            wy = col_bwd<R>(cv);
        }
        if (live) {
            const long long go = (long long)k * g.plane + col;
            if (xy_slab || (g.W > 0 && slab_index(k, g.nz, g.L) >= 0)) {
                const int xbase = XS ? xs_tile_base(g, x0) : 0;
                const float* xrow =
                    XS ? reinterpret_cast<const float*>(smem + M::warm + st * xs_set_bytes(g)) + ty * g.xs_bw : nullptr;
                const float* xprof =
                    XS ? reinterpret_cast<const float*>(smem + M::warm + NS * xs_set_bytes(g)) + xl : nullptr;
                const bool hf[4] = {false, false, true, true};
                pml_pair<4, false, XS, BEHF_ZQ_PAIRYZ>(g, p, x, y, k, a0, a1, uxx, wx, uyx, uzx, hf, uyy, wy, uxy, uzy, hf, uzz, wz, uxz,
                                       uyz, hf, xrow, xbase, xs_box_bytes(g) / 4, xprof);
            }
            const float2 dv = add2(add2(uxx, uyy), uzz);
            const float2 dq = add2(add2(wx, wy), wz);
            auto kc = [&](int q) {
                const int j = q < 4 ? P1 + q : P1 + q + 1;
                const KP kv = *reinterpret_cast<const KP*>(b + M::own_k + q * M::OK + oe * sizeof(K));
                return mul2(Pair<K>::f2(kv), f2(g.kmulf[j], g.kmulf[j]));
            };
            auto own = [&](int q) { return PS::f2(*reinterpret_cast<const P*>(b + M::own_f + q * M::OW + oe * sizeof(S))); };
            // two copies of the update: warps whose cells are all inside the updated region store unguarded
            auto update = [&](auto full) {
            auto put = [&](int field, float2 v) {
                const P sv = SRND ? SR<S>::pack(v, mix32(seed ^ (uint32_t)go ^ (0x85ebca6bu * (uint32_t)(field + 1))))
                                  : PS::pack(v);
                store_cells<S, decltype(full)::value>(reinterpret_cast<S*>(p.f[field]) + go, sv, a0, a1);
            };
            const float2 p1 = kc(0), p2 = kc(1), g1 = kc(2), g2 = kc(3);
            const float2 g3dq = mul2(mul2(p1, f2(g.c_s3, g.c_s3)), dq);  // S3 = P1 c_s3
            put(BEHF_P, sub2(own(6), fma2(p1, dv, mul2(p2, dq))));
            put(BEHF_SXX, add2(own(0), fma2(g1, add2(uyy, uzz), fma2(g2, uxx, g3dq))));
            put(BEHF_SYY, add2(own(1), fma2(g1, add2(uxx, uzz), fma2(g2, uyy, g3dq))));
            put(BEHF_SZZ, add2(own(2), fma2(g1, add2(uxx, uyy), fma2(g2, uzz, g3dq))));
            put(BEHF_SXY, fma2(kc(4), add2(uxy, uyx), own(3)));
            put(BEHF_SXZ, fma2(kc(5), add2(uxz, uzx), own(4)));
            put(BEHF_SYZ, fma2(kc(6), add2(uyz, uzy), own(5)));
            };
            if (wfull) update(std::true_type{});
            else update(std::false_type{});
        }
        __syncwarp();
        if (tx == 0) mbar_arrive(&bempty[st]);
    }
    if (failed) atomicExch(g.err, 1);
    tm_fence_before();
    bar_compute();
    if (ty == 0) {
        tm_fence_after();
        tm_dealloc(tbase);
    }
}

}  // namespace BEHF_TILED_NAMESPACE
}  // namespace behf
