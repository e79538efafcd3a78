// adjoint.cu -- discrete adjoint of one BEHF step and the coefficient-build transpose.
//
// The transpose of the forward kernels of kernels_plain.cu (which restate kernel.cu:172-225 for V and
// kernel.cu:430-490 for T; the reference itself has no adjoint).  Notation for one cell (adjoints l*):
//   T:  p' = p - P1 sum(du) - P2 sum(dw),  s_ii' = s_ii + S1 (du_jj + du_kk) + S2 du_ii + S3 sum(dw),
//       s_ij' = s_ij + S_ij (du_ij + du_ji)
//     -> derivative-group adjoints  lD_ii = -P1 lp + S2 ls_ii + S1 (ls_jj + ls_kk),  lD_w = -P2 lp + S3 sum(ls_ii),
//        lD_ij = S_ij ls_ij;  gradients  gP1 += -lp sum(du), gS2 += sum(ls_ii du_ii), ...
//   V:  q' = VW1 q - VW2 Sigma - VW3 Dp,  v' = v + VU1 Sigma - VU2 (q' - q)
//     -> mu = lq' - VU2 lv',  lq = VW1 mu + VU2 lv',  lSigma = VU1 lv' - VW2 mu,  lDp = -VW3 mu;
//        gradients  gVW1 += mu q, gVW2 += -mu Sigma, gVW3 += -mu Dp, gVU1 += lv' Sigma, gVU2 += -lv' (q' - q).
//   CPML (forward  psi' = A psi + B (A prev + D), prev' = D, D~ = D + psi'):
//        lD = lD~ + B (lpsi + lD~) + lprev;  then  lpsi = A (lpsi + lD~),  lprev = A B (lpsi_old + lD~).
//   A forward difference's transpose is minus the backward difference of the adjoint and vice versa.
#include <algorithm>

#include "behf_adjoint.cuh"

namespace behf {
namespace {

__device__ __forceinline__ long long slab_off(const Geom& g, int ax, int i, int j, int k, int s) {
    return ax == 0 ? ((long long)k * g.ny + j) * g.W + s
         : ax == 1 ? ((long long)k * g.W + s) * g.nx + i
                   : ((long long)s * g.ny + j) * g.nx + i;
}

__device__ __forceinline__ bool interior(const Geom& g, int i, int j, int k) {
    return g.W == 0 ||
           (slab_index(i, g.nx, g.L) < 0 && slab_index(j, g.ny, g.L) < 0 && slab_index(k, g.nz, g.L) < 0);
}

template <class S, int R>
struct Adj {
    typedef Traits<S> T;
    typedef typename T::C A;
    typedef typename T::K K;
    typedef typename T::W W;

    // forward snapshot (storage units)
    static __device__ __forceinline__ A ls(const void* f, long long o) { return T::ld(reinterpret_cast<const S*>(f)[o]); }
    static __device__ __forceinline__ A fwd(const void* f, long long o, long long s) {
        A acc = (A)stencil_w<R>(1) * (ls(f, o + s) - ls(f, o));
#pragma unroll
        for (int m = 2; m <= R; m++) acc += (A)stencil_w<R>(m) * (ls(f, o + m * s) - ls(f, o - (m - 1) * s));
        return acc;
    }
    static __device__ __forceinline__ A bwd(const void* f, long long o, long long s) {
        A acc = (A)stencil_w<R>(1) * (ls(f, o) - ls(f, o - s));
#pragma unroll
        for (int m = 2; m <= R; m++) acc += (A)stencil_w<R>(m) * (ls(f, o + (m - 1) * s) - ls(f, o - m * s));
        return acc;
    }
    static __device__ __forceinline__ A* ad(void* f) { return reinterpret_cast<A*>(f); }
    static __device__ __forceinline__ A coef(const Geom& g, const DevPtrs& p, int j, long long o) {
        const A v = (A)T::ldk(reinterpret_cast<const K*>(p.k[j])[o]);
        if constexpr (sizeof(A) == 8) return v * (A)g.kmuld[j];
        else return v * g.kmulf[j];
    }
    static __device__ __forceinline__ A vw1(const DevPtrs& p, int a, long long o) {
        return (A)reinterpret_cast<const W*>(p.k[VW1X + a])[o];
    }
    static __device__ __forceinline__ A prof(const void* v, int i) { return reinterpret_cast<const A*>(v)[i]; }

};

// Adjoint CPML memory update  lpsi = A (lpsi + lD),  lprv = A B (lpsi_old + lD)  of the four slots SB..SB+3 on
// every slab axis of one cell, split into a load phase and a store phase so that a kernel can issue all of a
// cell's loads before its first store.  Bit q of H set: slot SB+q uses the half-shifted profiles.
template <class A, int SB, int H>
struct MemUpd {
    A L[3][4], pa[3], pb[3];
    long long so[3];
    int s[3];
    __device__ __forceinline__ void load(const Geom& g, const DevPtrs& p, const AdjPtrs& a, int i, int j, int k) {
        s[0] = slab_index(i, g.nx, g.L);
        s[1] = slab_index(j, g.ny, g.L);
        s[2] = slab_index(k, g.nz, g.L);
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            if (s[ax] < 0) continue;
            const int pos = ax == 0 ? i : ax == 1 ? j : k;
            so[ax] = slab_off(g, ax, i, j, k, s[ax]);
            pa[ax] = reinterpret_cast<const A*>(p.pa[ax])[pos];
            pb[ax] = reinterpret_cast<const A*>(p.pb[ax])[pos];
#pragma unroll
            for (int q = 0; q < 4; q++) L[ax][q] = reinterpret_cast<const A*>(a.lpsi[ax][SB + q])[so[ax]];
        }
        if (H != 0) {  // the half-shifted profiles replace pa, pb for the flagged slots
#pragma unroll
            for (int ax = 0; ax < 3; ax++) {
                if (s[ax] < 0) continue;
                const int pos = ax == 0 ? i : ax == 1 ? j : k;
                pa2_[ax] = reinterpret_cast<const A*>(p.pa2[ax])[pos];
                pb2_[ax] = reinterpret_cast<const A*>(p.pb2[ax])[pos];
            }
        }
    }
    A pa2_[3], pb2_[3];
    __device__ __forceinline__ void store(const AdjPtrs& a, const A (&D)[3][4]) const {
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            if (s[ax] < 0) continue;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const bool h = (H >> q) & 1;
                const A Ap = h ? pa2_[ax] : pa[ax], B = h ? pb2_[ax] : pb[ax];
                const A Lm = L[ax][q] + D[ax][q];
                reinterpret_cast<A*>(a.lpsi[ax][SB + q])[so[ax]] = Ap * Lm;
                reinterpret_cast<A*>(a.lprv[ax][SB + q])[so[ax]] = Ap * B * Lm;
            }
        }
    }
};

#define CELL_INDEX                                                      \
    const int i = blockIdx.x * blockDim.x + threadIdx.x + R;            \
    const int j = blockIdx.y * blockDim.y + threadIdx.y + R;            \
    const int k = blockIdx.z + R;                                       \
    if (i >= g.nx - R || j >= g.ny - R || k >= g.nz - R) return;        \
    const long long sy = g.px, sz = g.plane;                            \
    const long long c = k * sz + j * sy + i;                            \
    (void)sy;                                                           \
    (void)sz;

// ------------------------------------------------------------------------------------------- step^T
// Per backward step: record^T (separate, atomic), then
//   k_adj_a  T^T per cell: derivative-group adjoints tmpT[7] (0 uxx, 1 uyy, 2 uzz, 3 w, 4 xy, 5 xz, 6 yz) and
//            the T-coefficient gradients;
//   k_gather<.., 0>  the T^T gather into lv, lq, the V-slot adjoint memory update of the previous backward
//            step (from its tmpV at this cell), then V^T per cell: tmpV[6] (0..2 Sigma_x,y,z, 3..5 Dp_x,y,z)
//            and the V-coefficient gradients;
//   k_gather<.., 1>  the V^T gather into ls, lp and the T-slot adjoint memory update of this step.
// A gather reads the adjoint memory of its own slots only, and each memory update runs after every gather
// that reads those slots.
template <class S, int R>
__global__ void __launch_bounds__(256) k_adj_a(Geom g, DevPtrs p, AdjPtrs a, int first) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
    CELL_INDEX
    // Every load of the cell is issued before its first store: the arrays never alias, but the compiler cannot
    // know that, and each store between two loads would cost one memory round trip.
    A lt[7];  // 0 sxx, 1 syy, 2 szz, 3 sxy, 4 sxz, 5 syz, 6 p
#pragma unroll
    for (int q = 0; q < 7; q++) lt[q] = Q::ad(a.lf[BEHF_SXX + q])[c];
    A kc[8];  // P1, P2, S1, S2, S3, SXYC, SXZC, SYZC
#pragma unroll
    for (int q = 0; q < 8; q++) kc[q] = Q::coef(g, p, P1 + q, c);
    const bool slab = !interior(g, i, j, k);
    const bool gr = a.grad && !slab;
    A du[10], go[8];
    if (gr) {
        du[0] = Q::bwd(a.cur[BEHF_VX], c, 1);   // uxx
        du[1] = Q::bwd(a.cur[BEHF_VY], c, sy);  // uyy
        du[2] = Q::bwd(a.cur[BEHF_VZ], c, sz);  // uzz
        du[3] = Q::bwd(a.cur[BEHF_QX], c, 1) + Q::bwd(a.cur[BEHF_QY], c, sy) + Q::bwd(a.cur[BEHF_QZ], c, sz);
        du[4] = Q::fwd(a.cur[BEHF_VX], c, sy);  // uxy
        du[5] = Q::fwd(a.cur[BEHF_VY], c, 1);   // uyx
        du[6] = Q::fwd(a.cur[BEHF_VX], c, sz);  // uxz
        du[7] = Q::fwd(a.cur[BEHF_VZ], c, 1);   // uzx
        du[8] = Q::fwd(a.cur[BEHF_VY], c, sz);  // uyz
        du[9] = Q::fwd(a.cur[BEHF_VZ], c, sy);  // uzy
#pragma unroll
        for (int q = 0; q < 8; q++) go[q] = Q::ad(a.g[P1 + q])[c];
    }
    // V-slot adjoint memory of the previous backward step: its tmpV at this cell (read by the V^T gather of that
    // step, which has completed), on slab cells
    const bool mem = slab && g.W > 0 && !first;
    A tv[6];
    MemUpd<A, 0, 0x3> mv;
    if (mem) {
#pragma unroll
        for (int q = 0; q < 6; q++) tv[q] = Q::ad(a.tmpV[q])[c];
        mv.load(g, p, a, i, j, k);
    }
    const A lp = lt[6], lxx = lt[0], lyy = lt[1], lzz = lt[2];
    const A p1 = kc[0], p2 = kc[1], s1 = kc[2], s2 = kc[3], s3 = kc[4];
    Q::ad(a.tmpT[0])[c] = -p1 * lp + s2 * lxx + s1 * (lyy + lzz);
    Q::ad(a.tmpT[1])[c] = -p1 * lp + s2 * lyy + s1 * (lxx + lzz);
    Q::ad(a.tmpT[2])[c] = -p1 * lp + s2 * lzz + s1 * (lxx + lyy);
    Q::ad(a.tmpT[3])[c] = -p2 * lp + s3 * (lxx + lyy + lzz);
    Q::ad(a.tmpT[4])[c] = kc[5] * lt[3];
    Q::ad(a.tmpT[5])[c] = kc[6] * lt[4];
    Q::ad(a.tmpT[6])[c] = kc[7] * lt[5];
    if (gr) {
        const A uxx = du[0], uyy = du[1], uzz = du[2], dq = du[3];
        Q::ad(a.g[P1])[c] = go[0] - lp * (uxx + uyy + uzz);
        Q::ad(a.g[P2])[c] = go[1] - lp * dq;
        Q::ad(a.g[S1])[c] = go[2] + lxx * (uyy + uzz) + lyy * (uxx + uzz) + lzz * (uxx + uyy);
        Q::ad(a.g[S2])[c] = go[3] + lxx * uxx + lyy * uyy + lzz * uzz;
        Q::ad(a.g[S3])[c] = go[4] + (lxx + lyy + lzz) * dq;
        Q::ad(a.g[SXYC])[c] = go[5] + lt[3] * (du[4] + du[5]);
        Q::ad(a.g[SXZC])[c] = go[6] + lt[4] * (du[6] + du[7]);
        Q::ad(a.g[SYZC])[c] = go[7] + lt[5] * (du[8] + du[9]);
    }
    if (mem) {
        // axis x: Sigma_x s0h, Dp_x s1h, Sigma_y s2, Sigma_z s3; y: Sigma_y, Dp_y, Sigma_x, Sigma_z;
        // z: Sigma_z, Dp_z, Sigma_x, Sigma_y
        const A D[3][4] = {{tv[0], tv[3], tv[1], tv[2]}, {tv[1], tv[4], tv[0], tv[2]}, {tv[2], tv[5], tv[0], tv[1]}};
        mv.store(a, D);
    }
}

// Gathers, z-marching: a 32 x 8 block owns an xy tile and walks a z range.  Each gather needs 12 corrected
// derivative-group adjoints: 4 with x stencils (staged per plane in shared memory with an x halo of R), 4 with
// y stencils (shared memory, y halo R) and 4 with z stencils (a shared-memory ring of the 2R+2 planes k-R ..
// k+R+1, each thread reading its own column).  Everything for plane k+1 is copied (cp.async, 16-byte chunks
// where the tile rows are 16-byte aligned) while plane k is computed.
// "Corrected" = the adjoint CPML correction of the stencil's own axis and slot applied at the cell it was read
// from: lD = lD~ + B (lpsi + lD~) + lprev on slab cells, lD~ elsewhere (zero off the updated cells).
constexpr int GX = 32, GY = 8;

struct StageSet {
    const void* arr[3][4];  // [axis][k]
    int slot[3][4];
    int half[3][4];
};

template <class S, int R>
struct G25 {
    typedef typename Traits<S>::C A;
    template <bool CHK>
    static __device__ __forceinline__ A corr(const Geom& g, const DevPtrs& p, const AdjPtrs& a, const void* arr,
                                             int ax, int slot, int half, int x, int y, int k) {
        if (x < 0 || x >= g.nx || y < 0 || y >= g.ny) return (A)0;
        A v = reinterpret_cast<const A*>(arr)[(long long)k * g.plane + (long long)y * g.px + x];
        if (CHK && g.W > 0) {
            const int pos = ax == 0 ? x : ax == 1 ? y : k;
            const int s = slab_index(pos, ax == 0 ? g.nx : ax == 1 ? g.ny : g.nz, g.L);
            if (s >= 0) {
                const long long so = slab_off(g, ax, x, y, k, s);
                const A B = reinterpret_cast<const A*>(half ? p.pb2[ax] : p.pb[ax])[pos];
                v += B * (reinterpret_cast<const A*>(a.lpsi[ax][slot])[so] + v) +
                     reinterpret_cast<const A*>(a.lprv[ax][slot])[so];
            }
        }
        return v;
    }
    // the CPML correction of a value already loaded (two independent loads on slab cells)
    static __device__ __forceinline__ A fix(const Geom& g, const DevPtrs& p, const AdjPtrs& a, A v, int ax, int slot,
                                            int half, int x, int y, int k) {
        if (x < 0 || x >= g.nx || y < 0 || y >= g.ny) return v;
        const int pos = ax == 0 ? x : ax == 1 ? y : k;
        const int s = slab_index(pos, ax == 0 ? g.nx : ax == 1 ? g.ny : g.nz, g.L);
        if (s < 0) return v;
        const long long so = slab_off(g, ax, x, y, k, s);
        const A B = reinterpret_cast<const A*>(half ? p.pb2[ax] : p.pb[ax])[pos];
        return v + B * (reinterpret_cast<const A*>(a.lpsi[ax][slot])[so] + v) +
               reinterpret_cast<const A*>(a.lprv[ax][slot])[so];
    }
    // w[d + R] = L[c + d]:  fwdL = sum_m w_m (L[+m] - L[1-m]),  bwdL = sum_m w_m (L[m-1] - L[-m])
    template <class F>
    static __device__ __forceinline__ A fwd(F w) {
        A acc = 0;
#pragma unroll
        for (int m = 1; m <= R; m++) acc += (A)stencil_w<R>(m) * (w(m) - w(1 - m));
        return acc;
    }
    template <class F>
    static __device__ __forceinline__ A bwd(F w) {
        A acc = 0;
#pragma unroll
        for (int m = 1; m <= R; m++) acc += (A)stencil_w<R>(m) * (w(m - 1) - w(-m));
        return acc;
    }
};

// Asynchronous global -> shared copies (cp.async, no registers held): the first `bytes` bytes come from src,
// the rest of the BYTES is zero-filled (bytes = 0 reads nothing).
__device__ __forceinline__ uint32_t sh_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }
template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src, int bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(sh_u32(dst)), "l"(src), "n"(BYTES), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Dynamic shared memory of a gather CTA (elements of A): two plane buffers of the x windows [4][GY][XWP] and
// of the y windows [4][YH][GX], then the z ring [4][ZS][GY * GX].  Rows of the x window start at the 16-byte
// aligned column i0 - R = 32 bx and are padded to whole 16-byte chunks; y-window and z-ring rows start at
// i0 = R + 32 bx, 16-byte aligned when R * sizeof(A) is (YV), else copied element by element.
template <class S, int R>
struct GMap {
    typedef typename Traits<S>::C A;
    static constexpr int CH = 16 / (int)sizeof(A);
    static constexpr int XW = GX + 2 * R;
    static constexpr int XWP = (XW + CH - 1) / CH * CH;
    static constexpr int YH = GY + 2 * R;
    static constexpr int ZS = 2 * R + 2;
    static constexpr bool YV = (R * (int)sizeof(A)) % 16 == 0;
    static constexpr int XB = 4 * GY * XWP, YB = 4 * YH * GX;
    static constexpr int X_OFF = 0, Y_OFF = 2 * XB, Z_OFF = Y_OFF + 2 * YB;
    static constexpr int BYTES = (Z_OFF + 4 * ZS * GY * GX) * (int)sizeof(A);
};

// KIND 0: T^T gather (X: T0 s4, T4 s6h, T5 s7h, T3 s5;  Y: T1 s4, T4 s6h, T6 s7h, T3 s5;
//                      Z: T2 s4, T5 s6h, T6 s7h, T3 s5), then V^T per cell.
// KIND 1: V^T gather (X: V0 s0h, V1 s2, V2 s3, V3 s1h;  Y: V1 s0h, V0 s2, V2 s3, V4 s1h;
//                      Z: V2 s0h, V0 s2, V1 s3, V5 s1h), then the T-slot memory update.
template <class S, int R, int KIND>
__global__ void __launch_bounds__(256, 2) k_gather(Geom g, DevPtrs p, AdjPtrs a, StageSet ss, int zc) {
    typedef G25<S, R> W;
    typedef Adj<S, R> Q;
    typedef GMap<S, R> M;
    typedef typename W::A A;
    extern __shared__ __align__(16) unsigned char gsm_raw[];
    A* const gsm = reinterpret_cast<A*>(gsm_raw);
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * GX + tx;
    const int i0 = R + blockIdx.x * GX, j0 = R + blockIdx.y * GY;
    const int i = i0 + tx, j = j0 + ty;
    const bool valid = i < g.nx - R && j < g.ny - R;
    const int kb = R + blockIdx.z * zc, ke = min(kb + zc, g.nz - R);
    if (kb >= ke) return;
    const long long sy = g.px, sz = g.plane;
    static_assert(M::YH <= 16 && M::XWP <= 64, "window larger than the block's copy pattern");
    auto shx = [&](int bf, int q, int r, int col) -> A& { return gsm[M::X_OFF + bf * M::XB + (q * GY + r) * M::XWP + col]; };
    auto shy = [&](int bf, int q, int r, int col) -> A& { return gsm[M::Y_OFF + bf * M::YB + (q * M::YH + r) * GX + col]; };
    auto zr = [&](int q, int slot) -> A* { return gsm + M::Z_OFF + (q * M::ZS + slot) * (GY * GX); };
    // block-uniform: does the x (y) window of this tile reach a CPML slab of its axis?
    const bool cx = g.W > 0 && (i0 - R < g.L || i0 + GX + R > g.nx - 1 - g.L);
    const bool cy = g.W > 0 && (j0 - R < g.L || j0 + GY + R > g.ny - 1 - g.L);
    // bytes of the 16-byte chunk at column x that lie inside the grid (rows outside it: 0)
    auto chunk_bytes = [&](int x, int y) {
        const int n = (g.nx - x) * (int)sizeof(A);
        return (y >= g.ny || n <= 0) ? 0 : (n < 16 ? n : 16);
    };
    // z ring: plane zz of the four z-stencil arrays into its slot (CPML-corrected element by element on a z-slab plane)
    auto zfill = [&](int zz) {
        const int slot = zz % M::ZS;
        const bool zslab = g.W > 0 && slab_index(zz, g.nz, g.L) >= 0;
        if (zslab || !M::YV) {
            if (valid) {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if (zslab) {
                        zr(q, slot)[t] = W::template corr<true>(g, p, a, ss.arr[2][q], 2, ss.slot[2][q], ss.half[2][q],
                                                                i, j, zz);
                    } else {
                        cp_async<sizeof(A)>(zr(q, slot) + t,
                                            reinterpret_cast<const A*>(ss.arr[2][q]) + zz * sz + j * sy + i,
                                            (int)sizeof(A));
                    }
                }
            }
        } else {
            // warp ty copies row ty: (array, chunk) pairs over the lanes
            constexpr int NCH = GX / M::CH;
            for (int u = tx; u < 4 * NCH; u += 32) {
                const int q = u / NCH, ch = u % NCH;
                const int x = i0 + ch * M::CH, y = j;
                const int nb = chunk_bytes(x, y);
                const long long off = nb ? zz * sz + (long long)y * sy + x : 0;
                cp_async<16>(zr(q, slot) + ty * GX + ch * M::CH, reinterpret_cast<const A*>(ss.arr[2][q]) + off, nb);
            }
        }
    };
    // x and y windows of plane kk into buffer bf (zero outside the grid)
    auto issue = [&](int kk, int bf) {
        const long long pk = (long long)kk * sz;
        {  // x window: warp ty copies row ty, 16-byte chunks
            constexpr int NCH = M::XWP / M::CH;
            const int y = j0 + ty;
            for (int u = tx; u < 4 * NCH; u += 32) {
                const int q = u / NCH, ch = u % NCH;
                const int x = i0 - R + ch * M::CH;
                const int nb = chunk_bytes(x, y);
                const long long off = nb ? pk + (long long)y * sy + x : 0;
                cp_async<16>(&shx(bf, q, ty, ch * M::CH), reinterpret_cast<const A*>(ss.arr[0][q]) + off, nb);
            }
        }
        if (M::YV) {  // y window: the YH rows x 4 arrays x (GX / CH) chunks over the block
            constexpr int NCH = GX / M::CH;
            for (int u = t; u < M::YH * 4 * NCH; u += GX * GY) {
                const int ch = u % NCH, rq = u / NCH, q = rq % 4, r = rq / 4;
                const int x = i0 + ch * M::CH, y = j0 - R + r;
                const int nb = chunk_bytes(x, y);
                const long long off = nb ? pk + (long long)y * sy + x : 0;
                cp_async<16>(&shy(bf, q, r, ch * M::CH), reinterpret_cast<const A*>(ss.arr[1][q]) + off, nb);
            }
        } else {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int r = ty + 8 * h;
                if (r < M::YH) {
                    const int x = i0 + tx, y = j0 - R + r;
                    const bool in = x < g.nx && y < g.ny;
                    const long long off = in ? pk + (long long)y * sy + x : 0;
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        cp_async<sizeof(A)>(&shy(bf, q, r, tx), reinterpret_cast<const A*>(ss.arr[1][q]) + off,
                                            in ? (int)sizeof(A) : 0);
                }
            }
        }
    };
    for (int zz = kb - R; zz <= kb + R; zz++) zfill(zz);
    issue(kb, 0);
    cp_async_commit();
    for (int k = kb; k < ke; k++) {
        const int bf = (k - kb) & 1;
        if (k + 1 < ke) {
            // the other window buffer and the ring slot of plane k - R - 1 were released by the barrier that ended
            // plane k - 1
            issue(k + 1, bf ^ 1);
            zfill(k + 1 + R);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        if (cx || cy) {  // CPML corrections of the copied windows near a slab (all loads, then the writes)
            A fxv[2][4], fyv[2][4];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int cc = tx + 32 * h, r = ty + 8 * h;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if (cx && cc < M::XW)
                        fxv[h][q] = W::fix(g, p, a, shx(bf, q, ty, cc), 0, ss.slot[0][q], ss.half[0][q], i0 - R + cc,
                                           j0 + ty, k);
                    if (cy && r < M::YH)
                        fyv[h][q] = W::fix(g, p, a, shy(bf, q, r, tx), 1, ss.slot[1][q], ss.half[1][q], i0 + tx,
                                           j0 - R + r, k);
                }
            }
            __syncthreads();  // every thread has read the raw windows
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int cc = tx + 32 * h, r = ty + 8 * h;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if (cx && cc < M::XW) shx(bf, q, ty, cc) = fxv[h][q];
                    if (cy && r < M::YH) shy(bf, q, r, tx) = fyv[h][q];
                }
            }
            __syncthreads();
        }
        if (valid) {
            const long long c = k * sz + j * sy + i;
            int zs[2 * R + 1];  // ring slots of planes k-R .. k+R
#pragma unroll
            for (int d = 0; d <= 2 * R; d++) zs[d] = (k - R + d) % M::ZS;
#define WX(q) [&](int d) { return shx(bf, q, ty, tx + R + d); }
#define WY(q) [&](int d) { return shy(bf, q, ty + R + d, tx); }
#define WZ(q) [&](int d) { return zr(q, zs[R + d])[t]; }
            // Each cell issues all its global loads before its first global store (see k_adj_a).
            if (KIND == 0) {
                // V^T at this cell with lv = lv_old - dl[0..2], lq' = lq_old - dl[3..5]
                A lvo[3], lqo[3], vu2[3], vw1[3], vu1[3], vw2[3], vw3[3];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    lvo[d] = Q::ad(a.lf[BEHF_VX + d])[c];
                    lqo[d] = Q::ad(a.lf[BEHF_QX + d])[c];
                    vu2[d] = Q::coef(g, p, VU2X + d, c);
                    vw1[d] = Q::vw1(p, d, c);
                    vu1[d] = Q::coef(g, p, VU1X + d, c);
                    vw2[d] = Q::coef(g, p, VW2X + d, c);
                    vw3[d] = Q::coef(g, p, (d == 2 && g.bug) ? VW3Y : VW3X + d, c);  // reference: vz uses VW3y
                }
                const bool gr = a.grad && interior(g, i, j, k);
                A sum[3], dp[3], qo[3], qn[3], go[15];
                if (gr) {
                    sum[0] = Q::fwd(a.cur[BEHF_SXX], c, 1) + Q::bwd(a.cur[BEHF_SXY], c, sy) + Q::bwd(a.cur[BEHF_SXZ], c, sz);
                    sum[1] = Q::fwd(a.cur[BEHF_SYY], c, sy) + Q::bwd(a.cur[BEHF_SXY], c, 1) + Q::bwd(a.cur[BEHF_SYZ], c, sz);
                    sum[2] = Q::fwd(a.cur[BEHF_SZZ], c, sz) + Q::bwd(a.cur[BEHF_SXZ], c, 1) + Q::bwd(a.cur[BEHF_SYZ], c, sy);
                    dp[0] = Q::fwd(a.cur[BEHF_P], c, 1);
                    dp[1] = Q::fwd(a.cur[BEHF_P], c, sy);
                    dp[2] = Q::fwd(a.cur[BEHF_P], c, sz);
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        qo[d] = Q::ls(a.qprev[d], c);
                        qn[d] = Q::ls(a.cur[BEHF_QX + d], c);
                    }
#pragma unroll
                    for (int q = 0; q < 15; q++) go[q] = Q::ad(a.g[q])[c];
                }
                A dl[6];
                dl[0] = W::fwd(WX(0)) + W::bwd(WY(1)) + W::bwd(WZ(1));
                dl[1] = W::fwd(WY(0)) + W::bwd(WX(1)) + W::bwd(WZ(2));
                dl[2] = W::fwd(WZ(0)) + W::bwd(WX(2)) + W::bwd(WY(2));
                dl[3] = W::fwd(WX(3));
                dl[4] = W::fwd(WY(3));
                dl[5] = W::fwd(WZ(3));
                A mu[3], lv[3];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    lv[d] = lvo[d] - dl[d];
                    const A lq = lqo[d] - dl[3 + d];
                    mu[d] = lq - vu2[d] * lv[d];
                    Q::ad(a.lf[BEHF_VX + d])[c] = lv[d];
                    Q::ad(a.lf[BEHF_QX + d])[c] = vw1[d] * mu[d] + vu2[d] * lv[d];
                    Q::ad(a.tmpV[d])[c] = vu1[d] * lv[d] - vw2[d] * mu[d];
                    Q::ad(a.tmpV[3 + d])[c] = -vw3[d] * mu[d];
                }
                if (gr) {
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        go[VW1X + d] += mu[d] * qo[d];
                        go[VW2X + d] += -mu[d] * sum[d];
                        go[VU1X + d] += lv[d] * sum[d];
                        go[VU2X + d] += -lv[d] * (qn[d] - qo[d]);
                    }
                    go[VW3X] += -mu[0] * dp[0];
                    const A w3z = -mu[2] * dp[2];
                    go[VW3Y] += -mu[1] * dp[1] + (g.bug ? w3z : (A)0);
                    go[VW3Z] += g.bug ? (A)0 : w3z;
#pragma unroll
                    for (int q = 0; q < 15; q++) Q::ad(a.g[q])[c] = go[q];
                }
            } else {
                A lo[7];  // sxx syy szz sxy sxz syz p
#pragma unroll
                for (int q = 0; q < 7; q++) lo[q] = Q::ad(a.lf[BEHF_SXX + q])[c];
                // T-slot adjoint memory of this step on slab cells (its gathers ran in the KIND 0 launch)
                const bool mem = !interior(g, i, j, k);
                A tt[7];
                MemUpd<A, 4, 0xC> mt;
                if (mem) {
#pragma unroll
                    for (int q = 0; q < 7; q++) tt[q] = Q::ad(a.tmpT[q])[c];
                    mt.load(g, p, a, i, j, k);
                }
                Q::ad(a.lf[BEHF_SXX])[c] = lo[0] - W::bwd(WX(0));
                Q::ad(a.lf[BEHF_SYY])[c] = lo[1] - W::bwd(WY(0));
                Q::ad(a.lf[BEHF_SZZ])[c] = lo[2] - W::bwd(WZ(0));
                Q::ad(a.lf[BEHF_SXY])[c] = lo[3] - (W::fwd(WY(1)) + W::fwd(WX(1)));
                Q::ad(a.lf[BEHF_SXZ])[c] = lo[4] - (W::fwd(WZ(1)) + W::fwd(WX(2)));
                Q::ad(a.lf[BEHF_SYZ])[c] = lo[5] - (W::fwd(WZ(2)) + W::fwd(WY(2)));
                Q::ad(a.lf[BEHF_P])[c] = lo[6] - (W::bwd(WX(3)) + W::bwd(WY(3)) + W::bwd(WZ(3)));
                if (mem) {
                    // axis x: uxx s4, wx s5, uyx s6h, uzx s7h; y: uyy, wy, uxy, uzy; z: uzz, wz, uxz, uyz
                    const A D[3][4] = {{tt[0], tt[3], tt[4], tt[5]}, {tt[1], tt[3], tt[4], tt[6]},
                                       {tt[2], tt[3], tt[5], tt[6]}};
                    mt.store(a, D);
                }
            }
#undef WX
#undef WY
#undef WZ
        }
        __syncthreads();
    }
}

#undef CELL_INDEX

// ------------------------------------------------------------------------------------------- record^T, source^T
template <class A>
__global__ void k_adj_record(AdjPtrs a, const long long* off, const int* comp, int nrec, const double* adj, int nt,
                             int it, AdjScales sc) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const int q = comp[r];
    atomicAdd(reinterpret_cast<A*>(a.lf[q]) + off[r], (A)(adj[(long long)r * nt + it] * sc.s[q]));
}

template <class A>
__global__ void k_adj_point(AdjPtrs a, long long o, int kind, double fac, const float* w, int nw, int it, double* gw,
                            double* gfac) {
    auto L = [&](int q) { return (double)reinterpret_cast<const A*>(a.lf[q])[o]; };
    if (kind == BEHF_SRC_FORCE_Z) {  // injected into vz between V and T; V^T leaves lv unchanged
        const double lvz = L(BEHF_VZ);
        gw[it] = fac * lvz;
        if (it < nw) *gfac += (double)w[it] * lvz;  // samples past the wavelet are not injected
    } else if (kind == BEHF_SRC_EXPLOSIVE) {
        gw[it] = fac * (L(BEHF_SXX) + L(BEHF_SYY) + L(BEHF_SZZ));
    } else {
        gw[it] = fac * L(BEHF_P);
    }
}

// ------------------------------------------------------------------------------------------- coefficient transpose
template <class A>
__global__ void k_grad_moduli(GradModArgs a) {
    const long long N = (long long)a.nx * a.ny * a.nz;
    const long long sy = a.nx, sz = (long long)a.nx * a.ny;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < N; m += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(m % a.nx);
        const long long r = m / a.nx;
        const int j = (int)(r % a.ny), k = (int)(r / a.ny);
        const int n3[3] = {a.nx, a.ny, a.nz}, x3[3] = {i, j, k};
        bool in = true;
        for (int d = 0; d < 3; d++) {
            const int lo = max(a.L, a.R) + 1;
            const int hi = a.L > 0 ? min(n3[d] - 2 - a.L, n3[d] - a.R - 1) : n3[d] - a.R - 1;
            in = in && x3[d] >= lo && x3[d] <= hi;
        }
        double acc[kNMod];
#pragma unroll
        for (int q = 0; q < kNMod; q++) acc[q] = 0.0;
        if (in) {
            auto md = [&](int q, long long o) { return (double)a.mod[q][o]; };
            // effective -> physical coefficient gradient at coefficient cell c (pitched index pc)
            auto gp = [&](int q, long long c) {
                const long long ci = c / sz, cj = (c / sy) % a.ny, cx = c % sy;
                return (double)reinterpret_cast<const A*>(a.g[q])[ci * a.plane + cj * a.px + cx] * a.ratio[q];
            };
            const double dt = a.dt;
            acc[BEHF_C] += (gp(P1, m) + gp(S3, m)) * dt;
            acc[BEHF_M] += gp(P2, m) * dt;
            acc[BEHF_H2U] += gp(S1, m) * dt;
            acc[BEHF_HH] += gp(S2, m) * dt;
            // harmonic shear averages: coefficient cell c = m - o for the four offsets o of each pair
            const long long ex[3] = {1, sy, sz};
            const int pairs[3][2] = {{0, 2}, {1, 2}, {0, 1}};  // SXZC, SYZC, SXYC
            const int pcoef[3] = {SXZC, SYZC, SXYC};
            const double mu_m = md(BEHF_MU, m);
            if (mu_m != 0.0) {
                for (int h = 0; h < 3; h++) {
                    const long long e1 = ex[pairs[h][0]], e2 = ex[pairs[h][1]];
                    const long long offs[4] = {0, e1, e2, e1 + e2};
                    for (int o = 0; o < 4; o++) {
                        const long long c = m - offs[o];
                        const double v0 = md(BEHF_MU, c), v1 = md(BEHF_MU, c + e1), v2 = md(BEHF_MU, c + e2),
                                     v3 = md(BEHF_MU, c + e1 + e2);
                        if (v0 == 0 || v1 == 0 || v2 == 0 || v3 == 0) continue;
                        const double hm = 1.0 / (0.25 * (1 / v0 + 1 / v1 + 1 / v2 + 1 / v3));
                        acc[BEHF_MU] += gp(pcoef[h], c) * dt * hm * hm / (4.0 * mu_m * mu_m);
                    }
                }
            }
            // staggered arithmetic averages: coefficient cell c = m (m first) and c = m - e_d (m second)
            for (int s = 0; s < 4; s++) {
                const long long c = s == 0 ? m : m - ex[s - 1];
                double rho[3], rhof[3], b[3], mm[3];
                for (int d = 0; d < 3; d++) {
                    rho[d] = 0.5 * (md(BEHF_RHO, c) + md(BEHF_RHO, c + ex[d]));
                    rhof[d] = 0.5 * (md(BEHF_RHOF, c) + md(BEHF_RHOF, c + ex[d]));
                    b[d] = 0.5 * (md(BEHF_C1, c) + md(BEHF_C1, c + ex[d]));
                    mm[d] = 0.5 * (md(BEHF_C2, c) + md(BEHF_C2, c + ex[d]));
                }
                const bool vw = !(b[0] == 0 || b[1] == 0 || b[2] == 0);
                const bool vu = !(rho[0] == 0 || rho[1] == 0 || rho[2] == 0);
                for (int d = 0; d < 3; d++) {
                    if (s != 0 && d != s - 1) continue;
                    double grho = 0, grhof = 0, gb = 0, gmm = 0;
                    const double rr = rho[d], rf = rhof[d];
                    if (vw) {
                        const double mp = mm[d] - rf * rf / rr;
                        const double D = mp + 0.5 * dt * b[d];
                        const double g1 = gp(VW1X + d, c), g2 = gp(VW2X + d, c), g3 = gp(VW3X + d, c);
                        const double gD = -g2 * dt * (rf / rr) / (D * D) - g3 * dt / (D * D);
                        const double gmp = g1 * (dt * b[d]) / (D * D) + gD;
                        gb += g1 * (-dt * mp / (D * D)) + gD * 0.5 * dt;
                        const double gratio = g2 * dt / D;
                        gmm += gmp;
                        grhof += gmp * (-2.0 * rf / rr) + gratio / rr;
                        grho += gmp * (rf * rf / (rr * rr)) - gratio * rf / (rr * rr);
                    }
                    if (vu) {
                        grho += gp(VU1X + d, c) * (-dt / (rr * rr)) + gp(VU2X + d, c) * (-rf / (rr * rr));
                        grhof += gp(VU2X + d, c) / rr;
                    }
                    acc[BEHF_RHO] += 0.5 * grho;
                    acc[BEHF_RHOF] += 0.5 * grhof;
                    acc[BEHF_C1] += 0.5 * gb;
                    acc[BEHF_C2] += 0.5 * gmm;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < kNMod; q++) a.gm[q][m] = acc[q];
    }
}

template <class S, int R>
cudaError_t adj_r(const Geom& g, const DevPtrs& p, const AdjPtrs& a, int first, cudaStream_t st) {
    const dim3 block(32, 8, 1);
    const int nxu = g.nx - 2 * R, nyu = g.ny - 2 * R, nzu = g.nz - 2 * R;
    const dim3 grid((nxu + 31) / 32, (nyu + 7) / 8, nzu);
    k_adj_a<S, R><<<grid, block, 0, st>>>(g, p, a, first);
    // gathers: z chunks so that about eight CTAs per SM are launched
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 132;
    }
    const int nxy = (int)(((nxu + GX - 1) / GX) * ((nyu + GY - 1) / GY));
    int nch = (8 * sms + nxy - 1) / nxy;
    nch = std::max(1, std::min(nch, std::max(1, nzu / 8)));
    const int zc = (nzu + nch - 1) / nch;
    const dim3 ggrid((nxu + GX - 1) / GX, (nyu + GY - 1) / GY, (nzu + zc - 1) / zc);
    StageSet t{}, v{};
    // T^T gather: x {T0 s4, T4 s6h, T5 s7h, T3 s5}, y {T1 s4, T4 s6h, T6 s7h, T3 s5}, z {T2 s4, T5 s6h, T6 s7h, T3 s5}
    const int tq[3][4] = {{0, 4, 5, 3}, {1, 4, 6, 3}, {2, 5, 6, 3}};
    const int ts[4] = {4, 6, 7, 5}, th[4] = {0, 1, 1, 0};
    const int tz_s[4] = {4, 6, 7, 5};
    // V^T gather: x {V0 s0h, V1 s2, V2 s3, V3 s1h}, y {V1 s0h, V0 s2, V2 s3, V4 s1h}, z {V2 s0h, V0 s2, V1 s3, V5 s1h}
    const int vq[3][4] = {{0, 1, 2, 3}, {1, 0, 2, 4}, {2, 0, 1, 5}};
    const int vs[4] = {0, 2, 3, 1}, vh[4] = {1, 0, 0, 1};
    for (int ax = 0; ax < 3; ax++)
        for (int q = 0; q < 4; q++) {
            t.arr[ax][q] = a.tmpT[tq[ax][q]];
            t.slot[ax][q] = ax == 2 ? tz_s[q] : ts[q];
            t.half[ax][q] = th[q];
            v.arr[ax][q] = a.tmpV[vq[ax][q]];
            v.slot[ax][q] = vs[q];
            v.half[ax][q] = vh[q];
        }
    const int smem = GMap<S, R>::BYTES;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_gather<S, R, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_gather<S, R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_gather<S, R, 0><<<ggrid, block, smem, st>>>(g, p, a, t, zc);
    k_gather<S, R, 1><<<ggrid, block, smem, st>>>(g, p, a, v, zc);
    return cudaGetLastError();
}

}  // namespace

template <class S>
cudaError_t adj_step(const Geom& g, const DevPtrs& p, const AdjPtrs& a, int first, cudaStream_t st) {
    switch (g.R) {
        case 1: return adj_r<S, 1>(g, p, a, first, st);
        case 2: return adj_r<S, 2>(g, p, a, first, st);
        case 3: return adj_r<S, 3>(g, p, a, first, st);
        case 4: return adj_r<S, 4>(g, p, a, first, st);
    }
    return cudaErrorInvalidValue;
}
template <class S>
cudaError_t adj_record(const AdjPtrs& a, const long long* off, const int* comp, int nrec, const double* adj, int nt,
                       int it, const AdjScales& sc, cudaStream_t st) {
    if (nrec <= 0) return cudaSuccess;
    k_adj_record<typename Traits<S>::C><<<(nrec + 255) / 256, 256, 0, st>>>(a, off, comp, nrec, adj, nt, it, sc);
    return cudaGetLastError();
}
template <class S>
cudaError_t adj_point(const AdjPtrs& a, long long o, int kind, double fac, const float* w, int nw, int it, double* gw,
                      double* gfac, cudaStream_t st) {
    k_adj_point<typename Traits<S>::C><<<1, 1, 0, st>>>(a, o, kind, fac, w, nw, it, gw, gfac);
    return cudaGetLastError();
}
template <class A>
cudaError_t adj_grad_moduli(const GradModArgs& a, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_grad_moduli<A><<<(sms > 0 ? sms : 132) * 8, 256, 0, st>>>(a);
    return cudaGetLastError();
}

#define BEHF_ADJ_INST(S)                                                                                         \
    template cudaError_t adj_step<S>(const Geom&, const DevPtrs&, const AdjPtrs&, int, cudaStream_t);          \
    template cudaError_t adj_record<S>(const AdjPtrs&, const long long*, const int*, int, const double*, int, int, \
                                       const AdjScales&, cudaStream_t);                                          \
    template cudaError_t adj_point<S>(const AdjPtrs&, long long, int, double, const float*, int, int, double*,  \
                                      double*, cudaStream_t);
BEHF_ADJ_INST(double)
BEHF_ADJ_INST(float)
BEHF_ADJ_INST(__half)
BEHF_ADJ_INST(__nv_bfloat16)
template cudaError_t adj_grad_moduli<float>(const GradModArgs&, cudaStream_t);
template cudaError_t adj_grad_moduli<double>(const GradModArgs&, cudaStream_t);

}  // namespace behf
