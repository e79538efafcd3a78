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
#include "kernels_tiled.cuh"

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
    // L2 prefetch of element o of an array of element type E (no register is written: the plane's loads that
    // follow find the line in L2 instead of waiting on DRAM)
    template <class E>
    static __device__ __forceinline__ void pf(const void* f, long long o) {
        asm volatile("prefetch.L2 [%0];" ::"l"(reinterpret_cast<const E*>(f) + o));
    }

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
// Backward step n (record^T of step n already applied to the adjoint fields, and T^T per cell of step n already
// done: tmpT[7] (0 uxx, 1 uyy, 2 uzz, 3 w, 4 xy, 5 xz, 6 yz) and the T-coefficient gradients):
//   k_gather<.., 0>  the T^T gather into lv, lq, then V^T per cell: tmpV[6] (0..2 Sigma_x,y,z, 3..5 Dp_x,y,z) and
//            the V-coefficient gradients;
//   k_gather<.., 1>  the V^T gather into ls, lp, the T-slot adjoint memory update of step n, and (fused, n >= 1)
//            T^T per cell of step n - 1 from the new ls, lp (tmpT of step n is read before it is overwritten);
//   k_vmem   the V-slot adjoint memory update of step n on the slab cells (after the V^T gather that reads it);
//   then source^T of step n and record^T of step n - 1, which also adds its injection's share to the fused T^T
//   at the receiver cells (k_adj_recfix).  k_adj_a is T^T per cell for the first backward step only.
// A gather reads the adjoint memory of its own slots only, and each memory update runs after every gather that
// reads those slots.  Every kernel issues all of a cell's global loads before its first global store: the arrays
// never alias, but the compiler cannot know that, and each store between two loads would cost a memory round
// trip.

// T^T per cell: derivative-group adjoints from the stress/pressure adjoints lt (sxx syy szz sxy sxz syz p) and the
// coefficients kc (P1 P2 S1 S2 S3 SXYC SXZC SYZC).
template <class A>
__device__ __forceinline__ void t_groups(const A (&lt)[7], const A (&kc)[8], A (&o)[7]) {
    const A lp = lt[6], lxx = lt[0], lyy = lt[1], lzz = lt[2];
    o[0] = -kc[0] * lp + kc[3] * lxx + kc[2] * (lyy + lzz);
    o[1] = -kc[0] * lp + kc[3] * lyy + kc[2] * (lxx + lzz);
    o[2] = -kc[0] * lp + kc[3] * lzz + kc[2] * (lxx + lyy);
    o[3] = -kc[1] * lp + kc[4] * (lxx + lyy + lzz);
    o[4] = kc[5] * lt[3];
    o[5] = kc[6] * lt[4];
    o[6] = kc[7] * lt[5];
}
// T-coefficient gradient increments (P1 P2 S1 S2 S3 SXYC SXZC SYZC) from lt and the forward derivatives du
// (uxx uyy uzz div-q uxy uyx uxz uzx uyz uzy).
template <class A>
__device__ __forceinline__ void t_grad(const A (&lt)[7], const A (&du)[10], A (&o)[8]) {
    const A lp = lt[6], lxx = lt[0], lyy = lt[1], lzz = lt[2];
    const A uxx = du[0], uyy = du[1], uzz = du[2], dq = du[3];
    o[0] = -lp * (uxx + uyy + uzz);
    o[1] = -lp * dq;
    o[2] = lxx * (uyy + uzz) + lyy * (uxx + uzz) + lzz * (uxx + uyy);
    o[3] = lxx * uxx + lyy * uyy + lzz * uzz;
    o[4] = (lxx + lyy + lzz) * dq;
    o[5] = lt[3] * (du[4] + du[5]);
    o[6] = lt[4] * (du[6] + du[7]);
    o[7] = lt[5] * (du[8] + du[9]);
}
// du at cell c from the forward fields vx vy vz qx qy qz (storage type, direct loads)
template <class S, int R>
__device__ __forceinline__ void vq_derivs(const void* const (&f)[6], long long c, long long sy, long long sz,
                                          typename Traits<S>::C (&du)[10]) {
    typedef Adj<S, R> Q;
    du[0] = Q::bwd(f[0], c, 1);   // uxx
    du[1] = Q::bwd(f[1], c, sy);  // uyy
    du[2] = Q::bwd(f[2], c, sz);  // uzz
    du[3] = Q::bwd(f[3], c, 1) + Q::bwd(f[4], c, sy) + Q::bwd(f[5], c, sz);
    du[4] = Q::fwd(f[0], c, sy);  // uxy
    du[5] = Q::fwd(f[1], c, 1);   // uyx
    du[6] = Q::fwd(f[0], c, sz);  // uxz
    du[7] = Q::fwd(f[2], c, 1);   // uzx
    du[8] = Q::fwd(f[1], c, sz);  // uyz
    du[9] = Q::fwd(f[2], c, sy);  // uzy
}
// The T coefficients at c; with a.derived (the forward ran the tiled kernels, which use S3 = P1 c_s3 instead of
// the stored S3) the derived S3.
template <class S, int R>
__device__ __forceinline__ void t_coefs(const Geom& g, const DevPtrs& p, const AdjPtrs& a, long long c,
                                        typename Traits<S>::C (&kc)[8]) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
#pragma unroll
    for (int q = 0; q < 8; q++)
        if (q != 4) kc[q] = Q::coef(g, p, P1 + q, c);
    kc[4] = a.derived ? kc[0] * (A)g.c_s3 : Q::coef(g, p, S3, c);
}
// With a.derived the S3 gradient belongs to P1 (chain rule through S3 = P1 c_s3); the S3 accumulator is unused.
template <class A>
__device__ __forceinline__ void t_grad_fold(const Geom& g, const AdjPtrs& a, A (&inc)[8]) {
    if (a.derived) {
        inc[0] += (A)g.c_s3 * inc[4];
        inc[4] = 0;
    }
}

// T^T per cell of the first backward step.
template <class S, int R>
__global__ void __launch_bounds__(256) k_adj_a(Geom g, DevPtrs p, AdjPtrs a) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
    CELL_INDEX
    A lt[7], kc[8];
#pragma unroll
    for (int q = 0; q < 7; q++) lt[q] = Q::ad(a.lf[BEHF_SXX + q])[c];
    t_coefs<S, R>(g, p, a, c, kc);
    const bool gr = a.grad && interior(g, i, j, k);
    A du[10], go[8];
    if (gr) {
        const void* const f[6] = {a.cur[BEHF_VX], a.cur[BEHF_VY], a.cur[BEHF_VZ],
                                  a.cur[BEHF_QX], a.cur[BEHF_QY], a.cur[BEHF_QZ]};
        vq_derivs<S, R>(f, c, sy, sz, du);
#pragma unroll
        for (int q = 0; q < 8; q++) go[q] = (q == 4 && a.derived) ? (A)0 : Q::ad(a.g[P1 + q])[c];
    }
    A tg[7];
    t_groups(lt, kc, tg);
#pragma unroll
    for (int q = 0; q < 7; q++) Q::ad(a.tmpT[q])[c] = tg[q];
    if (gr) {
        A inc[8];
        t_grad(lt, du, inc);
        t_grad_fold(g, a, inc);
#pragma unroll
        for (int q = 0; q < 8; q++)
            if (q != 4 || !a.derived) Q::ad(a.g[P1 + q])[c] = go[q] + inc[q];
    }
}

// Gathers, z-marching: a 32 x 8 block owns an xy tile and walks a z range.  Each gather needs 12 corrected
// derivative-group adjoints: 4 with x stencils (x window of the plane, halo R), 4 with y stencils (y window, halo
// R) and 4 with z stencils (a shared-memory ring of the 2R+2 planes k-R .. k+R+1, each thread reading its own
// column).  One thread issues the TMA copies (cp.async.bulk.tensor) of plane k+1 -- its eight windows and the
// ring's new plane k+1+R -- while plane k is computed; a full/empty mbarrier pair per stage orders them, every
// wait is bounded.
// "Corrected" = the adjoint CPML correction of the stencil's own axis and slot applied at the cell it was read
// from: lD = lD~ + B (lpsi + lD~) + lprev on slab cells, lD~ elsewhere (zero off the updated cells); applied in
// shared memory after the copies land (x/y windows of tiles that reach a slab, ring planes inside the z slab).
constexpr int GX = 32, GY = 8;
// Tuning: CTAs per SM the gathers' launch bounds aim for (registers capped at 65536 / (256 MINB)), and whether the
// 16-bit kinds stage the forward snapshot for the gradient stencils (1) or read it from global memory (0).
#ifndef BEHF_ADJ_MINB
#define BEHF_ADJ_MINB 2
#endif
#ifndef BEHF_ADJ_SNAP
#define BEHF_ADJ_SNAP 1
#endif
// 1: the coefficient gradients run in kernels of their own (MODE 2) after register-lean gathers (MODE 1), at
// BEHF_ADJ_MINB_SPLIT CTAs per SM; 0: fused into the gathers (MODE 0).
// at least this many waves of gather CTAs where the z chunking allows it (measured at 256^3, 600-step gradient:
// 4 waves 2.43 s, 8 waves 2.35 s, 16 waves 2.36 s)
#ifndef BEHF_ADJ_MINW
#define BEHF_ADJ_MINW 8
#endif
#ifndef BEHF_ADJ_SPLIT
#define BEHF_ADJ_SPLIT 1
#endif
#ifndef BEHF_ADJ_MINB_SPLIT
#define BEHF_ADJ_MINB_SPLIT 3
#endif
// the split gradient kernels (MODE 2): their CTAs per SM (41 KB of shared memory each; measured at 256^3, 600-step
// gradient: 3 per SM 2.37 s, 4 per SM 2.34 s, 5 per SM, spilling, 2.45 s)
#ifndef BEHF_ADJ_MINB_GRAD
#define BEHF_ADJ_MINB_GRAD 4
#endif
// the split V^T gather (T-slot memory and T^T per cell of the next step): its CTAs per SM
#ifndef BEHF_ADJ_MINB_G1
#define BEHF_ADJ_MINB_G1 3
#endif

// The adjoint CPML memory update of one cell on one slab axis ax (position pos along it, slab offset so), from
// the four derivative-group adjoints D of that axis:  lpsi = A (lpsi + D),  lprv = A B (lpsi_old + D).  TSLOT 0:
// the V slots 0..3 from tmpV (axis x: Sigma_x s0h, Dp_x s1h, Sigma_y s2, Sigma_z s3; y: Sigma_y, Dp_y, Sigma_x,
// Sigma_z; z: Sigma_z, Dp_z, Sigma_x, Sigma_y); TSLOT 1: the T slots 4..7 from tmpT (axis x: uxx s4, wx s5, uyx s6h,
// uzx s7h; y: uyy, wy, uxy, uzy; z: uzz, wz, uxz, uyz; tmpT 0 uxx, 1 uyy, 2 uzz, 3 w, 4 xy, 5 xz, 6 yz); h: the
// half-shifted profiles.  mem_groups gives the tmpT / tmpV index of each slot's D.
template <int TSLOT>
__device__ __forceinline__ void mem_groups(int ax, int (&dq)[4]) {
    dq[0] = ax;
    dq[1] = TSLOT ? 3 : ax + 3;
    dq[2] = TSLOT ? (ax == 2 ? 5 : 4) : (ax == 0 ? 1 : 0);
    dq[3] = TSLOT ? (ax == 0 ? 5 : 6) : (ax == 2 ? 1 : 2);
}
template <class A, int TSLOT>
__device__ __forceinline__ void mem_axis(const DevPtrs& p, const AdjPtrs& a, int ax, int pos, long long so,
                                         const A (&D)[4]) {
    constexpr int SB = TSLOT ? 4 : 0;
    A L[4];
#pragma unroll
    for (int q = 0; q < 4; q++) L[q] = reinterpret_cast<const A*>(a.lpsi[ax][SB + q])[so];
    const A pa = reinterpret_cast<const A*>(p.pa[ax])[pos], pb = reinterpret_cast<const A*>(p.pb[ax])[pos];
    const A pa2 = reinterpret_cast<const A*>(p.pa2[ax])[pos], pb2 = reinterpret_cast<const A*>(p.pb2[ax])[pos];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const bool h = TSLOT ? q >= 2 : q < 2;  // half-shifted profiles: V slots 0, 1; T slots 6, 7
        const A Ap = h ? pa2 : pa, B = h ? pb2 : pb;
        const A Lm = L[q] + D[q];
        reinterpret_cast<A*>(a.lpsi[ax][SB + q])[so] = Ap * Lm;
        reinterpret_cast<A*>(a.lprv[ax][SB + q])[so] = Ap * B * Lm;
    }
}
// The same update of one cell on every slab axis that holds it, in a tile kernel (the gradient kernels do it for
// the slab cells of their tiles): k_vmem<A, TSLOT>'s work for that cell.
template <class A, int TSLOT>
__device__ __forceinline__ void vmem_cell(const Geom& g, const DevPtrs& p, const AdjPtrs& a, int i, int j, int k,
                                          long long c) {
    constexpr int ND = TSLOT ? 7 : 6;
    A d[ND];
#pragma unroll
    for (int q = 0; q < ND; q++) d[q] = reinterpret_cast<const A*>(TSLOT ? a.tmpT[q] : a.tmpV[q])[c];
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        const int pos = ax == 0 ? i : ax == 1 ? j : k;
        const int s = slab_index(pos, ax == 0 ? g.nx : ax == 1 ? g.ny : g.nz, g.L);
        if (s < 0) continue;
        int dq[4];
        mem_groups<TSLOT>(ax, dq);
        const A D[4] = {d[dq[0]], d[dq[1]], d[dq[2]], d[dq[3]]};
        mem_axis<A, TSLOT>(p, a, ax, pos, slab_off(g, ax, i, j, k, s), D);
    }
}

struct StageSet {
    int slot[3][4];  // [axis][array]: adjoint CPML memory slot and half-shift flag of each staged array
    int half[3][4];
};

template <class S, int R>
struct GatherOps {
    typedef typename Traits<S>::C A;
    // The CPML correction v -> v + B (lpsi + v) + lprev of a value already loaded, in two phases: fix_load issues
    // its three loads unconditionally (at slab cell 0 when (x, y, k) is outside the grid or the slab of axis ax;
    // requires CPML), so that a caller's corrections share one memory round trip; fix_apply uses them.
    struct Fix {
        A B, ps, pv;
        bool on;
    };
    static __device__ __forceinline__ Fix fix_load(const Geom& g, const DevPtrs& p, const AdjPtrs& a, int ax, int slot,
                                                   int half, int x, int y, int k) {
        const bool in = x >= 0 && x < g.nx && y >= 0 && y < g.ny;
        const int pos = ax == 0 ? x : ax == 1 ? y : k;
        const int s = slab_index(pos, ax == 0 ? g.nx : ax == 1 ? g.ny : g.nz, g.L);
        Fix f;
        f.on = in && s >= 0;
        const long long so = f.on ? slab_off(g, ax, x, y, k, s) : 0;
        f.B = reinterpret_cast<const A*>(half ? p.pb2[ax] : p.pb[ax])[f.on ? pos : 0];
        f.ps = reinterpret_cast<const A*>(a.lpsi[ax][slot])[so];
        f.pv = reinterpret_cast<const A*>(a.lprv[ax][slot])[so];
        return f;
    }
    static __device__ __forceinline__ A fix_apply(const Fix& f, A v) { return f.on ? v + f.B * (f.ps + v) + f.pv : v; }
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

// Shared memory of a gather CTA: NS = 2 stages of [4 x windows][4 y windows] (adjoint arrays, type A), then the
// z ring [4][ZS] of row boxes.  x windows start at the 16-byte aligned column i0 - R = 32 bx, padded to whole
// 16-byte chunks (XWP); y windows and ring rows start at i0 = R + 32 bx when that is 16-byte aligned (YV), else at
// i0 - R with the x window's width (YC = column of i0 in them).  With SNAP (the 16-bit kinds) each stage also
// holds [4 x][4 y] windows of forward snapshot fields (type S) and a second ring holds their z rows, for the
// stencils of the coefficient gradients: KIND 0 stresses and pressure of step n (x: sxx sxy sxz p, y: syy sxy
// syz p, z: szz sxz syz p), KIND 1 velocities and Darcy velocities of step n - 1 (x: vx vy vz qx, y: vy vx vz qy,
// z: vz vx vy qz).  MODE 0: adjoint windows and, for the 16-bit kinds, the snapshot (gather and gradients fused);
// MODE 1: adjoint windows only (the gather); MODE 2: the snapshot only (the gradients).  Every box starts on a
// 128-byte boundary.
template <class S, int R, int MODE>
struct GMap {
    typedef typename Traits<S>::C A;
    static constexpr bool TMP = MODE != 2;
    static constexpr int XW = GX + 2 * R;
    static constexpr int YH = GY + 2 * R;
    static constexpr int CH = 16 / (int)sizeof(A);
    static constexpr int XWP = (XW + CH - 1) / CH * CH;
    static constexpr bool YV = (R * (int)sizeof(A)) % 16 == 0;
    static constexpr int YW = YV ? GX : XWP;
    static constexpr int YC = YV ? 0 : R;
    static constexpr bool SNAP = MODE == 2 || (MODE == 0 && BEHF_ADJ_SNAP && sizeof(S) == 2);
    static constexpr int CHS = 16 / (int)sizeof(S);
    static constexpr int XWPS = (XW + CHS - 1) / CHS * CHS;
    static constexpr bool YVS = (R * (int)sizeof(S)) % 16 == 0;
    static constexpr int YWS = YVS ? GX : XWPS;
    static constexpr int YCS = YVS ? 0 : R;
    static constexpr int ZS = 2 * R + 2;
    static constexpr int NS = 2;
    static constexpr int XBOX = TMP ? tiled::al128(XWP * GY * (int)sizeof(A)) : 0;
    static constexpr int YBOX = TMP ? tiled::al128(YW * YH * (int)sizeof(A)) : 0;
    static constexpr int ZBOX = TMP ? tiled::al128(YW * GY * (int)sizeof(A)) : 0;
    static constexpr int XBOXS = SNAP ? tiled::al128(XWPS * GY * (int)sizeof(S)) : 0;
    static constexpr int YBOXS = SNAP ? tiled::al128(YWS * YH * (int)sizeof(S)) : 0;
    static constexpr int ZBOXS = SNAP ? tiled::al128(YWS * GY * (int)sizeof(S)) : 0;
    static constexpr int SOFF = 4 * XBOX + 4 * YBOX;  // snapshot windows within a stage
    static constexpr int STAGE = SOFF + 4 * XBOXS + 4 * YBOXS;
    static constexpr int RING = NS * STAGE;
    static constexpr int RINGS = RING + 4 * ZS * ZBOX;
    static constexpr int BYTES = RINGS + 4 * ZS * ZBOXS;
    static constexpr uint32_t STAGE_TX = TMP ? 4u * (XWP * GY + YW * YH) * (uint32_t)sizeof(A) : 0u;
    static constexpr uint32_t Z_TX = TMP ? 4u * YW * GY * (uint32_t)sizeof(A) : 0u;
    static constexpr uint32_t STAGE_TXS = SNAP ? 4u * (XWPS * GY + YWS * YH) * (uint32_t)sizeof(S) : 0u;
    static constexpr uint32_t Z_TXS = SNAP ? 4u * YWS * GY * (uint32_t)sizeof(S) : 0u;
};

// KIND 0: T^T gather (X: T0 s4, T4 s6h, T5 s7h, T3 s5;  Y: T1 s4, T4 s6h, T6 s7h, T3 s5;
//                      Z: T2 s4, T5 s6h, T6 s7h, T3 s5), then V^T per cell.
// KIND 1: V^T gather (X: V0 s0h, V1 s2, V2 s3, V3 s1h;  Y: V1 s0h, V0 s2, V2 s3, V4 s1h;
//                      Z: V2 s0h, V0 s2, V1 s3, V5 s1h), then the T-slot memory update and, with fuse, T^T per
//                      cell of step n - 1.
// MODE 1 (split gathers): KIND 0 stores mu = lq' - VU2 lv' of the cells outside the slabs for the gradient
// kernel; KIND 1 does T^T per cell without its gradient.  MODE 2 (gradients, after the gather of the same KIND):
// KIND 0 the V-coefficient gradients of step n from mu, lv and the staged stresses and pressure; KIND 1 the
// T-coefficient gradients of step n - 1 from the new stress and pressure adjoints and the staged velocities.
// maps.m[0..3]: x windows, [4..7]: y windows, [8..11]: ring rows, in the order above; smaps: the same for the
// snapshot arrays (SNAP only).
template <class S, int R, int KIND, int MODE>
__global__ void __launch_bounds__(256, MODE == 0 ? BEHF_ADJ_MINB
                                       : MODE == 2                ? BEHF_ADJ_MINB_GRAD
                                       : KIND == 1                ? BEHF_ADJ_MINB_G1
                                                                  : BEHF_ADJ_MINB_SPLIT)
    k_gather(const __grid_constant__ GatherMaps maps, const __grid_constant__ GatherMaps smaps, Geom g, DevPtrs p,
             AdjPtrs a, StageSet ss, int zc, int fuse, int vmem) {
    typedef GatherOps<S, R> W;
    typedef Adj<S, R> Q;
    typedef GMap<S, R, MODE> M;
    typedef typename W::A A;
    using namespace tiled;
    extern __shared__ __align__(128) unsigned char gsm_raw[];
    __shared__ __align__(8) uint64_t bfull[M::NS], bempty[M::NS];
    unsigned char* sm = gsm_raw + ((128u - (smem_u32(gsm_raw) & 127u)) & 127u);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * GX + tx;
    const int i0 = R + blockIdx.x * GX, j0 = R + blockIdx.y * GY;
    const int i = i0 + tx, j = j0 + ty;
    const bool valid = i < g.nx - R && j < g.ny - R;
    const int kb = R + blockIdx.z * zc, ke = min(kb + zc, g.nz - R);
    if (kb >= ke) return;
    const long long sy = g.px, sz = g.plane;
    auto X = [&](int st, int q) { return reinterpret_cast<A*>(sm + st * M::STAGE + q * M::XBOX); };
    auto Y = [&](int st, int q) { return reinterpret_cast<A*>(sm + st * M::STAGE + 4 * M::XBOX + q * M::YBOX); };
    auto Z = [&](int q, int slot) { return reinterpret_cast<A*>(sm + M::RING + (q * M::ZS + slot) * M::ZBOX); };
    auto XS = [&](int st, int q) { return reinterpret_cast<S*>(sm + st * M::STAGE + M::SOFF + q * M::XBOXS); };
    auto YS = [&](int st, int q) {
        return reinterpret_cast<S*>(sm + st * M::STAGE + M::SOFF + 4 * M::XBOXS + q * M::YBOXS);
    };
    auto ZS_ = [&](int q, int slot) { return reinterpret_cast<S*>(sm + M::RINGS + (q * M::ZS + slot) * M::ZBOXS); };
    const int yx0 = M::YV ? i0 : i0 - R;     // first column of the y windows and ring rows
    const int yx0s = M::YVS ? i0 : i0 - R;   // the same for the snapshot
    // the snapshot is staged only where the tile and z range hold cells outside every CPML slab
    auto has_int = [&](int lo, int hi, int n) { return g.W == 0 || max(lo, g.L) <= min(hi, n - 2 - g.L); };
    const bool snap = M::SNAP && a.grad && (KIND == 0 || fuse) && has_int(i0, i0 + GX - 1, g.nx) &&
                      has_int(j0, j0 + GY - 1, g.ny) && has_int(kb, ke - 1, g.nz);
    if (MODE == 2 && !snap) {  // a gradient CTA without cells outside the slabs: at most the memory update
        if (vmem && valid)
            for (int k = kb; k < ke; k++)
                vmem_cell<A, KIND == 0 ? 1 : 0>(g, p, a, i, j, k, k * g.plane + j * (long long)g.px + i);
        return;
    }
    // block-uniform: does the x (y) window of this tile reach a CPML slab of its axis?
    const bool cx = M::TMP && g.W > 0 && (i0 - R < g.L || i0 + GX + R > g.nx - 1 - g.L);
    const bool cy = M::TMP && g.W > 0 && (j0 - R < g.L || j0 + GY + R > g.ny - 1 - g.L);
    const bool fixcta = cx || cy;

    if (tid == 0) {
        for (int s = 0; s < M::NS; s++) {
            mbar_init(&bfull[s], 1);
            mbar_init(&bempty[s], GY);  // one arrival per warp
        }
        fence_init();
    }
    __syncthreads();

    // stage st <- plane kk: the eight windows and the ring plane kk + R (warm-up: kk - R .. kk + R)
    auto issue = [&](int st, int kk, bool warm) {
        uint64_t* br = &bfull[st];
        const uint32_t nz_ = warm ? 2 * R + 1 : 1;
        mbar_expect_tx(br, M::STAGE_TX + M::Z_TX * nz_ + (snap ? M::STAGE_TXS + M::Z_TXS * nz_ : 0u));
        if (M::TMP) {
#pragma unroll
            for (int q = 0; q < 4; q++) tma3(X(st, q), &maps.m[q], br, i0 - R, j0, kk);
#pragma unroll
            for (int q = 0; q < 4; q++) tma3(Y(st, q), &maps.m[4 + q], br, yx0, j0 - R, kk);
            for (int z = warm ? kk - R : kk + R; z <= kk + R; z++)
#pragma unroll
                for (int q = 0; q < 4; q++) tma3(Z(q, z % M::ZS), &maps.m[8 + q], br, yx0, j0, z);
        }
        if (snap) {
#pragma unroll
            for (int q = 0; q < 4; q++) tma3(XS(st, q), &smaps.m[q], br, i0 - R, j0, kk);
#pragma unroll
            for (int q = 0; q < 4; q++) tma3(YS(st, q), &smaps.m[4 + q], br, yx0s, j0 - R, kk);
            for (int z = warm ? kk - R : kk + R; z <= kk + R; z++)
#pragma unroll
                for (int q = 0; q < 4; q++) tma3(ZS_(q, z % M::ZS), &smaps.m[8 + q], br, yx0s, j0, z);
        }
    };
    uint32_t fph = 0, eph = 0;
    uint32_t pend = 0;  // thread 0, bit s: stage s issued and not yet consumed (for the drain after a timeout)
    if (tid == 0) {
        issue(0, kb, true);
        pend = 1u;
    }
    // Own-cell arrays of plane kn (the ones the loads of the cell body below read from global memory, under the
    // same conditions) prefetched into L2 one plane ahead: the stencil inputs arrive by TMA, and without this
    // every plane's own loads wait on DRAM latency with nothing else in flight.
    typedef typename Traits<S>::K K;
    typedef typename Traits<S>::W Wt;
    auto prefetch_plane = [&](int kn) {
        const long long cn = kn * sz + j * sy + i;
        const bool inn = interior(g, i, j, kn);
        if constexpr (MODE == 2) {
            if (!(a.grad && inn)) return;
            if constexpr (KIND == 0) {
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    Q::template pf<A>(a.mu[d], cn);
                    Q::template pf<A>(a.lf[BEHF_VX + d], cn);
                    Q::template pf<S>(a.qprev[d], cn);
                    Q::template pf<S>(a.cur[BEHF_QX + d], cn);
                    if (a.derived) {
                        Q::template pf<K>(p.k[VU2X + d], cn);
                        Q::template pf<K>(p.k[VW3X + d], cn);
                    }
                }
#pragma unroll
                for (int q = 0; q < 15; q++)
                    if (!(a.derived && q >= VW2X && q <= VW2Z)) Q::template pf<A>(a.g[q], cn);
            } else {
                if (!fuse) return;
#pragma unroll
                for (int q = 0; q < 7; q++) Q::template pf<A>(a.lf[BEHF_SXX + q], cn);
#pragma unroll
                for (int q = 0; q < 8; q++)
                    if (q != 4 || !a.derived) Q::template pf<A>(a.g[P1 + q], cn);
            }
        } else if constexpr (KIND == 0) {
#pragma unroll
            for (int d = 0; d < 3; d++) {
                Q::template pf<A>(a.lf[BEHF_VX + d], cn);
                Q::template pf<A>(a.lf[BEHF_QX + d], cn);
                Q::template pf<K>(p.k[VU2X + d], cn);
                Q::template pf<Wt>(p.k[VW1X + d], cn);
                Q::template pf<K>(p.k[VU1X + d], cn);
                Q::template pf<K>(p.k[VW3X + d], cn);
                if (!a.derived) Q::template pf<K>(p.k[VW2X + d], cn);
            }
            if (MODE == 0 && a.grad && inn) {  // the fused V-coefficient gradients
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    Q::template pf<S>(a.qprev[d], cn);
                    Q::template pf<S>(a.cur[BEHF_QX + d], cn);
                }
#pragma unroll
                for (int q = 0; q < 15; q++)
                    if (!(a.derived && q >= VW2X && q <= VW2Z)) Q::template pf<A>(a.g[q], cn);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 7; q++) Q::template pf<A>(a.lf[BEHF_SXX + q], cn);
            if (fuse)
#pragma unroll
                for (int q = 0; q < 8; q++)
                    if (q != 4 || !a.derived) Q::template pf<K>(p.k[P1 + q], cn);
            if (MODE == 0 && fuse && a.grad && inn)  // the fused T-coefficient gradients
#pragma unroll
                for (int q = 0; q < 8; q++)
                    if (q != 4 || !a.derived) Q::template pf<A>(a.g[P1 + q], cn);
        }
    };
    bool failed = false;
    for (int k = kb, it = 0; k < ke; k++, it++) {
        const int st = it & 1;
        bool ok = true;
        if (a.pf && valid && k + 1 < ke) prefetch_plane(k + 1);
        if (tid == 0 && k + 1 < ke) {
            const int sn = st ^ 1;
            if (it >= 1) {  // stage sn was read in iteration it - 1: wait until every warp released it
                ok = mbar_wait(&bempty[sn], (eph >> sn) & 1u);
                eph ^= 1u << sn;
            }
            if (ok) {
                fence_async();
                issue(sn, k + 1, false);
                pend |= 1u << sn;
            }
        }
        if (ok) ok = mbar_wait(&bfull[st], (fph >> st) & 1u);
        // timeout: every thread leaves together (the x/y corrections below hold block barriers)
        if (fixcta ? !__syncthreads_and(ok) : !__all_sync(0xffffffffu, ok)) {
            failed = true;
            break;
        }
        fph ^= 1u << st;
        if (tid == 0) pend &= ~(1u << st);
        // ring planes that arrived with this stage and lie in the z slab: each thread corrects its own column
        if (M::TMP && g.W > 0 && valid) {
            for (int z = it == 0 ? k - R : k + R; z <= k + R; z++) {
                if (slab_index(z, g.nz, g.L) < 0) continue;
                typename W::Fix f[4];
#pragma unroll
                for (int q = 0; q < 4; q++) f[q] = W::fix_load(g, p, a, 2, ss.slot[2][q], ss.half[2][q], i, j, z);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    A* e = Z(q, z % M::ZS) + ty * M::YW + M::YC + tx;
                    *e = W::fix_apply(f[q], *e);
                }
            }
        }
        if (fixcta) {  // CPML corrections of the x/y windows near a slab: each thread rewrites its own elements
            if (cx) {  // x window: row ty, columns tx and tx + 32 < XW
                typename W::Fix f[2][4];
#pragma unroll
                for (int h = 0; h < 2; h++)
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        f[h][q] = W::fix_load(g, p, a, 0, ss.slot[0][q], ss.half[0][q], i0 - R + tx + 32 * h, j0 + ty, k);
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int cc = tx + 32 * h;
                    if (cc < M::XW)
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            A* e = X(st, q) + ty * M::XWP + cc;
                            *e = W::fix_apply(f[h][q], *e);
                        }
                }
            }
            if (cy) {  // y window: rows ty and ty + 8 < YH, column tx
                typename W::Fix f[2][4];
#pragma unroll
                for (int h = 0; h < 2; h++)
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        f[h][q] = W::fix_load(g, p, a, 1, ss.slot[1][q], ss.half[1][q], i0 + tx, j0 - R + ty + 8 * h, k);
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int r = ty + 8 * h;
                    if (r < M::YH)
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            A* e = Y(st, q) + r * M::YW + M::YC + tx;
                            *e = W::fix_apply(f[h][q], *e);
                        }
                }
            }
            __syncthreads();
        }
        if (valid) {
            const long long c = k * sz + j * sy + i;
            const bool inner = interior(g, i, j, k);
            // adjoint windows (M::TMP): array q of the x (y) windows at q * XE (q * YE) from the first; the ring
            // row of array q and plane k + d at q * ZS * ZE + zoff[d + R]
            constexpr int XE = M::XBOX / (int)sizeof(A), YE = M::YBOX / (int)sizeof(A), ZE = M::ZBOX / (int)sizeof(A);
            const A* xb = X(st, 0) + ty * M::XWP + tx + R;
            const A* yb = Y(st, 0) + (ty + R) * M::YW + M::YC + tx;
            const A* zb = Z(0, 0) + ty * M::YW + M::YC + tx;
            const int zs0 = (k - R) % M::ZS;  // ring slot of plane k - R
            int zoff[2 * R + 1];
            {
                int s0 = zs0;
#pragma unroll
                for (int d = 0; d <= 2 * R; d++) {
                    zoff[d] = s0 * ZE;
                    s0 = s0 + 1 == M::ZS ? 0 : s0 + 1;
                }
            }
#define WX(q) [&](int d) { return xb[(q) * XE + d]; }
#define WY(q) [&](int d) { return yb[(q) * YE + d * M::YW]; }
#define WZ(q) [&](int d) { return zb[(q) * M::ZS * ZE + zoff[R + d]]; }
            // snapshot windows (M::SNAP), the same arrangement in the storage type
            constexpr int XES = M::XBOXS / (int)sizeof(S), YES = M::YBOXS / (int)sizeof(S);
            constexpr int ZES = M::ZBOXS / (int)sizeof(S);
            const S* xs = XS(st, 0) + ty * M::XWPS + tx + R;
            const S* ys = YS(st, 0) + (ty + R) * M::YWS + M::YCS + tx;
            const S* zsb = ZS_(0, 0) + ty * M::YWS + M::YCS + tx;
            auto zsl = [&](int d) { return zs0 + R + d >= M::ZS ? zs0 + R + d - M::ZS : zs0 + R + d; };
#define SXW(q) [&](int d) { return Q::ls(xs, (q) * XES + d); }
#define SYW(q) [&](int d) { return Q::ls(ys, (q) * YES + d * M::YWS); }
#define SZW(q) [&](int d) { return Q::ls(zsb, ((q) * M::ZS + zsl(d)) * ZES); }
            // stress divergences and pressure gradient of the forward snapshot of step n (KIND 0)
            auto t_stencils = [&](A (&sum)[3], A (&dp)[3]) {
                if constexpr (M::SNAP) {  // x: sxx sxy sxz p;  y: syy sxy syz p;  z: szz sxz syz p
                    sum[0] = W::fwd(SXW(0)) + W::bwd(SYW(1)) + W::bwd(SZW(1));
                    sum[1] = W::fwd(SYW(0)) + W::bwd(SXW(1)) + W::bwd(SZW(2));
                    sum[2] = W::fwd(SZW(0)) + W::bwd(SXW(2)) + W::bwd(SYW(2));
                    dp[0] = W::fwd(SXW(3));
                    dp[1] = W::fwd(SYW(3));
                    dp[2] = W::fwd(SZW(3));
                } else {
                    sum[0] = Q::fwd(a.cur[BEHF_SXX], c, 1) + Q::bwd(a.cur[BEHF_SXY], c, sy) +
                             Q::bwd(a.cur[BEHF_SXZ], c, sz);
                    sum[1] = Q::fwd(a.cur[BEHF_SYY], c, sy) + Q::bwd(a.cur[BEHF_SXY], c, 1) +
                             Q::bwd(a.cur[BEHF_SYZ], c, sz);
                    sum[2] = Q::fwd(a.cur[BEHF_SZZ], c, sz) + Q::bwd(a.cur[BEHF_SXZ], c, 1) +
                             Q::bwd(a.cur[BEHF_SYZ], c, sy);
                    dp[0] = Q::fwd(a.cur[BEHF_P], c, 1);
                    dp[1] = Q::fwd(a.cur[BEHF_P], c, sy);
                    dp[2] = Q::fwd(a.cur[BEHF_P], c, sz);
                }
            };
            // velocity and Darcy-velocity derivatives of the forward snapshot of step n - 1 (KIND 1)
            auto v_stencils = [&](A (&du)[10]) {
                if constexpr (M::SNAP) {  // x: vx vy vz qx;  y: vy vx vz qy;  z: vz vx vy qz
                    du[0] = W::bwd(SXW(0));                                    // uxx
                    du[1] = W::bwd(SYW(0));                                    // uyy
                    du[2] = W::bwd(SZW(0));                                    // uzz
                    du[3] = W::bwd(SXW(3)) + W::bwd(SYW(3)) + W::bwd(SZW(3));  // div q
                    du[4] = W::fwd(SYW(1));                                    // uxy
                    du[5] = W::fwd(SXW(1));                                    // uyx
                    du[6] = W::fwd(SZW(1));                                    // uxz
                    du[7] = W::fwd(SXW(2));                                    // uzx
                    du[8] = W::fwd(SZW(2));                                    // uyz
                    du[9] = W::fwd(SYW(2));                                    // uzy
                } else {
                    vq_derivs<S, R>(a.vq1, c, sy, sz, du);
                }
            };
            // V-coefficient gradient increments of step n into go (accumulators 0..14) from mu, lv and the
            // snapshot's q before and after V, stress divergences and pressure gradient
            auto v_grad = [&](A (&go)[15], const A (&mu)[3], const A (&lv)[3], const A (&qo)[3], const A (&qn)[3],
                              const A (&sum)[3], const A (&dp)[3], const A (&vu2)[3], const A (&vw3)[3]) {
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    go[VW1X + d] += mu[d] * qo[d];
                    const A gw2 = -mu[d] * sum[d];
                    if (a.derived) {  // chain rule through VW2 = VU2 VW3 c_vw2
                        go[VU2X + d] += gw2 * vw3[d] * (A)g.c_vw2;
                        go[VW3X + d] += gw2 * vu2[d] * (A)g.c_vw2;
                    } else {
                        go[VW2X + d] += gw2;
                    }
                    go[VU1X + d] += lv[d] * sum[d];
                    go[VU2X + d] += -lv[d] * (qn[d] - qo[d]);
                }
                go[VW3X] += -mu[0] * dp[0];
                const A w3z = -mu[2] * dp[2];
                go[VW3Y] += -mu[1] * dp[1] + (g.bug ? w3z : (A)0);
                go[VW3Z] += g.bug ? (A)0 : w3z;
            };
            auto load_vgo = [&](A (&go)[15]) {
#pragma unroll
                for (int q = 0; q < 15; q++)
                    go[q] = (a.derived && q >= VW2X && q <= VW2Z) ? (A)0 : Q::ad(a.g[q])[c];
            };
            auto store_vgo = [&](const A (&go)[15]) {
#pragma unroll
                for (int q = 0; q < 15; q++)
                    if (!(a.derived && q >= VW2X && q <= VW2Z)) Q::ad(a.g[q])[c] = go[q];
            };
            auto load_tgo = [&](A (&go)[8]) {
#pragma unroll
                for (int q = 0; q < 8; q++) go[q] = (q == 4 && a.derived) ? (A)0 : Q::ad(a.g[P1 + q])[c];
            };
            auto store_tgo = [&](const A (&lt)[7], const A (&du)[10], const A (&go)[8]) {
                A inc[8];
                t_grad(lt, du, inc);
                t_grad_fold(g, a, inc);
#pragma unroll
                for (int q = 0; q < 8; q++)
                    if (q != 4 || !a.derived) Q::ad(a.g[P1 + q])[c] = go[q] + inc[q];
            };
            // Each cell issues all its global loads before its first global store (see k_adj_a).
            if constexpr (MODE == 2) {
                if constexpr (KIND == 0) {  // V-coefficient gradients of step n
                    if (a.grad && inner) {
                        A mu[3], lv[3], qo[3], qn[3], vu2[3], vw3[3], go[15], sum[3], dp[3];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            mu[d] = Q::ad(a.mu[d])[c];
                            lv[d] = Q::ad(a.lf[BEHF_VX + d])[c];
                            qo[d] = Q::ls(a.qprev[d], c);
                            qn[d] = Q::ls(a.cur[BEHF_QX + d], c);
                            vu2[d] = a.derived ? Q::coef(g, p, VU2X + d, c) : (A)0;
                            vw3[d] = a.derived ? Q::coef(g, p, VW3X + d, c) : (A)0;
                        }
                        load_vgo(go);
                        t_stencils(sum, dp);
                        v_grad(go, mu, lv, qo, qn, sum, dp, vu2, vw3);
                        store_vgo(go);
                    } else if (vmem && !inner) {  // the T-slot memory update of step n on the slab cells
                        vmem_cell<A, 1>(g, p, a, i, j, k, c);
                    }
                } else {  // T-coefficient gradients of step n - 1 (the stress/pressure adjoints the gather left)
                    if (fuse && a.grad && inner) {
                        A lt[7], go[8], du[10];
#pragma unroll
                        for (int q = 0; q < 7; q++) lt[q] = Q::ad(a.lf[BEHF_SXX + q])[c];
                        load_tgo(go);
                        v_stencils(du);
                        store_tgo(lt, du, go);
                    } else if (vmem && !inner) {  // the V-slot memory update of step n on the slab cells
                        vmem_cell<A, 0>(g, p, a, i, j, k, c);
                    }
                }
            } else if constexpr (KIND == 0) {
                // V^T at this cell with lv = lv_old - dl[0..2], lq' = lq_old - dl[3..5]
                A lvo[3], lqo[3], vu2[3], vw1[3], vu1[3], vw2[3], vw3[3], vw3p;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    lvo[d] = Q::ad(a.lf[BEHF_VX + d])[c];
                    lqo[d] = Q::ad(a.lf[BEHF_QX + d])[c];
                    vu2[d] = Q::coef(g, p, VU2X + d, c);
                    vw1[d] = Q::vw1(p, d, c);
                    vu1[d] = Q::coef(g, p, VU1X + d, c);
                    vw3[d] = Q::coef(g, p, VW3X + d, c);
                    // with a.derived (tiled forward) VW2 = VU2 VW3 c_vw2 with the cell's own-axis VW3
                    vw2[d] = a.derived ? vu2[d] * vw3[d] * (A)g.c_vw2 : Q::coef(g, p, VW2X + d, c);
                }
                vw3p = g.bug ? Q::coef(g, p, VW3Y, c) : vw3[2];  // reference: the dp term of vz uses VW3y
                const bool gr = a.grad && inner;
                A sum[3], dp[3], qo[3], qn[3], go[15];
                if (MODE == 0 && gr) {
                    t_stencils(sum, dp);
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        qo[d] = Q::ls(a.qprev[d], c);
                        qn[d] = Q::ls(a.cur[BEHF_QX + d], c);
                    }
                    load_vgo(go);
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
                    Q::ad(a.tmpV[3 + d])[c] = -(d == 2 ? vw3p : vw3[d]) * mu[d];
                }
                if (MODE == 0 && gr) {
                    v_grad(go, mu, lv, qo, qn, sum, dp, vu2, vw3);
                    store_vgo(go);
                }
                if (MODE == 1 && gr) {  // for the gradient kernel of this step
#pragma unroll
                    for (int d = 0; d < 3; d++) Q::ad(a.mu[d])[c] = mu[d];
                }
            } else {
                A lo[7];  // sxx syy szz sxy sxz syz p
#pragma unroll
                for (int q = 0; q < 7; q++) lo[q] = Q::ad(a.lf[BEHF_SXX + q])[c];
                // T-slot adjoint memory of this step on slab cells (its gathers ran in the KIND 0 launch), here in
                // the fused mode; the split mode updates it in its own launch before this one
                const bool mem = MODE == 0 && !inner;
                A tt[7];
                MemUpd<A, 4, 0xC> mt;
                if (mem) {
#pragma unroll
                    for (int q = 0; q < 7; q++) tt[q] = Q::ad(a.tmpT[q])[c];
                    mt.load(g, p, a, i, j, k);
                }
                // T^T per cell of step n - 1 (fuse): coefficients, and (fused gradients) on cells outside the
                // slabs the forward derivatives of step n - 1 and the gradient accumulators
                A kc[8];
                if (fuse) t_coefs<S, R>(g, p, a, c, kc);
                const bool gr = MODE == 0 && fuse && a.grad && inner;
                A du[10], go[8];
                if (gr) {
                    v_stencils(du);
                    load_tgo(go);
                }
                A lt[7];
                lt[0] = lo[0] - W::bwd(WX(0));
                lt[1] = lo[1] - W::bwd(WY(0));
                lt[2] = lo[2] - W::bwd(WZ(0));
                lt[3] = lo[3] - (W::fwd(WY(1)) + W::fwd(WX(1)));
                lt[4] = lo[4] - (W::fwd(WZ(1)) + W::fwd(WX(2)));
                lt[5] = lo[5] - (W::fwd(WZ(2)) + W::fwd(WY(2)));
                lt[6] = lo[6] - (W::bwd(WX(3)) + W::bwd(WY(3)) + W::bwd(WZ(3)));
#pragma unroll
                for (int q = 0; q < 7; q++) Q::ad(a.lf[BEHF_SXX + q])[c] = lt[q];
                if (mem) {
                    // axis x: uxx s4, wx s5, uyx s6h, uzx s7h; y: uyy, wy, uxy, uzy; z: uzz, wz, uxz, uyz
                    const A D[3][4] = {{tt[0], tt[3], tt[4], tt[5]}, {tt[1], tt[3], tt[4], tt[6]},
                                       {tt[2], tt[3], tt[5], tt[6]}};
                    mt.store(a, D);
                }
                if (fuse) {
                    A tg[7];
                    t_groups(lt, kc, tg);
#pragma unroll
                    for (int q = 0; q < 7; q++) Q::ad(a.tmpT[q])[c] = tg[q];
                }
                if (gr) store_tgo(lt, du, go);
            }
#undef SXW
#undef SYW
#undef SZW
#undef WX
#undef WY
#undef WZ
        }
        // generic-proxy writes to shared memory (the corrections) before the TMA that will overwrite it
        if (g.W > 0) fence_async();
        __syncwarp();
        if (tx == 0) mbar_arrive(&bempty[st]);
    }
    if (failed) atomicExch(g.err, 1);
    if (tid == 0)  // drain the copies still in flight before the CTA's shared memory is released
        for (int s = 0; s < M::NS; s++)
            if ((pend >> s) & 1u) {
                mbar_wait(&bfull[s], (fph >> s) & 1u);
                fph ^= 1u << s;
            }
}

#undef CELL_INDEX

// V-slot adjoint memory update of one step on the slab cells of the updated region, one slab cell of one axis per
// thread (a cell in two slabs is visited once per axis): from the cell's tmpV, the slots 0..3 of that axis
// (TSLOT 0); or, TSLOT 1, the T-slot update from tmpT, slots 4..7 (split gathers: after the T^T gather that reads
// those slots, before the V^T gather overwrites tmpT with the next step's).
__device__ __forceinline__ int slab_pos(int s, int n, int L) { return s < L ? s : n - 1 - L + (s - L); }
template <class A, int TSLOT>
__global__ void k_vmem(Geom g, DevPtrs p, AdjPtrs a) {
    const long long n0 = (long long)g.nz * g.ny * g.W, n1 = (long long)g.nz * g.W * g.nx;
    const long long n2 = (long long)g.W * g.ny * g.nx, tot = n0 + n1 + n2;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
         t += (long long)gridDim.x * blockDim.x) {
        int ax, i, j, k, pos;
        long long u = t;
        if (u < n0) {  // x slab [nz][ny][W]
            ax = 0;
            const int sl = (int)(u % g.W);
            const long long r = u / g.W;
            j = (int)(r % g.ny);
            k = (int)(r / g.ny);
            i = pos = slab_pos(sl, g.nx, g.L);
        } else if ((u -= n0) < n1) {  // y slab [nz][W][nx]
            ax = 1;
            i = (int)(u % g.nx);
            const long long r = u / g.nx;
            k = (int)(r / g.W);
            j = pos = slab_pos((int)(r % g.W), g.ny, g.L);
        } else {  // z slab [W][ny][nx]
            u -= n1;
            ax = 2;
            i = (int)(u % g.nx);
            const long long r = u / g.nx;
            j = (int)(r % g.ny);
            k = pos = slab_pos((int)(r / g.ny), g.nz, g.L);
        }
        if (i < g.R || i >= g.nx - g.R || j < g.R || j >= g.ny - g.R || k < g.R || k >= g.nz - g.R) continue;
        const long long c = (long long)k * g.plane + (long long)j * g.px + i;
        int dq[4];
        mem_groups<TSLOT>(ax, dq);
        A D[4];
#pragma unroll
        for (int q = 0; q < 4; q++) D[q] = reinterpret_cast<const A*>(TSLOT ? a.tmpT[dq[q]] : a.tmpV[dq[q]])[c];
        mem_axis<A, TSLOT>(p, a, ax, pos, u, D);
    }
}

// ------------------------------------------------------------------------------------------- record^T, source^T
template <class A>
__global__ void k_adj_record(AdjPtrs a, const long long* off, const int* comp, int nrec, const double* adj, int nt,
                             int it, AdjScales sc) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const int q = comp[r];
    atomicAdd(reinterpret_cast<A*>(a.lf[q]) + off[r], (A)(adj[(long long)r * nt + it] * sc.s[q]));
}

// record^T of step n - 1 after the fused T^T of that step: the injection into the adjoint fields, plus its share of
// tmpT and of the T-coefficient gradients at the receiver cell (atomic: receivers may share a cell).
template <class S, int R>
__global__ void k_adj_recfix(Geom g, DevPtrs p, AdjPtrs a, const long long* off, const int* comp, int nrec,
                             const double* adj, int nt, int it, AdjScales sc) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const int q = comp[r];
    const long long c = off[r];
    const A dv = (A)(adj[(long long)r * nt + it] * sc.s[q]);
    atomicAdd(reinterpret_cast<A*>(a.lf[q]) + c, dv);
    if (q < BEHF_SXX) return;  // velocity receivers: V^T reads lv directly
    const int k = (int)(c / g.plane), j = (int)((c % g.plane) / g.px), i = (int)(c % g.px);
    if (i < R || i >= g.nx - R || j < R || j >= g.ny - R || k < R || k >= g.nz - R) return;
    A lt[7], kc[8], tg[7];
#pragma unroll
    for (int u = 0; u < 7; u++) lt[u] = u == q - BEHF_SXX ? dv : (A)0;
    t_coefs<S, R>(g, p, a, c, kc);
    t_groups(lt, kc, tg);
#pragma unroll
    for (int u = 0; u < 7; u++) atomicAdd(Q::ad(a.tmpT[u]) + c, tg[u]);
    if (a.grad && interior(g, i, j, k)) {
        A du[10], inc[8];
        vq_derivs<S, R>(a.vq1, c, g.px, g.plane, du);
        t_grad(lt, du, inc);
        t_grad_fold(g, a, inc);
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (u != 4 || !a.derived) atomicAdd(Q::ad(a.g[P1 + u]) + c, inc[u]);
    }
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
cudaError_t adj_first_r(const Geom& g, const DevPtrs& p, const AdjPtrs& a, cudaStream_t st) {
    const dim3 block(32, 8, 1);
    const int nxu = g.nx - 2 * R, nyu = g.ny - 2 * R, nzu = g.nz - 2 * R;
    const dim3 grid((nxu + 31) / 32, (nyu + 7) / 8, nzu);
    k_adj_a<S, R><<<grid, block, 0, st>>>(g, p, a);
    return cudaGetLastError();
}

template <class S, int R>
cudaError_t adj_r(const Geom& g, const DevPtrs& p, const AdjPtrs& a, const AdjMaps& m, const GatherMaps* snapT,
                  const GatherMaps* snapV, int fuse, cudaStream_t st) {
    const dim3 block(32, 8, 1);
    const int nxu = g.nx - 2 * R, nyu = g.ny - 2 * R, nzu = g.nz - 2 * R;
    const int sms = device_sms();
    // z chunks that fill the last wave of resident CTAs, at most 64 planes, at least BEHF_ADJ_MINW waves (measured
    // at 192^3 with the fused gathers: 2 waves of 46-plane chunks 553 + 615 us per step, 5 waves of 17 planes
    // 499 + 516 us)
    const int nxy = (int)(((nxu + GX - 1) / GX) * ((nyu + GY - 1) / GY));
    const int resident = BEHF_ADJ_SPLIT ? BEHF_ADJ_MINB_SPLIT : BEHF_ADJ_MINB;
    const int zc = wave_zchunk(nxy, nzu, resident * sms, 8, 64, R, BEHF_ADJ_MINW);
    const dim3 ggrid((nxu + GX - 1) / GX, (nyu + GY - 1) / GY, (nzu + zc - 1) / zc);
    StageSet t{}, v{};
    // T^T gather: x {T0 s4, T4 s6h, T5 s7h, T3 s5}, y {T1 s4, T4 s6h, T6 s7h, T3 s5}, z {T2 s4, T5 s6h, T6 s7h, T3 s5}
    const int ts[4] = {4, 6, 7, 5}, th[4] = {0, 1, 1, 0};
    // V^T gather: x {V0 s0h, V1 s2, V2 s3, V3 s1h}, y {V1 s0h, V0 s2, V2 s3, V4 s1h}, z {V2 s0h, V0 s2, V1 s3, V5 s1h}
    const int vs[4] = {0, 2, 3, 1}, vh[4] = {1, 0, 0, 1};
    for (int ax = 0; ax < 3; ax++)
        for (int q = 0; q < 4; q++) {
            t.slot[ax][q] = ts[q];
            t.half[ax][q] = th[q];
            v.slot[ax][q] = vs[q];
            v.half[ax][q] = vh[q];
        }
    constexpr bool split = BEHF_ADJ_SPLIT != 0;
    constexpr int MG = split ? 1 : 0;  // the gathers' mode
    const int smemg = GMap<S, R, MG>::BYTES + 128, smemd = GMap<S, R, 2>::BYTES + 128;
    static PerDevice once;
    const cudaError_t ea = run_once(once, [&] {
        cudaError_t e = cudaFuncSetAttribute(k_gather<S, R, 0, MG>, cudaFuncAttributeMaxDynamicSharedMemorySize, smemg);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_gather<S, R, 1, MG>, cudaFuncAttributeMaxDynamicSharedMemorySize, smemg);
        if (e == cudaSuccess && split)
            e = cudaFuncSetAttribute(k_gather<S, R, 0, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smemd);
        if (e == cudaSuccess && split)
            e = cudaFuncSetAttribute(k_gather<S, R, 1, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smemd);
        return e;
    });
    if (ea != cudaSuccess) return ea;
    if ((split || GMap<S, R, 0>::SNAP) && a.grad && (!snapT || (fuse && !snapV))) return cudaErrorInvalidValue;
    // T^T gather + V^T; its V-coefficient gradients; V^T gather + T-slot memory + T^T of step n - 1; its
    // T-coefficient gradients
    typedef typename Traits<S>::C A;
    // The memory updates ride in the gradient kernels' launches when those run (their slab cells; each gradient
    // kernel runs after the gather that reads those slots and before tmpT / tmpV is overwritten), else in k_vmem.
    const int mt = split && a.grad && g.W > 0 && a.vmerge, mv = mt && fuse;
    k_gather<S, R, 0, MG><<<ggrid, block, smemg, st>>>(m.t, snapT ? *snapT : m.t, g, p, a, t, zc, 0, 0);
    if (split && a.grad) k_gather<S, R, 0, 2><<<ggrid, block, smemd, st>>>(m.t, *snapT, g, p, a, t, zc, 0, mt);
    if (split && g.W > 0 && !mt) k_vmem<A, 1><<<sms * 8, 256, 0, st>>>(g, p, a);
    k_gather<S, R, 1, MG><<<ggrid, block, smemg, st>>>(m.v, snapV ? *snapV : m.v, g, p, a, v, zc, fuse, 0);
    if (split && a.grad && fuse)
        k_gather<S, R, 1, 2><<<ggrid, block, smemd, st>>>(m.v, *snapV, g, p, a, v, zc, fuse, mv);
    if (g.W > 0 && !mv) k_vmem<A, 0><<<sms * 8, 256, 0, st>>>(g, p, a);
    return cudaGetLastError();
}

// Boxes of one gather's maps over arrays of T: x windows XWP x GY, y windows YW x YH, ring rows YW x GY.
template <class T, int XWP, int YW, int YH>
bool build_gather_maps(const Geom& g, void* const x[4], void* const y[4], void* const z[4], GatherMaps* gm) {
    bool ok = true;
    for (int q = 0; q < 4; q++) {
        ok = ok && tiled::encode<T>(&gm->m[q], g, x[q], XWP, GY);
        ok = ok && tiled::encode<T>(&gm->m[4 + q], g, y[q], YW, YH);
        ok = ok && tiled::encode<T>(&gm->m[8 + q], g, z[q], YW, GY);
    }
    return ok;
}

template <class S, int R>
cudaError_t build_maps_r(const Geom& g, const AdjPtrs& a, AdjMaps* m) {
    // same array order as the StageSet tables in adj_r
    void* const tx_[4] = {a.tmpT[0], a.tmpT[4], a.tmpT[5], a.tmpT[3]};
    void* const ty_[4] = {a.tmpT[1], a.tmpT[4], a.tmpT[6], a.tmpT[3]};
    void* const tz_[4] = {a.tmpT[2], a.tmpT[5], a.tmpT[6], a.tmpT[3]};
    void* const vx_[4] = {a.tmpV[0], a.tmpV[1], a.tmpV[2], a.tmpV[3]};
    void* const vy_[4] = {a.tmpV[1], a.tmpV[0], a.tmpV[2], a.tmpV[4]};
    void* const vz_[4] = {a.tmpV[2], a.tmpV[0], a.tmpV[1], a.tmpV[5]};
    if (!tiled::encoder()) return cudaErrorNotSupported;
    typedef GMap<S, R, 1> M;  // the adjoint-window boxes (the same in the fused mode)
    typedef typename M::A A;
    const bool ok = build_gather_maps<A, M::XWP, M::YW, M::YH>(g, tx_, ty_, tz_, &m->t) &&
                    build_gather_maps<A, M::XWP, M::YW, M::YH>(g, vx_, vy_, vz_, &m->v);
    return ok ? cudaSuccess : cudaErrorInvalidValue;
}

template <class S, int R>
cudaError_t build_snap_maps_r(const Geom& g, void* const f[kNField], GatherMaps* mt, GatherMaps* mv) {
    typedef GMap<S, R, 2> M;  // the snapshot boxes (the same in the fused mode)
    if (!BEHF_ADJ_SPLIT && !GMap<S, R, 0>::SNAP) return cudaSuccess;
    if (!tiled::encoder()) return cudaErrorNotSupported;
    void* const x[4] = {f[BEHF_SXX], f[BEHF_SXY], f[BEHF_SXZ], f[BEHF_P]};
    void* const y[4] = {f[BEHF_SYY], f[BEHF_SXY], f[BEHF_SYZ], f[BEHF_P]};
    void* const z[4] = {f[BEHF_SZZ], f[BEHF_SXZ], f[BEHF_SYZ], f[BEHF_P]};
    void* const vx[4] = {f[BEHF_VX], f[BEHF_VY], f[BEHF_VZ], f[BEHF_QX]};
    void* const vy[4] = {f[BEHF_VY], f[BEHF_VX], f[BEHF_VZ], f[BEHF_QY]};
    void* const vz[4] = {f[BEHF_VZ], f[BEHF_VX], f[BEHF_VY], f[BEHF_QZ]};
    const bool ok = build_gather_maps<S, M::XWPS, M::YWS, M::YH>(g, x, y, z, mt) &&
                    build_gather_maps<S, M::XWPS, M::YWS, M::YH>(g, vx, vy, vz, mv);
    return ok ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace

template <class S>
cudaError_t adj_build_maps(const Geom& g, const AdjPtrs& a, AdjMaps* m) {
    switch (g.R) {
        case 1: return build_maps_r<S, 1>(g, a, m);
        case 2: return build_maps_r<S, 2>(g, a, m);
        case 3: return build_maps_r<S, 3>(g, a, m);
        case 4: return build_maps_r<S, 4>(g, a, m);
    }
    return cudaErrorInvalidValue;
}
int adj_step_launches(const Geom& g, const AdjPtrs& a, int fuse) {
    constexpr bool split = BEHF_ADJ_SPLIT != 0;
    const bool mt = split && a.grad && g.W > 0 && a.vmerge, mv = mt && fuse;  // as in adj_r
    return 2 + (split && a.grad ? 1 + (fuse ? 1 : 0) : 0) + (split && g.W > 0 && !mt ? 1 : 0) +
           (g.W > 0 && !mv ? 1 : 0);
}
template <class S>
bool adj_snap_staged() {
    return BEHF_ADJ_SPLIT || (BEHF_ADJ_SNAP && sizeof(S) == 2);
}
template <class S>
cudaError_t adj_build_snap_maps(const Geom& g, void* const f[kNField], GatherMaps* mt, GatherMaps* mv) {
    switch (g.R) {
        case 1: return build_snap_maps_r<S, 1>(g, f, mt, mv);
        case 2: return build_snap_maps_r<S, 2>(g, f, mt, mv);
        case 3: return build_snap_maps_r<S, 3>(g, f, mt, mv);
        case 4: return build_snap_maps_r<S, 4>(g, f, mt, mv);
    }
    return cudaErrorInvalidValue;
}
template <class S>
cudaError_t adj_first(const Geom& g, const DevPtrs& p, const AdjPtrs& a, cudaStream_t st) {
    switch (g.R) {
        case 1: return adj_first_r<S, 1>(g, p, a, st);
        case 2: return adj_first_r<S, 2>(g, p, a, st);
        case 3: return adj_first_r<S, 3>(g, p, a, st);
        case 4: return adj_first_r<S, 4>(g, p, a, st);
    }
    return cudaErrorInvalidValue;
}
template <class S>
cudaError_t adj_step(const Geom& g, const DevPtrs& p, const AdjPtrs& a, const AdjMaps& m, const GatherMaps* snapT,
                     const GatherMaps* snapV, int fuse, cudaStream_t st) {
    switch (g.R) {
        case 1: return adj_r<S, 1>(g, p, a, m, snapT, snapV, fuse, st);
        case 2: return adj_r<S, 2>(g, p, a, m, snapT, snapV, fuse, st);
        case 3: return adj_r<S, 3>(g, p, a, m, snapT, snapV, fuse, st);
        case 4: return adj_r<S, 4>(g, p, a, m, snapT, snapV, fuse, st);
    }
    return cudaErrorInvalidValue;
}
template <class S>
cudaError_t adj_recfix(const Geom& g, const DevPtrs& p, const AdjPtrs& a, const long long* off, const int* comp,
                       int nrec, const double* adj, int nt, int it, const AdjScales& sc, cudaStream_t st) {
    if (nrec <= 0) return cudaSuccess;
    const int nb = (nrec + 255) / 256;
    switch (g.R) {
        case 1: k_adj_recfix<S, 1><<<nb, 256, 0, st>>>(g, p, a, off, comp, nrec, adj, nt, it, sc); break;
        case 2: k_adj_recfix<S, 2><<<nb, 256, 0, st>>>(g, p, a, off, comp, nrec, adj, nt, it, sc); break;
        case 3: k_adj_recfix<S, 3><<<nb, 256, 0, st>>>(g, p, a, off, comp, nrec, adj, nt, it, sc); break;
        case 4: k_adj_recfix<S, 4><<<nb, 256, 0, st>>>(g, p, a, off, comp, nrec, adj, nt, it, sc); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
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

// Neumaier summation: the total and the compensation of each accumulator (FP32), or an FP64 total.  One thread per
// cell index, every accumulator in turn; g is zeroed for the next segment.
__global__ void k_adj_fold(AdjFold f, long long n, int final) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        for (int q = 0; q < kNCoef; q++) {
            const float y = f.g[q][i];
            if (f.mode == 2) {
                const double t = f.tot64[q][i] + (double)y;
                if (final) f.g[q][i] = (float)t;
                else {
                    f.tot64[q][i] = t;
                    f.g[q][i] = 0.f;
                }
            } else {
                const float t = f.tot[q][i], s = t + y;
                const float c = f.comp[q][i] + (fabsf(t) >= fabsf(y) ? (t - s) + y : (y - s) + t);
                if (final) f.g[q][i] = s + c;
                else {
                    f.tot[q][i] = s;
                    f.comp[q][i] = c;
                    f.g[q][i] = 0.f;
                }
            }
        }
}
cudaError_t adj_fold(const AdjFold& f, long long n, int final, cudaStream_t st) {
    k_adj_fold<<<device_sms() * 8, 256, 0, st>>>(f, n, final);
    return cudaGetLastError();
}

#define BEHF_ADJ_INST(S)                                                                                         \
    template cudaError_t adj_build_maps<S>(const Geom&, const AdjPtrs&, AdjMaps*);                             \
    template bool adj_snap_staged<S>();                                                                        \
    template cudaError_t adj_build_snap_maps<S>(const Geom&, void* const*, GatherMaps*, GatherMaps*);          \
    template cudaError_t adj_first<S>(const Geom&, const DevPtrs&, const AdjPtrs&, cudaStream_t);              \
    template cudaError_t adj_step<S>(const Geom&, const DevPtrs&, const AdjPtrs&, const AdjMaps&,              \
                                     const GatherMaps*, const GatherMaps*, int, cudaStream_t);                 \
    template cudaError_t adj_recfix<S>(const Geom&, const DevPtrs&, const AdjPtrs&, const long long*,          \
                                       const int*, int, const double*, int, int, const AdjScales&,             \
                                       cudaStream_t);                                                          \
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
