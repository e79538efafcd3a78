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

    // derivative-group adjoint t at cell (i,j,k) with the adjoint CPML correction of `slot` on axis ax
    static __device__ __forceinline__ A lmod(const Geom& g, const DevPtrs& p, const AdjPtrs& a, int t, int ax,
                                             int slot, bool half, int i, int j, int k) {
        A v = reinterpret_cast<const A*>(a.tmp[t])[(long long)k * g.plane + (long long)j * g.px + i];
        if (g.W > 0) {
            const int pos = ax == 0 ? i : ax == 1 ? j : k;
            const int s = slab_index(pos, ax == 0 ? g.nx : ax == 1 ? g.ny : g.nz, g.L);
            if (s >= 0) {
                const long long so = slab_off(g, ax, i, j, k, s);
                const A B = half ? prof(p.pb2[ax], pos) : prof(p.pb[ax], pos);
                v += B * (reinterpret_cast<const A*>(a.lpsi[ax][slot])[so] + v) +
                     reinterpret_cast<const A*>(a.lprv[ax][slot])[so];
            }
        }
        return v;
    }
    // transposed stencils of a corrected derivative-group adjoint along axis ax, at cell (i,j,k):
    //   fwdL = sum_m w_m (L[+m] - L[-m+1]),  bwdL = sum_m w_m (L[+m-1] - L[-m])
    static __device__ __forceinline__ A fwdL(const Geom& g, const DevPtrs& p, const AdjPtrs& a, int t, int ax,
                                             int slot, bool half, int i, int j, int k) {
        const int di = ax == 0, dj = ax == 1, dk = ax == 2;
        A acc = 0;
#pragma unroll
        for (int m = 1; m <= R; m++)
            acc += (A)stencil_w<R>(m) * (lmod(g, p, a, t, ax, slot, half, i + m * di, j + m * dj, k + m * dk) -
                                         lmod(g, p, a, t, ax, slot, half, i - (m - 1) * di, j - (m - 1) * dj,
                                              k - (m - 1) * dk));
        return acc;
    }
    static __device__ __forceinline__ A bwdL(const Geom& g, const DevPtrs& p, const AdjPtrs& a, int t, int ax,
                                             int slot, bool half, int i, int j, int k) {
        const int di = ax == 0, dj = ax == 1, dk = ax == 2;
        A acc = 0;
#pragma unroll
        for (int m = 1; m <= R; m++)
            acc += (A)stencil_w<R>(m) * (lmod(g, p, a, t, ax, slot, half, i + (m - 1) * di, j + (m - 1) * dj,
                                              k + (m - 1) * dk) -
                                         lmod(g, p, a, t, ax, slot, half, i - m * di, j - m * dj, k - m * dk));
        return acc;
    }
    // adjoint CPML memory update of one slot
    static __device__ __forceinline__ void lmem(const Geom& g, const DevPtrs& p, const AdjPtrs& a, A lD, int ax,
                                                int slot, bool half, int pos, long long so) {
        const A Ap = half ? prof(p.pa2[ax], pos) : prof(p.pa[ax], pos);
        const A B = half ? prof(p.pb2[ax], pos) : prof(p.pb[ax], pos);
        A* ps = reinterpret_cast<A*>(a.lpsi[ax][slot]) + so;
        A* pv = reinterpret_cast<A*>(a.lprv[ax][slot]) + so;
        const A Lm = *ps + lD;
        *ps = Ap * Lm;
        *pv = Ap * B * Lm;
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

// ------------------------------------------------------------------------------------------- T^T
template <class S, int R>
__global__ void __launch_bounds__(256) k_adj_t1(Geom g, DevPtrs p, AdjPtrs a) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
    CELL_INDEX
    const A lp = Q::ad(a.lf[BEHF_P])[c], lxx = Q::ad(a.lf[BEHF_SXX])[c], lyy = Q::ad(a.lf[BEHF_SYY])[c];
    const A lzz = Q::ad(a.lf[BEHF_SZZ])[c], lxy = Q::ad(a.lf[BEHF_SXY])[c], lxz = Q::ad(a.lf[BEHF_SXZ])[c];
    const A lyz = Q::ad(a.lf[BEHF_SYZ])[c];
    const A p1 = Q::coef(g, p, P1, c), p2 = Q::coef(g, p, P2, c);
    const A s1 = Q::coef(g, p, S1, c), s2 = Q::coef(g, p, S2, c), s3 = Q::coef(g, p, S3, c);
    Q::ad(a.tmp[0])[c] = -p1 * lp + s2 * lxx + s1 * (lyy + lzz);
    Q::ad(a.tmp[1])[c] = -p1 * lp + s2 * lyy + s1 * (lxx + lzz);
    Q::ad(a.tmp[2])[c] = -p1 * lp + s2 * lzz + s1 * (lxx + lyy);
    Q::ad(a.tmp[3])[c] = -p2 * lp + s3 * (lxx + lyy + lzz);
    Q::ad(a.tmp[4])[c] = Q::coef(g, p, SXYC, c) * lxy;
    Q::ad(a.tmp[5])[c] = Q::coef(g, p, SXZC, c) * lxz;
    Q::ad(a.tmp[6])[c] = Q::coef(g, p, SYZC, c) * lyz;
    if (a.grad && interior(g, i, j, k)) {
        const A uxx = Q::bwd(a.cur[BEHF_VX], c, 1), uyy = Q::bwd(a.cur[BEHF_VY], c, sy);
        const A uzz = Q::bwd(a.cur[BEHF_VZ], c, sz);
        const A dq = Q::bwd(a.cur[BEHF_QX], c, 1) + Q::bwd(a.cur[BEHF_QY], c, sy) + Q::bwd(a.cur[BEHF_QZ], c, sz);
        const A uxy = Q::fwd(a.cur[BEHF_VX], c, sy), uyx = Q::fwd(a.cur[BEHF_VY], c, 1);
        const A uxz = Q::fwd(a.cur[BEHF_VX], c, sz), uzx = Q::fwd(a.cur[BEHF_VZ], c, 1);
        const A uyz = Q::fwd(a.cur[BEHF_VY], c, sz), uzy = Q::fwd(a.cur[BEHF_VZ], c, sy);
        Q::ad(a.g[P1])[c] += -lp * (uxx + uyy + uzz);
        Q::ad(a.g[P2])[c] += -lp * dq;
        Q::ad(a.g[S1])[c] += lxx * (uyy + uzz) + lyy * (uxx + uzz) + lzz * (uxx + uyy);
        Q::ad(a.g[S2])[c] += lxx * uxx + lyy * uyy + lzz * uzz;
        Q::ad(a.g[S3])[c] += (lxx + lyy + lzz) * dq;
        Q::ad(a.g[SXYC])[c] += lxy * (uxy + uyx);
        Q::ad(a.g[SXZC])[c] += lxz * (uxz + uzx);
        Q::ad(a.g[SYZC])[c] += lyz * (uyz + uzy);
    }
}

// groups: 0 uxx, 1 uyy, 2 uzz, 3 w (all three flux divergences), 4 xy, 5 xz, 6 yz
template <class S, int R>
__global__ void __launch_bounds__(256) k_adj_t2(Geom g, DevPtrs p, AdjPtrs a) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
    CELL_INDEX
    // forward: uxx = bwd_x vx (x slot 4), uxy = fwd_y vx (y slot 6, half), uxz = fwd_z vx (z slot 6, half), ...
    Q::ad(a.lf[BEHF_VX])[c] -= Q::fwdL(g, p, a, 0, 0, 4, false, i, j, k) + Q::bwdL(g, p, a, 4, 1, 6, true, i, j, k) +
                               Q::bwdL(g, p, a, 5, 2, 6, true, i, j, k);
    Q::ad(a.lf[BEHF_VY])[c] -= Q::fwdL(g, p, a, 1, 1, 4, false, i, j, k) + Q::bwdL(g, p, a, 4, 0, 6, true, i, j, k) +
                               Q::bwdL(g, p, a, 6, 2, 7, true, i, j, k);
    Q::ad(a.lf[BEHF_VZ])[c] -= Q::fwdL(g, p, a, 2, 2, 4, false, i, j, k) + Q::bwdL(g, p, a, 5, 0, 7, true, i, j, k) +
                               Q::bwdL(g, p, a, 6, 1, 7, true, i, j, k);
    Q::ad(a.lf[BEHF_QX])[c] -= Q::fwdL(g, p, a, 3, 0, 5, false, i, j, k);
    Q::ad(a.lf[BEHF_QY])[c] -= Q::fwdL(g, p, a, 3, 1, 5, false, i, j, k);
    Q::ad(a.lf[BEHF_QZ])[c] -= Q::fwdL(g, p, a, 3, 2, 5, false, i, j, k);
}

template <class S, int R>
__global__ void __launch_bounds__(256) k_adj_t3(Geom g, DevPtrs p, AdjPtrs a) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
    CELL_INDEX
    const int si = slab_index(i, g.nx, g.L), sj = slab_index(j, g.ny, g.L), sk = slab_index(k, g.nz, g.L);
    if (si < 0 && sj < 0 && sk < 0) return;
    A t[7];
#pragma unroll
    for (int q = 0; q < 7; q++) t[q] = Q::ad(a.tmp[q])[c];
    if (si >= 0) {
        const long long so = slab_off(g, 0, i, j, k, si);
        Q::lmem(g, p, a, t[0], 0, 4, false, i, so);
        Q::lmem(g, p, a, t[3], 0, 5, false, i, so);
        Q::lmem(g, p, a, t[4], 0, 6, true, i, so);
        Q::lmem(g, p, a, t[5], 0, 7, true, i, so);
    }
    if (sj >= 0) {
        const long long so = slab_off(g, 1, i, j, k, sj);
        Q::lmem(g, p, a, t[1], 1, 4, false, j, so);
        Q::lmem(g, p, a, t[3], 1, 5, false, j, so);
        Q::lmem(g, p, a, t[4], 1, 6, true, j, so);
        Q::lmem(g, p, a, t[6], 1, 7, true, j, so);
    }
    if (sk >= 0) {
        const long long so = slab_off(g, 2, i, j, k, sk);
        Q::lmem(g, p, a, t[2], 2, 4, false, k, so);
        Q::lmem(g, p, a, t[3], 2, 5, false, k, so);
        Q::lmem(g, p, a, t[5], 2, 6, true, k, so);
        Q::lmem(g, p, a, t[6], 2, 7, true, k, so);
    }
}

// ------------------------------------------------------------------------------------------- V^T
// groups: 0..2 Sigma_x, Sigma_y, Sigma_z;  3..5 Dp_x, Dp_y, Dp_z
template <class S, int R>
__global__ void __launch_bounds__(256) k_adj_v1(Geom g, DevPtrs p, AdjPtrs a) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
    CELL_INDEX
    const bool gr = a.grad && interior(g, i, j, k);
    A sum[3] = {0, 0, 0}, dp[3] = {0, 0, 0};
    if (gr) {
        sum[0] = Q::fwd(a.cur[BEHF_SXX], c, 1) + Q::bwd(a.cur[BEHF_SXY], c, sy) + Q::bwd(a.cur[BEHF_SXZ], c, sz);
        sum[1] = Q::fwd(a.cur[BEHF_SYY], c, sy) + Q::bwd(a.cur[BEHF_SXY], c, 1) + Q::bwd(a.cur[BEHF_SYZ], c, sz);
        sum[2] = Q::fwd(a.cur[BEHF_SZZ], c, sz) + Q::bwd(a.cur[BEHF_SXZ], c, 1) + Q::bwd(a.cur[BEHF_SYZ], c, sy);
        dp[0] = Q::fwd(a.cur[BEHF_P], c, 1);
        dp[1] = Q::fwd(a.cur[BEHF_P], c, sy);
        dp[2] = Q::fwd(a.cur[BEHF_P], c, sz);
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int vw3 = (d == 2 && g.bug) ? VW3Y : VW3X + d;
        A* lvp = Q::ad(a.lf[BEHF_VX + d]) + c;
        A* lqp = Q::ad(a.lf[BEHF_QX + d]) + c;
        const A lv = *lvp, lq = *lqp;
        const A vu2 = Q::coef(g, p, VU2X + d, c);
        const A mu = lq - vu2 * lv;
        *lqp = Q::vw1(p, d, c) * mu + vu2 * lv;
        Q::ad(a.tmp[d])[c] = Q::coef(g, p, VU1X + d, c) * lv - Q::coef(g, p, VW2X + d, c) * mu;
        Q::ad(a.tmp[3 + d])[c] = -Q::coef(g, p, vw3, c) * mu;
        if (gr) {
            const A qo = Q::ls(a.qprev[d], c), qn = Q::ls(a.cur[BEHF_QX + d], c);
            Q::ad(a.g[VW1X + d])[c] += mu * qo;
            Q::ad(a.g[VW2X + d])[c] += -mu * sum[d];
            Q::ad(a.g[vw3])[c] += -mu * dp[d];
            Q::ad(a.g[VU1X + d])[c] += lv * sum[d];
            Q::ad(a.g[VU2X + d])[c] += -lv * (qn - qo);
        }
    }
}

template <class S, int R>
__global__ void __launch_bounds__(256) k_adj_v2(Geom g, DevPtrs p, AdjPtrs a) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
    CELL_INDEX
    // forward: x1 = fwd_x sxx (x slot 0, half), x2 = bwd_y sxy (y slot 2), x3 = bwd_z sxz (z slot 2),
    //          y1 = fwd_y syy (y slot 0, half), y2 = bwd_x sxy (x slot 2), y3 = bwd_z syz (z slot 3),
    //          z1 = fwd_z szz (z slot 0, half), z2 = bwd_x sxz (x slot 3), z3 = bwd_y syz (y slot 3),
    //          s1..s3 = fwd p (slot 1, half)
    Q::ad(a.lf[BEHF_SXX])[c] -= Q::bwdL(g, p, a, 0, 0, 0, true, i, j, k);
    Q::ad(a.lf[BEHF_SYY])[c] -= Q::bwdL(g, p, a, 1, 1, 0, true, i, j, k);
    Q::ad(a.lf[BEHF_SZZ])[c] -= Q::bwdL(g, p, a, 2, 2, 0, true, i, j, k);
    Q::ad(a.lf[BEHF_SXY])[c] -= Q::fwdL(g, p, a, 0, 1, 2, false, i, j, k) + Q::fwdL(g, p, a, 1, 0, 2, false, i, j, k);
    Q::ad(a.lf[BEHF_SXZ])[c] -= Q::fwdL(g, p, a, 0, 2, 2, false, i, j, k) + Q::fwdL(g, p, a, 2, 0, 3, false, i, j, k);
    Q::ad(a.lf[BEHF_SYZ])[c] -= Q::fwdL(g, p, a, 1, 2, 3, false, i, j, k) + Q::fwdL(g, p, a, 2, 1, 3, false, i, j, k);
    Q::ad(a.lf[BEHF_P])[c] -= Q::bwdL(g, p, a, 3, 0, 1, true, i, j, k) + Q::bwdL(g, p, a, 4, 1, 1, true, i, j, k) +
                              Q::bwdL(g, p, a, 5, 2, 1, true, i, j, k);
}

template <class S, int R>
__global__ void __launch_bounds__(256) k_adj_v3(Geom g, DevPtrs p, AdjPtrs a) {
    typedef Adj<S, R> Q;
    typedef typename Q::A A;
    CELL_INDEX
    const int si = slab_index(i, g.nx, g.L), sj = slab_index(j, g.ny, g.L), sk = slab_index(k, g.nz, g.L);
    if (si < 0 && sj < 0 && sk < 0) return;
    A t[6];
#pragma unroll
    for (int q = 0; q < 6; q++) t[q] = Q::ad(a.tmp[q])[c];
    if (si >= 0) {
        const long long so = slab_off(g, 0, i, j, k, si);
        Q::lmem(g, p, a, t[0], 0, 0, true, i, so);
        Q::lmem(g, p, a, t[3], 0, 1, true, i, so);
        Q::lmem(g, p, a, t[1], 0, 2, false, i, so);
        Q::lmem(g, p, a, t[2], 0, 3, false, i, so);
    }
    if (sj >= 0) {
        const long long so = slab_off(g, 1, i, j, k, sj);
        Q::lmem(g, p, a, t[1], 1, 0, true, j, so);
        Q::lmem(g, p, a, t[4], 1, 1, true, j, so);
        Q::lmem(g, p, a, t[0], 1, 2, false, j, so);
        Q::lmem(g, p, a, t[2], 1, 3, false, j, so);
    }
    if (sk >= 0) {
        const long long so = slab_off(g, 2, i, j, k, sk);
        Q::lmem(g, p, a, t[2], 2, 0, true, k, so);
        Q::lmem(g, p, a, t[5], 2, 1, true, k, so);
        Q::lmem(g, p, a, t[0], 2, 2, false, k, so);
        Q::lmem(g, p, a, t[1], 2, 3, false, k, so);
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
__global__ void k_adj_point(AdjPtrs a, long long o, int kind, int phase, double fac, const float* w, int nw, int it,
                            double* gw, double* gfac) {
    auto L = [&](int q) { return (double)reinterpret_cast<const A*>(a.lf[q])[o]; };
    if (phase == 0) {
        if (kind != BEHF_SRC_FORCE_Z) return;
        const double lvz = L(BEHF_VZ);
        gw[it] = fac * lvz;
        if (it < nw) *gfac += (double)w[it] * lvz;  // samples past the wavelet are not injected
    } else {
        if (kind == BEHF_SRC_EXPLOSIVE) gw[it] = fac * (L(BEHF_SXX) + L(BEHF_SYY) + L(BEHF_SZZ));
        else if (kind == BEHF_SRC_PRESSURE) gw[it] = fac * L(BEHF_P);
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
cudaError_t adj_t_r(const Geom& g, const DevPtrs& p, const AdjPtrs& a, cudaStream_t st) {
    const dim3 block(32, 8, 1);
    const dim3 grid((g.nx - 2 * R + 31) / 32, (g.ny - 2 * R + 7) / 8, g.nz - 2 * R);
    k_adj_t1<S, R><<<grid, block, 0, st>>>(g, p, a);
    k_adj_t2<S, R><<<grid, block, 0, st>>>(g, p, a);
    if (g.W > 0) k_adj_t3<S, R><<<grid, block, 0, st>>>(g, p, a);
    return cudaGetLastError();
}
template <class S, int R>
cudaError_t adj_v_r(const Geom& g, const DevPtrs& p, const AdjPtrs& a, cudaStream_t st) {
    const dim3 block(32, 8, 1);
    const dim3 grid((g.nx - 2 * R + 31) / 32, (g.ny - 2 * R + 7) / 8, g.nz - 2 * R);
    k_adj_v1<S, R><<<grid, block, 0, st>>>(g, p, a);
    k_adj_v2<S, R><<<grid, block, 0, st>>>(g, p, a);
    if (g.W > 0) k_adj_v3<S, R><<<grid, block, 0, st>>>(g, p, a);
    return cudaGetLastError();
}

}  // namespace

template <class S>
cudaError_t adj_step_t(const Geom& g, const DevPtrs& p, const AdjPtrs& a, cudaStream_t st) {
    switch (g.R) {
        case 1: return adj_t_r<S, 1>(g, p, a, st);
        case 2: return adj_t_r<S, 2>(g, p, a, st);
        case 3: return adj_t_r<S, 3>(g, p, a, st);
        case 4: return adj_t_r<S, 4>(g, p, a, st);
    }
    return cudaErrorInvalidValue;
}
template <class S>
cudaError_t adj_step_v(const Geom& g, const DevPtrs& p, const AdjPtrs& a, cudaStream_t st) {
    switch (g.R) {
        case 1: return adj_v_r<S, 1>(g, p, a, st);
        case 2: return adj_v_r<S, 2>(g, p, a, st);
        case 3: return adj_v_r<S, 3>(g, p, a, st);
        case 4: return adj_v_r<S, 4>(g, p, a, st);
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
cudaError_t adj_point(const AdjPtrs& a, long long o, int kind, int phase, double fac, const float* w, int nw, int it,
                      double* gw, double* gfac, cudaStream_t st) {
    k_adj_point<typename Traits<S>::C><<<1, 1, 0, st>>>(a, o, kind, phase, fac, w, nw, it, gw, gfac);
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
    template cudaError_t adj_step_t<S>(const Geom&, const DevPtrs&, const AdjPtrs&, cudaStream_t);             \
    template cudaError_t adj_step_v<S>(const Geom&, const DevPtrs&, const AdjPtrs&, cudaStream_t);             \
    template cudaError_t adj_record<S>(const AdjPtrs&, const long long*, const int*, int, const double*, int, int, \
                                       const AdjScales&, cudaStream_t);                                          \
    template cudaError_t adj_point<S>(const AdjPtrs&, long long, int, int, double, const float*, int, int,      \
                                      double*, double*, cudaStream_t);
BEHF_ADJ_INST(double)
BEHF_ADJ_INST(float)
BEHF_ADJ_INST(__half)
BEHF_ADJ_INST(__nv_bfloat16)
template cudaError_t adj_grad_moduli<float>(const GradModArgs&, cudaStream_t);
template cudaError_t adj_grad_moduli<double>(const GradModArgs&, cudaStream_t);

}  // namespace behf
