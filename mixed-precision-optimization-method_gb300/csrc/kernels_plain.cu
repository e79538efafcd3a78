// kernels_plain.cu -- one thread per cell velocity and stress updates (all precisions, R = 1..4).
//
// The straightforward form of the BEHF update: every neighbour is a cached global load.  It is the
// correctness baseline of the tiled kernels and, in FP32, the "plain FP32 kernel" they are measured
// against.  Equations (reference kernel.cu):
//   V (FD_V*, kernel.cu:172-225): 12 staggered differences of sigma and p, trapezoidal CPML on the
//     slab cells, Crank-Nicolson Darcy  q' = VW1 q - VW2 sum(d sigma) - VW3 d p,
//     solid  v' = v + VU1 sum(d sigma) - VU2 (q' - q).
//   T (FD_T*, kernel.cu:430-490): 12 differences of v and q, CPML,
//     p' = p - P1 div v - P2 div q,  s_ii' = s_ii + S1 (d_jj v + d_kk v) + S2 d_ii v + S3 div q,
//     s_ij' = s_ij + S_ij (d_j v_i + d_i v_j).
// Forward differences (at i+1/2) take the half-shifted damping profile, backward ones the integer
// profile, as the reference pairs e_dxi2/dxi2 with forward and e_dxi/dxi with backward differences.
#include "behf_internal.cuh"

namespace behf {
namespace {

template <class S, int R>
struct Plain {
    typedef Traits<S> T;
    typedef typename T::C C;
    typedef typename T::K K;
    typedef typename T::W W;

    static __device__ __forceinline__ C ldf(const void* f, long long o) {
        return T::ld(__ldg(reinterpret_cast<const S*>(f) + o));
    }
    static __device__ __forceinline__ C fwd(const void* f, long long o, long long s) {
        C acc = (C)stencil_w<R>(1) * (ldf(f, o + s) - ldf(f, o));
#pragma unroll
        for (int m = 2; m <= R; m++) acc += (C)stencil_w<R>(m) * (ldf(f, o + m * s) - ldf(f, o - (m - 1) * s));
        return acc;
    }
    static __device__ __forceinline__ C bwd(const void* f, long long o, long long s) {
        C acc = (C)stencil_w<R>(1) * (ldf(f, o) - ldf(f, o - s));
#pragma unroll
        for (int m = 2; m <= R; m++) acc += (C)stencil_w<R>(m) * (ldf(f, o + (m - 1) * s) - ldf(f, o - m * s));
        return acc;
    }
    static __device__ __forceinline__ C coef(const Geom& g, const DevPtrs& p, int j, long long o) {
        const C v = T::ldk(__ldg(reinterpret_cast<const K*>(p.k[j]) + o));
        if constexpr (sizeof(C) == 8) return v * (C)g.kmuld[j];
        else return v * g.kmulf[j];
    }
    // psi = A psi + B (A prev + D); prev = D; return D + psi   (kernel.cu:188-216)
    static __device__ __forceinline__ C pml(C D, const DevPtrs& p, int ax, int slot, long long so, C A, C B) {
        W* ps = reinterpret_cast<W*>(p.psi[ax][slot]) + so;
        W* pv = reinterpret_cast<W*>(p.prv[ax][slot]) + so;
        const C pn = A * (C)(*ps) + B * (A * (C)(*pv) + D);
        *ps = (W)pn;
        *pv = (W)D;
        return D + (C)(W)pn;
    }
    static __device__ __forceinline__ C prof(const void* a, int i) { return reinterpret_cast<const C*>(a)[i]; }

    static __device__ void vel(const Geom& g, const DevPtrs& p, int i, int j, int k) {
        const long long sy = g.px, sz = g.plane;
        const long long c = k * sz + j * sy + i;
        C x1 = fwd(p.f[BEHF_SXX], c, 1), x2 = bwd(p.f[BEHF_SXY], c, sy), x3 = bwd(p.f[BEHF_SXZ], c, sz);
        C s1 = fwd(p.f[BEHF_P], c, 1);
        C y1 = fwd(p.f[BEHF_SYY], c, sy), y2 = bwd(p.f[BEHF_SXY], c, 1), y3 = bwd(p.f[BEHF_SYZ], c, sz);
        C s2 = fwd(p.f[BEHF_P], c, sy);
        C z1 = fwd(p.f[BEHF_SZZ], c, sz), z2 = bwd(p.f[BEHF_SXZ], c, 1), z3 = bwd(p.f[BEHF_SYZ], c, sy);
        C s3 = fwd(p.f[BEHF_P], c, sz);
        if (g.W > 0) {
            const int si = slab_index(i, g.nx, g.L), sj = slab_index(j, g.ny, g.L), sk = slab_index(k, g.nz, g.L);
            if (si >= 0) {
                const long long so = ((long long)k * g.ny + j) * g.W + si;
                const C A = prof(p.pa[0], i), B = prof(p.pb[0], i), A2 = prof(p.pa2[0], i), B2 = prof(p.pb2[0], i);
                x1 = pml(x1, p, 0, 0, so, A2, B2);
                s1 = pml(s1, p, 0, 1, so, A2, B2);
                y2 = pml(y2, p, 0, 2, so, A, B);
                z2 = pml(z2, p, 0, 3, so, A, B);
            }
            if (sj >= 0) {
                const long long so = ((long long)k * g.W + sj) * g.nx + i;
                const C A = prof(p.pa[1], j), B = prof(p.pb[1], j), A2 = prof(p.pa2[1], j), B2 = prof(p.pb2[1], j);
                y1 = pml(y1, p, 1, 0, so, A2, B2);
                s2 = pml(s2, p, 1, 1, so, A2, B2);
                x2 = pml(x2, p, 1, 2, so, A, B);
                z3 = pml(z3, p, 1, 3, so, A, B);
            }
            if (sk >= 0) {
                const long long so = ((long long)sk * g.ny + j) * g.nx + i;
                const C A = prof(p.pa[2], k), B = prof(p.pb[2], k), A2 = prof(p.pa2[2], k), B2 = prof(p.pb2[2], k);
                z1 = pml(z1, p, 2, 0, so, A2, B2);
                s3 = pml(s3, p, 2, 1, so, A2, B2);
                x3 = pml(x3, p, 2, 2, so, A, B);
                y3 = pml(y3, p, 2, 3, so, A, B);
            }
        }
        const C sum[3] = {x1 + x2 + x3, y1 + y2 + y3, z1 + z2 + z3};
        const C dp[3] = {s1, s2, s3};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int vw3 = (a == 2 && g.bug) ? VW3Y : VW3X + a;
            S* q = reinterpret_cast<S*>(p.f[BEHF_QX + a]) + c;
            S* v = reinterpret_cast<S*>(p.f[BEHF_VX + a]) + c;
            const C vw1 = (C)reinterpret_cast<const W*>(p.k[VW1X + a])[c];
            const C qo = T::ld(*q);
            const C qn = vw1 * qo - coef(g, p, VW2X + a, c) * sum[a] - coef(g, p, vw3, c) * dp[a];
            const S qs = T::st(qn);
            *q = qs;
            const C dq = T::ld(qs) - qo;
            *v = T::st(T::ld(*v) + coef(g, p, VU1X + a, c) * sum[a] - coef(g, p, VU2X + a, c) * dq);
        }
    }

    static __device__ void str(const Geom& g, const DevPtrs& p, int i, int j, int k) {
        const long long sy = g.px, sz = g.plane;
        const long long c = k * sz + j * sy + i;
        C uxx = bwd(p.f[BEHF_VX], c, 1), uyy = bwd(p.f[BEHF_VY], c, sy), uzz = bwd(p.f[BEHF_VZ], c, sz);
        C wx = bwd(p.f[BEHF_QX], c, 1), wy = bwd(p.f[BEHF_QY], c, sy), wz = bwd(p.f[BEHF_QZ], c, sz);
        C uxy = fwd(p.f[BEHF_VX], c, sy), uyx = fwd(p.f[BEHF_VY], c, 1);
        C uxz = fwd(p.f[BEHF_VX], c, sz), uzx = fwd(p.f[BEHF_VZ], c, 1);
        C uyz = fwd(p.f[BEHF_VY], c, sz), uzy = fwd(p.f[BEHF_VZ], c, sy);
        if (g.W > 0) {
            const int si = slab_index(i, g.nx, g.L), sj = slab_index(j, g.ny, g.L), sk = slab_index(k, g.nz, g.L);
            if (si >= 0) {
                const long long so = ((long long)k * g.ny + j) * g.W + si;
                const C A = prof(p.pa[0], i), B = prof(p.pb[0], i), A2 = prof(p.pa2[0], i), B2 = prof(p.pb2[0], i);
                uxx = pml(uxx, p, 0, 4, so, A, B);
                wx = pml(wx, p, 0, 5, so, A, B);
                uyx = pml(uyx, p, 0, 6, so, A2, B2);
                uzx = pml(uzx, p, 0, 7, so, A2, B2);
            }
            if (sj >= 0) {
                const long long so = ((long long)k * g.W + sj) * g.nx + i;
                const C A = prof(p.pa[1], j), B = prof(p.pb[1], j), A2 = prof(p.pa2[1], j), B2 = prof(p.pb2[1], j);
                uyy = pml(uyy, p, 1, 4, so, A, B);
                wy = pml(wy, p, 1, 5, so, A, B);
                uxy = pml(uxy, p, 1, 6, so, A2, B2);
                uzy = pml(uzy, p, 1, 7, so, A2, B2);
            }
            if (sk >= 0) {
                const long long so = ((long long)sk * g.ny + j) * g.nx + i;
                const C A = prof(p.pa[2], k), B = prof(p.pb[2], k), A2 = prof(p.pa2[2], k), B2 = prof(p.pb2[2], k);
                uzz = pml(uzz, p, 2, 4, so, A, B);
                wz = pml(wz, p, 2, 5, so, A, B);
                uxz = pml(uxz, p, 2, 6, so, A2, B2);
                uyz = pml(uyz, p, 2, 7, so, A2, B2);
            }
        }
        const C dv = uxx + uyy + uzz, dq = wx + wy + wz;
        const C g1 = coef(g, p, S1, c), g2 = coef(g, p, S2, c), g3 = coef(g, p, S3, c);
        auto upd = [&](int q, C inc) {
            S* f = reinterpret_cast<S*>(p.f[q]) + c;
            *f = T::st(T::ld(*f) + inc);
        };
        {
            S* f = reinterpret_cast<S*>(p.f[BEHF_P]) + c;
            *f = T::st(T::ld(*f) - coef(g, p, P1, c) * dv - coef(g, p, P2, c) * dq);
        }
        upd(BEHF_SXX, g1 * (uyy + uzz) + g2 * uxx + g3 * dq);
        upd(BEHF_SYY, g1 * (uxx + uzz) + g2 * uyy + g3 * dq);
        upd(BEHF_SZZ, g1 * (uxx + uyy) + g2 * uzz + g3 * dq);
        upd(BEHF_SXY, coef(g, p, SXYC, c) * (uxy + uyx));
        upd(BEHF_SYZ, coef(g, p, SYZC, c) * (uyz + uzy));
        upd(BEHF_SXZ, coef(g, p, SXZC, c) * (uxz + uzx));
    }
};

template <class S, int R, bool VEL>
__global__ void __launch_bounds__(256) k_plain(Geom g, DevPtrs p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + R;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + R;
    const int k = blockIdx.z + R;
    if (i >= g.nx - R || j >= g.ny - R || k >= g.nz - R) return;
    if (VEL) Plain<S, R>::vel(g, p, i, j, k);
    else Plain<S, R>::str(g, p, i, j, k);
}

template <class S, int R>
cudaError_t launch_r(const Geom& g, const DevPtrs& p, bool vel, cudaStream_t st) {
    const dim3 block(32, 8, 1);
    const dim3 grid((g.nx - 2 * R + 31) / 32, (g.ny - 2 * R + 7) / 8, g.nz - 2 * R);
    if (vel) k_plain<S, R, true><<<grid, block, 0, st>>>(g, p);
    else k_plain<S, R, false><<<grid, block, 0, st>>>(g, p);
    return cudaGetLastError();
}

}  // namespace

template <class S>
cudaError_t launch_plain(const Geom& g, const DevPtrs& p, bool vel, cudaStream_t st) {
    switch (g.R) {
        case 1: return launch_r<S, 1>(g, p, vel, st);
        case 2: return launch_r<S, 2>(g, p, vel, st);
        case 3: return launch_r<S, 3>(g, p, vel, st);
        case 4: return launch_r<S, 4>(g, p, vel, st);
    }
    return cudaErrorInvalidValue;
}

template cudaError_t launch_plain<double>(const Geom&, const DevPtrs&, bool, cudaStream_t);
template cudaError_t launch_plain<float>(const Geom&, const DevPtrs&, bool, cudaStream_t);
template cudaError_t launch_plain<__half>(const Geom&, const DevPtrs&, bool, cudaStream_t);
template cudaError_t launch_plain<__nv_bfloat16>(const Geom&, const DevPtrs&, bool, cudaStream_t);

}  // namespace behf
