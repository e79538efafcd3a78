// kernels_tiled_ws.cuh -- warp-specialised z-marching velocity / stress kernels (included by kernels_tiled_impl.cuh).
//
// Same tile, stencils and arithmetic as k_vel / k_str, but every global read goes through TMA: a ninth warp (the
// producer; one elected lane) issues, for plane k + NS - 1, the xy-halo boxes, the next z-ring plane and also the
// cell-owned boxes (the previous v / q or sigma / p and the coefficients, VW1 in FP32) into an NS-stage
// shared-memory ring, while the eight compute warps work on plane k.  The compute warps then read everything
// from shared memory and never wait on a global load (the classic kernels' own-cell loads are their dominant
// stall); bytes in flight per SM are set by the ring depth, not by the registers a thread can hold.
// Full/empty mbarriers order the stages; every wait is bounded as in the classic kernels.  The producer leaves only
// after the last copies it issued have landed, also when the compute warps left on an error.
#pragma once

namespace behf {
namespace BEHF_TILED_NAMESPACE {

#ifndef BEHF_WS_NS
#define BEHF_WS_NS 2
#endif
// CTAs per SM the launch bounds aim for: 2 for the 16-bit kinds (106 KB of shared memory each at R = 4), 1 for FP32.
#ifndef BEHF_WS_MINB16
#define BEHF_WS_MINB16 2
#endif
constexpr int NTH_WS = NTH + 32;

template <class S> struct WDepth {
    static constexpr int NS = BEHF_WS_NS;
    static constexpr int MINB = sizeof(S) == 2 ? BEHF_WS_MINB16 : 1;
};

// Shared-memory map: NS stages of [halo boxes | own field boxes | own FP32 Darcy boxes | own coefficient boxes],
// then the z ring of the four fields with a z derivative (2R + NS planes each, as in Map).
template <class S, int R, bool VEL>
struct WMap {
    typedef Geo<S, R> G;
    static constexpr int NS = WDepth<S>::NS;
    static constexpr int ZS = 2 * R + NS;
    static constexpr int X = al128(G::X_B), Y = al128(G::Y_B), XY = al128(G::XY_B), OW = al128(G::OWN_B);
    static constexpr int OK = al128(G::KOWN_B), OWW = al128(G::WOWN_B);
    static constexpr int NF = VEL ? 6 : 7, NW = VEL ? 3 : 0, NK = VEL ? 9 : 7;
    __host__ __device__ static constexpr int halo(int i) { return Map<S, R, VEL>::halo(i); }
    static constexpr int own_f = VEL ? 2 * X + 2 * Y + 2 * XY : 3 * XY + X + Y;
    static constexpr int own_w = own_f + NF * OW;
    static constexpr int own_k = own_w + NW * OWW;
    static constexpr int stage = own_k + NK * OK;
    static constexpr int ring = NS * stage;
    static constexpr int bytes = ring + 4 * ZS * OW;
    static constexpr uint32_t stage_tx = Map<S, R, VEL>::stage_tx + NF * G::OWN_B + NW * G::WOWN_B + NK * G::KOWN_B;
};

// Producer loop of one CTA (one lane): fills stage it % NS with plane kb + it once every compute warp has released
// the stage's previous plane, then waits until the last copies of every stage have landed.
template <int NS, class Issue>
__device__ __forceinline__ void ws_produce(uint64_t* full, uint64_t* empty, int kb, int ke, int* err, Issue&& issue) {
    int issued[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) issued[s] = 0;
    bool ok = true;
    for (int k = kb, it = 0; k < ke; k++, it++) {
        const int s = it % NS;
        if (it >= NS && !mbar_wait(&empty[s], ((it / NS) - 1) & 1)) {
            ok = false;
            break;
        }
        fence_async();
        issue(s, k, k == kb);  // the first plane also brings the z-ring warm-up
        issued[s]++;
    }
    if (!ok) atomicExch(err, 1);
#pragma unroll
    for (int s = 0; s < NS; s++)
        if (issued[s]) mbar_wait(&full[s], (issued[s] - 1) & 1);
}

// ----------------------------------------------------------------------------------------- velocity
template <class S, int R>
__global__ void __launch_bounds__(NTH_WS, WDepth<S>::MINB)
    k_vel_ws(const __grid_constant__ VMaps maps, const Geom g, const DevPtrs p, const int zchunk) {
    typedef Pair<S> PS;
    typedef typename PS::T P;
    typedef typename Traits<S>::K K;
    typedef typename Pair<K>::T KP;
    typedef Geo<S, R> G;
    typedef WMap<S, R, true> M;
    constexpr int NS = M::NS;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bfull[NS], bempty[NS];
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
        fence_init();
    }
    __syncthreads();

    if (ty == NWARP) {  // producer warp
        if (tx == 0) {
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
#pragma unroll
                for (int f = 0; f < 6; f++) tma3(b + M::own_f + f * M::OW, &maps.own[f], br, x0, y0, k);
#pragma unroll
                for (int a = 0; a < 3; a++) tma3(b + M::own_w + a * M::OWW, &maps.own[6 + a], br, x0, y0, k);
#pragma unroll
                for (int j = 0; j < 9; j++) tma3(b + M::own_k + j * M::OK, &maps.own[9 + j], br, x0, y0, k);
                const int z0 = warm ? k - R : k + R;
                for (int z = z0; z <= k + R; z++)
#pragma unroll
                    for (int f = 0; f < 4; f++)
                        tma3(smem + M::ring + (f * M::ZS + z % M::ZS) * M::OW, &maps.zlead[f], br, x0, y0, z);
            };
            ws_produce<NS>(bfull, bempty, kb, ke, g.err, issue);
        }
        return;
    }

    const int xl = 2 * tx, x = x0 + xl, y = y0 + ty;
    const bool a0 = x >= R && x < g.nx - R, a1 = x + 1 >= R && x + 1 < g.nx - R;
    const bool live = (y >= R && y < g.ny - R) && (a0 || a1);
    const long long col = (long long)y * g.px + x;
    const int oe = ty * TXC + xl;
    const uint32_t seed = g.sr ? mix32((uint32_t)(*g.step + g.step_off) * 0x9e3779b9u + 0x2545f491u) : 0u;

    bool failed = false;
    for (int k = kb, it = 0; k < ke; k++, it++) {
        const int st = it % NS;
        const bool ok = mbar_wait(&bfull[st], (it / NS) & 1);
        if (!__all_sync(0xffffffffu, ok)) {  // warp-uniform exit: every lane leaves together
            failed = true;
            break;
        }
        const unsigned char* b = smem + st * M::stage;
        if (live) {
            const long long go = (long long)k * g.plane + col;
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
                const bool hf[4] = {true, true, false, false};
                pml_pair<0, true>(g, p, x, y, k, a0, a1, x1, s1, y2, z2, hf, y1, s2, x2, z3, hf, z1, s3, x3, y3, hf);
            }
            const float2 sum[3] = {add2(add2(x1, x2), x3), add2(add2(y1, y2), y3), add2(add2(z1, z2), z3)};
            const float2 dp[3] = {s1, s2, s3};
            auto own = [&](int f) { return PS::f2(*reinterpret_cast<const P*>(b + M::own_f + f * M::OW + oe * sizeof(S))); };
            auto coef = [&](int j, int kidx) {
                const KP kv = *reinterpret_cast<const KP*>(b + M::own_k + j * M::OK + oe * sizeof(K));
                return mul2(Pair<K>::f2(kv), f2(g.kmulf[kidx], g.kmulf[kidx]));
            };
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
                const P qs = g.sr ? SR<S>::pack(qn, mix32(seed ^ (uint32_t)go ^ (0x3c6ef372u * (uint32_t)(a + 1))))
                                  : PS::pack(qn);
                store_pair<S>(reinterpret_cast<S*>(p.f[BEHF_QX + a]) + go, qs, a0, a1);
                // v' = v + VU1 sum(d sigma) - VU2 (q' - q)
                const float2 dq = sub2(PS::f2(qs), qo);
                const float2 vn = fma2(vu1, sum[a], fma2(make_float2(-vu2.x, -vu2.y), dq, own(a)));
                const P vs = g.sr ? SR<S>::pack(vn, mix32(seed ^ (uint32_t)go ^ (0x1b873593u * (uint32_t)(a + 1))))
                                  : PS::pack(vn);
                store_pair<S>(reinterpret_cast<S*>(p.f[BEHF_VX + a]) + go, vs, a0, a1);
            }
        }
        __syncwarp();
        if (tx == 0) mbar_arrive(&bempty[st]);
    }
    if (failed) atomicExch(g.err, 1);
}

// ----------------------------------------------------------------------------------------- stress
template <class S, int R>
__global__ void __launch_bounds__(NTH_WS, WDepth<S>::MINB)
    k_str_ws(const __grid_constant__ TMaps maps, const Geom g, const DevPtrs p, const int zchunk) {
    typedef Pair<S> PS;
    typedef typename PS::T P;
    typedef typename Traits<S>::K K;
    typedef typename Pair<K>::T KP;
    typedef Geo<S, R> G;
    typedef WMap<S, R, false> M;
    constexpr int NS = M::NS;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bfull[NS], bempty[NS];
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
        fence_init();
    }
    __syncthreads();

    if (ty == NWARP) {  // producer warp
        if (tx == 0) {
            auto issue = [&](int st, int k, bool warm) {
                unsigned char* b = smem + st * M::stage;
                uint64_t* br = &bfull[st];
                mbar_expect_tx(br, M::stage_tx + 4 * G::OWN_B * (warm ? 2 * R + 1 : 1));
                tma3(b + M::halo(0), &maps.halo[0], br, x0 - G::HX, y0 - R, k);  // vx (x, y halo)
                tma3(b + M::halo(1), &maps.halo[1], br, x0 - G::HX, y0 - R, k);  // vy
                tma3(b + M::halo(2), &maps.halo[2], br, x0 - G::HX, y0 - R, k);  // vz
                tma3(b + M::halo(3), &maps.halo[3], br, x0 - G::HX, y0, k);      // qx (x halo)
                tma3(b + M::halo(4), &maps.halo[4], br, x0, y0 - R, k);          // qy (y halo)
#pragma unroll
                for (int f = 0; f < 7; f++) tma3(b + M::own_f + f * M::OW, &maps.own[f], br, x0, y0, k);
#pragma unroll
                for (int j = 0; j < 7; j++) tma3(b + M::own_k + j * M::OK, &maps.own[7 + j], br, x0, y0, k);
                const int z0 = warm ? k - R : k + R;
                for (int z = z0; z <= k + R; z++)
#pragma unroll
                    for (int f = 0; f < 4; f++)
                        tma3(smem + M::ring + (f * M::ZS + z % M::ZS) * M::OW, &maps.zlead[f], br, x0, y0, z);
            };
            ws_produce<NS>(bfull, bempty, kb, ke, g.err, issue);
        }
        return;
    }

    const int xl = 2 * tx, x = x0 + xl, y = y0 + ty;
    const bool a0 = x >= R && x < g.nx - R, a1 = x + 1 >= R && x + 1 < g.nx - R;
    const bool live = (y >= R && y < g.ny - R) && (a0 || a1);
    const long long col = (long long)y * g.px + x;
    const int oe = ty * TXC + xl;
    const uint32_t seed = g.sr ? mix32((uint32_t)(*g.step + g.step_off) * 0x9e3779b9u + 0x6a09e667u) : 0u;

    bool failed = false;
    for (int k = kb, it = 0; k < ke; k++, it++) {
        const int st = it % NS;
        const bool ok = mbar_wait(&bfull[st], (it / NS) & 1);
        if (!__all_sync(0xffffffffu, ok)) {
            failed = true;
            break;
        }
        const unsigned char* b = smem + st * M::stage;
        if (live) {
            const long long go = (long long)k * g.plane + col;
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
                const bool hf[4] = {false, false, true, true};
                pml_pair<4, true>(g, p, x, y, k, a0, a1, uxx, wx, uyx, uzx, hf, uyy, wy, uxy, uzy, hf, uzz, wz, uxz, uyz, hf);
            }
            const float2 dv = add2(add2(uxx, uyy), uzz);
            const float2 dq = add2(add2(wx, wy), wz);
            auto kc = [&](int q) {
                const int j = q < 4 ? P1 + q : P1 + q + 1;
                const KP kv = *reinterpret_cast<const KP*>(b + M::own_k + q * M::OK + oe * sizeof(K));
                return mul2(Pair<K>::f2(kv), f2(g.kmulf[j], g.kmulf[j]));
            };
            auto own = [&](int q) { return PS::f2(*reinterpret_cast<const P*>(b + M::own_f + q * M::OW + oe * sizeof(S))); };
            auto put = [&](int field, float2 v) {
                const P sv = g.sr ? SR<S>::pack(v, mix32(seed ^ (uint32_t)go ^ (0x85ebca6bu * (uint32_t)(field + 1))))
                                  : PS::pack(v);
                store_pair<S>(reinterpret_cast<S*>(p.f[field]) + go, sv, a0, a1);
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
        }
        __syncwarp();
        if (tx == 0) mbar_arrive(&bempty[st]);
    }
    if (failed) atomicExch(g.err, 1);
}

}  // namespace BEHF_TILED_NAMESPACE
}  // namespace behf
