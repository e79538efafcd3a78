// behf_oracle.cpp -- CPU oracle for the BEHF poroelastic time stepper.
//
// TEST INFRASTRUCTURE ONLY: the checker of the CUDA path.  Nothing in the product library
// links, loads or calls this file.  See behf_oracle.h for the list of reference lines each
// part restates.  Built with -ffp-contract=off so that x86 and Arm hosts give identical bits.
#include "behf_oracle.h"

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ----------------------------------------------------------------------------------------
// Storage emulation.  binary16 uses the compiler's _Float16 (IEEE round-to-nearest-even on
// both gcc/x86 and gcc/aarch64).  bfloat16 is rounded by hand (RNE on the float bits).
struct BF16 {
    uint16_t b;
};
static inline float bf_to_f(BF16 v) {
    uint32_t u = (uint32_t)v.b << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
static inline BF16 f_to_bf(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    BF16 r;
    if ((u & 0x7f800000u) == 0x7f800000u) {  // inf / nan: truncate, keep nan quiet
        r.b = (uint16_t)((u >> 16) | ((u & 0x007fffffu) ? 0x0040u : 0u));
        return r;
    }
    u += 0x7fffu + ((u >> 16) & 1u);
    r.b = (uint16_t)(u >> 16);
    return r;
}

template <int P> struct Prec;
template <> struct Prec<ORC_F64> {
    typedef double S;  // state
    typedef double C;  // arithmetic
    typedef double K;  // coefficients
    typedef double W;  // CPML memory + Darcy factor
    static C ld(S v) { return v; }
    static S st(C v) { return v; }
    static C ldk(K v) { return v; }
    static K stk(double v) { return v; }
    static const bool pow2 = false;
};
template <> struct Prec<ORC_F32> {
    typedef float S;
    typedef float C;
    typedef float K;
    typedef float W;
    static C ld(S v) { return v; }
    static S st(C v) { return v; }
    static C ldk(K v) { return v; }
    static K stk(double v) { return (float)v; }
    static const bool pow2 = false;
};
template <> struct Prec<ORC_F16> {
    typedef _Float16 S;
    typedef float C;
    typedef _Float16 K;
    typedef float W;
    static C ld(S v) { return (float)v; }
    static S st(C v) { return (_Float16)v; }
    static C ldk(K v) { return (float)v; }
    static K stk(double v) { return (_Float16)(float)v; }
    static const bool pow2 = true;
};
template <> struct Prec<ORC_BF16> {
    typedef BF16 S;
    typedef float C;
    typedef _Float16 K;
    typedef float W;
    static C ld(S v) { return bf_to_f(v); }
    static S st(C v) { return f_to_bf(v); }
    static C ldk(K v) { return (float)v; }
    static K stk(double v) { return (_Float16)(float)v; }
    static const bool pow2 = true;
};

// Staggered first-derivative weights of order 2R (Taylor / Fornberg), R = 1..4.
static const double kStencil[4][4] = {
    {1.0, 0, 0, 0},
    {9.0 / 8.0, -1.0 / 24.0, 0, 0},
    {75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0, 0},
    {1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0},
};

// Slab index of a cell along one axis: [0,L) -> 0..L-1, [n-1-L, n) -> L..2L, else -1.
static inline int slab_index(int i, int n, int L) {
    if (i < L) return i;
    if (i >= n - 1 - L) return L + (i - (n - 1 - L));
    return -1;
}

static double g_step_seconds = 0.0;

static double wall_seconds() {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

static void set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

}  // namespace

// ----------------------------------------------------------------------------------------
// Medium (outputfunc.cpp:153-222).  The float/double mix follows the reference: the volume
// arrays are float, the rock constants double, and HH is formed from the float-rounded M.
extern "C" void orc_medium_borehole(int nz, int ny, int nx, float* const mod[ORC_NMOD]) {
    const double porousm = 8.0;
    const double eta = 1.0 * std::pow(10.0, -3);
    for (int iz = 0; iz < nz; iz++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                const size_t c = ((size_t)iz * ny + iy) * nx + ix;
                const int dx = ix - nx / 2, dy = iy - ny / 2;
                if (dx * dx + dy * dy <= 100) {  // fluid-filled borehole, radius 10 cells
                    float vp = 1500.0f, vf = 1500.0f, rhof = 1000.0f;
                    double Ks = rhof * vp * vp;  // float product, then widened
                    (void)Ks;
                    double Kf = rhof * vf * vf;
                    mod[ORC_RHO][c] = 1000.0f;
                    mod[ORC_RHOF][c] = rhof;
                    mod[ORC_MU][c] = 0.0f;
                    mod[ORC_C][c] = (float)Kf;
                    mod[ORC_M][c] = (float)Kf;
                    mod[ORC_HH][c] = (float)Kf;
                    mod[ORC_H2U][c] = (float)Kf;
                    mod[ORC_C1][c] = 0.0f;
                    mod[ORC_C2][c] = rhof;
                } else {  // porous formation
                    float vp = 5000.0f, vs = 3300.0f, rhos = 2450.0f, rhof = 1000.0f, vf = 1500.0f;
                    double por = 0.1;
                    float rho = (float)((1 - por) * rhos + por * rhof);
                    double perm = 2 * std::pow(10.0, -12);
                    float mu = (float)((1 - por) * rhos * vs * vs);
                    double Kb = rhos * (1 - por) * (vp * vp - vs * vs * 4.0 / 3.0);
                    double Ks = rhos * (vp * vp - vs * vs * 4.0 / 3.0);
                    double Kf = rhof * vf * vf;
                    double tao = 3.0;
                    double a1 = 1 - Kb / Ks;
                    float M = (float)(Kf * Ks / (por * Ks + (a1 - por) * Kf));
                    float HH = (float)(a1 * a1 * M + Kb + mu * 4.0 / 3.0);
                    float H2u = HH - 2 * mu;
                    mod[ORC_RHO][c] = rho;
                    mod[ORC_RHOF][c] = rhof;
                    mod[ORC_MU][c] = mu;
                    mod[ORC_M][c] = M;
                    mod[ORC_HH][c] = HH;
                    mod[ORC_H2U][c] = H2u;
                    mod[ORC_C][c] = (float)(M * a1);
                    mod[ORC_C1][c] = (float)(eta / perm);
                    mod[ORC_C2][c] = (float)((1 + 2 / porousm) * tao * rhof / por);
                }
            }
}

extern "C" void orc_rock_moduli(double Ks, double Kf, double Kdry, double mu, double rhos,
                                double rhof, double phi, double kappa, double eta, double tau,
                                double out[ORC_NMOD]) {
    const double porousm = 8.0;  // outputfunc.cpp:164
    if (phi >= 1.0) {            // pure fluid cell, as the borehole branch of outputfunc.cpp:169-187
        out[ORC_RHO] = rhof;
        out[ORC_RHOF] = rhof;
        out[ORC_MU] = 0.0;
        out[ORC_M] = out[ORC_C] = out[ORC_HH] = out[ORC_H2U] = Kf;
        out[ORC_C1] = 0.0;
        out[ORC_C2] = rhof;
        return;
    }
    const double rho = (1 - phi) * rhos + phi * rhof;
    const double a = 1 - Kdry / Ks;
    const double M = Kf * Ks / (phi * Ks + (a - phi) * Kf);
    const double HH = a * a * M + Kdry + mu * 4.0 / 3.0;
    out[ORC_RHO] = rho;
    out[ORC_RHOF] = rhof;
    out[ORC_MU] = mu;
    out[ORC_M] = M;
    out[ORC_HH] = HH;
    out[ORC_H2U] = HH - 2 * mu;
    out[ORC_C] = M * a;
    out[ORC_C1] = eta / kappa;
    out[ORC_C2] = (1 + 2 / porousm) * tau * rhof / phi;
}

// ----------------------------------------------------------------------------------------
// Physical staggered coefficients (main.cpp:322-359 averaging, 431-494 formulas), in double.
// Averages exist on cells 1..n-2 of every axis and are zero on the outer planes, as the
// reference's memset + interior loop leaves them.
extern "C" void orc_build_coeffs(int nx, int ny, int nz, double dt, const float* const mod[ORC_NMOD],
                                 double* const coef[ORC_NCOEF]) {
    const size_t sy = nx, sz = (size_t)nx * ny, N = sz * nz;
    for (int j = 0; j < ORC_NCOEF; j++) std::memset(coef[j], 0, N * sizeof(double));
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k < nz - 1; k++)
        for (int j = 1; j < ny - 1; j++)
            for (int i = 1; i < nx - 1; i++) {
                const size_t c = k * sz + j * sy + i;
                auto m = [&](int q, size_t o) { return (double)mod[q][o]; };
                auto harm4 = [&](size_t a, size_t b, size_t d, size_t e) {
                    double v0 = m(ORC_MU, a), v1 = m(ORC_MU, b), v2 = m(ORC_MU, d), v3 = m(ORC_MU, e);
                    if (v0 == 0 || v1 == 0 || v2 == 0 || v3 == 0) return 0.0;
                    return 1.0 / (0.25 * (1 / v0 + 1 / v1 + 1 / v2 + 1 / v3));
                };
                const double muxz = harm4(c, c + 1, c + sz, c + sz + 1);
                const double muyz = harm4(c, c + sy, c + sz, c + sz + sy);
                const double muxy = harm4(c, c + 1, c + sy, c + sy + 1);
                const size_t nb[3] = {c + 1, c + sy, c + sz};
                double rho[3], rhof[3], b[3], mm[3];
                for (int a = 0; a < 3; a++) {
                    rho[a] = 0.5 * (m(ORC_RHO, c) + m(ORC_RHO, nb[a]));
                    rhof[a] = 0.5 * (m(ORC_RHOF, c) + m(ORC_RHOF, nb[a]));
                    b[a] = 0.5 * (m(ORC_C1, c) + m(ORC_C1, nb[a]));
                    mm[a] = 0.5 * (m(ORC_C2, c) + m(ORC_C2, nb[a]));
                }
                if (!(b[0] == 0 || b[1] == 0 || b[2] == 0)) {
                    for (int a = 0; a < 3; a++) {
                        const double mp = mm[a] - rhof[a] * rhof[a] / rho[a];
                        const double D = mp + 0.5 * dt * b[a];
                        coef[ORC_VW1X + a][c] = (mp - 0.5 * dt * b[a]) / D;
                        coef[ORC_VW2X + a][c] = dt * (rhof[a] / rho[a]) / D;
                        coef[ORC_VW3X + a][c] = dt / D;
                    }
                }
                if (!(rho[0] == 0 || rho[1] == 0 || rho[2] == 0)) {
                    for (int a = 0; a < 3; a++) {
                        coef[ORC_VU1X + a][c] = dt / rho[a];
                        coef[ORC_VU2X + a][c] = rhof[a] / rho[a];
                    }
                }
                coef[ORC_P1][c] = m(ORC_C, c) * dt;
                coef[ORC_P2][c] = m(ORC_M, c) * dt;
                coef[ORC_S1][c] = m(ORC_H2U, c) * dt;
                coef[ORC_S2][c] = m(ORC_HH, c) * dt;
                coef[ORC_S3][c] = m(ORC_C, c) * dt;
                coef[ORC_SXYC][c] = muxy * dt;
                coef[ORC_SXZC][c] = muxz * dt;
                coef[ORC_SYZC][c] = muyz * dt;
            }
}

// CPML profile of one axis (main.cpp:537-563 and the right-face branches), double precision,
// slab membership by cell index: left [0,L), right [n-1-L, n).
extern "C" void orc_cpml_profile(int n, int L, double h, double dt, double v0, double rc, double* d,
                                 double* d2, double* e, double* e2) {
    const double DP = L * h;
    const double d0 = L > 0 ? 3.0 * v0 * std::log(1.0 / rc) / (2.0 * DP) : 0.0;
    const double xl = DP, xr = (n - 1) * h - DP;
    for (int i = 0; i < n; i++) {
        d[i] = d2[i] = e[i] = e2[i] = 0.0;
        const double x = i * h;
        if (L > 0 && i < L) {
            d[i] = d0 * std::pow((xl - x) / DP, 2);
            d2[i] = d0 * std::pow((xl - x - 0.5 * h) / DP, 2);
        } else if (L > 0 && i >= n - 1 - L) {
            d[i] = d0 * std::pow((x - xr) / DP, 2);
            d2[i] = d0 * std::pow((x + 0.5 * h - xr) / DP, 2);
        } else {
            continue;
        }
        e[i] = std::exp(-d[i] * dt);
        e2[i] = std::exp(-d2[i] * dt);
    }
}

extern "C" void orc_ricker(int nt, double dt, double f0, double t0, double amp, float* w) {
    const double pi = 3.14159265358979323846;
    for (int it = 0; it < nt; it++) {
        const double tau = it * dt - t0;
        const double a = pi * pi * f0 * f0 * tau * tau;
        w[it] = (float)(amp * -(1 - 2 * a) * std::exp(-a));
    }
}

// ----------------------------------------------------------------------------------------
// BEHF scheme run (the scheme the CUDA library implements).
namespace {

struct Axis {  // one axis of CPML memory: 8 derivatives (4 in V, 4 in T) x {psi, previous}
    int L = 0, W = 0, n = 0;
    std::vector<double> A, B, A2, B2;  // e and -dt d / 2, integer and half-shifted
};

template <int P, int R>
struct Runner {
    typedef Prec<P> Pr;
    typedef typename Pr::S S;
    typedef typename Pr::C C;
    typedef typename Pr::K K;
    typedef typename Pr::W W;

    int nx, ny, nz;
    size_t sy, sz, N;
    C cw[4];
    std::vector<S> f[ORC_NFIELD];
    std::vector<K> k16[ORC_NCOEF];  // coefficients (slot 0..2 unused: VW1 lives in vw1)
    C kmul[ORC_NCOEF];              // power-of-two multipliers of the stored coefficients
    std::vector<W> vw1[3];
    Axis ax[3];
    // CPML memory: [axis][8 derivatives][psi|prev] -> slab arrays
    std::vector<W> psi[3][8], prv[3][8];
    C Ax[3][2][1], dummy;
    std::vector<C> pa[3], pb[3], pa2[3], pb2[3];  // per-axis profiles in arithmetic type
    int bug;

    size_t slab_off(int a, int i, int j, int k, int s) const {
        if (a == 0) return ((size_t)k * ny + j) * ax[0].W + s;
        if (a == 1) return ((size_t)k * ax[1].W + s) * nx + i;
        return ((size_t)s * ny + j) * nx + i;
    }

    inline C ld(int q, size_t o) const { return Pr::ld(f[q][o]); }
    inline C fwd(int q, size_t o, size_t s) const {
        C acc = cw[0] * (ld(q, o + s) - ld(q, o));
        for (int m = 2; m <= R; m++) acc += cw[m - 1] * (ld(q, o + m * s) - ld(q, o - (m - 1) * s));
        return acc;
    }
    inline C bwd(int q, size_t o, size_t s) const {
        C acc = cw[0] * (ld(q, o) - ld(q, o - s));
        for (int m = 2; m <= R; m++) acc += cw[m - 1] * (ld(q, o + (m - 1) * s) - ld(q, o - m * s));
        return acc;
    }
    // Trapezoidal CPML memory update (kernel.cu:188-216): psi = A psi + B (A prev + D); prev = D; D += psi.
    inline C pml(C D, int a, int slot, bool half, int idx, size_t so) {
        const C A = half ? pa2[a][idx] : pa[a][idx];
        const C B = half ? pb2[a][idx] : pb[a][idx];
        W& ps = psi[a][slot][so];
        W& pv = prv[a][slot][so];
        const C pn = A * (C)ps + B * (A * (C)pv + D);
        ps = (W)pn;
        pv = (W)D;
        return D + (C)ps;
    }
    inline C coef(int j, size_t c) const { return Pr::ldk(k16[j][c]) * kmul[j]; }

    void step_v() {
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = R; k < nz - R; k++)
            for (int j = R; j < ny - R; j++) {
                const int sk = slab_index(k, nz, ax[2].L), sj = slab_index(j, ny, ax[1].L);
                for (int i = R; i < nx - R; i++) {
                    const size_t c = k * sz + j * sy + i;
                    const int si = slab_index(i, nx, ax[0].L);
                    C x1 = fwd(ORC_SXX, c, 1), x2 = bwd(ORC_SXY, c, sy), x3 = bwd(ORC_SXZ, c, sz);
                    C s1 = fwd(ORC_P, c, 1);
                    C y1 = fwd(ORC_SYY, c, sy), y2 = bwd(ORC_SXY, c, 1), y3 = bwd(ORC_SYZ, c, sz);
                    C s2 = fwd(ORC_P, c, sy);
                    C z1 = fwd(ORC_SZZ, c, sz), z2 = bwd(ORC_SXZ, c, 1), z3 = bwd(ORC_SYZ, c, sy);
                    C s3 = fwd(ORC_P, c, sz);
                    if (si >= 0) {
                        const size_t so = slab_off(0, i, j, k, si);
                        x1 = pml(x1, 0, 0, true, i, so);
                        s1 = pml(s1, 0, 1, true, i, so);
                        y2 = pml(y2, 0, 2, false, i, so);
                        z2 = pml(z2, 0, 3, false, i, so);
                    }
                    if (sj >= 0) {
                        const size_t so = slab_off(1, i, j, k, sj);
                        y1 = pml(y1, 1, 0, true, j, so);
                        s2 = pml(s2, 1, 1, true, j, so);
                        x2 = pml(x2, 1, 2, false, j, so);
                        z3 = pml(z3, 1, 3, false, j, so);
                    }
                    if (sk >= 0) {
                        const size_t so = slab_off(2, i, j, k, sk);
                        z1 = pml(z1, 2, 0, true, k, so);
                        s3 = pml(s3, 2, 1, true, k, so);
                        x3 = pml(x3, 2, 2, false, k, so);
                        y3 = pml(y3, 2, 3, false, k, so);
                    }
                    const C sum[3] = {x1 + x2 + x3, y1 + y2 + y3, z1 + z2 + z3};
                    const C dp[3] = {s1, s2, s3};
                    for (int a = 0; a < 3; a++) {
                        const int vw3 = (a == 2 && bug) ? ORC_VW3Y : ORC_VW3X + a;
                        const C qo = ld(ORC_QX + a, c);
                        const C qn = (C)vw1[a][c] * qo - coef(ORC_VW2X + a, c) * sum[a] - coef(vw3, c) * dp[a];
                        f[ORC_QX + a][c] = Pr::st(qn);
                        const C dq = Pr::ld(f[ORC_QX + a][c]) - qo;
                        const C vn = ld(ORC_VX + a, c) + coef(ORC_VU1X + a, c) * sum[a] - coef(ORC_VU2X + a, c) * dq;
                        f[ORC_VX + a][c] = Pr::st(vn);
                    }
                }
            }
    }

    void step_t() {
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = R; k < nz - R; k++)
            for (int j = R; j < ny - R; j++) {
                const int sk = slab_index(k, nz, ax[2].L), sj = slab_index(j, ny, ax[1].L);
                for (int i = R; i < nx - R; i++) {
                    const size_t c = k * sz + j * sy + i;
                    const int si = slab_index(i, nx, ax[0].L);
                    C uxx = bwd(ORC_VX, c, 1), uyy = bwd(ORC_VY, c, sy), uzz = bwd(ORC_VZ, c, sz);
                    C wx = bwd(ORC_QX, c, 1), wy = bwd(ORC_QY, c, sy), wz = bwd(ORC_QZ, c, sz);
                    C uxy = fwd(ORC_VX, c, sy), uyx = fwd(ORC_VY, c, 1);
                    C uxz = fwd(ORC_VX, c, sz), uzx = fwd(ORC_VZ, c, 1);
                    C uyz = fwd(ORC_VY, c, sz), uzy = fwd(ORC_VZ, c, sy);
                    if (si >= 0) {
                        const size_t so = slab_off(0, i, j, k, si);
                        uxx = pml(uxx, 0, 4, false, i, so);
                        wx = pml(wx, 0, 5, false, i, so);
                        uyx = pml(uyx, 0, 6, true, i, so);
                        uzx = pml(uzx, 0, 7, true, i, so);
                    }
                    if (sj >= 0) {
                        const size_t so = slab_off(1, i, j, k, sj);
                        uyy = pml(uyy, 1, 4, false, j, so);
                        wy = pml(wy, 1, 5, false, j, so);
                        uxy = pml(uxy, 1, 6, true, j, so);
                        uzy = pml(uzy, 1, 7, true, j, so);
                    }
                    if (sk >= 0) {
                        const size_t so = slab_off(2, i, j, k, sk);
                        uzz = pml(uzz, 2, 4, false, k, so);
                        wz = pml(wz, 2, 5, false, k, so);
                        uxz = pml(uxz, 2, 6, true, k, so);
                        uyz = pml(uyz, 2, 7, true, k, so);
                    }
                    const C dv = uxx + uyy + uzz, dq = wx + wy + wz;
                    const C g1 = coef(ORC_S1, c), g2 = coef(ORC_S2, c), g3 = coef(ORC_S3, c);
                    f[ORC_P][c] = Pr::st(ld(ORC_P, c) - coef(ORC_P1, c) * dv - coef(ORC_P2, c) * dq);
                    f[ORC_SXX][c] = Pr::st(ld(ORC_SXX, c) + g1 * (uyy + uzz) + g2 * uxx + g3 * dq);
                    f[ORC_SYY][c] = Pr::st(ld(ORC_SYY, c) + g1 * (uxx + uzz) + g2 * uyy + g3 * dq);
                    f[ORC_SZZ][c] = Pr::st(ld(ORC_SZZ, c) + g1 * (uxx + uyy) + g2 * uzz + g3 * dq);
                    f[ORC_SXY][c] = Pr::st(ld(ORC_SXY, c) + coef(ORC_SXYC, c) * (uxy + uyx));
                    f[ORC_SYZ][c] = Pr::st(ld(ORC_SYZ, c) + coef(ORC_SYZC, c) * (uyz + uzy));
                    f[ORC_SXZ][c] = Pr::st(ld(ORC_SXZ, c) + coef(ORC_SXZC, c) * (uxz + uzx));
                }
            }
    }

    int run(const orc_cfg* cfg, const float* const mod[ORC_NMOD], const float* wavelet, int nt, int nrec,
            const int* rec_ijk, const int* rec_comp, double* seis, double* fields_out) {
        nx = cfg->nx;
        ny = cfg->ny;
        nz = cfg->nz;
        sy = nx;
        sz = (size_t)nx * ny;
        N = sz * nz;
        bug = cfg->ref_bug_compat;
        for (int m = 0; m < 4; m++) cw[m] = (C)kStencil[R - 1][m];
        const double sv = cfg->scale[0], sq = cfg->scale[1], ss = cfg->scale[2], sp = cfg->scale[3];
        const double hi = 1.0 / cfg->h;
        const double fscale[ORC_NFIELD] = {sv, sv, sv, sq, sq, sq, ss, ss, ss, ss, ss, ss, sp};

        // Coefficients: physical (double) -> effective (scale ratios, 1/h) -> storage.
        std::vector<double> phys((size_t)ORC_NCOEF * N);
        double* pc[ORC_NCOEF];
        for (int j = 0; j < ORC_NCOEF; j++) pc[j] = phys.data() + (size_t)j * N;
        orc_build_coeffs(nx, ny, nz, cfg->dt, mod, pc);
        double ratio[ORC_NCOEF];
        for (int a = 0; a < 3; a++) {
            ratio[ORC_VW1X + a] = 1.0;
            ratio[ORC_VW2X + a] = sq / ss * hi;
            ratio[ORC_VW3X + a] = sq / sp * hi;
            ratio[ORC_VU1X + a] = sv / ss * hi;
            ratio[ORC_VU2X + a] = sv / sq;
        }
        ratio[ORC_P1] = sp / sv * hi;
        ratio[ORC_P2] = sp / sq * hi;
        ratio[ORC_S1] = ratio[ORC_S2] = ss / sv * hi;
        ratio[ORC_S3] = ss / sq * hi;
        ratio[ORC_SXYC] = ratio[ORC_SXZC] = ratio[ORC_SYZC] = ss / sv * hi;
        for (int a = 0; a < 3; a++) {
            vw1[a].resize(N);
            for (size_t c = 0; c < N; c++) vw1[a][c] = (W)pc[ORC_VW1X + a][c];
        }
        for (int j = ORC_VW2X; j < ORC_NCOEF; j++) {
            double mx = 0;
            for (size_t c = 0; c < N; c++) mx = std::fmax(mx, std::fabs(pc[j][c] * ratio[j]));
            int e = 0;
            if (Pr::pow2 && mx > 0) std::frexp(mx, &e);  // mx = m 2^e, m in [0.5,1)
            const double inv = std::ldexp(1.0, -e);
            kmul[j] = (C)std::ldexp(1.0, e);
            k16[j].resize(N);
            for (size_t c = 0; c < N; c++) k16[j][c] = Pr::stk(pc[j][c] * ratio[j] * inv);
        }
        phys.clear();
        phys.shrink_to_fit();

        // CPML profiles and slab memory.
        const int L = cfg->cpml_width;
        const int n3[3] = {nx, ny, nz};
        for (int a = 0; a < 3; a++) {
            const int n = n3[a];
            std::vector<double> d(n), d2(n), e(n), e2(n);
            orc_cpml_profile(n, L, cfg->h, cfg->dt, cfg->cpml_v0, cfg->cpml_r, d.data(), d2.data(), e.data(),
                             e2.data());
            pa[a].resize(n);
            pb[a].resize(n);
            pa2[a].resize(n);
            pb2[a].resize(n);
            for (int i = 0; i < n; i++) {
                pa[a][i] = (C)e[i];
                pb[a][i] = (C)(-cfg->dt * d[i] * 0.5);
                pa2[a][i] = (C)e2[i];
                pb2[a][i] = (C)(-cfg->dt * d2[i] * 0.5);
            }
            ax[a].n = n;
            ax[a].L = L;
            ax[a].W = L > 0 ? 2 * L + 1 : 0;
            const size_t slab = (a == 0) ? (size_t)nz * ny * ax[a].W
                                : (a == 1) ? (size_t)nz * ax[a].W * nx
                                           : (size_t)ax[a].W * ny * nx;
            for (int s = 0; s < 8; s++) {
                psi[a][s].assign(slab, (W)0);
                prv[a][s].assign(slab, (W)0);
            }
        }
        for (int q = 0; q < ORC_NFIELD; q++) f[q].assign(N, Pr::st((C)0));

        // Source.
        const size_t src = ((size_t)cfg->src_iz * ny + cfg->src_iy) * nx + cfg->src_ix;
        double force = 0;
        if (cfg->src_kind == ORC_SRC_FORCE_Z) {
            std::vector<double> c1(N);  // dt / rho_z at the source cell
            const int ii = cfg->src_ix, jj = cfg->src_iy, kk = cfg->src_iz;
            const double rz = 0.5 * ((double)mod[ORC_RHO][src] + (double)mod[ORC_RHO][src + sz]);
            (void)ii;
            (void)jj;
            (void)kk;
            if (!(rz > 0)) return -3;
            force = cfg->dt / rz * sv;
        }

        double t_start = wall_seconds();
        for (int it = 0; it < nt; it++) {
            if (it == cfg->time_from_step) t_start = wall_seconds();
            const double w = wavelet[it];
            if (cfg->src_kind == ORC_SRC_EXPLOSIVE) {
                for (int q = ORC_SXX; q <= ORC_SZZ; q++) f[q][src] = Pr::st(ld(q, src) + (C)(w * ss));
            } else if (cfg->src_kind == ORC_SRC_PRESSURE) {
                f[ORC_P][src] = Pr::st(ld(ORC_P, src) + (C)(w * sp));
            }
            step_v();
            if (cfg->src_kind == ORC_SRC_FORCE_Z) f[ORC_VZ][src] = Pr::st(ld(ORC_VZ, src) + (C)(w * force));
            step_t();
            for (int r = 0; r < nrec; r++) {
                const size_t o = ((size_t)rec_ijk[3 * r + 2] * ny + rec_ijk[3 * r + 1]) * nx + rec_ijk[3 * r];
                const int q = rec_comp[r];
                seis[(size_t)r * nt + it] = (double)ld(q, o) / fscale[q];
            }
        }
        g_step_seconds = wall_seconds() - t_start;
        if (fields_out) {
            for (int q = 0; q < ORC_NFIELD; q++)
                for (size_t c = 0; c < N; c++) fields_out[(size_t)q * N + c] = (double)ld(q, c) / fscale[q];
        }
        return 0;
    }
};

template <int P>
int run_p(const orc_cfg* cfg, const float* const mod[ORC_NMOD], const float* w, int nt, int nrec, const int* ri,
          const int* rc, double* seis, double* fo) {
    switch (cfg->radius) {
        case 1: { Runner<P, 1> r; return r.run(cfg, mod, w, nt, nrec, ri, rc, seis, fo); }
        case 2: { Runner<P, 2> r; return r.run(cfg, mod, w, nt, nrec, ri, rc, seis, fo); }
        case 3: { Runner<P, 3> r; return r.run(cfg, mod, w, nt, nrec, ri, rc, seis, fo); }
        case 4: { Runner<P, 4> r; return r.run(cfg, mod, w, nt, nrec, ri, rc, seis, fo); }
    }
    return -1;
}

}  // namespace

extern "C" double orc_last_step_seconds(void) { return g_step_seconds; }

extern "C" int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

extern "C" int orc_run(const orc_cfg* cfg, const float* const mod[ORC_NMOD], const float* wavelet, int nt,
                       int nrec, const int* rec_ijk, const int* rec_comp, double* seis, double* fields_out) {
    if (!cfg || cfg->radius < 1 || cfg->radius > 4) return -1;
    const int R = cfg->radius, L = cfg->cpml_width;
    const int n3[3] = {cfg->nx, cfg->ny, cfg->nz};
    for (int a = 0; a < 3; a++)
        if (n3[a] < 2 * R + 1 || (L > 0 && n3[a] < 2 * L + 2)) return -2;
    const int si[3] = {cfg->src_ix, cfg->src_iy, cfg->src_iz};
    for (int a = 0; a < 3; a++)
        if (si[a] < R || si[a] >= n3[a] - R) return -2;
    for (int r = 0; r < nrec; r++) {
        for (int a = 0; a < 3; a++)
            if (rec_ijk[3 * r + a] < 0 || rec_ijk[3 * r + a] >= n3[a]) return -2;
        if (rec_comp[r] < 0 || rec_comp[r] >= ORC_NFIELD) return -2;
    }
    set_threads(cfg->nthreads);
    switch (cfg->precision) {
        case ORC_F64: return run_p<ORC_F64>(cfg, mod, wavelet, nt, nrec, rec_ijk, rec_comp, seis, fields_out);
        case ORC_F32: return run_p<ORC_F32>(cfg, mod, wavelet, nt, nrec, rec_ijk, rec_comp, seis, fields_out);
        case ORC_F16: return run_p<ORC_F16>(cfg, mod, wavelet, nt, nrec, rec_ijk, rec_comp, seis, fields_out);
        case ORC_BF16: return run_p<ORC_BF16>(cfg, mod, wavelet, nt, nrec, rec_ijk, rec_comp, seis, fields_out);
    }
    return -1;
}

// ----------------------------------------------------------------------------------------
// Reference-arithmetic mode.  Every array is binary16; expressions follow the C++ promotion
// rules of kernel.cu: the double literals d_Cpmll (100.0), d_Cvwp*/d_Cvup* (1.0), d_Cpp*/d_Csp*
// (0.01) and 0.5 make the CPML, Darcy, velocity and stress expressions double, while the
// differences times the float literal H = 100 stay float.  Stores round double -> half directly.
uint16_t orc_f2h(float x) {
    _Float16 h = (_Float16)x;
    uint16_t u;
    std::memcpy(&u, &h, 2);
    return u;
}
float orc_h2f(uint16_t u) {
    _Float16 h;
    std::memcpy(&h, &u, 2);
    return (float)h;
}

namespace {
struct H16 {
    _Float16 v;
};
static inline float hf(uint16_t u) { return orc_h2f(u); }
static inline uint16_t hd(double d) {
    _Float16 h = (_Float16)d;  // single rounding double -> binary16
    uint16_t u;
    std::memcpy(&u, &h, 2);
    return u;
}
static inline uint16_t hs(float f) { return orc_f2h(f); }

// psi = psi*e*100 + (-dt*d*100*0.5)*(e*100*prev + D); prev = D; returns D + (float)psi.
static inline float ref_pml(uint16_t& psi, uint16_t& prv, float D, uint16_t e, uint16_t d, float dt) {
    const double t1 = (double)(hf(psi) * hf(e)) * 100.0;
    const double t2 = (double)(-dt * hf(d)) * 100.0 * 0.5;
    const double t3 = (double)hf(e) * 100.0 * (double)hf(prv) + (double)D;
    psi = hd(t1 + t2 * t3);
    prv = hs(D);
    return D + hf(psi);
}

static const char* kAuxNames[48] = {
    // V: psi (pml*) then previous derivatives (S*)
    "pmlxSxx", "pmlySxy", "pmlzSxz", "pmlxSxy", "pmlySyy", "pmlzSyz", "pmlxSxz", "pmlySyz", "pmlzSzz",
    "pmlxss", "pmlyss", "pmlzss",
    "SXxx", "SXxy", "SXxz", "SYxy", "SYyy", "SYyz", "SZxz", "SZyz", "SZzz", "SXss", "SYss", "SZss",
    // T
    "pmlxVux", "pmlyVuy", "pmlzVuz", "pmlxVuy", "pmlyVux", "pmlyVuz", "pmlzVuy", "pmlzVux", "pmlxVuz",
    "pmlxVwx", "pmlyVwy", "pmlzVwz",
    "Vuxx", "Vuxy", "Vuxz", "Vuyx", "Vuyy", "Vuyz", "Vuzx", "Vuzy", "Vuzz", "Vwxx", "Vwyy", "Vwzz"};
}  // namespace

extern "C" const char* orc_ref_aux_name(int i) { return (i >= 0 && i < 48) ? kAuxNames[i] : ""; }

extern "C" int orc_ref_run(int nx, int ny, int nz, float dt, int nt, int sn, const float* wavelet,
                           uint16_t* const st[16], const uint16_t* const cf[ORC_NCOEF], const uint16_t* const pr[12],
                           uint16_t* const ax[48], int nrec, const int* rec_lin, const int* rec_comp, float* seis,
                           int nthreads) {
    if (nx < 3 || ny < 3 || nz < 3) return -2;
    set_threads(nthreads);
    const size_t sy = nx, sz = (size_t)nx * ny;
    const float H = 100;  // kernel.cu: the 1/h literal of every FD kernel
    uint16_t *vux = st[0], *vuy = st[1], *vuz = st[2], *vwx = st[3], *vwy = st[4], *vwz = st[5];
    uint16_t *txx = st[6], *tyy = st[7], *tzz = st[8], *txy = st[9], *txz = st[10], *tyz = st[11], *ss = st[12];
    uint16_t *vwx2 = st[13], *vwy2 = st[14], *vwz2 = st[15];
    const uint16_t *dxi = pr[0], *dxi2 = pr[1], *e_dxi = pr[2], *e_dxi2 = pr[3];
    const uint16_t *dyj = pr[4], *dyj2 = pr[5], *e_dyj = pr[6], *e_dyj2 = pr[7];
    const uint16_t *dzk = pr[8], *dzk2 = pr[9], *e_dzk = pr[10], *e_dzk2 = pr[11];
    for (int it = 0; it < nt; it++) {
        // Source (kernel.cu:130-142)
        const float I = wavelet[it];
        txx[sn] = hs(hf(txx[sn]) + I);
        tyy[sn] = hs(hf(tyy[sn]) + I);
        tzz[sn] = hs(hf(tzz[sn]) + I);
        // V update on cells 1..n-2 (kernel.cu:145-229 arithmetic)
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 1; k < nz - 1; k++)
            for (int j = 1; j < ny - 1; j++)
                for (int i = 1; i < nx - 1; i++) {
                    const size_t c = k * sz + j * sy + i;
                    const size_t r = c + 1, l = c - 1, q = c + sy, h = c - sy, u = c + sz, b = c - sz;
                    float x1 = (hf(txx[r]) - hf(txx[c])) * H, x2 = (hf(txy[c]) - hf(txy[h])) * H;
                    float x3 = (hf(txz[c]) - hf(txz[b])) * H, s1 = (hf(ss[r]) - hf(ss[c])) * H;
                    float y1 = (hf(tyy[q]) - hf(tyy[c])) * H, y2 = (hf(txy[c]) - hf(txy[l])) * H;
                    float y3 = (hf(tyz[c]) - hf(tyz[b])) * H, s2 = (hf(ss[q]) - hf(ss[c])) * H;
                    float z1 = (hf(tzz[u]) - hf(tzz[c])) * H, z2 = (hf(txz[c]) - hf(txz[l])) * H;
                    float z3 = (hf(tyz[c]) - hf(tyz[h])) * H, s3 = (hf(ss[u]) - hf(ss[c])) * H;
                    x1 = ref_pml(ax[0][c], ax[12][c], x1, e_dxi2[c], dxi2[c], dt);
                    x2 = ref_pml(ax[1][c], ax[13][c], x2, e_dyj[c], dyj[c], dt);
                    x3 = ref_pml(ax[2][c], ax[14][c], x3, e_dzk[c], dzk[c], dt);
                    s1 = ref_pml(ax[9][c], ax[21][c], s1, e_dxi2[c], dxi2[c], dt);
                    y2 = ref_pml(ax[3][c], ax[15][c], y2, e_dxi[c], dxi[c], dt);
                    y1 = ref_pml(ax[4][c], ax[16][c], y1, e_dyj2[c], dyj2[c], dt);
                    y3 = ref_pml(ax[5][c], ax[17][c], y3, e_dzk[c], dzk[c], dt);
                    s2 = ref_pml(ax[10][c], ax[22][c], s2, e_dyj2[c], dyj2[c], dt);
                    z2 = ref_pml(ax[6][c], ax[18][c], z2, e_dxi[c], dxi[c], dt);
                    z3 = ref_pml(ax[7][c], ax[19][c], z3, e_dyj[c], dyj[c], dt);
                    z1 = ref_pml(ax[8][c], ax[20][c], z1, e_dzk2[c], dzk2[c], dt);
                    s3 = ref_pml(ax[11][c], ax[23][c], s3, e_dzk2[c], dzk2[c], dt);
                    const float sx = x1 + x2 + x3, sy_ = y1 + y2 + y3, szv = z1 + z2 + z3;
                    // Darcy (kernel.cu:218-220); vz uses VW3y like the reference.
                    vwx[c] = hd(1.0 * hf(cf[ORC_VW1X][c]) * hf(vwx[c]) - 1.0 * hf(cf[ORC_VW2X][c]) * sx -
                                1.0 * hf(cf[ORC_VW3X][c]) * s1);
                    vwy[c] = hd(1.0 * hf(cf[ORC_VW1Y][c]) * hf(vwy[c]) - 1.0 * hf(cf[ORC_VW2Y][c]) * sy_ -
                                1.0 * hf(cf[ORC_VW3Y][c]) * s2);
                    vwz[c] = hd(1.0 * hf(cf[ORC_VW1Z][c]) * hf(vwz[c]) - 1.0 * hf(cf[ORC_VW2Z][c]) * szv -
                                1.0 * hf(cf[ORC_VW3Y][c]) * s3);
                    // Solid (kernel.cu:223-225)
                    vux[c] = hd(hf(vux[c]) + 1.0 * hf(cf[ORC_VU1X][c]) * sx -
                                1.0 * hf(cf[ORC_VU2X][c]) * (hf(vwx[c]) - hf(vwx2[c])));
                    vuy[c] = hd(hf(vuy[c]) + 1.0 * hf(cf[ORC_VU1Y][c]) * sy_ -
                                1.0 * hf(cf[ORC_VU2Y][c]) * (hf(vwy[c]) - hf(vwy2[c])));
                    vuz[c] = hd(hf(vuz[c]) + 1.0 * hf(cf[ORC_VU1Z][c]) * szv -
                                1.0 * hf(cf[ORC_VU2Z][c]) * (hf(vwz[c]) - hf(vwz2[c])));
                    vwx2[c] = vwx[c];
                    vwy2[c] = vwy[c];
                    vwz2[c] = vwz[c];
                }
        // T update (kernel.cu:405-493 arithmetic)
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 1; k < nz - 1; k++)
            for (int j = 1; j < ny - 1; j++)
                for (int i = 1; i < nx - 1; i++) {
                    const size_t c = k * sz + j * sy + i;
                    const size_t r = c + 1, l = c - 1, q = c + sy, h = c - sy, u = c + sz, b = c - sz;
                    float uxx = (hf(vux[c]) - hf(vux[l])) * H, uyy = (hf(vuy[c]) - hf(vuy[h])) * H;
                    float uzz = (hf(vuz[c]) - hf(vuz[b])) * H;
                    float wx = (hf(vwx[c]) - hf(vwx[l])) * H, wy = (hf(vwy[c]) - hf(vwy[h])) * H;
                    float wz = (hf(vwz[c]) - hf(vwz[b])) * H;
                    float uxy = (hf(vux[q]) - hf(vux[c])) * H, uyx = (hf(vuy[r]) - hf(vuy[c])) * H;
                    float uxz = (hf(vux[u]) - hf(vux[c])) * H, uzx = (hf(vuz[r]) - hf(vuz[c])) * H;
                    float uyz = (hf(vuy[u]) - hf(vuy[c])) * H, uzy = (hf(vuz[q]) - hf(vuz[c])) * H;
                    uxx = ref_pml(ax[24][c], ax[36][c], uxx, e_dxi[c], dxi[c], dt);
                    uyy = ref_pml(ax[25][c], ax[40][c], uyy, e_dyj[c], dyj[c], dt);
                    uzz = ref_pml(ax[26][c], ax[44][c], uzz, e_dzk[c], dzk[c], dt);
                    wx = ref_pml(ax[33][c], ax[45][c], wx, e_dxi[c], dxi[c], dt);
                    wy = ref_pml(ax[34][c], ax[46][c], wy, e_dyj[c], dyj[c], dt);
                    wz = ref_pml(ax[35][c], ax[47][c], wz, e_dzk[c], dzk[c], dt);
                    uxy = ref_pml(ax[27][c], ax[37][c], uxy, e_dyj2[c], dyj2[c], dt);
                    uyx = ref_pml(ax[28][c], ax[39][c], uyx, e_dxi2[c], dxi2[c], dt);
                    uxz = ref_pml(ax[32][c], ax[38][c], uxz, e_dzk2[c], dzk2[c], dt);
                    uzx = ref_pml(ax[31][c], ax[42][c], uzx, e_dxi2[c], dxi2[c], dt);
                    uyz = ref_pml(ax[29][c], ax[41][c], uyz, e_dzk2[c], dzk2[c], dt);
                    uzy = ref_pml(ax[30][c], ax[43][c], uzy, e_dyj2[c], dyj2[c], dt);
                    const float du = uxx + uyy + uzz, dw = wx + wy + wz;
                    ss[c] = hd(hf(ss[c]) - 0.01 * hf(cf[ORC_P1][c]) * du - 0.01 * hf(cf[ORC_P2][c]) * dw);
                    txx[c] = hd(hf(txx[c]) + 0.01 * hf(cf[ORC_S1][c]) * (uyy + uzz) + 0.01 * hf(cf[ORC_S2][c]) * uxx +
                                0.01 * hf(cf[ORC_S3][c]) * dw);
                    tyy[c] = hd(hf(tyy[c]) + 0.01 * hf(cf[ORC_S1][c]) * (uxx + uzz) + 0.01 * hf(cf[ORC_S2][c]) * uyy +
                                0.01 * hf(cf[ORC_S3][c]) * dw);
                    tzz[c] = hd(hf(tzz[c]) + 0.01 * hf(cf[ORC_S1][c]) * (uxx + uyy) + 0.01 * hf(cf[ORC_S2][c]) * uzz +
                                0.01 * hf(cf[ORC_S3][c]) * dw);
                    txy[c] = hd(hf(txy[c]) + 0.01 * hf(cf[ORC_SXYC][c]) * (uxy + uyx));
                    tyz[c] = hd(hf(tyz[c]) + 0.01 * hf(cf[ORC_SYZC][c]) * (uyz + uzy));
                    txz[c] = hd(hf(txz[c]) + 0.01 * hf(cf[ORC_SXZC][c]) * (uxz + uzx));
                }
        for (int r = 0; r < nrec; r++) seis[(size_t)r * nt + it] = hf(st[rec_comp[r]][rec_lin[r]]);
    }
    return 0;
}

// Reference inputs (main.cpp:322-494 coefficients, 519-1371 CPML, 1482-1526 half conversion),
// single domain with all six faces absorbing.  Float arithmetic as in main.cpp.
extern "C" void orc_ref_inputs(int nx, int ny, int nz, float H, float DT, int NP, float v0, float RC,
                               const float* const mod[ORC_NMOD], uint16_t* const coef[ORC_NCOEF],
                               uint16_t* const prof[12]) {
    const size_t sy = nx, sz = (size_t)nx * ny, N = sz * nz;
    const float Cv = 1.0 * std::pow(10.0, 8), Cp = 1;
    const float Cvwp1 = 1.0, Cvwp2 = 1.0, Cvwp3 = 1.0, Cvup1 = 1.0, Cvup2 = 1.0;
    const float Cpp1 = 100, Cpp2 = 100, Csp1 = 100, Csp2 = 100, Csp3 = 100, Csp4 = 100, Cpml = 0.01;
    std::vector<float> cf((size_t)ORC_NCOEF * N, 0.0f);
    auto C = [&](int j, size_t c) -> float& { return cf[(size_t)j * N + c]; };
    for (int k = 1; k < nz - 1; k++)
        for (int j = 1; j < ny - 1; j++)
            for (int i = 1; i < nx - 1; i++) {
                const size_t c = k * sz + j * sy + i;
                const float* mu = mod[ORC_MU];
                auto harm = [&](size_t a, size_t b, size_t d, size_t e) -> float {
                    if (mu[a] == 0 || mu[b] == 0 || mu[d] == 0 || mu[e] == 0) return 0.0f;
                    return (float)(1 / (0.25 * (1 / mu[a] + 1 / mu[b] + 1 / mu[d] + 1 / mu[e])));
                };
                const float muxz = harm(c, c + 1, c + sz, c + sz + 1);
                const float muyz = harm(c, c + sy, c + sz, c + sz + sy);
                const float muxy = harm(c, c + 1, c + sy, c + sy + 1);
                const size_t nb[3] = {c + 1, c + sy, c + sz};
                float rf[3], rh[3], c1[3], c2[3];
                for (int a = 0; a < 3; a++) {
                    rf[a] = (float)(0.5 * (mod[ORC_RHOF][c] + mod[ORC_RHOF][nb[a]]));
                    rh[a] = (float)(0.5 * (mod[ORC_RHO][c] + mod[ORC_RHO][nb[a]]));
                    c1[a] = (float)(0.5 * (mod[ORC_C1][c] + mod[ORC_C1][nb[a]]));
                    c2[a] = (float)(0.5 * (mod[ORC_C2][c] + mod[ORC_C2][nb[a]]));
                }
                if (!(c1[0] == 0 || c1[1] == 0 || c1[2] == 0)) {
                    for (int a = 0; a < 3; a++) {
                        C(ORC_VW1X + a, c) = (float)(Cvwp1 * (c2[a] - (rf[a] * rf[a] / rh[a]) - 0.5 * DT * c1[a]) /
                                                     (c2[a] - (rf[a] * rf[a] / rh[a]) + 0.5 * DT * c1[a]));
                        C(ORC_VW2X + a, c) = (float)(Cv * DT * Cvwp2 * (rf[a] / rh[a]) /
                                                     (Cp * (c2[a] - (rf[a] * rf[a] / rh[a]) + 0.5 * DT * c1[a])));
                        C(ORC_VW3X + a, c) =
                            (float)(Cv * DT * Cvwp3 / (Cp * (c2[a] - rf[a] * rf[a] / rh[a] + 0.5 * DT * c1[a])));
                    }
                }
                if (!(rh[0] == 0 || rh[1] == 0 || rh[2] == 0)) {
                    for (int a = 0; a < 3; a++) {
                        C(ORC_VU1X + a, c) = Cv * DT * Cvup1 / (rh[a] * Cp);
                        C(ORC_VU2X + a, c) = rf[a] * Cvup2 / (rh[a]);
                    }
                }
                C(ORC_P1, c) = mod[ORC_C][c] * DT * Cp * Cpp1 / Cv;
                C(ORC_P2, c) = mod[ORC_M][c] * DT * Cp * Cpp2 / Cv;
                C(ORC_S1, c) = Cp * DT * mod[ORC_H2U][c] * Csp1 / Cv;
                C(ORC_S2, c) = Cp * DT * mod[ORC_HH][c] * Csp2 / Cv;
                C(ORC_S3, c) = Cp * DT * mod[ORC_C][c] * Csp3 / Cv;
                C(ORC_SXYC, c) = Cp * DT * muxy * Csp4 / Cv;
                C(ORC_SXZC, c) = Cp * DT * muxz * Csp4 / Cv;
                C(ORC_SYZC, c) = Cp * DT * muyz * Csp4 / Cv;
            }
    for (int j = 0; j < ORC_NCOEF; j++)
        for (size_t c = 0; c < N; c++) coef[j][c] = orc_f2h(C(j, c));

    // CPML profiles: every face absorbing.  Float positions/compares as main.cpp:537-563.
    const float DP = NP * H;
    const float xol = DP, xor_ = (nx - 1) * H - DP, yol = DP, yor = (ny - 1) * H - DP;
    const float zol = DP, zor = (nz - 1) * H - DP;
    const float d0 = (float)(3.0 * v0 * std::log(1.0 / RC) / (2.0 * DP));
    std::vector<float> p12((size_t)12 * N, 0.0f);
    auto Pf = [&](int j, size_t c) -> float& { return p12[(size_t)j * N + c]; };
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const size_t c = k * sz + j * sy + i;
                const float x = i * H, y = j * H, z = k * H;
                auto setp = [&](int base, float dv, float dv2) {
                    Pf(base + 0, c) = dv;
                    Pf(base + 1, c) = dv2;
                    Pf(base + 2, c) = std::exp(-(dv)*DT);
                    Pf(base + 3, c) = std::exp(-(dv2)*DT);
                };
                if (x >= 0 && x < xol)
                    setp(0, (float)(d0 * std::pow(((xol - x) / DP), 2)), (float)(d0 * std::pow(((xol - x - 0.5 * H) / DP), 2)));
                if (x >= xor_ && x < nx * H)
                    setp(0, (float)(d0 * std::pow(((x - xor_) / DP), 2)), (float)(d0 * std::pow(((x + 0.5 * H - xor_) / DP), 2)));
                if (y >= 0 && y < yol)
                    setp(4, (float)(d0 * std::pow(((yol - y) / DP), 2)), (float)(d0 * std::pow(((yol - y - 0.5 * H) / DP), 2)));
                if (y >= yor && y < ny * H)
                    setp(4, (float)(d0 * std::pow(((y - yor) / DP), 2)), (float)(d0 * std::pow(((y + 0.5 * H - yor) / DP), 2)));
                if (z >= 0 && z < zol)
                    setp(8, (float)(d0 * std::pow(((zol - z) / DP), 2)), (float)(d0 * std::pow(((zol - z - 0.5 * H) / DP), 2)));
                if (z >= zor && z < nz * H)
                    setp(8, (float)(d0 * std::pow(((z - zor) / DP), 2)), (float)(d0 * std::pow(((z + 0.5 * H - zor) / DP), 2)));
            }
    for (int j = 0; j < 12; j++)
        for (size_t c = 0; c < N; c++) prof[j][c] = orc_f2h(Pf(j, c) * Cpml);
}
