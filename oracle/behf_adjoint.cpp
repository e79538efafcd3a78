// behf_adjoint.cpp -- CPU FP64 discrete adjoint of the BEHF time stepper.
//
// TEST INFRASTRUCTURE ONLY: the checker of the CUDA adjoint.  Nothing in the product library links,
// loads or calls this file.  The reference has no adjoint; what is restated here is the transpose of
// the forward scheme of behf_oracle.cpp (orc_run in FP64), which restates kernel.cu:145-229 (V),
// kernel.cu:405-493 (T), kernel.cu:130-142 (source) and the coefficient build of main.cpp:322-494.
//
// Forward step n (physical units, all storage scales 1):
//   explosive / pressure source -> V -> vertical-force source -> T -> record.
// The forward is linear in the state (fields + CPML memory), so the adjoint state runs backwards:
//   record^T (adjoint source) -> T^T -> force^T -> V^T -> source^T,
// and the gradient with respect to each effective coefficient is the sum over steps of the adjoint
// of the field it multiplies times the forward factor it multiplies (the forward states come from
// sqrt(N)-style checkpoints: the segment is recomputed and its post-V states kept).
//
// orc_adjoint_ex can also round the 13 adjoint fields to binary16 times per-field scales between steps (an
// FP16-stored adjoint state) and report their peak magnitudes: the measure of what such storage would cost.
//
// Gradient domain: coefficients of cells outside every CPML slab and inside the updated region are
// differentiated; moduli gradients are exact for cells whose coefficient cells (c - {0,1}^3) all lie
// in that domain, and set to zero elsewhere (the absorbing layers are not inverted).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "behf_oracle.h"

namespace {

const double kW[4][4] = {
    {1.0, 0, 0, 0},
    {9.0 / 8.0, -1.0 / 24.0, 0, 0},
    {75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0, 0},
    {1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0},
};

inline int slab_of(int i, int n, int L) {
    if (L <= 0) return -1;
    if (i < L) return i;
    if (i >= n - 1 - L) return L + (i - (n - 1 - L));
    return -1;
}

struct Adj {
    int nx, ny, nz, R, L, W, bug;
    size_t sy, sz, N;
    double dt;
    double cw[4];
    std::vector<double> k[ORC_NCOEF];            // effective coefficients (physical x 1/h factors)
    double ratio[ORC_NCOEF];
    std::vector<double> pa[3], pb[3], pa2[3], pb2[3];
    size_t slab_n[3];

    // forward state
    std::vector<double> f[ORC_NFIELD];
    std::vector<double> psi[3][8], prv[3][8];
    // adjoint state
    std::vector<double> lf[ORC_NFIELD];
    std::vector<double> lpsi[3][8], lprv[3][8];
    std::vector<double> tmp[7];
    std::vector<double> g[ORC_NCOEF];

    int n3(int a) const { return a == 0 ? nx : a == 1 ? ny : nz; }
    size_t slab_off(int a, int i, int j, int kk, int s) const {
        if (a == 0) return ((size_t)kk * ny + j) * W + s;
        if (a == 1) return ((size_t)kk * W + s) * nx + i;
        return ((size_t)s * ny + j) * nx + i;
    }
    bool updated(int i, int j, int kk) const {
        return i >= R && i < nx - R && j >= R && j < ny - R && kk >= R && kk < nz - R;
    }
    bool interior(int i, int j, int kk) const {  // updated and outside every slab
        return updated(i, j, kk) && slab_of(i, nx, L) < 0 && slab_of(j, ny, L) < 0 && slab_of(kk, nz, L) < 0;
    }

    static double fwdv(const std::vector<double>& v, size_t o, size_t s, const double* w, int R) {
        double acc = w[0] * (v[o + s] - v[o]);
        for (int m = 2; m <= R; m++) acc += w[m - 1] * (v[o + m * s] - v[o - (m - 1) * s]);
        return acc;
    }
    static double bwdv(const std::vector<double>& v, size_t o, size_t s, const double* w, int R) {
        double acc = w[0] * (v[o] - v[o - s]);
        for (int m = 2; m <= R; m++) acc += w[m - 1] * (v[o + (m - 1) * s] - v[o - m * s]);
        return acc;
    }
    double fwd(const std::vector<double>& v, size_t o, size_t s) const { return fwdv(v, o, s, cw, R); }
    double bwd(const std::vector<double>& v, size_t o, size_t s) const { return bwdv(v, o, s, cw, R); }

    // ------------------------------------------------------------------ forward (orc_run FP64 order)
    double pml(double D, int a, int slot, bool half, int idx, size_t so) {
        const double A = half ? pa2[a][idx] : pa[a][idx];
        const double B = half ? pb2[a][idx] : pb[a][idx];
        double& ps = psi[a][slot][so];
        double& pv = prv[a][slot][so];
        const double pn = A * ps + B * (A * pv + D);
        ps = pn;
        pv = D;
        return D + ps;
    }

    void step_v() {
#pragma omp parallel for collapse(2) schedule(static)
        for (int kk = R; kk < nz - R; kk++)
            for (int j = R; j < ny - R; j++)
                for (int i = R; i < nx - R; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    const int si = slab_of(i, nx, L), sj = slab_of(j, ny, L), sk = slab_of(kk, nz, L);
                    double x1 = fwd(f[ORC_SXX], c, 1), x2 = bwd(f[ORC_SXY], c, sy), x3 = bwd(f[ORC_SXZ], c, sz);
                    double s1 = fwd(f[ORC_P], c, 1);
                    double y1 = fwd(f[ORC_SYY], c, sy), y2 = bwd(f[ORC_SXY], c, 1), y3 = bwd(f[ORC_SYZ], c, sz);
                    double s2 = fwd(f[ORC_P], c, sy);
                    double z1 = fwd(f[ORC_SZZ], c, sz), z2 = bwd(f[ORC_SXZ], c, 1), z3 = bwd(f[ORC_SYZ], c, sy);
                    double s3 = fwd(f[ORC_P], c, sz);
                    if (si >= 0) {
                        const size_t so = slab_off(0, i, j, kk, si);
                        x1 = pml(x1, 0, 0, true, i, so);
                        s1 = pml(s1, 0, 1, true, i, so);
                        y2 = pml(y2, 0, 2, false, i, so);
                        z2 = pml(z2, 0, 3, false, i, so);
                    }
                    if (sj >= 0) {
                        const size_t so = slab_off(1, i, j, kk, sj);
                        y1 = pml(y1, 1, 0, true, j, so);
                        s2 = pml(s2, 1, 1, true, j, so);
                        x2 = pml(x2, 1, 2, false, j, so);
                        z3 = pml(z3, 1, 3, false, j, so);
                    }
                    if (sk >= 0) {
                        const size_t so = slab_off(2, i, j, kk, sk);
                        z1 = pml(z1, 2, 0, true, kk, so);
                        s3 = pml(s3, 2, 1, true, kk, so);
                        x3 = pml(x3, 2, 2, false, kk, so);
                        y3 = pml(y3, 2, 3, false, kk, so);
                    }
                    const double sum[3] = {x1 + x2 + x3, y1 + y2 + y3, z1 + z2 + z3};
                    const double dp[3] = {s1, s2, s3};
                    for (int a = 0; a < 3; a++) {
                        const int vw3 = (a == 2 && bug) ? ORC_VW3Y : ORC_VW3X + a;
                        const double qo = f[ORC_QX + a][c];
                        const double qn = k[ORC_VW1X + a][c] * qo - k[ORC_VW2X + a][c] * sum[a] - k[vw3][c] * dp[a];
                        f[ORC_QX + a][c] = qn;
                        const double dq = qn - qo;
                        f[ORC_VX + a][c] = f[ORC_VX + a][c] + k[ORC_VU1X + a][c] * sum[a] - k[ORC_VU2X + a][c] * dq;
                    }
                }
    }

    void step_t() {
#pragma omp parallel for collapse(2) schedule(static)
        for (int kk = R; kk < nz - R; kk++)
            for (int j = R; j < ny - R; j++)
                for (int i = R; i < nx - R; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    const int si = slab_of(i, nx, L), sj = slab_of(j, ny, L), sk = slab_of(kk, nz, L);
                    double uxx = bwd(f[ORC_VX], c, 1), uyy = bwd(f[ORC_VY], c, sy), uzz = bwd(f[ORC_VZ], c, sz);
                    double wx = bwd(f[ORC_QX], c, 1), wy = bwd(f[ORC_QY], c, sy), wz = bwd(f[ORC_QZ], c, sz);
                    double uxy = fwd(f[ORC_VX], c, sy), uyx = fwd(f[ORC_VY], c, 1);
                    double uxz = fwd(f[ORC_VX], c, sz), uzx = fwd(f[ORC_VZ], c, 1);
                    double uyz = fwd(f[ORC_VY], c, sz), uzy = fwd(f[ORC_VZ], c, sy);
                    if (si >= 0) {
                        const size_t so = slab_off(0, i, j, kk, si);
                        uxx = pml(uxx, 0, 4, false, i, so);
                        wx = pml(wx, 0, 5, false, i, so);
                        uyx = pml(uyx, 0, 6, true, i, so);
                        uzx = pml(uzx, 0, 7, true, i, so);
                    }
                    if (sj >= 0) {
                        const size_t so = slab_off(1, i, j, kk, sj);
                        uyy = pml(uyy, 1, 4, false, j, so);
                        wy = pml(wy, 1, 5, false, j, so);
                        uxy = pml(uxy, 1, 6, true, j, so);
                        uzy = pml(uzy, 1, 7, true, j, so);
                    }
                    if (sk >= 0) {
                        const size_t so = slab_off(2, i, j, kk, sk);
                        uzz = pml(uzz, 2, 4, false, kk, so);
                        wz = pml(wz, 2, 5, false, kk, so);
                        uxz = pml(uxz, 2, 6, true, kk, so);
                        uyz = pml(uyz, 2, 7, true, kk, so);
                    }
                    const double dv = uxx + uyy + uzz, dq = wx + wy + wz;
                    const double g1 = k[ORC_S1][c], g2 = k[ORC_S2][c], g3 = k[ORC_S3][c];
                    f[ORC_P][c] = f[ORC_P][c] - k[ORC_P1][c] * dv - k[ORC_P2][c] * dq;
                    f[ORC_SXX][c] = f[ORC_SXX][c] + g1 * (uyy + uzz) + g2 * uxx + g3 * dq;
                    f[ORC_SYY][c] = f[ORC_SYY][c] + g1 * (uxx + uzz) + g2 * uyy + g3 * dq;
                    f[ORC_SZZ][c] = f[ORC_SZZ][c] + g1 * (uxx + uyy) + g2 * uzz + g3 * dq;
                    f[ORC_SXY][c] = f[ORC_SXY][c] + k[ORC_SXYC][c] * (uxy + uyx);
                    f[ORC_SYZ][c] = f[ORC_SYZ][c] + k[ORC_SYZC][c] * (uyz + uzy);
                    f[ORC_SXZ][c] = f[ORC_SXZ][c] + k[ORC_SXZC][c] * (uxz + uzx);
                }
    }

    // ------------------------------------------------------------------ adjoint pieces
    // lambda of the CPML-modified derivative -> lambda of the plain derivative, with the current adjoint
    // memory (adjoints of psi_new and prev_new):  lD = lDt + B (lpsi + lDt) + lprev.
    double lmod(double lDt, int a, int slot, bool half, int idx, size_t so) const {
        const double B = half ? pb2[a][idx] : pb[a][idx];
        return lDt + B * (lpsi[a][slot][so] + lDt) + lprv[a][slot][so];
    }
    // memory update after the gather: Lambda = lpsi + lDt; lpsi = A Lambda; lprev = A B Lambda.
    void lmem(double lDt, int a, int slot, bool half, int idx, size_t so) {
        const double A = half ? pa2[a][idx] : pa[a][idx];
        const double B = half ? pb2[a][idx] : pb[a][idx];
        const double Lm = lpsi[a][slot][so] + lDt;
        lpsi[a][slot][so] = A * Lm;
        lprv[a][slot][so] = A * B * Lm;
    }

    // T^T.  snap: fields after V (+force) of this step (v, q used by T).
    void adj_t(const std::vector<double>* snap) {
        // 1. per-cell adjoints of the 7 derivative groups + coefficient gradients
#pragma omp parallel for collapse(2) schedule(static)
        for (int kk = 0; kk < nz; kk++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    if (!updated(i, j, kk)) {
                        for (int t = 0; t < 7; t++) tmp[t][c] = 0;
                        continue;
                    }
                    const double lp = lf[ORC_P][c], lxx = lf[ORC_SXX][c], lyy = lf[ORC_SYY][c], lzz = lf[ORC_SZZ][c];
                    const double lxy = lf[ORC_SXY][c], lxz = lf[ORC_SXZ][c], lyz = lf[ORC_SYZ][c];
                    const double P1 = k[ORC_P1][c], P2 = k[ORC_P2][c], S1 = k[ORC_S1][c], S2 = k[ORC_S2][c], S3 = k[ORC_S3][c];
                    tmp[0][c] = -P1 * lp + S2 * lxx + S1 * (lyy + lzz);
                    tmp[1][c] = -P1 * lp + S2 * lyy + S1 * (lxx + lzz);
                    tmp[2][c] = -P1 * lp + S2 * lzz + S1 * (lxx + lyy);
                    tmp[3][c] = -P2 * lp + S3 * (lxx + lyy + lzz);
                    tmp[4][c] = k[ORC_SXYC][c] * lxy;
                    tmp[5][c] = k[ORC_SXZC][c] * lxz;
                    tmp[6][c] = k[ORC_SYZC][c] * lyz;
                    if (interior(i, j, kk)) {
                        const double uxx = bwd(snap[ORC_VX], c, 1), uyy = bwd(snap[ORC_VY], c, sy), uzz = bwd(snap[ORC_VZ], c, sz);
                        const double dq = bwd(snap[ORC_QX], c, 1) + bwd(snap[ORC_QY], c, sy) + bwd(snap[ORC_QZ], c, sz);
                        const double uxy = fwd(snap[ORC_VX], c, sy), uyx = fwd(snap[ORC_VY], c, 1);
                        const double uxz = fwd(snap[ORC_VX], c, sz), uzx = fwd(snap[ORC_VZ], c, 1);
                        const double uyz = fwd(snap[ORC_VY], c, sz), uzy = fwd(snap[ORC_VZ], c, sy);
                        g[ORC_P1][c] += -lp * (uxx + uyy + uzz);
                        g[ORC_P2][c] += -lp * dq;
                        g[ORC_S1][c] += lxx * (uyy + uzz) + lyy * (uxx + uzz) + lzz * (uxx + uyy);
                        g[ORC_S2][c] += lxx * uxx + lyy * uyy + lzz * uzz;
                        g[ORC_S3][c] += (lxx + lyy + lzz) * dq;
                        g[ORC_SXYC][c] += lxy * (uxy + uyx);
                        g[ORC_SXZC][c] += lxz * (uxz + uzx);
                        g[ORC_SYZC][c] += lyz * (uyz + uzy);
                    }
                }
        // 2. the 12 CPML-modified adjoint derivatives, stored per cell
        std::vector<double> L12[12];
        for (auto& v : L12) v.assign(N, 0.0);
        enum { UXX, UYY, UZZ, WX, WY, WZ, UYX, UXY, UZX, UXZ, UZY, UYZ };
#pragma omp parallel for collapse(2) schedule(static)
        for (int kk = R; kk < nz - R; kk++)
            for (int j = R; j < ny - R; j++)
                for (int i = R; i < nx - R; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    double v[12] = {tmp[0][c], tmp[1][c], tmp[2][c], tmp[3][c], tmp[3][c], tmp[3][c],
                                    tmp[4][c], tmp[4][c], tmp[5][c], tmp[5][c], tmp[6][c], tmp[6][c]};
                    const int si = slab_of(i, nx, L), sj = slab_of(j, ny, L), sk = slab_of(kk, nz, L);
                    if (si >= 0) {
                        const size_t so = slab_off(0, i, j, kk, si);
                        v[UXX] = lmod(tmp[0][c], 0, 4, false, i, so);
                        v[WX] = lmod(tmp[3][c], 0, 5, false, i, so);
                        v[UYX] = lmod(tmp[4][c], 0, 6, true, i, so);
                        v[UZX] = lmod(tmp[5][c], 0, 7, true, i, so);
                    }
                    if (sj >= 0) {
                        const size_t so = slab_off(1, i, j, kk, sj);
                        v[UYY] = lmod(tmp[1][c], 1, 4, false, j, so);
                        v[WY] = lmod(tmp[3][c], 1, 5, false, j, so);
                        v[UXY] = lmod(tmp[4][c], 1, 6, true, j, so);
                        v[UZY] = lmod(tmp[6][c], 1, 7, true, j, so);
                    }
                    if (sk >= 0) {
                        const size_t so = slab_off(2, i, j, kk, sk);
                        v[UZZ] = lmod(tmp[2][c], 2, 4, false, kk, so);
                        v[WZ] = lmod(tmp[3][c], 2, 5, false, kk, so);
                        v[UXZ] = lmod(tmp[5][c], 2, 6, true, kk, so);
                        v[UYZ] = lmod(tmp[6][c], 2, 7, true, kk, so);
                    }
                    for (int t = 0; t < 12; t++) L12[t][c] = v[t];
                }
        // 3. gather into the velocity and flux adjoints (updated cells only; ghost adjoints are unused)
#pragma omp parallel for collapse(2) schedule(static)
        for (int kk = R; kk < nz - R; kk++)
            for (int j = R; j < ny - R; j++)
                for (int i = R; i < nx - R; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    lf[ORC_VX][c] -= fwd(L12[UXX], c, 1) + bwd(L12[UXY], c, sy) + bwd(L12[UXZ], c, sz);
                    lf[ORC_VY][c] -= fwd(L12[UYY], c, sy) + bwd(L12[UYX], c, 1) + bwd(L12[UYZ], c, sz);
                    lf[ORC_VZ][c] -= fwd(L12[UZZ], c, sz) + bwd(L12[UZX], c, 1) + bwd(L12[UZY], c, sy);
                    lf[ORC_QX][c] -= fwd(L12[WX], c, 1);
                    lf[ORC_QY][c] -= fwd(L12[WY], c, sy);
                    lf[ORC_QZ][c] -= fwd(L12[WZ], c, sz);
                }
        // 4. adjoint CPML memory of the T slots
        for (int kk = R; kk < nz - R; kk++)
            for (int j = R; j < ny - R; j++)
                for (int i = R; i < nx - R; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    const int si = slab_of(i, nx, L), sj = slab_of(j, ny, L), sk = slab_of(kk, nz, L);
                    if (si >= 0) {
                        const size_t so = slab_off(0, i, j, kk, si);
                        lmem(tmp[0][c], 0, 4, false, i, so);
                        lmem(tmp[3][c], 0, 5, false, i, so);
                        lmem(tmp[4][c], 0, 6, true, i, so);
                        lmem(tmp[5][c], 0, 7, true, i, so);
                    }
                    if (sj >= 0) {
                        const size_t so = slab_off(1, i, j, kk, sj);
                        lmem(tmp[1][c], 1, 4, false, j, so);
                        lmem(tmp[3][c], 1, 5, false, j, so);
                        lmem(tmp[4][c], 1, 6, true, j, so);
                        lmem(tmp[6][c], 1, 7, true, j, so);
                    }
                    if (sk >= 0) {
                        const size_t so = slab_off(2, i, j, kk, sk);
                        lmem(tmp[2][c], 2, 4, false, kk, so);
                        lmem(tmp[3][c], 2, 5, false, kk, so);
                        lmem(tmp[5][c], 2, 6, true, kk, so);
                        lmem(tmp[6][c], 2, 7, true, kk, so);
                    }
                }
    }

    // V^T.  cur: fields after V of this step (sigma, p as V read them; q after V).  qprev: q before V.
    void adj_v(const std::vector<double>* cur, const std::vector<double>* qprev) {
#pragma omp parallel for collapse(2) schedule(static)
        for (int kk = 0; kk < nz; kk++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    if (!updated(i, j, kk)) {
                        for (int t = 0; t < 6; t++) tmp[t][c] = 0;
                        continue;
                    }
                    const bool in = interior(i, j, kk);
                    double sum[3] = {0, 0, 0}, dp[3] = {0, 0, 0};
                    if (in) {
                        sum[0] = fwd(cur[ORC_SXX], c, 1) + bwd(cur[ORC_SXY], c, sy) + bwd(cur[ORC_SXZ], c, sz);
                        sum[1] = fwd(cur[ORC_SYY], c, sy) + bwd(cur[ORC_SXY], c, 1) + bwd(cur[ORC_SYZ], c, sz);
                        sum[2] = fwd(cur[ORC_SZZ], c, sz) + bwd(cur[ORC_SXZ], c, 1) + bwd(cur[ORC_SYZ], c, sy);
                        dp[0] = fwd(cur[ORC_P], c, 1);
                        dp[1] = fwd(cur[ORC_P], c, sy);
                        dp[2] = fwd(cur[ORC_P], c, sz);
                    }
                    for (int a = 0; a < 3; a++) {
                        const int vw3 = (a == 2 && bug) ? ORC_VW3Y : ORC_VW3X + a;
                        const double lv = lf[ORC_VX + a][c], lq = lf[ORC_QX + a][c];
                        const double VU2 = k[ORC_VU2X + a][c];
                        const double mu = lq - VU2 * lv;
                        lf[ORC_QX + a][c] = k[ORC_VW1X + a][c] * mu + VU2 * lv;
                        tmp[a][c] = k[ORC_VU1X + a][c] * lv - k[ORC_VW2X + a][c] * mu;
                        tmp[3 + a][c] = -k[vw3][c] * mu;
                        if (in) {
                            const double qo = qprev[ORC_QX + a][c], qn = cur[ORC_QX + a][c];
                            g[ORC_VW1X + a][c] += mu * qo;
                            g[ORC_VW2X + a][c] += -mu * sum[a];
                            g[vw3][c] += -mu * dp[a];
                            g[ORC_VU1X + a][c] += lv * sum[a];
                            g[ORC_VU2X + a][c] += -lv * (qn - qo);
                        }
                    }
                }
        std::vector<double> L12[12];
        for (auto& v : L12) v.assign(N, 0.0);
        enum { X1, X2, X3, Y1, Y2, Y3, Z1, Z2, Z3, S1, S2, S3 };
#pragma omp parallel for collapse(2) schedule(static)
        for (int kk = R; kk < nz - R; kk++)
            for (int j = R; j < ny - R; j++)
                for (int i = R; i < nx - R; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    const double sx = tmp[0][c], syv = tmp[1][c], szv = tmp[2][c];
                    double v[12] = {sx, sx, sx, syv, syv, syv, szv, szv, szv, tmp[3][c], tmp[4][c], tmp[5][c]};
                    const int si = slab_of(i, nx, L), sj = slab_of(j, ny, L), sk = slab_of(kk, nz, L);
                    if (si >= 0) {
                        const size_t so = slab_off(0, i, j, kk, si);
                        v[X1] = lmod(sx, 0, 0, true, i, so);
                        v[S1] = lmod(tmp[3][c], 0, 1, true, i, so);
                        v[Y2] = lmod(syv, 0, 2, false, i, so);
                        v[Z2] = lmod(szv, 0, 3, false, i, so);
                    }
                    if (sj >= 0) {
                        const size_t so = slab_off(1, i, j, kk, sj);
                        v[Y1] = lmod(syv, 1, 0, true, j, so);
                        v[S2] = lmod(tmp[4][c], 1, 1, true, j, so);
                        v[X2] = lmod(sx, 1, 2, false, j, so);
                        v[Z3] = lmod(szv, 1, 3, false, j, so);
                    }
                    if (sk >= 0) {
                        const size_t so = slab_off(2, i, j, kk, sk);
                        v[Z1] = lmod(szv, 2, 0, true, kk, so);
                        v[S3] = lmod(tmp[5][c], 2, 1, true, kk, so);
                        v[X3] = lmod(sx, 2, 2, false, kk, so);
                        v[Y3] = lmod(syv, 2, 3, false, kk, so);
                    }
                    for (int t = 0; t < 12; t++) L12[t][c] = v[t];
                }
#pragma omp parallel for collapse(2) schedule(static)
        for (int kk = R; kk < nz - R; kk++)
            for (int j = R; j < ny - R; j++)
                for (int i = R; i < nx - R; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    lf[ORC_SXX][c] -= bwd(L12[X1], c, 1);
                    lf[ORC_SYY][c] -= bwd(L12[Y1], c, sy);
                    lf[ORC_SZZ][c] -= bwd(L12[Z1], c, sz);
                    lf[ORC_SXY][c] -= fwd(L12[X2], c, sy) + fwd(L12[Y2], c, 1);
                    lf[ORC_SXZ][c] -= fwd(L12[X3], c, sz) + fwd(L12[Z2], c, 1);
                    lf[ORC_SYZ][c] -= fwd(L12[Y3], c, sz) + fwd(L12[Z3], c, sy);
                    lf[ORC_P][c] -= bwd(L12[S1], c, 1) + bwd(L12[S2], c, sy) + bwd(L12[S3], c, sz);
                }
        for (int kk = R; kk < nz - R; kk++)
            for (int j = R; j < ny - R; j++)
                for (int i = R; i < nx - R; i++) {
                    const size_t c = kk * sz + j * sy + i;
                    const int si = slab_of(i, nx, L), sj = slab_of(j, ny, L), sk = slab_of(kk, nz, L);
                    if (si >= 0) {
                        const size_t so = slab_off(0, i, j, kk, si);
                        lmem(tmp[0][c], 0, 0, true, i, so);
                        lmem(tmp[3][c], 0, 1, true, i, so);
                        lmem(tmp[1][c], 0, 2, false, i, so);
                        lmem(tmp[2][c], 0, 3, false, i, so);
                    }
                    if (sj >= 0) {
                        const size_t so = slab_off(1, i, j, kk, sj);
                        lmem(tmp[1][c], 1, 0, true, j, so);
                        lmem(tmp[4][c], 1, 1, true, j, so);
                        lmem(tmp[0][c], 1, 2, false, j, so);
                        lmem(tmp[2][c], 1, 3, false, j, so);
                    }
                    if (sk >= 0) {
                        const size_t so = slab_off(2, i, j, kk, sk);
                        lmem(tmp[2][c], 2, 0, true, kk, so);
                        lmem(tmp[5][c], 2, 1, true, kk, so);
                        lmem(tmp[0][c], 2, 2, false, kk, so);
                        lmem(tmp[1][c], 2, 3, false, kk, so);
                    }
                }
    }
};

}  // namespace

extern "C" int orc_adjoint_ex(const orc_cfg* cfg, const float* const mod[ORC_NMOD], const float* wavelet, int nt,
                              int nrec, const int* rec_ijk, const int* rec_comp, const double* adj_src, int stride,
                              double* seis_out, double* grad_wavelet, double* grad_coef, double* grad_mod,
                              const double* lf_scale, double* lf_max, long long* lf_saturated) {
    if (!cfg || cfg->radius < 1 || cfg->radius > 4 || nt < 1) return -1;
    Adj A;
    A.nx = cfg->nx;
    A.ny = cfg->ny;
    A.nz = cfg->nz;
    A.R = cfg->radius;
    A.L = cfg->cpml_width;
    A.W = A.L > 0 ? 2 * A.L + 1 : 0;
    A.bug = cfg->ref_bug_compat;
    A.dt = cfg->dt;
    A.sy = A.nx;
    A.sz = (size_t)A.nx * A.ny;
    A.N = A.sz * A.nz;
    const size_t N = A.N, sz = A.sz;
    for (int m = 0; m < 4; m++) A.cw[m] = kW[A.R - 1][m];
    const int n3[3] = {A.nx, A.ny, A.nz};
    for (int a = 0; a < 3; a++)
        if (n3[a] < 2 * A.R + 1 || (A.L > 0 && n3[a] < 2 * A.L + 2)) return -2;
    const int src[3] = {cfg->src_ix, cfg->src_iy, cfg->src_iz};
    for (int a = 0; a < 3; a++)
        if (src[a] < A.R || src[a] >= n3[a] - A.R) return -2;
    for (int r = 0; r < nrec; r++)
        for (int a = 0; a < 3; a++)
            if (rec_ijk[3 * r + a] < 0 || rec_ijk[3 * r + a] >= n3[a] || rec_comp[r] < 0 || rec_comp[r] >= ORC_NFIELD)
                return -2;

    // effective coefficients: physical x 1/h where the term is a difference
    const double hi = 1.0 / cfg->h;
    {
        std::vector<double> phys((size_t)ORC_NCOEF * N);
        double* pc[ORC_NCOEF];
        for (int j = 0; j < ORC_NCOEF; j++) pc[j] = phys.data() + (size_t)j * N;
        orc_build_coeffs(A.nx, A.ny, A.nz, cfg->dt, mod, pc);
        for (int a = 0; a < 3; a++) {
            A.ratio[ORC_VW1X + a] = 1.0;
            A.ratio[ORC_VW2X + a] = hi;
            A.ratio[ORC_VW3X + a] = hi;
            A.ratio[ORC_VU1X + a] = hi;
            A.ratio[ORC_VU2X + a] = 1.0;
        }
        A.ratio[ORC_P1] = A.ratio[ORC_P2] = A.ratio[ORC_S1] = A.ratio[ORC_S2] = A.ratio[ORC_S3] = hi;
        A.ratio[ORC_SXYC] = A.ratio[ORC_SXZC] = A.ratio[ORC_SYZC] = hi;
        for (int j = 0; j < ORC_NCOEF; j++) {
            A.k[j].resize(N);
            for (size_t c = 0; c < N; c++) A.k[j][c] = pc[j][c] * A.ratio[j];
            A.g[j].assign(N, 0.0);
        }
    }
    for (int a = 0; a < 3; a++) {
        const int n = n3[a];
        std::vector<double> d(n), d2(n), e(n), e2(n);
        orc_cpml_profile(n, A.L, cfg->h, cfg->dt, cfg->cpml_v0, cfg->cpml_r, d.data(), d2.data(), e.data(), e2.data());
        A.pa[a].resize(n);
        A.pb[a].resize(n);
        A.pa2[a].resize(n);
        A.pb2[a].resize(n);
        for (int i = 0; i < n; i++) {
            A.pa[a][i] = e[i];
            A.pb[a][i] = -cfg->dt * d[i] * 0.5;
            A.pa2[a][i] = e2[i];
            A.pb2[a][i] = -cfg->dt * d2[i] * 0.5;
        }
        A.slab_n[a] = (a == 0) ? (size_t)A.nz * A.ny * A.W : (a == 1) ? (size_t)A.nz * A.W * A.nx : (size_t)A.W * A.ny * A.nx;
        for (int s = 0; s < 8; s++) {
            A.psi[a][s].assign(A.slab_n[a], 0.0);
            A.prv[a][s].assign(A.slab_n[a], 0.0);
            A.lpsi[a][s].assign(A.slab_n[a], 0.0);
            A.lprv[a][s].assign(A.slab_n[a], 0.0);
        }
    }
    for (int q = 0; q < ORC_NFIELD; q++) {
        A.f[q].assign(N, 0.0);
        A.lf[q].assign(N, 0.0);
    }
    for (int t = 0; t < 7; t++) A.tmp[t].assign(N, 0.0);

    const size_t so = ((size_t)cfg->src_iz * A.ny + cfg->src_iy) * A.nx + cfg->src_ix;
    double force = 0;
    if (cfg->src_kind == ORC_SRC_FORCE_Z) {
        const double rz = 0.5 * ((double)mod[ORC_RHO][so] + (double)mod[ORC_RHO][so + sz]);
        if (!(rz > 0)) return -3;
        force = cfg->dt / rz;
    }
    std::vector<size_t> roff(nrec);
    for (int r = 0; r < nrec; r++)
        roff[r] = ((size_t)rec_ijk[3 * r + 2] * A.ny + rec_ijk[3 * r + 1]) * A.nx + rec_ijk[3 * r];

    auto inject = [&](int it) {
        const double w = wavelet[it];
        if (cfg->src_kind == ORC_SRC_EXPLOSIVE) {
            for (int q = ORC_SXX; q <= ORC_SZZ; q++) A.f[q][so] = A.f[q][so] + w;
        } else if (cfg->src_kind == ORC_SRC_PRESSURE) {
            A.f[ORC_P][so] = A.f[ORC_P][so] + w;
        }
    };
    auto inject_force = [&](int it) {
        if (cfg->src_kind == ORC_SRC_FORCE_Z) A.f[ORC_VZ][so] = A.f[ORC_VZ][so] + wavelet[it] * force;
    };

    // forward with checkpoints (fields + CPML memory) every S steps
    const int S = stride > 0 ? stride : std::max(1, (int)std::lround(std::sqrt((double)nt)));
    const int nseg = (nt + S - 1) / S;
    struct Ck {
        std::vector<double> f[ORC_NFIELD];
        std::vector<double> psi[3][8], prv[3][8];
    };
    std::vector<Ck> ck(nseg);
    auto save = [&](Ck& c) {
        for (int q = 0; q < ORC_NFIELD; q++) c.f[q] = A.f[q];
        for (int a = 0; a < 3; a++)
            for (int s = 0; s < 8; s++) {
                c.psi[a][s] = A.psi[a][s];
                c.prv[a][s] = A.prv[a][s];
            }
    };
    auto load = [&](const Ck& c) {
        for (int q = 0; q < ORC_NFIELD; q++) A.f[q] = c.f[q];
        for (int a = 0; a < 3; a++)
            for (int s = 0; s < 8; s++) {
                A.psi[a][s] = c.psi[a][s];
                A.prv[a][s] = c.prv[a][s];
            }
    };
    for (int it = 0; it < nt; it++) {
        if (it % S == 0) save(ck[it / S]);
        inject(it);
        A.step_v();
        inject_force(it);
        A.step_t();
        if (seis_out)
            for (int r = 0; r < nrec; r++) seis_out[(size_t)r * nt + it] = A.f[rec_comp[r]][roff[r]];
    }

    // backward, segment by segment
    double gforce = 0;
    std::vector<std::vector<double>> snap;  // snap[i]: fields after V (+force) of step s0+i-1; snap[0]: checkpoint
    for (int sgi = nseg - 1; sgi >= 0; sgi--) {
        const int s0 = sgi * S, s1 = std::min(nt, s0 + S);
        load(ck[sgi]);
        snap.assign((size_t)(s1 - s0 + 1) * ORC_NFIELD, std::vector<double>());
        for (int q = 0; q < ORC_NFIELD; q++) snap[q] = A.f[q];
        for (int it = s0; it < s1; it++) {
            inject(it);
            A.step_v();
            inject_force(it);
            const size_t b = (size_t)(it - s0 + 1) * ORC_NFIELD;
            for (int q = 0; q < ORC_NFIELD; q++) snap[b + q] = A.f[q];
            A.step_t();
        }
        for (int it = s1 - 1; it >= s0; it--) {
            // record^T
            if (adj_src)
                for (int r = 0; r < nrec; r++) A.lf[rec_comp[r]][roff[r]] += adj_src[(size_t)r * nt + it];
            const std::vector<double>* cur = &snap[(size_t)(it - s0 + 1) * ORC_NFIELD];
            const std::vector<double>* prev = &snap[(size_t)(it - s0) * ORC_NFIELD];
            A.adj_t(cur);
            double gw = 0;
            if (cfg->src_kind == ORC_SRC_FORCE_Z) {
                gw = A.lf[ORC_VZ][so] * force;
                gforce += A.lf[ORC_VZ][so] * wavelet[it];
            }
            A.adj_v(cur, prev);
            if (cfg->src_kind == ORC_SRC_EXPLOSIVE) gw = A.lf[ORC_SXX][so] + A.lf[ORC_SYY][so] + A.lf[ORC_SZZ][so];
            else if (cfg->src_kind == ORC_SRC_PRESSURE) gw = A.lf[ORC_P][so];
            if (grad_wavelet) grad_wavelet[it] = gw;
            // adjoint-state storage: the largest magnitude of each adjoint field, and optionally the state
            // rounded to binary16 times a per-field scale between steps (what an FP16-stored adjoint keeps)
            for (int q = 0; q < ORC_NFIELD && (lf_max || lf_scale); q++) {
                double mx = lf_max ? lf_max[q] : 0.0;
                long long sat = 0;
                const double sc = lf_scale ? lf_scale[q] : 0.0;
                for (size_t c = 0; c < N; c++) {
                    double& v = A.lf[q][c];
                    mx = std::max(mx, std::fabs(v));
                    if (sc > 0) {
                        const double w = (double)(_Float16)(v * sc);
                        if (std::isinf(w)) sat++;
                        v = w / sc;
                    }
                }
                if (lf_max) lf_max[q] = mx;
                if (lf_saturated) *lf_saturated += sat;
            }
        }
    }

    if (grad_coef)
        for (int j = 0; j < ORC_NCOEF; j++)
            for (size_t c = 0; c < N; c++) grad_coef[(size_t)j * N + c] = A.g[j][c];
    if (!grad_mod) return 0;

    // coefficient build transposed: effective -> physical -> moduli (main.cpp:322-494 formulas)
    std::vector<double> gm((size_t)ORC_NMOD * N, 0.0);
    auto GM = [&](int q, size_t c) -> double& { return gm[(size_t)q * N + c]; };
    auto m = [&](int q, size_t c) { return (double)mod[q][c]; };
    const double dt = cfg->dt;
    const size_t sy = A.sy;
    for (int kk = 1; kk < A.nz - 1; kk++)
        for (int j = 1; j < A.ny - 1; j++)
            for (int i = 1; i < A.nx - 1; i++) {
                const size_t c = kk * sz + j * sy + i;
                double gp[ORC_NCOEF];
                for (int q = 0; q < ORC_NCOEF; q++) gp[q] = A.g[q][c] * A.ratio[q];
                GM(ORC_C, c) += (gp[ORC_P1] + gp[ORC_S3]) * dt;
                GM(ORC_M, c) += gp[ORC_P2] * dt;
                GM(ORC_H2U, c) += gp[ORC_S1] * dt;
                GM(ORC_HH, c) += gp[ORC_S2] * dt;
                auto harm_adj = [&](double gh, size_t a0, size_t a1, size_t a2, size_t a3) {
                    const size_t cs[4] = {a0, a1, a2, a3};
                    double inv = 0;
                    for (size_t x : cs) {
                        if (m(ORC_MU, x) == 0) return;
                        inv += 1.0 / m(ORC_MU, x);
                    }
                    const double hm = 1.0 / (0.25 * inv);
                    for (size_t x : cs) GM(ORC_MU, x) += gh * dt * hm * hm / (4.0 * m(ORC_MU, x) * m(ORC_MU, x));
                };
                harm_adj(gp[ORC_SXZC], c, c + 1, c + sz, c + sz + 1);
                harm_adj(gp[ORC_SYZC], c, c + sy, c + sz, c + sz + sy);
                harm_adj(gp[ORC_SXYC], c, c + 1, c + sy, c + sy + 1);
                const size_t nb[3] = {c + 1, c + sy, c + sz};
                double rho[3], rhof[3], b[3], mm[3];
                for (int a = 0; a < 3; a++) {
                    rho[a] = 0.5 * (m(ORC_RHO, c) + m(ORC_RHO, nb[a]));
                    rhof[a] = 0.5 * (m(ORC_RHOF, c) + m(ORC_RHOF, nb[a]));
                    b[a] = 0.5 * (m(ORC_C1, c) + m(ORC_C1, nb[a]));
                    mm[a] = 0.5 * (m(ORC_C2, c) + m(ORC_C2, nb[a]));
                }
                const bool vw = !(b[0] == 0 || b[1] == 0 || b[2] == 0);
                const bool vu = !(rho[0] == 0 || rho[1] == 0 || rho[2] == 0);
                for (int a = 0; a < 3; a++) {
                    double grho = 0, grhof = 0, gb = 0, gmm = 0;
                    if (vw) {
                        const double r = rho[a], rf = rhof[a];
                        const double mp = mm[a] - rf * rf / r;
                        const double D = mp + 0.5 * dt * b[a];
                        const double g1 = gp[ORC_VW1X + a], g2 = gp[ORC_VW2X + a], g3 = gp[ORC_VW3X + a];
                        // VW1 = (mp - dt b/2)/D, VW2 = dt (rf/r)/D, VW3 = dt/D
                        const double gmp_direct = g1 * (dt * b[a]) / (D * D);
                        const double gD = -g2 * dt * (rf / r) / (D * D) - g3 * dt / (D * D);
                        const double gmp = gmp_direct + gD;
                        gb += g1 * (-dt * mp / (D * D)) + gD * 0.5 * dt;
                        const double gratio = g2 * dt / D;
                        gmm += gmp;
                        grhof += gmp * (-2.0 * rf / r) + gratio / r;
                        grho += gmp * (rf * rf / (r * r)) - gratio * rf / (r * r);
                    }
                    if (vu) {
                        const double r = rho[a], rf = rhof[a];
                        grho += gp[ORC_VU1X + a] * (-dt / (r * r)) + gp[ORC_VU2X + a] * (-rf / (r * r));
                        grhof += gp[ORC_VU2X + a] / r;
                    }
                    GM(ORC_RHO, c) += 0.5 * grho;
                    GM(ORC_RHO, nb[a]) += 0.5 * grho;
                    GM(ORC_RHOF, c) += 0.5 * grhof;
                    GM(ORC_RHOF, nb[a]) += 0.5 * grhof;
                    GM(ORC_C1, c) += 0.5 * gb;
                    GM(ORC_C1, nb[a]) += 0.5 * gb;
                    GM(ORC_C2, c) += 0.5 * gmm;
                    GM(ORC_C2, nb[a]) += 0.5 * gmm;
                }
            }
    if (cfg->src_kind == ORC_SRC_FORCE_Z) {  // force = dt / rho_z, rho_z = (rho[s] + rho[s+z]) / 2
        const double rz = 0.5 * ((double)mod[ORC_RHO][so] + (double)mod[ORC_RHO][so + sz]);
        const double gr = gforce * (-cfg->dt / (rz * rz)) * 0.5;
        GM(ORC_RHO, so) += gr;
        GM(ORC_RHO, so + sz) += gr;
    }
    // keep only cells whose dependent coefficient cells all lie in the differentiated domain
    int lo[3], hi3[3];
    for (int a = 0; a < 3; a++) {
        const int n = n3[a];
        lo[a] = std::max(A.L, A.R) + 1;
        hi3[a] = A.L > 0 ? std::min(n - 2 - A.L, n - A.R - 1) : n - A.R - 1;
    }
    for (int kk = 0; kk < A.nz; kk++)
        for (int j = 0; j < A.ny; j++)
            for (int i = 0; i < A.nx; i++) {
                const bool in = i >= lo[0] && i <= hi3[0] && j >= lo[1] && j <= hi3[1] && kk >= lo[2] && kk <= hi3[2];
                const size_t c = kk * sz + j * sy + i;
                for (int q = 0; q < ORC_NMOD; q++) grad_mod[(size_t)q * N + c] = in ? GM(q, c) : 0.0;
            }
    return 0;
}

extern "C" int orc_adjoint(const orc_cfg* cfg, const float* const mod[ORC_NMOD], const float* wavelet, int nt,
                           int nrec, const int* rec_ijk, const int* rec_comp, const double* adj_src, int stride,
                           double* seis_out, double* grad_wavelet, double* grad_coef, double* grad_mod) {
    return orc_adjoint_ex(cfg, mod, wavelet, nt, nrec, rec_ijk, rec_comp, adj_src, stride, seis_out, grad_wavelet,
                          grad_coef, grad_mod, nullptr, nullptr, nullptr);
}
