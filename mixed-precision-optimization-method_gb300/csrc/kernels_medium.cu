// kernels_medium.cu -- device-side synthetic media (layers + Gaussian-correlated perturbations +
// a Gaussian anomaly), so that 1024^3 media never cross the host link.
//
// Algorithm (mirrored on the host by behf.problems.spec_medium):
//   noise   z(f, c) = sqrt(-2 ln u1) cos(2 pi u2) in double, u1/u2 = 24-bit fields of
//           splitmix64(c | f << 32 | seed << 36) offset by half a unit, f = 0..3, c = linear cell
//   smooth  separable Gaussian of std corr/2 cells (half-width ceil(4 std), weights normalised to 1),
//           periodic wrap, passes in x then y then z, result divided by (sum w^2)^(3/2) -> unit variance
//   rock    layer rock by z, then K_dry *= 1 + pct g0, mu *= 1 + pct g1, phi *= 1 + pct g2,
//           kappa *= exp(sigma_kappa g3); anomaly G = exp(-r^2/R^2): K_dry *= 1 + dK G,
//           kappa *= kf^G
//   moduli  Biot-Gassmann of outputfunc.cpp:202-217 (see behf.problems.rock_moduli)
#include <cmath>
#include <vector>

#include "behf_internal.cuh"
#include "behf_medium.cuh"

namespace behf {
namespace {

__host__ __device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__global__ void k_noise(float* out, long long N, int f, int seed) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h =
            splitmix64((unsigned long long)c | ((unsigned long long)f << 32) | ((unsigned long long)seed << 36));
        const double u1 = ((double)(h >> 40) + 0.5) * (1.0 / 16777216.0);
        const double u2 = ((double)((h >> 16) & 0xFFFFFFull) + 0.5) * (1.0 / 16777216.0);
        out[c] = (float)(sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2));
    }
}

// One periodic Gaussian pass along axis `ax` (0 = x, 1 = y, 2 = z).
__global__ void k_smooth(const float* in, float* out, int nx, int ny, int nz, int ax, const float* w, int half) {
    const long long N = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % nx);
        const long long r = c / nx;
        const int j = (int)(r % ny), k = (int)(r / ny);
        const int n = ax == 0 ? nx : ax == 1 ? ny : nz;
        const int p = ax == 0 ? i : ax == 1 ? j : k;
        const long long stride = ax == 0 ? 1 : ax == 1 ? nx : (long long)nx * ny;
        const long long base = c - (long long)p * stride;
        float acc = 0.f;
        for (int t = -half; t <= half; t++) {
            int q = p - t;  // np.roll(f, t): out[p] = in[p - t]
            q %= n;
            if (q < 0) q += n;
            acc += w[t + half] * in[base + (long long)q * stride];
        }
        out[c] = acc;
    }
}

__device__ void rock_moduli_dev(const double r[10], float out[kNMod], long long c, long long N) {
    const double Ks = r[0], Kf = r[1], Kdry = r[2], mu = r[3], rhos = r[4], rhof = r[5], phi = r[6], kappa = r[7],
                 eta = r[8], tau = r[9];
    double m[kNMod];
    if (phi >= 1.0) {
        m[BEHF_RHO] = rhof;
        m[BEHF_RHOF] = rhof;
        m[BEHF_MU] = 0;
        m[BEHF_M] = m[BEHF_C] = m[BEHF_HH] = m[BEHF_H2U] = Kf;
        m[BEHF_C1] = 0;
        m[BEHF_C2] = rhof;
    } else {
        const double a = 1 - Kdry / Ks;
        const double M = Kf * Ks / (phi * Ks + (a - phi) * Kf);
        const double HH = a * a * M + Kdry + mu * 4.0 / 3.0;
        m[BEHF_RHO] = (1 - phi) * rhos + phi * rhof;
        m[BEHF_RHOF] = rhof;
        m[BEHF_MU] = mu;
        m[BEHF_M] = M;
        m[BEHF_C] = M * a;
        m[BEHF_HH] = HH;
        m[BEHF_H2U] = HH - 2 * mu;
        m[BEHF_C1] = eta / kappa;
        m[BEHF_C2] = (1 + 2 / 8.0) * tau * rhof / phi;
    }
    for (int q = 0; q < kNMod; q++) out[q] = (float)m[q];
}

struct MedArgs {
    int nx, ny, nz;
    int nlayers;
    double rock[4][10];
    int iface[3];
    const float* g[4];  // smoothed unit-variance fields or null
    double pct, skappa, gnorm;
    int anomaly;
    double ac[3], ar, adk, akf;
    float* mod[kNMod];
};

__global__ void k_moduli(MedArgs a) {
    const long long N = (long long)a.nx * a.ny * a.nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % a.nx);
        const long long rr = c / a.nx;
        const int j = (int)(rr % a.ny), k = (int)(rr / a.ny);
        int L = 0;
        while (L < a.nlayers - 1 && k >= a.iface[L]) L++;
        double r[10];
        for (int t = 0; t < 10; t++) r[t] = a.rock[L][t];
        if (a.g[0]) {
            const double g0 = a.g[0][c] * a.gnorm, g1 = a.g[1][c] * a.gnorm, g2 = a.g[2][c] * a.gnorm,
                         g3 = a.g[3][c] * a.gnorm;
            r[2] *= 1 + a.pct * g0;
            r[3] *= 1 + a.pct * g1;
            if (r[6] < 1.0) r[6] *= 1 + a.pct * g2;
            r[7] *= exp(a.skappa * g3);
        }
        if (a.anomaly) {
            const double dx = i - a.ac[0], dy = j - a.ac[1], dz = k - a.ac[2];
            const double G = exp(-(dx * dx + dy * dy + dz * dz) / (a.ar * a.ar));
            r[2] *= 1 + a.adk * G;
            r[7] *= pow(a.akf, G);
        }
        float out[kNMod];
        rock_moduli_dev(r, out, c, N);
        for (int q = 0; q < kNMod; q++) a.mod[q][c] = out[q];
    }
}

}  // namespace

cudaError_t generate_medium(const behf_medium_spec& s, int nx, int ny, int nz, float* const mod[kNMod], float* work,
                            cudaStream_t st, int nblk) {
    const long long N = (long long)nx * ny * nz;
    MedArgs a{};
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.nlayers = s.nlayers < 1 ? 1 : (s.nlayers > 4 ? 4 : s.nlayers);
    for (int L = 0; L < a.nlayers; L++) {
        const behf_rock& r = s.layers[L];
        const double v[10] = {r.Ks, r.Kf, r.Kdry, r.mu, r.rhos, r.rhof, r.phi, r.kappa, r.eta, r.tau};
        for (int t = 0; t < 10; t++) a.rock[L][t] = v[t];
    }
    for (int t = 0; t < 3; t++) a.iface[t] = s.interface_z[t];
    a.pct = s.pct;
    a.skappa = s.log_kappa_sigma;
    a.anomaly = s.anomaly;
    for (int t = 0; t < 3; t++) a.ac[t] = s.anom_center[t];
    a.ar = s.anom_radius_cells > 0 ? s.anom_radius_cells : 1.0;
    a.adk = s.anom_dkdry;
    a.akf = s.anom_kappa_factor > 0 ? s.anom_kappa_factor : 1.0;
    for (int q = 0; q < kNMod; q++) a.mod[q] = mod[q];
    float* wdev = nullptr;
    cudaError_t e = cudaSuccess;
    if (s.pct != 0 || s.log_kappa_sigma != 0) {
        // work holds 5 volumes: 4 smoothed fields + 1 scratch
        const double sig = s.corr_cells / 2.0;
        const int half = (int)std::ceil(4 * sig);
        std::vector<float> w(2 * half + 1);
        double sum = 0, sum2 = 0;
        std::vector<double> wd(2 * half + 1);
        for (int t = -half; t <= half; t++) wd[t + half] = std::exp(-0.5 * (t / sig) * (t / sig));
        for (double v : wd) sum += v;
        for (auto& v : wd) {
            v /= sum;
            sum2 += v * v;
        }
        for (size_t t = 0; t < wd.size(); t++) w[t] = (float)wd[t];
        a.gnorm = 1.0 / std::pow(std::sqrt(sum2), 3);
        if ((e = cudaMalloc(&wdev, w.size() * 4)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(wdev, w.data(), w.size() * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess) goto out;
        {
            float* tmp = work + 4 * N;
            for (int f = 0; f < 4; f++) {
                float* g = work + (long long)f * N;
                k_noise<<<nblk, 256, 0, st>>>(g, N, f, s.seed);
                k_smooth<<<nblk, 256, 0, st>>>(g, tmp, nx, ny, nz, 0, wdev, half);
                k_smooth<<<nblk, 256, 0, st>>>(tmp, g, nx, ny, nz, 1, wdev, half);
                k_smooth<<<nblk, 256, 0, st>>>(g, tmp, nx, ny, nz, 2, wdev, half);
                if ((e = cudaMemcpyAsync(g, tmp, N * 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) goto out;
                a.g[f] = g;
            }
        }
    }
    k_moduli<<<nblk, 256, 0, st>>>(a);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
out:
    if (wdev) cudaFree(wdev);
    return e;
}

}  // namespace behf
