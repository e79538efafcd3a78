// behf_main.cpp -- command-line driver over libbehf: the role of the reference's main() and the output half
// of callCUDAKernel (main.cpp:59-1760, kernel.cu:1728-2571) on one GPU.
//
//   behf_run [--preset borehole|small64|layered256|random1024] [--scale S] [--nt N] [--precision f16|bf16|f32|f64]
//            [--radius R] [--kernel auto|plain|tiled] [--variant auto|classic|ws|tmem|tmem_xs]
//            [--snap 1000,2000,3000] [--snap-field sxx]
//            [--out DIR] [--format text|binary|both] [--chunk N] [--ref-bug-compat 0|1] [--quiet] [--setup-only]
//
// It sets up the problem (grid, medium, CPML, Ricker source, receivers), runs the time loop through the C ABI
// in chunks that end at the snapshot steps, and writes
//   sis_<name>.dat        seismograms of one recorded field, one row per receiver, one column per step
//                         (the reference's sisx.dat / sisx2.dat / sisx3.dat, kernel.cu:2557-2571)
//   <name>pro_<it>.dat    the y-mid xz slice of the snapshot field after step it (the reference's
//                         "txxpro<rank> <it>.dat", kernel.cu:2247-2387, one file for the whole domain)
// in the reference's text layout (wfile / wfile3d, outputfunc.cpp:35-50, 97-123) and/or a binary layout
// (<file>.bin: "BEHFOUT1", int32 ndim, int32 dtype (1 = float32), int64 dims[ndim], float32 data).
// <name> is the reference's array name of the field (vux, vuy, vuz, vwx, vwy, vwz, txx, tyy, tzz, txy, txz,
// tyz, ss).  --setup-only writes the problem's inputs instead (wavelet.bin, receivers.bin as int32 rows
// ix iy iz field, moduli.bin when the medium is built on the host) and prints the grid, without touching a GPU.
// The last line on stdout is a one-line JSON summary.  Exit status 0 on success, 1 on a usage
// error, 2 on a library error (its text goes to stderr).
#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "behf.h"

namespace {

const char* const kFieldName[BEHF_NFIELD] = {"vx", "vy", "vz", "qx", "qy", "qz", "sxx",
                                             "syy", "szz", "sxy", "sxz", "syz", "p"};
// Array names of the same fields in the reference (common.h: d_vux .. d_ss).
const char* const kRefName[BEHF_NFIELD] = {"vux", "vuy", "vuz", "vwx", "vwy", "vwz", "txx",
                                           "tyy", "tzz", "txy", "txz", "tyz", "ss"};

struct Rock {  // parameters of one rock (the inputs of create_model_all, outputfunc.cpp:153-222)
    double Ks, Kf, Kdry, mu, rhos, rhof, phi, kappa, eta, tau;
};
const Rock kSandstone = {37e9, 2.25e9, 9e9, 7e9, 2650.0, 1000.0, 0.2, 1e-12, 1e-3, 2.4};
const Rock kStiff = {37e9, 2.25e9, 20e9, 15e9, 2650.0, 1000.0, 0.1, 1e-14, 1e-3, 2.4};

struct Options {
    std::string preset = "borehole";
    double scale = 1.0;
    int nt = 0;
    std::string precision;
    int radius = 0;
    std::string kernel = "auto";
    int variant = 0;  // BEHF_OPT_TILED_VARIANT (0 automatic)
    std::vector<int> snaps;
    bool snaps_set = false;
    int snap_field = BEHF_SXX;
    std::string out = ".";
    bool text = true, binary = false;
    int chunk = -1;
    int bug = -1;
    bool quiet = false;
    bool setup_only = false;
};

struct Problem {
    behf_grid g{};
    int precision = BEHF_FP16;
    int src_kind = BEHF_SRC_EXPLOSIVE;
    int sx = 0, sy = 0, sz = 0;
    double f0 = 30.0;
    bool ref_ricker = false;
    bool bug = false;
    std::vector<float> moduli;         // [9][nz][ny][nx] host moduli, or empty (device generator)
    behf_medium_spec spec{};           // used when moduli is empty
    std::vector<int> rec_ijk, rec_comp;
    int nt = 0;
};

void usage(FILE* f) {
    std::fprintf(f,
                 "usage: behf_run [--preset borehole|small64|layered256|random1024] [--scale S] [--nt N]\n"
                 "                [--precision f16|bf16|f32|f64] [--radius R] [--kernel auto|plain|tiled]\n"
                 "                [--variant auto|classic|ws|tmem|tmem_xs]\n"
                 "                [--snap it,it,...] [--snap-field NAME] [--out DIR] [--format text|binary|both]\n"
                 "                [--chunk N] [--ref-bug-compat 0|1] [--quiet] [--setup-only]\n");
}

int field_index(const char* s) {
    for (int i = 0; i < BEHF_NFIELD; i++)
        if (!std::strcmp(s, kFieldName[i]) || !std::strcmp(s, kRefName[i])) return i;
    return -1;
}

int precision_index(const std::string& s) {
    if (s == "f64") return BEHF_FP64;
    if (s == "f32") return BEHF_FP32;
    if (s == "f16") return BEHF_FP16;
    if (s == "bf16") return BEHF_BF16;
    return -1;
}

bool parse(int argc, char** argv, Options& o) {
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        auto val = [&](const char* name) -> const char* {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "behf_run: %s needs a value\n", name);
                return nullptr;
            }
            return argv[++i];
        };
        const char* v = nullptr;
        if (a == "--help" || a == "-h") {
            usage(stdout);
            std::exit(0);
        } else if (a == "--quiet") {
            o.quiet = true;
        } else if (a == "--setup-only") {
            o.setup_only = true;
        } else if (!(v = val(a.c_str()))) {
            return false;
        } else if (a == "--preset") {
            o.preset = v;
        } else if (a == "--scale") {
            o.scale = std::atof(v);
        } else if (a == "--nt") {
            o.nt = std::atoi(v);
        } else if (a == "--precision") {
            o.precision = v;
            if (precision_index(o.precision) < 0) return false;
        } else if (a == "--radius") {
            o.radius = std::atoi(v);
        } else if (a == "--kernel") {
            o.kernel = v;
        } else if (a == "--variant") {
            const std::string t = v;
            const char* const names[5] = {"auto", "classic", "ws", "tmem", "tmem_xs"};
            o.variant = -1;
            for (int q = 0; q < 5; q++)
                if (t == names[q]) o.variant = q;
            if (o.variant < 0) return false;
        } else if (a == "--snap") {
            o.snaps.clear();
            o.snaps_set = true;
            for (const char* p = v; *p;) {
                char* end = nullptr;
                const long it = std::strtol(p, &end, 10);
                if (end == p) return false;
                o.snaps.push_back((int)it);
                p = (*end == ',') ? end + 1 : end;
            }
        } else if (a == "--snap-field") {
            o.snap_field = field_index(v);
            if (o.snap_field < 0) return false;
        } else if (a == "--out") {
            o.out = v;
        } else if (a == "--format") {
            const std::string f = v;
            o.text = (f == "text" || f == "both");
            o.binary = (f == "binary" || f == "both");
            if (!o.text && !o.binary) return false;
        } else if (a == "--chunk") {
            o.chunk = std::atoi(v);
        } else if (a == "--ref-bug-compat") {
            o.bug = std::atoi(v);
        } else {
            std::fprintf(stderr, "behf_run: unknown option %s\n", a.c_str());
            return false;
        }
    }
    return o.scale > 0 && o.nt >= 0 && o.radius >= 0 && o.radius <= 4;
}

// Biot-Gassmann moduli of one rock, in the order of the BEHF_* moduli enum (float, as the reference's volumes).
void rock_moduli(const Rock& r, float out[BEHF_NMOD]) {
    const double alpha = 1.0 - r.Kdry / r.Ks;
    const double M = r.Kf * r.Ks / (r.phi * r.Ks + (alpha - r.phi) * r.Kf);
    const double H = alpha * alpha * M + r.Kdry + 4.0 * r.mu / 3.0;
    out[BEHF_RHO] = (float)((1.0 - r.phi) * r.rhos + r.phi * r.rhof);
    out[BEHF_RHOF] = (float)r.rhof;
    out[BEHF_MU] = (float)r.mu;
    out[BEHF_M] = (float)M;
    out[BEHF_C] = (float)(alpha * M);
    out[BEHF_HH] = (float)H;
    out[BEHF_H2U] = (float)(H - 2.0 * r.mu);
    out[BEHF_C1] = (float)(r.eta / r.kappa);
    out[BEHF_C2] = (float)((1.0 + 2.0 / 8.0) * r.tau * r.rhof / r.phi);
}

// The reference's borehole medium (outputfunc.cpp:153-222): a fluid column of radius 10 cells around the
// z axis through (nx/2, ny/2) inside a porous formation, with the reference's float/double rounding steps.
void borehole_moduli(int nx, int ny, int nz, std::vector<float>& mod) {
    const float vp = 5000.f, vs = 3300.f, rhos = 2450.f, rhof = 1000.f, vf = 1500.f;
    const double por = 0.1;
    const float rho = (float)((1 - por) * rhos + por * rhof);
    const float mu = (float)((1 - por) * (double)rhos * (double)vs * (double)vs);
    const double vp2 = (double)(vp * vp), vs2 = (double)(vs * vs);
    const double kb = (double)rhos * (1 - por) * (vp2 - vs2 * 4.0 / 3.0);
    const double ks = (double)rhos * (vp2 - vs2 * 4.0 / 3.0);
    const double kf = (double)((rhof * vf) * vf);
    const double a1 = 1 - kb / ks;
    const float M = (float)(kf * ks / (por * ks + (a1 - por) * kf));
    const float HH = (float)(a1 * a1 * (double)M + kb + (double)mu * 4.0 / 3.0);
    const double eta = 1.0 * std::pow(10.0, -3), perm = 2 * std::pow(10.0, -12);
    const float form[BEHF_NMOD] = {rho, rhof, mu, M, (float)((double)M * a1), HH, HH - 2.f * mu,
                                   (float)(eta / perm), (float)((1 + 2 / 8.0) * 3.0 * (double)rhof / por)};
    const float kff = (1000.f * 1500.f) * 1500.f;
    const float fluid[BEHF_NMOD] = {1000.f, 1000.f, 0.f, kff, kff, kff, kff, 0.f, 1000.f};
    const size_t plane = (size_t)nx * ny, vol = plane * nz;
    mod.assign((size_t)BEHF_NMOD * vol, 0.f);
    for (int q = 0; q < BEHF_NMOD; q++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                const int dx = ix - nx / 2, dy = iy - ny / 2;
                const float v = (dx * dx + dy * dy <= 100) ? fluid[q] : form[q];
                for (int iz = 0; iz < nz; iz++) mod[q * vol + iz * plane + (size_t)iy * nx + ix] = v;
            }
}

void spec_rock(behf_rock& d, const Rock& r) {
    d.Ks = r.Ks; d.Kf = r.Kf; d.Kdry = r.Kdry; d.mu = r.mu; d.rhos = r.rhos;
    d.rhof = r.rhof; d.phi = r.phi; d.kappa = r.kappa; d.eta = r.eta; d.tau = r.tau;
}

double p_velocity(const Rock& r) {
    float m[BEHF_NMOD];
    rock_moduli(r, m);
    return std::sqrt((double)m[BEHF_HH] / (double)m[BEHF_RHO]);
}

// Receivers on a regular ix x iy grid at depth iz, each recording the given fields.
void surface_receivers(Problem& p, int n_side, int lo, int hi, int iz, std::initializer_list<int> comps) {
    for (int j = 0; j < n_side; j++)
        for (int i = 0; i < n_side; i++)
            for (int c : comps) {
                const int ix = n_side > 1 ? (int)std::lround(lo + (double)(hi - lo) * i / (n_side - 1)) : lo;
                const int iy = n_side > 1 ? (int)std::lround(lo + (double)(hi - lo) * j / (n_side - 1)) : lo;
                p.rec_ijk.insert(p.rec_ijk.end(), {ix, iy, iz});
                p.rec_comp.push_back(c);
            }
}

bool make_problem(const Options& o, Problem& p) {
    behf_grid& g = p.g;
    // grid shrink factor, rounded half to even (as Python's round)
    auto scaled = [&](int v, int lo) { return std::max(lo, (int)std::nearbyint(v * o.scale)); };
    if (o.preset == "borehole") {
        // main.cpp:20-23, 84-99: 180 x 180 x 300 cells of 1 cm plus a 30-cell CPML, 1 us steps, 10 kHz,
        // source 20 cells below the top CPML on the axis, txx recorded on the vertical line through it.
        const int NX = scaled(180, 24), NY = scaled(180, 24), NZ = scaled(300, 24), NP = scaled(30, 4);
        g.nx = NX + 2 * NP; g.ny = NY + 2 * NP; g.nz = NZ + 2 * NP;
        g.h = 0.01; g.dt = 1e-6; g.radius = 1; g.cpml_width = NP; g.cpml_v0 = 4000.0; g.cpml_r = 1e-6;
        g.scales[0] = 1e8; g.scales[1] = 1e8; g.scales[2] = 1.0; g.scales[3] = 1.0;
        p.f0 = 1e4; p.nt = 3500; p.ref_ricker = true; p.bug = true; p.precision = BEHF_FP16;
        p.sx = g.nx / 2; p.sy = g.ny / 2; p.sz = std::min(20 + NP, g.nz - NP - 2);
        borehole_moduli(g.nx, g.ny, g.nz, p.moduli);
        for (int iz = 0; iz < g.nz; iz++) {
            p.rec_ijk.insert(p.rec_ijk.end(), {p.sx, p.sy, iz});
            p.rec_comp.push_back(BEHF_SXX);
        }
    } else if (o.preset == "small64" || o.preset == "layered256" || o.preset == "random1024") {
        const bool small = o.preset == "small64", layered = o.preset == "layered256";
        const int n = scaled(small ? 64 : layered ? 256 : 1024, 8);
        const int L = small ? 10 : 20;
        g.nx = g.ny = g.nz = n;
        g.h = 5.0; g.dt = 4e-4; g.radius = 4; g.cpml_width = L; g.cpml_r = 1e-6;
        p.f0 = small ? 30.0 : layered ? 25.0 : 20.0;
        p.nt = small ? 500 : layered ? 2000 : 3000;
        p.precision = BEHF_FP16;
        behf_medium_spec& s = p.spec;
        std::memset(&s, 0, sizeof s);
        spec_rock(s.layers[0], kSandstone);
        s.nlayers = 1;
        s.seed = 1234;
        s.corr_cells = 10.0;
        const int c = n / 2;
        if (small) {
            g.cpml_v0 = p_velocity(kSandstone);
            p.sx = p.sy = p.sz = c;
            for (int i = 0; i < 32; i++) {
                const int ix = (int)std::lround(L + 2 + (double)(n - 2 * L - 5) * i / 31);
                for (int comp : {BEHF_VZ, BEHF_P}) {
                    p.rec_ijk.insert(p.rec_ijk.end(), {ix, c, std::min(c + 10, n - L - 2)});
                    p.rec_comp.push_back(comp);
                }
            }
        } else if (layered) {
            spec_rock(s.layers[1], kStiff);
            s.nlayers = 2;
            s.interface_z[0] = n / 2;
            g.cpml_v0 = p_velocity(kStiff);
            p.sx = p.sy = c; p.sz = std::max(L + 6, (L + n / 2) / 2);
            surface_receivers(p, 16, L + 4, n - L - 5, L + 2, {BEHF_VZ, BEHF_P});
        } else {
            s.pct = 0.05;
            s.log_kappa_sigma = 0.5;
            g.cpml_v0 = p_velocity(kSandstone) * 1.1;
            p.src_kind = BEHF_SRC_FORCE_Z;
            p.sx = p.sy = c; p.sz = std::min(n / 4, n - L - 6);
            surface_receivers(p, std::min(512, n - 2 * L - 4), L + 2, n - L - 3, L + 2, {BEHF_VZ, BEHF_P});
        }
    } else {
        std::fprintf(stderr, "behf_run: unknown preset %s\n", o.preset.c_str());
        return false;
    }
    if (o.nt > 0) p.nt = o.nt;
    if (!o.precision.empty()) p.precision = precision_index(o.precision);
    if (o.radius > 0) g.radius = o.radius;
    if (o.bug >= 0) p.bug = o.bug != 0;
    return true;
}

// Ricker wavelet -(1 - 2 pi^2 f^2 tau^2) exp(-pi^2 f^2 tau^2), tau = t - 1.2/f.  The borehole preset evaluates
// it the way kernel.cu:1890-1898 does (float t = it*DT and T0, the product in double with pi = 3.1415926535);
// the other presets in double throughout.
std::vector<float> ricker(int nt, double dt, double f0, bool ref_form) {
    std::vector<float> w(nt);
    if (ref_form) {
        const double pi = 3.1415926535;
        const float DT = (float)dt, F0 = (float)f0, T0 = (float)(1.2 / (double)F0);
        for (int it = 0; it < nt; it++) {
            const float tt = it * DT;
            const double d = (double)(tt - T0);
            const double a2 = 2 * pi * pi * F0 * F0 * d * d;
            const double a = pi * pi * F0 * F0 * d * d;
            w[it] = (float)(-(1 - a2) * std::exp(-a));
        }
    } else {
        const double pi = 3.14159265358979323846, t0 = 1.2 / f0;
        for (int it = 0; it < nt; it++) {
            const double tau = it * dt - t0;
            const double a = pi * pi * f0 * f0 * tau * tau;
            w[it] = (float)(-(1 - 2 * a) * std::exp(-a));
        }
    }
    return w;
}

// ----------------------------------------------------------------------------------------------- outputs
// Text layout of the reference's wfile / wfile3d: every value as "%e ", a newline after the last column of
// a row and one more after the row (a blank line between rows).
bool write_text(const std::string& path, const float* data, long long rows, long long cols) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::vector<char> buf(1 << 20);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    for (long long r = 0; r < rows; r++) {
        for (long long c = 0; c < cols; c++) std::fprintf(f, "%e ", data[r * cols + c]);
        std::fputs("\n\n", f);
    }
    return std::fclose(f) == 0;
}

// dtype 1 = float32, 2 = int32 (4-byte values either way)
bool write_binary(const std::string& path, const void* data, const std::vector<int64_t>& dims, int32_t dtype) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const char magic[8] = {'B', 'E', 'H', 'F', 'O', 'U', 'T', '1'};
    const int32_t head[2] = {(int32_t)dims.size(), dtype};
    size_t n = 1;
    for (int64_t d : dims) n *= (size_t)d;
    bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(head, 4, 2, f) == 2 &&
              std::fwrite(dims.data(), 8, dims.size(), f) == dims.size() && std::fwrite(data, 4, n, f) == n;
    return std::fclose(f) == 0 && ok;
}

struct Writer {
    const Options& o;
    std::vector<std::string> files;
    bool put(const std::string& stem, const float* data, long long rows, long long cols) {
        if (o.text) {
            const std::string p = o.out + "/" + stem + ".dat";
            if (!write_text(p, data, rows, cols)) return fail(p);
            files.push_back(p);
        }
        if (o.binary) {
            const std::string p = o.out + "/" + stem + ".bin";
            if (!write_binary(p, data, {rows, cols}, 1)) return fail(p);
            files.push_back(p);
        }
        return true;
    }
    bool fail(const std::string& p) {
        std::fprintf(stderr, "behf_run: cannot write %s: %s\n", p.c_str(), std::strerror(errno));
        return false;
    }
};

struct Ctx {
    behf_ctx* c = nullptr;
    ~Ctx() {
        if (c) behf_destroy(c);
    }
};

int lib_fail(const char* what, behf_status st) {
    std::fprintf(stderr, "behf_run: %s failed (%d): %s\n", what, st, behf_last_error());
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
    Options o;
    if (!parse(argc, argv, o)) {
        usage(stderr);
        return 1;
    }
    Problem p;
    if (!make_problem(o, p)) return 1;
    if (!o.snaps_set) {
        for (int it : {1000, 2000, 3000})  // kernel.cu:2247-2387
            if (o.preset == "borehole" && it < p.nt) o.snaps.push_back(it);
    }
    if (mkdir(o.out.c_str(), 0755) != 0 && errno != EEXIST) {
        std::fprintf(stderr, "behf_run: cannot create %s: %s\n", o.out.c_str(), std::strerror(errno));
        return 1;
    }
    const behf_grid& g = p.g;
    const std::vector<float> wavelet = ricker(p.nt, g.dt, p.f0, p.ref_ricker);
    if (g.scales[0] == 0) {
        behf_grid& gm = p.g;
        double amp = 0;
        for (float v : wavelet) amp = std::max(amp, (double)std::fabs(v));
        gm.src_amp_hint = amp;
        gm.src_f0_hint = p.f0;
    }

    const int nrec = (int)p.rec_comp.size();
    if (o.setup_only) {
        std::vector<int32_t> rec((size_t)nrec * 4);
        for (int r = 0; r < nrec; r++) {
            for (int k = 0; k < 3; k++) rec[(size_t)r * 4 + k] = p.rec_ijk[(size_t)r * 3 + k];
            rec[(size_t)r * 4 + 3] = p.rec_comp[r];
        }
        bool ok = write_binary(o.out + "/wavelet.bin", wavelet.data(), {(int64_t)p.nt}, 1) &&
                  write_binary(o.out + "/receivers.bin", rec.data(), {(int64_t)nrec, 4}, 2);
        if (!p.moduli.empty())
            ok = ok && write_binary(o.out + "/moduli.bin", p.moduli.data(), {BEHF_NMOD, g.nz, g.ny, g.nx}, 1);
        if (!ok) {
            std::fprintf(stderr, "behf_run: cannot write the set-up files in %s\n", o.out.c_str());
            return 1;
        }
        std::printf("{\"preset\": \"%s\", \"grid\": [%d, %d, %d], \"h\": %.17g, \"dt\": %.17g, \"radius\": %d, "
                    "\"cpml_width\": %d, \"cpml_v0\": %.17g, \"cpml_r\": %.17g, \"scales\": [%.17g, %.17g, %.17g, %.17g], "
                    "\"src_kind\": %d, \"src\": [%d, %d, %d], \"f0\": %.17g, \"nt\": %d, \"precision\": %d, "
                    "\"ref_bug_compat\": %s, \"host_medium\": %s}\n",
                    o.preset.c_str(), g.nx, g.ny, g.nz, g.h, g.dt, g.radius, g.cpml_width, g.cpml_v0, g.cpml_r,
                    g.scales[0], g.scales[1], g.scales[2], g.scales[3], p.src_kind, p.sx, p.sy, p.sz, p.f0, p.nt,
                    p.precision, p.bug ? "true" : "false", p.moduli.empty() ? "false" : "true");
        return 0;
    }

    Ctx ctx;
    behf_status st = behf_create(&g, p.precision, &ctx.c);
    if (st) return lib_fail("behf_create", st);
    if (p.bug && (st = behf_set_option(ctx.c, BEHF_OPT_REF_BUG_COMPAT, 1))) return lib_fail("set_option", st);
    const int kern = o.kernel == "plain" ? BEHF_KERNEL_PLAIN : o.kernel == "tiled" ? BEHF_KERNEL_TILED : BEHF_KERNEL_AUTO;
    if ((st = behf_set_option(ctx.c, BEHF_OPT_KERNEL, kern))) return lib_fail("set_option(kernel)", st);
    if (o.variant > 0 && (st = behf_set_option(ctx.c, BEHF_OPT_TILED_VARIANT, o.variant)))
        return lib_fail("set_option(variant)", st);
    if (o.chunk >= 0 && (st = behf_set_option(ctx.c, BEHF_OPT_GRAPH_CHUNK, o.chunk))) return lib_fail("set_option", st);
    if (!p.moduli.empty()) {
        const size_t vol = (size_t)g.nx * g.ny * g.nz;
        const float* mods[BEHF_NMOD];
        for (int q = 0; q < BEHF_NMOD; q++) mods[q] = p.moduli.data() + q * vol;
        st = behf_set_medium(ctx.c, mods);
    } else {
        st = behf_generate_medium(ctx.c, &p.spec);
    }
    if (st) return lib_fail("medium", st);
    if ((st = behf_set_source(ctx.c, p.src_kind, p.sx, p.sy, p.sz, wavelet.data(), p.nt))) return lib_fail("set_source", st);
    if ((st = behf_set_receivers(ctx.c, nrec, p.rec_ijk.data(), p.rec_comp.data(), p.nt))) return lib_fail("set_receivers", st);

    Writer out{o, {}};
    std::vector<float> field, slice;
    double run_s = 0;
    int done = 0;
    std::vector<int> snap_stops;  // snapshot after step it = after it + 1 steps
    for (int it : o.snaps)
        if (it >= 0 && it < p.nt) snap_stops.push_back(it + 1);
    std::sort(snap_stops.begin(), snap_stops.end());
    snap_stops.erase(std::unique(snap_stops.begin(), snap_stops.end()), snap_stops.end());
    auto advance = [&](int stop) -> behf_status {
        if (stop <= done) return BEHF_OK;
        const auto t0 = std::chrono::steady_clock::now();
        const behf_status s = behf_run(ctx.c, stop - done);
        run_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        done = stop;
        return s;
    };
    for (int stop : snap_stops) {
        if ((st = advance(stop))) return lib_fail("behf_run", st);
        // the xz slice at y = ny/2 (wfile3d's j = ny / 2)
        field.resize((size_t)g.nx * g.ny * g.nz);
        if ((st = behf_get_field(ctx.c, o.snap_field, field.data()))) return lib_fail("behf_get_field", st);
        slice.resize((size_t)g.nz * g.nx);
        const int j = g.ny / 2;
        for (int iz = 0; iz < g.nz; iz++)
            std::memcpy(&slice[(size_t)iz * g.nx], &field[((size_t)iz * g.ny + j) * g.nx], sizeof(float) * g.nx);
        if (!out.put(std::string(kRefName[o.snap_field]) + "pro_" + std::to_string(stop - 1), slice.data(), g.nz, g.nx))
            return 1;
        if (!o.quiet) std::printf("it=%d snapshot %s\n", stop - 1, kRefName[o.snap_field]);
    }
    if ((st = advance(p.nt))) return lib_fail("behf_run", st);

    // seismograms: one file per recorded field, receivers in the order given, one column per step
    std::vector<double> seis((size_t)nrec * p.nt);
    int recorded = 0;
    if ((st = behf_get_seismograms(ctx.c, seis.data(), &recorded))) return lib_fail("behf_get_seismograms", st);
    for (int f = 0; f < BEHF_NFIELD; f++) {
        std::vector<float> rows;
        long long nr = 0;
        for (int r = 0; r < nrec; r++) {
            if (p.rec_comp[r] != f) continue;
            for (int it = 0; it < recorded; it++) rows.push_back((float)seis[(size_t)r * recorded + it]);
            nr++;
        }
        if (nr && !out.put(std::string("sis_") + kRefName[f], rows.data(), nr, recorded)) return 1;
    }
    std::vector<double> norms(BEHF_NFIELD);
    const behf_status health = behf_health(ctx.c, norms.data());
    behf_info info{};
    behf_get_info(ctx.c, &info);
    const double cells = (double)g.nx * g.ny * g.nz;
    std::printf("{\"preset\": \"%s\", \"grid\": [%d, %d, %d], \"steps\": %d, \"precision\": %d, \"kernel\": %d, "
                "\"radius\": %d, \"run_s\": %.6f, \"gpts\": %.6f, \"health_ok\": %s, \"receivers\": %d, \"files\": [",
                o.preset.c_str(), g.nx, g.ny, g.nz, recorded, info.precision, info.kernel, info.radius, run_s,
                run_s > 0 ? cells * p.nt / run_s / 1e9 : 0.0, health == BEHF_OK ? "true" : "false", nrec);
    for (size_t i = 0; i < out.files.size(); i++) std::printf("%s\"%s\"", i ? ", " : "", out.files[i].c_str());
    std::printf("]}\n");
    return health == BEHF_OK ? 0 : 2;
}
