// behf_api.cu -- the C ABI of libbehf (include/behf.h): context, device memory, set-up and the
// graph-captured time loop.  Replaces the reference's host/device boundary: main.cpp:1529-1743
// (allocation and copies of the blockInfo arrays) and callCUDAKernel (kernel.cu:1728-2698).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "behf_adjoint.cuh"
#include "behf_aux.cuh"
#include "behf_internal.cuh"
#include "behf_medium.cuh"
#include "kernels_tiled.cuh"

using namespace behf;

namespace {
thread_local std::string g_err;

// Tiled-kernel variant chosen by BEHF_OPT_TILED_VARIANT = 0 (Geom::ws): the warp-specialised kernels with the z
// derivatives in tensor memory for the 16-bit kinds, the warp-specialised kernels for FP32 (1024^3 on one GB300:
// FP16 30.5 / 33.7 / 35.2, BF16 28.7 / 32.1 / 34.0, FP32 20.8 / 21.7 / 21.2 Gpt/s for classic / warp-specialised /
// tensor-memory z).
// Automatic tiled-kernel variant (Geom::ws = BEHF_OPT_TILED_VARIANT - 1): the tensor-memory kernels with the x-slab
// staging for FP16 and BF16, the fastest at 1024^3; the warp-specialised kernels for FP32, whose z derivatives
// alternate the taps of each pair (the tensor-memory kernels add them in plane order, one sign after the other:
// 5 % faster in FP32, but their rounding moved a 400-step FP32 gradient to 2.6e-4 of the FP64 adjoint, beyond the
// 1e-4 bar).
int auto_variant(int precision) { return precision == BEHF_FP16 || precision == BEHF_BF16 ? 3 : 1; }

behf_status fail(behf_status code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(BEHF_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                 \
    } while (0)

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

size_t elem_size(int prec) { return prec == BEHF_FP64 ? 8 : prec == BEHF_FP32 ? 4 : 2; }
size_t kelem_size(int prec) { return prec == BEHF_FP64 ? 8 : prec == BEHF_FP32 ? 4 : 2; }
size_t welem_size(int prec) { return prec == BEHF_FP64 ? 8 : 4; }  // CPML memory, VW1, profiles

// CPML profile of one axis (main.cpp:537-563): quadratic d on the slabs [0,L) and [n-1-L, n),
// half-shifted d2, d0 = 3 v0 ln(1/R) / (2 L h).
void cpml_profile(int n, int L, double h, double v0, double rc, std::vector<double>& d, std::vector<double>& d2) {
    d.assign(n, 0.0);
    d2.assign(n, 0.0);
    if (L <= 0) return;
    const double DP = L * h, d0 = 3.0 * v0 * std::log(1.0 / rc) / (2.0 * DP);
    const double xl = DP, xr = (n - 1) * h - DP;
    for (int i = 0; i < n; i++) {
        const double x = i * h;
        if (i < L) {
            d[i] = d0 * std::pow((xl - x) / DP, 2);
            d2[i] = d0 * std::pow((xl - x - 0.5 * h) / DP, 2);
        } else if (i >= n - 1 - L) {
            d[i] = d0 * std::pow((x - xr) / DP, 2);
            d2[i] = d0 * std::pow((x + 0.5 * h - xr) / DP, 2);
        }
    }
}

double pow2_round(double s) { return std::ldexp(1.0, (int)std::lround(std::log2(s))); }

}  // namespace

namespace behf {
// Error text for entry points defined in other translation units.
void report_error(const char* msg) { g_err = msg; }
}  // namespace behf

struct behf_ctx {
    behf_grid grid{};
    int prec = BEHF_FP32;
    int dev = 0;
    cudaStream_t stream = nullptr;
    Geom g{};
    DevPtrs p{};
    size_t es = 0, ks = 0, ws = 0;
    long long nfield = 0;  // elements per pitched array
    std::vector<std::pair<void*, size_t>> allocs;
    int64_t device_bytes = 0;
    float* d_rho = nullptr;  // cell-centred density kept for the force source
    double scales[4] = {1, 1, 1, 1};
    bool auto_scales = true, medium_set = false;
    // profile overrides
    bool prof_override[3] = {false, false, false};
    std::vector<double> prof_d[3], prof_d2[3];
    // source
    bool src_set = false;
    int src_kind = 0, src_ijk[3] = {0, 0, 0};
    float* d_wavelet = nullptr;
    int nw = 0;
    // receivers
    int nrec = 0, cap = 0;
    long long* d_rec_off = nullptr;
    int* d_rec_comp = nullptr;
    double* d_seis = nullptr;
    // time
    int* d_it = nullptr;
    long long step = 0;
    // graph
    int chunk = 16;
    cudaGraphExec_t gexec = nullptr;
    int kernel_opt = BEHF_KERNEL_AUTO;
    int64_t launches = 0;        // kernels enqueued (host count)
    int64_t graph_nodes = 0;     // kernels per captured graph
    cudaEvent_t* tev = nullptr;  // per-launch events when timing (2 per launch)
    int tev_used = 0;
    std::vector<int> tkind;
    // health scratch
    double* d_part = nullptr;
    int* d_flag = nullptr;
    double* d_norm = nullptr;
    int nblk_health = 0;
    // tiled kernels: TMA descriptors (built once, the arrays never move) and the device error word
    bool tiled_ok = false;
    int tile_rows = 8;    // tiled kernels: rows per tile (8, or 4: kernels_tiled_*_rows4.cu)
    tiled::VMaps* vmaps = nullptr;
    tiled::TMaps* tmaps = nullptr;
    int* d_err = nullptr;
    // gradient support: the cell-centred moduli kept on the device (BEHF_OPT_GRADIENT) and the
    // checkpoint spacing of the gradient's forward pass
    bool keep_medium = false;
    float* d_mod[kNMod] = {};
    int ck_stride = 0;
    int ck_outer = 0;  // gradient: outer checkpoint spacing of the two-level scheme (0 automatic)
    int snap_cache_mib = -1;  // gradient: device memory for snapshots kept from the forward pass (-1 automatic)
    int grad_comp = 1;    // gradient: FP32 accumulators folded per segment (0 plain, 1 Neumaier, 2 FP64 total)
    int rc_overlap = 1;   // gradient: recompute of the next segment on a second stream (one checkpoint level)
    int coef_dither = 0;  // BEHF_OPT_COEF_ROUNDING

    ~behf_ctx() {
        if (gexec) cudaGraphExecDestroy(gexec);
        std::free(vmaps);
        std::free(tmaps);
        for (auto& a : allocs) cudaFree(a.first);
        if (stream) cudaStreamDestroy(stream);
    }
    behf_status dalloc(void** out, size_t bytes) {
        void* ptr = nullptr;
        cudaError_t e = cudaMalloc(&ptr, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(BEHF_ERR_ALLOC, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
        }
        allocs.emplace_back(ptr, bytes);
        device_bytes += (int64_t)bytes;
        *out = ptr;
        return BEHF_OK;
    }
    void dfree(void* ptr) {
        if (!ptr) return;
        for (size_t i = 0; i < allocs.size(); i++)
            if (allocs[i].first == ptr) {
                device_bytes -= (int64_t)allocs[i].second;
                allocs.erase(allocs.begin() + i);
                break;
            }
        cudaFree(ptr);
    }
    void invalidate_graph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
    }
    long long cell_offset(int i, int j, int k) const { return (long long)k * g.plane + (long long)j * g.px + i; }
    double field_scale(int q) const {
        return q <= BEHF_VZ ? scales[0] : q <= BEHF_QZ ? scales[1] : q <= BEHF_SYZ ? scales[2] : scales[3];
    }
};

namespace {

template <class S>
cudaError_t launch_update(behf_ctx* c, bool vel) {
    const bool tiled = c->kernel_opt != BEHF_KERNEL_PLAIN && c->tiled_ok;
    if (tiled) {
        const void* maps = vel ? (const void*)c->vmaps : (const void*)c->tmaps;
        return c->tile_rows == 4 ? launch_tiled_rows4<S>(c->g, c->p, maps, vel, c->stream)
                                 : launch_tiled<S>(c->g, c->p, maps, vel, c->stream);
    }
    return launch_plain<S>(c->g, c->p, vel, c->stream);
}

// The tiled kernels' tensor maps for the context's tile height (the two heights' maps have one layout; their boxes
// differ), allocated on first use.
template <class S>
bool setup_tiled(behf_ctx* c) {
    if (!(c->tile_rows == 4 ? tiled_supported_rows4<S>(c->g) : tiled_supported<S>(c->g))) return false;
    if (!c->vmaps) c->vmaps = static_cast<tiled::VMaps*>(std::aligned_alloc(64, (sizeof(tiled::VMaps) + 63) / 64 * 64));
    if (!c->tmaps) c->tmaps = static_cast<tiled::TMaps*>(std::aligned_alloc(64, (sizeof(tiled::TMaps) + 63) / 64 * 64));
    if (!c->vmaps || !c->tmaps) return false;
    return (c->tile_rows == 4 ? tiled_build_maps_rows4<S>(c->g, c->p, c->vmaps, c->tmaps)
                              : tiled_build_maps<S>(c->g, c->p, c->vmaps, c->tmaps)) == cudaSuccess;
}

bool setup_tiled_any(behf_ctx* c) {
    switch (c->prec) {
        case BEHF_FP32: return setup_tiled<float>(c);
        case BEHF_FP16: return setup_tiled<__half>(c);
        case BEHF_BF16: return setup_tiled<__nv_bfloat16>(c);
    }
    return false;
}

cudaError_t dispatch_update(behf_ctx* c, bool vel) {
    switch (c->prec) {
        case BEHF_FP64: return launch_update<double>(c, vel);
        case BEHF_FP32: return launch_update<float>(c, vel);
        case BEHF_FP16: return launch_update<__half>(c, vel);
        case BEHF_BF16: return launch_update<__nv_bfloat16>(c, vel);
    }
    return cudaErrorInvalidValue;
}

// Source injection factor: storage scale of the injected field, or dt / rho_z * s_v for the force
// (rho_z = arithmetic mean along z, main.cpp:353).  Host copies: call outside graph capture.
cudaError_t source_factor(behf_ctx* c, double* fac) {
    *fac = 0;
    if (!c->src_set) return cudaSuccess;
    if (c->src_kind == BEHF_SRC_EXPLOSIVE) *fac = c->scales[2];
    else if (c->src_kind == BEHF_SRC_PRESSURE) *fac = c->scales[3];
    else {
        const long long N = (long long)c->grid.nx * c->grid.ny;
        const long long o = ((long long)c->src_ijk[2] * c->grid.ny + c->src_ijk[1]) * c->grid.nx + c->src_ijk[0];
        float r0 = 0, r1 = 0;
        cudaError_t e = cudaMemcpy(&r0, c->d_rho + o, 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(&r1, c->d_rho + o + N, 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return e;
        const double rz = 0.5 * ((double)r0 + (double)r1);
        *fac = rz > 0 ? c->grid.dt / rz * c->scales[0] : 0.0;
    }
    return cudaSuccess;
}

// Timing brackets: when c->tev is set, each launch of kind k is bracketed by events 2*i, 2*i+1 and
// its kind recorded in c->tkind.
struct TimedLaunch {
    behf_ctx* c;
    int kind;
    TimedLaunch(behf_ctx* cc, int k) : c(cc), kind(k) {
        if (c->tev) cudaEventRecord(c->tev[2 * c->tev_used], c->stream);
    }
    ~TimedLaunch() {
        if (c->tev) {
            cudaEventRecord(c->tev[2 * c->tev_used + 1], c->stream);
            c->tkind.push_back(kind);
            c->tev_used++;
        }
        c->launches++;
    }
};

template <class S>
cudaError_t enqueue_steps_t(behf_ctx* c, int n, double fac) {
    const long long so = c->src_set ? c->cell_offset(c->src_ijk[0], c->src_ijk[1], c->src_ijk[2]) : 0;
    RecScales rs;
    for (int q = 0; q < kNField; q++) rs.s[q] = c->field_scale(q);
    for (int s = 0; s < n; s++) {
        cudaError_t e;
        if (c->src_set && c->src_kind != BEHF_SRC_FORCE_Z) {
            TimedLaunch t(c, 0);
            e = aux_source<S>(c->p, so, c->src_kind, c->d_wavelet, c->nw, c->d_it, s, fac, c->stream);
            if (e != cudaSuccess) return e;
        }
        c->g.step_off = s;
        {
            TimedLaunch t(c, 1);
            if ((e = dispatch_update(c, true)) != cudaSuccess) return e;
        }
        if (c->src_set && c->src_kind == BEHF_SRC_FORCE_Z) {
            TimedLaunch t(c, 0);
            e = aux_source<S>(c->p, so, c->src_kind, c->d_wavelet, c->nw, c->d_it, s, fac, c->stream);
            if (e != cudaSuccess) return e;
        }
        {
            TimedLaunch t(c, 2);
            if ((e = dispatch_update(c, false)) != cudaSuccess) return e;
        }
        c->g.step_off = 0;
        if (c->nrec > 0) {
            TimedLaunch t(c, 3);
            if ((e = aux_record<S>(c->p, c->d_rec_off, c->d_rec_comp, c->nrec, c->d_seis, c->cap, c->d_it, s, rs,
                                   c->stream)) != cudaSuccess)
                return e;
        }
    }
    c->launches++;
    return aux_tick(c->d_it, n, c->stream);
}

cudaError_t enqueue_steps(behf_ctx* c, int n, double fac) {
    switch (c->prec) {
        case BEHF_FP64: return enqueue_steps_t<double>(c, n, fac);
        case BEHF_FP32: return enqueue_steps_t<float>(c, n, fac);
        case BEHF_FP16: return enqueue_steps_t<__half>(c, n, fac);
        case BEHF_BF16: return enqueue_steps_t<__nv_bfloat16>(c, n, fac);
    }
    return cudaErrorInvalidValue;
}

behf_status upload_profiles(behf_ctx* c) {
    const int n3[3] = {c->grid.nx, c->grid.ny, c->grid.nz};
    const double dt = c->grid.dt;
    for (int a = 0; a < 3; a++) {
        std::vector<double> d, d2;
        if (c->prof_override[a]) {
            d = c->prof_d[a];
            d2 = c->prof_d2[a];
        } else {
            cpml_profile(n3[a], c->grid.cpml_width, c->grid.h, c->grid.cpml_v0, c->grid.cpml_r, d, d2);
        }
        const int n = n3[a];
        std::vector<double> A(n), B(n), A2(n), B2(n);
        for (int i = 0; i < n; i++) {
            // e = exp(-d dt) where the profile is active, 0 elsewhere (the reference's calloc'd e_d*)
            const bool on = c->g.W > 0 && slab_index(i, n, c->g.L) >= 0;
            A[i] = on ? std::exp(-d[i] * dt) : 0.0;
            B[i] = on ? -dt * d[i] * 0.5 : 0.0;
            A2[i] = on ? std::exp(-d2[i] * dt) : 0.0;
            B2[i] = on ? -dt * d2[i] * 0.5 : 0.0;
        }
        const std::vector<double>* src[4] = {&A, &B, &A2, &B2};
        void* dst[4] = {c->p.pa[a], c->p.pb[a], c->p.pa2[a], c->p.pb2[a]};
        for (int t = 0; t < 4; t++) {
            if (c->ws == 8) {
                CK(cudaMemcpy(dst[t], src[t]->data(), n * 8, cudaMemcpyHostToDevice));
            } else {
                std::vector<float> f(n);
                for (int i = 0; i < n; i++) f[i] = (float)(*src[t])[i];
                CK(cudaMemcpy(dst[t], f.data(), n * 4, cudaMemcpyHostToDevice));
            }
        }
    }
    return BEHF_OK;
}

behf_status zero_state(behf_ctx* c) {
    for (int q = 0; q < kNField; q++) CK(cudaMemsetAsync(c->p.f[q], 0, c->nfield * c->es, c->stream));
    if (c->g.W > 0) {
        const size_t sl[3] = {(size_t)c->grid.nz * c->grid.ny * c->g.W, (size_t)c->grid.nz * c->g.W * c->grid.nx,
                              (size_t)c->g.W * c->grid.ny * c->grid.nx};
        for (int a = 0; a < 3; a++)
            for (int s = 0; s < 8; s++) {
                CK(cudaMemsetAsync(c->p.psi[a][s], 0, sl[a] * c->ws, c->stream));
                CK(cudaMemsetAsync(c->p.prv[a][s], 0, sl[a] * c->ws, c->stream));
            }
    }
    if (c->d_seis) CK(cudaMemsetAsync(c->d_seis, 0, (size_t)c->nrec * c->cap * 8, c->stream));
    CK(cudaMemsetAsync(c->d_it, 0, sizeof(int), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->step = 0;
    return BEHF_OK;
}

template <class S>
behf_status build_coefs(behf_ctx* c, const float* const mod[kNMod]) {
    CoefArgs a{};
    for (int q = 0; q < kNMod; q++) a.mod[q] = mod[q];
    a.nx = c->grid.nx;
    a.ny = c->grid.ny;
    a.nz = c->grid.nz;
    a.px = c->g.px;
    a.plane = c->g.plane;
    a.dt = c->grid.dt;
    a.dither = c->coef_dither;
    const double sv = c->scales[0], sq = c->scales[1], ss = c->scales[2], sp = c->scales[3];
    const double hi = 1.0 / c->grid.h;
    for (int d = 0; d < 3; d++) {
        a.ratio[VW1X + d] = 1.0;
        a.ratio[VW2X + d] = sq / ss * hi;
        a.ratio[VW3X + d] = sq / sp * hi;
        a.ratio[VU1X + d] = sv / ss * hi;
        a.ratio[VU2X + d] = sv / sq;
    }
    a.ratio[P1] = sp / sv * hi;
    a.ratio[P2] = sp / sq * hi;
    a.ratio[S1] = a.ratio[S2] = ss / sv * hi;
    a.ratio[S3] = ss / sq * hi;
    a.ratio[SXYC] = a.ratio[SXZC] = a.ratio[SYZC] = ss / sv * hi;
    for (int q = 0; q < kNCoef; q++) {
        a.inv[q] = 1.0;
        a.out[q] = c->p.k[q];
    }
    unsigned long long* d_max = nullptr;
    behf_status st = c->dalloc((void**)&d_max, kNCoef * 8);
    if (st) return st;
    CK(cudaMemsetAsync(d_max, 0, kNCoef * 8, c->stream));
    a.maxbits = d_max;
    const bool pow2 = (c->prec == BEHF_FP16 || c->prec == BEHF_BF16);
    if (pow2) {
        a.pass = 0;
        CK(aux_build_coefs<S>(a, c->stream));
        unsigned long long mb[kNCoef];
        CK(cudaMemcpyAsync(mb, d_max, sizeof mb, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        for (int q = 3; q < kNCoef; q++) {
            double mx;
            std::memcpy(&mx, &mb[q], 8);
            int e = 0;
            if (mx > 0) std::frexp(mx, &e);  // mx = f 2^e, f in [0.5, 1)
            a.inv[q] = std::ldexp(1.0, -e);
            c->g.kmuld[q] = std::ldexp(1.0, e);
            c->g.kmulf[q] = (float)c->g.kmuld[q];
        }
    } else {
        for (int q = 0; q < kNCoef; q++) {
            c->g.kmuld[q] = 1.0;
            c->g.kmulf[q] = 1.0f;
        }
    }
    c->g.c_vw2 = (float)(sp * sq / (sv * ss));
    c->g.c_s3 = (float)(ss * sv / (sp * sq));
    a.pass = 1;
    CK(aux_build_coefs<S>(a, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->dfree(d_max);
    return BEHF_OK;
}

behf_status set_medium_dev(behf_ctx* c, const float* const mod[kNMod]) {
    const long long N = (long long)c->grid.nx * c->grid.ny * c->grid.nz;
    if (c->auto_scales) {
        unsigned long long* d_st = nullptr;
        behf_status st = c->dalloc((void**)&d_st, 3 * 8);
        if (st) return st;
        const double big = 1.7976931348623157e308;
        unsigned long long init[3] = {0, 0, 0};
        std::memcpy(&init[2], &big, 8);
        CK(cudaMemcpyAsync(d_st, init, sizeof init, cudaMemcpyHostToDevice, c->stream));
        CK(aux_med_stats(mod[BEHF_RHO], mod[BEHF_HH], mod[BEHF_C1], N, d_st, c->stream));
        unsigned long long r[3];
        CK(cudaMemcpyAsync(r, d_st, sizeof r, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->dfree(d_st);
        double zmax, rmax, bmin;
        std::memcpy(&zmax, &r[0], 8);
        std::memcpy(&rmax, &r[1], 8);
        std::memcpy(&bmin, &r[2], 8);
        const double amp = c->grid.src_amp_hint > 0 ? c->grid.src_amp_hint : 1.0;
        const double f0 = c->grid.src_f0_hint > 0 ? c->grid.src_f0_hint : 30.0;
        // the wavelet peak lands at 2^4 in storage units: fields near the source stay far below the FP16 maximum
        // (measured: 2^11 saturates an explosive source) while the far field moves up out of the subnormals
        const double ss = 16.0 / amp;
        const double sv = ss * (zmax > 0 ? zmax : 1.0);
        double kq = (bmin < big && rmax > 0) ? bmin / (rmax * 2.0 * M_PI * f0) : 1.0;
        kq = std::fmin(std::fmax(kq, 1.0), 1e6);
        c->scales[0] = pow2_round(sv);
        c->scales[1] = pow2_round(sv * kq);
        c->scales[2] = pow2_round(ss);
        c->scales[3] = pow2_round(ss);
    }
    CK(cudaMemcpyAsync(c->d_rho, mod[BEHF_RHO], N * 4, cudaMemcpyDeviceToDevice, c->stream));
    if (c->keep_medium) {
        for (int q = 0; q < kNMod; q++) {
            if (!c->d_mod[q]) {
                behf_status sa = c->dalloc((void**)&c->d_mod[q], (size_t)N * 4);
                if (sa) return sa;
            }
            CK(cudaMemcpyAsync(c->d_mod[q], mod[q], N * 4, cudaMemcpyDeviceToDevice, c->stream));
        }
    }
    behf_status st = BEHF_OK;
    switch (c->prec) {
        case BEHF_FP64: st = build_coefs<double>(c, mod); break;
        case BEHF_FP32: st = build_coefs<float>(c, mod); break;
        case BEHF_FP16: st = build_coefs<__half>(c, mod); break;
        case BEHF_BF16: st = build_coefs<__nv_bfloat16>(c, mod); break;
    }
    if (st) return st;
    c->medium_set = true;
    c->invalidate_graph();
    return BEHF_OK;
}

}  // namespace

extern "C" {

const char* behf_last_error(void) { return g_err.c_str(); }
const char* behf_version(void) { return "behf-gb300 0.1 (sm_103a)"; }

behf_status behf_create(const behf_grid* gr, int precision, behf_ctx** out) {
    if (!gr || !out) return fail(BEHF_ERR_INVALID, "null argument");
    *out = nullptr;
    if (precision < BEHF_FP64 || precision > BEHF_BF16) return fail(BEHF_ERR_INVALID, "bad precision %d", precision);
    const int R = gr->radius, L = gr->cpml_width;
    if (R < 1 || R > 4) return fail(BEHF_ERR_INVALID, "radius %d not in 1..4", R);
    if (!(gr->h > 0) || !(gr->dt > 0)) return fail(BEHF_ERR_INVALID, "h and dt must be positive");
    const int n3[3] = {gr->nx, gr->ny, gr->nz};
    for (int a = 0; a < 3; a++) {
        if (n3[a] < 2 * R + 1) return fail(BEHF_ERR_INVALID, "axis %d: %d cells < 2R+1", a, n3[a]);
        if (L < 0 || (L > 0 && n3[a] < 2 * L + 2))
            return fail(BEHF_ERR_INVALID, "axis %d: %d cells too small for CPML width %d", a, n3[a], L);
    }
    if (L > 0 && (!(gr->cpml_v0 > 0) || !(gr->cpml_r > 0 && gr->cpml_r < 1)))
        return fail(BEHF_ERR_INVALID, "CPML needs v0 > 0 and 0 < r < 1");
    auto* c = new (std::nothrow) behf_ctx();
    if (!c) return fail(BEHF_ERR_ALLOC, "host allocation failed");
    c->grid = *gr;
    c->prec = precision;
    cudaGetDevice(&c->dev);
    c->es = elem_size(precision);
    c->ks = kelem_size(precision);
    c->ws = welem_size(precision);
    Geom& g = c->g;
    g.nx = gr->nx;
    g.ny = gr->ny;
    g.nz = gr->nz;
    g.R = R;
    g.L = L;
    g.W = L > 0 ? (2 * L + 1 + 3) / 4 * 4 : 0;  // slab row pitch: 2L+1 cells rounded up to 16 bytes of FP32
    // the tensor-memory kernels' TMA box of x-slab memory: an edge tile's slab cells (at most L + 1, at most a tile
    // row of 64) plus up to 3 cells of alignment
    g.xs_bw = L > 0 ? std::min(64, (std::min(L + 1, 64) + 3 + 3) / 4 * 4) : 0;
    g.slab_pf = L > 0 && gr->nx % 4 == 0 ? 1 : 0;
    g.px = ((long long)gr->nx + 15) / 16 * 16;
    g.plane = g.px * gr->ny;
    g.bug = 0;
    g.zchunk_req = 0;
    g.ws = auto_variant(precision);
    g.sr = 0;
    g.step = nullptr;
    g.step_off = 0;
    c->nfield = g.plane * gr->nz;
    bool all0 = true;
    for (int s = 0; s < 4; s++) all0 = all0 && gr->scales[s] == 0;
    c->auto_scales = all0;
    if (!all0) {
        for (int s = 0; s < 4; s++) {
            if (!(gr->scales[s] > 0)) {
                delete c;
                return fail(BEHF_ERR_INVALID, "scales must be all positive or all zero");
            }
            c->scales[s] = gr->scales[s];
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return fail(BEHF_ERR_CUDA, "stream creation failed: %s", cudaGetErrorString(e));
    }
    behf_status st = BEHF_OK;
    auto A = [&](void** ptr, size_t bytes) {
        if (st == BEHF_OK) st = c->dalloc(ptr, align256(bytes));
    };
    for (int q = 0; q < kNField; q++) A(&c->p.f[q], c->nfield * c->es);
    for (int q = 0; q < kNCoef; q++) A(&c->p.k[q], c->nfield * (q < 3 ? c->ws : c->ks));
    if (g.W > 0) {
        const size_t sl[3] = {(size_t)gr->nz * gr->ny * g.W, (size_t)gr->nz * g.W * gr->nx,
                              (size_t)g.W * gr->ny * gr->nx};
        for (int a = 0; a < 3; a++)
            for (int s = 0; s < 8; s++) {
                A(&c->p.psi[a][s], sl[a] * c->ws);
                A(&c->p.prv[a][s], sl[a] * c->ws);
            }
    }
    for (int a = 0; a < 3; a++) {
        A(&c->p.pa[a], n3[a] * c->ws);
        A(&c->p.pb[a], n3[a] * c->ws);
        A(&c->p.pa2[a], n3[a] * c->ws);
        A(&c->p.pb2[a], n3[a] * c->ws);
    }
    A((void**)&c->d_rho, (size_t)gr->nx * gr->ny * gr->nz * 4);
    A((void**)&c->d_it, sizeof(int));
    c->nblk_health = aux_grid_blocks();
    A((void**)&c->d_part, (size_t)c->nblk_health * 8);
    A((void**)&c->d_flag, sizeof(int));
    A((void**)&c->d_norm, kNField * 8);
    A((void**)&c->d_err, sizeof(int));
    if (st) {
        delete c;
        return st;
    }
    for (int q = 0; q < kNCoef; q++) {
        if (cudaMemsetAsync(c->p.k[q], 0, c->nfield * (q < 3 ? c->ws : c->ks), c->stream) != cudaSuccess) st = BEHF_ERR_CUDA;
        g.kmuld[q] = 1.0;
        g.kmulf[q] = 1.0f;
    }
    if (st == BEHF_OK && cudaMemset(c->d_err, 0, sizeof(int)) != cudaSuccess) st = BEHF_ERR_CUDA;
    g.err = c->d_err;
    g.step = c->d_it;
    if (st == BEHF_OK) st = upload_profiles(c);
    if (st == BEHF_OK) st = zero_state(c);
    if (st == BEHF_OK) c->tiled_ok = setup_tiled_any(c);
    if (st) {
        delete c;
        return st == BEHF_ERR_CUDA && g_err.empty() ? fail(st, "initialisation failed") : st;
    }
    *out = c;
    return BEHF_OK;
}

behf_status behf_destroy(behf_ctx* c) {
    if (!c) return BEHF_OK;
    DeviceScope device_scope(c->dev);
    cudaStreamSynchronize(c->stream);
    delete c;
    return BEHF_OK;
}

behf_status behf_set_medium_device(behf_ctx* c, const float* const mod[BEHF_NMOD]) {
    if (!c || !mod) return fail(BEHF_ERR_INVALID, "null argument");
    DeviceScope device_scope(c->dev);
    for (int q = 0; q < kNMod; q++)
        if (!mod[q]) return fail(BEHF_ERR_INVALID, "modulus array %d is null", q);
    return set_medium_dev(c, mod);
}

behf_status behf_set_medium(behf_ctx* c, const float* const mod[BEHF_NMOD]) {
    if (!c || !mod) return fail(BEHF_ERR_INVALID, "null argument");
    DeviceScope device_scope(c->dev);
    const size_t N = (size_t)c->grid.nx * c->grid.ny * c->grid.nz;
    float* dm[kNMod] = {};
    behf_status st = BEHF_OK;
    for (int q = 0; q < kNMod && st == BEHF_OK; q++) {
        if (!mod[q]) st = fail(BEHF_ERR_INVALID, "modulus array %d is null", q);
        else st = c->dalloc((void**)&dm[q], N * 4);
        if (st == BEHF_OK) {
            cudaError_t e = cudaMemcpyAsync(dm[q], mod[q], N * 4, cudaMemcpyHostToDevice, c->stream);
            if (e != cudaSuccess) st = fail(BEHF_ERR_CUDA, "medium upload: %s", cudaGetErrorString(e));
        }
    }
    if (st == BEHF_OK) st = set_medium_dev(c, dm);
    cudaStreamSynchronize(c->stream);
    for (int q = 0; q < kNMod; q++)
        if (dm[q]) c->dfree(dm[q]);
    return st;
}

behf_status behf_generate_medium(behf_ctx* c, const behf_medium_spec* spec) {
    if (!c || !spec) return fail(BEHF_ERR_INVALID, "null argument");
    DeviceScope device_scope(c->dev);
    if (spec->nlayers < 1 || spec->nlayers > 4) return fail(BEHF_ERR_INVALID, "nlayers must be 1..4");
    const bool noise = spec->pct != 0 || spec->log_kappa_sigma != 0;
    if (noise && !(spec->corr_cells > 0)) return fail(BEHF_ERR_INVALID, "corr_cells must be positive");
    if (spec->seed < 0 || spec->seed >= (1 << 20)) return fail(BEHF_ERR_INVALID, "seed must be in [0, 2^20)");
    const long long N = (long long)c->grid.nx * c->grid.ny * c->grid.nz;
    float* dm[kNMod] = {};
    float* work = nullptr;
    behf_status st = BEHF_OK;
    for (int q = 0; q < kNMod && st == BEHF_OK; q++) st = c->dalloc((void**)&dm[q], (size_t)N * 4);
    if (st == BEHF_OK && noise) st = c->dalloc((void**)&work, (size_t)N * 4 * 5);
    if (st == BEHF_OK) {
        cudaError_t e = generate_medium(*spec, c->grid.nx, c->grid.ny, c->grid.nz, dm, work, c->stream,
                                        aux_grid_blocks());
        if (e != cudaSuccess) st = fail(BEHF_ERR_CUDA, "medium generation failed: %s", cudaGetErrorString(e));
    }
    if (work) c->dfree(work);
    if (st == BEHF_OK) st = set_medium_dev(c, dm);
    cudaStreamSynchronize(c->stream);
    for (int q = 0; q < kNMod; q++) c->dfree(dm[q]);
    return st;
}

behf_status behf_set_cpml_profile(behf_ctx* c, int axis, const double* d, const double* d2) {
    if (!c || axis < 0 || axis > 2 || !d || !d2) return fail(BEHF_ERR_INVALID, "bad argument");
    DeviceScope device_scope(c->dev);
    const int n = axis == 0 ? c->grid.nx : axis == 1 ? c->grid.ny : c->grid.nz;
    c->prof_d[axis].assign(d, d + n);
    c->prof_d2[axis].assign(d2, d2 + n);
    c->prof_override[axis] = true;
    return upload_profiles(c);
}

behf_status behf_set_source(behf_ctx* c, int kind, int ix, int iy, int iz, const float* w, int nt) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    if (kind < BEHF_SRC_EXPLOSIVE || kind > BEHF_SRC_FORCE_Z) return fail(BEHF_ERR_INVALID, "bad source kind %d", kind);
    const int R = c->g.R;
    const int ijk[3] = {ix, iy, iz}, n3[3] = {c->grid.nx, c->grid.ny, c->grid.nz};
    for (int a = 0; a < 3; a++)
        if (ijk[a] < R || ijk[a] >= n3[a] - R)
            return fail(BEHF_ERR_INVALID, "source axis %d index %d outside the updated cells [%d,%d)", a, ijk[a], R,
                        n3[a] - R);
    if (nt < 0 || (nt > 0 && !w)) return fail(BEHF_ERR_INVALID, "bad wavelet");
    if (c->d_wavelet) {
        c->dfree(c->d_wavelet);
        c->d_wavelet = nullptr;
    }
    behf_status st = c->dalloc((void**)&c->d_wavelet, align256((size_t)(nt > 0 ? nt : 1) * 4));
    if (st) return st;
    if (nt > 0) CK(cudaMemcpy(c->d_wavelet, w, (size_t)nt * 4, cudaMemcpyHostToDevice));
    c->nw = nt;
    c->src_kind = kind;
    for (int a = 0; a < 3; a++) c->src_ijk[a] = ijk[a];
    c->src_set = true;
    c->invalidate_graph();
    return BEHF_OK;
}

behf_status behf_set_receivers(behf_ctx* c, int nrec, const int* ijk, const int* comp, int capacity) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    if (nrec < 0 || capacity < 0 || (nrec > 0 && (!ijk || !comp)))
        return fail(BEHF_ERR_INVALID, "bad receiver arguments");
    std::vector<long long> off(nrec);
    const int n3[3] = {c->grid.nx, c->grid.ny, c->grid.nz};
    for (int r = 0; r < nrec; r++) {
        for (int a = 0; a < 3; a++)
            if (ijk[3 * r + a] < 0 || ijk[3 * r + a] >= n3[a])
                return fail(BEHF_ERR_INVALID, "receiver %d axis %d index %d out of the grid", r, a, ijk[3 * r + a]);
        if (comp[r] < 0 || comp[r] >= kNField) return fail(BEHF_ERR_INVALID, "receiver %d: bad field %d", r, comp[r]);
        off[r] = c->cell_offset(ijk[3 * r], ijk[3 * r + 1], ijk[3 * r + 2]);
    }
    c->dfree(c->d_rec_off);
    c->dfree(c->d_rec_comp);
    c->dfree(c->d_seis);
    c->d_rec_off = nullptr;
    c->d_rec_comp = nullptr;
    c->d_seis = nullptr;
    c->nrec = 0;
    c->cap = 0;
    if (nrec > 0) {
        behf_status st = c->dalloc((void**)&c->d_rec_off, align256((size_t)nrec * 8));
        if (!st) st = c->dalloc((void**)&c->d_rec_comp, align256((size_t)nrec * 4));
        if (!st) st = c->dalloc((void**)&c->d_seis, align256((size_t)nrec * (capacity > 0 ? capacity : 1) * 8));
        if (st) return st;
        CK(cudaMemcpy(c->d_rec_off, off.data(), (size_t)nrec * 8, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_rec_comp, comp, (size_t)nrec * 4, cudaMemcpyHostToDevice));
        CK(cudaMemset(c->d_seis, 0, (size_t)nrec * (capacity > 0 ? capacity : 1) * 8));
        c->nrec = nrec;
        c->cap = capacity;
    }
    c->invalidate_graph();
    return BEHF_OK;
}

behf_status behf_run_async(behf_ctx* c, int nsteps) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    if (!c->medium_set) return fail(BEHF_ERR_STATE, "behf_set_medium must come before behf_run");
    if (nsteps < 0) return fail(BEHF_ERR_INVALID, "negative step count");
    if (c->nrec > 0 && c->step + nsteps > c->cap)
        return fail(BEHF_ERR_INVALID, "receiver capacity %d exceeded (step %lld + %d)", c->cap, c->step, nsteps);
    int left = nsteps;
    double fac = 0;
    CK(source_factor(c, &fac));
    if (c->chunk > 0 && left >= c->chunk) {
        if (!c->gexec) {
            cudaGraph_t graph = nullptr;
            CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            const int64_t l0 = c->launches;
            cudaError_t e = enqueue_steps(c, c->chunk, fac);
            c->graph_nodes = c->launches - l0;
            c->launches = l0;
            cudaError_t e2 = cudaStreamEndCapture(c->stream, &graph);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                return fail(BEHF_ERR_CUDA, "graph capture failed: %s",
                            cudaGetErrorString(e != cudaSuccess ? e : e2));
            }
            e = cudaGraphInstantiate(&c->gexec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                c->gexec = nullptr;
                return fail(BEHF_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
            }
        }
        while (left >= c->chunk) {
            CK(cudaGraphLaunch(c->gexec, c->stream));
            c->launches += c->graph_nodes;
            left -= c->chunk;
        }
    }
    if (left > 0) CK(enqueue_steps(c, left, fac));
    c->step += nsteps;
    return BEHF_OK;
}

behf_status behf_checkpoint_plan(int nt, int checkpoint, int checkpoint_outer, size_t ck_bytes, size_t snap_bytes,
                                 size_t fixed_bytes, size_t avail, int* inner, int* outer, size_t* bytes) {
    if (nt < 1 || checkpoint < 0 || checkpoint_outer < 0 || !inner || !outer)
        return fail(BEHF_ERR_INVALID, "bad checkpoint plan arguments");
    // memory of inner spacing s2 under outer spacing s1 (s1 == s2: one level)
    auto need = [&](int s2, int s1) -> size_t {
        const size_t nout = (size_t)(nt + s1 - 1) / s1, nin = s1 > s2 ? (size_t)(s1 + s2 - 1) / s2 : 0;
        return (nout + nin) * ck_bytes + (size_t)(s2 + 1) * snap_bytes + fixed_bytes;
    };
    int S = checkpoint > 0 ? checkpoint : std::max(1, (int)std::lround(std::sqrt((double)nt)));
    S = std::min(S, nt);
    int So = S;
    if (checkpoint_outer > 0) {
        So = (std::max(checkpoint_outer, S) + S - 1) / S * S;
    } else if (need(S, S) > avail) {
        // two levels: the inner spacing halves (unless BEHF_OPT_CHECKPOINT fixes it) until, for the outer spacing
        // k S that needs the least memory, the scheme fits
        for (int s2 = S; s2 >= 1; s2 = checkpoint > 0 ? 0 : s2 / 2) {
            size_t best = 0;
            int bs1 = s2;
            for (long long k = 2; k * s2 < 2LL * nt; k++) {
                const size_t n = need(s2, (int)(k * s2));
                if (!best || n < best) {
                    best = n;
                    bs1 = (int)(k * s2);
                }
            }
            if (best && best <= avail) {
                S = s2;
                So = bs1;
                break;
            }
        }
        // nothing fits: one level, whose allocation reports the shortfall
    }
    *inner = S;
    *outer = So;
    if (bytes) *bytes = need(S, So);
    return BEHF_OK;
}

behf_status behf_sync(behf_ctx* c) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    CK(cudaStreamSynchronize(c->stream));
    int err = 0;
    CK(cudaMemcpy(&err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        cudaMemset(c->d_err, 0, sizeof(int));
        return fail(BEHF_ERR_TIMEOUT, "a tiled kernel's pipeline wait timed out; the step's results are invalid");
    }
    return BEHF_OK;
}

behf_status behf_run(behf_ctx* c, int nsteps) {
    behf_status st = behf_run_async(c, nsteps);
    if (st) return st;
    return behf_sync(c);
}

behf_status behf_get_seismograms(behf_ctx* c, double* out, int* nrec_steps) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    const int ns = (int)(c->step < c->cap ? c->step : c->cap);
    if (nrec_steps) *nrec_steps = ns;
    if (!out || c->nrec == 0) return BEHF_OK;
    CK(cudaStreamSynchronize(c->stream));
    if (ns == c->cap) {
        CK(cudaMemcpy(out, c->d_seis, (size_t)c->nrec * c->cap * 8, cudaMemcpyDeviceToHost));
    } else if (ns > 0) {
        CK(cudaMemcpy2D(out, (size_t)ns * 8, c->d_seis, (size_t)c->cap * 8, (size_t)ns * 8, c->nrec,
                        cudaMemcpyDeviceToHost));
    }
    return BEHF_OK;
}

static behf_status field_io(behf_ctx* c, int q, float* host, bool get) {
    if (!c || !host) return fail(BEHF_ERR_INVALID, "null argument");
    DeviceScope device_scope(c->dev);
    if (q < 0 || q >= kNField) return fail(BEHF_ERR_INVALID, "bad field %d", q);
    const size_t N = (size_t)c->grid.nx * c->grid.ny * c->grid.nz;
    float* tmp = nullptr;
    behf_status st = c->dalloc((void**)&tmp, N * 4);
    if (st) return st;
    cudaError_t e = cudaSuccess;
    const double sc = c->field_scale(q);
    const Geom& g = c->g;
    if (!get) e = cudaMemcpyAsync(tmp, host, N * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        switch (c->prec) {
            case BEHF_FP64: e = get ? aux_get<double>(c->p.f[q], tmp, g.nx, g.ny, g.nz, g.px, g.plane, sc, c->stream)
                                    : aux_set<double>(c->p.f[q], tmp, g.nx, g.ny, g.nz, g.px, g.plane, sc, c->stream); break;
            case BEHF_FP32: e = get ? aux_get<float>(c->p.f[q], tmp, g.nx, g.ny, g.nz, g.px, g.plane, sc, c->stream)
                                    : aux_set<float>(c->p.f[q], tmp, g.nx, g.ny, g.nz, g.px, g.plane, sc, c->stream); break;
            case BEHF_FP16: e = get ? aux_get<__half>(c->p.f[q], tmp, g.nx, g.ny, g.nz, g.px, g.plane, sc, c->stream)
                                    : aux_set<__half>(c->p.f[q], tmp, g.nx, g.ny, g.nz, g.px, g.plane, sc, c->stream); break;
            default: e = get ? aux_get<__nv_bfloat16>(c->p.f[q], tmp, g.nx, g.ny, g.nz, g.px, g.plane, sc, c->stream)
                             : aux_set<__nv_bfloat16>(c->p.f[q], tmp, g.nx, g.ny, g.nz, g.px, g.plane, sc, c->stream);
        }
    }
    if (e == cudaSuccess && get) e = cudaMemcpyAsync(host, tmp, N * 4, cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e2 = cudaStreamSynchronize(c->stream);
    c->dfree(tmp);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return fail(BEHF_ERR_CUDA, "field transfer failed: %s", cudaGetErrorString(e));
    return BEHF_OK;
}

behf_status behf_get_field(behf_ctx* c, int q, float* out) { return field_io(c, q, out, true); }
behf_status behf_set_field(behf_ctx* c, int q, const float* in) { return field_io(c, q, const_cast<float*>(in), false); }

behf_status behf_reset(behf_ctx* c) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    return zero_state(c);
}

behf_status behf_set_option(behf_ctx* c, int opt, int value) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    switch (opt) {
        case BEHF_OPT_KERNEL:
            if (value < BEHF_KERNEL_AUTO || value > BEHF_KERNEL_TILED) return fail(BEHF_ERR_INVALID, "bad kernel %d", value);
            if (value == BEHF_KERNEL_TILED && !c->tiled_ok)
                return fail(BEHF_ERR_UNSUPPORTED, "tiled kernel not available for this precision/radius/grid");
            c->kernel_opt = value;
            break;
        case BEHF_OPT_REF_BUG_COMPAT: c->g.bug = value ? 1 : 0; break;
        case BEHF_OPT_GRAPH_CHUNK:
            if (value < 0) return fail(BEHF_ERR_INVALID, "negative chunk");
            c->chunk = value;
            break;
        case BEHF_OPT_GRADIENT:
            if (c->medium_set && value && !c->d_mod[0])
                return fail(BEHF_ERR_STATE, "BEHF_OPT_GRADIENT must be set before the medium");
            c->keep_medium = value != 0;
            break;
        case BEHF_OPT_CHECKPOINT:
            if (value < 0) return fail(BEHF_ERR_INVALID, "negative checkpoint spacing");
            c->ck_stride = value;
            break;
        case BEHF_OPT_CHECKPOINT_OUTER:
            if (value < 0) return fail(BEHF_ERR_INVALID, "negative outer checkpoint spacing");
            c->ck_outer = value;
            break;
        case BEHF_OPT_SNAPSHOT_CACHE:
            if (value < -1) return fail(BEHF_ERR_INVALID, "snapshot cache must be -1 (automatic), 0 or a size in MiB");
            c->snap_cache_mib = value;
            break;
        case BEHF_OPT_COEF_ROUNDING:
            if (value < 0 || value > 1) return fail(BEHF_ERR_INVALID, "coefficient rounding must be 0 or 1");
            if (c->medium_set) return fail(BEHF_ERR_STATE, "BEHF_OPT_COEF_ROUNDING must be set before the medium");
            c->coef_dither = value;
            break;
        case BEHF_OPT_STATE_ROUNDING:
            if (value < 0 || value > 1) return fail(BEHF_ERR_INVALID, "state rounding must be 0 or 1");
            c->g.sr = (c->prec == BEHF_FP16 || c->prec == BEHF_BF16) ? value : 0;
            break;
        case BEHF_OPT_ZCHUNK:
            if (value < 0) return fail(BEHF_ERR_INVALID, "negative z chunk");
            c->g.zchunk_req = value;
            break;
        case BEHF_OPT_GRAD_COMPENSATION:
            if (value < 0 || value > 2) return fail(BEHF_ERR_INVALID, "gradient compensation must be 0, 1 or 2");
            c->grad_comp = value;
            break;
        case BEHF_OPT_RECOMPUTE_OVERLAP:
            if (value < 0 || value > 1) return fail(BEHF_ERR_INVALID, "recompute overlap must be 0 or 1");
            c->rc_overlap = value;
            break;
        case BEHF_OPT_TILE_ROWS: {
            const int rows = value == 0 ? 8 : value;
            if (rows != 4 && rows != 8) return fail(BEHF_ERR_INVALID, "tile rows must be 0 (automatic), 4 or 8");
            if (rows != c->tile_rows) {
                const int old = c->tile_rows;
                c->tile_rows = rows;
                if (c->tiled_ok && !setup_tiled_any(c)) {  // keep the previous height if the new one cannot run
                    c->tile_rows = old;
                    setup_tiled_any(c);
                    return fail(BEHF_ERR_INVALID, "%d-row tiles are not supported on this grid", rows);
                }
            }
            break;
        }
        case BEHF_OPT_TILED_VARIANT:
            if (value < 0 || value > 4) return fail(BEHF_ERR_INVALID, "tiled variant must be 0 .. 4");
            c->g.ws = value == 0 ? auto_variant(c->prec) : value - 1;
            break;
        default: return fail(BEHF_ERR_INVALID, "unknown option %d", opt);
    }
    c->invalidate_graph();
    return BEHF_OK;
}

behf_status behf_get_info(behf_ctx* c, behf_info* out) {
    if (!c || !out) return fail(BEHF_ERR_INVALID, "null argument");
    out->step = c->step;
    out->device_bytes = c->device_bytes;
    for (int s = 0; s < 4; s++) out->scales[s] = c->scales[s];
    // algorithmic bytes per cell update: 13 fields read + written, 23 coefficients read, CPML memory
    // (8 derivatives x {psi, prev} x read+write) on the slab fraction of each axis
    const double n3[3] = {(double)c->grid.nx, (double)c->grid.ny, (double)c->grid.nz};
    double cpml = 0;
    for (int a = 0; a < 3; a++) cpml += c->g.W > 0 ? 16.0 * 2.0 * c->ws * (2 * c->g.L + 1) / n3[a] : 0.0;
    out->bytes_per_cell = 26.0 * c->es + 3.0 * c->ws + 20.0 * c->ks + cpml;
    out->kernel = (c->kernel_opt != BEHF_KERNEL_PLAIN && c->tiled_ok) ? BEHF_KERNEL_TILED : BEHF_KERNEL_PLAIN;
    out->radius = c->g.R;
    out->precision = c->prec;
    out->launches = c->launches;
    out->tiled_variant = c->g.ws + 1;
    out->zchunk = c->g.zchunk_req;
    out->tile_rows = c->tile_rows;
    return BEHF_OK;
}

behf_status behf_update_wavelet(behf_ctx* c, int it0, const float* w, int n) {
    if (!c || (n > 0 && !w) || it0 < 0 || n < 0) return fail(BEHF_ERR_INVALID, "bad argument");
    DeviceScope device_scope(c->dev);
    if (!c->src_set) return fail(BEHF_ERR_STATE, "behf_set_source must come first");
    if (it0 + n > c->nw) {  // grow, keeping the old samples
        float* nw = nullptr;
        behf_status st = c->dalloc((void**)&nw, align256((size_t)(it0 + n) * 4));
        if (st) return st;
        CK(cudaMemsetAsync(nw, 0, (size_t)(it0 + n) * 4, c->stream));
        if (c->nw > 0) CK(cudaMemcpyAsync(nw, c->d_wavelet, (size_t)c->nw * 4, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->dfree(c->d_wavelet);
        c->d_wavelet = nw;
        c->nw = it0 + n;
        c->invalidate_graph();
    }
    if (n > 0) CK(cudaMemcpyAsync(c->d_wavelet + it0, w, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    return BEHF_OK;
}

behf_status behf_get_seismograms_range(behf_ctx* c, int it0, int n, double* out) {
    if (!c || n < 0 || it0 < 0 || (n > 0 && !out)) return fail(BEHF_ERR_INVALID, "bad argument");
    DeviceScope device_scope(c->dev);
    if (it0 + n > c->cap) return fail(BEHF_ERR_INVALID, "range beyond the receiver capacity %d", c->cap);
    if (c->nrec == 0 || n == 0) return BEHF_OK;
    CK(cudaMemcpy2DAsync(out, (size_t)n * 8, c->d_seis + it0, (size_t)c->cap * 8, (size_t)n * 8, c->nrec,
                         cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return BEHF_OK;
}

behf_status behf_time_kernels(behf_ctx* c, int nsteps, double* ms) {
    if (!c || !ms || nsteps <= 0) return fail(BEHF_ERR_INVALID, "bad argument");
    DeviceScope device_scope(c->dev);
    if (!c->medium_set) return fail(BEHF_ERR_STATE, "behf_set_medium must come before timing");
    if (c->nrec > 0 && c->step + nsteps > c->cap) return fail(BEHF_ERR_INVALID, "receiver capacity exceeded");
    const int maxl = 4 * nsteps;
    std::vector<cudaEvent_t> ev(2 * maxl);
    for (auto& e : ev) CK(cudaEventCreate(&e));
    double fac = 0;
    CK(source_factor(c, &fac));
    c->tev = ev.data();
    c->tev_used = 0;
    c->tkind.clear();
    cudaError_t e = enqueue_steps(c, nsteps, fac);
    c->tev = nullptr;
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    double sum[4] = {0, 0, 0, 0};
    int cnt[4] = {0, 0, 0, 0};
    for (int i = 0; i < c->tev_used && e == cudaSuccess; i++) {
        float t = 0;
        e = cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]);
        sum[c->tkind[i]] += t;
        cnt[c->tkind[i]]++;
    }
    for (auto& x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) return fail(BEHF_ERR_CUDA, "kernel timing failed: %s", cudaGetErrorString(e));
    for (int k = 0; k < 4; k++) ms[k] = cnt[k] ? sum[k] / cnt[k] : 0.0;
    c->step += nsteps;
    return BEHF_OK;
}

behf_status behf_get_stream(behf_ctx* c, void** s) {
    if (!c || !s) return fail(BEHF_ERR_INVALID, "null argument");
    *s = (void*)c->stream;
    return BEHF_OK;
}

behf_status behf_health(behf_ctx* c, double* norms) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    const double limit = storage_max(c->prec);
    const Geom& g = c->g;
    CK(cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
    for (int q = 0; q < kNField; q++) {
        cudaError_t e;
        switch (c->prec) {
            case BEHF_FP64: e = aux_health<double>(c->p.f[q], g.nx, g.ny, g.nz, g.px, g.plane, limit, c->d_part, c->nblk_health, c->d_flag, c->d_norm + q, c->stream); break;
            case BEHF_FP32: e = aux_health<float>(c->p.f[q], g.nx, g.ny, g.nz, g.px, g.plane, limit, c->d_part, c->nblk_health, c->d_flag, c->d_norm + q, c->stream); break;
            case BEHF_FP16: e = aux_health<__half>(c->p.f[q], g.nx, g.ny, g.nz, g.px, g.plane, limit, c->d_part, c->nblk_health, c->d_flag, c->d_norm + q, c->stream); break;
            default: e = aux_health<__nv_bfloat16>(c->p.f[q], g.nx, g.ny, g.nz, g.px, g.plane, limit, c->d_part, c->nblk_health, c->d_flag, c->d_norm + q, c->stream);
        }
        if (e != cudaSuccess) return fail(BEHF_ERR_CUDA, "health kernel: %s", cudaGetErrorString(e));
    }
    double h[kNField];
    int flag = 0;
    CK(cudaMemcpyAsync(h, c->d_norm, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (norms) std::memcpy(norms, h, sizeof h);
    if (flag) return fail(BEHF_ERR_NONFINITE, "a field holds NaN/Inf or saturates its storage format");
    return BEHF_OK;
}

}  // extern "C"

namespace {

// ------------------------------------------------------------------------------------------------ gradient
// Adjoint-state gradient with sqrt(N) checkpointing.  Forward from rest over nt steps, saving the full state
// (fields + CPML memory) every ck steps; then per segment, last first: restore, recompute the segment keeping
// every step's fields after V (and the force source), and run the adjoint steps backwards through it.
// adj: [nrec][nt] host, dJ/d seismogram (physical units); obs != NULL: adj = seis - obs, J = |adj|^2 / 2.
struct DevBuf {
    behf_ctx* c;
    std::vector<void*> ptrs;
    explicit DevBuf(behf_ctx* cc) : c(cc) {}
    ~DevBuf() {
        for (void* p : ptrs) c->dfree(p);
    }
    behf_status get(void** out, size_t bytes) {
        behf_status st = c->dalloc(out, align256(bytes ? bytes : 1));
        if (!st) ptrs.push_back(*out);
        return st;
    }
};

template <class S>
behf_status gradient_impl(behf_ctx* c, int nt, const double* adj_host, const double* obs, double* misfit,
                          double* gw_host, double* const gm_host[kNMod]) {
    typedef typename Traits<S>::C A;
    if (!c->medium_set) return fail(BEHF_ERR_STATE, "behf_set_medium must come before the gradient");
    if (!c->keep_medium || !c->d_mod[0])
        return fail(BEHF_ERR_STATE, "set BEHF_OPT_GRADIENT before the medium to compute gradients");
    if (!c->src_set) return fail(BEHF_ERR_STATE, "the gradient needs a source");
    if (nt < 1) return fail(BEHF_ERR_INVALID, "nt must be positive");
    if (c->nrec < 1 || c->cap < nt) return fail(BEHF_ERR_INVALID, "receivers with capacity >= nt are required");
    const Geom& g = c->g;
    const size_t nf = (size_t)c->nfield, asz = sizeof(A);
    const size_t N = (size_t)c->grid.nx * c->grid.ny * c->grid.nz;
    const size_t sl[3] = {(size_t)c->grid.nz * c->grid.ny * g.W, (size_t)c->grid.nz * g.W * c->grid.nx,
                          (size_t)g.W * c->grid.ny * c->grid.nx};
    int S_ = c->ck_stride > 0 ? c->ck_stride : std::max(1, (int)std::lround(std::sqrt((double)nt)));
    DevBuf buf(c);
    AdjPtrs a{};
    behf_status st = BEHF_OK;
    for (int q = 0; q < kNField && !st; q++) st = buf.get(&a.lf[q], nf * asz);
    for (int q = 0; q < 7 && !st; q++) st = buf.get(&a.tmpT[q], nf * asz);
    for (int q = 0; q < 6 && !st; q++) st = buf.get(&a.tmpV[q], nf * asz);
    for (int q = 0; q < kNCoef && !st; q++) st = buf.get(&a.g[q], nf * asz);
    for (int q = 0; q < 3 && !st; q++) st = buf.get(&a.mu[q], nf * asz);
    if (g.W > 0)
        for (int ax = 0; ax < 3 && !st; ax++)
            for (int s = 0; s < 8 && !st; s++) {
                st = buf.get(&a.lpsi[ax][s], sl[ax] * asz);
                if (!st) st = buf.get(&a.lprv[ax][s], sl[ax] * asz);
            }
    // checkpoint: 13 fields then 48 CPML arrays; snapshot: 13 fields
    size_t ck_bytes = kNField * align256(nf * c->es);
    if (g.W > 0)
        for (int ax = 0; ax < 3; ax++) ck_bytes += 16 * align256(sl[ax] * c->ws);
    const size_t snap_bytes = kNField * align256(nf * c->es);
    // Checkpoint scheme (behf_checkpoint_plan): one level, or two when one does not fit the free device memory
    // less max(2 GiB, 2 %) or BEHF_OPT_CHECKPOINT_OUTER asks for it.
    if (st) return st;
    size_t avail = 0;
    if (c->ck_outer <= 0) {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        const size_t margin = std::max((size_t)2 << 30, tot / 50);
        avail = fr > margin ? fr - margin : 0;
    }
    int So_ = S_;
    {
        size_t planned = 0;
        st = behf_checkpoint_plan(nt, c->ck_stride, c->ck_outer, ck_bytes, snap_bytes, (size_t)c->nrec * nt * 8,
                                  c->ck_outer > 0 ? (size_t)-1 : avail, &S_, &So_, &planned);
        if (st) return st;
    }
    const int nseg = (nt + S_ - 1) / S_;      // snapshot segments (one level: also the checkpoint segments)
    const int nout = (nt + So_ - 1) / So_;      // outer segments (= nseg with one level)
    const bool two = So_ > S_;
    char* ck = nullptr;
    char* ckin = nullptr;  // two levels: the checkpoints inside one outer segment
    char* snap = nullptr;
    double *d_adj = nullptr, *d_gw = nullptr, *d_gfac = nullptr, *d_gm = nullptr;
    if (!st) st = buf.get((void**)&ck, ck_bytes * nout);
    if (!st && two) st = buf.get((void**)&ckin, ck_bytes * ((So_ + S_ - 1) / S_));
    if (!st) st = buf.get((void**)&snap, snap_bytes * (S_ + 1));
    if (!st) st = buf.get((void**)&d_adj, (size_t)c->nrec * nt * 8);
    if (!st) st = buf.get((void**)&d_gw, (size_t)nt * 8);
    if (!st) st = buf.get((void**)&d_gfac, 8);
    if (st) return st;
    for (int q = 0; q < kNField; q++) CK(cudaMemsetAsync(a.lf[q], 0, nf * asz, c->stream));
    for (int q = 0; q < 7; q++) CK(cudaMemsetAsync(a.tmpT[q], 0, nf * asz, c->stream));
    for (int q = 0; q < 6; q++) CK(cudaMemsetAsync(a.tmpV[q], 0, nf * asz, c->stream));
    for (int q = 0; q < kNCoef; q++) CK(cudaMemsetAsync(a.g[q], 0, nf * asz, c->stream));
    if (g.W > 0)
        for (int ax = 0; ax < 3; ax++)
            for (int s = 0; s < 8; s++) {
                CK(cudaMemsetAsync(a.lpsi[ax][s], 0, sl[ax] * asz, c->stream));
                CK(cudaMemsetAsync(a.lprv[ax][s], 0, sl[ax] * asz, c->stream));
            }
    CK(cudaMemsetAsync(d_gw, 0, (size_t)nt * 8, c->stream));
    CK(cudaMemsetAsync(d_gfac, 0, 8, c->stream));
    a.grad = 1;
    a.derived = (c->kernel_opt != BEHF_KERNEL_PLAIN && c->tiled_ok) ? 1 : 0;
    {  // the adjoint kernels' L2 prefetch and the memory updates inside the gradient kernels: on unless
       // BEHF_ADJ_PREFETCH=0 / BEHF_ADJ_VMERGE=0 (diagnostic switches for timing; the same results)
        const char* e = getenv("BEHF_ADJ_PREFETCH");
        a.pf = (e && e[0] == '0') ? 0 : 1;
        const char* v = getenv("BEHF_ADJ_VMERGE");
        a.vmerge = (v && v[0] == '0') ? 0 : 1;
    }
    // compensated summation of the FP32 accumulators: segment sums folded into running totals
    AdjFold fold{};
    const bool folding = sizeof(A) == 4 && c->grad_comp > 0;
    if (folding) {
        fold.mode = c->grad_comp;
        for (int q = 0; q < kNCoef && !st; q++) {
            fold.g[q] = reinterpret_cast<float*>(a.g[q]);
            if (fold.mode == 2) {
                st = buf.get((void**)&fold.tot64[q], nf * 8);
                if (!st) CK(cudaMemsetAsync(fold.tot64[q], 0, nf * 8, c->stream));
            } else {
                st = buf.get((void**)&fold.tot[q], nf * 4);
                if (!st) st = buf.get((void**)&fold.comp[q], nf * 4);
                if (!st) CK(cudaMemsetAsync(fold.tot[q], 0, nf * 4, c->stream));
                if (!st) CK(cudaMemsetAsync(fold.comp[q], 0, nf * 4, c->stream));
            }
        }
        if (st) return st;
    }
    AdjMaps* maps = static_cast<AdjMaps*>(std::aligned_alloc(alignof(AdjMaps), sizeof(AdjMaps)));
    if (!maps) return fail(BEHF_ERR_ALLOC, "host allocation of the adjoint tensor maps");
    std::unique_ptr<AdjMaps, void (*)(void*)> maps_owner(maps, std::free);
    CK(adj_build_maps<S>(g, a, maps));
    // Snapshots of a segment: slot u holds the fields after V (+ force) of step s0 + u - 1, slot 0 the state after
    // step s0 - 1 (its velocities and Darcy velocities are those after its V).  The last segments keep the
    // snapshots of the forward pass in a cache and need no recompute: as many as the free device memory allows
    // (BEHF_OPT_SNAPSHOT_CACHE: -1 all of it but max(8 GiB, 10 %), 0 none, else that many MiB); their slot 0 is the
    // segment's checkpoint, which holds the 13 fields in the same layout.  The others share one buffer.
    std::vector<char*> cache(nseg, nullptr);
    // Overlap (one level): segment sg - 1 is recomputed on a second stream, into the other of two snapshot buffers
    // (segment parity), while segment sg runs its adjoint steps.  The adjoint reads only the coefficients, the CPML
    // profiles and the snapshots, never the forward state the recompute overwrites; events order each buffer's
    // reuse.  The second buffer is allocated only when some segment will be recomputed and it fits.
    char* snap2 = nullptr;
    {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        const size_t cmargin = std::max((size_t)8 << 30, tot / 10);
        size_t budget = fr > cmargin ? fr - cmargin : 0;
        if (c->snap_cache_mib > 0) budget = std::min(budget, (size_t)c->snap_cache_mib << 20);
        const bool all_cached = c->snap_cache_mib != 0 && budget / (snap_bytes * (size_t)S_) >= (size_t)nseg;
        const size_t need = snap_bytes * (S_ + 1), margin = std::max((size_t)2 << 30, tot / 50);
        if (c->rc_overlap && !two && nseg > 1 && !all_cached && fr > need + margin) {
            st = buf.get((void**)&snap2, need);
            if (st) return st;
        }
    }
    const bool overlap = snap2 != nullptr;
    if (c->snap_cache_mib != 0 && !two) {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        const size_t margin = std::max((size_t)8 << 30, tot / 10);
        size_t budget = fr > margin ? fr - margin : 0;
        if (c->snap_cache_mib > 0) budget = std::min(budget, (size_t)c->snap_cache_mib << 20);
        const size_t per = snap_bytes * (size_t)S_;
        const int ncached = (int)std::min<size_t>((size_t)nseg, budget / per);
        for (int k = 0; k < ncached; k++)
            if (buf.get((void**)&cache[nseg - 1 - k], per) != BEHF_OK) {  // keep what fitted
                cache[nseg - 1 - k] = nullptr;
                break;
            }
    }
    auto cached = [&](int sg) { return sg >= 0 && cache[sg] != nullptr; };  // sg -1: a segment never cached
    // the recompute buffer of an uncached segment: the shared one, or with overlap the one of the segment's parity
    auto rbuf = [&](int sg) { return overlap && (sg & 1) ? 1 : 0; };
    auto snap_ptr = [&](int sg, int idx, int f) -> char* {
        const size_t fo = align256(nf * c->es) * f;
        if (cached(sg)) return idx == 0 ? ck + ck_bytes * sg + fo : cache[sg] + snap_bytes * (idx - 1) + fo;
        return (rbuf(sg) ? snap2 : snap) + snap_bytes * idx + fo;
    };
    // tensor maps of a segment's snapshot slots (the 16-bit kinds stage snapshot windows in the gathers)
    std::vector<GatherMaps> snap_mt, snap_mv;
    int maps_seg = INT_MIN;  // segment whose buffers the maps describe (-1 / -2: the first / second shared buffer)
    auto build_snap_maps = [&](int sg) -> cudaError_t {
        if (!adj_snap_staged<S>()) return cudaSuccess;
        const int key = cached(sg) ? sg : -1 - rbuf(sg);
        if (key == maps_seg) return cudaSuccess;
        snap_mt.resize(S_ + 1);
        snap_mv.resize(S_ + 1);
        for (int u = 0; u <= S_; u++) {
            void* f[kNField];
            for (int q = 0; q < kNField; q++) f[q] = snap_ptr(sg, u, q);
            const cudaError_t e = adj_build_snap_maps<S>(g, f, &snap_mt[u], &snap_mv[u]);
            if (e != cudaSuccess) return e;
        }
        maps_seg = key;
        return cudaSuccess;
    };

    auto copy_state = [&](char* dst, bool save) -> cudaError_t {
        char* q = dst;
        for (int f = 0; f < kNField; f++, q += align256(nf * c->es)) {
            cudaError_t e = save ? cudaMemcpyAsync(q, c->p.f[f], nf * c->es, cudaMemcpyDeviceToDevice, c->stream)
                                 : cudaMemcpyAsync(c->p.f[f], q, nf * c->es, cudaMemcpyDeviceToDevice, c->stream);
            if (e != cudaSuccess) return e;
        }
        if (g.W > 0)
            for (int ax = 0; ax < 3; ax++)
                for (int s = 0; s < 16; s++, q += align256(sl[ax] * c->ws)) {
                    void* m = s < 8 ? c->p.psi[ax][s] : c->p.prv[ax][s - 8];
                    cudaError_t e = save ? cudaMemcpyAsync(q, m, sl[ax] * c->ws, cudaMemcpyDeviceToDevice, c->stream)
                                         : cudaMemcpyAsync(m, q, sl[ax] * c->ws, cudaMemcpyDeviceToDevice, c->stream);
                    if (e != cudaSuccess) return e;
                }
        return cudaSuccess;
    };
    auto snap_fields = [&](int sg, int idx) -> cudaError_t {
        for (int f = 0; f < kNField; f++) {
            cudaError_t e = cudaMemcpyAsync(snap_ptr(sg, idx, f), c->p.f[f], nf * c->es, cudaMemcpyDeviceToDevice,
                                            c->stream);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    double fac = 0;
    CK(source_factor(c, &fac));
    const long long so = c->cell_offset(c->src_ijk[0], c->src_ijk[1], c->src_ijk[2]);
    // one forward step with the d_it counter, keeping the fields after V (+ force) in slot idx of segment sg
    // (idx < 0: no snapshot)
    // (to_snapshot: stop after the snapshot, without the stress update and the tick; the out-of-place recompute
    // below does those for the step with its next step)
    auto snap_step = [&](int sg, int idx, bool record, bool to_snapshot = false) -> cudaError_t {
        cudaError_t e;
        if (c->src_kind != BEHF_SRC_FORCE_Z &&
            (e = aux_source<S>(c->p, so, c->src_kind, c->d_wavelet, c->nw, c->d_it, 0, fac, c->stream)) != cudaSuccess)
            return e;
        if ((e = dispatch_update(c, true)) != cudaSuccess) return e;
        if (c->src_kind == BEHF_SRC_FORCE_Z &&
            (e = aux_source<S>(c->p, so, c->src_kind, c->d_wavelet, c->nw, c->d_it, 0, fac, c->stream)) != cudaSuccess)
            return e;
        if (idx >= 0 && (e = snap_fields(sg, idx)) != cudaSuccess) return e;
        if (to_snapshot) {
            c->launches += 2;
            return cudaSuccess;
        }
        if ((e = dispatch_update(c, false)) != cudaSuccess) return e;
        if (record) {
            RecScales rs;
            for (int q = 0; q < kNField; q++) rs.s[q] = c->field_scale(q);
            if ((e = aux_record<S>(c->p, c->d_rec_off, c->d_rec_comp, c->nrec, c->d_seis, c->cap, c->d_it, 0, rs,
                                   c->stream)) != cudaSuccess)
                return e;
        }
        c->launches += 4 + (record ? 1 : 0);
        return aux_tick(c->d_it, 1, c->stream);
    };

    // The recompute steps out of place with the kernels that read the fields only through tensor maps (the
    // warp-specialised and tensor-memory variants; the classic and plain kernels read them directly): instead of
    // copying 13 fields into each snapshot slot, the stress update of step it - 1 reads slot u - 1 and writes the
    // stresses and pressure of slot u, and the velocity update of step it reads slot u - 1's velocities and slot
    // u's stresses and writes slot u's velocities.  The CPML memory stays in place, updated in the same order.
    // BEHF_RC_OOP=0 keeps the copies (a diagnostic switch; the same results).
    const char* oop_env = getenv("BEHF_RC_OOP");
    const bool oop = !(oop_env && oop_env[0] == '0') && c->kernel_opt != BEHF_KERNEL_PLAIN && c->tiled_ok &&
                     c->g.ws >= 1 && sizeof(S) < 8;
    std::unique_ptr<void, decltype(&std::free)> ovm(nullptr, &std::free), otm(nullptr, &std::free);
    if (oop) {  // the field maps are re-encoded per step; the rest are the context's
        ovm.reset(std::aligned_alloc(64, (sizeof(tiled::VMaps) + 63) / 64 * 64));
        otm.reset(std::aligned_alloc(64, (sizeof(tiled::TMaps) + 63) / 64 * 64));
        if (!ovm || !otm) return fail(BEHF_ERR_ALLOC, "out of host memory");
        std::memcpy(ovm.get(), c->vmaps, sizeof(tiled::VMaps));
        std::memcpy(otm.get(), c->tmaps, sizeof(tiled::TMaps));
        // the updates write only the updated cells: the slots' ghost ring must hold the zeros a copy of the
        // fields would bring (ordered before the backward pass by the synchronisation after the forward pass)
        CK(cudaMemsetAsync(snap, 0, snap_bytes * (S_ + 1), c->stream));
        if (snap2) CK(cudaMemsetAsync(snap2, 0, snap_bytes * (S_ + 1), c->stream));
    }
    auto launch_maps = [&](const DevPtrs& po, const void* maps, bool vel) -> cudaError_t {
        return c->tile_rows == 4 ? launch_tiled_rows4<S>(c->g, po, maps, vel, c->stream)
                                 : launch_tiled<S>(c->g, po, maps, vel, c->stream);
    };
    // recompute a segment from its checkpoint on c->stream, keeping the fields after V (+ force) of every step
    auto recompute = [&](int sg, int s0, int s1, char* ckp) -> cudaError_t {
        cudaError_t e;
        if ((e = copy_state(ckp, false)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(c->d_it, 0, sizeof(int), c->stream)) != cudaSuccess) return e;
        if (s0 > 0 && (e = aux_tick(c->d_it, s0, c->stream)) != cudaSuccess) return e;
        if ((e = snap_fields(sg, 0)) != cudaSuccess) return e;
        if (!oop) {
            for (int it = s0; it < s1; it++)
                if ((e = snap_step(sg, it - s0 + 1, false)) != cudaSuccess) return e;
            return cudaSuccess;
        }
        // step s0 in place up to its snapshot (slot 1); the segment's last stress update is not needed
        if ((e = snap_step(sg, 1, false, true)) != cudaSuccess) return e;
        for (int u = 2; u <= s1 - s0; u++) {
            void *prev[kNField], *vf[kNField];
            DevPtrs po = c->p;
            for (int q = 0; q < kNField; q++) {
                prev[q] = snap_ptr(sg, u - 1, q);
                po.f[q] = snap_ptr(sg, u, q);
                vf[q] = q <= BEHF_QZ ? prev[q] : po.f[q];
            }
            e = c->tile_rows == 4 ? tiled_field_maps_rows4<S>(c->g, vf, prev, ovm.get(), otm.get())
                                  : tiled_field_maps<S>(c->g, vf, prev, ovm.get(), otm.get());
            if (e != cudaSuccess) return e;
            if ((e = launch_maps(po, otm.get(), false)) != cudaSuccess) return e;  // stresses of step it - 1
            if ((e = aux_tick(c->d_it, 1, c->stream)) != cudaSuccess) return e;
            if (c->src_kind != BEHF_SRC_FORCE_Z &&
                (e = aux_source<S>(po, so, c->src_kind, c->d_wavelet, c->nw, c->d_it, 0, fac, c->stream)) != cudaSuccess)
                return e;
            if ((e = launch_maps(po, ovm.get(), true)) != cudaSuccess) return e;  // velocities of step it
            if (c->src_kind == BEHF_SRC_FORCE_Z &&
                (e = aux_source<S>(po, so, c->src_kind, c->d_wavelet, c->nw, c->d_it, 0, fac, c->stream)) != cudaSuccess)
                return e;
            c->launches += 4;
        }
        return cudaSuccess;
    };
    // the second stream of the overlap and its events (done: a buffer's recompute finished; free: the adjoint
    // steps that read a buffer finished); destroyed, after its work, before the buffers are freed
    struct Side {
        cudaStream_t s = nullptr;
        cudaEvent_t done[2] = {}, free[2] = {};
        ~Side() {
            if (s) cudaStreamSynchronize(s);
            for (int i = 0; i < 2; i++) {
                if (done[i]) cudaEventDestroy(done[i]);
                if (free[i]) cudaEventDestroy(free[i]);
            }
            if (s) cudaStreamDestroy(s);
        }
    } side;
    if (overlap) {
        CK(cudaStreamCreateWithFlags(&side.s, cudaStreamNonBlocking));
        for (int i = 0; i < 2; i++) {
            CK(cudaEventCreateWithFlags(&side.done[i], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&side.free[i], cudaEventDisableTiming));
        }
    }
    int prefetched = -1;  // the last segment whose recompute was enqueued on the second stream
    auto recompute_on_side = [&](int sg) -> cudaError_t {
        const int s0 = sg * S_, s1 = std::min(nt, s0 + S_);
        const int b = rbuf(sg);
        cudaError_t e = cudaStreamWaitEvent(side.s, side.free[b], 0);  // the adjoint steps of buffer b's last use
        if (e != cudaSuccess) return e;
        cudaStream_t main = c->stream;
        c->stream = side.s;
        e = recompute(sg, s0, s1, ck + ck_bytes * sg);
        c->stream = main;
        if (e != cudaSuccess) return e;
        prefetched = sg;
        return cudaEventRecord(side.done[b], side.s);
    };

    // forward pass with checkpoints (seismograms recorded as in behf_run); cached segments step by step
    st = zero_state(c);
    if (st) return st;
    for (int sg = 0; sg < nout; sg++) {
        const int s0 = sg * So_, s1 = std::min(nt, s0 + So_);
        CK(copy_state(ck + ck_bytes * sg, true));
        if (!cached(sg)) {
            st = behf_run_async(c, s1 - s0);
            if (st) return st;
        } else {
            for (int it = s0; it < s1; it++) CK(snap_step(sg, it - s0 + 1, true));
            c->step += s1 - s0;
        }
    }
    st = behf_sync(c);
    if (st) return st;

    // adjoint source (host): residual and misfit, scaled by alpha so the adjoint state stays O(1)
    const int nrec = c->nrec;
    std::vector<double> adj((size_t)nrec * nt);
    std::vector<int> comp(nrec);
    CK(cudaMemcpy(comp.data(), c->d_rec_comp, (size_t)nrec * 4, cudaMemcpyDeviceToHost));
    if (obs) {
        std::vector<double> seis((size_t)nrec * nt);
        CK(cudaMemcpy2D(seis.data(), (size_t)nt * 8, c->d_seis, (size_t)c->cap * 8, (size_t)nt * 8, nrec,
                        cudaMemcpyDeviceToHost));
        double J = 0;
        for (size_t i = 0; i < adj.size(); i++) {
            adj[i] = seis[i] - obs[i];
            J += 0.5 * adj[i] * adj[i];
        }
        if (misfit) *misfit = J;
    } else {
        std::memcpy(adj.data(), adj_host, adj.size() * 8);
    }
    double amax = 0;
    for (int r = 0; r < nrec; r++)
        for (int it = 0; it < nt; it++)
            amax = std::fmax(amax, std::fabs(adj[(size_t)r * nt + it]) / c->field_scale(comp[r]));
    const double alpha = amax > 0 ? 1.0 / amax : 1.0;
    AdjScales sc;
    for (int q = 0; q < kNField; q++) sc.s[q] = alpha / c->field_scale(q);
    CK(cudaMemcpy(d_adj, adj.data(), adj.size() * 8, cudaMemcpyHostToDevice));

    for (int og = nout - 1; og >= 0; og--) {
        const int o0 = og * So_, o1 = std::min(nt, o0 + So_);
        const int nin = two ? (o1 - o0 + S_ - 1) / S_ : 1;
        if (two) {  // run the outer segment forward again from its checkpoint, keeping a checkpoint every S_ steps
            CK(copy_state(ck + ck_bytes * og, false));
            CK(cudaMemcpyAsync(c->d_it, &o0, sizeof(int), cudaMemcpyHostToDevice, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            for (int j = 0; j < nin; j++) {
                CK(copy_state(ckin + ck_bytes * j, true));
                for (int it = o0 + j * S_; it < std::min(o1, o0 + (j + 1) * S_); it++) CK(snap_step(-1, -1, false));
            }
        }
        for (int j = nin - 1; j >= 0; j--) {
            const int sg = two ? -1 : og;  // the segment's index in the snapshot cache (never cached with two levels)
            const int s0 = o0 + j * S_, s1 = std::min(o1, s0 + S_);
            char* ckp = two ? ckin + ck_bytes * j : ck + ck_bytes * og;
            if (!cached(sg)) {
                if (!overlap) {
                    CK(recompute(sg, s0, s1, ckp));
                } else {
                    if (prefetched != sg) CK(recompute_on_side(sg));  // the first recomputed segment
                    CK(cudaStreamWaitEvent(c->stream, side.done[rbuf(sg)], 0));
                }
            }
            // the next segment's recompute, on the second stream, while this one runs its adjoint steps
            if (overlap && sg >= 1 && !cached(sg - 1)) CK(recompute_on_side(sg - 1));
            CK(build_snap_maps(sg));
            // backward step it: T^T per cell of it is done (the first step: here, after its record^T; later steps:
            // fused into the V^T gather of step it + 1, completed by the record^T of it)
            for (int it = s1 - 1; it >= s0; it--) {
                for (int f = 0; f < kNField; f++) a.cur[f] = snap_ptr(sg, it - s0 + 1, f);
                for (int d = 0; d < 3; d++) a.qprev[d] = snap_ptr(sg, it - s0, BEHF_QX + d);
                for (int d = 0; d < 6; d++) a.vq1[d] = snap_ptr(sg, it - s0, BEHF_VX + d);
                if (it == nt - 1) {
                    CK(adj_record<S>(a, c->d_rec_off, c->d_rec_comp, nrec, d_adj, nt, it, sc, c->stream));
                    CK(adj_first<S>(g, c->p, a, c->stream));
                    c->launches += 2;
                }
                const int fuse = it >= 1 ? 1 : 0;
                const bool sm = !snap_mt.empty();
                CK(adj_step<S>(g, c->p, a, *maps, sm ? &snap_mt[it - s0 + 1] : nullptr,
                               sm ? &snap_mv[it - s0] : nullptr, fuse, c->stream));
                CK(adj_point<S>(a, so, c->src_kind, fac, c->d_wavelet, c->nw, it, d_gw, d_gfac, c->stream));
                if (fuse)
                    CK(adj_recfix<S>(g, c->p, a, c->d_rec_off, c->d_rec_comp, nrec, d_adj, nt, it - 1, sc,
                                     c->stream));
                c->launches += adj_step_launches(g, a, fuse) + 1 + fuse;  // + source^T, record^T
            }
            if (folding) {
                CK(adj_fold(fold, (long long)nf, 0, c->stream));
                c->launches++;
            }
            if (overlap && !cached(sg)) CK(cudaEventRecord(side.free[rbuf(sg)], c->stream));
        }
    }
    if (folding) {
        CK(adj_fold(fold, (long long)nf, 1, c->stream));
        c->launches++;
    }
    CK(cudaMemcpyAsync(c->d_it, &nt, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    st = behf_sync(c);
    if (st) return st;
    c->step = nt;

    if (gw_host) {
        CK(cudaMemcpy(gw_host, d_gw, (size_t)nt * 8, cudaMemcpyDeviceToHost));
        for (int it = 0; it < nt; it++) gw_host[it] /= alpha;
    }
    bool want_mod = false;
    for (int q = 0; q < kNMod; q++) want_mod = want_mod || gm_host[q];
    if (!want_mod) return BEHF_OK;
    if ((st = buf.get((void**)&d_gm, N * 8 * kNMod))) return st;
    GradModArgs ga{};
    for (int q = 0; q < kNMod; q++) {
        ga.mod[q] = c->d_mod[q];
        ga.gm[q] = d_gm + N * q;
    }
    for (int q = 0; q < kNCoef; q++) ga.g[q] = a.g[q];
    const double sv = c->scales[0], sq = c->scales[1], ss = c->scales[2], sp = c->scales[3];
    const double hi = 1.0 / c->grid.h;
    for (int d = 0; d < 3; d++) {
        ga.ratio[VW1X + d] = 1.0;
        ga.ratio[VW2X + d] = sq / ss * hi;
        ga.ratio[VW3X + d] = sq / sp * hi;
        ga.ratio[VU1X + d] = sv / ss * hi;
        ga.ratio[VU2X + d] = sv / sq;
    }
    ga.ratio[P1] = sp / sv * hi;
    ga.ratio[P2] = sp / sq * hi;
    ga.ratio[S1] = ga.ratio[S2] = ss / sv * hi;
    ga.ratio[S3] = ss / sq * hi;
    ga.ratio[SXYC] = ga.ratio[SXZC] = ga.ratio[SYZC] = ss / sv * hi;
    ga.nx = c->grid.nx;
    ga.ny = c->grid.ny;
    ga.nz = c->grid.nz;
    ga.R = g.R;
    ga.L = g.W > 0 ? g.L : 0;
    ga.px = g.px;
    ga.plane = g.plane;
    ga.dt = c->grid.dt;
    CK(adj_grad_moduli<A>(ga, c->stream));
    c->launches++;
    CK(cudaStreamSynchronize(c->stream));
    for (int q = 0; q < kNMod; q++) {
        if (!gm_host[q]) continue;
        CK(cudaMemcpy(gm_host[q], d_gm + N * q, N * 8, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < N; i++) gm_host[q][i] /= alpha;
    }
    if (c->src_kind == BEHF_SRC_FORCE_Z && gm_host[BEHF_RHO]) {
        // force = dt / rho_z * s_v with rho_z = (rho[src] + rho[src + z]) / 2
        double gfac = 0;
        float r[2];
        const size_t o = ((size_t)c->src_ijk[2] * c->grid.ny + c->src_ijk[1]) * c->grid.nx + c->src_ijk[0];
        const size_t plane = (size_t)c->grid.nx * c->grid.ny;
        CK(cudaMemcpy(&gfac, d_gfac, 8, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&r[0], c->d_mod[BEHF_RHO] + o, 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&r[1], c->d_mod[BEHF_RHO] + o + plane, 4, cudaMemcpyDeviceToHost));
        const double rz = 0.5 * ((double)r[0] + (double)r[1]);
        const double gr = gfac / alpha * (-c->grid.dt * c->scales[0] / (rz * rz)) * 0.5;
        const int n3[3] = {c->grid.nx, c->grid.ny, c->grid.nz};
        auto inside = [&](int kz) {
            const int xs[3] = {c->src_ijk[0], c->src_ijk[1], kz};
            for (int d = 0; d < 3; d++) {
                const int lo = std::max(ga.L, ga.R) + 1;
                const int hi3 = ga.L > 0 ? std::min(n3[d] - 2 - ga.L, n3[d] - ga.R - 1) : n3[d] - ga.R - 1;
                if (xs[d] < lo || xs[d] > hi3) return false;
            }
            return true;
        };
        if (inside(c->src_ijk[2])) gm_host[BEHF_RHO][o] += gr;
        if (inside(c->src_ijk[2] + 1)) gm_host[BEHF_RHO][o + plane] += gr;
    }
    return BEHF_OK;
}

behf_status gradient_dispatch(behf_ctx* c, int nt, const double* adj, const double* obs, double* misfit, double* gw,
                              double* const gm[kNMod]) {
    double* none[kNMod] = {};
    double* const* g = gm ? gm : none;
    switch (c->prec) {
        case BEHF_FP64: return gradient_impl<double>(c, nt, adj, obs, misfit, gw, g);
        case BEHF_FP32: return gradient_impl<float>(c, nt, adj, obs, misfit, gw, g);
        case BEHF_FP16: return gradient_impl<__half>(c, nt, adj, obs, misfit, gw, g);
        case BEHF_BF16: return gradient_impl<__nv_bfloat16>(c, nt, adj, obs, misfit, gw, g);
    }
    return fail(BEHF_ERR_INVALID, "bad precision");
}

}  // namespace

extern "C" {

behf_status behf_gradient(behf_ctx* c, int nt, const double* adj_src, double* grad_wavelet,
                          double* const grad_moduli[BEHF_NMOD]) {
    if (!c || !adj_src) return fail(BEHF_ERR_INVALID, "null argument");
    DeviceScope device_scope(c->dev);
    return gradient_dispatch(c, nt, adj_src, nullptr, nullptr, grad_wavelet, grad_moduli);
}

behf_status behf_misfit_gradient(behf_ctx* c, int nt, const double* observed, double* misfit, double* grad_wavelet,
                                 double* const grad_moduli[BEHF_NMOD]) {
    if (!c || !observed) return fail(BEHF_ERR_INVALID, "null argument");
    DeviceScope device_scope(c->dev);
    return gradient_dispatch(c, nt, nullptr, observed, misfit, grad_wavelet, grad_moduli);
}

behf_status behf_selftest_wait(behf_ctx* c) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    CK(aux_wait_selftest(c->d_err, c->stream));
    c->launches++;
    return behf_sync(c);
}

behf_status behf_autotune(behf_ctx* c, int trial_steps, int* zchunk_out, double* ms_out) {
    if (!c) return fail(BEHF_ERR_INVALID, "null context");
    DeviceScope device_scope(c->dev);
    if (!c->medium_set) return fail(BEHF_ERR_STATE, "behf_set_medium must come before behf_autotune");
    if (trial_steps < 1) return fail(BEHF_ERR_INVALID, "trial_steps must be positive");
    const int planes = c->grid.nz - 2 * c->g.R;
    std::vector<int> zc = {0};
    for (int z = 16; z < planes; z *= 2) zc.push_back(z);
    zc.push_back(planes);
    // (tile rows, variant, z chunk): the heights and variants only where the tiled kernels run
    struct Cand {
        int rows, v, z;
    };
    std::vector<Cand> cand;
    const bool tiled = c->kernel_opt != BEHF_KERNEL_PLAIN && c->tiled_ok;
    for (int rows : {8, 4}) {
        if (!tiled && rows != c->tile_rows) continue;
        for (int v = tiled ? 0 : c->g.ws; v <= (tiled ? 3 : c->g.ws); v++)
            for (int z : zc) cand.push_back({rows, v, z});
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double best = 1e300;
    int best_z = 0, best_v = c->g.ws, best_rows = c->tile_rows;
    behf_status st = BEHF_OK;
    const int nrec = c->nrec;
    c->nrec = 0;  // trial steps record nothing
    for (const Cand& cd : cand) {
        const int v = cd.v, z = cd.z;
        if (cd.rows != c->tile_rows) {  // the other height's tensor maps
            c->tile_rows = cd.rows;
            if (tiled && !setup_tiled_any(c)) continue;
        }
        c->g.ws = v;
        c->g.zchunk_req = z;
        c->invalidate_graph();
        if ((st = zero_state(c))) break;
        if ((st = behf_run_async(c, 1))) break;
        cudaEventRecord(e0, c->stream);
        if ((st = behf_run_async(c, trial_steps))) break;
        cudaEventRecord(e1, c->stream);
        if ((st = behf_sync(c))) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms / trial_steps < best) {
            best = ms / trial_steps;
            best_z = z;
            best_v = v;
            best_rows = cd.rows;
        }
    }
    c->nrec = nrec;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_rows != c->tile_rows) {
        c->tile_rows = best_rows;
        if (tiled && !setup_tiled_any(c) && !st) st = fail(BEHF_ERR_CUDA, "tensor maps for %d-row tiles", best_rows);
    }
    c->g.ws = best_v;
    c->g.zchunk_req = best_z;
    c->invalidate_graph();
    if (st) return st;
    st = zero_state(c);
    if (st) return st;
    if (zchunk_out) *zchunk_out = best_z;
    if (ms_out) *ms_out = best;
    return BEHF_OK;
}

behf_status behf_run_batch(behf_ctx* const* ctxs, int n, int nsteps) {
    if (!ctxs || n < 0 || nsteps < 0) return fail(BEHF_ERR_INVALID, "bad batch arguments");
    for (int i = 0; i < n; i++)
        if (!ctxs[i]) return fail(BEHF_ERR_INVALID, "context %d is null", i);
    // round-robin pieces of one graph chunk per context so the contexts' streams overlap on the device
    int done = 0;
    while (done < nsteps) {
        int piece = nsteps - done;
        for (int i = 0; i < n; i++) {
            const int ch = ctxs[i]->chunk > 0 ? ctxs[i]->chunk : 16;
            piece = std::min(piece, ch);
        }
        for (int i = 0; i < n; i++) {
            behf_status st = behf_run_async(ctxs[i], piece);
            if (st) return st;
        }
        done += piece;
    }
    for (int i = 0; i < n; i++) {
        behf_status st = behf_sync(ctxs[i]);
        if (st) return st;
    }
    return BEHF_OK;
}

}  // extern "C"
