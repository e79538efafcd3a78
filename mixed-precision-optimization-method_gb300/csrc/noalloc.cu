// noalloc.cu -- behf_field_norm_noalloc: the field energy norm and health flag of behf_health, for
// callers that must not allocate device memory.
//
// Who needs it: a host application that owns every byte of device memory through its own pool (a
// seismic-imaging framework that has reserved the GPU for its wavefields, or PyTorch's caching
// allocator holding it), or a monitoring thread that checks a running simulation between steps.
// For them a cudaMalloc either fails because nothing is left, or a cudaFree stalls the whole device
// because it synchronizes.  behf_health needs a context, and a context allocates.  This entry point
// takes only the caller's field and output pointers and allocates nothing.
//
// Scratch: the per-block partial sums live in the file-scope device array g_norm_scratch below
// (kMaxPartials doubles, 512 KiB, held by every GPU that loads the library until the process exits).
// Host code must not hand the array's name to a kernel: on the host it is only a stand-in symbol.
// The first call on each device looks up the array's device address with cudaGetSymbolAddress (with
// that device current) and caches it; make that first call before any stream capture.  Every call
// shares the array, so calls that overlap on the GPU (different streams, or different host threads)
// race on it.  Each call rewrites the partials it reads, so nothing needs clearing between calls.
#include <cstdio>
#include <mutex>

#include "behf_internal.cuh"

namespace behf {
void report_error(const char* msg);
}

namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 64;
constexpr long long kCellsPerBlock = (long long)kThreads * kCellsPerThread;  // 16384
constexpr int kMaxPartials = 65536;                                          // => 2^30 cells
constexpr long long kMaxCells = kCellsPerBlock * kMaxPartials;
constexpr int kMaxDevices = 64;

// One partial sum of squares per block over its finite, unsaturated cells; the sign bit marks a block that also
// saw NaN/Inf/saturation (-0.0 when it saw nothing else), so the final sum keeps the finite cells of such blocks,
// as behf_health does.
static __device__ __align__(256) double g_norm_scratch[kMaxPartials];

std::mutex g_scratch_mu;
double* g_scratch_addr[kMaxDevices] = {};

template <class S>
__global__ void k_norm_part(const void* f, int nx, int ny, long long px, long long plane, long long N, double limit,
                            double* part) {
    double acc = 0.0;
    int bad = 0;
    const long long c0 = (long long)blockIdx.x * kCellsPerBlock;
    const long long c1 = c0 + kCellsPerBlock < N ? c0 + kCellsPerBlock : N;
    for (long long c = c0 + threadIdx.x; c < c1; c += kThreads) {
        const int i = (int)(c % nx);
        const long long r = c / nx;
        const int j = (int)(r % ny), k = (int)(r / ny);
        const double v = (double)behf::Traits<S>::ld(reinterpret_cast<const S*>(f)[k * plane + j * px + i]);
        if (!(fabs(v) < limit)) bad = 1;
        else acc += v * v;
    }
    __shared__ double red[kThreads / 32];
    __shared__ int anybad;
    if (threadIdx.x == 0) anybad = 0;
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    if (bad) atomicOr(&anybad, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < kThreads / 32; w++) s += red[w];
        part[blockIdx.x] = anybad ? -s : s;  // s >= +0.0, so the sign bit carries only the flag
    }
}

// Fixed-order final sum of the nb partials (deterministic), and the health flag.
__global__ void k_norm_final(const double* part, int nb, double* norm_out, int* flag_out) {
    double s = 0;
    int bad = 0;
    for (int b = threadIdx.x; b < nb; b += 32) {
        const double v = part[b];
        if (signbit(v)) bad = 1;
        s += fabs(v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (threadIdx.x == 0) {
        *norm_out = s;
        *flag_out = bad;
    }
}

// Device address of g_norm_scratch on the current device, looked up once per device.
cudaError_t scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_norm_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

template <class S>
cudaError_t launch(const void* f, int nx, int ny, long long px, long long plane, long long N, double limit,
                   double* scratch, int nb, double* norm_out, int* flag_out, cudaStream_t st) {
    k_norm_part<S><<<nb, kThreads, 0, st>>>(f, nx, ny, px, plane, N, limit, scratch);
    k_norm_final<<<1, 32, 0, st>>>(scratch, nb, norm_out, flag_out);
    return cudaGetLastError();
}

}  // namespace

extern "C" behf_status behf_field_norm_noalloc(const void* field, int precision, int nx, int ny, int nz,
                                               long long pitch, long long plane, double* norm_out, int* flag_out,
                                               void* stream) {
    char msg[256];
    if (!field || !norm_out || !flag_out) {
        behf::report_error("behf_field_norm_noalloc: null field or output pointer");
        return BEHF_ERR_INVALID;
    }
    if (precision < BEHF_FP64 || precision > BEHF_BF16) {
        behf::report_error("behf_field_norm_noalloc: bad precision");
        return BEHF_ERR_INVALID;
    }
    if (nx <= 0 || ny <= 0 || nz <= 0 || pitch < nx || plane < pitch * ny) {
        behf::report_error("behf_field_norm_noalloc: bad sizes (need nx, ny, nz > 0, pitch >= nx, plane >= pitch*ny)");
        return BEHF_ERR_INVALID;
    }
    const long long N = (long long)nx * ny * nz;
    if (N > kMaxCells) {
        snprintf(msg, sizeof msg,
                 "behf_field_norm_noalloc: %lld cells exceed the limit of %lld (its fixed scratch holds %d partial "
                 "sums of %lld cells); use behf_health for larger fields",
                 N, kMaxCells, kMaxPartials, kCellsPerBlock);
        behf::report_error(msg);
        return BEHF_ERR_INVALID;
    }
    double* scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) {
        snprintf(msg, sizeof msg, "behf_field_norm_noalloc: scratch address lookup failed: %s", cudaGetErrorString(e));
        behf::report_error(msg);
        return BEHF_ERR_CUDA;
    }
    const int nb = (int)((N + kCellsPerBlock - 1) / kCellsPerBlock);
    const double limit = behf::storage_max(precision);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (precision) {
        case BEHF_FP64: e = launch<double>(field, nx, ny, pitch, plane, N, limit, scratch, nb, norm_out, flag_out, st); break;
        case BEHF_FP32: e = launch<float>(field, nx, ny, pitch, plane, N, limit, scratch, nb, norm_out, flag_out, st); break;
        case BEHF_FP16: e = launch<__half>(field, nx, ny, pitch, plane, N, limit, scratch, nb, norm_out, flag_out, st); break;
        default: e = launch<__nv_bfloat16>(field, nx, ny, pitch, plane, N, limit, scratch, nb, norm_out, flag_out, st);
    }
    if (e != cudaSuccess) {
        snprintf(msg, sizeof msg, "behf_field_norm_noalloc: launch failed: %s", cudaGetErrorString(e));
        behf::report_error(msg);
        return BEHF_ERR_CUDA;
    }
    return BEHF_OK;
}
