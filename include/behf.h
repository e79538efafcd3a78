/*
 * behf.h -- C ABI of the GB300 BEHF poroelastic time stepper (libbehf.so).
 *
 * The reference drives its GPU through one call,
 *     void callCUDAKernel(blockInfo*, nxt, nyt, nzt, DT, F0, sn, coord, ..., NT)   (kernel.cu:1728,
 *     declared main.cpp:59),
 * after main.cpp has built the medium, the coefficients and the CPML profiles on the host and
 * copied ~99 device arrays into a blockInfo (main.cpp:1529-1743).  That call then runs the whole
 * time loop, samples txx along one line every step and writes the output files itself.
 *
 * This header splits that boundary into setup, run and output calls over an opaque context.
 * Every call returns a behf_status and never exits the process (the reference's CUDA_CHECK calls
 * exit(), kernel.cu:42-52).  A context is single-thread affine and owns one CUDA stream; separate
 * contexts may be driven from separate threads.  A context lives on the device that was current
 * when it was created: each call on it makes that device current for the call and restores the
 * caller's device afterwards, so contexts on several GPUs can be driven from one process.  All host pointers are copied; the caller keeps
 * ownership.  Arrays are C order [nz][ny][nx] (x fastest), as the reference's
 * offset = ix + iy*nxt + iz*nxt*nyt (kernel.cu:162).
 */
#ifndef BEHF_H
#define BEHF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int behf_status;
#define BEHF_OK 0
#define BEHF_ERR_INVALID (-1)   /* bad argument or size */
#define BEHF_ERR_CUDA (-2)      /* a CUDA runtime call failed */
#define BEHF_ERR_ALLOC (-3)     /* device or host allocation failed */
#define BEHF_ERR_STATE (-4)     /* call out of order (e.g. run before the medium is set) */
#define BEHF_ERR_NONFINITE (-5) /* the health check found a NaN/Inf or an overflow in a field */
#define BEHF_ERR_UNSUPPORTED (-6)
#define BEHF_ERR_TIMEOUT (-7)   /* a kernel's bounded pipeline wait gave up; results of that run are invalid */

/* Storage precision of the wavefields (arithmetic is FP32 for the 16/32-bit kinds, FP64 for FP64). */
typedef enum { BEHF_FP64 = 0, BEHF_FP32 = 1, BEHF_FP16 = 2, BEHF_BF16 = 3 } behf_precision;

/* Field indices: solid velocity, Darcy flux, the six stresses, pore pressure.
 * Reference names: vux vuy vuz vwx vwy vwz txx tyy tzz txy txz tyz ss (common.h:10-12). */
enum {
    BEHF_VX = 0, BEHF_VY, BEHF_VZ, BEHF_QX, BEHF_QY, BEHF_QZ,
    BEHF_SXX, BEHF_SYY, BEHF_SZZ, BEHF_SXY, BEHF_SXZ, BEHF_SYZ, BEHF_P, BEHF_NFIELD
};

/* Cell-centred moduli, the outputs of the reference's create_model_all (outputfunc.cpp:153-222):
 * rho, rho_f, mu, M, C (= alpha M), H (= lambda_u + 2 mu), lambda_u (H2u), b = eta/kappa (C1),
 * m = (1 + 2/8) tau rho_f / phi (C2). */
enum { BEHF_RHO = 0, BEHF_RHOF, BEHF_MU, BEHF_M, BEHF_C, BEHF_HH, BEHF_H2U, BEHF_C1, BEHF_C2, BEHF_NMOD };

/* Source kinds.  EXPLOSIVE adds the wavelet to txx, tyy, tzz before the velocity update, as the
 * reference's Source kernel does (kernel.cu:130-142).  PRESSURE adds it to the pore pressure.
 * FORCE_Z adds wavelet * dt / rho_z to vz after the velocity update (a body-force density). */
typedef enum { BEHF_SRC_EXPLOSIVE = 0, BEHF_SRC_PRESSURE = 1, BEHF_SRC_FORCE_Z = 2 } behf_source_kind;

typedef struct {
    int nx, ny, nz;          /* grid incl. CPML cells and the never-updated ghost ring of width radius */
    double h;                /* grid spacing (m); the reference hard-codes 1/h = 100 (kernel.cu:158) */
    double dt;               /* time step (s) */
    int radius;              /* staggered stencil half-width R, 1..4 (order 2R; the reference is R = 1) */
    int cpml_width;          /* CPML cells per face L (reference NP, main.cpp:23); 0 = none */
    double cpml_v0;          /* profile velocity (reference v0 = 4000, main.cpp:558) */
    double cpml_r;           /* target reflection (reference RC = 1e-6, main.cpp:88) */
    double scales[4];        /* per-field storage scales s_v, s_q, s_sigma, s_p; all 0 = automatic */
    double src_amp_hint;     /* automatic scales: expected wavelet peak (0 = 1) */
    double src_f0_hint;      /* automatic scales: dominant frequency in Hz (0 = 30) */
} behf_grid;

typedef struct behf_ctx behf_ctx;

typedef struct {
    int64_t step;            /* steps taken since the last reset */
    int64_t device_bytes;    /* bytes this context holds on the device */
    double scales[4];        /* scales in use */
    double bytes_per_cell;   /* algorithmic HBM bytes of one cell update (state + coefficients + CPML) */
    int kernel;              /* kernel family in use (behf_kernel) */
    int radius, precision;
    int64_t launches;        /* kernels enqueued by this context so far (graph launches count their nodes) */
    int tiled_variant;       /* tiled kernels in use: 1 classic, 2 warp-specialised, 3 warp-specialised + TMEM z,
                                4 the same + x-slab CPML memory by TMA */
    int zchunk;              /* z planes per CTA requested for the tiled kernels (0 = automatic) */
    int tile_rows;           /* rows per tile of the tiled kernels (8 or 4) */
} behf_info;

/* Kernel family: PLAIN = one thread per cell with cached neighbour loads; TILED = the z-marching
 * shared-memory kernel (FP16/BF16/FP32, R = 4 and R = 1).  AUTO picks TILED where it exists. */
typedef enum { BEHF_KERNEL_AUTO = 0, BEHF_KERNEL_PLAIN = 1, BEHF_KERNEL_TILED = 2 } behf_kernel;

/* Options for behf_set_option. */
enum {
    BEHF_OPT_KERNEL = 0,         /* behf_kernel */
    BEHF_OPT_REF_BUG_COMPAT = 1, /* 1: vz Darcy update uses the y-staggered VW3 as kernel.cu:220 does */
    BEHF_OPT_GRAPH_CHUNK = 2,    /* steps per captured CUDA graph (0 = no graph) */
    BEHF_OPT_GRADIENT = 3,       /* 1: keep the cell-centred moduli on the device (9 x 4 B per cell) so that
                                    behf_gradient can map coefficient gradients to moduli; set before the medium */
    BEHF_OPT_CHECKPOINT = 4,     /* steps between checkpoints of the gradient's forward pass (0 = round(sqrt(nt))) */
    BEHF_OPT_ZCHUNK = 5,         /* tiled kernels: z planes each CTA marches (0 = automatic: at most 64, fewer when
                                    needed to give every SM work) */
    BEHF_OPT_COEF_ROUNDING = 6,  /* FP16/BF16 kinds, set before the medium: 0 coefficients rounded to nearest,
                                    1 unbiased (hash-dithered) rounding that removes the wave-speed bias of
                                    coherent rounding in homogeneous regions */
    BEHF_OPT_STATE_ROUNDING = 7, /* FP16/BF16 kinds, tiled kernels: 0 fields stored rounded to nearest, 1 stochastic
                                    rounding (seeded by step, field and cell), which keeps increments smaller than
                                    half a unit in the last place in expectation instead of dropping them */
    BEHF_OPT_SNAPSHOT_CACHE = 8, /* gradient: device memory for keeping the forward pass's per-step snapshots of the
                                    last checkpoint segments, which then need no recompute (-1 = automatic: the free
                                    memory but max(8 GiB, 10 % of the device); 0 = none; n > 0 = at most n MiB) */
    BEHF_OPT_CHECKPOINT_OUTER = 9, /* gradient: outer checkpoint spacing of the two-level scheme, rounded up to a
                                    multiple of BEHF_OPT_CHECKPOINT (0 = automatic: one level when it fits the
                                    device memory, else two levels with the inner spacing halved until they fit) */
    BEHF_OPT_TILED_VARIANT = 10, /* tiled kernels: 0 = automatic (4 for FP16 / BF16, 2 for FP32), 1 = classic (own-cell data by direct loads of the
                                    compute threads), 2 = warp-specialised (a producer warp brings every input,
                                    own-cell data included, through TMA), 3 = warp-specialised with the z derivatives
                                    accumulated plane by plane in tensor memory (TMEM), 4 = 3 with the CPML memory
                                    and damping profiles of the x-edge tiles' slab cells also brought by TMA (as 3
                                    where an x-edge tile's slab cells do not fit its box) */
    BEHF_OPT_GRAD_COMPENSATION = 11, /* gradient with an FP32 adjoint (16/32-bit kinds): the coefficient-gradient
                                    accumulators sum each checkpoint segment in FP32, then fold it into running
                                    totals: 1 = Neumaier-compensated FP32 totals (default), 0 = no fold (plain FP32
                                    accumulation over all steps), 2 = FP64 totals (reference for the error) */
    BEHF_OPT_TILE_ROWS = 13,     /* tiled kernels: rows per tile (each a warp), 0 = automatic (8), 8 or 4 (64 x 4 tiles: four
                                    compute warps and a producer per CTA, up to four CTAs per SM); the autotuner
                                    times both */
    BEHF_OPT_RECOMPUTE_OVERLAP = 12, /* gradient, one checkpoint level: 1 = the recompute of the next segment from its
                                    checkpoint runs on a second stream, into a second snapshot buffer, while the
                                    current segment's adjoint steps run (default; only when the second buffer fits
                                    the free device memory less max(2 GiB, 2 %)), 0 = one after the other.  The
                                    results are the same bit for bit. */
};

/* Create a context; allocates the wavefields, coefficients and CPML slab memory on the current
 * device.  Replaces main.cpp:1529-1627 (cudaMalloc of the blockInfo arrays). */
behf_status behf_create(const behf_grid* grid, int precision, behf_ctx** out);
behf_status behf_destroy(behf_ctx* ctx);

/* Medium from host arrays (copied), moduli[BEHF_NMOD] each [nz][ny][nx] float.  Builds the staggered
 * coefficients on the device.  Replaces main.cpp:322-494 (averaging + coefficients), 1482-1526
 * (FP16 conversion) and 1640-1743 (H2D copies). */
behf_status behf_set_medium(behf_ctx* ctx, const float* const moduli[BEHF_NMOD]);
/* Same, from device arrays (not freed, not kept). */
behf_status behf_set_medium_device(behf_ctx* ctx, const float* const moduli[BEHF_NMOD]);

/* Synthetic media generated on the device (no host volumes).  A rock is the parameter set of the
 * reference's create_model_all (outputfunc.cpp:153-222); phi >= 1 marks pure fluid. */
typedef struct {
    double Ks, Kf, Kdry, mu, rhos, rhof, phi, kappa, eta, tau;
} behf_rock;

typedef struct {
    int nlayers;                 /* 1..4 layers in z */
    behf_rock layers[4];
    int interface_z[3];          /* layer l spans [interface_z[l-1], interface_z[l]) cells */
    int seed;                    /* perturbation seed (0 .. 2^20-1) */
    double corr_cells;           /* correlation length exp(-r^2/l^2) in cells */
    double pct;                  /* relative std of K_dry, mu, phi (0 = no perturbation) */
    double log_kappa_sigma;      /* std of ln kappa */
    int anomaly;                 /* 1: Gaussian anomaly exp(-r^2/R^2) */
    double anom_center[3];       /* cell coordinates (x, y, z) */
    double anom_radius_cells;
    double anom_dkdry;           /* K_dry *= 1 + anom_dkdry G */
    double anom_kappa_factor;    /* kappa *= anom_kappa_factor^G */
} behf_medium_spec;

/* Build the moduli of a synthetic medium on the device, then the coefficients (as behf_set_medium).
 * The noise is splitmix64-hashed per (cell, field, seed), Box-Muller in FP64, smoothed by a periodic
 * separable Gaussian of std l/2 and scaled to unit variance. */
behf_status behf_generate_medium(behf_ctx* ctx, const behf_medium_spec* spec);

/* Explicit 1-D CPML profiles for one axis (0 = x, 1 = y, 2 = z), n entries each: damping d at the
 * integer points and d2 at the half-shifted points (1/s).  Overrides the profile built from
 * cpml_width/v0/r (main.cpp:519-1371).  Call before behf_set_medium or behf_reset. */
behf_status behf_set_cpml_profile(behf_ctx* ctx, int axis, const double* d, const double* d2);

/* Source at cell (ix, iy, iz) with wavelet[nt] (host, copied).  Steps past nt inject nothing.
 * Replaces the Ricker/Source pair of kernel.cu:1898,2064-2071 (host value + full-grid launch). */
behf_status behf_set_source(behf_ctx* ctx, int kind, int ix, int iy, int iz, const float* wavelet, int nt);

/* Receivers: ijk[3*nrec] cell indices (ix, iy, iz), comp[nrec] field indices.  Sampled on the
 * device after every step into an FP64 [nrec][capacity] buffer; replaces the per-step full-volume
 * D2H copy and host pick of kernel.cu:2197-2243. */
behf_status behf_set_receivers(behf_ctx* ctx, int nrec, const int* ijk, const int* comp, int capacity);

/* Advance nsteps time steps (Source -> V -> T -> receivers each step, kernel.cu:2064-2192 order).
 * behf_run waits for completion; behf_run_async only enqueues on the context's stream. */
behf_status behf_run(behf_ctx* ctx, int nsteps);
behf_status behf_run_async(behf_ctx* ctx, int nsteps);
behf_status behf_sync(behf_ctx* ctx);

/* Replace wavelet samples [it0, it0+n) (host, copied; extends the wavelet if needed).  With
 * behf_get_seismograms_range this streams a run step by step from and to host memory. */
behf_status behf_update_wavelet(behf_ctx* ctx, int it0, const float* w, int n);
/* Seismogram columns [it0, it0+n) of every receiver, physical units, [nrec][n] into out (host). */
behf_status behf_get_seismograms_range(behf_ctx* ctx, int it0, int n, double* out);

/* Advance nsteps with direct launches, timing every launch with CUDA events on the context's
 * stream; ms[4] receives the mean duration (ms) of the source, velocity, stress and receiver
 * kernels.  For roofline accounting. */
behf_status behf_time_kernels(behf_ctx* ctx, int nsteps, double* ms);

/* Seismograms recorded so far, physical units, [nrec][nsteps_recorded] into out (host). */
behf_status behf_get_seismograms(behf_ctx* ctx, double* out, int* nsteps_recorded);
/* One field in physical units, [nz][ny][nx] float (host).  For wfile3d-style snapshots. */
behf_status behf_get_field(behf_ctx* ctx, int field, float* out);
behf_status behf_set_field(behf_ctx* ctx, int field, const float* in);
/* Zero wavefields, CPML memory and seismograms; step = 0.  Keeps medium, source and receivers. */
behf_status behf_reset(behf_ctx* ctx);

behf_status behf_set_option(behf_ctx* ctx, int option, int value);
behf_status behf_get_info(behf_ctx* ctx, behf_info* out);
/* The context's cudaStream_t, for event timing by the caller. */
behf_status behf_get_stream(behf_ctx* ctx, void** stream);

/* Health check (energy-norm reduction in FP64 over every field, on the device): writes the sum of
 * squares of each field in storage units to norms[BEHF_NFIELD] and returns BEHF_ERR_NONFINITE if any
 * value is NaN/Inf or saturates the storage format (reaches its largest finite value: 65504 for FP16,
 * (2 - 2^-7) 2^127 for BF16); flagged values are left out of the sums.  The reference has no counterpart (it prints
 * or ignores errors, kernel.cu:1926-1929). */
behf_status behf_health(behf_ctx* ctx, double* norms);

/* Energy norm and health flag of one field, without allocating any device memory.  No counterpart
 * in the reference.  For callers that cannot allocate: a host application that owns all device
 * memory through its own pool (nothing left for cudaMalloc), or a monitoring thread that checks a
 * running simulation and must not stall the device with cudaFree.
 *   field      device array of `precision` values laid out [nz][ny][pitch] with plane stride `plane`
 *   norm_out   device double: sum of squares of the nx*ny*nz values (the storage units of the field); values
 *              that set the flag are left out of it, as behf_health leaves them out
 *   flag_out   device int: 1 if any value is NaN/Inf or at the top of the storage range (65504 for FP16,
 *              (2 - 2^-7) 2^127 for BF16, FLT_MAX / DBL_MAX for FP32 / FP64), else 0
 *   stream     cudaStream_t to run on (NULL: the default stream); the call does not synchronize
 * Fields up to 2^30 cells (1024^3); larger sizes are rejected with BEHF_ERR_INVALID.  Scratch is a
 * fixed 512 KiB device array inside the library, held by every GPU that loads it until exit.  The
 * first call on each device looks up that array's address: make it before any stream capture.  All
 * calls share the array, so calls that overlap on the GPU race. */
behf_status behf_field_norm_noalloc(const void* field, int precision, int nx, int ny, int nz, long long pitch,
                                    long long plane, double* norm_out, int* flag_out, void* stream);

/* Adjoint-state gradient (no counterpart in the reference, which has no adjoint).  Runs the forward from rest
 * over nt steps with checkpoints every BEHF_OPT_CHECKPOINT steps (full state: fields + CPML memory), then the
 * exact discrete adjoint of the same steps backwards, recomputing one segment at a time from its checkpoint.
 *   adj_src        [nrec][nt] host: dJ/d seismogram sample, physical units (the adjoint source)
 *   grad_wavelet   [nt] host or NULL: dJ/d wavelet sample
 *   grad_moduli    BEHF_NMOD host arrays [nz][ny][nx] (entries may be NULL): dJ/d cell-centred modulus, exact
 *                  on cells whose staggered coefficient cells lie outside the CPML slabs and the ghost ring
 *                  (the absorbing layers are not inverted), zero elsewhere.
 * Needs BEHF_OPT_GRADIENT before the medium, a source, and receivers of capacity >= nt.  The adjoint runs in
 * the context's arithmetic type (FP32 for the 16-bit kinds, FP64 for FP64).  Afterwards the seismograms are
 * those of the forward pass (behf_get_seismograms); the wavefields are not meaningful (behf_reset). */
behf_status behf_gradient(behf_ctx* ctx, int nt, const double* adj_src, double* grad_wavelet,
                          double* const grad_moduli[BEHF_NMOD]);
/* Same for the L2 misfit J = 1/2 sum (seis - observed)^2 (observed [nrec][nt] host, physical units): the
 * adjoint source is the residual of the forward pass; J is written to *misfit. */
behf_status behf_misfit_gradient(behf_ctx* ctx, int nt, const double* observed, double* misfit,
                                 double* grad_wavelet, double* const grad_moduli[BEHF_NMOD]);

/* Biot's physical parameters of behf_physical_gradient: the drained Lame parameter lambda, the shear modulus mu,
 * the bulk density rho, the fluid density rho_f, the Biot modulus M, the Biot coefficient alpha and the
 * permeability kappa. */
enum { BEHF_PH_LAMBDA = 0, BEHF_PH_MU, BEHF_PH_RHO, BEHF_PH_RHOF, BEHF_PH_M, BEHF_PH_ALPHA, BEHF_PH_KAPPA, BEHF_NPHYS };

/* Chain rule from the moduli gradients of behf_gradient / behf_misfit_gradient to the physical parameters (no
 * counterpart in the reference, which has no adjoint).  Host arithmetic only, cell by cell over ncell cells.
 * The moduli relate to the parameters as the reference's create_model_all builds them (outputfunc.cpp:202-217):
 * C = alpha M, lambda_u = lambda + alpha^2 M, H = lambda_u + 2 mu, b = eta / kappa, m = (m / rho_f) rho_f, with eta
 * and m / rho_f = (1 + 2/8) tau / phi held fixed per cell.
 *   moduli        BEHF_NMOD host arrays [ncell] float (the medium passed to behf_set_medium); rho_f, M, C, b, m
 *                 are required
 *   grad_moduli   BEHF_NMOD host arrays [ncell] double (NULL entries count as zero)
 *   eta           fluid viscosity (Pa s; the reference's 1e-3, outputfunc.cpp:166)
 *   grad_phys     BEHF_NPHYS host arrays [ncell] double, dJ / d parameter (NULL entries are skipped) */
behf_status behf_physical_gradient(long long ncell, const float* const moduli[BEHF_NMOD],
                                   const double* const grad_moduli[BEHF_NMOD], double eta,
                                   double* const grad_phys[BEHF_NPHYS]);

/* Autotuner (no counterpart in the reference, which fixes its 16 x 8 block, kernel.cu:17-19): times trial_steps
 * steps for each tile height (BEHF_OPT_TILE_ROWS 8 and 4), tiled-kernel variant (BEHF_OPT_TILED_VARIANT 1..4) and
 * z-chunk length (BEHF_OPT_ZCHUNK
 * candidates 0, 16, 32, ... up to the grid), keeps the fastest, and resets the wavefields (behf_reset).
 * Writes the chosen z-chunk and its milliseconds per step; the chosen variant and height are in
 * behf_info.tiled_variant and behf_info.tile_rows. */
behf_status behf_autotune(behf_ctx* ctx, int trial_steps, int* zchunk_out, double* ms_per_step_out);

/* Batched shots on one GPU (no counterpart in the reference): advances n independent contexts by nsteps each,
 * enqueuing graph-chunk-sized pieces round-robin on their own streams so the shots overlap on the device, then
 * waits for all.  Equivalent to behf_run on each context in turn. */
behf_status behf_run_batch(behf_ctx* const* ctxs, int n, int nsteps);

/* Checkpoint plan of behf_gradient (host arithmetic only, no context or device): the inner spacing (steps between
 * the checkpoints that are recomputed with per-step snapshots) and the outer spacing (== inner: one level; a
 * multiple of it: two levels, each outer segment run forward again for its inner checkpoints) of a gradient over
 * nt steps, and the device bytes they take.  checkpoint / checkpoint_outer are BEHF_OPT_CHECKPOINT /
 * BEHF_OPT_CHECKPOINT_OUTER (0 = automatic: inner round(sqrt(nt)); two levels only when one needs more than
 * avail bytes, the inner spacing then halving until the outer spacing that needs the least memory fits).
 * ck_bytes / snap_bytes: one checkpoint (13 fields + CPML memory) / one snapshot (13 fields); fixed_bytes: the
 * rest that scales with nt (the adjoint source).  behf_gradient calls it with the free device memory less
 * max(2 GiB, 2 %). */
behf_status behf_checkpoint_plan(int nt, int checkpoint, int checkpoint_outer, size_t ck_bytes, size_t snap_bytes,
                                 size_t fixed_bytes, size_t avail, int* inner, int* outer, size_t* bytes);

/* Self-test of failure detection (no counterpart in the reference): launches on the context's stream one block
 * that waits, with the bounded wait of the TMA pipelines (about 2 s), on a barrier that nothing releases, then
 * syncs.  Returns BEHF_ERR_TIMEOUT, as behf_sync does after a pipeline wait gave up; the context stays usable
 * (the error word is cleared). */
behf_status behf_selftest_wait(behf_ctx* ctx);

/* Text of the last error on this thread. */
const char* behf_last_error(void);
/* Library version string. */
const char* behf_version(void);

#ifdef __cplusplus
}
#endif
#endif
