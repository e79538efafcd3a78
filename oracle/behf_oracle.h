/*
 * behf_oracle.h -- CPU oracle for the BEHF poroelastic staggered-grid time stepper.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a CPU restatement of the reference's update
 * equations, used as the checker for the CUDA path (tests, the smoke check and the
 * CPU-baseline leg of the benchmark).  The product path never links or calls it.
 *
 * What it restates (reference file:line):
 *   medium        outputfunc.cpp:153-222  (create_model_all: Biot-Gassmann moduli)
 *   averaging     main.cpp:322-359        (harmonic mu, arithmetic rho/rhof/C1/C2)
 *   coefficients  main.cpp:431-494        (VW1/2/3, VU1/2, P1/2, S1/2/3, Sxy/xz/yz)
 *   CPML profile  main.cpp:519-563        (quadratic d(x), half-shifted d2, e = exp(-d dt))
 *   V update      kernel.cu:145-229       (FD_Vtop; Vmid/Vbottom differ only in the z guard)
 *   T update      kernel.cu:405-493       (FD_Ttop)
 *   source        kernel.cu:130-142, 1898 (Source, Ricker wavelet)
 *   step order    kernel.cu:2064-2192     (Source -> V -> T -> record)
 *
 * Two modes:
 *   - orc_run:     the BEHF scheme as the CUDA library implements it (stencil radius 1..4,
 *                  per-field scales, CPML confined to slabs).  Storage precision is emulated
 *                  (FP64, FP32, FP16, BF16) so the FP64 run is the parity target and the
 *                  FP16 run predicts the GPU's FP16 rounding.
 *   - orc_ref_run: the reference kernels' exact arithmetic (radius 1, every array in FP16,
 *                  double-promoted update expressions, 1/h literal 100), checked bit for bit
 *                  against the reference kernel bodies compiled on the CPU.
 */
#ifndef BEHF_ORACLE_H
#define BEHF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Field order (shared with the CUDA library). */
enum { ORC_VX = 0, ORC_VY, ORC_VZ, ORC_QX, ORC_QY, ORC_QZ,
       ORC_SXX, ORC_SYY, ORC_SZZ, ORC_SXY, ORC_SXZ, ORC_SYZ, ORC_P, ORC_NFIELD };
/* Cell-centred moduli order (create_model_all outputs). */
enum { ORC_RHO = 0, ORC_RHOF, ORC_MU, ORC_M, ORC_C, ORC_HH, ORC_H2U, ORC_C1, ORC_C2, ORC_NMOD };
/* Staggered coefficient order (main.cpp:431-494). */
enum { ORC_VW1X = 0, ORC_VW1Y, ORC_VW1Z, ORC_VW2X, ORC_VW2Y, ORC_VW2Z, ORC_VW3X, ORC_VW3Y, ORC_VW3Z,
       ORC_VU1X, ORC_VU1Y, ORC_VU1Z, ORC_VU2X, ORC_VU2Y, ORC_VU2Z,
       ORC_P1, ORC_P2, ORC_S1, ORC_S2, ORC_S3, ORC_SXYC, ORC_SXZC, ORC_SYZC, ORC_NCOEF };
/* Storage precisions. */
enum { ORC_F64 = 0, ORC_F32 = 1, ORC_F16 = 2, ORC_BF16 = 3 };
/* Source kinds. */
enum { ORC_SRC_EXPLOSIVE = 0, ORC_SRC_PRESSURE = 1, ORC_SRC_FORCE_Z = 2 };

typedef struct {
    int nx, ny, nz;          /* grid incl. CPML and the zero ghost ring of width radius */
    int radius;              /* staggered stencil half-width R (1..4): order 2R */
    double h, dt;            /* spacing (m), step (s) */
    int precision;           /* ORC_F64 .. ORC_BF16: storage precision emulated */
    int ref_bug_compat;      /* 1: vz Darcy update uses VW3y (kernel.cu:220), as the reference does */
    int cpml_width;          /* L: profile active on [0,L) and [n-1-L, n) per axis */
    double cpml_v0, cpml_r;  /* d0 = 3 v0 ln(1/R) / (2 L h) */
    double scale[4];         /* per-field scales: s_v, s_q, s_sigma, s_p (1,1,1,1 = physical) */
    int src_kind, src_ix, src_iy, src_iz;
    double src_factor;       /* FORCE_Z only: velocity increment per unit wavelet (dt/rho_z) */
    int nthreads;            /* OpenMP threads (<=0: all) */
    int time_from_step;      /* orc_last_step_seconds covers steps [time_from_step, nt) */
} orc_cfg;

/* Reference borehole medium (outputfunc.cpp:153-222), cell-centred, float [nz][ny][nx]. */
void orc_medium_borehole(int nz, int ny, int nx, float* const mod[ORC_NMOD]);

/* Biot-Gassmann moduli of one rock (outputfunc.cpp:202-217) written to cell `i` of mod[]. */
void orc_rock_moduli(double Ks, double Kf, double Kdry, double mu, double rhos, double rhof,
                     double phi, double kappa, double eta, double tau, double out[ORC_NMOD]);

/* Physical staggered coefficients (double, [nz][ny][nx]) from the moduli (main.cpp:322-494). */
void orc_build_coeffs(int nx, int ny, int nz, double dt, const float* const mod[ORC_NMOD],
                      double* const coef[ORC_NCOEF]);

/* 1-D CPML profile of one axis: d, d2 (half-shifted), e = exp(-d dt), e2.  Zero off the slabs. */
void orc_cpml_profile(int n, int L, double h, double dt, double v0, double rc,
                      double* d, double* d2, double* e, double* e2);

/* Ricker wavelet of kernel.cu:1898 in double: w[it] = amp * -(1-2 pi^2 f^2 tau^2) exp(-pi^2 f^2 tau^2),
 * tau = it*dt - t0. */
void orc_ricker(int nt, double dt, double f0, double t0, double amp, float* w);

/* BEHF run.  mod: cell-centred moduli; wavelet[nt]; receivers rec_ijk[3*nrec] (ix,iy,iz),
 * rec_comp[nrec] (field index).  seis[nrec*nt] receives physical values.  If fields_out is
 * non-NULL it receives the 13 final fields in physical units, [13][nz][ny][nx].
 * Returns 0 on success, negative on invalid input. */
int orc_run(const orc_cfg* cfg, const float* const mod[ORC_NMOD], const float* wavelet, int nt,
            int nrec, const int* rec_ijk, const int* rec_comp, double* seis, double* fields_out);

/* FP64 discrete adjoint of orc_run (behf_adjoint.cpp), physical units (storage scales ignored).
 * Runs the forward from rest with checkpoints every `stride` steps (<= 0: round(sqrt(nt))), then the
 * adjoint with the adjoint source adj_src[nrec*nt] (dJ/d seismogram sample; NULL = zero) added at the
 * receivers.  Outputs (each may be NULL): seis_out[nrec*nt] forward seismograms; grad_wavelet[nt]
 * dJ/d wavelet sample; grad_coef[23*N] dJ/d effective coefficient (physical coefficient times 1/h where
 * it multiplies a difference), accumulated over cells outside every CPML slab; grad_mod[9*N] dJ/d
 * cell-centred moduli, exact on cells whose coefficient cells all lie outside the slabs, else 0.
 * Returns 0, or negative on invalid input. */
int orc_adjoint(const orc_cfg* cfg, const float* const mod[ORC_NMOD], const float* wavelet, int nt,
                int nrec, const int* rec_ijk, const int* rec_comp, const double* adj_src, int stride,
                double* seis_out, double* grad_wavelet, double* grad_coef, double* grad_mod);

/* orc_adjoint with adjoint-state storage emulation: lf_scale[13] (NULL = none) rounds each adjoint field to
 * binary16 times lf_scale[q] after every backward step (an FP16-stored adjoint state; CPML adjoint memory and
 * the gradients stay FP64); lf_max[13] (NULL = none; accumulated into, so zero it first) receives the largest
 * magnitude of each adjoint field over the steps; lf_saturated (NULL = none) counts values that overflowed. */
int orc_adjoint_ex(const orc_cfg* cfg, const float* const mod[ORC_NMOD], const float* wavelet, int nt,
                   int nrec, const int* rec_ijk, const int* rec_comp, const double* adj_src, int stride,
                   double* seis_out, double* grad_wavelet, double* grad_coef, double* grad_mod,
                   const double* lf_scale, double* lf_max, long long* lf_saturated);

/* Wall seconds of the time-step loop of the last orc_run (set-up excluded); OpenMP thread count. */
double orc_last_step_seconds(void);
int orc_threads(void);

/* Reference-arithmetic run (radius 1, FP16 everywhere).  All arrays are [nz][ny][nx] binary16
 * bit patterns.  state[16]: the 13 fields in field order, then vwx2, vwy2, vwz2.
 * coef[23]: the reference's FP16 coefficient arrays (already scaled as main.cpp does).
 * prof[12]: dxi, dxi2, e_dxi, e_dxi2, dyj, dyj2, e_dyj, e_dyj2, dzk, dzk2, e_dzk, e_dzk2 (x Cpml).
 * aux[48]: psi and previous-derivative arrays, V then T, in the order of orc_ref_aux_names.
 * Source adds wavelet[it] to txx, tyy, tzz at linear index sn before each V.  seis[nrec*nt] gets
 * (float) of field rec_comp[r] at linear index rec_lin[r] after each T.  Modified in place. */
int orc_ref_run(int nx, int ny, int nz, float dt, int nt, int sn, const float* wavelet,
                uint16_t* const state[16], const uint16_t* const coef[ORC_NCOEF],
                const uint16_t* const prof[12], uint16_t* const aux[48],
                int nrec, const int* rec_lin, const int* rec_comp, float* seis, int nthreads);

/* Reference FP16 inputs from cell-centred moduli, as main.cpp:322-494 and 519-1526 compute them
 * for a single domain with all six faces absorbing (Cv=1e8, Cp=1, x100 scaling, Cpml=0.01). */
void orc_ref_inputs(int nx, int ny, int nz, float h, float dt, int np, float v0, float rc,
                    const float* const mod[ORC_NMOD], uint16_t* const coef[ORC_NCOEF],
                    uint16_t* const prof[12]);

/* Names of the 48 aux arrays of orc_ref_run (for fixtures). */
const char* orc_ref_aux_name(int i);

/* Binary16 helpers (round-to-nearest-even). */
uint16_t orc_f2h(float x);
float orc_h2f(uint16_t h);

#ifdef __cplusplus
}
#endif
#endif
