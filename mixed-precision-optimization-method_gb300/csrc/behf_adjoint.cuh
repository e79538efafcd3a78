// behf_adjoint.cuh -- discrete adjoint of the BEHF step (adjoint.cu): device pointers and launchers.
//
// The forward step n is  source -> V -> force source -> T -> record,  linear in the state (13 fields in
// storage units + CPML memory).  Its adjoint runs  record^T -> T^T -> force^T -> V^T -> source^T  on
// adjoint fields of the forward arithmetic type A (float, or double for FP64 storage), and accumulates
// the gradient with respect to each effective coefficient (stored value x power-of-two multiplier) on
// cells outside every CPML slab.  The pieces:
//   per cell: adjoints of the derivative groups (7 for T, 6 for V) into tmpT / tmpV, coefficient gradients
//      from the forward snapshot of this step;
//   gather: each field's adjoint takes minus the transposed stencils of the derivative adjoints of its
//      neighbours, each corrected on the fly by the adjoint CPML memory of the neighbour's slab;
//   per slab cell: the adjoint CPML memory update  L = lpsi + lD;  lpsi = A L;  lprev = A B L;
// in two TMA-pipelined z-marching gathers per step (the second also does T^T per cell of the next backward
// step), a slab-only memory kernel and the sparse record^T / source^T launches (adjoint.cu).
#pragma once
#include <cuda.h>

#include "behf_internal.cuh"

namespace behf {

struct AdjPtrs {
    void* lf[kNField];       // adjoint fields, type A, pitched like the forward fields
    void* lpsi[3][8];        // adjoint CPML memory, type A, slab layout of the forward memory
    void* lprv[3][8];
    void* tmpT[7];           // per-cell derivative-group adjoints of T^T and V^T, type A, pitched
    void* tmpV[6];           // (zero off the updated cells)
    void* g[kNCoef];         // gradient accumulators per effective coefficient, type A, pitched
    void* mu[3];             // mu = lq' - VU2 lv' of V^T per cell outside the slabs, type A, pitched (for the
                             // separate gradient kernels)
    const void* cur[kNField];  // forward snapshot of this step after V (and the force source), type S
    const void* qprev[3];    // q before V of this step, type S
    const void* vq1[6];      // vx vy vz qx qy qz after V of step n - 1 (the fused T^T of that step), type S
    int grad;                // accumulate coefficient gradients
    int derived;             // the forward ran the tiled kernels: VW2 = VU2 VW3 c_vw2, S3 = P1 c_s3 (the stored
                             // VW2 and S3 are not read, their gradients go to VU2, VW3 and P1)
    int pf;                  // gathers and gradient kernels: prefetch each cell's own arrays of the next plane into L2
    int vmerge;              // the gradient kernels also do the CPML memory updates of their slab cells
};

// Tensor maps of the twelve staged arrays of one gather (x windows, y windows, z-ring rows; adjoint.cu), and of
// both gathers of a gradient run (built once: the scratch arrays do not move).
struct alignas(64) GatherMaps {
    CUtensorMap m[12];
};
struct alignas(64) AdjMaps {
    GatherMaps t, v;  // T^T gather (tmpT), V^T gather (tmpV)
};

struct AdjScales {
    double s[kNField];       // multiplier of the adjoint source per recorded field (alpha / storage scale)
};

// Encode the gathers' tensor maps for the scratch arrays of `a` (host; cudaErrorNotSupported without the driver's
// tensor-map encoder).
template <class S>
cudaError_t adj_build_maps(const Geom& g, const AdjPtrs& a, AdjMaps* m);
// The gathers of the 16-bit kinds stage forward snapshot fields for the coefficient-gradient stencils through
// tensor maps built per snapshot buffer by adj_build_snap_maps: mt over its stresses and pressure (the T^T gather
// of the step), mv over its velocities and Darcy velocities (the fused T^T of the step before).
template <class S>
bool adj_snap_staged();
// Kernels one adj_step launches (for the host launch count): the gathers, the gradient kernels and the memory
// updates that do not ride in them.
int adj_step_launches(const Geom& g, const AdjPtrs& a, int fuse);
template <class S>
cudaError_t adj_build_snap_maps(const Geom& g, void* const f[kNField], GatherMaps* mt, GatherMaps* mv);
// T^T per cell of the first backward step (after its record^T).
template <class S>
cudaError_t adj_first(const Geom& g, const DevPtrs& p, const AdjPtrs& a, cudaStream_t st);
// Backward step n with T^T per cell of step n done: the T^T gather + V^T, the V^T gather + T-slot memory update
// (+ T^T per cell of step n - 1 with fuse = 1, from a.vq1), the V-slot memory update.  snapT / snapV: the maps of
// a.cur and of the snapshot of step n - 1 (required when adj_snap_staged<S>() and a.grad, else ignored).
template <class S>
cudaError_t adj_step(const Geom& g, const DevPtrs& p, const AdjPtrs& a, const AdjMaps& m, const GatherMaps* snapT,
                     const GatherMaps* snapV, int fuse, cudaStream_t st);
// record^T of step it after a fused T^T of that step: adj_record plus its share of tmpT and of the T-coefficient
// gradients at the receiver cells.
template <class S>
cudaError_t adj_recfix(const Geom& g, const DevPtrs& p, const AdjPtrs& a, const long long* off, const int* comp,
                       int nrec, const double* adj, int nt, int it, const AdjScales& sc, cudaStream_t st);
// record^T: lf[comp[r]][off[r]] += adj[r * nt + it] * sc.s[comp[r]]  (atomic: receivers may share a cell)
template <class S>
cudaError_t adj_record(const AdjPtrs& a, const long long* off, const int* comp, int nrec, const double* adj, int nt,
                       int it, const AdjScales& sc, cudaStream_t st);
// source^T at one cell after the step: force gw[it] = fac * lvz, gfac += w[it] * lvz (it < nw); explosive
// gw[it] = fac * (lsxx + lsyy + lszz); pressure gw[it] = fac * lp.
template <class S>
cudaError_t adj_point(const AdjPtrs& a, long long o, int kind, double fac, const float* w, int nw, int it, double* gw,
                      double* gfac, cudaStream_t st);

// Coefficient-build transpose (main.cpp:322-494 formulas): moduli gradient gm[9][nz][ny][nx] (double,
// unpitched) from the effective-coefficient gradients g[] (ratio[] = effective / physical coefficient),
// zero outside the cells whose coefficient cells c - {0,1}^3 all carry gradients.
struct GradModArgs {
    const float* mod[kNMod];
    const void* g[kNCoef];
    double ratio[kNCoef];
    double* gm[kNMod];
    int nx, ny, nz, R, L;
    long long px, plane;
    double dt;
};
template <class A> cudaError_t adj_grad_moduli(const GradModArgs& a, cudaStream_t st);

// Compensated summation of the FP32 coefficient-gradient accumulators.  The backward steps of one checkpoint
// segment add into g[] (FP32) as before; at the segment's end adj_fold moves each g[q][i] into a running total
// and zeroes it: mode 1 Neumaier-compensated FP32 (tot += g with the lost low-order part kept in comp), mode 2
// an FP64 total (the reference for measuring the accumulation error).  final = 1 writes tot + comp (mode 1) or the
// rounded FP64 total (mode 2) back into g[] for the moduli transpose.
struct AdjFold {
    float* g[kNCoef];
    float* tot[kNCoef];
    float* comp[kNCoef];
    double* tot64[kNCoef];
    int mode;
};
cudaError_t adj_fold(const AdjFold& f, long long n, int final, cudaStream_t st);

}  // namespace behf
