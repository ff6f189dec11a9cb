// Device descriptor of one emitter object (the Maxwell-Liouville part of the E half
// step); kernels in emitter_kernels.cu, host set-up in engine.cpp.
#pragma once

#include <cuda_runtime.h>

#include "fdtd_device.hpp"

namespace chiml {
namespace dev {

constexpr int kMaxEmitterLevels = 8;

// Density matrices and their derivative histories are FP64 in every precision form.
// Layout: element e of member m of cell q is at (m * n2 + e) * nc + q, so that the
// threads of a warp (consecutive cells) read consecutive addresses.
struct EmitterDev {
    int N, n2, nm, nc;            // levels, N*N, ensemble members, emitter cells
    const double* h0;             // [nm][N] diagonal energies
    const double2* mu;            // [3][n2] coupling-scaled dipole operators
    const double2* negMu;         // [3][n2] their negatives
    int addMu[3];                 // operator c has a nonzero element
    int comp[3];                  // component c is coupled
    int gatherZCopy;              // Ez gathered by copy (2-D TMz)
    const int* gamRow;            // relaxation rows, CSR: [n2 + 1]
    const int* gamCol;
    const double* gamVal;
    double dt, hbar, na;
    // Hermitian form: real symmetric dipole operators and a relaxation that maps element
    // pairs onto conjugate pairs; the update then needs only the upper triangle
    int herm;
    unsigned hmask;               // Hermitian form: elements of H that can be nonzero (bit i, i < 32)
    // ABM4 step weights (predictor 55, -59, 37, -9; corrector 9, 19, -5, 1, each x dt/24)
    // and 1/hbar, formed once on the host: FP64 division is slow on this GPU
    double abP[4], abC[4], invHbar;
    const long long* cellGrid;    // [nc] grid index of each cell
    // per-cell dipoles (extension): the operator of cell q is w_q * (the z operator), w as
    // [3][nc]; null for the object's operators everywhere. The coupling uses E . w with
    // the z operator, and P_c = w_c * (the z polarisation)
    const double* cellDip;
    const int* cellP;             // [nc] P-box index of each cell
    long long unit[3];            // grid index step along x, y, z
    double2* rho;                 // [nm * n2 * nc]
    double2* kd;                  // 4 slots of derivatives, slot stride nm * n2 * nc
    double* P;                    // [3][pBox] polarisation per component
    const double* negHalfInvEps;  // [pBox] -0.5 / eps at the P-box points (eps the relative permittivity)
    int pDims[3], addN[3], boxBase[3], zOff;
    int lx, lz;                   // grid extents for P-box -> grid indices
    int pBox;
    // outputs
    int nDtc;
    const int* dtcLev;
    int dtcTimeInt;
    double nPoints;               // emitter points (population normalisation)
    double2* popPartial;          // [blocks][nDtc]
    double* totPartial;           // [blocks][3]
    int partialBlocks;
    double2* pop;                 // [nDtc][nEvents]
    int nEvents;
    double* totP;                 // [3][nSteps], null when the polarisation is not written
    int nSteps;
    // Split form of the Hermitian update (FP32 fields): the density matrices as float-float
    // pairs (hi + lo, a 48-bit significand), the derivative histories in FP32, the level
    // energy differences (h0_i - h0_j) / hbar as float-float pairs, the coupling and the
    // relaxation in FP32. Set when the fields are FP32 and the Hermitian form applies.
    int split;
    float4* rhoF;                 // [nm * n2 * nc] (re hi, re lo, im hi, im lo), layout as rho
    float2* kdF;                  // 4 slots of derivatives, layout as kd
    const float2* dlevF;          // [nm][n2] (h0_i - h0_j) / hbar at element i + j N, hi/lo
    const float* negMuHF;         // [3][n2] Re(-mu) / hbar
    const float* gamValF;         // relaxation values (CSR of gamRow / gamCol)
    float abPf[4], abCf[4];       // ABM4 weights in FP32
};

// P into E on the (n+1)-box (addP), then one density update of every cell and member
// (updateDensity) and the output reductions. `step` is the device step counter, equal
// to the number of completed steps when these run.
template <typename T>
void launch_emitter_step(const EmitterDev& e, T* const fields[3], const int* step, void* stream);

// The same step for the emitter objects of many simulations (the batched sweep): the
// addP launch and one density-update launch per group (general form for 2, 3, 4 levels
// and other; Hermitian form for 2, 3, 4 levels), each over the packed blocks of its jobs,
// then one reduce block per job.
template <typename T>
struct EmitJob {
    EmitterDev e;
    T* f[3];
    const int* step;
};
// addP blocks per component (3 components per job)
__host__ __device__ inline int emitter_addp_blocks_per_comp(const EmitterDev& e) {
    return (e.addN[0] * e.addN[1] * e.addN[2] + 255) / 256;
}
int emitter_update_blocks(const EmitterDev& e);
int emitter_level_group(int N, bool herm);               // update group: 0..3 general (N = 2, 3, 4, other), 4..6 Hermitian (N = 2, 3, 4)
template <typename T>
void launch_emitter_packed(const EmitJob<T>* jobs, int njobs, WorkMap addp, const WorkMap update[7], void* stream);

}  // namespace dev
}  // namespace chiml
