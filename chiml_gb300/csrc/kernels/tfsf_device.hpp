// Device descriptor of one TFSF surface: the 1-D incident lines (complex FP64), their
// CPML psi lists, the pulse table and the surface corrections. Kernels in
// tfsf_kernels.cu, host set-up in engine.cpp.
#pragma once

#include <cuda_runtime.h>

namespace chiml {
namespace dev {

constexpr int kTfsfMaxPsi = 4;
constexpr int kTfsfRowChunk = 256;  // cells of a correction row per block (the block size)

// The curl run of a line: U[indI + r] += pj (J[posK + r] - J[negK + r])
// + pk (K[posJ + r] - K[negJ + r]) for r < n.
struct TfsfRunDev {
    int indI, n, posJ, negJ, posK, negK;
    double pj, pk;
};

// One CPML psi list of a line: psi = b psi + c N[loc + d] + cOff N[locOff + d],
// U[gridLoc + d] += Db psi, for d < n; N is line nbr (of the same grid kind).
struct TfsfPsiDev {
    int nbr, loc, locOff, gridLoc, n;
    double Db;
    const double* b;
    const double* c;
    const double* cOff;
    double2* psi;
};

// A line: its incident grid and its pulse grid. Where eps = mu = 1 and there are no
// poles D / B equals the field (division by 1 is exact) and U holds both (D null). A
// line in layered material keeps D apart: per element the poles move first
// (P = alpha P + xi P_prev + gamma U, U of the previous step), the curl goes to D, then
// U = D / eps - sum_p P_p / eps.
struct TfsfLineDev {
    int present, useJ, useK, nbrJ, nbrK;
    double2 prefact;
    double2* U;    // [gridLen]
    double2* pul;  // [pulseLen]
    double2* D;    // [gridLen] or null
    const double* eps;  // [gridLen]: eps of each element (the D lines and the division of surface terms)
    int nPole;
    double2* P;      // [nPole][gridLen]
    double2* Pprev;  // [nPole][gridLen]
    const double* pa;  // [nPole][gridLen] alpha, xi, gamma (zero past an element's poles)
    const double* px;
    const double* pg;
    TfsfRunDev run, pulseRun;
    int nPml, nPmlPulse;
    TfsfPsiDev pml[kTfsfMaxPsi], pmlPulse[kTfsfMaxPsi];
    int recIdx, recOffIdx;
};

// A surface row: toD sends it to the D field of comp; div >= 0 divides each value by
// eps of line div at the same incident index first.
struct TfsfSegDev {
    long long cell0, cellStride;
    int incd0, incdStride, n, line, comp, toD, div;
    double pref;
};

struct TfsfDev {
    int gridLen, pulseLen, mTot, pulAddStart, nSteps;
    int layered;               // some line has a D grid or some term goes to D / is divided by eps
    TfsfLineDev line[6];       // 0..2 Ex..Ez, 3..5 Hx..Hz
    const double2* pulseTab;   // [step][line][mTot]: sum of the pulses at the line's pulse points
    double2* rec;              // [line][2 (nSteps + 1)]: recorded incident values (flux normalisation)
    unsigned int* ticket;      // blocks finished in the current E half (zero between launches)
    // surface corrections: rows of cells that get one term each (the bulk of every face),
    // one block per 256 cells of a row: F[comp][cell0 + r s] += pref * Re(line[incd0 + r t])
    const TfsfSegDev* seg[2];  // [0] H corrections, [1] E corrections
    const int2* segWork[2];    // per block: {row, chunk of 256 cells}
    int segBlocks[2];
    // cells that get several terms (face edges), per cell (CSR over the terms, in the
    // reference's order): F[comp][cell] (D where the term's flag says) += pref * Re(line[incd])
    int nCell[2];
    const long long* cell[2];
    const int* comp[2];
    const int* start[2];       // [nCell + 1]
    const int* termLine[2];
    const int* termIncd[2];
    const double* termPref[2];
    const int* termFlag[2];    // bit 0: to D; bits 1..: 1 + the line whose eps divides (0: none)
};

// Per step, after the H pass: H corrections, the 1-D step of every line (with the
// incident records), E corrections. fields: the main grid's E (0..2), H (3..5) and the
// D fields of E (6..8, null where absent).
template <typename T>
void launch_tfsf_step(const TfsfDev& t, T* const fields[9], const int* step, void* stream);

}  // namespace dev
}  // namespace chiml
