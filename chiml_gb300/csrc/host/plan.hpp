// The compiled form of a simulation that the CUDA kernels (and the CPU oracle)
// execute: grid dimensions, a per-cell class code for every Yee component, a
// small table of per-class coefficients, 1-D CPML profiles, and the source,
// detector and DFT-flux descriptors.
//
// Every cell of component c follows one update rule:
//
//   psi_t  <- b_t[a] * psi_t + cpsi_t[a] * (G_t[i] - G_t[i + off_t])          (if psi_t flag)
//   U[i]   += (cint_t + nplain_t * db_t + (kflag_t ? kprof_t[a] : 0))
//               * (G_t[i] - G_t[i + off_t])  + npsi_t * dbpsi_t * psi_t[i]     (for t = J, K)
//
// where U is E/H or D (per class), G_J / G_K are the two neighbouring field
// components, a is the cell's coordinate along the term's derivative axis, and
// the class table supplies cint/nplain/kflag/npsi. This reproduces the sum of
// chiML's interior curl lists (FDTD_MANAGER/parallelFDTDField.hpp:628-856)
// and CPML lists (PML/parallelPML.hpp:321-697) cell by cell; build_plan checks
// the compressed form against a literal accumulation of those lists.
#pragma once

#include <array>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "model.hpp"

namespace chiml {

// With CHIML_HOST_TIMES set in the environment, mark() prints the wall seconds since the
// previous mark (or construction) to stderr: the phases of the plan build and of finalize.
struct PhaseClock {
    bool on = std::getenv("CHIML_HOST_TIMES") != nullptr;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    void mark(const char* what) {
        if (!on) return;
        const auto t1 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "host %-14s %8.4f s\n", what, std::chrono::duration<double>(t1 - t0).count());
        t0 = t1;
    }
};

// Grid layout kept from chiML's Grid (GRID/Grid.hpp:201-205): x fastest, then z,
// then y, with a one-cell halo on every side (2-D: lz == 1, no z halo).
struct Dims {
    int nx = 0, ny = 0, nz = 1;  // physical points (n_vec_)
    int lx = 0, ly = 0, lz = 1;  // local extents including the halo
    bool threeD = false;
    long long cells() const { return static_cast<long long>(lx) * ly * lz; }
    long long idx(int x, int y, int z) const { return x + static_cast<long long>(lx) * (z + static_cast<long long>(lz) * y); }
};

// Component ids: 0..2 = Ex,Ey,Ez ; 3..5 = Hx,Hy,Hz
enum Comp { EX = 0, EY = 1, EZ = 2, HX = 3, HY = 4, HZ = 5 };

struct TermPlan {
    bool present = false;   // the component has this neighbour field
    int field = -1;         // component id of G_t
    int axis = 0;           // derivative axis (0 x, 1 y, 2 z)
    long long off = 0;      // index offset of the neighbour (i + off)
    double db = 0.0;        // DbFieldBase of the CPML term (dt / d, signed)
    double dbpsi = 0.0;     // Db of the CPML term (+-dt)
    bool hasPsi = false;    // psi storage exists for this term
    std::vector<double> kprof;  // per coordinate along axis: CPML coefficient of deriv-normal slab cells
    std::vector<double> b, cpsi; // per coordinate along axis: psi recursion coefficients
    // per coordinate along axis: 1 where some cell carries the CPML term along the axis or
    // updates psi (the CPML slabs of the term, whose bounds the pass kernels take)
    std::vector<uint8_t> slabUse;
};

struct ClassInfo {
    uint8_t toD = 0;       // 1: the curl and CPML terms update D instead of the field
    uint8_t lor = 0;       // 1: Lorentz P update before and D -> E after (upLorD list)
    uint8_t ordip = 0;     // 1: oriented-dipole D -> E (upOrDipD list)
    int obj = 0;           // object whose poles apply (lor)
    double eps = 1.0;      // eps_inf used by D -> E
    double cint[2] = {0.0, 0.0};  // interior curl coefficients of terms J, K
    uint8_t nplain[2] = {0, 0};
    uint8_t kflag[2] = {0, 0};
    uint8_t npsi[2] = {0, 0};
    uint8_t psiUpd[2] = {0, 0};  // psi recursion applied at this cell
    bool operator==(const ClassInfo& o) const;
};

struct CompPlan {
    bool present = false;
    bool isE = true;
    bool hasD = false;
    std::vector<uint8_t> code;     // per cell, index into classes
    std::vector<ClassInfo> classes;
    TermPlan term[2];              // J (uses grid_j), K (uses grid_k)
    int nPoles = 0;                // number of Lorentz pole grids of this component
};

// Oriented-dipole Lorentz cells (upOrDipP list) on the cell-corner grid.
struct OrDipPlan {
    bool present = false;
    int nPoles = 0;
    std::vector<long long> cells;           // grid index of each updated cell
    std::vector<int> obj;                   // object of each cell
    std::vector<std::array<double, 3>> dip; // per pole per cell: dip_x, dip_y, dip_z (cells * nPoles)
    long long offA[3] = {0, 0, 0};          // E_c neighbour offsets for the averaged dot product
};

struct SourcePlan {
    int comp = EZ;
    std::vector<long long> cells;
    std::vector<double> value;  // dt * Re(sum of pulses) per step (index = step)
};

// A box of grid cells sampled by a time-domain detector.
struct DetectorPlan {
    DetectorSpec spec;
    int timeInt = 1;
    double tConv = 1.0, convFactor = 1.0;
    std::array<double, 3> realLoc = {0, 0, 0};
    bool power = false;
    struct Field {
        int comp;           // component id, or 6+c for D_c
        std::array<int, 3> off;
        std::array<int, 3> outSz;  // storage box size
        std::vector<long long> cells;  // outGrid order (x + sx*(z + sz*y)), -1 where not stored
    };
    std::vector<Field> fields;
    std::array<int, 3> sz = {1, 1, 1};
    // frequency-domain detectors (parallelDetectorFREQ_Base, DTC/parallelDTC_FREQ.hpp): each
    // field's DFT box (parallelStorageFreqDTC, no propagation direction) holds its points
    // x fastest, then z, then y; `freqPts` of the szFreq = product of sz box points are stored
    double freqConv = 1.0;
    long long szFreq = 0;
};

// One DFT accumulator box (parallelStorageFreqDTC) of a flux region.
struct FreqStore {
    int comp = 0;
    std::array<int, 3> loc = {0, 0, 0}, sz = {1, 1, 1};
    int propDir = 0;              // 0 X, 1 Y, 2 Z
    std::array<int, 3> inSz = {0, 0, 0};  // fieldInFreq_.sz_
    std::array<int, 3> outN = {0, 0, 0}; // outGrid dims {nfreq, sz1, sz0}
    std::vector<long long> cells; // grid index of accumulated points, outGrid point order
    long long accOffset = 0;      // offset (in points) into the flux's accumulator
};

struct FluxFace {
    double weight = 1.0;
    int sz = 0;
    std::vector<int> Ej, Ek, Hj, Hk;   // indices into FluxPlan::stores
    int cor = 0, transCor1 = 0, transCor2 = 0, corI = 0, corJ = 0, corK = 0;
    std::array<int, 3> faceSz = {1, 1, 1};
};

struct FluxPlan {
    FluxSpec spec;
    std::vector<FreqStore> stores;
    std::vector<FluxFace> faces;
    long long npts = 0;            // total accumulated points
    double dt = 0.0;
    double fluxConv = 1.0, incdConv[3] = {1, 1, 1}, freqConv = 1.0, dLam = 0.0, dOmg = 0.0;
    bool real3D = false;
};

// The emitters of one object, ready to step (ML/parallelQE.hpp, parallelQE.cpp). Each
// emitter cell holds one density matrix per ensemble member (one Hamiltonian per
// combination of level energies, ML/Hamiltonian.cpp). Matrices are nlevel x nlevel,
// stored flat as the reference does (element i + nlevel*j is row i, column j of the
// column-major BLAS calls).
struct EmitterPlan {
    int nlevel = 0;
    int nMembers = 0;
    std::vector<double> h0;             // [member * nlevel + level]: diagonal energies (FDTD units)
    std::vector<double> weight;         // [member]: initial rho[0]
    std::array<std::vector<cplx>, 3> mu;     // x/y/z_expectation_ (coupling-scaled), nlevel^2 each
    std::array<std::vector<cplx>, 3> negMu;  // neg_x/y/z_expectation_
    std::array<bool, 3> addMu = {false, false, false};  // the operator has a nonzero element
    // per emitter cell (extension, EmitterSpec::cellDipole): the operator of the cell is
    // w * mu[z], w = scale * direction; empty: the object's operators everywhere
    std::vector<std::array<double, 3>> cellDip;
    // relaxation: for each flat index ii the (jj, rate) pairs, outDeriv[ii] += rho[jj] * rate
    std::vector<std::vector<std::pair<int, double>>> gam;
    double dt = 0.0, hbar = 0.0, na = 0.0;
    int zOff = 0;
    std::array<bool, 3> comp = {false, false, false};  // component c is coupled (E_c exists)
    bool gatherZCopy = false;                          // Ez gathered by copy (2-D TMz) instead of averaging
    // geometry in grid coordinates (halo included). P-box point (i, j, k) sits at grid point
    // boxBase + (i, j, k); the cell at (x, y, z) from the emitters' lowest point has P-box
    // point (x+1, y+1, z+zOff). E points boxBase + (i, j, k), i < addN, receive P.
    std::array<int, 3> boxBase = {0, 0, 0};
    std::array<int, 3> nCell = {1, 1, 1};     // cell box extent
    std::vector<long long> cellGrid;          // per emitter cell (reference order): grid index
    std::array<int, 3> pDims = {1, 1, 1};     // P box extents; P index i + px*(k + pz*j)
    std::vector<int> cellP;                   // per emitter cell: P-box index of the cell
    std::array<int, 3> addN = {1, 1, 1};
    // outputs
    int nPoints = 0;                          // emitter points (population normalisation)
    bool outputPol = false;
    std::string polFile;
    std::vector<int> dtcLevs;
    std::vector<std::string> dtcFiles;
    int dtcTimeInt = 1;
};

// ---- TFSF plane-wave surfaces (SOURCE/parallelTFSF.*, PML/PML.*) ----
// Incident fields live on 1-D complex grids ("lines"), one per field component the
// main grid has; line c = 0..2 Ex..Ez, 3..5 Hx..Hy. Each line has the incident grid
// (updated as D / B, then divided by eps / mu), its own CPML, and a short "pulse" grid
// in the uniform surface material whose values are recorded for flux normalisation.

// A run of equal material along a line (paramUpIncdField, parallelTFSF.hpp:17-38):
// U[indI + r] += pj (J[posK + r] - J[negK + r]) + pk (K[posJ + r] - K[negJ + r]).
struct TfsfRun {
    int indI = 0, posJ = 0, negJ = 0, posK = 0, negK = 0, n = 0;
    double pj = 0.0, pk = 0.0;
};

// One psi list of a line's CPML (IncdCPML::getUpList, PML/PML.hpp:222-271; addPsi and
// updatePsiField, PML/PML.cpp:12-31): psi = b psi + c G[loc + d] + cOff G[locOff + d],
// then U[gridLoc + d] += Db psi, for d < n. G is the neighbour line nbr.
struct TfsfPsi {
    int nbr = -1;
    int loc = 0, locOff = 0, gridLoc = 0, n = 0;
    double Db = 0.0;
    std::vector<double> b, c, cOff;
};

// A line crossing layered material (surfaces in non-vacuum material, genEpMu and
// genFieldUpParam, parallelTFSF.hpp:591-720) has per-element eps (mu) and pole
// coefficients: each step first moves the poles, P = alpha P + xi P_prev + gamma U
// (updateIncdPols, parallelTFSF.cpp:44-58, U the line before this step), then the curl
// goes to the D grid, then U = D / eps - sum_p P_p / eps (incdD2U, parallelTFSF.cpp:60-68).
struct TfsfLine {
    bool present = false;
    bool useJ = false, useK = false;  // the j / k neighbour lines take part in the curl
    int nbrJ = -1, nbrK = -1;          // neighbour line ids (component (c+1)%3, (c+2)%3 of the other kind)
    std::vector<double> epMu;          // per incident-grid element: eps (E) or mu (H), gridLen values
    std::vector<int> obj;              // per incident-grid element: the object it samples (incdPhys)
    bool dLine = false;                // stepped through a D grid (eps other than 1 or poles on the line)
    bool epChange = false;             // eps varies along the line: surface terms are divided by it
    int nPole = 0;                     // poles per element (the most any element's object has)
    std::vector<double> pa, px, pg;    // [nPole][gridLen] alpha, xi, gamma; zero past an object's poles
    std::vector<TfsfRun> runs;         // incident grid, length gridLen
    std::vector<TfsfRun> pulseRuns;    // pulse grid, length pulseLen
    std::vector<TfsfPsi> pml, pmlPulse;
    std::vector<double> dist;          // per pulse point: distance from the source (distVecE/H)
    cplx prefact = 0.0;                // pulse prefactor (prefactE_/prefactH_)
    int recIdx = 0, recOffIdx = 0;     // pulse-grid points recorded each step
};

// The surface terms of every main-grid cell that gets some; the terms of cell q are
// [start[q], start[q + 1]) in the reference's order: F[comp[q]][cell[q]] (its D field
// where toD) += pref * Re(line[line][incd]) (divided first by eps of line div at incd
// where div >= 0).
struct TfsfAdds {
    std::vector<long long> cell;
    std::vector<int> comp;              // main field component 0..5
    std::vector<long long> start{0};    // [cells + 1]
    std::vector<int> line, incd;
    std::vector<double> pref;
    std::vector<uint8_t> toD;
    std::vector<int> div;               // -1, or the line whose eps divides the value (addIncdFieldsEPChange)
    std::size_t cells() const { return cell.size(); }
    std::size_t terms() const { return line.size(); }
};

// One row of one surface (a daxpy of addIncdFields): cell cell0 + r * cellStride of
// component comp (its D field where toD) gets pref * Re(line[incd0 + r * incdStride]),
// r < n; where div >= 0 the value is first divided by eps of line div at the same index
// (addIncdFieldsEPChange, SOURCE/parallelTFSF.cpp:98-107).
struct TfsfSegment {
    long long cell0 = 0, cellStride = 0;
    int incd0 = 0, incdStride = 0, n = 0, line = 0, comp = 0;
    double pref = 0.0;
    bool toD = false;
    int div = -1;
};

struct TfsfPlan {
    int gridLen = 0, pulseLen = 0, mTot = 0, mMax = 0, pmlThick = 0, pulAddStart = 0;
    std::array<int, 3> m = {0, 0, 0};
    double dt = 0.0;
    TfsfLine line[6];
    std::vector<PulseSpec> pulses;
    TfsfAdds addH, addE;  // applied before and after the 1-D step
    std::vector<TfsfSegment> segH, segE;   // the same corrections as surface rows
};

struct Plan {
    Inputs in;
    Dims dims;
    double dt = 0.0;
    int nSteps = 0;
    std::vector<double> tcur;  // time at the start of each step (tcur_ accumulation), size nSteps + 1
    bool disp = false, dielectricMatInPML = false;
    CompPlan comp[6];
    OrDipPlan ordip;
    std::vector<SourcePlan> sources;
    std::vector<DetectorPlan> detectors;       // time-domain (text, binary)
    std::vector<DetectorPlan> freqDetectors;   // frequency-domain
    std::vector<FluxPlan> fluxes;
    std::vector<EmitterPlan> emitters;
    std::vector<TfsfPlan> tfsf;
    // relative permittivity on the cell-centred grid (epsRelOrDip_), where the emitter
    // polarisation is divided into E; filled only when there are emitters
    std::vector<double> epsP;
    // object pole coefficients, flattened: per object, per pole; alphaInc is alpha + xi - 1
    // formed directly (the increment form of the FP32 kernels)
    std::vector<std::vector<double>> alpha, xi, gamma, alphaInc;
};

// Builds the plan; throws InputError / UnsupportedError.
Plan build_plan(const Inputs& in);

// Emitter plans of the input (emitters.cpp); Epresent: which of Ex, Ey, Ez the grid has;
// epsOrDip: the relative permittivity on the cell-centred grid.
void build_emitters(const Inputs& in, const Dims& D, double dt, const bool Epresent[3],
                    const double* epsOrDip, Plan& P);

// TFSF plans of the input (tfsf.cpp); phys[c]: object id per cell of main component c
// (0..5; null when absent), -1 on the halo.
void build_tfsf(const Inputs& in, const Dims& D, double dt, const int* const phys[6],
                const std::vector<Object>& objs, Plan& P);

// Wigner 3j symbol for integer arguments (emitters.cpp).
double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3);

}  // namespace chiml
