// TFSF kernels for sm_103a: the surface corrections and the 1-D incident-line step of a
// TFSF plane-wave surface (parallelTFSFBase::updateFields / step,
// SOURCE/parallelTFSF.hpp:1058-1186; updateIncdFieldJ/K/JK, SOURCE/parallelTFSF.cpp:11-42;
// IncdCPML addPsi / updatePsiField, PML/PML.cpp:12-31; surface adds, addIncdFields,
// SOURCE/parallelTFSF.cpp:84-90).
//
//   k_tfsf_half   launched twice per step. The first launch steps the H lines and adds
//                 the H corrections (from the E lines), the second steps the E lines and
//                 adds the E corrections (from the new H lines). Every line element is
//                 updated by one thread in the reference's per-element order (pulse add,
//                 J and K curl terms, then each CPML psi list touching it): a half only
//                 reads lines of the other kind, so its elements are independent. A line
//                 in layered material (updateIncdPols, incdD2U, SOURCE/parallelTFSF.cpp:
//                 44-68) moves its poles from the element's previous value first, takes
//                 the curl into its D grid, then divides by the element's eps. The
//                 corrections: face rows of cells with one term each, one thread per cell
//                 along the row; cells on face edges (several terms) one thread each,
//                 adding their terms in the reference's order: F (or D inside a dispersive
//                 layer) += pref * Re(line value), the value first divided by eps where
//                 eps varies along the line (addIncdFieldsEPChange,
//                 SOURCE/parallelTFSF.cpp:98-107).
//                 The second launch also writes the incident values recorded for flux
//                 normalisation, from the block that finishes last.
// The lines are complex FP64 in both precision forms (a few thousand points).
#include "tfsf_device.hpp"
#include "launch_dep.hpp"

namespace chiml {
namespace dev {

namespace {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
// (s, 0) * v for a real s
__device__ __forceinline__ double2 rmul(double s, double2 v) { return make_double2(s * v.x, s * v.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// The main-grid field of component c (0..5: E, H; 6..8: D of E), selected without a
// dynamic index into an array (which would live in local memory).
template <typename T>
struct Fields9 {
    T* f[9];
    __device__ __forceinline__ T* operator[](int c) const {
        T* r = f[0];
#pragma unroll
        for (int k = 1; k < 9; ++k) r = c == k ? f[k] : r;
        return r;
    }
};

// Re(line value) of a surface term, divided by eps of line div where div >= 0 (LAY: the
// surface crosses layered material; without it no term is divided and no code for it is
// compiled in).
template <bool LAY>
__device__ __forceinline__ double termValue(const TfsfDev& t, int line, int incd, int div) {
    double x = t.line[line].U[incd].x;
    if (LAY && div >= 0) x = x / t.line[div].eps[incd];
    return x;
}

// Surface corrections of cell q of list `which` (0 H, 1 E): the terms to the field and
// those to its D field are two separate sums, each in the reference's order.
template <typename T, bool LAY>
__device__ __forceinline__ void addCell(const TfsfDev& t, int which, int q, const Fields9<T>& F) {
    if (q >= t.nCell[which]) return;
    const int c = t.comp[which][q];
    T* f = F[c];
    T* dF = F[6 + c % 3];
    const long long cell = t.cell[which][q];
    bool anyU = false, anyD = false;
    double v = 0.0, w = 0.0;
    for (int k = t.start[which][q]; k < t.start[which][q + 1]; ++k) {
        const int flag = t.termFlag[which][k];
        const double add = t.termPref[which][k] * termValue<LAY>(t, t.termLine[which][k], t.termIncd[which][k], (flag >> 1) - 1);
        if (LAY && (flag & 1)) {
            if (!anyD) w = static_cast<double>(dF[cell]);
            anyD = true;
            w += add;
        } else {
            if (!anyU) v = static_cast<double>(f[cell]);
            anyU = true;
            v += add;
        }
    }
    if (anyU) f[cell] = static_cast<T>(v);
    if (anyD) dF[cell] = static_cast<T>(w);
}

// Element x of one grid of line c (incident grid when pulseGrid is false).
template <bool LAY>
__device__ __forceinline__ void lineElement(const TfsfDev& t, int c, bool pulseGrid, int x, int s) {
    const TfsfLineDev& L = t.line[c];
    const bool dLine = LAY && !pulseGrid && L.D != nullptr;
    if (dLine) {
        // poles from the element's value before this step (updateIncdPols)
        const double2 u = L.U[x];
        for (int p = 0; p < L.nPole; ++p) {
            const long long i = static_cast<long long>(p) * t.gridLen + x;
            const double2 old = L.P[i];
            double2 n = rmul(L.pa[i], old);
            n = cadd(n, rmul(L.px[i], L.Pprev[i]));
            n = cadd(n, rmul(L.pg[i], u));
            L.Pprev[i] = old;
            L.P[i] = n;
        }
    }
    double2* G = pulseGrid ? L.pul : (dLine ? L.D : L.U);
    double2 v = G[x];
    const int pr = x - t.pulAddStart;
    if (pr >= 0 && pr < t.mTot) v = cadd(v, cmul(L.prefact, t.pulseTab[(static_cast<long long>(s) * 6 + c) * t.mTot + pr]));
    const TfsfRunDev& R = pulseGrid ? L.pulseRun : L.run;
    const int r = x - R.indI;
    if (r >= 0 && r < R.n) {
        if (L.useJ) {
            const double2* J = pulseGrid ? t.line[L.nbrJ].pul : t.line[L.nbrJ].U;
            v = cadd(v, rmul(R.pj, J[R.posK + r]));
            v = cadd(v, rmul(-1.0 * R.pj, J[R.negK + r]));
        }
        if (L.useK) {
            const double2* K = pulseGrid ? t.line[L.nbrK].pul : t.line[L.nbrK].U;
            v = cadd(v, rmul(R.pk, K[R.posJ + r]));
            v = cadd(v, rmul(-1.0 * R.pk, K[R.negJ + r]));
        }
    }
    const int np = pulseGrid ? L.nPmlPulse : L.nPml;
    for (int q = 0; q < np; ++q) {
        const TfsfPsiDev& P = pulseGrid ? L.pmlPulse[q] : L.pml[q];
        const int d = x - P.gridLoc;
        if (d < 0 || d >= P.n) continue;
        const double2* N = pulseGrid ? t.line[P.nbr].pul : t.line[P.nbr].U;
        double2 ps = rmul(P.b[d], P.psi[d]);
        ps = cadd(ps, rmul(P.c[d], N[P.loc + d]));
        ps = cadd(ps, rmul(P.cOff[d], N[P.locOff + d]));
        P.psi[d] = ps;
        v = cadd(v, rmul(P.Db, ps));
    }
    G[x] = v;
    if (dLine) {
        // incdD2U: U = D / eps, then U += (-P_p) / eps for each pole
        const double e = L.eps[x];
        double2 u = make_double2(v.x / e, v.y / e);
        for (int p = 0; p < L.nPole; ++p) {
            const double2 q = L.P[static_cast<long long>(p) * t.gridLen + x];
            u = cadd(u, make_double2((-1.0 * q.x) / e, (-1.0 * q.y) / e));
        }
        L.U[x] = u;
    }
}

// Element e of the lines c0 .. c0 + 2 (incident grid, then pulse grid, per line).
template <bool LAY>
__device__ __forceinline__ void lineAny(const TfsfDev& t, int c0, int e, int s) {
    const int per = t.gridLen + t.pulseLen;
    if (e >= 3 * per) return;
    const int c = c0 + e / per;
    if (!t.line[c].present) return;
    const int x = e % per;
    if (x < t.gridLen) lineElement<LAY>(t, c, false, x, s);
    else lineElement<LAY>(t, c, true, x - t.gridLen, s);
}

constexpr int kTfsfThreads = kTfsfRowChunk;

// Incident records after the step: E values of this step and the H values the next step
// starts from (the H lines do not change until then); step 0's H values are zero, and
// like the reference no H values are kept for the step after the last.
__device__ __forceinline__ void recordIncident(const TfsfDev& t, int s, int c) {
    const int slot = c < 3 ? s : s + 1;
    if (slot >= t.nSteps) return;  // slot nSteps is never a step's start: it stays zero
    const TfsfLineDev& L = t.line[c];
    const long long base = static_cast<long long>(c) * 2 * (t.nSteps + 1) + 2LL * slot;
    t.rec[base] = L.present ? L.pul[L.recIdx] : make_double2(0.0, 0.0);
    t.rec[base + 1] = L.present ? L.pul[L.recOffIdx] : make_double2(0.0, 0.0);
}

// One half of the TFSF step: blocks [0, lineBlocks) step the lines of kind c0 (3: H,
// 0: E), the other blocks add the corrections of list `which` (0: H corrections, from
// the E lines; 1: E corrections, from the H lines). The two parts touch disjoint data:
// the corrections read the lines of the other kind, which this half does not write.
// With `record`, the block that finishes last (a ticket counter, no waiting) writes the
// incident records once every line of the half has been stepped.
template <typename T, bool LAY>
__global__ void __launch_bounds__(kTfsfThreads) k_tfsf_half(const TfsfDev t, int c0, int which, int lineBlocks, int record,
                                                            const Fields9<T> F, const int* __restrict__ step) {
    waitPriorGrid();
    const int s = *step;
    if (s >= t.nSteps) return;
    const int b = static_cast<int>(blockIdx.x);
    if (b < lineBlocks) {
        lineAny<LAY>(t, c0, b * kTfsfThreads + threadIdx.x, s);
    } else {
        const int sb = b - lineBlocks;
        if (sb < t.segBlocks[which]) {
            const int2 w = t.segWork[which][sb];
            const TfsfSegDev& g = t.seg[which][w.x];
            const int r = w.y * kTfsfThreads + static_cast<int>(threadIdx.x);
            if (r < g.n) {
                T* f = F[(LAY && g.toD) ? 6 + g.comp : g.comp];
                const long long cell = g.cell0 + r * g.cellStride;
                const int incd = g.incd0 + r * g.incdStride;
                f[cell] = static_cast<T>(static_cast<double>(f[cell]) + g.pref * termValue<LAY>(t, g.line, incd, g.div));
            }
        } else {
            addCell<T, LAY>(t, which, (sb - t.segBlocks[which]) * kTfsfThreads + threadIdx.x, F);
        }
    }
    if (!record) return;
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();  // this block's line values are visible before its ticket
        last = atomicAdd(t.ticket, 1u) == gridDim.x - 1;
        if (last) {
            *t.ticket = 0u;
            __threadfence();
        }
    }
    __syncthreads();
    if (last && threadIdx.x < 6) recordIncident(t, s, threadIdx.x);
}

}  // namespace

template <typename T>
void launch_tfsf_step(const TfsfDev& t, T* const fields[9], const int* step, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int lineBlocks = (3 * (t.gridLen + t.pulseLen) + kTfsfThreads - 1) / kTfsfThreads;
    Fields9<T> F;
    for (int k = 0; k < 9; ++k) F.f[k] = fields[k];
    for (int half = 0; half < 2; ++half) {
        const int addBlocks = t.segBlocks[half] + (t.nCell[half] + kTfsfThreads - 1) / kTfsfThreads;
        const dim3 grid(static_cast<unsigned>(lineBlocks + addBlocks));
        if (t.layered)
            launchAfterPrior(k_tfsf_half<T, true>, grid, dim3(kTfsfThreads), s, t, half == 0 ? 3 : 0, half, lineBlocks, half == 1 ? 1 : 0, F, step);
        else
            launchAfterPrior(k_tfsf_half<T, false>, grid, dim3(kTfsfThreads), s, t, half == 0 ? 3 : 0, half, lineBlocks, half == 1 ? 1 : 0, F, step);
    }
}

template void launch_tfsf_step<float>(const TfsfDev&, float* const[9], const int*, void*);
template void launch_tfsf_step<double>(const TfsfDev&, double* const[9], const int*, void*);

}  // namespace dev
}  // namespace chiml
