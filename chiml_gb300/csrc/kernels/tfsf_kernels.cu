// TFSF kernels for sm_103a: the surface corrections and the 1-D incident-line step of a
// TFSF plane-wave surface (parallelTFSFBase::updateFields / step,
// SOURCE/parallelTFSF.hpp:1058-1186; updateIncdFieldJ/K/JK, SOURCE/parallelTFSF.cpp:11-42;
// IncdCPML addPsi / updatePsiField, PML/PML.cpp:12-31; surface adds, addIncdFields,
// SOURCE/parallelTFSF.cpp:84-90).
//
//   k_tfsf_add    one thread per corrected main-grid cell, its terms in the reference's
//                 order: F += pref * Re(incident line value)
//   k_tfsf_lines  one block: records the H incident values, steps the H lines, then the
//                 E lines, and records the E incident values. Within a phase every line
//                 element is updated by one thread in the reference's per-element order
//                 (pulse add, J and K curl terms, then each CPML psi list touching it):
//                 the phase only reads lines of the other kind, so its elements are
//                 independent. Complex FP64 in both precision forms (the lines are a
//                 few thousand points).
#include "tfsf_device.hpp"

namespace chiml {
namespace dev {

namespace {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
// (s, 0) * v for a real s
__device__ __forceinline__ double2 rmul(double s, double2 v) { return make_double2(s * v.x, s * v.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <typename T>
__global__ void __launch_bounds__(256) k_tfsf_add(const TfsfDev t, int which, T* F0, T* F1, T* F2, T* F3, T* F4, T* F5) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= t.nCell[which]) return;
    T* const F[6] = {F0, F1, F2, F3, F4, F5};
    T* f = F[t.comp[which][q]];
    const long long cell = t.cell[which][q];
    double v = static_cast<double>(f[cell]);
    for (int k = t.start[which][q]; k < t.start[which][q + 1]; ++k)
        v += t.termPref[which][k] * t.line[t.termLine[which][k]].U[t.termIncd[which][k]].x;
    f[cell] = static_cast<T>(v);
}

// Element x of one grid of line c (incident grid when pulseGrid is false).
__device__ __forceinline__ void lineElement(const TfsfDev& t, int c, bool pulseGrid, int x, int s) {
    const TfsfLineDev& L = t.line[c];
    double2* G = pulseGrid ? L.pul : L.U;
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
}

// Every element of every grid of the lines c0 .. c0 + 2, strided over the block.
__device__ __forceinline__ void linePhase(const TfsfDev& t, int c0, int s) {
    const int per = t.gridLen + t.pulseLen;
    for (int e = threadIdx.x; e < 3 * per; e += blockDim.x) {
        const int c = c0 + e / per;
        if (!t.line[c].present) continue;
        const int x = e % per;
        if (x < t.gridLen) lineElement(t, c, false, x, s);
        else lineElement(t, c, true, x - t.gridLen, s);
    }
}

__device__ __forceinline__ void record(const TfsfDev& t, int c0, int s) {
    if (threadIdx.x >= 3) return;
    const int c = c0 + threadIdx.x;
    const TfsfLineDev& L = t.line[c];
    const long long base = static_cast<long long>(c) * 2 * (t.nSteps + 1) + 2LL * s;
    t.rec[base] = L.present ? L.pul[L.recIdx] : make_double2(0.0, 0.0);
    t.rec[base + 1] = L.present ? L.pul[L.recOffIdx] : make_double2(0.0, 0.0);
}

__global__ void __launch_bounds__(1024) k_tfsf_lines(const TfsfDev t, const int* __restrict__ step) {
    const int s = *step;
    if (s >= t.nSteps) return;
    record(t, 3, s);  // H incident values before the step (parallelFDTDField.hpp:1240-1245)
    __syncthreads();
    linePhase(t, 3, s);
    __syncthreads();
    linePhase(t, 0, s);
    __syncthreads();
    record(t, 0, s);  // E incident values after it (parallelFDTDField.hpp:1249-1254)
}

}  // namespace

template <typename T>
void launch_tfsf_step(const TfsfDev& t, T* const fields[6], const int* step, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (t.nCell[0] > 0)
        k_tfsf_add<T><<<(t.nCell[0] + 255) / 256, 256, 0, s>>>(t, 0, fields[0], fields[1], fields[2], fields[3], fields[4],
                                                              fields[5]);
    k_tfsf_lines<<<1, 1024, 0, s>>>(t, step);
    if (t.nCell[1] > 0)
        k_tfsf_add<T><<<(t.nCell[1] + 255) / 256, 256, 0, s>>>(t, 1, fields[0], fields[1], fields[2], fields[3], fields[4],
                                                              fields[5]);
}

template void launch_tfsf_step<float>(const TfsfDev&, float* const[6], const int*, void*);
template void launch_tfsf_step<double>(const TfsfDev&, double* const[6], const int*, void*);

}  // namespace dev
}  // namespace chiml
