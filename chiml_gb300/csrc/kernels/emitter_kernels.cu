// Emitter kernels for sm_103a: the Maxwell-Liouville step of every emitter cell after
// D -> E, restating ML/parallelQE.hpp:674-770 for one process.
//
//   k_emitter_addp    E += -P/(2 eps) at two P points per E point over the (n+1)-box
//                     (MLUpdateFxnReal::addP, UTIL/FDTD_up_eq.cpp:1367-1380)
//   k_emitter_update  one thread per emitter cell: gathers E at the cell centre
//                     (getE_TE / getE_TM, FDTD_up_eq.cpp:1400-1430), then for each
//                     ensemble member the ABM4 predictor-corrector of
//                     d rho/dt = (i/hbar)[H, rho] + Gamma rho (PCABAM4 / denDeriv,
//                     parallelQE.hpp:727-770) with H = h0 - E . mu (Hamiltonian::getHam),
//                     and P = sum over members of na Re(rho . mu) (updateQEPol,
//                     UTIL/FDTD_up_eq.hpp:620); block partial sums of the populations and
//                     of P for the outputs
//   k_emitter_reduce  fixed-order sum of the block partials (deterministic run to run)
//
// All density-matrix arithmetic is FP64 in both precision forms. The four derivative
// histories rotate through four slots by step number instead of being copied.
#include <cstdint>

#include "emitter_device.hpp"

namespace chiml {
namespace dev {

namespace {

constexpr int kMaxDtc = 8;
constexpr int kEmThreads = 128;

struct C2 {
    double x, y;
};
__device__ __forceinline__ C2 c2(double a, double b) { return C2{a, b}; }
__device__ __forceinline__ C2 cmul(C2 a, C2 b) { return C2{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ C2 cadd(C2 a, C2 b) { return C2{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ C2 cconj(C2 a) { return C2{a.x, -a.y}; }
__device__ __forceinline__ C2 ld(const double2* p) {
    const double2 v = *p;
    return C2{v.x, v.y};
}
__device__ __forceinline__ void st(double2* p, C2 v) { *p = make_double2(v.x, v.y); }
// y + (a, 0) * x, the complex axpy of a real step coefficient
__device__ __forceinline__ C2 caxpy(double a, C2 x, C2 y) { return cadd(y, cmul(c2(a, 0.0), x)); }

// (i/hbar) H den + its conjugate transpose, plus the relaxation rows (denDeriv, MKL form)
template <int NT>
__device__ __forceinline__ void den_deriv(const EmitterDev& e, int N, const C2* H, const C2* den, C2* out, C2* tmp) {
    const int n = NT ? NT : N;
    const C2 alpha = c2(0.0, 1.0 / e.hbar);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            C2 s = c2(0.0, 0.0);
            for (int l = 0; l < n; ++l) s = cadd(s, cmul(H[i + l * n], den[l + j * n]));
            tmp[i + j * n] = cmul(alpha, s);
        }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) out[i * n + j] = cadd(tmp[i * n + j], cconj(tmp[j * n + i]));
    for (int ii = 0; ii < n * n; ++ii)
        for (int p = e.gamRow[ii]; p < e.gamRow[ii + 1]; ++p) {
            const C2 d = den[e.gamCol[p]];
            out[ii] = cadd(out[ii], c2(d.x * e.gamVal[p], d.y * e.gamVal[p]));
        }
}

// addP of component c over points t = tBegin, tBegin + tStride, ...
template <typename T>
__device__ __forceinline__ void addpRange(const EmitterDev& e, T* Ex, T* Ey, T* Ez, int c, int tBegin, int tStride) {
    if (!e.comp[c]) return;
    T* E = c == 0 ? Ex : (c == 1 ? Ey : Ez);
    const int ox = (c == 0), oy = (c == 1), oz = (c == 2) ? e.zOff : 0;
    const int n = e.addN[0] * e.addN[1] * e.addN[2];
    const double* P = e.P + static_cast<long long>(c) * e.pBox;
    for (int t = tBegin; t < n; t += tStride) {
        const int ii = t % e.addN[0];
        const int r = t / e.addN[0];
        const int jj = r % e.addN[1];
        const int kk = r / e.addN[1];
        const int pa = ii + e.pDims[0] * (kk + e.pDims[2] * jj);
        const int pb = (ii + ox) + e.pDims[0] * ((kk + oz) + e.pDims[2] * (jj + oy));
        const long long g = (e.boxBase[0] + ii) +
                            static_cast<long long>(e.lx) * ((e.boxBase[2] + kk) + static_cast<long long>(e.lz) * (e.boxBase[1] + jj));
        double v = static_cast<double>(E[g]);
        v += -0.5 * P[pa] / e.epsBox[pa];
        v += -0.5 * P[pb] / e.epsBox[pb];
        E[g] = static_cast<T>(v);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_emitter_addp(const EmitterDev e, T* Ex, T* Ey, T* Ez) {
    addpRange(e, Ex, Ey, Ez, blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Block `blk` of the density update (cells kEmThreads * blk ...), writing partial row blk.
template <typename T, int NT>
__device__ __forceinline__ void updateBlock(const EmitterDev& e, const T* __restrict__ Ex, const T* __restrict__ Ey,
                                            const T* __restrict__ Ez, const int* __restrict__ stepPtr, int blk) {
    constexpr int MAXN2 = (NT ? NT * NT : kMaxEmitterLevels * kMaxEmitterLevels);
    const int N = NT ? NT : e.N;
    const int n2 = N * N;
    const int q = blk * kEmThreads + threadIdx.x;
    const int s = *stepPtr;
    const bool popStep = (s % e.dtcTimeInt) == 0;
    C2 popAcc[kMaxDtc];
    for (int d = 0; d < kMaxDtc; ++d) popAcc[d] = c2(0.0, 0.0);
    double Pc[3] = {0.0, 0.0, 0.0};
    if (q < e.nc) {
        // E at the cell centre
        const long long g = e.cellGrid[q];
        const T* Es[3] = {Ex, Ey, Ez};
        double Ec[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < 3; ++c) {
            if (!e.comp[c]) continue;
            if (c == 2 && e.gatherZCopy) Ec[c] = static_cast<double>(Es[c][g]);
            else Ec[c] = 0.5 * static_cast<double>(Es[c][g]) + 0.5 * static_cast<double>(Es[c][g - e.unit[c]]);
        }
        const bool zeroE = (Ec[0] == 0.0 && Ec[1] == 0.0 && Ec[2] == 0.0);
        const long long slotStride = static_cast<long long>(e.nm) * n2 * e.nc;
        const int s0 = (s - 1) & 3, s1 = (s - 2) & 3, s2 = (s - 3) & 3, s3 = s & 3;  // k_n, k_n-1, k_n-2, k_n-3
        const double dt = e.dt;
        const double c55 = 55.0 * dt / 24.0, cm59 = -59.0 * dt / 24.0, c37 = 37.0 * dt / 24.0, cm9 = -9.0 * dt / 24.0;
        const double c9 = 9.0 * dt / 24.0, c19 = 19.0 * dt / 24.0, cm5 = -5.0 * dt / 24.0, c1 = dt / 24.0;
        C2 H[MAXN2], a[MAXN2], b[MAXN2], tmp[MAXN2];
        for (int m = 0; m < e.nm; ++m) {
            // Hamiltonian::getHam
            for (int i = 0; i < n2; ++i) H[i] = c2(0.0, 0.0);
            for (int i = 0; i < N; ++i) H[i * N + i] = c2(e.h0[m * N + i], 0.0);
            if (!zeroE)
                for (int c = 0; c < 3; ++c)
                    if (e.addMu[c])
                        for (int i = 0; i < n2; ++i) H[i] = cadd(H[i], cmul(c2(Ec[c], 0.0), ld(&e.negMu[c * n2 + i])));
            const long long base = static_cast<long long>(m) * n2 * e.nc + q;
            // predictor
            for (int i = 0; i < n2; ++i) {
                const long long o = base + static_cast<long long>(i) * e.nc;
                C2 p = ld(&e.rho[o]);
                p = caxpy(c55, ld(&e.kd[s0 * slotStride + o]), p);
                p = caxpy(cm59, ld(&e.kd[s1 * slotStride + o]), p);
                p = caxpy(c37, ld(&e.kd[s2 * slotStride + o]), p);
                p = caxpy(cm9, ld(&e.kd[s3 * slotStride + o]), p);
                a[i] = p;
            }
            den_deriv<NT>(e, N, H, a, b, tmp);  // b = derivative at the prediction
            // corrector
            for (int i = 0; i < n2; ++i) {
                const long long o = base + static_cast<long long>(i) * e.nc;
                C2 r = ld(&e.rho[o]);
                r = caxpy(c9, b[i], r);
                r = caxpy(c19, ld(&e.kd[s0 * slotStride + o]), r);
                r = caxpy(cm5, ld(&e.kd[s1 * slotStride + o]), r);
                r = caxpy(c1, ld(&e.kd[s2 * slotStride + o]), r);
                a[i] = r;
                st(&e.rho[o], r);
            }
            den_deriv<NT>(e, N, H, a, b, tmp);  // derivative at the new density: the next k_n
            for (int i = 0; i < n2; ++i) st(&e.kd[s3 * slotStride + base + static_cast<long long>(i) * e.nc], b[i]);
            if (popStep)
                for (int d = 0; d < e.nDtc; ++d) popAcc[d] = cadd(popAcc[d], a[e.dtcLev[d]]);
            for (int c = 0; c < 3; ++c) {
                if (!e.comp[c]) continue;
                C2 sdot = c2(0.0, 0.0);
                for (int i = 0; i < n2; ++i) sdot = cadd(sdot, cmul(cconj(a[i]), ld(&e.mu[c * n2 + i])));
                Pc[c] += e.na * sdot.x;
            }
        }
        for (int c = 0; c < 3; ++c)
            if (e.comp[c]) e.P[static_cast<long long>(c) * e.pBox + e.cellP[q]] = Pc[c];
    }
    // block partial sums, fixed tree order
    constexpr int NQ = 2 * kMaxDtc + 3;
    __shared__ double red[NQ][kEmThreads];
    for (int d = 0; d < kMaxDtc; ++d) {
        red[2 * d][threadIdx.x] = popAcc[d].x;
        red[2 * d + 1][threadIdx.x] = popAcc[d].y;
    }
    for (int c = 0; c < 3; ++c) red[2 * kMaxDtc + c][threadIdx.x] = Pc[c];
    __syncthreads();
    for (int w = kEmThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < NQ; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int d = 0; d < e.nDtc; ++d)
            e.popPartial[static_cast<long long>(blk) * e.nDtc + d] = make_double2(red[2 * d][0], red[2 * d + 1][0]);
        for (int c = 0; c < 3; ++c) e.totPartial[blk * 3 + c] = red[2 * kMaxDtc + c][0];
    }
}

template <typename T, int NT>
__global__ void __launch_bounds__(kEmThreads) k_emitter_update(const EmitterDev e, const T* __restrict__ Ex,
                                                               const T* __restrict__ Ey, const T* __restrict__ Ez,
                                                               const int* __restrict__ stepPtr) {
    updateBlock<T, NT>(e, Ex, Ey, Ez, stepPtr, blockIdx.x);
}

__device__ __forceinline__ void reduceBody(const EmitterDev& e, const int* __restrict__ stepPtr) {
    const int s = *stepPtr;
    __shared__ double red[256];
    const bool popStep = (s % e.dtcTimeInt) == 0;
    const int nq = 2 * e.nDtc + 3;
    for (int k = 0; k < nq; ++k) {
        const bool isPop = k < 2 * e.nDtc;
        if (isPop && !popStep) continue;
        if (!isPop && (!e.totP || s >= e.nSteps)) continue;
        double v = 0.0;
        for (int b = threadIdx.x; b < e.partialBlocks; b += blockDim.x) {
            if (isPop) {
                const double2 p = e.popPartial[static_cast<long long>(b) * e.nDtc + k / 2];
                v += (k & 1) ? p.y : p.x;
            } else {
                v += e.totPartial[b * 3 + (k - 2 * e.nDtc)];
            }
        }
        red[threadIdx.x] = v;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (isPop) {
                double* dst = reinterpret_cast<double*>(&e.pop[static_cast<long long>(k / 2) * e.nEvents + s / e.dtcTimeInt]);
                dst[k & 1] = red[0] / e.nPoints;
            } else {
                const int c = k - 2 * e.nDtc;
                if (e.comp[c]) e.totP[static_cast<long long>(c) * e.nSteps + s] = red[0];
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_emitter_reduce(const EmitterDev e, const int* __restrict__ stepPtr) {
    reduceBody(e, stepPtr);
}

// ---- packed launches (batched sweep): work[b] = {job, block of that job} ----

template <typename T>
__global__ void __launch_bounds__(256) k_emitter_addp_packed(const EmitJob<T>* __restrict__ jobs, const int2* __restrict__ work) {
    const int2 w = work[blockIdx.x];
    const EmitJob<T>& j = jobs[w.x];
    const int bpc = emitter_addp_blocks_per_comp(j.e);
    const int c = w.y / bpc, b = w.y % bpc;
    addpRange(j.e, j.f[0], j.f[1], j.f[2], c, b * 256 + static_cast<int>(threadIdx.x), bpc * 256);
}

template <typename T, int NT>
__global__ void __launch_bounds__(kEmThreads) k_emitter_update_packed(const EmitJob<T>* __restrict__ jobs,
                                                                      const int2* __restrict__ work) {
    const int2 w = work[blockIdx.x];
    const EmitJob<T>& j = jobs[w.x];
    updateBlock<T, NT>(j.e, j.f[0], j.f[1], j.f[2], j.step, w.y);
}

template <typename T>
__global__ void __launch_bounds__(256) k_emitter_reduce_packed(const EmitJob<T>* __restrict__ jobs) {
    const EmitJob<T>& j = jobs[blockIdx.x];
    reduceBody(j.e, j.step);
}

}  // namespace

int emitter_update_blocks(const EmitterDev& e) { return (e.nc + kEmThreads - 1) / kEmThreads; }
int emitter_level_group(int N) { return N == 2 ? 0 : (N == 3 ? 1 : (N == 4 ? 2 : 3)); }

template <typename T>
void launch_emitter_packed(const EmitJob<T>* jobs, int njobs, WorkMap addp, const WorkMap update[4], void* stream) {
    if (njobs <= 0) return;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (addp.blocks > 0) k_emitter_addp_packed<T><<<addp.blocks, 256, 0, s>>>(jobs, addp.work);
    if (update[0].blocks > 0) k_emitter_update_packed<T, 2><<<update[0].blocks, kEmThreads, 0, s>>>(jobs, update[0].work);
    if (update[1].blocks > 0) k_emitter_update_packed<T, 3><<<update[1].blocks, kEmThreads, 0, s>>>(jobs, update[1].work);
    if (update[2].blocks > 0) k_emitter_update_packed<T, 4><<<update[2].blocks, kEmThreads, 0, s>>>(jobs, update[2].work);
    if (update[3].blocks > 0) k_emitter_update_packed<T, 0><<<update[3].blocks, kEmThreads, 0, s>>>(jobs, update[3].work);
    k_emitter_reduce_packed<T><<<njobs, 256, 0, s>>>(jobs);
}

template void launch_emitter_packed<float>(const EmitJob<float>*, int, WorkMap, const WorkMap[4], void*);
template void launch_emitter_packed<double>(const EmitJob<double>*, int, WorkMap, const WorkMap[4], void*);

template <typename T>
void launch_emitter_step(const EmitterDev& e, T* const fields[3], const int* step, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 ga(emitter_addp_blocks_per_comp(e), 3);
    k_emitter_addp<T><<<ga, 256, 0, s>>>(e, fields[0], fields[1], fields[2]);
    const int blocks = (e.nc + kEmThreads - 1) / kEmThreads;
    switch (e.N) {
        case 2: k_emitter_update<T, 2><<<blocks, kEmThreads, 0, s>>>(e, fields[0], fields[1], fields[2], step); break;
        case 3: k_emitter_update<T, 3><<<blocks, kEmThreads, 0, s>>>(e, fields[0], fields[1], fields[2], step); break;
        case 4: k_emitter_update<T, 4><<<blocks, kEmThreads, 0, s>>>(e, fields[0], fields[1], fields[2], step); break;
        default: k_emitter_update<T, 0><<<blocks, kEmThreads, 0, s>>>(e, fields[0], fields[1], fields[2], step); break;
    }
    k_emitter_reduce<<<1, 256, 0, s>>>(e, step);
}

template void launch_emitter_step<float>(const EmitterDev&, float* const[3], const int*, void*);
template void launch_emitter_step<double>(const EmitterDev&, double* const[3], const int*, void*);

}  // namespace dev
}  // namespace chiml
