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
// The FP64 form keeps all density-matrix arithmetic in FP64; with FP32 fields the Hermitian
// update runs in FP32 with the state as float-float pairs (memberHermSplit). The four
// derivative histories rotate through four slots by step number instead of being copied.
#include <cstdint>

#include "emitter_device.hpp"
#include "launch_dep.hpp"

#ifndef CHIML_EM_SPLIT_MINB_SMALL
#define CHIML_EM_SPLIT_MINB_SMALL 6
#endif
#ifndef CHIML_EM_SPLIT_MINB
#define CHIML_EM_SPLIT_MINB 4
#endif

namespace chiml {
namespace dev {

namespace {

constexpr int kMaxDtc = 8;
constexpr int kEmThreads = 128;

struct C2 {
    double x, y;
};
__device__ __forceinline__ C2 c2(double a, double b) { return C2{a, b}; }
__device__ __forceinline__ C2 cadd(C2 a, C2 b) { return C2{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ C2 cconj(C2 a) { return C2{a.x, -a.y}; }
__device__ __forceinline__ C2 ld(const double2* p) {
    const double2 v = *p;
    return C2{v.x, v.y};
}
__device__ __forceinline__ void st(double2* p, C2 v) { *p = make_double2(v.x, v.y); }
// y + (a, 0) * x, the complex axpy of a real step coefficient: the imaginary part of
// (a, 0) contributes exact zeros, so two FMAs give the same value for finite operands.
__device__ __forceinline__ C2 caxpy(double a, C2 x, C2 y) { return C2{fma(a, x.x, y.x), fma(a, x.y, y.y)}; }
// s + a * b, four FMAs
__device__ __forceinline__ C2 cmac(C2 a, C2 b, C2 s) {
    s.x = fma(a.x, b.x, s.x);
    s.x = fma(-a.y, b.y, s.x);
    s.y = fma(a.x, b.y, s.y);
    s.y = fma(a.y, b.x, s.y);
    return s;
}

// Per-thread population sums over the ensemble members of a density-update block, kept in
// shared memory rather than registers (the update needs every register it can get):
// gPopSh[d * kEmThreads + thread] for population detector d.
__shared__ double2 gPopSh[kMaxDtc * kEmThreads];

__device__ __forceinline__ void addPop(int d, double x, double y) {
    double2& p = gPopSh[d * kEmThreads + threadIdx.x];
    p.x += x;
    p.y += y;
}

// v[k] for a register array: with NT fixed, a chain of selects instead of a dynamic
// index, which would move the array to local memory.
template <int NT>
__device__ __forceinline__ C2 pick(const C2* v, int k) {
    if constexpr (NT == 0) {
        return v[k];
    } else {
        C2 r = v[0];
#pragma unroll
        for (int i = 1; i < NT * NT; ++i)
            if (k == i) r = v[i];
        return r;
    }
}

// (i/hbar) H den + its conjugate transpose, plus the relaxation rows (denDeriv, MKL form).
// The factor i/hbar is purely imaginary: (0, w) * s = (-w s.y, w s.x) exactly. With
// t(r, c) = (i/hbar) sum_l H[r + l n] den[l + c n], the element pair (i, j), (j, i) of the
// result is t(i, j) + conj(t(j, i)) and its exact conjugate (the sum commutes and conj
// is exact), so each pair i <= j is formed once.
// FP64 issue rate is the bound of this kernel, so the complex products are FMA chains.
template <int NT>
__device__ __forceinline__ void den_deriv(const EmitterDev& e, int N, double invHbar, const C2* H, const C2* den, C2* out) {
    const int n = NT ? NT : N;
#pragma unroll
    for (int i = 0; i < (NT ? NT : n); ++i)
#pragma unroll
        for (int j = i; j < (NT ? NT : n); ++j) {
            C2 sij = c2(0.0, 0.0), sji = c2(0.0, 0.0);
#pragma unroll
            for (int l = 0; l < (NT ? NT : n); ++l) {
                sij = cmac(H[i + l * n], den[l + j * n], sij);
                if (j != i) sji = cmac(H[j + l * n], den[l + i * n], sji);
            }
            if (j == i) sji = sij;
            const C2 tij = C2{-invHbar * sij.y, invHbar * sij.x};
            const C2 tji = C2{-invHbar * sji.y, invHbar * sji.x};
            // the MKL form stores t column-major and adds conj of the transpose:
            // out[j * n + i] = t(i, j) + conj(t(j, i)), out[i * n + j] its conjugate
            const C2 o = cadd(tij, cconj(tji));
            out[j * n + i] = o;
            if (j != i) out[i * n + j] = cconj(o);
        }
#pragma unroll
    for (int ii = 0; ii < (NT ? NT * NT : n * n); ++ii)
        for (int p = e.gamRow[ii]; p < e.gamRow[ii + 1]; ++p) {
            const C2 d = pick<NT>(den, e.gamCol[p]);
            const double g = e.gamVal[p];
            out[ii] = C2{fma(d.x, g, out[ii].x), fma(d.y, g, out[ii].y)};
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
        v = fma(P[pa], e.negHalfInvEps[pa], v);  // -0.5 P / eps, the reciprocal formed on the host
        v = fma(P[pb], e.negHalfInvEps[pb], v);
        E[g] = static_cast<T>(v);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_emitter_addp(const EmitterDev e, T* Ex, T* Ey, T* Ez) {
    waitPriorGrid();
    addpRange(e, Ex, Ey, Ez, blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// ---- Hermitian form (EmitterDev::herm) ----
// With real symmetric dipole operators and a relaxation that maps every element pair
// (r, c), (c, r) onto conjugate pairs, the reference's density matrices stay Hermitian and
// H = h0 - E . mu is real symmetric. The step then needs only the upper triangle: the
// diagonal is real, (c, r) = conj (r, c). Element (r, c) has storage index r + c N.

// Element (r, c) of a Hermitian matrix of which only the upper triangle (r <= c) is held,
// at storage index r + c NT; the lower triangle is the conjugate of its mirror. With r and
// c known at compile time the lower elements cost no registers.
template <int NT>
__device__ __forceinline__ C2 hel(const C2* a, int r, int c) {
    return r <= c ? a[r + c * NT] : C2{a[c + r * NT].x, -a[c + r * NT].y};
}
// Element (r, c) of a real symmetric matrix held as its upper triangle.
template <int NT>
__device__ __forceinline__ double sel(const double* h, int r, int c) {
    return r <= c ? h[r + c * NT] : h[c + r * NT];
}
// hel at a flat index k = r + c NT known only at run time: a chain of selects over the
// upper triangle, and for a lower element the sign of the imaginary part flipped by an
// integer operation (keeping the FP64 pipe, which bounds the update, free of it).
template <int NT>
__device__ __forceinline__ C2 pickHerm(const C2* a, int k) {
    const int r = k % NT, c = k / NT;
    const bool lower = r > c;
    const int ku = lower ? c + r * NT : k;
    C2 v = a[0];
#pragma unroll
    for (int i = 1; i < NT * NT; ++i)
        if ((i % NT) <= (i / NT) && ku == i) v = a[i];
    const unsigned long long flip = lower ? 0x8000000000000000ULL : 0ULL;
    v.y = __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(__double_as_longlong(v.y)) ^ flip));
    return v;
}

// Upper-triangle derivative: out(r, c) = t(r, c) + conj t(c, r) for r < c, and the real
// diagonal t(r, r) + conj t(r, r) = 2 Re t(r, r); t = i Hs den with Hs = H / hbar real
// (scaled once per step). With s(i, j) = sum_l Hs(i, l) den(l, j):
//   out(i, j) = (-(Im s(i, j) + Im s(j, i)), Re s(i, j) - Re s(j, i)),
// each sum formed in one FMA chain.
// hmask: bit i set when element i of H can be nonzero (the diagonal, and wherever a coupled
// dipole operator is nonzero); products with the other elements are exact zeros and are
// skipped (the branch is uniform over the emitter). The diagonal of den is real.
template <int NT>
__device__ __forceinline__ void den_deriv_herm(const EmitterDev& e, const double* Hs, const C2* den, C2* out, unsigned hmask) {
#pragma unroll
    for (int i = 0; i < NT; ++i) {
        // Re t(i, i) = -Im s(i, i); den(i, i) is real
        double sy = 0.0;
#pragma unroll
        for (int l = 0; l < NT; ++l)
            if (l != i && (hmask >> (i + l * NT) & 1u)) sy = fma(sel<NT>(Hs, i, l), hel<NT>(den, l, i).y, sy);
        out[i + i * NT] = C2{-2.0 * sy, 0.0};
#pragma unroll
        for (int j = i + 1; j < NT; ++j) {
            double ox = 0.0, oy = 0.0;
#pragma unroll
            for (int l = 0; l < NT; ++l) {
                if (hmask >> (i + l * NT) & 1u) {
                    const C2 d = hel<NT>(den, l, j);
                    if (l != j) ox = fma(-sel<NT>(Hs, i, l), d.y, ox);
                    oy = fma(sel<NT>(Hs, i, l), d.x, oy);
                }
                if (hmask >> (j + l * NT) & 1u) {
                    const C2 d = hel<NT>(den, l, i);
                    if (l != i) ox = fma(-sel<NT>(Hs, j, l), d.y, ox);
                    oy = fma(-sel<NT>(Hs, j, l), d.x, oy);
                }
            }
            out[i + j * NT] = C2{ox, oy};
        }
    }
#pragma unroll
    for (int ii = 0; ii < NT * NT; ++ii) {
        if ((ii % NT) > (ii / NT)) continue;  // lower triangle: the conjugate of its mirror
        for (int p = e.gamRow[ii]; p < e.gamRow[ii + 1]; ++p) {
            const C2 d = pickHerm<NT>(den, e.gamCol[p]);
            const double g = e.gamVal[p];
            out[ii] = C2{fma(d.x, g, out[ii].x), (ii % NT) == (ii / NT) ? 0.0 : fma(d.y, g, out[ii].y)};
        }
    }
}

// One ensemble member of one cell in the Hermitian form: loads and stores the upper
// triangle only (the diagonal's real part), about half the FP64 work and bytes of the
// general form.
template <int NT>
__device__ __forceinline__ void memberHerm(const EmitterDev& e, const double Ec[3], bool zeroE, int m, long long base,
                                           const double2* __restrict__ k0, const double2* __restrict__ k1,
                                           const double2* __restrict__ k2, double2* __restrict__ k3, bool popStep,
                                           double* Pc) {
    constexpr int N2 = NT * NT;
    const double c55 = e.abP[0], cm59 = e.abP[1], c37 = e.abP[2], cm9 = e.abP[3];
    const double c9 = e.abC[0], c19 = e.abC[1], cm5 = e.abC[2], c1 = e.abC[3];
    // H / hbar, upper triangle (H is real symmetric)
    double H[N2];
#pragma unroll
    for (int i = 0; i < N2; ++i) H[i] = 0.0;
#pragma unroll
    for (int i = 0; i < NT; ++i) H[i * NT + i] = e.h0[m * NT + i];
    if (!zeroE)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (e.addMu[c])
#pragma unroll
                for (int i = 0; i < N2; ++i)
                    if ((i % NT) <= (i / NT) && (e.hmask >> i & 1u)) H[i] = fma(Ec[c], e.negMu[c * N2 + i].x, H[i]);
#pragma unroll
    for (int i = 0; i < N2; ++i)
        if ((i % NT) <= (i / NT) && (e.hmask >> i & 1u)) H[i] *= e.invHbar;
    const double* rhoD = reinterpret_cast<const double*>(e.rho);
    // up to three levels the current density stays in registers for the corrector; above,
    // it is read again (an L1 hit) to leave the registers to the derivative
    constexpr bool KEEP = NT <= 3;
    C2 a[N2], b[N2], r0[KEEP ? N2 : 1];
    // predictor on the upper triangle
#pragma unroll
    for (int c = 0; c < NT; ++c)
#pragma unroll
        for (int r = 0; r <= c; ++r) {
            const int i = r + c * NT;
            const long long o = base + static_cast<long long>(i) * e.nc;
            if (r == c) {
                const double rr = rhoD[2 * o];
                double p = fma(c55, reinterpret_cast<const double*>(k0)[2 * o], rr);
                p = fma(cm59, reinterpret_cast<const double*>(k1)[2 * o], p);
                p = fma(c37, reinterpret_cast<const double*>(k2)[2 * o], p);
                p = fma(cm9, reinterpret_cast<const double*>(k3)[2 * o], p);
                if constexpr (KEEP) r0[i] = C2{rr, 0.0};
                a[i] = C2{p, 0.0};
            } else {
                const C2 rr = ld(&e.rho[o]);
                C2 p = caxpy(c55, ld(&k0[o]), rr);
                p = caxpy(cm59, ld(&k1[o]), p);
                p = caxpy(c37, ld(&k2[o]), p);
                p = caxpy(cm9, ld(&k3[o]), p);
                if constexpr (KEEP) r0[i] = rr;
                a[i] = p;
            }
        }
    den_deriv_herm<NT>(e, H, a, b, e.hmask);
    // corrector
#pragma unroll
    for (int c = 0; c < NT; ++c)
#pragma unroll
        for (int r = 0; r <= c; ++r) {
            const int i = r + c * NT;
            const long long o = base + static_cast<long long>(i) * e.nc;
            if (r == c) {
                double v = fma(c9, b[i].x, KEEP ? r0[KEEP ? i : 0].x : rhoD[2 * o]);
                v = fma(c19, reinterpret_cast<const double*>(k0)[2 * o], v);
                v = fma(cm5, reinterpret_cast<const double*>(k1)[2 * o], v);
                v = fma(c1, reinterpret_cast<const double*>(k2)[2 * o], v);
                a[i] = C2{v, 0.0};
                reinterpret_cast<double*>(e.rho)[2 * o] = v;
            } else {
                C2 v = caxpy(c9, b[i], KEEP ? r0[KEEP ? i : 0] : ld(&e.rho[o]));
                v = caxpy(c19, ld(&k0[o]), v);
                v = caxpy(cm5, ld(&k1[o]), v);
                v = caxpy(c1, ld(&k2[o]), v);
                a[i] = v;
                st(&e.rho[o], v);
            }
        }
    den_deriv_herm<NT>(e, H, a, b, e.hmask);  // derivative at the new density: the next k_n
#pragma unroll
    for (int c = 0; c < NT; ++c)
#pragma unroll
        for (int r = 0; r <= c; ++r) {
            const int i = r + c * NT;
            const long long o = base + static_cast<long long>(i) * e.nc;
            if (r == c) reinterpret_cast<double*>(k3)[2 * o] = b[i].x;
            else st(&k3[o], b[i]);
        }
    if (popStep)
#pragma unroll
        for (int d = 0; d < kMaxDtc; ++d)
            if (d < e.nDtc) {
                const C2 v = pickHerm<NT>(a, e.dtcLev[d]);
                addPop(d, v.x, v.y);
            }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        // Re(conj(a) . mu) with mu real: zero for an operator without nonzero elements, and
        // only the elements hmask marks can be nonzero
        if (!e.comp[c] || !e.addMu[c]) continue;
        double sdot = 0.0;
#pragma unroll
        for (int i = 0; i < N2; ++i)
            if (e.hmask >> i & 1u) sdot = fma(hel<NT>(a, i % NT, i / NT).x, e.mu[c * N2 + i].x, sdot);
        Pc[c] += e.na * sdot;
    }
}

// ---- Split form of the Hermitian update ----
//
// With FP32 fields the density update runs on the FP32 pipe, which has 64 times the FP64
// pipe's issue rate on this GPU. Each real of the density matrix is held as a float-float
// pair (hi + lo with |lo| <= ulp(hi) / 2, a 48-bit significand: Dekker's double-length
// representation), so that the state loses nothing over 10^5 steps; the four derivative
// histories are FP32. A step forms each ABM4 increment (a weighted sum of derivatives times
// dt) in FP32 and adds it to the pair exactly (Knuth's TwoSum, then a renormalising
// FastTwoSum). The derivative itself, i [H / hbar, rho] + Gamma rho, is evaluated in FP32
// on rho's hi part, except for its largest and most regular term, the free precession
// i (h0_i - h0_j) / hbar rho_ij: the level difference is a float-float pair, so that the
// precession frequency carries no rounding that would add up to a phase drift over a
// long run. Population outputs are read from the pairs in FP64.
struct F2 {
    float x, y;
};

// hi + lo as an FP64 value
__device__ __forceinline__ double dfToDouble(float hi, float lo) { return static_cast<double>(hi) + static_cast<double>(lo); }

// (hi, lo) + v exactly, renormalised
__device__ __forceinline__ void dfAdd(float& hi, float& lo, float v) {
    const float s = hi + v;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (v - bb);  // TwoSum error of hi + v
    const float l2 = lo + err;
    const float h = s + l2;                        // FastTwoSum(s, l2), |s| >= |l2|
    lo = l2 - (h - s);
    hi = h;
}

// (hi, lo) + (bh, bl), renormalised (the pair sum of Dekker's double-length arithmetic)
__device__ __forceinline__ void dfAddPair(float& hi, float& lo, float bh, float bl) {
    const float s = hi + bh;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (bh - bb);
    const float l2 = (lo + bl) + err;
    const float h = s + l2;
    lo = l2 - (h - s);
    hi = h;
}

// The split form sums each cell's members on the FP32 pipe: the population of detector d
// as a (re hi, re lo, im hi, im lo) float4 in the 16 bytes of gPopSh[d][thread], turned
// into the double2 the block reduction reads once the cell's members are done.
__device__ __forceinline__ void addPopSplit(int d, float4 v) {
    float4& p = reinterpret_cast<float4&>(gPopSh[d * kEmThreads + threadIdx.x]);
    dfAddPair(p.x, p.y, v.x, v.y);
    dfAddPair(p.z, p.w, v.z, v.w);
}
__device__ __forceinline__ void popSplitToDouble(int d) {
    const float4 p = reinterpret_cast<const float4&>(gPopSh[d * kEmThreads + threadIdx.x]);
    gPopSh[d * kEmThreads + threadIdx.x] = make_double2(dfToDouble(p.x, p.y), dfToDouble(p.z, p.w));
}

// Upper-triangle derivative of the split form (the arrangement of den_deriv_herm): HE the
// coupling -E . mu / hbar (real symmetric, upper triangle, FP32), den the density's hi
// parts, dl the level differences of this member, cmask the nonzero elements of HE.
template <int NT>
__device__ __forceinline__ void den_deriv_split(const EmitterDev& e, const float* HE, const F2* den, const float2* dl,
                                                F2* out, unsigned cmask) {
#pragma unroll
    for (int i = 0; i < NT; ++i) {
        float sy = 0.f;
#pragma unroll
        for (int l = 0; l < NT; ++l)
            if (l != i && (cmask >> (i + l * NT) & 1u)) {
                const float h = (i <= l) ? HE[i + l * NT] : HE[l + i * NT];
                const float dy = (l <= i) ? den[l + i * NT].y : -den[i + l * NT].y;
                sy = fmaf(h, dy, sy);
            }
        out[i + i * NT] = F2{-2.f * sy, 0.f};
#pragma unroll
        for (int j = i + 1; j < NT; ++j) {
            float ox = 0.f, oy = 0.f;
#pragma unroll
            for (int l = 0; l < NT; ++l) {
                if (cmask >> (i + l * NT) & 1u) {
                    const float h = (i <= l) ? HE[i + l * NT] : HE[l + i * NT];
                    const F2 d = (l <= j) ? den[l + j * NT] : F2{den[j + l * NT].x, -den[j + l * NT].y};
                    if (l != j) ox = fmaf(-h, d.y, ox);
                    oy = fmaf(h, d.x, oy);
                }
                if (cmask >> (j + l * NT) & 1u) {
                    const float h = (j <= l) ? HE[j + l * NT] : HE[l + j * NT];
                    const F2 d = (l <= i) ? den[l + i * NT] : F2{den[i + l * NT].x, -den[i + l * NT].y};
                    if (l != i) ox = fmaf(-h, d.y, ox);
                    oy = fmaf(-h, d.x, oy);
                }
            }
            // free precession i (d_i - d_j) rho_ij with the difference as hi + lo
            const float2 dd = dl[i + j * NT];
            const F2 r = den[i + j * NT];
            ox = ox - fmaf(dd.y, r.y, dd.x * r.y);
            oy = oy + fmaf(dd.y, r.x, dd.x * r.x);
            out[i + j * NT] = F2{ox, oy};
        }
    }
#pragma unroll
    for (int ii = 0; ii < NT * NT; ++ii) {
        if ((ii % NT) > (ii / NT)) continue;
        for (int p = e.gamRow[ii]; p < e.gamRow[ii + 1]; ++p) {
            const int k = e.gamCol[p];
            const int r = k % NT, c = k / NT;
            const bool lower = r > c;
            const int ku = lower ? c + r * NT : k;
            F2 d = den[0];
#pragma unroll
            for (int t = 1; t < NT * NT; ++t)
                if ((t % NT) <= (t / NT) && ku == t) d = den[t];
            if (lower) d.y = -d.y;
            const float g = e.gamValF[p];
            out[ii] = F2{fmaf(d.x, g, out[ii].x), (ii % NT) == (ii / NT) ? 0.f : fmaf(d.y, g, out[ii].y)};
        }
    }
}

// One ensemble member of one cell in the split form (the upper triangle, as memberHerm).
template <int NT>
__device__ __forceinline__ void memberHermSplit(const EmitterDev& e, const float* HE, int m, long long base,
                                                const float2* __restrict__ k0, const float2* __restrict__ k1,
                                                const float2* __restrict__ k2, float2* __restrict__ k3, bool popStep,
                                                float2* PcF, unsigned cmask) {
    constexpr int N2 = NT * NT;
    const float c55 = e.abPf[0], cm59 = e.abPf[1], c37 = e.abPf[2], cm9 = e.abPf[3];
    const float c9 = e.abCf[0], c19 = e.abCf[1], cm5 = e.abCf[2], c1 = e.abCf[3];
    const float2* dl = e.dlevF + m * N2;
    float4 r0[N2];  // the state (hi, lo pairs)
    F2 a[N2], b[N2];
    // predictor: rho + increment, in FP32 on the hi parts (the derivative's input)
#pragma unroll
    for (int c = 0; c < NT; ++c)
#pragma unroll
        for (int r = 0; r <= c; ++r) {
            const int i = r + c * NT;
            const long long o = base + static_cast<long long>(i) * e.nc;
            if (r == c) {
                const float2 rr = *reinterpret_cast<const float2*>(&e.rhoF[o]);
                float inc = c55 * reinterpret_cast<const float*>(k0)[2 * o];
                inc = fmaf(cm59, reinterpret_cast<const float*>(k1)[2 * o], inc);
                inc = fmaf(c37, reinterpret_cast<const float*>(k2)[2 * o], inc);
                inc = fmaf(cm9, reinterpret_cast<const float*>(k3)[2 * o], inc);
                r0[i] = make_float4(rr.x, rr.y, 0.f, 0.f);
                a[i] = F2{rr.x + inc, 0.f};
            } else {
                const float4 rr = e.rhoF[o];
                const float2 x0 = k0[o], x1 = k1[o], x2 = k2[o], x3 = k3[o];
                float ix = c55 * x0.x, iy = c55 * x0.y;
                ix = fmaf(cm59, x1.x, ix);
                iy = fmaf(cm59, x1.y, iy);
                ix = fmaf(c37, x2.x, ix);
                iy = fmaf(c37, x2.y, iy);
                ix = fmaf(cm9, x3.x, ix);
                iy = fmaf(cm9, x3.y, iy);
                r0[i] = rr;
                a[i] = F2{rr.x + ix, rr.z + iy};
            }
        }
    den_deriv_split<NT>(e, HE, a, dl, b, cmask);
    // corrector: rho + increment exactly into the pairs
#pragma unroll
    for (int c = 0; c < NT; ++c)
#pragma unroll
        for (int r = 0; r <= c; ++r) {
            const int i = r + c * NT;
            const long long o = base + static_cast<long long>(i) * e.nc;
            if (r == c) {
                float inc = c9 * b[i].x;
                inc = fmaf(c19, reinterpret_cast<const float*>(k0)[2 * o], inc);
                inc = fmaf(cm5, reinterpret_cast<const float*>(k1)[2 * o], inc);
                inc = fmaf(c1, reinterpret_cast<const float*>(k2)[2 * o], inc);
                float hi = r0[i].x, lo = r0[i].y;
                dfAdd(hi, lo, inc);
                r0[i] = make_float4(hi, lo, 0.f, 0.f);
                *reinterpret_cast<float2*>(&e.rhoF[o]) = make_float2(hi, lo);
                a[i] = F2{hi, 0.f};
            } else {
                const float2 x0 = k0[o], x1 = k1[o], x2 = k2[o];
                float ix = c9 * b[i].x, iy = c9 * b[i].y;
                ix = fmaf(c19, x0.x, ix);
                iy = fmaf(c19, x0.y, iy);
                ix = fmaf(cm5, x1.x, ix);
                iy = fmaf(cm5, x1.y, iy);
                ix = fmaf(c1, x2.x, ix);
                iy = fmaf(c1, x2.y, iy);
                float4 v = r0[i];
                dfAdd(v.x, v.y, ix);
                dfAdd(v.z, v.w, iy);
                r0[i] = v;
                e.rhoF[o] = v;
                a[i] = F2{v.x, v.z};
            }
        }
    den_deriv_split<NT>(e, HE, a, dl, b, cmask);  // derivative at the new density: the next k_n
#pragma unroll
    for (int c = 0; c < NT; ++c)
#pragma unroll
        for (int r = 0; r <= c; ++r) {
            const int i = r + c * NT;
            const long long o = base + static_cast<long long>(i) * e.nc;
            if (r == c) reinterpret_cast<float*>(k3)[2 * o] = b[i].x;
            else k3[o] = make_float2(b[i].x, b[i].y);
        }
    if (popStep)
#pragma unroll
        for (int d = 0; d < kMaxDtc; ++d)
            if (d < e.nDtc) {
                const int k = e.dtcLev[d];
                const int r = k % NT, c = k / NT;
                const bool lower = r > c;
                const int ku = lower ? c + r * NT : k;
                float4 v = r0[0];
#pragma unroll
                for (int t = 1; t < N2; ++t)
                    if ((t % NT) <= (t / NT) && ku == t) v = r0[t];
                if (lower) v.z = -v.z, v.w = -v.w;
                addPopSplit(d, v);
            }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        // Re(conj(a) . mu) with mu real, over the elements hmask marks
        if (!e.comp[c] || !e.addMu[c]) continue;
        float sdot = 0.f;
#pragma unroll
        for (int i = 0; i < N2; ++i)
            if (e.hmask >> i & 1u) {
                const int r = i % NT, cc = i / NT;
                const float ax = r <= cc ? a[i].x : a[cc + r * NT].x;
                sdot = fmaf(ax, static_cast<float>(e.mu[c * N2 + i].x), sdot);
            }
        dfAdd(PcF[c].x, PcF[c].y, sdot);  // the sum over members; times na once per cell
    }
}

// Block `blk` of the density update (cells kEmThreads * blk ...), writing partial row blk.
// SPLIT: the split form of the Hermitian update (T = float, memberHermSplit).
template <typename T, int NT, bool HERM = false, bool SPLIT = false>
__device__ __forceinline__ void updateBlock(const EmitterDev& e, const T* __restrict__ Ex, const T* __restrict__ Ey,
                                            const T* __restrict__ Ez, const int* __restrict__ stepPtr, int blk) {
    constexpr int MAXN2 = (NT ? NT * NT : kMaxEmitterLevels * kMaxEmitterLevels);
    const int N = NT ? NT : e.N;
    const int n2 = N * N;
    const int q = blk * kEmThreads + threadIdx.x;
    const int s = *stepPtr;
    const bool popStep = (s % e.dtcTimeInt) == 0;
    if (popStep)
#pragma unroll
        for (int d = 0; d < kMaxDtc; ++d)
            if (d < e.nDtc) gPopSh[d * kEmThreads + threadIdx.x] = make_double2(0.0, 0.0);
    double Pc[3] = {0.0, 0.0, 0.0};
    if (q < e.nc) {
        // E at the cell centre
        const long long g = e.cellGrid[q];
        const T* Es[3] = {Ex, Ey, Ez};
        double Ec[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (!e.comp[c]) continue;
            if constexpr (SPLIT) {
                // FP32 fields, FP32 coupling: the average on the FP32 pipe
                if (c == 2 && e.gatherZCopy) Ec[c] = static_cast<double>(Es[c][g]);
                else Ec[c] = static_cast<double>(0.5f * static_cast<float>(Es[c][g]) + 0.5f * static_cast<float>(Es[c][g - e.unit[c]]));
            } else {
                if (c == 2 && e.gatherZCopy) Ec[c] = static_cast<double>(Es[c][g]);
                else Ec[c] = 0.5 * static_cast<double>(Es[c][g]) + 0.5 * static_cast<double>(Es[c][g - e.unit[c]]);
            }
        }
        if (e.cellDip) {
            // a per-cell dipole w: the coupling is (E . w) times the z operator
            const double ew = Ec[0] * e.cellDip[q] + Ec[1] * e.cellDip[e.nc + q] + Ec[2] * e.cellDip[2 * e.nc + q];
            Ec[0] = 0.0;
            Ec[1] = 0.0;
            Ec[2] = ew;
        }
        const bool zeroE = (Ec[0] == 0.0 && Ec[1] == 0.0 && Ec[2] == 0.0);
        const long long slotStride = static_cast<long long>(e.nm) * n2 * e.nc;
        const int s0 = (s - 1) & 3, s1 = (s - 2) & 3, s2 = (s - 3) & 3, s3 = s & 3;  // k_n, k_n-1, k_n-2, k_n-3
        const double c55 = e.abP[0], cm59 = e.abP[1], c37 = e.abP[2], cm9 = e.abP[3];
        const double c9 = e.abC[0], c19 = e.abC[1], cm5 = e.abC[2], c1 = e.abC[3];
        const double invHbar = e.invHbar;
        const double2* __restrict__ k0 = e.kd + s0 * slotStride;
        const double2* __restrict__ k1 = e.kd + s1 * slotStride;
        const double2* __restrict__ k2 = e.kd + s2 * slotStride;
        double2* __restrict__ k3 = e.kd + s3 * slotStride;
        if constexpr (HERM && SPLIT) {
            // the coupling -E . mu / hbar once per cell (it does not depend on the member)
            constexpr int N2 = NT * NT;
            float HE[N2];
            unsigned cmask = 0;
#pragma unroll
            for (int i = 0; i < N2; ++i) HE[i] = 0.f;
            if (!zeroE)
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    if (e.addMu[c])
#pragma unroll
                        for (int i = 0; i < N2; ++i)
                            if ((i % NT) <= (i / NT) && (e.hmask >> i & 1u))
                                HE[i] = fmaf(static_cast<float>(Ec[c]), e.negMuHF[c * N2 + i], HE[i]);
            // the nonzero couplings, mirrored (HE is symmetric)
#pragma unroll
            for (int i = 0; i < N2; ++i)
                if ((i % NT) <= (i / NT) && HE[i] != 0.f) cmask |= (1u << i) | (1u << ((i / NT) + (i % NT) * NT));
            const float2* __restrict__ f0 = e.kdF + s0 * slotStride;
            const float2* __restrict__ f1 = e.kdF + s1 * slotStride;
            const float2* __restrict__ f2 = e.kdF + s2 * slotStride;
            float2* __restrict__ f3 = e.kdF + s3 * slotStride;
            float2 PcF[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            for (int m = 0; m < e.nm; ++m)
                memberHermSplit<NT>(e, HE, m, static_cast<long long>(m) * n2 * e.nc + q, f0, f1, f2, f3, popStep, PcF,
                                    cmask);
#pragma unroll
            for (int c = 0; c < 3; ++c)
                if (e.comp[c] && e.addMu[c]) Pc[c] = e.na * dfToDouble(PcF[c].x, PcF[c].y);
            if (popStep)
#pragma unroll
                for (int d = 0; d < kMaxDtc; ++d)
                    if (d < e.nDtc) popSplitToDouble(d);
        } else if constexpr (HERM) {
            for (int m = 0; m < e.nm; ++m)
                memberHerm<NT>(e, Ec, zeroE, m, static_cast<long long>(m) * n2 * e.nc + q, k0, k1, k2, k3, popStep,
                               Pc);
        } else {
        C2 H[MAXN2], a[MAXN2], b[MAXN2];
        for (int m = 0; m < e.nm; ++m) {
            // Hamiltonian::getHam
#pragma unroll
            for (int i = 0; i < (NT ? MAXN2 : n2); ++i) H[i] = c2(0.0, 0.0);
#pragma unroll
            for (int i = 0; i < (NT ? NT : N); ++i) H[i * N + i] = c2(e.h0[m * N + i], 0.0);
            if (!zeroE)
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    if (e.addMu[c])
#pragma unroll
                        for (int i = 0; i < (NT ? MAXN2 : n2); ++i) H[i] = caxpy(Ec[c], ld(&e.negMu[c * n2 + i]), H[i]);
            const long long base = static_cast<long long>(m) * n2 * e.nc + q;
            // predictor; for two levels the history values stay in registers for the
            // corrector, for more they are read again (cache hits)
            constexpr bool KEEP = NT == 2;
            constexpr int KN = KEEP ? MAXN2 : 1;
            C2 r0[KN], h0v[KN], h1v[KN], h2v[KN];
#pragma unroll
            for (int i = 0; i < (NT ? MAXN2 : n2); ++i) {
                const long long o = base + static_cast<long long>(i) * e.nc;
                const C2 rr = ld(&e.rho[o]), x0 = ld(&k0[o]), x1 = ld(&k1[o]), x2 = ld(&k2[o]);
                if constexpr (KEEP) {
                    r0[i] = rr;
                    h0v[i] = x0;
                    h1v[i] = x1;
                    h2v[i] = x2;
                }
                C2 p = caxpy(c55, x0, rr);
                p = caxpy(cm59, x1, p);
                p = caxpy(c37, x2, p);
                p = caxpy(cm9, ld(&k3[o]), p);
                a[i] = p;
            }
            den_deriv<NT>(e, N, invHbar, H, a, b);  // b = derivative at the prediction
            // corrector
#pragma unroll
            for (int i = 0; i < (NT ? MAXN2 : n2); ++i) {
                const long long o = base + static_cast<long long>(i) * e.nc;
                C2 rr, x0, x1, x2;
                if constexpr (KEEP) {
                    rr = r0[i];
                    x0 = h0v[i];
                    x1 = h1v[i];
                    x2 = h2v[i];
                } else {
                    rr = ld(&e.rho[o]);
                    x0 = ld(&k0[o]);
                    x1 = ld(&k1[o]);
                    x2 = ld(&k2[o]);
                }
                C2 r = caxpy(c9, b[i], rr);
                r = caxpy(c19, x0, r);
                r = caxpy(cm5, x1, r);
                r = caxpy(c1, x2, r);
                a[i] = r;
                st(&e.rho[o], r);
            }
            den_deriv<NT>(e, N, invHbar, H, a, b);  // derivative at the new density: the next k_n
#pragma unroll
            for (int i = 0; i < (NT ? MAXN2 : n2); ++i) st(&k3[base + static_cast<long long>(i) * e.nc], b[i]);
            if (popStep)
#pragma unroll
                for (int d = 0; d < kMaxDtc; ++d)
                    if (d < e.nDtc) {
                        const C2 v = pick<NT>(a, e.dtcLev[d]);
                        addPop(d, v.x, v.y);
                    }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (!e.comp[c]) continue;
                // Re(conj(a) . mu), the real part of zdotc
                double sdot = 0.0;
#pragma unroll
                for (int i = 0; i < (NT ? MAXN2 : n2); ++i) {
                    const C2 mu = ld(&e.mu[c * n2 + i]);
                    sdot = fma(a[i].x, mu.x, sdot);
                    sdot = fma(a[i].y, mu.y, sdot);
                }
                Pc[c] += e.na * sdot;
            }
        }
        }
        if (e.cellDip) {
            // P_c = w_c times the polarisation of the z operator
            const double pz = Pc[2];
#pragma unroll
            for (int c = 0; c < 3; ++c) Pc[c] = pz * e.cellDip[static_cast<long long>(c) * e.nc + q];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (e.comp[c]) e.P[static_cast<long long>(c) * e.pBox + e.cellP[q]] = Pc[c];
    }
    // Block partial sums of the quantities this step outputs (block-uniform conditions): each
    // quantity's kEmThreads per-thread values sit in shared memory; four threads sum 32 of
    // them each and two shuffles combine the four (a quarter of the additions of a tree over
    // every thread, on the FP64 pipe this kernel is bound by).
    static_assert(4 * (2 * kMaxDtc + 3) <= kEmThreads, "four threads per summed quantity");
    __shared__ double pSh[3 * kEmThreads];
    const bool doP = e.totP != nullptr;
    if (!popStep && !doP) return;
#pragma unroll
    for (int c = 0; c < 3; ++c) pSh[c * kEmThreads + threadIdx.x] = Pc[c];
    __syncthreads();
    const int nPop = popStep ? 2 * e.nDtc : 0;  // tasks: populations (x, y), then P x, y, z
    const int nTask = nPop + (doP ? 3 : 0);
    const int task = threadIdx.x >> 2, part = threadIdx.x & 3;
    double sum = 0.0;
    if (task < nTask) {
        const bool pop = task < nPop;
        const double* src = pop ? reinterpret_cast<const double*>(gPopSh) + 2 * (task >> 1) * kEmThreads + (task & 1)
                                : pSh + (task - nPop) * kEmThreads;
        const int stride = pop ? 2 : 1;
#pragma unroll 8
        for (int j = part * (kEmThreads / 4); j < (part + 1) * (kEmThreads / 4); ++j) sum += src[j * stride];
    }
    sum += __shfl_down_sync(0xffffffffu, sum, 2, 4);
    sum += __shfl_down_sync(0xffffffffu, sum, 1, 4);
    if (part == 0 && task < nTask) {
        if (task < nPop) {
            double* dst = reinterpret_cast<double*>(&e.popPartial[static_cast<long long>(blk) * e.nDtc + (task >> 1)]);
            dst[task & 1] = sum;
        } else if (e.comp[task - nPop]) {
            e.totPartial[blk * 3 + (task - nPop)] = sum;
        }
    }
}

// Resident blocks per SM the register budget is sized for: the FP64 forms are bound by the
// FP64 pipe and keep every register; the split form runs on the FP32 pipe and is closer to
// the memory bound, where more resident cells hide more latency: six blocks for up to three
// levels (80 registers, C3's update 0.53 -> 0.49 ms), four for more (fewer spill).
template <bool SPLIT, int NT = 0>
constexpr int emitterMinBlocks() {
    return SPLIT ? (NT > 0 && NT <= 3 ? CHIML_EM_SPLIT_MINB_SMALL : CHIML_EM_SPLIT_MINB) : 1;
}

template <typename T, int NT, bool HERM = false, bool SPLIT = false>
__global__ void __launch_bounds__(kEmThreads, emitterMinBlocks<SPLIT, NT>()) k_emitter_update(const EmitterDev e, const T* __restrict__ Ex,
                                                               const T* __restrict__ Ey, const T* __restrict__ Ez,
                                                               const int* __restrict__ stepPtr) {
    waitPriorGrid();
    updateBlock<T, NT, HERM, SPLIT>(e, Ex, Ey, Ez, stepPtr, blockIdx.x);
}

// Quantity k of the step's outputs (populations x / y per detector, then total P x, y, z)
// summed over the block partials by one block, in a fixed order: thread t takes the
// partials t + j * kReduceThreads, four independent loads at a time into four
// accumulators, then a tree over the threads.
constexpr int kReduceQuantities = 2 * kMaxDtc + 3;
constexpr int kReduceThreads = 1024;
__device__ __forceinline__ double reducePartial(const EmitterDev& e, bool isPop, int k, int b) {
    if (isPop) {
        const double2 p = e.popPartial[static_cast<long long>(b) * e.nDtc + k / 2];
        return (k & 1) ? p.y : p.x;
    }
    return e.totPartial[b * 3 + (k - 2 * e.nDtc)];
}
__device__ __forceinline__ void reduceBody(const EmitterDev& e, const int* __restrict__ stepPtr, int k) {
    const int s = *stepPtr;
    __shared__ double red[kReduceThreads];
    const bool popStep = (s % e.dtcTimeInt) == 0;
    if (k >= 2 * e.nDtc + 3) return;
    const bool isPop = k < 2 * e.nDtc;
    if (isPop && !popStep) return;
    if (!isPop && (!e.totP || s >= e.nSteps)) return;
    double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
    const int n = e.partialBlocks;
    constexpr int R = kReduceThreads;
    int b = threadIdx.x;
    for (; b + 3 * R < n; b += 4 * R) {
        const double x0 = reducePartial(e, isPop, k, b), x1 = reducePartial(e, isPop, k, b + R);
        const double x2 = reducePartial(e, isPop, k, b + 2 * R), x3 = reducePartial(e, isPop, k, b + 3 * R);
        v0 += x0;
        v1 += x1;
        v2 += x2;
        v3 += x3;
    }
    if (b < n) v0 += reducePartial(e, isPop, k, b);
    if (b + R < n) v1 += reducePartial(e, isPop, k, b + R);
    if (b + 2 * R < n) v2 += reducePartial(e, isPop, k, b + 2 * R);
    red[threadIdx.x] = (v0 + v1) + (v2 + v3);
    __syncthreads();
    for (int w = R / 2; w > 0; w >>= 1) {
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
}

// one block per output quantity (blockIdx.y)
__global__ void __launch_bounds__(kReduceThreads) k_emitter_reduce(const EmitterDev e, const int* __restrict__ stepPtr) {
    waitPriorGrid();
    reduceBody(e, stepPtr, blockIdx.y);
}

// ---- packed launches (batched sweep): work[b] = {job, block of that job} ----

template <typename T>
__global__ void __launch_bounds__(256) k_emitter_addp_packed(const EmitJob<T>* __restrict__ jobs, const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    const EmitJob<T>& j = jobs[w.x];
    const int bpc = emitter_addp_blocks_per_comp(j.e);
    const int c = w.y / bpc, b = w.y % bpc;
    addpRange(j.e, j.f[0], j.f[1], j.f[2], c, b * 256 + static_cast<int>(threadIdx.x), bpc * 256);
}

// The Hermitian form of a batch in FP32 fields is the split form (EmitterDev::split).
template <typename T, int NT, bool HERM = false>
__global__ void __launch_bounds__(kEmThreads, emitterMinBlocks<HERM && sizeof(T) == 4, NT>()) k_emitter_update_packed(const EmitJob<T>* __restrict__ jobs,
                                                                      const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    const EmitJob<T>& j = jobs[w.x];
    updateBlock<T, NT, HERM, HERM && sizeof(T) == 4>(j.e, j.f[0], j.f[1], j.f[2], j.step, w.y);
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) k_emitter_reduce_packed(const EmitJob<T>* __restrict__ jobs) {
    waitPriorGrid();
    const EmitJob<T>& j = jobs[blockIdx.x];
    reduceBody(j.e, j.step, blockIdx.y);
}

}  // namespace

int emitter_update_blocks(const EmitterDev& e) { return (e.nc + kEmThreads - 1) / kEmThreads; }
int emitter_level_group(int N, bool herm) {
    if (herm && N >= 2 && N <= 4) return 2 + N;  // 4, 5, 6: the Hermitian form
    return N == 2 ? 0 : (N == 3 ? 1 : (N == 4 ? 2 : 3));
}

template <typename T>
void launch_emitter_packed(const EmitJob<T>* jobs, int njobs, WorkMap addp, const WorkMap update[7], void* stream) {
    if (njobs <= 0) return;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (addp.blocks > 0) launchAfterPrior(k_emitter_addp_packed<T>, dim3(addp.blocks), dim3(256), s, jobs, addp.work);
    if (update[0].blocks > 0) launchAfterPrior(k_emitter_update_packed<T, 2>, dim3(update[0].blocks), dim3(kEmThreads), s, jobs, update[0].work);
    if (update[1].blocks > 0) launchAfterPrior(k_emitter_update_packed<T, 3>, dim3(update[1].blocks), dim3(kEmThreads), s, jobs, update[1].work);
    if (update[2].blocks > 0) launchAfterPrior(k_emitter_update_packed<T, 4>, dim3(update[2].blocks), dim3(kEmThreads), s, jobs, update[2].work);
    if (update[3].blocks > 0) launchAfterPrior(k_emitter_update_packed<T, 0>, dim3(update[3].blocks), dim3(kEmThreads), s, jobs, update[3].work);
    if (update[4].blocks > 0)
        launchAfterPrior(k_emitter_update_packed<T, 2, true>, dim3(update[4].blocks), dim3(kEmThreads), s, jobs, update[4].work);
    if (update[5].blocks > 0)
        launchAfterPrior(k_emitter_update_packed<T, 3, true>, dim3(update[5].blocks), dim3(kEmThreads), s, jobs, update[5].work);
    if (update[6].blocks > 0)
        launchAfterPrior(k_emitter_update_packed<T, 4, true>, dim3(update[6].blocks), dim3(kEmThreads), s, jobs, update[6].work);
    launchAfterPrior(k_emitter_reduce_packed<T>, dim3(njobs, kReduceQuantities), dim3(kReduceThreads), s, jobs);
}

template void launch_emitter_packed<float>(const EmitJob<float>*, int, WorkMap, const WorkMap[7], void*);
template void launch_emitter_packed<double>(const EmitJob<double>*, int, WorkMap, const WorkMap[7], void*);

template <typename T>
void launch_emitter_step(const EmitterDev& e, T* const fields[3], const int* step, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 ga(emitter_addp_blocks_per_comp(e), 3);
    launchAfterPrior(k_emitter_addp<T>, dim3(ga), dim3(256), s, e, fields[0], fields[1], fields[2]);
    const int blocks = (e.nc + kEmThreads - 1) / kEmThreads;
    // the Hermitian form in FP32 fields is the split form (EmitterDev::split)
    constexpr bool SPLIT = sizeof(T) == 4;
    if (e.herm && e.N >= 2 && e.N <= 4) {
        if (e.N == 2) launchAfterPrior(k_emitter_update<T, 2, true, SPLIT>, dim3(blocks), dim3(kEmThreads), s, e, fields[0], fields[1], fields[2], step);
        else if (e.N == 3) launchAfterPrior(k_emitter_update<T, 3, true, SPLIT>, dim3(blocks), dim3(kEmThreads), s, e, fields[0], fields[1], fields[2], step);
        else launchAfterPrior(k_emitter_update<T, 4, true, SPLIT>, dim3(blocks), dim3(kEmThreads), s, e, fields[0], fields[1], fields[2], step);
    } else switch (e.N) {
        case 2: launchAfterPrior(k_emitter_update<T, 2>, dim3(blocks), dim3(kEmThreads), s, e, fields[0], fields[1], fields[2], step); break;
        case 3: launchAfterPrior(k_emitter_update<T, 3>, dim3(blocks), dim3(kEmThreads), s, e, fields[0], fields[1], fields[2], step); break;
        case 4: launchAfterPrior(k_emitter_update<T, 4>, dim3(blocks), dim3(kEmThreads), s, e, fields[0], fields[1], fields[2], step); break;
        default: launchAfterPrior(k_emitter_update<T, 0>, dim3(blocks), dim3(kEmThreads), s, e, fields[0], fields[1], fields[2], step); break;
    }
    launchAfterPrior(k_emitter_reduce, dim3(1, kReduceQuantities), dim3(kReduceThreads), s, e, step);
}

template void launch_emitter_step<float>(const EmitterDev&, float* const[3], const int*, void*);
template void launch_emitter_step<double>(const EmitterDev&, double* const[3], const int*, void*);

}  // namespace dev
}  // namespace chiml
