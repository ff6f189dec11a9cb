// Time-step kernels for sm_103a (GB300).
//
// k_pass runs one half step of every component of one kind (H, or E with its
// polarisations) in a single pass over the grid: per cell it reads the class
// code, applies the CPML psi recursion, the interior or CPML curl terms and,
// for dispersive cells, the Lorentz ADE before and D -> E after. It fuses the
// reference's per-run BLAS chains (TwoCompCurl, UpdateLorPol, DtoU,
// addPsi/updatePsiField: UTIL/FDTD_up_eq.cpp:10-62,425-448,838-848,
// PML/parallelPML.cpp:12-40) into one read and one write of each array.
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "fdtd_device.hpp"
#include "launch_dep.hpp"

namespace chiml {
namespace dev {

// One pole of the Lorentz recursion at one point: p (P, updated) and pm (P- or J, see
// kIncrementPoles), from the drive term g = gamma E (or gamma d (d . <E>)).
template <typename T>
__device__ __forceinline__ void poleStep(T& p, T& pm, T A, T B, T g) {
    if (kIncrementPoles<T>) {
        T j = B * pm;
        j += A * p;
        j += g;
        p = p + j;
        pm = j;
    } else {
        const T old = p;
        T np = A * old;
        np += B * pm;
        np += g;
        p = np;
        pm = old;
    }
}

// One component of one cell, any class (the arithmetic every pass form shares).
template <typename T, bool EPASS>
__device__ __forceinline__ void cellGeneric(const Pass<T>& p, int ci, long long i, const int coord[3]) {
    const Comp<T>& c = p.c[ci];
    const uint8_t code = c.code[i];
    if (code == 0) return;
    if (code >= c.ncls) {
        atomicOr(p.err, kErrClassCode);
        return;
    }
    const Class<T> k = c.cls[code];
    if (EPASS && k.lor) {
        if (k.obj < 0 || k.obj >= p.nObj || p.poleCount[k.obj] > c.nPoles) {
            atomicOr(p.err, kErrPoleCount);
            return;
        }
        const T e = c.U[i];
        const int s = p.poleStart[k.obj];
        const int n = p.poleCount[k.obj];
        for (int q = 0; q < n; ++q) {
            T pq = c.P[q][i], pm = c.Pprev[q][i];
            poleStep(pq, pm, p.poleA[s + q], p.poleB[s + q], p.gamma[s + q] * e);
            c.P[q][i] = pq;
            c.Pprev[q][i] = pm;
        }
    }
    T add = T(0);
    bool any = false;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        if (!c.tpresent[t]) continue;
        const int a = coord[c.axis[t]];
        const T coef = k.cint[t] + T(k.nplain[t]) * c.db[t] + (k.kflag[t] ? c.kprof[t][a] : T(0));
        const bool psiTerm = c.hasPsi[t] && k.psiUpd[t];
        if (coef == T(0) && !psiTerm) continue;
        const T diff = c.G[t][i] - c.G[t][i + c.off[t]];
        if (coef != T(0)) {
            add += coef * diff;
            any = true;
        }
        // psi of a cell that never updates it stays zero: only updated cells add it
        if (psiTerm) {
            T ps = c.psi[t][i];
            ps = c.b[t][a] * ps + c.cpsi[t][a] * diff;
            c.psi[t][i] = ps;
            if (k.npsi[t]) {
                add += T(k.npsi[t]) * c.dbpsi[t] * ps;
                any = true;
            }
        }
    }
    if (any) {
        if (k.toD) c.D[i] += add;
        else c.U[i] += add;
    }
    if (EPASS && k.lor) {
        T e = c.D[i];
        e *= k.epsInv;
        for (int q = 0; q < c.nPoles; ++q) e += k.negEpsInv * c.P[q][i];
        c.U[i] = e;
    }
    if (EPASS && k.ordip) {
        // orDipDtoU (FDTD_up_eq.cpp:862-875)
        T e = c.D[i];
        e *= k.epsInv;
        const long long o = p.od.off[ci];
        for (int q = 0; q < p.od.nPoles; ++q) {
            e += k.odCoef * p.od.P[ci][q][i];
            e += k.odCoef * p.od.P[ci][q][i + o];
        }
        c.U[i] = e;
    }
}

// Oriented-dipole polarisations from E^n, before the E curl (UpdateLorPolOrDip,
// UTIL/FDTD_up_eq.cpp:450-521): per pole P = alpha P + xi P_prev + gamma d (d . <E>),
// <E_c> the average of E_c at the point and one cell below along c.
template <typename T>
__device__ __forceinline__ void ordipEntry(const Pass<T>& p, long long j) {
    const OrDipDev<T>& od = p.od;
    if (j >= od.n) return;
    const long long i = od.cell[j];
    const int o = od.obj[j];
    if (o < 0 || o >= p.nObj || p.poleCount[o] > od.nPoles) {
        atomicOr(p.err, kErrPoleCount);
        return;
    }
    const T* Ex = p.c[0].U;
    const T* Ey = p.c[1].U;
    const T* Ez = p.c[2].U;
    const int s = p.poleStart[o];
    const int np = p.poleCount[o];
    for (int pp = 0; pp < np; ++pp) {
        const T dx = od.dip[(pp * 3 + 0) * od.n + j];
        const T dy = od.dip[(pp * 3 + 1) * od.n + j];
        const T dz = od.dip[(pp * 3 + 2) * od.n + j];
        T dot = dx * Ex[i] / T(2);
        dot += T(1) * (dx * Ex[i - od.off[0]] / T(2));
        dot += T(1) * (dy * Ey[i] / T(2));
        dot += T(1) * (dy * Ey[i - od.off[1]] / T(2));
        dot += T(1) * (dz * Ez[i] / T(2));
        dot += T(1) * (dz * Ez[i - od.off[2]] / T(2));
        const T A = p.poleA[s + pp], B = p.poleB[s + pp], g = p.gamma[s + pp];
        const T dd[3] = {dx, dy, dz};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            T pa = od.P[a][pp][i], pm = od.Pprev[a][pp][i];
            if (kIncrementPoles<T>) {
                poleStep(pa, pm, A, B, g * (dd[a] * dot));
            } else {
                // UpdateLorPolOrDip's order: alpha P + xi P-, then + gamma d (d . <E>)
                const T old = pa;
                T np = A * old;
                np = np + B * pm;
                pa = np + g * (dd[a] * dot);
                pm = old;
            }
            od.P[a][pp][i] = pa;
            od.Pprev[a][pp][i] = pm;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_ordip_pol(const Pass<T> p) {
    waitPriorGrid();
    ordipEntry(p, blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x);
}

// One cell of the generic form, every component of the pass.
template <typename T, bool EPASS>
__device__ __forceinline__ void passCell(const Pass<T>& p, int x, int y, int z) {
    if (x >= p.lx || z >= p.lz || y >= p.ly) return;
    const long long i = x + p.pitch * (z + static_cast<long long>(p.lz) * y);
    const int coord[3] = {x, y, z};
#pragma unroll
    for (int ci = 0; ci < 3; ++ci)
        if (p.c[ci].present) cellGeneric<T, EPASS>(p, ci, i, coord);
}

// Blocks of 32 (x) by 1 (z) by kGenBY (y) cells.
constexpr int kGenBY = 8;

template <typename T, bool EPASS>
__global__ void __launch_bounds__(256) k_pass(const Pass<T> p) {
    waitPriorGrid();
    passCell<T, EPASS>(p, blockIdx.x * 32 + threadIdx.x, blockIdx.z * kGenBY + threadIdx.z, blockIdx.y);
}

// The dispersive (Lorentz) cells of the E pass, from a list: the interior form
// leaves them out so that its common path stays small.
template <typename T>
__global__ void __launch_bounds__(256) k_pass_lorentz(const Pass<T> p) {
    waitPriorGrid();
    const long long j = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (j >= p.nLor) return;
    const long long i = p.lorCell[j];
    const int x = static_cast<int>(i % p.pitch);
    const long long r = i / p.pitch;
    const int z = static_cast<int>(r % p.lz);
    const int y = static_cast<int>(r / p.lz);
    const int coord[3] = {x, y, z};
    cellGeneric<T, true>(p, p.lorComp[j], i, coord);
}

// 3-D form of the same update for grids whose halo cells carry no update.
// A block covers a 32 (x) by kP3BZ (z) tile of interior cells of one
// component and walks CY planes along y, the slowest axis of the layout. The
// component (and with it the two derivative axes) is a template parameter.
// Every load a cell needs (class code, the field, both neighbour pairs, psi
// inside the slab) is issued before the class is known; the neighbour along y
// is carried in a register from the previous plane, and the plane PD ahead is
// prefetched into L2. A block decides once whether its tile and planes touch
// the CPML slab of either of its component's terms: blocks that do not run the
// plain path, with no profile or psi logic. The class table (FastClass:
// coefficients folded on the host, flag bits) is read through the read-only
// cache; the cells of a warp mostly share a class. Dispersive cells of the E
// pass are left to k_pass_lorentz. Per cell the arithmetic is that of
// cellGeneric.
constexpr int kP3BZ = 8;
#ifndef CHIML_MARCH_UNROLL
#define CHIML_MARCH_UNROLL 1
#endif
constexpr int kMarchUnroll = CHIML_MARCH_UNROLL;  // planes of the march unrolled together
#ifndef CHIML_P3_CY
#define CHIML_P3_CY 16
#endif
#ifndef CHIML_P3_PD
#define CHIML_P3_PD 2
#endif
constexpr int kP3CY = CHIML_P3_CY;  // planes marched per block
constexpr int kP3PD = CHIML_P3_PD;  // planes ahead of the march that are prefetched into L2

__device__ __forceinline__ void prefetchL2(const void* a) { asm volatile("prefetch.global.L2 [%0];" ::"l"(a)); }


// The dispersive part of one E-pass cell of the FP32 interior form, with cellGeneric's
// arithmetic: the Lorentz ADE from E^n (u), D += curl, then D -> E with the pole sum
// (UpdateLorPol, DtoU, orDipDtoU: UTIL/FDTD_up_eq.cpp:425-448, 838-875). -1/eps_inf and
// -0.5/eps_inf are exact scalings of the class's 1/eps_inf.
template <typename T>
__device__ __forceinline__ T dispersiveE(const Pass<T>& p, int ci, uint32_t fl, int obj, T epsInv, long long i, T u, T add,
                                        bool write) {
    const Comp<T>& c = p.c[ci];
    if (fl & kFcLor) {
        if (obj < 0 || obj >= p.nObj || p.poleCount[obj] > c.nPoles) {
            atomicOr(p.err, kErrPoleCount);
            return u;
        }
        const int s = p.poleStart[obj];
        const int n = p.poleCount[obj];
        // unrolled to the pole bound with guards, so that the loads of every pole are in
        // flight together
#pragma unroll
        for (int q = 0; q < kMaxPoles; ++q) {
            if (q >= n) break;
            T pq = c.P[q][i], pm = c.Pprev[q][i];
            poleStep(pq, pm, p.poleA[s + q], p.poleB[s + q], p.gamma[s + q] * u);
            c.P[q][i] = pq;
            c.Pprev[q][i] = pm;
        }
    }
    T d = c.D[i];
    if (write) {
        d += add;
        c.D[i] = d;
    }
    T e = d * epsInv;
    if (fl & kFcLor) {
        const T ne = -epsInv;
#pragma unroll
        for (int q = 0; q < kMaxPoles; ++q) {
            if (q >= c.nPoles) break;
            e += ne * c.P[q][i];
        }
    } else {
        const T oc = T(-0.5) * epsInv;
        const long long o = p.od.off[ci];
#pragma unroll
        for (int q = 0; q < kMaxPoles; ++q) {
            if (q >= p.od.nPoles) break;
            e += oc * p.od.P[ci][q][i];
            e += oc * p.od.P[ci][q][i + o];
        }
    }
    return e;
}

template <typename T>
__device__ __forceinline__ void dispersiveCell(const Pass<T>& p, int ci, uint32_t fl, int obj, T epsInv, long long i, T u,
                                               T add, bool write) {
    p.c[ci].U[i] = dispersiveE<T>(p, ci, fl, obj, epsInv, i, u, add, write);
}

// The update of one cell of component CI from its loaded values (class code cd, field u,
// the two curl terms' cell and neighbour values g and n, and in the CPML blocks the slab
// state of each term): class lookup, curl and CPML terms, the inline dispersive update of
// the FP32 E pass, and the stores.
template <typename T, bool EPASS, int CI, typename I, bool PML, bool P0, bool P1>
__device__ __forceinline__ void cellTail(const Pass<T>& p, I i, uint8_t cd, T u, const T g[2], const T n[2],
                                         const bool in[2], const T kp[2], const T bq[2], const T cq[2], const T ps[2]) {
    const Comp<T>& c = p.c[CI];
    T* __restrict__ U = c.U;
    T* __restrict__ Dd = c.D;
    T* __restrict__ psi0 = c.psi[0];
    T* __restrict__ psi1 = c.psi[1];
    if (cd == 0) return;
    if (cd >= c.ncls) {
        atomicOr(p.err, kErrClassCode);
        return;
    }
    const FastClass<T>* kc = c.fcls + cd;
    const T coef0 = kc->coef[0], coef1 = kc->coef[1];
    const uint32_t fl = kc->flags;
    if (EPASS && !kInlineDispersive<T> && (fl & (kFcLor | kFcOrDip))) return;  // run by k_pass_lorentz
    if (((fl & kFcSlab0) && !in[0]) || ((fl & kFcSlab1) && !in[1])) {
        atomicOr(p.err, kErrSlab);
        return;
    }
    T add = T(0);
    if (PML) {
        const T coef[2] = {coef0, coef1};
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            if (!(t == 0 ? P0 : P1)) continue;
            const T ct = (fl & (t == 0 ? kFcKp0 : kFcKp1)) ? coef[t] + kp[t] : coef[t];
            const T diff = g[t] - n[t];
            add += ct * diff;
            if (fl & (t == 0 ? kFcPsi0 : kFcPsi1)) {
                const T q = bq[t] * ps[t] + cq[t] * diff;
                (t == 0 ? psi0 : psi1)[i] = q;
                add += kc->psiCoef[t] * q;
            }
        }
    } else {
        if (P0) add += coef0 * (g[0] - n[0]);
        if (P1) add += coef1 * (g[1] - n[1]);
    }
    if (EPASS && kInlineDispersive<T> && (fl & (kFcLor | kFcOrDip))) {
        dispersiveCell<T>(p, CI, fl, static_cast<int>(kc->obj), kc->epsInv, i, u, add, (fl & kFcWrite) != 0);
    } else if (EPASS && (fl & kFcDtoE)) {
        // D -> E without poles: E = D / eps_inf (the P sum of cellGeneric adds zeros)
        T d = Dd[i];
        if (fl & kFcWrite) {
            d += add;
            Dd[i] = d;
        }
        U[i] = d * kc->epsInv;
    } else if (fl & kFcWrite) {
        if (fl & kFcToD) Dd[i] += add;
        else U[i] = u + add;
    }
}

// A soft source on one E cell in the persistent form: the E pass adds it to the cell's
// field before the update, as the source launch would have (E + v, then the curl).
template <typename T>
struct PSrcCell {
    int comp;
    int cell;  // device layout index
    T v;       // the source's value at the current step
};

// A field value written by another block of the same launch: loaded through L2 (the
// persistent form reads its neighbours' fields after a grid barrier).
template <bool COH, typename T>
__device__ __forceinline__ T ldField(const T* p) {
    if constexpr (COH) return __ldcg(p);
    else return *p;
}

// D2: a 2-D grid (lz == 1), where the term along z is absent. COH: neighbour fields are
// loaded through L2 (the persistent form). SRC: the E pass adds the soft sources
// ps[0 .. nps) to their cells' fields before the update.
template <typename T, bool EPASS, int CI, typename I, int CY, int PD, bool PML, bool D2 = false, bool COH = false,
          bool SRC = false>
__device__ __forceinline__ void pass3dRun(const Pass<T>& p, int x, int z, int y0, int y1, const PSrcCell<T>* ps = nullptr,
                                          int nps = 0) {
    constexpr int A0 = (CI + 2) % 3;  // derivative axis of term J
    constexpr int A1 = (CI + 1) % 3;  // derivative axis of term K
    constexpr bool P0 = !(D2 && A0 == 2);  // term J present
    constexpr bool P1 = !(D2 && A1 == 2);  // term K present
    constexpr int TY = (A0 == 1) ? 0 : ((A1 == 1) ? 1 : -1);  // term along y, or none
    const Comp<T>& c = p.c[CI];
    const I plane = static_cast<I>(p.pitch) * p.lz;
    I i = x + static_cast<I>(p.pitch) * (z + static_cast<I>(p.lz) * y0);
    const T* __restrict__ G0 = c.G[0];
    const T* __restrict__ G1 = c.G[1];
    // every array of the pass is its own allocation: no access aliases another
    T* __restrict__ U = c.U;
    T* __restrict__ Dd = c.D;
    const uint8_t* __restrict__ code = c.code;
    T* __restrict__ psi0 = c.psi[0];
    T* __restrict__ psi1 = c.psi[1];
    const I off0 = static_cast<I>(c.off[0]);
    const I off1 = static_cast<I>(c.off[1]);
    // CPML profile of the terms along x or z at this thread's coordinate
    bool inC[2] = {false, false};
    T kpC[2] = {T(0), T(0)}, bqC[2] = {T(0), T(0)}, cqC[2] = {T(0), T(0)};
    if (PML) {
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const int ax = t == 0 ? A0 : A1;
            if (ax == 1 || (D2 && ax == 2)) continue;
            const int a = ax == 0 ? x : z;
            inC[t] = a < c.slabLo[t] || a >= c.slabHi[t];
            if (inC[t]) {
                kpC[t] = c.kprof[t][a];
                if (c.hasPsi[t]) {
                    bqC[t] = c.b[t][a];
                    cqC[t] = c.cpsi[t][a];
                }
            }
        }
    }
    // field of the y term carried between planes: H holds G(y), E holds G(y-1)
    T carry = T(0);
    if constexpr (TY >= 0) carry = EPASS ? ldField<COH>(c.G[TY] + (i - plane)) : ldField<COH>(c.G[TY] + i);

#pragma unroll kMarchUnroll
    for (int y = y0; y < y1; ++y, i += plane) {
        if (PD > 0 && y + PD < y1) {
            const I ip = i + PD * plane;
            prefetchL2(code + ip);
            prefetchL2(U + ip);
            if (P0) prefetchL2(G0 + ip);
            if (P1) prefetchL2(G1 + ip);
        }
        const uint8_t cd = code[i];
        T u = U[i];
        if constexpr (SRC && EPASS) {
            for (int k = 0; k < nps; ++k)
                if (ps[k].comp == CI && ps[k].cell == static_cast<int>(i)) u += ps[k].v;
        }
        T g[2] = {T(0), T(0)}, n[2] = {T(0), T(0)};
        if (TY == 0) {
            if (EPASS) {
                g[0] = ldField<COH>(G0 + i);
                n[0] = carry;
                carry = g[0];
            } else {
                g[0] = carry;
                n[0] = ldField<COH>(G0 + (i + plane));
                carry = n[0];
            }
        } else if (P0) {
            g[0] = ldField<COH>(G0 + i);
            n[0] = ldField<COH>(G0 + (i + off0));
        }
        if (TY == 1) {
            if (EPASS) {
                g[1] = ldField<COH>(G1 + i);
                n[1] = carry;
                carry = g[1];
            } else {
                g[1] = carry;
                n[1] = ldField<COH>(G1 + (i + plane));
                carry = n[1];
            }
        } else if (P1) {
            g[1] = ldField<COH>(G1 + i);
            n[1] = ldField<COH>(G1 + (i + off1));
        }
        bool in[2] = {inC[0], inC[1]};
        T kp[2] = {kpC[0], kpC[1]}, bq[2] = {bqC[0], bqC[1]}, cq[2] = {cqC[0], cqC[1]};
        T ps[2] = {T(0), T(0)};
        if (PML) {
            if constexpr (TY >= 0) {
                in[TY] = y < c.slabLo[TY] || y >= c.slabHi[TY];
                kp[TY] = bq[TY] = cq[TY] = T(0);
                if (in[TY]) {
                    kp[TY] = c.kprof[TY][y];
                    if (c.hasPsi[TY]) {
                        bq[TY] = c.b[TY][y];
                        cq[TY] = c.cpsi[TY][y];
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < 2; ++t)
                if ((t == 0 ? P0 : P1) && c.hasPsi[t] && in[t]) ps[t] = (t == 0 ? psi0 : psi1)[i];
        }
        cellTail<T, EPASS, CI, I, PML, P0, P1>(p, i, cd, u, g, n, in, kp, bq, cq, ps);
    }
}

// Whether the block's tile or planes reach into the CPML slab of a term of component c.
template <typename T>
__device__ __forceinline__ bool blockTouchesSlab(const Comp<T>& c, int ci, int xa, int xb, int ya, int yb, int za, int zb) {
    const int axes[2] = {(ci + 2) % 3, (ci + 1) % 3};
    bool touch = false;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int lo = axes[t] == 0 ? xa : (axes[t] == 1 ? ya : za);
        const int hi = axes[t] == 0 ? xb : (axes[t] == 1 ? yb : zb);
        if (lo < c.slabLo[t] || hi >= c.slabHi[t]) touch = true;
    }
    return touch;
}

template <typename T, bool EPASS, int CI, typename I, int CY, int PD>
__device__ __forceinline__ void pass3d(const Pass<T>& p) {
    const int x = 1 + blockIdx.x * 32 + threadIdx.x;
    const int z = 1 + blockIdx.y * kP3BZ + threadIdx.y;
    const int y0 = 1 + (blockIdx.z / 3) * CY;
    const int y1 = min(y0 + CY, p.ly - 1);
    const int xa = 1 + blockIdx.x * 32, za = 1 + blockIdx.y * kP3BZ;
    const bool pml = blockTouchesSlab(p.c[CI], CI, xa, min(xa + 31, p.lx - 2), y0, y1 - 1, za,
                                      min(za + kP3BZ - 1, p.lz - 2));
    if (x > p.lx - 2 || z > p.lz - 2 || y0 > p.ly - 2) return;
    if (pml) pass3dRun<T, EPASS, CI, I, CY, PD, true>(p, x, z, y0, y1);
    else pass3dRun<T, EPASS, CI, I, CY, PD, false>(p, x, z, y0, y1);
}

// Resident blocks per SM the register budget is sized for: full occupancy (32 registers)
// for the FP32 forms with 32-bit indices.
#ifndef CHIML_E_MINB
#define CHIML_E_MINB 8
#endif
template <typename T, bool EPASS, typename I>
constexpr int passMinBlocks() {
    return sizeof(T) == 4 ? (sizeof(I) == 4 ? (EPASS ? CHIML_E_MINB : 8) : 6) : 4;
}

template <typename T, bool EPASS, typename I, int CY, int PD>
__global__ void __launch_bounds__(256, passMinBlocks<T, EPASS, I>()) k_pass3d(const Pass<T> p) {
    waitPriorGrid();
    const int ci = blockIdx.z % 3;
    if (ci == 0) pass3d<T, EPASS, 0, I, CY, PD>(p);
    else if (ci == 1) pass3d<T, EPASS, 1, I, CY, PD>(p);
    else pass3d<T, EPASS, 2, I, CY, PD>(p);
}

template <typename T, typename I, int CY, int PD>
static void launch_pass3d(const Pass<T>& p, bool ePass, cudaStream_t s) {
    dim3 block(32, kP3BZ, 1);
    dim3 grid((p.lx - 2 + 31) / 32, (p.lz - 2 + kP3BZ - 1) / kP3BZ, 3 * ((p.ly - 2 + CY - 1) / CY));
    if (ePass) launchAfterPrior(k_pass3d<T, true, I, CY, PD>, grid, block, s, p);
    else launchAfterPrior(k_pass3d<T, false, I, CY, PD>, grid, block, s, p);
}

// 2-D form (lz == 1): a block of 32 x-columns by 8 warps; warp w of y-block by marches
// CY rows along y from row 1 + (8 by + w) CY. The CPML decision is per warp.
constexpr int kP2W = 8;
#ifndef CHIML_P2CY
#define CHIML_P2CY kP2CYDefault
#endif

template <typename T, bool EPASS, int CI, int CY, int PD, bool SRC = false>
__device__ __forceinline__ void pass2d(const Pass<T>& p, int bx, int by, const PSrcCell<T>* ps = nullptr, int nps = 0) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int xa = 1 + bx * 32;
    const int x = xa + lane;
    const int y0 = 1 + (by * kP2W + w) * CY;
    if (y0 > p.ly - 2) return;
    const int y1 = min(y0 + CY, p.ly - 1);
    const bool pml = blockTouchesSlab(p.c[CI], CI, xa, min(xa + 31, p.lx - 2), y0, y1 - 1, 0, 0);
    if (x > p.lx - 2) return;
    if (pml) pass3dRun<T, EPASS, CI, int, CY, PD, true, true, false, SRC>(p, x, 0, y0, y1, ps, nps);
    else pass3dRun<T, EPASS, CI, int, CY, PD, false, true, false, SRC>(p, x, 0, y0, y1, ps, nps);
}

template <typename T, bool EPASS, int CY, bool SRC = false>
__device__ __forceinline__ void pass2dAny(const Pass<T>& p, int ci, int bx, int by, const PSrcCell<T>* ps = nullptr,
                                          int nps = 0) {
    if (ci == 0) pass2d<T, EPASS, 0, CY, 2, SRC>(p, bx, by, ps, nps);
    else if (ci == 1) pass2d<T, EPASS, 1, CY, 2, SRC>(p, bx, by, ps, nps);
    else pass2d<T, EPASS, 2, CY, 2, SRC>(p, bx, by, ps, nps);
}

constexpr int kP2CY = CHIML_P2CY;

// pass2d with the march depth cy chosen at run time (the packed form).
template <typename T, bool EPASS, int CI>
__device__ __forceinline__ void pass2dRt(const Pass<T>& p, int bx, int by, int cy) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int xa = 1 + bx * 32;
    const int x = xa + lane;
    const int y0 = 1 + (by * kP2W + w) * cy;
    if (y0 > p.ly - 2) return;
    const int y1 = min(y0 + cy, p.ly - 1);
    const bool pml = blockTouchesSlab(p.c[CI], CI, xa, min(xa + 31, p.lx - 2), y0, y1 - 1, 0, 0);
    if (x > p.lx - 2) return;
    if (pml) pass3dRun<T, EPASS, CI, int, kP2CY, 2, true, true>(p, x, 0, y0, y1);
    else pass3dRun<T, EPASS, CI, int, kP2CY, 2, false, true>(p, x, 0, y0, y1);
}

// A grid this small (cells) marches kP2CYSmall rows per warp instead of kP2CY: a march is
// a chain of dependent row loads, and a small grid has too few warps to hide it.
constexpr int kP2CYSmall = 2;
constexpr long long kP2SmallCells = 1LL << 22;

template <typename T, bool EPASS, int CY = kP2CY>
__global__ void __launch_bounds__(256) k_pass2d(const Pass<T> p) {
    waitPriorGrid();
    if (!p.c[blockIdx.z].present) return;
    pass2dAny<T, EPASS, CY>(p, blockIdx.z, blockIdx.x, blockIdx.y);
}

// The 2-D E pass with its soft sources (Pass::nSrcIn entries): each block reads the
// sources' values at the current step, and the cell of each source adds its value to the
// field before the update, which is the order of the source launch it replaces (E + v,
// then the curl terms).
template <typename T, int CY>
__global__ void __launch_bounds__(256) k_pass2d_src(const Pass<T> p) {
    waitPriorGrid();
    if (!p.c[blockIdx.z].present) return;
    __shared__ PSrcCell<T> ps[kInlineMaxSrc];
    const int nps = p.nSrcIn < kInlineMaxSrc ? p.nSrcIn : kInlineMaxSrc;
    const int st = *p.step;
    for (int j = threadIdx.x; j < nps; j += blockDim.x)
        ps[j] = PSrcCell<T>{p.srcComp[j], static_cast<int>(p.srcCell[j]),
                            static_cast<T>(st < p.srcSteps ? p.srcValue[static_cast<long long>(p.srcId[j]) * p.srcSteps + st] : 0.0)};
    __syncthreads();
    pass2dAny<T, true, CY, true>(p, blockIdx.z, blockIdx.x, blockIdx.y, ps, nps);
}

__host__ __device__ inline int pass2d_gx(int lx) { return (lx - 2 + 31) / 32; }
__host__ __device__ inline int pass2d_gy(int ly, int cy = kP2CY) { return (ly - 2 + kP2W * cy - 1) / (kP2W * cy); }

template <typename T>
void launch_pass(const Pass<T>& p, bool ePass, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (ePass && p.od.n > 0)
        launchAfterPrior(k_ordip_pol<T>, dim3(static_cast<unsigned>((p.od.n + 255) / 256)), dim3(256), s, p);
    if (p.interior3d) {
        if (p.index64) launch_pass3d<T, long long, kP3CY, kP3PD>(p, ePass, s);
        else launch_pass3d<T, int, kP3CY, kP3PD>(p, ePass, s);
        if (ePass && p.nLor > 0 && !kInlineDispersive<T>)
            launchAfterPrior(k_pass_lorentz<T>, dim3(static_cast<unsigned>((p.nLor + 255) / 256)), dim3(256), s, p);
    } else if (p.interior2d) {
        const bool src = ePass && p.nSrcIn > 0;
        if (static_cast<long long>(p.lx) * p.ly < kP2SmallCells) {
            dim3 grid(pass2d_gx(p.lx), pass2d_gy(p.ly, kP2CYSmall), 3);
            if (src) launchAfterPrior(k_pass2d_src<T, kP2CYSmall>, grid, dim3(256), s, p);
            else if (ePass) launchAfterPrior(k_pass2d<T, true, kP2CYSmall>, grid, dim3(256), s, p);
            else launchAfterPrior(k_pass2d<T, false, kP2CYSmall>, grid, dim3(256), s, p);
        } else {
            dim3 grid(pass2d_gx(p.lx), pass2d_gy(p.ly), 3);
            if (src) launchAfterPrior(k_pass2d_src<T, kP2CY>, grid, dim3(256), s, p);
            else if (ePass) launchAfterPrior(k_pass2d<T, true, kP2CY>, grid, dim3(256), s, p);
            else launchAfterPrior(k_pass2d<T, false, kP2CY>, grid, dim3(256), s, p);
        }
        if (ePass && p.nLor > 0 && !kInlineDispersive<T>)
            launchAfterPrior(k_pass_lorentz<T>, dim3(static_cast<unsigned>((p.nLor + 255) / 256)), dim3(256), s, p);
    } else {
        // 2-D grids, and 3-D grids with updated halo cells: one thread per cell,
        // all components of the pass
        dim3 block(32, 1, kGenBY);
        dim3 grid((p.lx + 31) / 32, p.lz, (p.ly + kGenBY - 1) / kGenBY);
        if (ePass) launchAfterPrior(k_pass<T, true>, grid, block, s, p);
        else launchAfterPrior(k_pass<T, false>, grid, block, s, p);
    }
}

// f.f[c] for a component c known only at run time, as a chain of selects over the
// parameter array: a dynamic index into a kernel parameter array would copy the whole
// array to local memory in every thread.
template <typename T>
__device__ __forceinline__ T* fieldOf(const Fields<T>& f, int c) {
    T* r = f.f[0];
#pragma unroll
    for (int k = 1; k < 9; ++k)
        if (c == k) r = f.f[k];
    return r;
}

template <typename T>
__device__ __forceinline__ void sourceEntry(const SourceTable& s, const Fields<T>& f, const int* step, int j) {
    if (j >= s.n) return;
    const int st = *step;
    if (st >= s.nSteps) return;
    const double v = s.value[static_cast<long long>(s.src[j]) * s.nSteps + st];
    atomicAdd(&fieldOf(f, s.comp[j])[s.cell[j]], static_cast<T>(v));
}

template <typename T>
__global__ void k_sources(const SourceTable s, const Fields<T> f, const int* __restrict__ step) {
    waitPriorGrid();
    sourceEntry(s, f, step, blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T>
void launch_sources(const SourceTable& s, const Fields<T>& f, const int* step, void* stream) {
    if (s.n == 0) return;
    launchAfterPrior(k_sources<T>, dim3((s.n + 127) / 128), dim3(128), static_cast<cudaStream_t>(stream), s, f, step);
}

template <typename T>
__device__ __forceinline__ void recordEntry(const RecordTable& r, const Fields<T>& f, const int* step, int j) {
    if (j >= r.n) return;
    const int d = r.det[j];
    const int st = *step;
    const int ti = r.timeInt[d];
    if (st % ti != 0) return;
    const int ev = st / ti;
    if (ev >= r.nEvents[d]) return;
    const long long c = r.cell[j];
    const double v = (c < 0) ? 0.0 : static_cast<double>(fieldOf(f, r.comp[j])[c]);
    r.rec[r.recBase[d] + static_cast<long long>(ev) * r.nvals[d] + r.outIndex[j]] = v;
    if (!isfinite(v)) atomicOr(r.err, kErrNumeric);
}

template <typename T>
__global__ void k_record(const RecordTable r, const Fields<T> f, const int* __restrict__ step) {
    recordEntry(r, f, step, blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T>
void launch_record(const RecordTable& r, const Fields<T>& f, const int* step, void* stream) {
    if (r.n == 0) return;
    k_record<T><<<(r.n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(r, f, step);
}

template <typename T>
__device__ __forceinline__ void dftSampleEntry(const DftTable<T>& d, const Fields<T>& f, const int* step, long long p) {
    const int st = *step;
    if (st % d.timeInt != 0 || p >= d.npts) return;
    const int slot = (st / d.timeInt) & (d.K - 1);
    const T v = fieldOf(f, d.comp[p])[d.cell[p]];
    d.ring[static_cast<long long>(slot) * d.stride + p] = v;
    if (!isfinite(v)) atomicOr(d.err, kErrNumeric);
}

template <typename T>
__global__ void __launch_bounds__(256) k_dft_sample(const DftTable<T> d, const Fields<T> f, const int* __restrict__ step) {
    dftSampleEntry(d, f, step, blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x);
}

template <typename T>
void launch_dft_sample(const DftTable<T>& d, const Fields<T>& f, const int* step, void* stream) {
    if (d.npts == 0) return;
    k_dft_sample<T><<<static_cast<unsigned>((d.npts + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(d, f, step);
}

// Fold of the ring into the accumulators: a block takes a tile of kFoldTP
// points by kFoldTF frequencies; each thread keeps a 4-point by 4-frequency
// register tile of FP-T partial sums (re and im) over all samples of the fold
// and adds them to the FP64 accumulators once at the end. Samples and phasor
// rows are staged kFoldKS samples at a time into two shared-memory buffers by
// 16-byte cp.async copies, so the next stage loads while this one computes.
// Per staged sample a thread does 32 FMAs for three 16-byte shared loads.
constexpr int kFoldTP = 128;  // points per tile (32 threads x 4)
constexpr int kFoldTF = 32;   // frequencies per tile (8 threads x 4)

template <typename T>
struct FoldCfg {
    static constexpr int KS = sizeof(T) == 4 ? 32 : 16;  // samples per stage: 2 stages fit 48 KB
};

__device__ __forceinline__ void cpAsync16(void* dst, const void* src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__device__ __forceinline__ void lds4(const float* p, float v[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
}
__device__ __forceinline__ void lds4(const double* p, double v[4]) {
    const double2 a = *reinterpret_cast<const double2*>(p);
    const double2 b = *reinterpret_cast<const double2*>(p + 2);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
}

// (hi, lo) + v with FP32 TwoSum arithmetic, renormalised: Dekker's double-length sum.
__device__ __forceinline__ void ffAdd(float& hi, float& lo, float v) {
    const float s = hi + v;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (v - bb);
    const float l2 = lo + err;
    const float h = s + l2;
    lo = l2 - (h - s);
    hi = h;
}

// Staggered folds. The point tiles of a table are split into G = K / kFoldStagger
// groups (point tile q belongs to group q mod G), and every kFoldStagger-th sample one
// group folds: group g folds at the samples n with n + 1 = (g + 1 + m G) kFoldStagger,
// each time taking the samples since its previous fold (K of them, or n + 1 at its
// first fold). Every sample is folded by every group within K samples of being
// written, so the ring of K slots suffices, and each step carries 1 / kFoldStagger of
// a group fold: the fold work is spread evenly over the steps instead of arriving as
// one launch every K samples.
// (kFoldStagger: fdtd_device.hpp, shared with the host, which launches a table's fold
// kernel only at the steps where one of its groups folds)

// The sample range one group still has to fold after sample `last` (the flush at the
// end of a run): first sample and count (count 0 when nothing is pending).
__device__ __forceinline__ void foldPending(int K, int group, int last, int& first, int& count) {
    const int n0 = group * kFoldStagger + kFoldStagger - 1;  // the group's first fold
    int folded = -1;  // last sample the group has folded
    if (last >= n0) folded = n0 + ((last - n0) / K) * K;
    first = folded + 1;
    count = last - folded;
}

// One tile (kFoldTP points from p0, kFoldTF frequencies from f0) over `count` samples
// from sample `first` (all threads of the block).
template <typename T>
__device__ __forceinline__ void foldTile(const DftTable<T>& d, long long p0, int f0, int first, int count) {
    constexpr int KS = FoldCfg<T>::KS;
    constexpr int EV = 16 / sizeof(T);  // values per 16-byte copy
    __shared__ __align__(16) T smp[2][KS][kFoldTP];
    __shared__ __align__(16) T ph[2][KS][kFoldTF * 2];  // per sample: kFoldTF cos, then kFoldTF -sin
    const int nf = d.nfreq;
    const int tf = threadIdx.x & 7;   // frequencies 4*tf .. 4*tf+3 of the tile
    const int tp = threadIdx.x >> 3;  // points 4*tp .. 4*tp+3 of the tile
    const int stages = (count + KS - 1) / KS;
    // copies of stage s into buffer s & 1 (the ring pitch and the phasor rows are 16-byte multiples)
    auto issue = [&](int sg) {
        const int b = sg & 1;
        const int k0 = sg * KS;
        const int kn = min(KS, count - k0);
        for (int q = threadIdx.x; q < KS * (kFoldTP / EV); q += blockDim.x) {
            const int k = q / (kFoldTP / EV), c = q % (kFoldTP / EV);
            if (k < kn) {
                const int slot = (first + k0 + k) & (d.K - 1);
                cpAsync16(&smp[b][k][c * EV], d.ring + static_cast<long long>(slot) * d.stride + p0 + c * EV);
            }
        }
        for (int q = threadIdx.x; q < KS * (kFoldTF * 2 / EV); q += blockDim.x) {
            const int k = q / (kFoldTF * 2 / EV), c = q % (kFoldTF * 2 / EV);
            const int plane = c / (kFoldTF / EV), cc = c % (kFoldTF / EV);
            if (k < kn)
                cpAsync16(&ph[b][k][plane * kFoldTF + cc * EV],
                          d.phasor + (static_cast<long long>(first + k0 + k) * 2 + plane) * d.nfreqPad + f0 + cc * EV);
        }
        cpAsyncCommit();
    };
    T are[4][4], aim[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int m = 0; m < 4; ++m) are[j][m] = aim[j][m] = T(0);
    __syncthreads();  // the previous tile's last stage is no longer read
    issue(0);
    for (int sg = 0; sg < stages; ++sg) {
        if (sg + 1 < stages) issue(sg + 1);
        else cpAsyncCommit();
        cpAsyncWait1();
        __syncthreads();
        const int b = sg & 1;
        const int kn = min(KS, count - sg * KS);
        for (int k = 0; k < kn; ++k) {
            // the eight threads of a point group read consecutive 16-byte chunks of each
            // phasor plane: no bank conflicts
            T v[4], c[4], sn[4];
            lds4(&smp[b][k][4 * tp], v);
            lds4(&ph[b][k][4 * tf], c);             // cos of frequencies 4 tf .. 4 tf + 3
            lds4(&ph[b][k][kFoldTF + 4 * tf], sn);  // -sin
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    are[j][m] += c[m] * v[j];
                    aim[j][m] += sn[m] * v[j];
                }
        }
        __syncthreads();  // buffer b is free for stage sg + 2
    }
    cpAsyncWait0();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const long long p = p0 + 4 * tp + j;
        if (p >= d.npts) continue;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int f = f0 + 4 * tf + m;
            if (f >= nf) continue;
            if constexpr (kFloatFloatAcc<T>) {
                float2* r = reinterpret_cast<float2*>(d.re) + p * nf + f;
                float2* q = reinterpret_cast<float2*>(d.im) + p * nf + f;
                float2 a = *r, b = *q;
                ffAdd(a.x, a.y, static_cast<float>(are[j][m]));
                ffAdd(b.x, b.y, static_cast<float>(aim[j][m]));
                *r = a;
                *q = b;
            } else {
                d.re[p * nf + f] += static_cast<double>(are[j][m]);
                d.im[p * nf + f] += static_cast<double>(aim[j][m]);
            }
        }
    }
}

// The group that folds after the sample of the current step, with its first sample and
// count; false when no group folds at this step.
template <typename T>
__device__ __forceinline__ bool foldGroupNow(const DftTable<T>& d, const int* step, int& group, int& first, int& count) {
    const int st = *step;
    if (st % d.timeInt != 0) return false;
    const int n = st / d.timeInt;
    if ((n + 1) % kFoldStagger != 0) return false;
    group = ((n + 1) / kFoldStagger - 1) % (d.K / kFoldStagger);
    count = min(d.K, n + 1);
    first = n + 1 - count;
    return true;
}

// Step fold: the tiles of the group that folds now, tileBegin, tileBegin + tileStride, ...
// counted within the group.
template <typename T>
__device__ __forceinline__ void foldStep(const DftTable<T>& d, const int* step, long long tileBegin, long long tileStride) {
    int g, first, count;
    if (!foldGroupNow(d, step, g, first, count)) return;
    const int G = d.K / kFoldStagger;
    const int fTiles = (d.nfreq + kFoldTF - 1) / kFoldTF;
    const long long pTiles = (d.npts + kFoldTP - 1) / kFoldTP;
    if (g >= pTiles) return;
    const long long tiles = ((pTiles - g + G - 1) / G) * fTiles;  // point tiles g, g + G, ... of the group
    for (long long j = tileBegin; j < tiles; j += tileStride) {
        const long long q = g + static_cast<long long>(G) * (j / fTiles);
        foldTile(d, q * kFoldTP, static_cast<int>(j % fTiles) * kFoldTF, first, count);
    }
}

// Flush at the end of a run: every tile folds what its group has pending after sample
// `last`; tiles tileBegin, tileBegin + tileStride, ... of the whole table.
template <typename T>
__device__ __forceinline__ void foldFlush(const DftTable<T>& d, int last, long long tileBegin, long long tileStride) {
    const int G = d.K / kFoldStagger;
    const int fTiles = (d.nfreq + kFoldTF - 1) / kFoldTF;
    const long long tiles = ((d.npts + kFoldTP - 1) / kFoldTP) * fTiles;
    for (long long t = tileBegin; t < tiles; t += tileStride) {
        const long long q = t / fTiles;
        int first, count;
        foldPending(d.K, static_cast<int>(q % G), last, first, count);
        if (count > 0) foldTile(d, q * kFoldTP, static_cast<int>(t % fTiles) * kFoldTF, first, count);
    }
}

// Resident blocks per SM the fold's register budget is sized for: the FP32 tile fits 63
// registers without spilling, so four blocks (the shared-memory limit) stay resident to
// cover the ring and accumulator loads; the FP64 form keeps its registers.
template <typename T>
constexpr int foldMinBlocks() {
    return sizeof(T) == 4 ? 4 : 1;
}

template <typename T>
__global__ void __launch_bounds__(256, foldMinBlocks<T>()) k_dft_fold(const DftTable<T> d, const int* __restrict__ step) {
    waitPriorGrid();
    foldStep(d, step, blockIdx.x, gridDim.x);
}

template <typename T>
__global__ void __launch_bounds__(256, foldMinBlocks<T>()) k_dft_flush(const DftTable<T> d, int last) {
    foldFlush(d, last, blockIdx.x, gridDim.x);
}

template <typename T>
void launch_dft_fold(const DftTable<T>& d, const int* step, void* stream) {
    if (d.npts == 0) return;
    const long long pTiles = (d.npts + kFoldTP - 1) / kFoldTP;
    const long long G = d.K / kFoldStagger;
    const long long tiles = ((pTiles + G - 1) / G) * ((d.nfreq + kFoldTF - 1) / kFoldTF);
    const unsigned grid = static_cast<unsigned>(tiles < 152 * 4 ? tiles : 152 * 4);
    launchAfterPrior(k_dft_fold<T>, dim3(grid), dim3(256), static_cast<cudaStream_t>(stream), d, step);
}

template <typename T>
void launch_dft_flush(const DftTable<T>& d, int samples, void* stream) {
    if (d.npts == 0 || samples <= 0) return;
    const long long tiles = ((d.npts + kFoldTP - 1) / kFoldTP) * ((d.nfreq + kFoldTF - 1) / kFoldTF);
    const unsigned grid = static_cast<unsigned>(tiles < 152 * 4 ? tiles : 152 * 4);
    k_dft_flush<T><<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(d, samples - 1);
}

__global__ void k_increment(int* step) { *step += 1; }

template <typename T>
__global__ void __launch_bounds__(256) k_step_tail(const StepTail<T> t) {
    waitPriorGrid();
    __shared__ int next;  // the step number after this step's increment
    if (threadIdx.x == 0) next = *t.step + 1;
    __syncthreads();
    const int b = static_cast<int>(blockIdx.x);
    if (b < t.recBlocks) {
        recordEntry(t.rec, t.f, &next, b * 256 + static_cast<int>(threadIdx.x));
    } else if (t.nDft > 0) {
        const int sb = b - t.recBlocks;
        int q = 0;
        while (q + 1 < t.nDft && t.dftStart[q + 1] <= sb) ++q;
        dftSampleEntry(t.dft[q], t.f, &next, (sb - t.dftStart[q]) * 256LL + threadIdx.x);
    }
    // every block has read the counter before it takes its ticket; the last one advances it
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(t.ticket, 1u) == gridDim.x - 1) {
            *t.step = next;
            *t.ticket = 0u;
            __threadfence();
        }
    }
}

void launch_increment(int* step, void* stream) { k_increment<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(step); }

template <typename T>
void launch_step_tail(const StepTail<T>& t, void* stream) {
    launchAfterPrior(k_step_tail<T>, dim3(static_cast<unsigned>(t.blocks)), dim3(256), static_cast<cudaStream_t>(stream), t);
}

// ---- persistent form of small 2-D grids ----

__device__ __forceinline__ unsigned long long globalTimerNs() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned int loadAcquire(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier of a cooperative launch: every block adds one arrival to the counter and
// waits until it reaches `target` (the arrivals of all barriers so far). The wait is
// bounded: after limitNs, or once another block has given up, it sets kErrTimeout and
// returns false, and the caller ends the launch. The fences before the arrival and after
// the wait order every block's field writes before the other blocks' reads.
__device__ bool gridBarrier(unsigned int* bar, unsigned int target, unsigned int* err, unsigned long long limitNs) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        __threadfence();
        atomicAdd(bar, 1u);
        const unsigned long long t0 = globalTimerNs();
        while (loadAcquire(bar) < target) {
            if (loadAcquire(err) & kErrTimeout) {
                ok = 0;
                break;
            }
            if (globalTimerNs() - t0 > limitNs) {
                atomicOr(err, kErrTimeout);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Records and DFT samples of one component set (E and D, or H) at sample index `idx`, the
// launch's threads striding over the record entries and then every table's points.
template <typename T>
__device__ void persistSamples(const Persist2d<T>& a, int idx, bool wantH) {
    const long long nThreads = static_cast<long long>(gridDim.x) * blockDim.x;
    const long long total = a.rec.n + a.dftPoints;
    for (long long j = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; j < total; j += nThreads) {
        if (j < a.rec.n) {
            const RecordTable& r = a.rec;
            const int comp = r.comp[j];
            if ((comp >= 3 && comp <= 5) != wantH) continue;
            const int d = r.det[j];
            const int ti = r.timeInt[d];
            if (idx % ti != 0) continue;
            const int ev = idx / ti;
            if (ev >= r.nEvents[d]) continue;
            const long long c = r.cell[j];
            const double v = (c < 0) ? 0.0 : static_cast<double>(__ldcg(fieldOf(a.f, comp) + c));
            r.rec[r.recBase[d] + static_cast<long long>(ev) * r.nvals[d] + r.outIndex[j]] = v;
            if (!isfinite(v)) atomicOr(r.err, kErrNumeric);
        } else {
            long long pt = j - a.rec.n;
            int q = 0;
            while (q + 1 < a.nDft && pt >= a.dft[q].npts) pt -= a.dft[q++].npts;
            const DftTable<T>& d = a.dft[q];
            const int comp = d.comp[pt];
            if ((comp >= 3 && comp <= 5) != wantH) continue;
            if (idx % d.timeInt != 0) continue;
            const int slot = (idx / d.timeInt) & (d.K - 1);
            const T v = __ldcg(fieldOf(a.f, comp) + d.cell[pt]);
            d.ring[static_cast<long long>(slot) * d.stride + pt] = v;
            if (!isfinite(v)) atomicOr(d.err, kErrNumeric);
        }
    }
}

// One pass of the persistent form: the 2-D units (component, y-block, x-block) of the
// pass, unit u on block u mod gridDim.x (the same block every step, so that each cell's
// own field, psi and polarisations stay with one SM).
template <typename T, bool EPASS, int CY>
__device__ void persistPass(const Pass<T>& p, const PSrcCell<T>* ps, int nps) {
    const int gx = pass2d_gx(p.lx), gy = pass2d_gy(p.ly, CY);
    const int units = 3 * gx * gy;
    for (int u = blockIdx.x; u < units; u += gridDim.x) {
        const int ci = u / (gx * gy), r = u % (gx * gy);
        if (!p.c[ci].present) continue;
        const int bx = r % gx, by = r / gx;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int xa = 1 + bx * 32, x = xa + lane;
        const int y0 = 1 + (by * kP2W + w) * CY;
        if (y0 > p.ly - 2 || x > p.lx - 2) continue;
        const int y1 = min(y0 + CY, p.ly - 1);
        const bool pml = blockTouchesSlab(p.c[ci], ci, xa, min(xa + 31, p.lx - 2), y0, y1 - 1, 0, 0);
#define CHIML_PERSIST_RUN(CIV)                                                                           \
    if (pml) pass3dRun<T, EPASS, CIV, int, CY, 0, true, true, true, true>(p, x, 0, y0, y1, ps, nps);    \
    else pass3dRun<T, EPASS, CIV, int, CY, 0, false, true, true, true>(p, x, 0, y0, y1, ps, nps);
        if (ci == 0) {
            CHIML_PERSIST_RUN(0)
        } else if (ci == 1) {
            CHIML_PERSIST_RUN(1)
        } else {
            CHIML_PERSIST_RUN(2)
        }
#undef CHIML_PERSIST_RUN
    }
}

// nsteps whole steps from step0. Per step: the H pass, with the E-side samples of the
// previous step (E is not written in the H pass); a barrier; the E pass with the sources,
// with the H-side samples of this step (H is not written in the E pass); a barrier. The
// E-side samples of the last step close the launch, which then sets the step counter.
template <typename T, int CY>
__global__ void __launch_bounds__(256) k_persist2d(const Persist2d<T> a, int step0, int nsteps) {
    __shared__ PSrcCell<T> ps[kPersistMaxSrc];
    const int nps = a.src.n < kPersistMaxSrc ? a.src.n : kPersistMaxSrc;
    unsigned int target = 0;
    for (int k = 0; k < nsteps; ++k) {
        const int st = step0 + k;
        persistPass<T, false, CY>(a.h, ps, 0);
        if (k > 0) persistSamples(a, st, false);
        target += gridDim.x;
        if (!gridBarrier(a.bar, target, a.h.err, a.limitNs)) return;
        // the sources of this step (their values were read before the first pass of the
        // block; the list is rewritten only between the block's barriers)
        for (int j = threadIdx.x; j < nps; j += blockDim.x)
            ps[j] = PSrcCell<T>{a.src.comp[j], static_cast<int>(a.src.cell[j]),
                                static_cast<T>(st < a.src.nSteps ? a.src.value[static_cast<long long>(a.src.src[j]) * a.src.nSteps + st] : 0.0)};
        __syncthreads();
        persistPass<T, true, CY>(a.e, ps, nps);
        persistSamples(a, st + 1, true);
        target += gridDim.x;
        if (!gridBarrier(a.bar, target, a.h.err, a.limitNs)) return;
    }
    persistSamples(a, step0 + nsteps, false);
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.step = step0 + nsteps;
}

constexpr int kPersistCY = 2;  // rows per warp of a persistent pass unit

template <typename T>
int persist2d_blocks(const Pass<T>& h, const Pass<T>& e, int device) {
    int perSM = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_persist2d<T, kPersistCY>, 256, 0) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    // no more blocks than the larger pass has units
    const int units = 3 * std::max(pass2d_gx(h.lx) * pass2d_gy(h.ly, kPersistCY), pass2d_gx(e.lx) * pass2d_gy(e.ly, kPersistCY));
    return std::min(perSM * sms, units);
}

template <typename T>
int launch_persist2d(const Persist2d<T>& a, int blocks, int step0, int nsteps, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(a.bar, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return static_cast<int>(e);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(blocks));
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return static_cast<int>(cudaLaunchKernelEx(&cfg, k_persist2d<T, kPersistCY>, a, step0, nsteps));
}

__global__ void k_barrier_selftest(unsigned int* bar, unsigned int target, unsigned int* err, unsigned long long limitNs) {
    gridBarrier(bar, target, err, limitNs);
}

int launch_barrier_selftest(int blocks, int missing, unsigned long long limitNs, unsigned int* bar, unsigned int* err,
                            void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(bar, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return static_cast<int>(e);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(blocks));
    cfg.blockDim = dim3(32);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const unsigned int target = static_cast<unsigned int>(blocks + missing);
    return static_cast<int>(cudaLaunchKernelEx(&cfg, k_barrier_selftest, bar, target, err, limitNs));
}

// ---- packed launches (batched sweep) ----

template <typename T>
long long pass_blocks(const Pass<T>& p) {
    return static_cast<long long>((p.lx + 31) / 32) * p.lz * ((p.ly + kGenBY - 1) / kGenBY);
}
template <typename T>
long long pass2d_blocks_per_comp(const Pass<T>& p) {
    return static_cast<long long>(pass2d_gx(p.lx)) * pass2d_gy(p.ly, p.march > 0 ? p.march : kP2CY);
}
long long lorentz_blocks(long long n) { return (n + 255) / 256; }
long long ordip_blocks(long long n) { return (n + 255) / 256; }
int sources_blocks(int n) { return (n + 127) / 128; }
int record_blocks(int n) { return (n + 127) / 128; }
long long dft_sample_blocks(long long npts) { return (npts + 255) / 256; }
long long dft_fold_blocks(long long npts, int nfreq) {
    return ((npts + kFoldTP - 1) / kFoldTP) * ((nfreq + kFoldTF - 1) / kFoldTF);
}

// Block (bx, bz, by) of a member's generic pass grid from its linear block index.
template <typename T, bool EPASS>
__global__ void __launch_bounds__(256) k_pass_packed(const Pass<T>* __restrict__ jobs, const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    const Pass<T>& p = jobs[w.x];
    const int gx = (p.lx + 31) / 32;
    const int bx = w.y % gx;
    const int r = w.y / gx;
    const int bz = r % p.lz;
    const int by = r / p.lz;
    passCell<T, EPASS>(p, bx * 32 + (threadIdx.x & 31), by * kGenBY + (threadIdx.x >> 5), bz);
}

// 2-D form: the block index of a job encodes (component, y-block, x-block).
template <typename T, bool EPASS>
__global__ void __launch_bounds__(256, 6) k_pass2d_packed(const Pass<T>* __restrict__ jobs, const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    const Pass<T>& p = jobs[w.x];
    // each member's own march depth (the batch autotuner's choice for its grid shape)
    const int cy = p.march > 0 ? p.march : kP2CY;
    const int gx = pass2d_gx(p.lx), gy = pass2d_gy(p.ly, cy);
    const int bx = w.y % gx;
    const int r = w.y / gx;
    const int ci = r / gy, by = r % gy;
    if (ci == 0) pass2dRt<T, EPASS, 0>(p, bx, by, cy);
    else if (ci == 1) pass2dRt<T, EPASS, 1>(p, bx, by, cy);
    else pass2dRt<T, EPASS, 2>(p, bx, by, cy);
}

template <typename T>
__global__ void __launch_bounds__(256) k_lorentz_packed(const Pass<T>* __restrict__ jobs, const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    const Pass<T>& p = jobs[w.x];
    const long long j = w.y * 256LL + threadIdx.x;
    if (j >= p.nLor) return;
    const long long i = p.lorCell[j];
    const int x = static_cast<int>(i % p.pitch);
    const long long r = i / p.pitch;
    const int coord[3] = {x, static_cast<int>(r / p.lz), static_cast<int>(r % p.lz)};
    cellGeneric<T, true>(p, p.lorComp[j], i, coord);
}

template <typename T>
__global__ void __launch_bounds__(256) k_ordip_packed(const Pass<T>* __restrict__ jobs, const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    ordipEntry(jobs[w.x], w.y * 256LL + threadIdx.x);
}

template <typename T>
__global__ void __launch_bounds__(128) k_sources_packed(const SrcJob<T>* __restrict__ jobs, const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    const SrcJob<T>& j = jobs[w.x];
    sourceEntry(j.s, j.f, j.step, w.y * 128 + static_cast<int>(threadIdx.x));
}

template <typename T>
__global__ void __launch_bounds__(128) k_record_packed(const RecJob<T>* __restrict__ jobs, const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    const RecJob<T>& j = jobs[w.x];
    recordEntry(j.r, j.f, j.step, w.y * 128 + static_cast<int>(threadIdx.x));
}

template <typename T>
__global__ void __launch_bounds__(256) k_dft_sample_packed(const DftJob<T>* __restrict__ jobs, const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    const DftJob<T>& j = jobs[w.x];
    dftSampleEntry(j.d, j.f, j.step, w.y * 256LL + threadIdx.x);
}

template <typename T>
__global__ void __launch_bounds__(256, foldMinBlocks<T>()) k_dft_fold_packed(const DftJob<T>* __restrict__ jobs, const int2* __restrict__ work) {
    waitPriorGrid();
    const int2 w = work[blockIdx.x];
    const DftJob<T>& j = jobs[w.x];
    int g, first, count;
    if (!foldGroupNow(j.d, j.step, g, first, count)) return;
    const int fTiles = (j.d.nfreq + kFoldTF - 1) / kFoldTF;
    const long long q = w.y / fTiles;  // point tile of this block
    if (q % (j.d.K / kFoldStagger) != g) return;
    foldTile(j.d, q * kFoldTP, static_cast<int>(w.y % fTiles) * kFoldTF, first, count);
}

__global__ void k_increment_packed(int* const* __restrict__ steps, int n) {
    waitPriorGrid();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) *steps[j] += 1;
}

template <typename T>
void launch_pass_packed(const Pass<T>* jobs, WorkMap m, bool ePass, void* stream) {
    if (m.blocks <= 0) return;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (ePass) launchAfterPrior(k_pass_packed<T, true>, dim3(m.blocks), dim3(256), s, jobs, m.work);
    else launchAfterPrior(k_pass_packed<T, false>, dim3(m.blocks), dim3(256), s, jobs, m.work);
}
template <typename T>
void launch_pass2d_packed(const Pass<T>* jobs, WorkMap m, bool ePass, void* stream) {
    if (m.blocks <= 0) return;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (ePass) launchAfterPrior(k_pass2d_packed<T, true>, dim3(m.blocks), dim3(256), s, jobs, m.work);
    else launchAfterPrior(k_pass2d_packed<T, false>, dim3(m.blocks), dim3(256), s, jobs, m.work);
}
template <typename T>
void launch_lorentz_packed(const Pass<T>* jobs, WorkMap m, void* stream) {
    if (m.blocks > 0) launchAfterPrior(k_lorentz_packed<T>, dim3(m.blocks), dim3(256), static_cast<cudaStream_t>(stream), jobs, m.work);
}
template <typename T>
void launch_ordip_packed(const Pass<T>* jobs, WorkMap m, void* stream) {
    if (m.blocks > 0) launchAfterPrior(k_ordip_packed<T>, dim3(m.blocks), dim3(256), static_cast<cudaStream_t>(stream), jobs, m.work);
}
template <typename T>
void launch_sources_packed(const SrcJob<T>* jobs, WorkMap m, void* stream) {
    if (m.blocks > 0) launchAfterPrior(k_sources_packed<T>, dim3(m.blocks), dim3(128), static_cast<cudaStream_t>(stream), jobs, m.work);
}
template <typename T>
void launch_record_packed(const RecJob<T>* jobs, WorkMap m, void* stream) {
    if (m.blocks > 0) launchAfterPrior(k_record_packed<T>, dim3(m.blocks), dim3(128), static_cast<cudaStream_t>(stream), jobs, m.work);
}
template <typename T>
void launch_dft_sample_packed(const DftJob<T>* jobs, WorkMap m, void* stream) {
    if (m.blocks > 0) launchAfterPrior(k_dft_sample_packed<T>, dim3(m.blocks), dim3(256), static_cast<cudaStream_t>(stream), jobs, m.work);
}
template <typename T>
void launch_dft_fold_packed(const DftJob<T>* jobs, WorkMap m, void* stream) {
    if (m.blocks > 0) launchAfterPrior(k_dft_fold_packed<T>, dim3(m.blocks), dim3(256), static_cast<cudaStream_t>(stream), jobs, m.work);
}
void launch_increment_packed(int* const* steps, int n, void* stream) {
    if (n > 0) launchAfterPrior(k_increment_packed, dim3((n + 127) / 128), dim3(128), static_cast<cudaStream_t>(stream), steps, n);
}

#define CHIML_PACKED(T)                                                                   \
    template long long pass_blocks<T>(const Pass<T>&);                                    \
    template long long pass2d_blocks_per_comp<T>(const Pass<T>&);                         \
    template void launch_pass2d_packed<T>(const Pass<T>*, WorkMap, bool, void*);          \
    template void launch_lorentz_packed<T>(const Pass<T>*, WorkMap, void*);               \
    template void launch_pass_packed<T>(const Pass<T>*, WorkMap, bool, void*);            \
    template void launch_ordip_packed<T>(const Pass<T>*, WorkMap, void*);                 \
    template void launch_sources_packed<T>(const SrcJob<T>*, WorkMap, void*);             \
    template void launch_record_packed<T>(const RecJob<T>*, WorkMap, void*);              \
    template void launch_dft_sample_packed<T>(const DftJob<T>*, WorkMap, void*);          \
    template void launch_dft_fold_packed<T>(const DftJob<T>*, WorkMap, void*);
CHIML_PACKED(float)
CHIML_PACKED(double)
#undef CHIML_PACKED

template void launch_pass<double>(const Pass<double>&, bool, void*);
template void launch_pass<float>(const Pass<float>&, bool, void*);
template void launch_sources<double>(const SourceTable&, const Fields<double>&, const int*, void*);
template void launch_sources<float>(const SourceTable&, const Fields<float>&, const int*, void*);
template void launch_step_tail<double>(const StepTail<double>&, void*);
template void launch_step_tail<float>(const StepTail<float>&, void*);
template int persist2d_blocks<double>(const Pass<double>&, const Pass<double>&, int);
template int persist2d_blocks<float>(const Pass<float>&, const Pass<float>&, int);
template int launch_persist2d<double>(const Persist2d<double>&, int, int, int, void*);
template int launch_persist2d<float>(const Persist2d<float>&, int, int, int, void*);
template void launch_record<double>(const RecordTable&, const Fields<double>&, const int*, void*);
template void launch_record<float>(const RecordTable&, const Fields<float>&, const int*, void*);
template void launch_dft_sample<double>(const DftTable<double>&, const Fields<double>&, const int*, void*);
template void launch_dft_sample<float>(const DftTable<float>&, const Fields<float>&, const int*, void*);
template void launch_dft_fold<double>(const DftTable<double>&, const int*, void*);
template void launch_dft_fold<float>(const DftTable<float>&, const int*, void*);
template void launch_dft_flush<double>(const DftTable<double>&, int, void*);
template void launch_dft_flush<float>(const DftTable<float>&, int, void*);

}  // namespace dev
}  // namespace chiml
