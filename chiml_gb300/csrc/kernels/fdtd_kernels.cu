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

#include "fdtd_device.hpp"

namespace chiml {
namespace dev {

template <typename T, bool EPASS>
__global__ void __launch_bounds__(256) k_pass(const Pass<T> p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y * blockDim.y + threadIdx.y;
    const int y = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= p.lx || z >= p.lz || y >= p.ly) return;
    const long long i = x + static_cast<long long>(p.lx) * (z + static_cast<long long>(p.lz) * y);
    const int coord[3] = {x, y, z};
#pragma unroll
    for (int ci = 0; ci < 3; ++ci) {
        const Comp<T>& c = p.c[ci];
        if (!c.present) continue;
        const uint8_t code = c.code[i];
        if (code == 0) continue;
        if (code >= c.ncls) {
            atomicOr(p.err, kErrClassCode);
            continue;
        }
        const Class<T> k = c.cls[code];
        if (EPASS && k.lor) {
            if (k.obj < 0 || k.obj >= p.nObj || p.poleCount[k.obj] > c.nPoles) {
                atomicOr(p.err, kErrPoleCount);
                continue;
            }
            const T e = c.U[i];
            const int s = p.poleStart[k.obj];
            const int n = p.poleCount[k.obj];
            for (int q = 0; q < n; ++q) {
                const T old = c.P[q][i];
                T np = p.alpha[s + q] * old;
                np += p.xi[s + q] * c.Pprev[q][i];
                np += p.gamma[s + q] * e;
                c.P[q][i] = np;
                c.Pprev[q][i] = old;
            }
        }
        T add = T(0);
        bool any = false;
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            if (!c.tpresent[t]) continue;
            const int a = coord[c.axis[t]];
            const T coef = k.cint[t] + T(k.nplain[t]) * c.db[t] + (k.kflag[t] ? c.kprof[t][a] : T(0));
            const bool psiTerm = c.hasPsi[t] && (k.psiUpd[t] || k.npsi[t]);
            if (coef == T(0) && !psiTerm) continue;
            const T diff = c.G[t][i] - c.G[t][i + c.off[t]];
            if (coef != T(0)) {
                add += coef * diff;
                any = true;
            }
            if (c.hasPsi[t]) {
                if (k.psiUpd[t]) {
                    T ps = c.psi[t][i];
                    ps = c.b[t][a] * ps + c.cpsi[t][a] * diff;
                    c.psi[t][i] = ps;
                    if (k.npsi[t]) {
                        add += T(k.npsi[t]) * c.dbpsi[t] * ps;
                        any = true;
                    }
                } else if (k.npsi[t]) {
                    add += T(k.npsi[t]) * c.dbpsi[t] * c.psi[t][i];
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
    }
}

// 3-D form of the same update for grids whose halo cells carry no update.
// A block covers a 32 (x) by kP3BZ (z) tile of interior cells of one
// component and walks kP3CY planes along y, the slowest axis of the layout.
// The component (and with it the two derivative axes) is a template
// parameter. Every load a cell needs in the common case (class code, the
// field, both neighbour pairs, psi inside the slab) is issued before the class
// is known, so a warp keeps several independent loads in flight; the class
// only selects the arithmetic. The neighbour along y is carried in a register
// from the previous plane. Per cell the arithmetic is the same as k_pass.
constexpr int kP3BZ = 8;
constexpr int kP3CY = 16;

template <typename T, bool EPASS, int CI, typename I>
__device__ __forceinline__ void pass3d(const Pass<T>& p, const Class<T>* __restrict__ tab) {
    constexpr int A0 = (CI + 2) % 3;  // derivative axis of term J
    constexpr int A1 = (CI + 1) % 3;  // derivative axis of term K
    constexpr int TY = (A0 == 1) ? 0 : ((A1 == 1) ? 1 : -1);  // term along y, or none
    constexpr bool UP = !EPASS;       // H: neighbour at +1 ; E: neighbour at -1
    const Comp<T>& c = p.c[CI];
    const int x = 1 + blockIdx.x * 32 + threadIdx.x;
    const int z = 1 + blockIdx.y * kP3BZ + threadIdx.y;
    const int y0 = 1 + (blockIdx.z / 3) * kP3CY;
    if (x > p.lx - 2 || z > p.lz - 2 || y0 > p.ly - 2) return;
    const int y1 = min(y0 + kP3CY, p.ly - 1);
    const I plane = static_cast<I>(p.lx) * p.lz;
    I i = x + static_cast<I>(p.lx) * (z + static_cast<I>(p.lz) * y0);

    const uint8_t* __restrict__ code = c.code;
    T* __restrict__ U = c.U;
    const T* __restrict__ G[2] = {c.G[0], c.G[1]};
    const I off[2] = {static_cast<I>(c.off[0]), static_cast<I>(c.off[1])};
    // profile values of the terms along x or z are fixed for the thread
    bool in[2] = {false, false};
    T kp[2] = {T(0), T(0)}, bq[2] = {T(0), T(0)}, cq[2] = {T(0), T(0)};
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int ax = t == 0 ? A0 : A1;
        if (ax == 1) continue;
        const int a = ax == 0 ? x : z;
        in[t] = a < c.slabLo[t] || a >= c.slabHi[t];
        if (in[t]) {
            kp[t] = c.kprof[t][a];
            if (c.hasPsi[t]) {
                bq[t] = c.b[t][a];
                cq[t] = c.cpsi[t][a];
            }
        }
    }
    T carry = T(0);
    if constexpr (TY >= 0) carry = UP ? G[TY][i] : G[TY][i - plane];

    for (int y = y0; y < y1; ++y, i += plane) {
        const uint8_t cd = code[i];
        const T u = U[i];
        T g[2], n[2];
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            if (t == TY) {
                if (UP) {
                    g[t] = carry;
                    n[t] = G[t][i + plane];
                    carry = n[t];
                } else {
                    g[t] = G[t][i];
                    n[t] = carry;
                    carry = g[t];
                }
            } else {
                g[t] = G[t][i];
                n[t] = G[t][i + off[t]];
            }
        }
        if constexpr (TY >= 0) {
            in[TY] = y < c.slabLo[TY] || y >= c.slabHi[TY];
            kp[TY] = T(0);
            if (in[TY]) {
                kp[TY] = c.kprof[TY][y];
                if (c.hasPsi[TY]) {
                    bq[TY] = c.b[TY][y];
                    cq[TY] = c.cpsi[TY][y];
                }
            }
        }
        T ps[2] = {T(0), T(0)};
#pragma unroll
        for (int t = 0; t < 2; ++t)
            if (c.hasPsi[t] && in[t]) ps[t] = c.psi[t][i];

        if (cd == 0) continue;
        if (cd >= c.ncls) {
            atomicOr(p.err, kErrClassCode);
            continue;
        }
        const Class<T>& k = tab[cd];
        if (EPASS && k.lor) {
            if (k.obj < 0 || k.obj >= p.nObj || p.poleCount[k.obj] > c.nPoles) {
                atomicOr(p.err, kErrPoleCount);
                continue;
            }
            const int s = p.poleStart[k.obj];
            const int np = p.poleCount[k.obj];
            for (int q = 0; q < np; ++q) {
                const T old = c.P[q][i];
                T v = p.alpha[s + q] * old;
                v += p.xi[s + q] * c.Pprev[q][i];
                v += p.gamma[s + q] * u;
                c.P[q][i] = v;
                c.Pprev[q][i] = old;
            }
        }
        T add = T(0);
        bool any = false;
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            if (!in[t] && (k.kflag[t] | k.psiUpd[t] | k.npsi[t])) {
                atomicOr(p.err, kErrSlab);
                continue;
            }
            const T coef = k.cint[t] + T(k.nplain[t]) * c.db[t] + (k.kflag[t] ? kp[t] : T(0));
            const T diff = g[t] - n[t];
            if (coef != T(0)) {
                add += coef * diff;
                any = true;
            }
            if (c.hasPsi[t] && in[t]) {
                if (k.psiUpd[t]) {
                    const T q = bq[t] * ps[t] + cq[t] * diff;
                    c.psi[t][i] = q;
                    if (k.npsi[t]) {
                        add += T(k.npsi[t]) * c.dbpsi[t] * q;
                        any = true;
                    }
                } else if (k.npsi[t]) {
                    add += T(k.npsi[t]) * c.dbpsi[t] * ps[t];
                    any = true;
                }
            }
        }
        if (any) {
            if (k.toD) c.D[i] += add;
            else U[i] = u + add;
        }
        if (EPASS && k.lor) {
            T e = c.D[i];
            e *= k.epsInv;
            for (int q = 0; q < c.nPoles; ++q) e += k.negEpsInv * c.P[q][i];
            U[i] = e;
        }
    }
}

template <typename T, bool EPASS, typename I>
__global__ void __launch_bounds__(256) k_pass3d(const Pass<T> p) {
    __shared__ Class<T> tab[256];
    const int ci = blockIdx.z % 3;
    const Comp<T>& c = p.c[ci];
    for (int q = threadIdx.x + threadIdx.y * 32; q < c.ncls; q += 32 * kP3BZ) tab[q] = c.cls[q];
    __syncthreads();
    if (ci == 0) pass3d<T, EPASS, 0, I>(p, tab);
    else if (ci == 1) pass3d<T, EPASS, 1, I>(p, tab);
    else pass3d<T, EPASS, 2, I>(p, tab);
}

template <typename T>
void launch_pass(const Pass<T>& p, bool ePass, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (p.interior3d) {
        dim3 block(32, kP3BZ, 1);
        dim3 grid((p.lx - 2 + 31) / 32, (p.lz - 2 + kP3BZ - 1) / kP3BZ, 3 * ((p.ly - 2 + kP3CY - 1) / kP3CY));
        if (p.index64) {
            if (ePass) k_pass3d<T, true, long long><<<grid, block, 0, s>>>(p);
            else k_pass3d<T, false, long long><<<grid, block, 0, s>>>(p);
        } else {
            if (ePass) k_pass3d<T, true, int><<<grid, block, 0, s>>>(p);
            else k_pass3d<T, false, int><<<grid, block, 0, s>>>(p);
        }
    } else {
        // 2-D grids, and 3-D grids with updated halo cells: one thread per cell,
        // all components of the pass
        dim3 block(32, 1, 8);
        dim3 grid((p.lx + 31) / 32, p.lz, (p.ly + 7) / 8);
        if (ePass) k_pass<T, true><<<grid, block, 0, s>>>(p);
        else k_pass<T, false><<<grid, block, 0, s>>>(p);
    }
}

template <typename T>
__global__ void k_sources(const SourceTable s, const Fields<T> f, const int* __restrict__ step) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= s.n) return;
    const int st = *step;
    if (st >= s.nSteps) return;
    const double v = s.value[static_cast<long long>(s.src[j]) * s.nSteps + st];
    atomicAdd(&f.f[s.comp[j]][s.cell[j]], static_cast<T>(v));
}

template <typename T>
void launch_sources(const SourceTable& s, const Fields<T>& f, const int* step, void* stream) {
    if (s.n == 0) return;
    k_sources<T><<<(s.n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(s, f, step);
}

template <typename T>
__global__ void k_record(const RecordTable r, const Fields<T> f, const int* __restrict__ step) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= r.n) return;
    const int d = r.det[j];
    const int st = *step;
    const int ti = r.timeInt[d];
    if (st % ti != 0) return;
    const int ev = st / ti;
    if (ev >= r.nEvents[d]) return;
    const long long c = r.cell[j];
    const double v = (c < 0) ? 0.0 : static_cast<double>(f.f[r.comp[j]][c]);
    r.rec[r.recBase[d] + static_cast<long long>(ev) * r.nvals[d] + r.outIndex[j]] = v;
}

template <typename T>
void launch_record(const RecordTable& r, const Fields<T>& f, const int* step, void* stream) {
    if (r.n == 0) return;
    k_record<T><<<(r.n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(r, f, step);
}

template <typename T>
__global__ void __launch_bounds__(256) k_dft_sample(const DftTable<T> d, const Fields<T> f, const int* __restrict__ step) {
    const long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    const int st = *step;
    if (st % d.timeInt != 0 || p >= d.npts) return;
    const int slot = (st / d.timeInt) % d.K;
    d.ring[static_cast<long long>(slot) * d.npts + p] = f.f[d.comp[p]][d.cell[p]];
}

template <typename T>
void launch_dft_sample(const DftTable<T>& d, const Fields<T>& f, const int* step, void* stream) {
    if (d.npts == 0) return;
    k_dft_sample<T><<<static_cast<unsigned>((d.npts + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(d, f, step);
}

constexpr int kFoldPts = 32;   // points per tile of the fold kernel
constexpr int kFoldWarps = 8;  // 256 threads: lane -> frequency, warp -> 4 points of the tile

// Fold of K ring samples into the accumulators. Shared memory holds the K
// phasor rows (nfreq cos/-sin pairs each) and the tile's K x kFoldPts samples.
template <typename T>
__global__ void __launch_bounds__(256) k_dft_fold(const DftTable<T> d, const int* __restrict__ step, int flushCount,
                                                  int firstSample) {
    extern __shared__ unsigned char smem_raw[];
    T* ph = reinterpret_cast<T*>(smem_raw);          // [K][nfreq][2]
    T* smp = ph + static_cast<long long>(d.K) * d.nfreq * 2;  // [K][kFoldPts]
    int count, first;
    if (flushCount > 0) {
        count = flushCount;
        first = firstSample;
    } else {
        const int st = *step;
        if (st % d.timeInt != 0) return;
        const int n = st / d.timeInt;
        if (n % d.K != d.K - 1) return;
        count = d.K;
        first = n - (d.K - 1);
    }
    const int nf = d.nfreq;
    for (int q = threadIdx.x; q < count * nf * 2; q += blockDim.x)
        ph[q] = d.phasor[static_cast<long long>(first) * nf * 2 + q];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long tiles = (d.npts + kFoldPts - 1) / kFoldPts;
    for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const long long p0 = tile * kFoldPts;
        __syncthreads();
        for (int q = threadIdx.x; q < count * kFoldPts; q += blockDim.x) {
            const int k = q / kFoldPts, pp = q % kFoldPts;
            const long long p = p0 + pp;
            const int slot = (first + k) % d.K;
            smp[q] = (p < d.npts) ? d.ring[static_cast<long long>(slot) * d.npts + p] : T(0);
        }
        __syncthreads();
        constexpr int PPW = kFoldPts / kFoldWarps;  // points per warp
        for (int fb = 0; fb < nf; fb += 32) {
            const int fq = fb + lane;
            if (fq >= nf) break;
            T are[PPW], aim[PPW];
#pragma unroll
            for (int j = 0; j < PPW; ++j) are[j] = aim[j] = T(0);
            for (int k = 0; k < count; ++k) {
                const T c = ph[(k * nf + fq) * 2 + 0];
                const T sn = ph[(k * nf + fq) * 2 + 1];
#pragma unroll
                for (int j = 0; j < PPW; ++j) {
                    const T v = smp[k * kFoldPts + warp * PPW + j];
                    are[j] += c * v;
                    aim[j] += sn * v;
                }
            }
#pragma unroll
            for (int j = 0; j < PPW; ++j) {
                const long long p = p0 + warp * PPW + j;
                if (p >= d.npts) continue;
                d.re[p * nf + fq] += static_cast<double>(are[j]);
                d.im[p * nf + fq] += static_cast<double>(aim[j]);
            }
        }
    }
}

template <typename T>
static size_t fold_smem(const DftTable<T>& d) {
    return (static_cast<size_t>(d.K) * d.nfreq * 2 + static_cast<size_t>(d.K) * kFoldPts) * sizeof(T);
}

template <typename T>
void launch_dft_fold(const DftTable<T>& d, const int* step, int flushCount, int firstSample, void* stream) {
    if (d.npts == 0) return;
    const size_t sm = fold_smem(d);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_dft_fold<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    const long long tiles = (d.npts + kFoldPts - 1) / kFoldPts;
    const unsigned grid = static_cast<unsigned>(tiles < 152 * 4 ? tiles : 152 * 4);
    k_dft_fold<T><<<grid, 256, sm, static_cast<cudaStream_t>(stream)>>>(d, step, flushCount, firstSample);
}

__global__ void k_increment(int* step) { *step += 1; }

void launch_increment(int* step, void* stream) { k_increment<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(step); }

template void launch_pass<double>(const Pass<double>&, bool, void*);
template void launch_pass<float>(const Pass<float>&, bool, void*);
template void launch_sources<double>(const SourceTable&, const Fields<double>&, const int*, void*);
template void launch_sources<float>(const SourceTable&, const Fields<float>&, const int*, void*);
template void launch_record<double>(const RecordTable&, const Fields<double>&, const int*, void*);
template void launch_record<float>(const RecordTable&, const Fields<float>&, const int*, void*);
template void launch_dft_sample<double>(const DftTable<double>&, const Fields<double>&, const int*, void*);
template void launch_dft_sample<float>(const DftTable<float>&, const Fields<float>&, const int*, void*);
template void launch_dft_fold<double>(const DftTable<double>&, const int*, int, int, void*);
template void launch_dft_fold<float>(const DftTable<float>&, const int*, int, int, void*);

}  // namespace dev
}  // namespace chiml
