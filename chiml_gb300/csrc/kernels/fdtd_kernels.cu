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

template <typename T>
void launch_pass(const Pass<T>& p, bool ePass, void* stream) {
    dim3 block(32, p.lz > 1 ? 4 : 1, p.lz > 1 ? 2 : 8);
    dim3 grid((p.lx + block.x - 1) / block.x, (p.lz + block.y - 1) / block.y, (p.ly + block.z - 1) / block.z);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (ePass) k_pass<T, true><<<grid, block, 0, s>>>(p);
    else k_pass<T, false><<<grid, block, 0, s>>>(p);
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
__global__ void __launch_bounds__(256) k_dft(const DftTable d, const Fields<T> f, const int* __restrict__ step) {
    const long long j = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    const int st = *step;
    if (st % d.timeInt != 0) return;
    if (j >= d.npts * d.nfreq) return;
    const long long pt = j / d.nfreq;
    const int fq = static_cast<int>(j - pt * d.nfreq);
    const double v = static_cast<double>(f.f[d.comp[pt]][d.cell[pt]]);
    const double* ph = d.phasor + (static_cast<long long>(st) * d.nfreq + fq) * 2;
    d.re[j] += ph[0] * v;
    d.im[j] += ph[1] * v;
}

template <typename T>
void launch_dft(const DftTable& d, const Fields<T>& f, const int* step, void* stream) {
    const long long n = d.npts * d.nfreq;
    if (n == 0) return;
    k_dft<T><<<static_cast<unsigned>((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(d, f, step);
}

__global__ void k_increment(int* step) { *step += 1; }

void launch_increment(int* step, void* stream) { k_increment<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(step); }

template void launch_pass<double>(const Pass<double>&, bool, void*);
template void launch_pass<float>(const Pass<float>&, bool, void*);
template void launch_sources<double>(const SourceTable&, const Fields<double>&, const int*, void*);
template void launch_sources<float>(const SourceTable&, const Fields<float>&, const int*, void*);
template void launch_record<double>(const RecordTable&, const Fields<double>&, const int*, void*);
template void launch_record<float>(const RecordTable&, const Fields<float>&, const int*, void*);
template void launch_dft<double>(const DftTable&, const Fields<double>&, const int*, void*);
template void launch_dft<float>(const DftTable&, const Fields<float>&, const int*, void*);

}  // namespace dev
}  // namespace chiml
