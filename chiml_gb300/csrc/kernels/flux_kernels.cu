// Flux integration on the device (parallelFlux.hpp:325-545 as a gather plus a weighted sum).
//
//   k_flux_partial  one block per (tile of kFluxTile integration points, up to 256 frequencies):
//                   each thread forms the four face-grid values of its frequency at every
//                   point of the tile from the accumulators (the threads of a warp read
//                   consecutive frequencies of one point), the integrand and its Simpson
//                   weight, and writes the tile's partial sum (FP64 form: in FP64; split
//                   form: in FP32 within the tile).
//   k_flux_sum      sums a face's partials in tile order (a fixed order: the result does not
//                   depend on scheduling) and scales by fluxConv * face weight.
#include "flux_device.hpp"

namespace chiml {
namespace dev {

namespace {

// Complex values of the integrand in the arithmetic of the form: FP64, or FP32 for the
// split form, whose accumulators are float-float pairs (hi, lo) in the same 8 bytes: there
// each value is taken to FP32 (hi + lo) and the tile's products and sums run on the FP32
// pipe (GB300's FP64 rate is 1/64 of it); the tiles' partial sums are combined in FP64.
template <typename R>
struct Cx {
    R x, y;
};

template <typename R>
__device__ __forceinline__ R accValue(const double* __restrict__ a, long long idx) {
    if constexpr (sizeof(R) == 8) {
        return a[idx];
    } else {
        const float2 v = reinterpret_cast<const float2*>(a)[idx];
        return v.x + v.y;
    }
}

template <typename R>
__device__ __forceinline__ Cx<R> gridValue(const FluxFaceDev& F, int w, int s, int ff, int nfreq, const double* __restrict__ re,
                                           const double* __restrict__ im) {
    Cx<R> g{R(0), R(0)};
    const long long k1 = F.start[w][s + 1];
    for (long long k = F.start[w][s]; k < k1; ++k) {
        const long long idx = F.pt[w][k] * nfreq + ff;
        const R sc = static_cast<R>(F.scale[w][k]);
        g.x += sc * accValue<R>(re, idx);
        g.y += sc * accValue<R>(im, idx);
    }
    return g;
}

// a * conj(b)
template <typename R>
__device__ __forceinline__ Cx<R> mulConj(Cx<R> a, Cx<R> b) {
    return Cx<R>{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}

// The tile's weighted sum of E_j conj(H_k) - E_k conj(H_j), then scaled by 1 / nt^2 once
// (the reference divides every product by nt^2: the same value up to rounding, without
// four divisions per point and frequency).
template <typename R>
__global__ void __launch_bounds__(kFluxThreads) k_flux_partial(const FluxFaceDev* __restrict__ faces, const int4* __restrict__ tiles,
                                                               int nfreq, const double* __restrict__ re, const double* __restrict__ im,
                                                               double invNt2, double2* __restrict__ partial) {
    const int ff = blockIdx.y * blockDim.x + threadIdx.x;
    if (ff >= nfreq) return;
    const int4 t = tiles[blockIdx.x];
    const FluxFaceDev& F = faces[t.x];
    Cx<R> acc{R(0), R(0)};
    for (int s = t.y; s < t.z; ++s) {
        Cx<R> v{R(0), R(0)};
        if (F.has[0]) v = mulConj<R>(gridValue<R>(F, 0, s, ff, nfreq, re, im), gridValue<R>(F, 3, s, ff, nfreq, re, im));
        if (F.has[1]) {
            const Cx<R> u = mulConj<R>(gridValue<R>(F, 1, s, ff, nfreq, re, im), gridValue<R>(F, 2, s, ff, nfreq, re, im));
            v.x -= u.x;
            v.y -= u.y;
        }
        const R w = static_cast<R>(F.wx[s % F.nx] * F.wy[s / F.nx]);
        acc.x += w * v.x;
        acc.y += w * v.y;
    }
    partial[static_cast<long long>(blockIdx.x) * nfreq + ff] =
        make_double2(static_cast<double>(acc.x) * invNt2, static_cast<double>(acc.y) * invNt2);
}

__global__ void k_flux_sum(const FluxFaceDev* __restrict__ faces, int nFaces, int nfreq, const double2* __restrict__ partial,
                           double2* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nFaces * nfreq) return;
    const int face = i / nfreq, ff = i % nfreq;
    const FluxFaceDev& F = faces[face];
    double2 s = make_double2(0.0, 0.0);
    for (int t = 0; t < F.nTiles; ++t) {
        const double2 p = partial[static_cast<long long>(F.firstTile + t) * nfreq + ff];
        s.x += p.x;
        s.y += p.y;
    }
    out[static_cast<long long>(ff) * nFaces + face] = make_double2(F.pref * s.x, F.pref * s.y);
}

}  // namespace

void launch_flux_faces(const FluxFaceDev* faces, int nFaces, const int4* tiles, int nTiles, int nfreq, const double* re,
                       const double* im, bool pairs, double nt2, double2* partial, double2* out, void* stream) {
    if (nFaces == 0 || nfreq == 0) return;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nTiles > 0) {
        // whole warps over the frequencies: blocks of up to kFluxThreads threads
        const int per = (nfreq + 31) / 32 * 32;
        const int bs = per < kFluxThreads ? per : kFluxThreads;
        const dim3 grid(static_cast<unsigned>(nTiles), static_cast<unsigned>((nfreq + bs - 1) / bs));
        if (pairs) k_flux_partial<float><<<grid, bs, 0, s>>>(faces, tiles, nfreq, re, im, 1.0 / nt2, partial);
        else k_flux_partial<double><<<grid, bs, 0, s>>>(faces, tiles, nfreq, re, im, 1.0 / nt2, partial);
    }
    const int n = nFaces * nfreq;
    k_flux_sum<<<(n + 127) / 128, 128, 0, s>>>(faces, nFaces, nfreq, partial, out);
}

}  // namespace dev
}  // namespace chiml
