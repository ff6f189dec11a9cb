// Device form of the flux integration at the end of a run: the combination of each face's
// accumulated points into its four field grids and getFlux's integral over the face
// (parallelFlux.hpp:325-545), evaluated from the DFT accumulators where they live, so that
// only nfreq values per face come back to the host. Kernels in flux_kernels.cu.
#pragma once

#include <cuda_runtime.h>

namespace chiml {
namespace dev {

constexpr int kFluxTile = 64;      // integration points per partial sum
constexpr int kFluxThreads = 256;  // frequencies per block (at most)

// One face: grid w (0 Ej, 1 Ek, 2 Hj, 3 Hk) at integration point s takes the terms
// [start[w][s], start[w][s + 1]) of scale * accumulator[pt]; the integrand at s is
// (Ej conj(Hk) - Ek conj(Hj)) / nt^2 with weight wx[s % nx] * wy[s / nx].
struct FluxFaceDev {
    int nx, sz;
    int has[4];
    const long long* start[4];
    const long long* pt[4];
    const double* scale[4];
    const double* wx;
    const double* wy;
    double pref;     // fluxConv * face weight
    int firstTile, nTiles;
};

// Integrated flux of every face: out[f * nFaces + face] (host memory layout of the writer).
// faces and tiles ({face, s0, s1, unused}) are device arrays; partial holds
// nTiles * nfreq values; re / im are the accumulators [point][freq], FP64 or (pairs)
// float-float pairs in the same 8 bytes.
void launch_flux_faces(const FluxFaceDev* faces, int nFaces, const int4* tiles, int nTiles, int nfreq, const double* re,
                       const double* im, bool pairs, double nt2, double2* partial, double2* out, void* stream);

}  // namespace dev
}  // namespace chiml
