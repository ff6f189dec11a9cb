// End-of-run products of a simulation: detector files and DFT-flux spectra,
// written in chiML's formats.
#pragma once

#include <array>
#include <string>
#include <vector>

#include "plan.hpp"

namespace chiml {

// Values gathered during the run, in the layout the writers expect.
struct RunRecord {
    // detectors[k][e] = concatenated field boxes (fields in plan order, each
    // box in storage order) at output event e (step e * timeInt)
    std::vector<std::vector<std::vector<double>>> detectors;
    // flux accumulators per flux: re/im [point][freq], and the number of DFT samples
    std::vector<std::vector<double>> fluxRe, fluxIm;
    std::vector<int> fluxSamples;
    // per flux, optionally: the integrated flux of every face, [freq * nFaces + face]
    // (computed on the device); when present the accumulators are not needed
    std::vector<std::vector<cplx>> fluxFaces;
    // per emitter: the total polarisation of each coupled component, one value per step
    // (parallelQE.cpp:41-44 accumP_), and per population detector its events
    std::vector<std::array<std::vector<double>, 3>> emitterP;
    std::vector<std::vector<std::vector<cplx>>> emitterPop;
    // incident fields of the TFSF surface (E_incd_ / H_incd_, parallelFDTDField.hpp:1238-1255):
    // per component two samples per step, 2 * (nSteps + 1) values; empty without a surface
    std::array<std::vector<cplx>, 3> incE, incH;
    // frequency-domain detectors: re/im [point][freq] over the concatenated fields of each
    // detector, and its number of samples
    std::vector<std::vector<double>> freqRe, freqIm;
    std::vector<int> freqSamples;
};

// Number of values one output event of detector k stores.
long long detector_event_values(const DetectorPlan& dp);
// Number of output events of a detector over nSteps steps (including t = 0).
int detector_events(const DetectorPlan& dp, int nSteps);

// Writes every detector file (TXT: parallelDTC_TXT.cpp:13-55; BIN: parallelDTC_BIN.cpp:12-50).
void write_detectors(const Plan& P, const RunRecord& R, const std::string& outDir, int stepsDone);
// The combination and integration of one flux face as data (parallelFlux.hpp:325-405 combine
// the accumulated points into four face grids Ej, Ek, Hj, Hk; getFlux, :406-545, integrates
// (Ej conj(Hk) - Ek conj(Hj)) / nt^2 over the face with simps2D). Grid point c = x + nx * y
// (x along the face's cor axis, y along transCor1) takes, for grid w, the terms
// [start[w][c], start[w][c + 1]) of (accumulator point, scale), in the reference's order.
struct FluxFaceMap {
    int nx = 0, ny = 0, sz = 0;  // integration grid and the points the product fills
    double dx = 0.0, dy = 0.0;
    double pref = 1.0;            // fluxConv * face weight
    bool has[4] = {false, false, false, false};
    std::vector<long long> start[4];
    std::vector<long long> pt[4];
    std::vector<double> scale[4];
    // simps2D as a linear form: weight of point (x, y) = wx[x] * wy[y] (length 1, weight 1,
    // along an axis of one point)
    std::vector<double> wx, wy;
};

// The weights w with simps(v, n, d) = sum_i w[i] v[i] (parallelFlux.hpp:548-576).
std::vector<double> simps_weights(int n, double d);
// The maps of the faces of flux q. Throws where the reference's combination or integration
// would fail.
std::vector<FluxFaceMap> flux_face_maps(const Plan& P, std::size_t q);
// The four combined frequency-domain grids of each face of a flux, [face][Ej, Ek, Hj, Hk],
// each [point][freq] in the reference's Grid order (frequency fastest, then the face's cor
// axis, then transCor1); a grid the face does not have is empty.
typedef std::vector<std::array<std::vector<cplx>, 4>> FluxGrids;
// The integrated flux of every face of flux q from its accumulators, [freq * nFaces + face],
// in the reference's arithmetic. With `seed`, each grid starts from the seed's values instead
// of zero (a loaded incident field, negated); with `grids`, the combined grids are kept.
std::vector<cplx> flux_face_values(const Plan& P, std::size_t q, const std::vector<FluxFaceMap>& maps,
                                   const std::vector<double>& re, const std::vector<double>& im, int nt,
                                   const FluxGrids* seed = nullptr, FluxGrids* grids = nullptr);
// The flux fields file of parallelFluxDTC::saveFields / loadFields (parallelFlux.hpp:616-720):
// int nfreq, the flux region's size (3 ints), the number of faces for each of Ej, Ek, Hj, Hk
// (4 ints), then every face's Ej grid, every face's Ek, Hj and Hk grids, each as its size
// (3 ints: nfreq, points along transCor1, along cor) and its complex values.
void write_flux_fields(const Plan& P, std::size_t q, const std::vector<FluxFaceMap>& maps, const FluxGrids& grids,
                       const std::string& path);
// Reads such a file, checks it against flux q as loadFields does, and returns its grids
// scaled by `weight` (the reference loads with -1).
FluxGrids read_flux_fields(const Plan& P, std::size_t q, const std::vector<FluxFaceMap>& maps, const std::string& path,
                           double weight);
// Writes "<name>.dat" of every flux (parallelFlux.hpp:325-560) from R.fluxFaces, or from the
// accumulators where those are absent.
void write_fluxes(const Plan& P, const RunRecord& R, const std::string& outDir);

// Writes every frequency-domain detector (parallelDetectorFREQ_Base::toFile / toMap with the
// incident fields, DTC/parallelDTC_FREQ.hpp:390-583, as main.cpp:73-105 calls them).
void write_freq_detectors(const Plan& P, const RunRecord& R, const std::string& outDir);

// Writes the emitter polarisation file (parallelQEReal::outputPol, parallelQE.cpp:520-557) and
// the population files (QEPopDtc::toFile, QEPopDtc.cpp:37-61).
void write_emitters(const Plan& P, const RunRecord& R, const std::string& outDir);

std::string out_path(const std::string& outDir, const std::string& name);

}  // namespace chiml
