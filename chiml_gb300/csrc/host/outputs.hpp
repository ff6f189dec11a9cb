// End-of-run products of a simulation: detector files and DFT-flux spectra,
// written in chiML's formats.
#pragma once

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
// Combines the flux accumulators and writes "<name>.dat" (parallelFlux.hpp:325-560).
void write_fluxes(const Plan& P, const RunRecord& R, const std::string& outDir);

// Writes every frequency-domain detector (parallelDetectorFREQ_Base::toFile / toMap with the
// incident fields, DTC/parallelDTC_FREQ.hpp:390-583, as main.cpp:73-105 calls them).
void write_freq_detectors(const Plan& P, const RunRecord& R, const std::string& outDir);

// Writes the emitter polarisation file (parallelQEReal::outputPol, parallelQE.cpp:520-557) and
// the population files (QEPopDtc::toFile, QEPopDtc.cpp:37-61).
void write_emitters(const Plan& P, const RunRecord& R, const std::string& outDir);

std::string out_path(const std::string& outDir, const std::string& name);

}  // namespace chiml
