// CPU FP64 oracle of chiML's time-step loop (test infrastructure only).
//
// The oracle executes the compiled plan cell by cell in double precision with
// the arithmetic and ordering of the reference's update functions:
//   step order           FDTD_MANAGER/parallelFDTDField.hpp:1228-1303
//   curl updates         UTIL/FDTD_up_eq.cpp:10-35   (TwoCompCurl / OneCompCurlJ/K)
//   CPML psi and terms   PML/parallelPML.cpp:12-40   (addPsi / addGridOnly / updatePsiField)
//   Lorentz polarisation UTIL/FDTD_up_eq.cpp:425-448 (UpdateLorPol)
//   D -> E               UTIL/FDTD_up_eq.cpp:838-848 (DtoU)
//   soft sources         SOURCE/parallelSourceNormal.cpp:15-37
//   DFT accumulation     DTC/parallelStorageFreqDTC.cpp:21-30, DTC/parallelFlux.hpp:296-314
//   detector sampling    DTC/parallelStorageDTC.cpp:17-48
// Its outputs are pinned by the golden files of the reference's own CPU build
// (tests/golden). Only tests, the smoke check and the CPU-baseline leg of the
// benchmark call it; the product path never does.
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../chiml_gb300/csrc/host/outputs.hpp"
#include "../chiml_gb300/csrc/host/plan.hpp"

namespace {

using namespace chiml;

struct OracleSim {
    Plan P;
    std::vector<double> F[6];
    std::vector<double> Dd[3];
    std::vector<double> psi[6][2];
    std::vector<std::vector<double>> lorP[3], prevP[3];
    RunRecord rec;
    int step = 0;

    explicit OracleSim(const Plan& plan) : P(plan) {
        const std::size_t N = static_cast<std::size_t>(P.dims.cells());
        for (int c = 0; c < 6; ++c) {
            if (!P.comp[c].present) continue;
            F[c].assign(N, 0.0);
            for (int t = 0; t < 2; ++t)
                if (P.comp[c].term[t].present && P.comp[c].term[t].hasPsi) psi[c][t].assign(N, 0.0);
        }
        for (int c = 0; c < 3; ++c) {
            if (!P.comp[c].present) continue;
            if (P.comp[c].hasD) Dd[c].assign(N, 0.0);
            for (int p = 0; p < P.comp[c].nPoles; ++p) {
                lorP[c].emplace_back(N, 0.0);
                prevP[c].emplace_back(N, 0.0);
            }
        }
        rec.detectors.resize(P.detectors.size());
        for (auto& fp : P.fluxes) {
            std::size_t n = static_cast<std::size_t>(fp.npts) * fp.spec.freqList.size();
            rec.fluxRe.emplace_back(n, 0.0);
            rec.fluxIm.emplace_back(n, 0.0);
            rec.fluxSamples.push_back(0);
        }
        // detectors and flux take their t = 0 sample at construction (parallelFDTDField.cpp:831-837)
        record(0.0);
        dft(0);
    }

    const double* fieldOf(int comp) const { return comp < 6 ? F[comp].data() : Dd[comp - 6].data(); }

    void record(double) {
        for (std::size_t k = 0; k < P.detectors.size(); ++k) {
            const DetectorPlan& dp = P.detectors[k];
            if (step % dp.timeInt != 0) continue;
            std::vector<double> v;
            for (auto& f : dp.fields) {
                const double* src = fieldOf(f.comp);
                for (long long id : f.cells) v.push_back(id < 0 ? 0.0 : src[id]);
            }
            rec.detectors[k].push_back(std::move(v));
        }
    }

    void dft(int st) {
        for (std::size_t q = 0; q < P.fluxes.size(); ++q) {
            const FluxPlan& fp = P.fluxes[q];
            if (st % fp.spec.timeInt != 0) continue;
            const double tt = P.tcur[st];
            const std::vector<double>& fl = fp.spec.freqList;
            const std::size_t nf = fl.size();
            std::vector<double> cr(nf), ci(nf);
            for (std::size_t f = 0; f < nf; ++f) {
                std::complex<double> e = std::exp(std::complex<double>(0.0, -1.0 * tt * fl[f]));
                cr[f] = e.real();
                ci[f] = e.imag();
            }
            for (const FreqStore& s : fp.stores) {
                const double* src = F[s.comp].data();
#pragma omp parallel for schedule(static)
                for (std::size_t p = 0; p < s.cells.size(); ++p) {
                    double v = src[s.cells[p]];
                    std::size_t base = static_cast<std::size_t>(s.accOffset + static_cast<long long>(p)) * nf;
                    for (std::size_t f = 0; f < nf; ++f) {
                        rec.fluxRe[q][base + f] += cr[f] * v;
                        rec.fluxIm[q][base + f] += ci[f] * v;
                    }
                }
            }
            rec.fluxSamples[q] += 1;
        }
    }

    // One half step of component c: psi recursion + curl/CPML terms onto E/H or D.
    void curl(int c) {
        const CompPlan& cp = P.comp[c];
        const Dims& D = P.dims;
        double* U = F[c].data();
        double* Dc = (c < 3 && cp.hasD) ? Dd[c].data() : nullptr;
        const TermPlan* T = cp.term;
        const double* G[2] = {T[0].present ? F[T[0].field].data() : nullptr, T[1].present ? F[T[1].field].data() : nullptr};
#pragma omp parallel for schedule(static)
        for (int y = 0; y < D.ly; ++y)
            for (int z = 0; z < D.lz; ++z)
                for (int x = 0; x < D.lx; ++x) {
                    long long i = D.idx(x, y, z);
                    if (cp.code[i] == 0) continue;
                    const ClassInfo& k = cp.classes[cp.code[i]];
                    int coord[3] = {x, y, z};
                    double add = 0.0;
                    bool any = false;
                    for (int t = 0; t < 2; ++t) {
                        if (!T[t].present) continue;
                        int a = coord[T[t].axis];
                        double coef = k.cint[t] + k.nplain[t] * T[t].db + (k.kflag[t] ? T[t].kprof[a] : 0.0);
                        bool psiTerm = T[t].hasPsi && (k.psiUpd[t] || k.npsi[t]);
                        if (coef == 0.0 && !psiTerm) continue;
                        double diff = G[t][i] - G[t][i + T[t].off];
                        if (k.psiUpd[t]) {
                            double& ps = psi[c][t][i];
                            ps = T[t].b[a] * ps + T[t].cpsi[a] * diff;
                        }
                        if (coef != 0.0) {
                            add += coef * diff;
                            any = true;
                        }
                        if (k.npsi[t] && T[t].hasPsi) {
                            add += k.npsi[t] * T[t].dbpsi * psi[c][t][i];
                            any = true;
                        }
                    }
                    if (!any) continue;
                    if (k.toD) Dc[i] += add;
                    else U[i] += add;
                }
    }

    void polarisation(int c) {
        const CompPlan& cp = P.comp[c];
        if (cp.nPoles == 0) return;
        const Dims& D = P.dims;
        const double* E = F[c].data();
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < D.cells(); ++i) {
            const ClassInfo& k = cp.classes[cp.code[i]];
            if (!k.lor) continue;
            const auto& al = P.alpha[k.obj];
            const auto& xi = P.xi[k.obj];
            const auto& ga = P.gamma[k.obj];
            for (std::size_t p = 0; p < al.size(); ++p) {
                double old = lorP[c][p][i];
                double np = al[p] * old;
                np += xi[p] * prevP[c][p][i];
                np += ga[p] * E[i];
                lorP[c][p][i] = np;
                prevP[c][p][i] = old;
            }
        }
    }

    void d2e(int c) {
        const CompPlan& cp = P.comp[c];
        if (!cp.hasD) return;
        const Dims& D = P.dims;
        double* E = F[c].data();
        const double* Dc = Dd[c].data();
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < D.cells(); ++i) {
            const ClassInfo& k = cp.classes[cp.code[i]];
            if (!k.lor) continue;
            double e = Dc[i];
            e *= 1.0 / k.eps;
            for (int p = 0; p < cp.nPoles; ++p) e += (-1.0 / k.eps) * lorP[c][p][i];
            E[i] = e;
        }
    }

    void stepOnce() {
        // H half step (updateH + H CPML)
        for (int c = 3; c < 6; ++c)
            if (P.comp[c].present) curl(c);
        // soft sources at t_n (after H, before E)
        for (auto& s : P.sources) {
            double v = s.value[static_cast<std::size_t>(step)];
            for (long long id : s.cells) F[s.comp][id] += v;
        }
        // E half step: polarisations from E^n, curl onto E or D, D -> E
        for (int c = 0; c < 3; ++c)
            if (P.comp[c].present) polarisation(c);
        for (int c = 0; c < 3; ++c)
            if (P.comp[c].present) curl(c);
        for (int c = 0; c < 3; ++c)
            if (P.comp[c].present) d2e(c);
        ++step;
        record(P.tcur[step]);
        dft(step);
    }
};

thread_local std::string g_err;

}  // namespace

extern "C" {

const char* chiml_oracle_last_error() { return g_err.c_str(); }

void* chiml_oracle_create(const char* json_path) {
    try {
        Inputs in = read_inputs_file(json_path);
        Plan P = build_plan(in);
        return new OracleSim(P);
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

int chiml_oracle_steps_total(void* h) { return static_cast<OracleSim*>(h)->P.nSteps; }

// Host threads the step loops use.
int chiml_oracle_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

long long chiml_oracle_cells(void* h) { return static_cast<OracleSim*>(h)->P.dims.cells(); }

void chiml_oracle_dims(void* h, int* out6) {
    const Dims& D = static_cast<OracleSim*>(h)->P.dims;
    out6[0] = D.lx;
    out6[1] = D.ly;
    out6[2] = D.lz;
    out6[3] = D.nx;
    out6[4] = D.ny;
    out6[5] = D.nz;
}

int chiml_oracle_step(void* h, int n) {
    OracleSim* s = static_cast<OracleSim*>(h);
    for (int k = 0; k < n && s->step < s->P.nSteps; ++k) s->stepOnce();
    return s->step;
}

// Copies component c (0..5 fields, 6..8 D) into out (cells doubles); returns 0 or -1.
int chiml_oracle_get_field(void* h, int c, double* out) {
    OracleSim* s = static_cast<OracleSim*>(h);
    const std::vector<double>* v = (c < 6) ? &s->F[c] : &s->Dd[c - 6];
    if (v->empty()) return -1;
    std::memcpy(out, v->data(), v->size() * sizeof(double));
    return 0;
}

int chiml_oracle_finalize(void* h, const char* out_dir) {
    OracleSim* s = static_cast<OracleSim*>(h);
    try {
        write_detectors(s->P, s->rec, out_dir ? out_dir : "", s->step);
        write_fluxes(s->P, s->rec, out_dir ? out_dir : "");
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

void chiml_oracle_destroy(void* h) { delete static_cast<OracleSim*>(h); }

// Runs a whole simulation; returns wall seconds of the step loop, or -1 on error.
double chiml_oracle_run(const char* json_path, const char* out_dir, int steps) {
    void* h = chiml_oracle_create(json_path);
    if (!h) return -1.0;
    OracleSim* s = static_cast<OracleSim*>(h);
    int n = (steps < 0) ? s->P.nSteps : steps;
    auto t0 = std::chrono::steady_clock::now();
    chiml_oracle_step(h, n);
    auto t1 = std::chrono::steady_clock::now();
    int rc = chiml_oracle_finalize(h, out_dir);
    chiml_oracle_destroy(h);
    if (rc != 0) return -1.0;
    return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
