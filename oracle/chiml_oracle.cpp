// CPU FP64 oracle of chiML's time-step loop (test infrastructure only).
//
// The oracle executes the compiled plan cell by cell in double precision with
// the arithmetic and ordering of the reference's update functions:
//   step order           FDTD_MANAGER/parallelFDTDField.hpp:1228-1303
//   curl updates         UTIL/FDTD_up_eq.cpp:10-35   (TwoCompCurl / OneCompCurlJ/K)
//   CPML psi and terms   PML/parallelPML.cpp:12-40   (addPsi / addGridOnly / updatePsiField)
//   Lorentz polarisation UTIL/FDTD_up_eq.cpp:425-448 (UpdateLorPol), 450-521 (UpdateLorPolOrDip)
//   D -> E               UTIL/FDTD_up_eq.cpp:838-848 (DtoU), 862-875 (orDipDtoU)
//   soft sources         SOURCE/parallelSourceNormal.cpp:15-37
//   DFT accumulation     DTC/parallelStorageFreqDTC.cpp:21-30, DTC/parallelFlux.hpp:296-314
//   detector sampling    DTC/parallelStorageDTC.cpp:17-48, DTC/parallelDTC_FREQ.hpp:258-264 (frequency domain)
//   TFSF surfaces        SOURCE/parallelTFSF.hpp:1058-1186, SOURCE/parallelTFSF.cpp:11-94, PML/PML.cpp:12-31
//   emitters             ML/parallelQE.hpp:614-770 (addQE, updateDensity, denDeriv, PCABAM4),
//                        UTIL/FDTD_up_eq.cpp:1367-1420 (addP, getE_TE/TM), ML/Hamiltonian.cpp:59-69
//   per-cell dipoles     an extension without a reference counterpart (EmitterPlan::cellDip):
//                        the coupling (E . w) times the z operator, P_c = w_c times the z
//                        polarisation; pinned by its reduction to the reference (w = z gives
//                        the reference's outputs) and by the GPU's FP64 form
// Its outputs are pinned by the golden files of the reference's own CPU build
// (tests/golden). Only tests, the smoke check and the CPU-baseline leg of the
// benchmark call it; the product path never does.
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../chiml_gb300/csrc/host/outputs.hpp"
#include "../chiml_gb300/csrc/host/plan.hpp"

namespace {

using namespace chiml;

// One emitter object stepped as ML/parallelQE.hpp:674-770 does for one process:
// addQE (P into E, then updateDensity: gather E, PCABAM4 per member and cell,
// populations, P from rho). The BLAS calls are restated with the arithmetic order
// of the reference build's BLAS (dot-product zgemm, element-wise zaxpy/zdotc).
struct EmitterSim {
    const EmitterPlan& e;
    const Dims& D;
    int N, n2, nm, nc;
    std::vector<cplx> rho;                  // [member][cell][n2]
    std::vector<cplx> kd[4];                // derivatives at n, n-1, n-2, n-3
    std::vector<double> Pbox[3];
    std::array<std::vector<double>, 3> totP;
    std::vector<cplx> curPop;
    std::vector<std::vector<cplx>> allPop;
    int tstep = 0;
    std::vector<cplx> H, pred, kp, tmp;

    EmitterSim(const EmitterPlan& ep, const Dims& dd) : e(ep), D(dd) {
        N = e.nlevel;
        n2 = N * N;
        nm = e.nMembers;
        nc = static_cast<int>(e.cellGrid.size());
        rho.assign(static_cast<std::size_t>(nm) * nc * n2, cplx(0.0, 0.0));
        for (int m = 0; m < nm; ++m)
            for (int c = 0; c < nc; ++c) rho[(static_cast<std::size_t>(m) * nc + c) * n2] = cplx(e.weight[m], 0.0);
        for (auto& k : kd) k.assign(rho.size(), cplx(0.0, 0.0));
        const std::size_t pb = static_cast<std::size_t>(e.pDims[0]) * e.pDims[1] * e.pDims[2];
        for (auto& p : Pbox) p.assign(pb, 0.0);
        curPop.assign(e.dtcLevs.size(), cplx(0.0, 0.0));
        allPop.assign(e.dtcLevs.size(), {});
        H.resize(n2);
        pred.resize(n2);
        kp.resize(n2);
        tmp.resize(n2);
    }

    // Hamiltonian::getHam (Hamiltonian.cpp:59-69)
    void getHam(int m, cplx ex, cplx ey, cplx ez) {
        for (int i = 0; i < n2; ++i) H[i] = cplx(0.0, 0.0);
        for (int i = 0; i < N; ++i) H[i * N + i] = cplx(e.h0[static_cast<std::size_t>(m) * N + i], 0.0);
        if (ex == 0.0 && ey == 0.0 && ez == 0.0) return;
        const cplx a[3] = {ex, ey, ez};
        for (int c = 0; c < 3; ++c)
            if (e.addMu[c])
                for (int i = 0; i < n2; ++i) H[i] += a[c] * e.negMu[c][i];
    }

    // denDeriv, MKL form (parallelQE.hpp:727-744): temp = (i/hbar) H den, out = temp + temp^H, + relaxation
    void denDeriv(const cplx* den, cplx* out) {
        const cplx alpha(0.0, 1.0 / e.hbar);
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                cplx s = 0.0;
                for (int l = 0; l < N; ++l) s += H[i + l * N] * den[l + j * N];
                tmp[i + j * N] = cplx(0.0) + alpha * s;
            }
        const cplx one(1.0, 0.0);
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) out[i * N + j] = one * tmp[i * N + j] + one * std::conj(tmp[j * N + i]);
        for (std::size_t ii = 0; ii < e.gam.size(); ++ii)
            for (auto& g : e.gam[ii]) out[ii] += den[g.first] * g.second;
    }

    void axpy(double a, const cplx* x, cplx* y) {
        const cplx ca(a, 0.0);
        for (int i = 0; i < n2; ++i) y[i] += ca * x[i];
    }

    // PCABAM4 (parallelQE.hpp:751-770) for member m, cell c
    void pcabam4(int m, int c, cplx ex, cplx ey, cplx ez) {
        const std::size_t o = (static_cast<std::size_t>(m) * nc + c) * n2;
        cplx* r = &rho[o];
        cplx* k0 = &kd[0][o];
        cplx* k1 = &kd[1][o];
        cplx* k2 = &kd[2][o];
        cplx* k3 = &kd[3][o];
        const double dt = e.dt;
        for (int i = 0; i < n2; ++i) pred[i] = r[i];
        axpy(55.0 * dt / 24.0, k0, pred.data());
        axpy(-59.0 * dt / 24.0, k1, pred.data());
        axpy(37.0 * dt / 24.0, k2, pred.data());
        axpy(-9.0 * dt / 24.0, k3, pred.data());
        getHam(m, ex, ey, ez);
        denDeriv(pred.data(), kp.data());
        axpy(9.0 * dt / 24.0, kp.data(), r);
        axpy(19.0 * dt / 24.0, k0, r);
        axpy(-5.0 * dt / 24.0, k1, r);
        axpy(dt / 24.0, k2, r);
        for (int i = 0; i < n2; ++i) {
            k3[i] = k2[i];
            k2[i] = k1[i];
            k1[i] = k0[i];
        }
        getHam(m, ex, ey, ez);
        denDeriv(r, k0);
    }

    // addQE: P into E (MLUpdateFxnReal::addP, FDTD_up_eq.cpp:1367-1380), then updateDensity
    void step(std::vector<double>* F, const std::vector<double>& eps) {
        const int off[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, e.zOff}};
        const int px = e.pDims[0], pz = e.pDims[2];
        for (int c = 0; c < 3; ++c) {
            if (!e.comp[c]) continue;
            double* E = F[c].data();
            for (int kk = 0; kk < e.addN[2]; ++kk)
                for (int jj = 0; jj < e.addN[1]; ++jj)
                    for (int ii = 0; ii < e.addN[0]; ++ii) {
                        const long long g = D.idx(e.boxBase[0] + ii, e.boxBase[1] + jj, e.boxBase[2] + kk);
                        const long long gb = D.idx(e.boxBase[0] + ii + off[c][0], e.boxBase[1] + jj + off[c][1],
                                                   e.boxBase[2] + kk + off[c][2]);
                        const double pa = Pbox[c][ii + px * (kk + pz * jj)];
                        const double pb = Pbox[c][(ii + off[c][0]) + px * ((kk + off[c][2]) + pz * (jj + off[c][1]))];
                        E[g] += -0.5 * pa / eps[g];
                        E[g] += -0.5 * pb / eps[gb];
                    }
        }
        // updateDensity (parallelQE.hpp:614-678)
        const long long unit[3] = {1, static_cast<long long>(D.lx) * D.lz, D.lx};
        std::vector<cplx> eAt(static_cast<std::size_t>(nc) * 3, cplx(0.0, 0.0));
        for (int q = 0; q < nc; ++q) {
            const long long g = e.cellGrid[q];
            for (int c = 0; c < 3; ++c) {
                if (!e.comp[c]) continue;
                const double* E = F[c].data();
                if (c == 2 && e.gatherZCopy) eAt[q * 3 + c] = cplx(E[g], 0.0);
                else eAt[q * 3 + c] = cplx(0.5 * E[g] + 0.5 * E[g - unit[c]], 0.0);
            }
            if (!e.cellDip.empty()) {
                // per-cell dipole w (extension): the coupling is (E . w) times the z operator
                const std::array<double, 3>& w = e.cellDip[static_cast<std::size_t>(q)];
                const double ew = eAt[q * 3 + 0].real() * w[0] + eAt[q * 3 + 1].real() * w[1] + eAt[q * 3 + 2].real() * w[2];
                eAt[q * 3 + 0] = eAt[q * 3 + 1] = cplx(0.0, 0.0);
                eAt[q * 3 + 2] = cplx(ew, 0.0);
            }
        }
        for (auto& p : Pbox) std::fill(p.begin(), p.end(), 0.0);
        for (int m = 0; m < nm; ++m)
            for (int q = 0; q < nc; ++q) {
                pcabam4(m, q, eAt[q * 3 + 0], eAt[q * 3 + 1], eAt[q * 3 + 2]);
                const cplx* r = &rho[(static_cast<std::size_t>(m) * nc + q) * n2];
                for (std::size_t d = 0; d < e.dtcLevs.size(); ++d)
                    if (tstep % e.dtcTimeInt == 0) curPop[d] += r[e.dtcLevs[d]];
                if (!e.cellDip.empty()) {
                    // P_c = w_c times the polarisation of the z operator
                    cplx s = 0.0;
                    for (int i = 0; i < n2; ++i) s += std::conj(r[i]) * e.mu[2][i];
                    for (int c = 0; c < 3; ++c)
                        if (e.comp[c]) Pbox[c][e.cellP[q]] += e.na * std::real(s) * e.cellDip[static_cast<std::size_t>(q)][c];
                    continue;
                }
                for (int c = 0; c < 3; ++c) {
                    if (!e.comp[c]) continue;
                    cplx s = 0.0;
                    for (int i = 0; i < n2; ++i) s += std::conj(r[i]) * e.mu[c][i];
                    Pbox[c][e.cellP[q]] += e.na * std::real(s);
                }
            }
        if (e.outputPol)
            for (int c = 0; c < 3; ++c)
                if (e.comp[c]) totP[c].push_back(std::accumulate(Pbox[c].begin(), Pbox[c].end(), 0.0));
        for (std::size_t d = 0; d < e.dtcLevs.size(); ++d) {
            if (tstep % e.dtcTimeInt == 0) allPop[d].push_back(curPop[d] / static_cast<double>(e.nPoints));
            curPop[d] = 0.0;
        }
        ++tstep;
    }
};

// TFSF surface: the 1-D incident lines stepped with complex arithmetic, and the surface
// corrections (parallelTFSFBase::updateFields / step, SOURCE/parallelTFSF.hpp:1058-1186;
// updateIncdFieldJ/K/JK, incdD2U, fillPulseVec, addIncdFields, SOURCE/parallelTFSF.cpp:11-94;
// IncdCPML addPsi / updatePsiField, PML/PML.cpp:12-31).
struct TfsfSim {
    const TfsfPlan& T;
    std::vector<cplx> U[6], Dl[6], pul[6];  // incident field, its D / B, pulse grid
    std::vector<std::vector<cplx>> P[6], Pprev[6];  // pole polarisations of a line in layered material
    std::vector<std::vector<cplx>> psi[6], psiPul[6];
    std::vector<cplx> pulseVec;
    double tStep = 0.0;

    explicit TfsfSim(const TfsfPlan& t) : T(t) {
        for (int c = 0; c < 6; ++c) {
            const TfsfLine& L = T.line[c];
            if (!L.present) continue;
            U[c].assign(T.gridLen, 0.0);
            Dl[c].assign(T.gridLen, 0.0);
            pul[c].assign(T.pulseLen, 0.0);
            P[c].assign(static_cast<std::size_t>(L.nPole), std::vector<cplx>(T.gridLen, 0.0));
            Pprev[c] = P[c];
            for (auto& p : L.pml) psi[c].emplace_back(p.n, 0.0);
            for (auto& p : L.pmlPulse) psiPul[c].emplace_back(p.n, 0.0);
        }
        pulseVec.assign(T.mTot, 0.0);
    }

    cplx rec(int c, bool off) const { return T.line[c].present ? pul[c][off ? T.line[c].recOffIdx : T.line[c].recIdx] : cplx(0.0); }

    void addSurface(const TfsfAdds& a, std::vector<double>* F, std::vector<double>* Dd) const {
        const std::vector<cplx>* lines = U;
        for (std::size_t c = 0; c < a.cells(); ++c)
            for (long long q = a.start[c]; q < a.start[c + 1]; ++q) {
                double x = std::real(lines[a.line[q]][a.incd[q]]);
                if (a.div[q] >= 0) x = x / T.line[a.div[q]].epMu[a.incd[q]];
                const double v = a.pref[q] * x;
                if (a.toD[q]) Dd[a.comp[c]][a.cell[c]] += v;
                else F[a.comp[c]][a.cell[c]] += v;
            }
    }

    // updateIncdField*: pulse, curl runs, then the line's CPML
    void updateLine(int c, std::vector<cplx>& G, const std::vector<TfsfRun>& runs, const std::vector<TfsfPsi>& pml,
                    std::vector<std::vector<cplx>>& ps, const std::vector<cplx>* nbr) {
        const TfsfLine& L = T.line[c];
        for (int r = 0; r < T.mTot; ++r) G[T.pulAddStart + r] = G[T.pulAddStart + r] + L.prefact * pulseVec[r];
        for (const TfsfRun& run : runs) {
            if (L.useJ) {
                const std::vector<cplx>& J = nbr[L.nbrJ];
                for (int r = 0; r < run.n; ++r) G[run.indI + r] += cplx(run.pj, 0.0) * J[run.posK + r];
                for (int r = 0; r < run.n; ++r) G[run.indI + r] += cplx(-1.0 * run.pj, 0.0) * J[run.negK + r];
            }
            if (L.useK) {
                const std::vector<cplx>& K = nbr[L.nbrK];
                for (int r = 0; r < run.n; ++r) G[run.indI + r] += cplx(run.pk, 0.0) * K[run.posJ + r];
                for (int r = 0; r < run.n; ++r) G[run.indI + r] += cplx(-1.0 * run.pk, 0.0) * K[run.negJ + r];
            }
        }
        for (std::size_t q = 0; q < pml.size(); ++q) {
            const TfsfPsi& p = pml[q];
            std::vector<cplx>& s = ps[q];
            const std::vector<cplx>& N = nbr[p.nbr];
            for (int dd = 0; dd < p.n; ++dd) s[dd] = cplx(p.b[dd]) * s[dd];
            for (int dd = 0; dd < p.n; ++dd) s[dd] = s[dd] + cplx(p.c[dd]) * N[p.loc + dd];
            for (int dd = 0; dd < p.n; ++dd) s[dd] = s[dd] + cplx(p.cOff[dd]) * N[p.locOff + dd];
            for (int dd = 0; dd < p.n; ++dd) G[p.gridLoc + dd] += cplx(p.Db, 0.0) * s[dd];
        }
    }

    void fillPulse(int c) {
        const TfsfLine& L = T.line[c];
        for (int r = 0; r < T.mTot; ++r) pulseVec[r] = 0.0;
        for (const PulseSpec& p : T.pulses)
            for (int r = 0; r < T.mTot; ++r) pulseVec[r] = pulseVec[r] + p.value(tStep * T.dt - L.dist[r]);
    }

    // updateIncdPols (SOURCE/parallelTFSF.cpp:44-58): P = alpha P + xi P_prev + gamma U
    // from the line before this step; elements past an object's poles have zero constants
    void updatePoles(int c) {
        const TfsfLine& L = T.line[c];
        const std::size_t len = static_cast<std::size_t>(T.gridLen);
        for (int p = 0; p < L.nPole; ++p)
            for (std::size_t x = 0; x < len; ++x) {
                const cplx old = P[c][p][x];
                cplx v = cplx(L.pa[p * len + x], 0.0) * old;
                v = v + cplx(L.px[p * len + x], 0.0) * Pprev[c][p][x];
                v = v + cplx(L.pg[p * len + x], 0.0) * U[c][x];
                P[c][p][x] = v;
                Pprev[c][p][x] = old;
            }
    }

    // incdD2U (SOURCE/parallelTFSF.cpp:60-68): U = D / eps, then U += -P_p / eps per pole
    void d2u(int c) {
        const TfsfLine& L = T.line[c];
        for (int x = 0; x < T.gridLen; ++x) U[c][x] = Dl[c][x] / L.epMu[x];
        for (int p = 0; p < L.nPole; ++p)
            for (int x = 0; x < T.gridLen; ++x) U[c][x] = U[c][x] + (-1.0 * P[c][p][x]) / L.epMu[x];
    }

    void stepLines() {
        for (int h = 3; h < 6; ++h) {
            if (!T.line[h].present) continue;
            fillPulse(h);
            updateLine(h, Dl[h], T.line[h].runs, T.line[h].pml, psi[h], U);
            updateLine(h, pul[h], T.line[h].pulseRuns, T.line[h].pmlPulse, psiPul[h], pul);
            d2u(h);
        }
        for (int e = 0; e < 3; ++e) {
            if (!T.line[e].present) continue;
            fillPulse(e);
            updatePoles(e);
            updateLine(e, Dl[e], T.line[e].runs, T.line[e].pml, psi[e], U);
            updateLine(e, pul[e], T.line[e].pulseRuns, T.line[e].pmlPulse, psiPul[e], pul);
            d2u(e);
        }
        tStep += 1.0;
    }
};

struct OracleSim {
    Plan P;
    std::vector<double> F[6];
    std::vector<double> Dd[3];
    std::vector<double> psi[6][2];
    std::vector<std::vector<double>> lorP[3], prevP[3];
    std::vector<std::vector<double>> odP[3], odPrev[3];  // oriented-dipole polarisations (cell-centred grid)
    RunRecord rec;
    std::vector<std::unique_ptr<EmitterSim>> qe;
    std::vector<std::unique_ptr<TfsfSim>> tfsf;
    int step = 0;

    explicit OracleSim(const Plan& plan) : P(plan) {
        for (auto& ep : P.emitters) qe.emplace_back(new EmitterSim(ep, P.dims));
        for (auto& tp : P.tfsf) tfsf.emplace_back(new TfsfSim(tp));
        if (!P.tfsf.empty())
            for (int c = 0; c < 3; ++c) {
                rec.incE[c].assign(2 * (static_cast<std::size_t>(P.nSteps) + 1), 0.0);
                rec.incH[c].assign(2 * (static_cast<std::size_t>(P.nSteps) + 1), 0.0);
            }
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
        if (P.ordip.present)
            for (int c = 0; c < 3; ++c)
                for (int p = 0; p < P.ordip.nPoles; ++p) {
                    odP[c].emplace_back(N, 0.0);
                    odPrev[c].emplace_back(N, 0.0);
                }
        rec.detectors.resize(P.detectors.size());
        for (auto& fp : P.fluxes) {
            std::size_t n = static_cast<std::size_t>(fp.npts) * fp.spec.freqList.size();
            rec.fluxRe.emplace_back(n, 0.0);
            rec.fluxIm.emplace_back(n, 0.0);
            rec.fluxSamples.push_back(0);
        }
        for (auto& dp : P.freqDetectors) {
            std::size_t npts = 0;
            for (auto& F : dp.fields) npts += F.cells.size();
            rec.freqRe.emplace_back(npts * dp.spec.freqList.size(), 0.0);
            rec.freqIm.emplace_back(npts * dp.spec.freqList.size(), 0.0);
            rec.freqSamples.push_back(0);
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
        // frequency-domain detectors: parallelDetectorFREQ_Base::output (DTC/parallelDTC_FREQ.hpp:258-264)
        for (std::size_t k = 0; k < P.freqDetectors.size(); ++k) {
            const DetectorPlan& dp = P.freqDetectors[k];
            if (st % dp.timeInt != 0) continue;
            const double tt = P.tcur[st];
            const std::vector<double>& fl = dp.spec.freqList;
            const std::size_t nf = fl.size();
            std::vector<double> cr(nf), ci(nf);
            for (std::size_t f = 0; f < nf; ++f) {
                std::complex<double> e = std::exp(std::complex<double>(0.0, -1.0 * tt * fl[f]));
                cr[f] = e.real();
                ci[f] = e.imag();
            }
            std::size_t off = 0;
            for (const auto& F : dp.fields) {
                const double* src = fieldOf(F.comp);
                for (std::size_t p = 0; p < F.cells.size(); ++p) {
                    const double v = src[F.cells[p]];
                    const std::size_t base = (off + p) * nf;
                    for (std::size_t f = 0; f < nf; ++f) {
                        rec.freqRe[k][base + f] += cr[f] * v;
                        rec.freqIm[k][base + f] += ci[f] * v;
                    }
                }
                off += F.cells.size();
            }
            rec.freqSamples[k] += 1;
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
        const long long off = P.ordip.offA[c];
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < D.cells(); ++i) {
            const ClassInfo& k = cp.classes[cp.code[i]];
            if (k.ordip) {
                // orDipDtoU (FDTD_up_eq.cpp:862-875): P averaged over the two cell-centred points
                double e = Dc[i];
                e *= 1.0 / k.eps;
                for (int p = 0; p < P.ordip.nPoles; ++p) {
                    e += (-0.5 / k.eps) * odP[c][p][i];
                    e += (-0.5 / k.eps) * odP[c][p][i + off];
                }
                E[i] = e;
                continue;
            }
            if (!k.lor) continue;
            double e = Dc[i];
            e *= 1.0 / k.eps;
            for (int p = 0; p < cp.nPoles; ++p) e += (-1.0 / k.eps) * lorP[c][p][i];
            E[i] = e;
        }
    }

    // UpdateLorPolOrDip (FDTD_up_eq.cpp:450-521): per pole, P = alpha P + xi P_prev
    // + gamma d (d . <E>), where <E> averages each E component over the cell-centred
    // point and the point one cell below along that component.
    void orDipPolarisation() {
        const OrDipPlan& od = P.ordip;
        if (!od.present) return;
        const double* Ex = F[0].data();
        const double* Ey = F[1].data();
        const double* Ez = F[2].data();
        const long long ox = od.offA[0], oy = od.offA[1], oz = od.offA[2];
        const int np = od.nPoles;
#pragma omp parallel for schedule(static)
        for (std::size_t j = 0; j < od.cells.size(); ++j) {
            const long long i = od.cells[j];
            const int o = od.obj[j];
            const auto& al = P.alpha[o];
            const auto& xi = P.xi[o];
            const auto& ga = P.gamma[o];
            for (std::size_t pp = 0; pp < al.size(); ++pp) {
                const auto& dv = od.dip[j * np + pp];
                double* Px = &odP[0][pp][i];
                double* Py = &odP[1][pp][i];
                double* Pz = &odP[2][pp][i];
                const double jx = *Px, jy = *Py, jz = *Pz;
                *Px = al[pp] * *Px;
                *Px = *Px + xi[pp] * odPrev[0][pp][i];
                *Py = al[pp] * *Py;
                *Py = *Py + xi[pp] * odPrev[1][pp][i];
                *Pz = al[pp] * *Pz;
                *Pz = *Pz + xi[pp] * odPrev[2][pp][i];
                double dot = dv[0] * Ex[i] / 2.0;
                dot += 1.0 * (dv[0] * Ex[i - ox] / 2.0);
                dot += 1.0 * (dv[1] * Ey[i] / 2.0);
                dot += 1.0 * (dv[1] * Ey[i - oy] / 2.0);
                dot += 1.0 * (dv[2] * Ez[i] / 2.0);
                dot += 1.0 * (dv[2] * Ez[i - oz] / 2.0);
                *Px = *Px + ga[pp] * (dv[0] * dot);
                *Py = *Py + ga[pp] * (dv[1] * dot);
                *Pz = *Pz + ga[pp] * (dv[2] * dot);
                odPrev[0][pp][i] = jx;
                odPrev[1][pp][i] = jy;
                odPrev[2][pp][i] = jz;
            }
        }
    }

    void stepOnce() {
        // H half step (updateH + H CPML)
        for (int c = 3; c < 6; ++c)
            if (P.comp[c].present) curl(c);
        // TFSF after the H update: record H incident, H corrections, 1-D step, E corrections,
        // record E incident (parallelFDTDField.hpp:1237-1255)
        for (auto& t : tfsf) {
            for (int c = 0; c < 3; ++c) {
                rec.incH[c][2 * step + 0] = t->rec(3 + c, false);
                rec.incH[c][2 * step + 1] = t->rec(3 + c, true);
            }
            t->addSurface(t->T.addH, F, Dd);
            t->stepLines();
            t->addSurface(t->T.addE, F, Dd);
            for (int c = 0; c < 3; ++c) {
                rec.incE[c][2 * step + 0] = t->rec(c, false);
                rec.incE[c][2 * step + 1] = t->rec(c, true);
            }
        }
        // soft sources at t_n (after H, before E)
        for (auto& s : P.sources) {
            double v = s.value[static_cast<std::size_t>(step)];
            for (long long id : s.cells) F[s.comp][id] += v;
        }
        // E half step: polarisations from E^n (oriented dipoles first, updatePolE), curl onto E or D, D -> E
        orDipPolarisation();
        for (int c = 0; c < 3; ++c)
            if (P.comp[c].present) polarisation(c);
        for (int c = 0; c < 3; ++c)
            if (P.comp[c].present) curl(c);
        for (int c = 0; c < 3; ++c)
            if (P.comp[c].present) d2e(c);
        // emitters after D -> E (parallelFDTDField.hpp:1282-1283)
        for (auto& q : qe) q->step(F, P.epsP);
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
        write_freq_detectors(s->P, s->rec, out_dir ? out_dir : "");
        s->rec.emitterP.clear();
        s->rec.emitterPop.clear();
        for (auto& q : s->qe) {
            s->rec.emitterP.push_back(q->totP);
            s->rec.emitterPop.push_back(q->allPop);
        }
        write_emitters(s->P, s->rec, out_dir ? out_dir : "");
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
