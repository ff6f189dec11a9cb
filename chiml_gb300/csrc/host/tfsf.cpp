// TFSF plane-wave surfaces: the set-up of parallelTFSFBase (SOURCE/parallelTFSF.hpp:117-1050)
// and of its 1-D CPMLs (IncdCPML, PML/PML.hpp:37-348) restated for one process on the
// local grid. The plan holds index runs and coefficients; stepping is done by the
// engine (device) and the oracle (host) from the same plan.
//
// Supported: any non-negative integer propagation vector m (normal and oblique
// incidence, 2-D and 3-D), linear, circular and elliptical polarisation, surfaces in
// vacuum. Rejected: a negative m component (the reference samples the surface material
// only on the plus surfaces and, for negative m, divides the incident fields by a zero
// permittivity: every output is NaN), and surfaces crossing or lying in non-vacuum
// material (the reference's layered-medium path, parallelTFSF.hpp:591-694).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <parallel/algorithm>

#include "plan.hpp"

namespace chiml {
namespace {

enum Dir { DX = 0, DY = 1, DZ = 2 };

struct TfsfBuilder {
    const Inputs& in;
    const Dims& D;
    double dt;
    std::array<double, 3> d;
    const TfsfSpec& t;
    const int* const* phys;
    TfsfPlan& T;

    bool twoD = false;
    std::array<int, 3> nvec{};  // n_vec of the main grids (halo included; 1 along z in 2-D)
    std::array<int, 3> m{}, sz{}, loc{}, originLoc{};
    int mTot = 0, mMax = 0, gridLen = 0, pmlThick = 0, quadrant = 0, mInd = -1;
    double theta = 0, phi = 0, psi = 0, alpha = 0, phiP = 0, psiP = 0, dr = -1;
    bool present[6] = {false, false, false, false, false, false};
    std::vector<TfsfSegment>* segs = nullptr;  // where genSurface records its rows

    TfsfBuilder(const Inputs& i, const Dims& dd, double dtt, const TfsfSpec& tt, const int* const* ph, TfsfPlan& tp)
        : in(i), D(dd), dt(dtt), d(i.d), t(tt), phys(ph), T(tp) {}

    // ---- parallelTFSFBase constructor, parallelTFSF.hpp:179-380 ----
    void build() {
        m = t.m;
        sz = t.sz;
        loc = t.loc;
        theta = t.theta;
        phi = t.phi;
        psi = t.psi;
        for (int c = 0; c < 6; ++c) present[c] = phys[c] != nullptr;
        twoD = D.lz == 1;
        nvec = {D.lx, D.ly, D.lz};
        for (int v : m)
            if (v < 0)
                throw UnsupportedError(
                    "TFSF propagation with a negative m component (the reference's incident fields are NaN there)");
        mTot = std::abs(m[0]) + std::abs(m[1]) + std::abs(m[2]);
        mMax = std::max(*std::max_element(m.begin(), m.end()), std::abs(*std::min_element(m.begin(), m.end())));
        gridLen = 2 * mMax + mTot * (10 + 2 * t.pmlThick + sz[0] + sz[1] + sz[2]);
        pmlThick = t.pmlThick * mTot;
        if ((m[0] == 0 && m[1] == 0) || (m[2] == 0 && m[1] == 0) || (m[0] == 0 && m[2] == 0)) {
            if (m[0] != 0) mInd = 0;
            if (m[1] != 0) mInd = 1;
            if (m[2] != 0) mInd = 2;
        }
        // the surface must be a plane or a box (parallelTFSF.hpp:249-256)
        const int zFieldLx = D.lx, zFieldLy = D.ly;
        if ((!twoD && ((sz[0] <= 1 && sz[1] <= 1) || (sz[0] <= 1 && sz[2] <= 1) || (sz[1] <= 1 && sz[2] <= 1))) ||
            (twoD && sz[0] <= 1 && sz[1] <= 1 && zFieldLx != 3 && zFieldLy != 3))
            throw InputError("TFSF sources are not point/line sources sources");
        if (mTot == 0) throw InputError("The m array must have at least one non-zero number");
        const std::array<double, 3> drTemp = {d[0] * std::cos(phi) * std::sin(theta) / static_cast<double>(m[0]),
                                              d[1] * std::sin(phi) * std::sin(theta) / static_cast<double>(m[1]),
                                              d[2] * std::cos(theta) / static_cast<double>(m[2])};
        for (int ii = 0; ii < 3; ++ii)
            if (m[ii] != 0) dr = drTemp[ii];
        for (int ii = 0; ii < 3; ++ii)
            if (m[ii] != 0 && std::abs(drTemp[ii] - dr) > 1e-13)
                throw InputError("p[ii]*d[ii]/m[ii] must equal dr for all ii in x, y, z");
        originLoc = loc;
        if (phi <= M_PI / 2.0 && phi > 0) {
            quadrant = 1;
        } else if (phi <= M_PI && phi > M_PI / 2.0) {
            quadrant = 2;
            originLoc[0] += sz[0] - 1;
        } else if (phi <= 3 * M_PI / 2.0 && phi > M_PI) {
            quadrant = 3;
            originLoc[1] += sz[1] - 1;
            originLoc[0] += sz[0] - 1;
        } else if ((phi <= 2 * M_PI && phi > 3.0 * M_PI / 2.0) || phi == 0) {
            quadrant = 4;
            originLoc[1] += sz[1] - 1;
        }
        if (theta > M_PI / 2.0 || theta < 0.0) {
            quadrant *= -1;
            originLoc[2] += sz[2] - 1;
        }
        if (sz[1] == 1 && m[0] != 0 && m[2] != 0)
            throw InputError("Angle of propgation has a component along the TFSF surface without any other surfaces to cancel it.");
        else if (sz[0] == 1 && m[2] != 0 && m[1] != 0)
            throw InputError("Angle of propgation has a component along the TFSF surface without any other surfaces to cancel it.");
        else if (sz[2] == 1 && !twoD && m[0] != 0 && m[1] != 0)
            throw InputError("Angle of propgation has a component along the TFSF surface without any other surfaces to cancel it.");
        phiP = phi;
        psiP = psi;
        if (theta == 0 || theta == M_PI) phiP = M_PI / 2.0;
        if (t.circPol == Pol::R || t.circPol == Pol::L) {
            const double c = std::pow(t.kRatio, 2.0);
            psiP = 0.5 * std::asin(std::sqrt((std::pow(std::cos(2 * psi), 2) * 4 * c + std::pow((1 + c) * std::sin(2 * psi), 2.0)) /
                                             std::pow(1.0 + c, 2.0)));
            alpha = std::acos(((c - 1.0) * std::sin(2 * psi)) /
                              std::sqrt(std::pow(std::cos(2.0 * psi), 2.0) * 4.0 * c + std::pow((1.0 + c) * std::sin(2.0 * psi), 2.0)));
            if (std::abs(std::tan(psi)) > 1) psiP = M_PI / 2.0 - psiP;
            if (t.circPol == Pol::R) alpha *= -1.0;
        }
        PhaseClock clk0;
        checkVacuumSurfaces();
        clk0.mark("tfsf-vacuum");

        T.m = m;
        T.mTot = mTot;
        T.mMax = mMax;
        T.gridLen = gridLen;
        T.pmlThick = pmlThick;
        T.pulseLen = 2 * pmlThick + 20 * mTot;
        T.pulAddStart = pmlThick + 3 * mTot;
        T.dt = dt;
        T.pulses = t.pulses;
        // lines: H then E, (i, j, k) cycled (parallelTFSF.hpp:321-327)
        const int distH[3] = {m[1] + m[2], m[0] + m[2], m[0] + m[1]};
        const int distE[3] = {m[0], m[1], m[2]};
        for (int i = 0; i < 3; ++i) initLine(3 + i, false, distH[i], i, (i + 1) % 3, (i + 2) % 3);
        for (int i = 0; i < 3; ++i) initLine(i, true, distE[i], i, (i + 1) % 3, (i + 2) % 3);
        // scaleDistVecSpeed multiplies by sqrt(eps mu) of the line: 1 in vacuum
        const cplx psiJ = std::cos(psiP);
        const cplx psiK = std::sin(psiP) * std::exp(cplx(0.0, alpha));
        const double epMu = 1.0;
        cplx pH[3], pE[3];
        pH[0] = (psiK * std::sin(phiP) + psiJ * std::cos(theta) * std::cos(phiP)) * dt / (mTot * dr) / epMu;
        pH[1] = (-1.0 * psiK * std::cos(phiP) + psiJ * std::cos(theta) * std::sin(phiP)) * dt / (mTot * dr) / epMu;
        pH[2] = (-1.0 * psiJ * std::sin(theta)) * dt / (mTot * dr) / epMu;
        pE[0] = (psiJ * std::sin(phiP) - psiK * std::cos(theta) * std::cos(phiP)) * dt / (mTot * dr) / epMu;
        pE[1] = (-1.0 * psiJ * std::cos(phiP) - psiK * std::cos(theta) * std::sin(phiP)) * dt / (mTot * dr) / epMu;
        pE[2] = (psiK * std::sin(theta)) * dt / (mTot * dr) / epMu;
        for (int i = 0; i < 3; ++i) {
            T.line[3 + i].prefact = pH[i];
            T.line[i].prefact = pE[i];
        }
        // surfaces (parallelTFSF.hpp:332-340)
        const bool pl = (theta == 0 || ((theta == M_PI / 2.0 && std::abs(quadrant) == 4) || std::abs(quadrant) == 1)) ? false : true;
        std::vector<SurfaceTerm> hTerms, eTerms;
        {
            // at most two terms per component and surface cell: room for all of them
            const std::size_t area = 2 * (static_cast<std::size_t>(sz[0]) * sz[1] + static_cast<std::size_t>(sz[1]) * sz[2] +
                                          static_cast<std::size_t>(sz[0]) * sz[2]);
            hTerms.reserve(6 * area);
            eTerms.reserve(6 * area);
        }
        PhaseClock clk;
        segs = &T.segH;
        for (int i = 0; i < 3; ++i) addStructs(3 + i, false, pl, hTerms);
        segs = &T.segE;
        for (int i = 0; i < 3; ++i) addStructs(i, true, pl, eTerms);
        segs = nullptr;
        clk.mark("tfsf-surfaces");
        gather(hTerms, T.addH);
        gather(eTerms, T.addE);
        clk.mark("tfsf-gather");
        // the lines' CPMLs (parallelTFSF.hpp:342-378)
        for (int c = 0; c < 6; ++c) {
            if (!T.line[c].present) continue;
            T.line[c].pml = incdCPML(c, gridLen);
            T.line[c].pmlPulse = incdCPML(c, T.pulseLen);
        }
    }

    // The incident lines take their material from the plus surfaces of the box, sampled
    // one cell beyond the box on each axis (genEpMu, parallelTFSF.hpp:591-694); this build
    // requires vacuum there, where every line is uniform with eps = mu = 1.
    void checkVacuumSurfaces() const {
        const int surInds[6] = {2, 2, 1, 1, 0, 0};
        const int indStart = twoD ? 2 : 0;
        for (int c = 0; c < 6; ++c) {
            if (!phys[c]) continue;
            const int* ph = phys[c];
            for (int ii = indStart; ii < 6; ++ii) {
                if (ii % 2 == 0) continue;  // only the plus surfaces are sampled
                const int s = surInds[ii];
                const int a0 = (s != 2) ? (s + 2) % 3 : 0, a1 = (s != 2) ? (s + 1) % 3 : 1;
                const int pl0 = sz[a0], pl1 = sz[a1];
                const int f0 = nvec[a0], f1 = nvec[a1];
                if ((pl0 <= 1 && (!twoD || (pl1 <= 1 && (f0 > 3 || f1 > 3)))) ||
                    (pl1 <= 1 && (!twoD || (pl0 <= 1 && (f0 > 3 || f1 > 3)))))
                    continue;
                for (int u = 0; u < pl0; ++u)
                    for (int v = 0; v < pl1; ++v) {
                        std::array<int, 3> q = {0, 0, 0};
                        q[s] = loc[s] + sz[s] + 1;
                        q[a0] = loc[a0] + u + 1;
                        q[a1] = loc[a1] + v + 1;
                        if (twoD) q[2] = 0;
                        if (q[0] < 0 || q[0] >= D.lx || q[1] < 0 || q[1] >= D.ly || q[2] < 0 || q[2] >= D.lz) continue;
                        if (ph[static_cast<std::size_t>(D.idx(q[0], q[1], q[2]))] > 0)
                            throw UnsupportedError("TFSF surfaces in non-vacuum material are not supported");
                    }
            }
        }
    }

    // ---- initializeIncdFields / genFieldUpParam, parallelTFSF.hpp:500-730 ----
    // Line c (0..2 E, 3..5 H) of component i; j, k the cycled directions.
    void initLine(int c, bool E, int distBase, int i, int j, int k) {
        TfsfLine& L = T.line[c];
        if (!present[c]) return;
        L.present = true;
        L.epMu = 1.0;
        L.dist.resize(mTot);
        for (int rr = 0; rr < mTot; ++rr) L.dist[rr] = static_cast<double>(distBase + 2 * rr) / 2.0 * dr;
        L.runs = upParams(E, gridLen, i, j, k);
        L.pulseRuns = upParams(E, T.pulseLen, i, j, k);
        // neighbours: the other kind's components j and k
        const int other = E ? 3 : 0;
        L.nbrJ = other + j;
        L.nbrK = other + k;
        L.useJ = present[L.nbrJ];
        L.useK = present[L.nbrK];
        L.recIdx = pmlThick + mMax + 5 * mTot;
        L.recOffIdx = pmlThick + mMax + 5 * mTot - distBase % 2;
    }

    // One run over a uniform line (the material is vacuum everywhere on it).
    std::vector<TfsfRun> upParams(bool E, int len, int i, int j, int k) const {
        (void)i;
        std::vector<TfsfRun> out;
        int ii = mTot;
        while (ii < len - mTot) {
            TfsfRun r;
            r.pj = dt / d[k];
            r.pk = dt / d[j];
            r.indI = ii;
            r.posJ = ii + (E ? m[j] / 2 : -1 * m[j] / 2);
            r.negJ = ii + (E ? -1 * (m[j] + m[j] % 2) / 2 : (m[j] + m[j] % 2) / 2);
            r.posK = ii + (E ? -1 * (m[k] + m[k] % 2) / 2 : (m[k] + m[k] % 2) / 2);
            r.negK = ii + (E ? m[k] / 2 : -1 * m[k] / 2);
            ++ii;
            while (ii < len - mTot) ++ii;  // uniform material: one run
            r.n = ii - r.indI;
            out.push_back(r);
        }
        return out;
    }

    // ---- IncdCPML, PML/PML.hpp:117-271 ----
    std::vector<TfsfPsi> incdCPML(int c, int gridLenI) const {
        const bool E = c < 3;
        const int ci = c % 3;
        const int cor_ii = ci, cor_jj = (ci + 1) % 3, cor_kk = (ci + 2) % 3;
        double mOffHalf = 0.0;
        if (ci == 0) mOffHalf = (!E ? m[1] % 2 + m[2] % 2 : m[0] % 2) / 2.0;
        if (ci == 1) mOffHalf = (!E ? m[2] % 2 + m[0] % 2 : m[1] % 2) / 2.0;
        if (ci == 2) mOffHalf = (!E ? m[0] % 2 + m[1] % 2 : m[2] % 2) / 2.0;
        (void)cor_ii;
        const int other = E ? 3 : 0;
        const bool gridJ = present[other + cor_jj];  // grid_j_ (the line polarised along j)
        const bool gridK = present[other + cor_kk];  // grid_k_
        const bool psiJ = gridK && (nvec[2] != 1 || cor_jj != DZ);
        const bool psiK = gridJ && (nvec[2] != 1 || cor_kk != DZ);
        std::vector<TfsfPsi> out;
        const int thick = pmlThick;
        if (gridK && m[cor_jj] != 0) {
            if (!psiJ) throw InputError("TFSF CPML without its auxiliary field");
            out.push_back(upList(c, cor_jj, other + cor_kk, mOffHalf, true, gridLenI - 1 - thick - mTot, thick));
            out.push_back(upList(c, cor_jj, other + cor_kk, mOffHalf, false, std::abs(mTot), thick));
        }
        if (gridJ && m[cor_kk] != 0) {
            if (!psiK) throw InputError("TFSF CPML without its auxiliary field");
            out.push_back(upList(c, cor_kk, other + cor_jj, mOffHalf, true, gridLenI - 1 - thick - mTot, thick));
            out.push_back(upList(c, cor_kk, other + cor_jj, mOffHalf, false, std::abs(mTot), thick));
        }
        return out;
    }

    // getUpList, PML/PML.hpp:222-271 (eps = mu = 1 on both ends)
    TfsfPsi upList(int c, int dir, int nbr, double distOff, bool pl, int startPt, int dirMax) const {
        const bool E = c < 3;
        const int ci = c % 3;
        const int jDir = (ci + 1) % 3;
        TfsfPsi p;
        p.nbr = nbr;
        const double epsV = 1.0, muV = 1.0;
        p.Db = dt / (d[dir] * (E ? epsV : muV));
        p.gridLoc = startPt;
        p.n = dirMax;
        const int md = m[dir];
        if ((dir == jDir) ^ !E) {
            p.loc = startPt + (E ? (md) / 2 : -1 * (md) / 2);
            p.locOff = startPt + (E ? -1 * (md + md % 2) / 2 : (md + md % 2) / 2);
        } else {
            p.loc = startPt + (E ? -1 * (md + md % 2) / 2 : (md + md % 2) / 2);
            p.locOff = startPt + (E ? (md) / 2 : -1 * (md) / 2);
        }
        const double mExp = t.pmlM, maExp = t.pmlMa, kappaMax = 1.0, aMax = t.pmlAMax;
        const double sigmaMax = 0.8 * (mExp + 1) / std::abs(dr);
        const double iiMax = static_cast<double>(dirMax - 1);
        p.b.assign(dirMax, 0.0);
        p.c.assign(dirMax, 0.0);
        p.cOff.assign(dirMax, 0.0);
        for (int dd = 0; dd < dirMax; ++dd) {
            const double dist = pl ? dirMax - 1 - (static_cast<double>(dd) + distOff) : static_cast<double>(dd) + distOff;
            const bool in = 0.0 <= dist && dist <= iiMax;
            const double sig = in ? sigmaMax / std::sqrt(epsV * muV) * std::pow((iiMax - dist) / iiMax, mExp) : 0.0;
            const double kap = in ? 1.0 + (kappaMax - 1.0) * std::pow((iiMax - dist) / iiMax, mExp) : 1.0;
            const double a = in ? aMax * std::pow((dist) / iiMax, maExp) : 0.0;
            p.b[dd] = std::exp(-1.0 * (sig / kap + a) * dt);
            const double cc = (sig == 0 && a == 0) ? 0 : sig / (sig * kap + std::pow(kap, 2.0) * a) * (std::exp(-1.0 * (sig / kap + a) * dt) - 1.0);
            p.c[dd] = cc;
            p.cOff[dd] = cc;
            if (!E) p.c[dd] *= -1.0;
            else p.cOff[dd] *= -1.0;
        }
        return p;
    }

    // ---- surfaces: initializeIncdAddStructs / genSurface, parallelTFSF.hpp:761-985 ----
    struct SurfaceTerm {
        long long cell;
        int comp, line, incd;
        double pref;
        bool toD;
    };

    void addStructs(int c, bool E, bool pl, std::vector<SurfaceTerm>& out) {
        if (!present[c]) return;
        const int ci = c % 3;
        const int cor_ii = ci, cor_jj = (ci + 1) % 3, cor_kk = (ci + 2) % 3;
        const int other = E ? 3 : 0;
        const int incdJ = other + cor_jj, incdK = other + cor_kk;  // incd_j, incd_k
        const int dirJ = cor_jj, dirK = cor_kk;
        if (sz[cor_ii] > 1 || nvec[cor_ii] <= 3) {
            if (sz[cor_jj] > 1 || nvec[2] == 1) {
                if (present[incdJ]) {
                    genSurface(c, incdJ, dirK, pl, E, out);
                    if (sz[cor_kk] > 1) genSurface(c, incdJ, dirK, !pl, E, out);
                }
            }
            if (sz[cor_kk] > 1 || nvec[2] == 1) {
                if (present[incdK]) {
                    genSurface(c, incdK, dirJ, pl, E, out);
                    if (sz[cor_jj] > 1) genSurface(c, incdK, dirJ, !pl, E, out);
                }
            }
        }
    }

    // polarisation helpers: component ids 0..2 E, 3..5 H
    static bool isX(int c) { return c == 0 || c == 5 || c == 4; }   // EX, HZ, HY
    static bool isY(int c) { return c == 1 || c == 3 || c == 5; }   // EY, HX, HZ
    static bool isZc(int c) { return c == 2 || c == 3 || c == 4; }  // EZ, HX, HY

    void genSurface(int pol, int polIncd, int dir, bool pl, bool E, std::vector<SurfaceTerm>& out) {
        std::array<int, 3> fieldEnd = {0, 0, 0};
        if (isX(pol)) fieldEnd[0] = 1;
        if (isY(pol)) fieldEnd[1] = 1;
        if (nvec[2] != 1 && isZc(pol)) fieldEnd[2] = 1;
        double mOffSet = 0, mOffHalf = 0;
        if (isX(polIncd)) {
            mOffSet += static_cast<double>(m[0]) / 2.0;
            mOffHalf += static_cast<double>(m[0] % 2) / 2.0;
        }
        if (isY(polIncd)) {
            mOffSet += static_cast<double>(m[1]) / 2.0;
            mOffHalf += static_cast<double>(m[1] % 2) / 2.0;
        }
        if (isZc(polIncd)) {
            mOffSet += static_cast<double>(m[2]) / 2.0;
            mOffHalf += static_cast<double>(m[2] % 2) / 2.0;
        }
        bool isJ = true;
        int cor = -1, transCor1 = -1, transCor2 = -1;
        std::array<int, 3> addVec1{}, addVec2{};
        long long strideMain = 0;
        const bool threeD = !twoD;
        if (dir == DX) {
            if (pol == 4 || pol == 1) isJ = false;  // HY, EY
            if (threeD && mInd != 2) {
                cor = 0; transCor1 = 2; transCor2 = 1;
                addVec1 = {0, 0, 1};
                addVec2 = {0, 1, 0};
                strideMain = D.lx;
            } else {
                cor = 0; transCor1 = 1; transCor2 = 2;
                addVec1 = {0, 1, 0};
                addVec2 = {0, 0, 1};
                strideMain = static_cast<long long>(D.lx) * D.lz;
            }
        } else if (dir == DY) {
            if (pol == 5 || pol == 2) isJ = false;  // HZ, EZ
            if (mInd != 0) {
                cor = 1; transCor1 = 0; transCor2 = 2;
                addVec1 = {1, 0, 0};
                addVec2 = {0, 0, 1};
                strideMain = 1;
            } else {
                cor = 1; transCor1 = 2; transCor2 = 0;
                addVec1 = {0, 0, 1};
                addVec2 = {1, 0, 0};
                strideMain = D.lx;
            }
        } else {
            if (pol == 3 || pol == 0) isJ = false;  // HX, EX
            if (mInd != 0) {
                cor = 2; transCor1 = 0; transCor2 = 1;
                addVec1 = {1, 0, 0};
                addVec2 = {0, 1, 0};
                strideMain = 1;
            } else {
                cor = 2; transCor1 = 1; transCor2 = 0;
                addVec1 = {0, 1, 0};
                addVec2 = {1, 0, 0};
                strideMain = static_cast<long long>(D.lx) * D.lz;
            }
        }
        (void)strideMain;
        const double prefactor = (E ^ isJ ^ pl) ? dt / d[cor] : -1.0 * dt / d[cor];
        const int strideIncd = m[transCor1];
        const int addIncdProp = m[transCor2];
        std::array<int, 3> locTemp = loc, szTemp = sz;
        locTemp[cor] = pl ? (loc[cor] + sz[cor] - 1) : (E ? loc[cor] : loc[cor] - 1);
        szTemp[cor] = 1;
        locTemp = surLoc(locTemp, szTemp);
        if (twoD) locTemp[2] = 0;
        if (!(locTemp[0] != -1 && locTemp[1] != -1 && locTemp[2] != -1)) return;
        const int sz0Max = szVal(transCor1, fieldEnd[transCor1], locTemp[transCor1], szTemp);
        int sz1 = szVal(transCor2, fieldEnd[transCor2], locTemp[transCor2], szTemp);
        if (twoD) sz1 = 1;
        std::array<int, 3> locRelOr = locTemp;
        if (!pl && !E) locRelOr[cor] += 1;
        for (int ii = 0; ii < 3; ++ii) locRelOr[ii] = (locRelOr[ii] - 1) - originLoc[ii];
        if (E && m[cor] > 0 && locRelOr[cor] == 0)
            mOffSet -= m[cor];
        else if (E && m[cor] < 0 && -1 * locRelOr[cor] == sz[cor] - 1 && sz[cor] != 1)
            mOffSet -= m[cor];
        const int mOff = static_cast<int>(std::floor(mOffSet - mOffHalf));
        const int ir = std::abs(m[0] * locRelOr[0]) + std::abs(m[1] * locRelOr[1]) + std::abs(m[2] * locRelOr[2]);
        const long long cellStride = addVec1[0] + static_cast<long long>(D.lx) * (addVec1[2] + static_cast<long long>(D.lz) * addVec1[1]);
        for (int ll = 0; ll < sz1; ++ll) {
            // one run per row: the line material is uniform (vacuum), no poles: the U list
            const int incdStart = ir + pmlThick + mOff + 6 * mTot + ll * addIncdProp;
            if (segs && sz0Max > 0) {
                TfsfSegment sg;
                sg.cell0 = D.idx(locTemp[0] + ll * addVec2[0], locTemp[1] + ll * addVec2[1], locTemp[2] + ll * addVec2[2]);
                sg.cellStride = cellStride;
                sg.incd0 = incdStart;
                sg.incdStride = strideIncd;
                sg.n = sz0Max;
                sg.line = polIncd;
                sg.comp = pol;
                sg.pref = prefactor;
                segs->push_back(sg);
            }
            for (int s0 = 0; s0 < sz0Max; ++s0) {
                const int x = locTemp[0] + ll * addVec2[0] + s0 * addVec1[0];
                const int y = locTemp[1] + ll * addVec2[1] + s0 * addVec1[1];
                const int z = locTemp[2] + ll * addVec2[2] + s0 * addVec1[2];
                SurfaceTerm st;
                st.cell = D.idx(x, y, z);
                st.comp = pol;
                st.line = polIncd;
                st.incd = incdStart + s0 * strideIncd;
                st.pref = prefactor;
                st.toD = false;
                if (st.cell < 0 || st.cell >= D.cells() || st.incd < 0 || st.incd >= gridLen)
                    throw InputError("TFSF surface outside the grid");
                out.push_back(st);
            }
        }
    }

    // getSurLoc (one process: procLoc 0, ln_vec = n_vec)
    std::array<int, 3> surLoc(const std::array<int, 3>& l, const std::array<int, 3>& s) const {
        std::array<int, 3> r = {-1, -1, -1};
        for (int ii = 0; ii < 3; ++ii) {
            if (l[ii] >= 0 && l[ii] < nvec[ii] - 2) r[ii] = l[ii] + 1;
            else if (l[ii] < 0 && l[ii] + s[ii] > 0) r[ii] = 1;
        }
        return r;
    }

    // getSzVal
    int szVal(int cor, int fieldEnd, int surLocC, const std::array<int, 3>& s) const {
        if (s[cor] + loc[cor] > nvec[cor] - 2) return nvec[cor] - 2 - surLocC + 1;
        return loc[cor] + s[cor] - (surLocC - 1) - fieldEnd;
    }

    // Terms grouped by main cell (component, cell), each cell's terms in the order they
    // were made (a cell's corrections are summed in that order); cells in key order, which
    // no result depends on (each cell's sum is its own).
    void gather(const std::vector<SurfaceTerm>& terms, TfsfAdds& out) const {
        const std::size_t n = terms.size();
        std::vector<std::pair<long long, long long>> kv(n);  // (key, term index): unique pairs
#pragma omp parallel for schedule(static)
        for (long long q = 0; q < static_cast<long long>(n); ++q)
            kv[static_cast<std::size_t>(q)] = {terms[static_cast<std::size_t>(q)].comp * D.cells() + terms[static_cast<std::size_t>(q)].cell, q};
        __gnu_parallel::sort(kv.begin(), kv.end());
        out = TfsfAdds();
        out.line.reserve(n);
        out.incd.reserve(n);
        out.pref.reserve(n);
        out.toD.reserve(n);
        for (std::size_t p = 0; p < n; ++p) {
            const SurfaceTerm& st = terms[static_cast<std::size_t>(kv[p].second)];
            if (p == 0 || kv[p].first != kv[p - 1].first) {
                if (p != 0) out.start.push_back(static_cast<long long>(out.line.size()));
                out.cell.push_back(st.cell);
                out.comp.push_back(st.comp);
            }
            out.line.push_back(st.line);
            out.incd.push_back(st.incd);
            out.pref.push_back(st.pref);
            out.toD.push_back(st.toD ? 1 : 0);
        }
        if (n) out.start.push_back(static_cast<long long>(out.line.size()));
    }
};

}  // namespace

void build_tfsf(const Inputs& in, const Dims& D, double dt, const int* const phys[6],
                const std::vector<Object>& objs, Plan& P) {
    (void)objs;
    for (const TfsfSpec& t : in.tfsf) {
        // parallelFDTDField.cpp:626-628: a surface with zero x and y size is skipped
        if (t.sz[0] == 0 && t.sz[1] == 0) continue;
        TfsfPlan T;
        TfsfBuilder b(in, D, dt, t, phys, T);
        b.build();
        P.tfsf.push_back(std::move(T));
    }
}

}  // namespace chiml
