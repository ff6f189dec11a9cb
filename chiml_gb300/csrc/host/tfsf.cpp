// TFSF plane-wave surfaces: the set-up of parallelTFSFBase (SOURCE/parallelTFSF.hpp:117-1050)
// and of its 1-D CPMLs (IncdCPML, PML/PML.hpp:37-348) restated for one process on the
// local grid. The plan holds index runs and coefficients; stepping is done by the
// engine (device) and the oracle (host) from the same plan.
//
// Supported: any non-negative integer propagation vector m (normal and oblique
// incidence, 2-D and 3-D), linear, circular and elliptical polarisation, surfaces in
// vacuum, in one uniform material, or crossing material layered along a normal
// propagation direction (dielectric and Drude/Lorentz layers: the lines then carry
// per-element eps and poles, and corrections inside dispersive layers go to D).
// Rejected: a negative m component (the reference samples the surface material only on
// the plus surfaces and, for negative m, divides the incident fields by a zero
// permittivity: every output is NaN), and the material layouts the reference itself
// refuses (genEpMu's checks, parallelTFSF.hpp:621-681).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <thread>

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
    const std::vector<Object>& objs;
    TfsfPlan& T;

    bool twoD = false;
    std::array<int, 3> nvec{};  // n_vec of the main grids (halo included; 1 along z in 2-D)
    std::array<int, 3> m{}, sz{}, loc{}, originLoc{};
    int mTot = 0, mMax = 0, gridLen = 0, pmlThick = 0, quadrant = 0, mInd = -1;
    double theta = 0, phi = 0, psi = 0, alpha = 0, phiP = 0, psiP = 0, dr = -1;
    bool present[6] = {false, false, false, false, false, false};
    std::vector<TfsfSegment>* segs = nullptr;  // where genSurface records its rows

    TfsfBuilder(const Inputs& i, const Dims& dd, double dtt, const TfsfSpec& tt, const int* const* ph,
                const std::vector<Object>& ob, TfsfPlan& tp)
        : in(i), D(dd), dt(dtt), d(i.d), t(tt), phys(ph), objs(ob), T(tp) {}

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
        PhaseClock clk0;
        for (int i = 0; i < 3; ++i) initLine(3 + i, false, distH[i], i, (i + 1) % 3, (i + 2) % 3);
        for (int i = 0; i < 3; ++i) initLine(i, true, distE[i], i, (i + 1) % 3, (i + 2) % 3);
        clk0.mark("tfsf-lines");
        // scaleDistVecSpeed (parallelTFSF.hpp:393-411, 697-702): each distance times
        // sqrt(eps mu) of the line's first elements; in 2-D the missing lines are
        // replaced by the ones named there
        auto epAt = [&](int c, int x) { return T.line[c].epMu[static_cast<std::size_t>(x)]; };
        auto scaleDist = [&](int c, int ep, int mu) {
            if (!T.line[c].present) return;
            for (int rr = 0; rr < mTot; ++rr) T.line[c].dist[rr] = std::sqrt(epAt(ep, rr) * epAt(mu, rr)) * T.line[c].dist[rr];
        };
        if (present[0] && present[3]) {
            for (int i = 0; i < 3; ++i) {
                scaleDist(i, i, 3 + i);
                scaleDist(3 + i, i, 3 + i);
            }
        } else if (present[0]) {
            scaleDist(0, 0, 5);
            scaleDist(1, 1, 5);
            scaleDist(5, 0, 5);
        } else {
            scaleDist(3, 2, 3);
            scaleDist(4, 2, 4);
            scaleDist(2, 2, 3);
        }
        // the pulse prefactors are divided by eps (mu) of the line at the recorded point
        // (parallelTFSF.hpp:413-419); a missing line's own value is replaced as there
        const int fo = pmlThick + mMax + 5 * mTot;
        auto epFo = [&](int c, int alt) { return present[c] ? epAt(c, fo) : (present[alt] ? epAt(alt, fo) : 1.0); };
        const cplx psiJ = std::cos(psiP);
        const cplx psiK = std::sin(psiP) * std::exp(cplx(0.0, alpha));
        cplx pH[3], pE[3];
        pH[0] = (psiK * std::sin(phiP) + psiJ * std::cos(theta) * std::cos(phiP)) * dt / (mTot * dr) / epFo(3, 5);
        pH[1] = (-1.0 * psiK * std::cos(phiP) + psiJ * std::cos(theta) * std::sin(phiP)) * dt / (mTot * dr) / epFo(4, 5);
        pH[2] = (-1.0 * psiJ * std::sin(theta)) * dt / (mTot * dr) / epFo(5, 3);
        pE[0] = (psiJ * std::sin(phiP) - psiK * std::cos(theta) * std::cos(phiP)) * dt / (mTot * dr) / epFo(0, 2);
        pE[1] = (-1.0 * psiJ * std::cos(phiP) - psiK * std::cos(theta) * std::sin(phiP)) * dt / (mTot * dr) / epFo(1, 2);
        pE[2] = (psiK * std::sin(theta)) * dt / (mTot * dr) / epFo(2, 0);
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
        {
            std::exception_ptr hErr;
            std::thread hg([&] {
                try {
                    gather(hTerms, T.addH);
                } catch (...) {
                    hErr = std::current_exception();
                }
            });
            gather(eTerms, T.addE);
            hg.join();
            if (hErr) std::rethrow_exception(hErr);
        }
        clk.mark("tfsf-gather");
        // the lines' CPMLs (parallelTFSF.hpp:425-466): vacuum constants on the incident
        // grid; on the pulse grid eps and mu of the lines named there, at element mMax
        const int pulEps[6] = {0, 1, 2, 2, 2, 0}, pulMu[6] = {5, 5, 3, 3, 4, 5};
        for (int c = 0; c < 6; ++c) {
            if (!T.line[c].present) continue;
            T.line[c].pml = incdCPML(c, gridLen, 1.0, 1.0);
            const double ep = present[pulEps[c]] ? epAt(pulEps[c], mMax) : 1.0;
            const double mu = present[pulMu[c]] ? epAt(pulMu[c], mMax) : 1.0;
            T.line[c].pmlPulse = incdCPML(c, T.pulseLen, ep, mu);
        }
    }

    // Object id of main-grid component c at the plane point (x, y, z) in interior
    // coordinates (the halo cell is index 0), as the reference's getPlane* read it
    // (GRID/parallelGrid.hpp:964-1176).
    int planePhys(int c, int x, int y, int z) const {
        const int gx = x + 1, gy = y + 1, gz = twoD ? 0 : z + 1;
        if (gx < 0 || gx >= D.lx || gy < 0 || gy >= D.ly || gz < 0 || gz >= D.lz)
            throw UnsupportedError("TFSF surface plane outside the grid");
        return phys[c][static_cast<std::size_t>(D.idx(gx, gy, gz))];
    }

    // genEpMu (parallelTFSF.hpp:591-694): the incident line of component c takes eps (E)
    // or mu (H, always 1 here) and the object of each element from the plus surfaces of
    // the box, sampled one cell beyond it: a surface parallel to the propagation whose
    // material changes gives one value per slice across the (normal) propagation
    // direction, a uniform one fills the whole line. The reference's three consistency
    // checks are kept with its messages.
    void genEpMu(int c, bool E, const std::array<int, 3>& fieldEnd, std::vector<double>& ep, std::vector<int>& ob) const {
        ep.assign(static_cast<std::size_t>(gridLen), 0.0);
        ob.assign(static_cast<std::size_t>(gridLen), 0);
        const int off = E ? 0 : -1;
        const int fieldOff = pmlThick + mMax + 5 * mTot;
        const int surInds[6] = {2, 2, 1, 1, 0, 0};
        const int locOff[6] = {off, sz[2], off, sz[1], off, sz[0]};
        const int indStart = twoD ? 2 : 0;
        const bool threeD = !twoD;
        for (int ii = indStart; ii < 6; ++ii) {
            const int s = surInds[ii];
            const std::array<int, 2> pLoc = {s != 2 ? loc[(s + 2) % 3] : loc[0], s != 2 ? loc[(s + 1) % 3] : loc[1]};
            const std::array<int, 2> pSz = {s != 2 ? sz[(s + 2) % 3] : sz[0], s != 2 ? sz[(s + 1) % 3] : sz[1]};
            const std::array<int, 2> fSz = {s != 2 ? nvec[(s + 2) % 3] : nvec[0], s != 2 ? nvec[(s + 1) % 3] : nvec[1]};
            if ((pSz[0] <= 1 && (threeD || (pSz[1] <= 1 && (fSz[0] > 3 || fSz[1] > 3)))) ||
                (pSz[1] <= 1 && (threeD || (pSz[0] <= 1 && (fSz[0] > 3 || fSz[1] > 3)))))
                continue;
            if (ii % 2 == 0) continue;  // only the plus surfaces (m has no negative component here)
            // the plane as getPlaneYZ / XZ / XY return it
            std::vector<int> pv(static_cast<std::size_t>(pSz[0]) * pSz[1], 0);
            const int at = loc[s] + locOff[ii];
            for (int v = 0; v < pSz[1]; ++v)
                for (int u = 0; u < pSz[0]; ++u) {
                    int x, y, z;
                    if (s == 0) {  // [z + sz2 y]
                        x = at; y = pLoc[1] + v; z = pLoc[0] + u;
                    } else if (s == 1) {  // [x + sz0 z]
                        x = pLoc[0] + u; y = at; z = pLoc[1] + v;
                    } else {  // [x + sz0 y]
                        x = pLoc[0] + u; y = pLoc[1] + v; z = at;
                    }
                    if (s != 1 && pLoc[1] + v >= nvec[1] - 2) {
                        pv[static_cast<std::size_t>(u + pSz[0] * v)] = 0;  // rows past the grid stay 0
                        continue;
                    }
                    pv[static_cast<std::size_t>(u + pSz[0] * v)] = planePhys(c, x, y, z);
                }
            std::vector<double> ev(pv.size());
            for (std::size_t q = 0; q < pv.size(); ++q) {
                const int pp = pv[q];
                if (pp >= static_cast<int>(objs.size())) throw InputError("TFSF surface samples an unknown object");
                ev[q] = pp > 0 ? (E ? objs[static_cast<std::size_t>(pp)].epsInf : 1.0) : 1.0;
            }
            bool change = false;
            for (int a : pv)
                if (a != pv[0] && a > -1) change = true;
            if (change) {
                if (mInd == -1) throw InputError("Material changes crossing TFSF boundaries only defined for normal incidence.");
                if (mInd == s) throw InputError("Material changes can't occur along surface that is propagating the pulse.");
                int epSz, epStride;
                const bool across = mInd == 0 || (mInd == 2 && s == 0);
                if (across) {
                    epSz = pSz[1];
                    epStride = pSz[0];
                } else {
                    epSz = pSz[0];
                    epStride = 1;
                }
                for (int jj = 0; jj < sz[mInd]; ++jj) {
                    const int row = (jj < sz[mInd] - fieldEnd[mInd]) ? jj : jj - 1;
                    const int ind = across ? row : pSz[0] * row;
                    double asum = 0.0;  // dasum: the absolute values in order
                    for (int q = 0; q < epSz; ++q) asum += std::abs(ev[static_cast<std::size_t>(ind + q * epStride)]);
                    if (std::abs(asum - ev[static_cast<std::size_t>(ind)] * epSz) > 1e-10)
                        throw InputError("1) The material is not consistent across all TFSF surfaces for each slice perpendicular to the propagating direction");
                    const int e = fieldOff + (m[mInd] >= 0 ? jj : sz[mInd] - jj - 1);
                    if (e < 0 || e >= gridLen) throw InputError("TFSF slice outside the incident line");
                    if (ep[static_cast<std::size_t>(e)] == 0) {
                        ep[static_cast<std::size_t>(e)] = ev[static_cast<std::size_t>(ind)];
                        ob[static_cast<std::size_t>(e)] = pv[static_cast<std::size_t>(ind)] > -1 ? pv[static_cast<std::size_t>(ind)] : 0;
                    } else if (ep[static_cast<std::size_t>(e)] != ev[static_cast<std::size_t>(ind)]) {
                        throw InputError("2) The material is not consistent across all TFSF surfaces for each slice perpendicular to the propagating direction");
                    }
                }
                const int last = fieldOff + sz[mInd];
                if (last > gridLen) throw InputError("TFSF slice outside the incident line");
                std::fill(ep.begin(), ep.begin() + fieldOff, ep[static_cast<std::size_t>(fieldOff)]);
                std::fill(ep.begin() + last, ep.end(), ep[static_cast<std::size_t>(last - 1)]);
                std::fill(ob.begin(), ob.begin() + fieldOff, ob[static_cast<std::size_t>(fieldOff)]);
                std::fill(ob.begin() + last, ob.end(), ob[static_cast<std::size_t>(last - 1)]);
            } else if (s != mInd || sz[0] == 1 || sz[1] == 1 || sz[2] == 1) {
                if (ev.empty()) throw InputError("TFSF surface plane without points");
                for (double a : ep)
                    if (a != ev[0] && a != 0.0)
                        throw InputError("3) The material is not consistent across all TFSF surfaces for each slice perpendicular to the propagating direction.");
                std::fill(ep.begin(), ep.end(), ev[0]);
                std::fill(ob.begin(), ob.end(), *std::max_element(pv.begin(), pv.end()));
            }
        }
        for (double a : ep)
            if (a == 0.0)
                throw UnsupportedError("TFSF line without a material (the reference divides its incident field by zero there)");
        for (int o : ob)
            if (o < 0 || o >= static_cast<int>(objs.size())) throw InputError("TFSF line samples an unknown object");
    }

    // ---- initializeIncdFields / genFieldUpParam, parallelTFSF.hpp:500-730 ----
    // Line c (0..2 E, 3..5 H) of component i; j, k the cycled directions.
    void initLine(int c, bool E, int distBase, int i, int j, int k) {
        TfsfLine& L = T.line[c];
        if (!present[c]) return;
        L.present = true;
        std::array<int, 3> fieldEnd = {0, 0, 0};
        if (E) {
            if (sz[i] == nvec[i] - 2) fieldEnd[i] = 1;
        } else {
            if (sz[j] == nvec[j] - 2) fieldEnd[j] = 1;
            if (sz[k] == nvec[k] - 2) fieldEnd[k] = 1;
        }
        L.dist.resize(mTot);
        for (int rr = 0; rr < mTot; ++rr) L.dist[rr] = static_cast<double>(distBase + 2 * rr) / 2.0 * dr;
        genEpMu(c, E, fieldEnd, L.epMu, L.obj);
        // poles of the elements the curl runs cover (genFieldUpParam, updateIncdPols): the
        // electric poles of each element's object; the H lines have none (no magnetic poles)
        L.nPole = 0;
        if (E)
            for (int x = mTot; x < gridLen - mTot; ++x)
                L.nPole = std::max(L.nPole, static_cast<int>(objs[static_cast<std::size_t>(L.obj[static_cast<std::size_t>(x)])].gamma.size()));
        const std::size_t len = static_cast<std::size_t>(gridLen);
        L.pa.assign(static_cast<std::size_t>(L.nPole) * len, 0.0);
        L.px.assign(L.pa.size(), 0.0);
        L.pg.assign(L.pa.size(), 0.0);
        for (int x = mTot; x < gridLen - mTot && L.nPole > 0; ++x) {
            const Object& o = objs[static_cast<std::size_t>(L.obj[static_cast<std::size_t>(x)])];
            for (std::size_t p = 0; p < o.gamma.size(); ++p) {
                L.pa[p * len + static_cast<std::size_t>(x)] = o.alpha[p];
                L.px[p * len + static_cast<std::size_t>(x)] = o.xi[p];
                L.pg[p * len + static_cast<std::size_t>(x)] = o.gamma[p];
            }
        }
        L.epChange = false;
        for (double a : L.epMu)
            if (a != L.epMu[0]) L.epChange = true;
        L.dLine = L.nPole > 0;
        for (double a : L.epMu)
            if (a != 1.0) L.dLine = true;
        if (!E && L.dLine) throw UnsupportedError("TFSF line with a permeability other than 1");
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

    // The curl runs of a line (genFieldUpParam): the reference starts a new run where the
    // element's object changes, with the same offsets and prefactors, so the runs of one
    // line are stepped here as one run over the same elements.
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
            while (ii < len - mTot) ++ii;
            r.n = ii - r.indI;
            out.push_back(r);
        }
        return out;
    }

    // ---- IncdCPML, PML/PML.hpp:117-271 ----
    // epsV, muV: the material constants of both ends (epsPl = epsMn, muPl = muMn here)
    std::vector<TfsfPsi> incdCPML(int c, int gridLenI, double epsV, double muV) const {
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
            out.push_back(upList(c, cor_jj, other + cor_kk, mOffHalf, true, gridLenI - 1 - thick - mTot, thick, epsV, muV));
            out.push_back(upList(c, cor_jj, other + cor_kk, mOffHalf, false, std::abs(mTot), thick, epsV, muV));
        }
        if (gridJ && m[cor_kk] != 0) {
            if (!psiK) throw InputError("TFSF CPML without its auxiliary field");
            out.push_back(upList(c, cor_kk, other + cor_jj, mOffHalf, true, gridLenI - 1 - thick - mTot, thick, epsV, muV));
            out.push_back(upList(c, cor_kk, other + cor_jj, mOffHalf, false, std::abs(mTot), thick, epsV, muV));
        }
        return out;
    }

    // getUpList, PML/PML.hpp:222-271
    TfsfPsi upList(int c, int dir, int nbr, double distOff, bool pl, int startPt, int dirMax, double epsV, double muV) const {
        const bool E = c < 3;
        const int ci = c % 3;
        const int jDir = (ci + 1) % 3;
        TfsfPsi p;
        p.nbr = nbr;
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
        int div;
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
        // the material of the corrected component's own line decides, per run of equal
        // pole count along the row, whether the run goes to D (the object has poles) and,
        // where eps varies along that line, the values are divided by it
        const TfsfLine& Lc = T.line[pol];
        const int div = Lc.epChange ? pol : -1;
        auto lineObj = [&](long long idx) -> const Object& {
            if (idx < 0 || idx >= gridLen) throw UnsupportedError("TFSF surface run reads its line's material outside the line");
            return objs[static_cast<std::size_t>(Lc.obj[static_cast<std::size_t>(idx)])];
        };
        for (int ll = 0; ll < sz1; ++ll) {
            const int base = ir + pmlThick + mOff + 6 * mTot + ll * addIncdProp;
            int s0 = 0;
            while (s0 < sz0Max) {
                const int incdStart = base + s0 * strideIncd;
                const int r0 = s0;
                ++s0;
                // the reference compares the run start with incdStart + s0 * stride, s0
                // counted from the row start (parallelTFSF.hpp:955-957)
                const std::size_t poles0 = lineObj(incdStart).gamma.size();
                while (true) {
                    const Object& o = lineObj(incdStart + static_cast<long long>(s0) * strideIncd);
                    if (!((!E || o.gamma.size() == poles0) && s0 < sz0Max)) break;
                    ++s0;
                }
                const int n = s0 - r0;
                const bool toD = E && !lineObj(incdStart).alpha.empty();
                const long long cell0 =
                    D.idx(locTemp[0] + ll * addVec2[0] + r0 * addVec1[0], locTemp[1] + ll * addVec2[1] + r0 * addVec1[1],
                          locTemp[2] + ll * addVec2[2] + r0 * addVec1[2]);
                if (segs) {
                    TfsfSegment sg;
                    sg.cell0 = cell0;
                    sg.cellStride = cellStride;
                    sg.incd0 = incdStart;
                    sg.incdStride = strideIncd;
                    sg.n = n;
                    sg.line = polIncd;
                    sg.comp = pol;
                    sg.pref = prefactor;
                    sg.toD = toD;
                    sg.div = toD ? -1 : div;
                    segs->push_back(sg);
                }
                for (int r = 0; r < n; ++r) {
                    SurfaceTerm st;
                    st.cell = cell0 + r * cellStride;
                    st.comp = pol;
                    st.line = polIncd;
                    st.incd = incdStart + r * strideIncd;
                    st.pref = prefactor;
                    st.toD = toD;
                    st.div = toD ? -1 : div;
                    if (st.cell < 0 || st.cell >= D.cells() || st.incd < 0 || st.incd >= gridLen)
                        throw InputError("TFSF surface outside the grid");
                    out.push_back(st);
                }
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
    // no result depends on (each cell's sum is its own). The (key, term) pairs are ordered
    // by a least-significant-digit radix sort on the key's bytes: stable, so the terms of
    // a key keep the order they were made in.
    void gather(const std::vector<SurfaceTerm>& terms, TfsfAdds& out) const {
        const std::size_t n = terms.size();
        std::vector<std::pair<long long, long long>> kv(n), tmp(n);  // (key, term index)
        long long maxKey = 0;
        for (std::size_t q = 0; q < n; ++q) {
            kv[q] = {terms[q].comp * D.cells() + terms[q].cell, static_cast<long long>(q)};
            maxKey = std::max(maxKey, kv[q].first);
        }
        for (int shift = 0; shift < 64 && (maxKey >> shift) != 0; shift += 8) {
            std::size_t count[257] = {0};
            for (const auto& e : kv) ++count[((e.first >> shift) & 0xff) + 1];
            for (int b = 0; b < 256; ++b) count[b + 1] += count[b];
            for (const auto& e : kv) tmp[count[(e.first >> shift) & 0xff]++] = e;
            kv.swap(tmp);
        }
        out = TfsfAdds();
        out.line.reserve(n);
        out.incd.reserve(n);
        out.pref.reserve(n);
        out.toD.reserve(n);
        out.div.reserve(n);
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
            out.div.push_back(st.div);
        }
        if (n) out.start.push_back(static_cast<long long>(out.line.size()));
    }
};

}  // namespace

void build_tfsf(const Inputs& in, const Dims& D, double dt, const int* const phys[6],
                const std::vector<Object>& objs, Plan& P) {
    for (const TfsfSpec& t : in.tfsf) {
        // parallelFDTDField.cpp:626-628: a surface with zero x and y size is skipped
        if (t.sz[0] == 0 && t.sz[1] == 0) continue;
        TfsfPlan T;
        TfsfBuilder b(in, D, dt, t, phys, objs, T);
        b.build();
        P.tfsf.push_back(std::move(T));
    }
}

}  // namespace chiml
