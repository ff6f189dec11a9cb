// Emitter plans: the quantum-emitter (Maxwell-Liouville) objects of an input turned into
// the data the time-step loop needs. Restates, for one process:
//   GenerateAllELevCombos          FDTD_MANAGER/parallelFDTDField.cpp:1698-1715
//   Hamiltonian::Hamiltonian       ML/Hamiltonian.cpp:3-47
//   BasisSet::expectationVals      ML/BasisSet.cpp:8-35  (spherical-harmonic integrals, 3j symbols)
//   parallelQEBase ctor, linblad   ML/parallelQE.hpp:262-371 (relaxation superoperator)
//   generateDenLists               ML/parallelQE.hpp:387-470 (box geometry, single process)
#include <algorithm>
#include <cmath>
#include <utility>

#include "plan.hpp"

namespace chiml {

namespace {

double factorial(int n) {
    double f = 1.0;
    for (int i = 2; i <= n; ++i) f *= i;
    return f;
}

}  // namespace

// Wigner 3j symbol (j1 j2 j3; m1 m2 m3) for integer arguments by Racah's formula.
double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
    if (m1 + m2 + m3 != 0) return 0.0;
    if (j1 < 0 || j2 < 0 || j3 < 0) return 0.0;
    if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
    if (j3 > j1 + j2 || j3 < std::abs(j1 - j2)) return 0.0;
    const double tri = factorial(j1 + j2 - j3) * factorial(j1 - j2 + j3) * factorial(-j1 + j2 + j3) /
                       factorial(j1 + j2 + j3 + 1);
    const double pre = std::sqrt(tri * factorial(j1 + m1) * factorial(j1 - m1) * factorial(j2 + m2) *
                                 factorial(j2 - m2) * factorial(j3 + m3) * factorial(j3 - m3));
    const int kmin = std::max(0, std::max(j2 - j3 - m1, j1 - j3 + m2));
    const int kmax = std::min(j1 + j2 - j3, std::min(j1 - m1, j2 + m2));
    double sum = 0.0;
    for (int k = kmin; k <= kmax; ++k) {
        const double den = factorial(k) * factorial(j3 - j2 + k + m1) * factorial(j3 - j1 + k - m2) *
                           factorial(j1 + j2 - j3 - k) * factorial(j1 - k - m1) * factorial(j2 - k + m2);
        sum += ((k % 2) ? -1.0 : 1.0) / den;
    }
    const int ph = j1 - j2 - m3;
    return ((ph % 2 == 0) ? 1.0 : -1.0) * pre * sum;
}

namespace {

// Integral of Y*_{l1 m1} Y_{l2 m2} Y_{l3 m3} over the sphere (BasisSet::sphHarmonicIntegrator, BasisSet.cpp:38-44).
double sph_integral(std::array<int, 2> f1, std::array<int, 2> f2, std::array<int, 2> f3) {
    double s = std::sqrt((f1[0] * 2 + 1) * (f2[0] * 2 + 1) * (f3[0] * 2 + 1) / (4 * M_PI));
    s *= std::pow(-1.0, f1[1]) * wigner3j(f1[0], f2[0], f3[0], 0, 0, 0) * wigner3j(f1[0], f2[0], f3[0], -f1[1], f2[1], f3[1]);
    return s;
}

// Matrix of the position operator along one axis in the (l, m) basis (BasisSet::expectationVals, BasisSet.cpp:8-35).
std::vector<cplx> expectation(const std::vector<std::array<int, 2>>& basis, int axis) {
    const std::array<int, 2> op0 = {1, 0}, op1 = {1, 1}, op2 = {1, -1};
    std::vector<cplx> v;
    const std::size_t n = basis.size();
    for (std::size_t ii = 0; ii < n; ++ii)
        for (std::size_t jj = 0; jj < n; ++jj) {
            if (axis == 0) v.push_back(sph_integral(basis[ii], op2, basis[jj]) - sph_integral(basis[ii], op1, basis[jj]));
            else if (axis == 1) v.push_back(cplx(0, sph_integral(basis[ii], op1, basis[jj]) + sph_integral(basis[ii], op2, basis[jj])));
            else v.push_back(std::sqrt(2) * sph_integral(basis[ii], op0, basis[jj]));
        }
    const cplx s(std::sqrt(2 * M_PI / 3), 0.0);
    for (auto& x : v) x = x * s;
    return v;
}

// C = alpha op(A) op(B) + beta C for square column-major matrices, with the loop order of
// the reference BLAS dgemm (A transposed when ta, B transposed when tb).
void dgemm_sq(bool ta, bool tb, int n, double alpha, const double* A, const double* B, double beta, double* C) {
    auto a = [&](int i, int j) { return A[i + j * n]; };
    auto b = [&](int i, int j) { return B[i + j * n]; };
    if (!ta) {
        for (int j = 0; j < n; ++j) {
            if (beta == 0.0) for (int i = 0; i < n; ++i) C[i + j * n] = 0.0;
            else if (beta != 1.0) for (int i = 0; i < n; ++i) C[i + j * n] *= beta;
            for (int l = 0; l < n; ++l) {
                const double t = alpha * (tb ? b(j, l) : b(l, j));
                for (int i = 0; i < n; ++i) C[i + j * n] += t * a(i, l);
            }
        }
    } else {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                double t = 0.0;
                for (int l = 0; l < n; ++l) t += a(l, i) * (tb ? b(j, l) : b(l, j));
                C[i + j * n] = (beta == 0.0) ? alpha * t : alpha * t + beta * C[i + j * n];
            }
    }
}

// Lindblad term A rho A^T - 1/2 A^T A rho - 1/2 rho A^T A for a real ladder operator
// (parallelQEBase::linblad, parallelQE.hpp:359-371).
std::vector<double> lindblad(const std::vector<double>& A, const std::vector<double>& den, int n) {
    std::vector<double> out(n * n, 0.0), tmp(n * n, 0.0);
    dgemm_sq(true, false, n, 1.0, A.data(), den.data(), 0.0, tmp.data());
    dgemm_sq(false, false, n, 1.0, tmp.data(), A.data(), 0.0, out.data());
    dgemm_sq(true, false, n, 1.0, A.data(), A.data(), 0.0, tmp.data());
    dgemm_sq(false, false, n, -0.5, tmp.data(), den.data(), 1.0, out.data());
    dgemm_sq(false, true, n, 1.0, den.data(), A.data(), 0.0, tmp.data());
    dgemm_sq(false, false, n, -0.5, tmp.data(), A.data(), 1.0, out.data());
    return out;
}

// Every combination of level energies with its weight, level 0 outermost
// (GenerateAllELevCombos, parallelFDTDField.cpp:1698-1715).
void level_combos(const std::vector<EnergyLevel>& levs, std::size_t depth, std::vector<double>& cur, double w,
                  std::vector<std::pair<std::vector<double>, double>>& out) {
    if (depth == levs.size()) {
        out.emplace_back(cur, w);
        return;
    }
    for (std::size_t ii = 0; ii < levs[depth].energyStates.size(); ++ii) {
        for (int ee = 0; ee < levs[depth].levDescribed; ++ee) cur.push_back(levs[depth].energyStates[ii]);
        level_combos(levs, depth + 1, cur, w * levs[depth].weights[ii], out);
        for (int ee = 0; ee < levs[depth].levDescribed; ++ee) cur.pop_back();
    }
}

}  // namespace

// PCG32 (O'Neill's PCG-XSH-RR generator: 64-bit LCG state, 32-bit output), the stream of the
// per-cell dipole draws; uniform() returns a 53-bit double in [0, 1) from two outputs.
class Pcg32 {
public:
    explicit Pcg32(unsigned long long seed, unsigned long long stream = 54u) {
        inc_ = (stream << 1u) | 1u;
        next();
        state_ += seed;
        next();
    }
    uint32_t next() {
        const unsigned long long old = state_;
        state_ = old * 6364136223846793005ULL + inc_;
        const uint32_t xorshifted = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = static_cast<uint32_t>(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    double uniform() {
        const uint32_t a = next() >> 5, b = next() >> 6;
        return (a * 67108864.0 + b) / 9007199254740992.0;
    }

private:
    unsigned long long state_ = 0, inc_ = 1;
};

void build_emitters(const Inputs& in, const Dims& D, double dt, const bool Epresent[3], const double* epsOrDip,
                    Plan& P) {
    for (const EmitterSpec& em : in.emitters) {
        EmitterPlan e;
        const int N = static_cast<int>(em.basis.size());
        e.nlevel = N;
        std::vector<std::pair<std::vector<double>, double>> combos;
        std::vector<double> cur;
        level_combos(in.qeELevs, 0, cur, 1.0, combos);
        if (combos.empty()) throw InputError("an emitter has no energy levels");
        e.nMembers = static_cast<int>(combos.size());
        for (auto& c : combos) {
            if (static_cast<int>(c.first.size()) != N)
                throw InputError("the emitter energy levels describe " + std::to_string(c.first.size()) +
                                 " levels but the basis set has " + std::to_string(N));
            e.h0.insert(e.h0.end(), c.first.begin(), c.first.end());
            e.weight.push_back(c.second);
        }
        for (int ax = 0; ax < 3; ++ax) {
            std::vector<cplx> ex = expectation(em.basis, ax);
            e.mu[ax] = ex;
            e.negMu[ax] = ex;
            for (std::size_t ii = 0; ii < em.couplings.size() && ii < ex.size(); ++ii) {
                e.mu[ax][ii] *= em.couplings[ii];
                e.negMu[ax][ii] *= -1.0 * em.couplings[ii];
            }
            e.addMu[ax] = std::any_of(e.mu[ax].begin(), e.mu[ax].end(), [](cplx v) { return v != 0.0; });
        }
        // relaxation superoperator rows (parallelQE.hpp:231-241 given; 311-355 from channels)
        const int n2 = N * N;
        std::vector<std::vector<double>> gam(n2, std::vector<double>(n2, 0.0));
        if (!em.gam.empty()) {
            gam = em.gam;
        } else {
            for (const RelaxOp& r : em.relax) {
                if (r.n0 < 0 || r.n0 >= N || r.nf < 0 || r.nf >= N) throw InputError("relaxation state outside the basis");
                std::vector<double> A(n2, 0.0), den(n2, 0.0);
                A[r.n0 * N + r.nf] = 1.0;
                auto accumulate = [&](double rate) {
                    den.assign(n2, 0.0);
                    den[0] = 1.0;
                    std::vector<double> l = lindblad(A, den, N);
                    for (int k = 0; k < n2; ++k) gam[0][k] += rate * l[k];
                    for (int ii = 1; ii < n2; ++ii) {
                        den[ii] = 1.0;
                        den[ii - 1] = 0.0;
                        l = lindblad(A, den, N);
                        for (int k = 0; k < n2; ++k) gam[ii][k] += rate * l[k];
                    }
                };
                accumulate(r.rate);
                if (r.dephasing > 0.0) {
                    A[r.n0 * N + r.nf] = 0.0;
                    A[r.n0 * N + r.n0] = std::sqrt(2.0);
                    accumulate(r.dephasing);
                }
            }
        }
        e.gam.assign(gam.size(), {});
        for (std::size_t ii = 0; ii < gam.size(); ++ii)
            for (std::size_t jj = 0; jj < gam[ii].size(); ++jj)
                if (gam[ii][jj] != 0.0) e.gam[ii].emplace_back(static_cast<int>(jj), gam[ii][jj]);
        if (static_cast<int>(e.gam.size()) > n2) throw InputError("relaxation matrix larger than the density matrix");
        for (auto& row : e.gam)
            for (auto& pr : row)
                if (pr.first < 0 || pr.first >= n2) throw InputError("relaxation matrix larger than the density matrix");
        e.dt = dt;
        e.hbar = kHbar * kEps0 * std::pow(kSpeedOfLight, 3) / std::pow(in.a * in.I0, 2.0);
        e.na = em.molDen * std::pow(in.a, 3);
        // coupled components (parallelQE.cpp:15-135)
        e.comp[0] = e.comp[1] = Epresent[0] && Epresent[1];
        if (Epresent[0] != Epresent[1]) throw InputError("If Ex field is in the qe then there must be an Ey film");
        e.comp[2] = Epresent[2];
        e.zOff = (Epresent[0] && Epresent[2]) ? 1 : 0;
        e.gatherZCopy = Epresent[2] && !Epresent[0];
        // box geometry (generateDenLists, parallelQE.hpp:387-470)
        if (em.locs.empty()) throw InputError("an emitter object holds no grid point");
        std::array<int, 3> mn = {1 << 30, 1 << 30, 1 << 30}, mx = {0, 0, 0};
        for (auto& l : em.locs)
            for (int k = 0; k < 3; ++k) {
                mn[k] = std::min(mn[k], l[k]);
                mx[k] = std::max(mx[k], l[k]);
            }
        const bool twoD = (D.lz == 1);
        for (int k = 0; k < 3; ++k) e.nCell[k] = mx[k] - mn[k] + 1;
        if (twoD) e.nCell[2] = 1;
        e.boxBase = {mn[0], mn[1], twoD ? 0 : mn[2]};
        e.pDims = {e.nCell[0] + 2, e.nCell[1] + 2, e.nCell[2] + 1 + e.zOff};
        e.addN = {e.nCell[0] + 1, e.nCell[1] + 1, twoD ? 1 : e.nCell[2] + 1};
        // every grid point the P feedback and the gather touch lies inside the grid
        const int ext[3] = {D.lx, D.ly, D.lz};
        const int touched[3] = {e.addN[0] + 1, e.addN[1] + 1, twoD ? 1 : e.addN[2] + e.zOff};
        for (int k = 0; k < 3; ++k)
            if (e.boxBase[k] < 0 || e.boxBase[k] + touched[k] > ext[k])
                throw InputError("an emitter object reaches the edge of the grid");
        for (auto& l : em.locs) {
            const int x = l[0] - mn[0], y = l[1] - mn[1], z = twoD ? 0 : l[2] - mn[2];
            const int pi = x + 1, pj = y + 1, pk = z + e.zOff;
            e.cellGrid.push_back(D.idx(e.boxBase[0] + pi, e.boxBase[1] + pj, e.boxBase[2] + pk));
            e.cellP.push_back(pi + e.pDims[0] * (pk + e.pDims[2] * pj));
        }
        if (em.cellDipole) {
            // per-cell dipoles (extension): w = scale * direction for every cell, in cell order
            const bool alongZ = !e.addMu[0] && !e.addMu[1] && e.addMu[2];
            if (!alongZ) throw UnsupportedError("per-cell dipoles need an emitter operator along z (basis states with m = 0)");
            if (em.randomDirection && twoD) throw UnsupportedError("random dipole directions need a 3-D grid");
            Pcg32 rng(em.dipoleSeed);
            const double a = em.dipoleScale[0], b = em.dipoleScale[1];
            e.cellDip.reserve(em.locs.size());
            for (std::size_t q = 0; q < em.locs.size(); ++q) {
                std::array<double, 3> w = {0.0, 0.0, 1.0};
                if (em.randomDirection) {
                    // uniform on the sphere: z uniform on (-1, 1], azimuth uniform on [0, 2 pi)
                    const double z = 1.0 - 2.0 * rng.uniform();
                    const double ph = 2.0 * M_PI * rng.uniform();
                    const double r = std::sqrt(std::max(0.0, 1.0 - z * z));
                    w = {r * std::cos(ph), r * std::sin(ph), z};
                }
                if (b > a) {
                    const double sc = a + (b - a) * rng.uniform();
                    for (double& v : w) v *= sc;
                } else {
                    for (double& v : w) v *= a;
                }
                e.cellDip.push_back(w);
            }
            e.addMu = {false, false, true};
        }
        e.nPoints = static_cast<int>(em.locs.size());
        e.outputPol = em.outputPol;
        e.polFile = em.polFile;
        e.dtcLevs = em.dtcLevs;
        e.dtcFiles = em.dtcFiles;
        e.dtcTimeInt = em.dtcTimeInt;
        for (int lv : e.dtcLevs)
            if (lv < 0 || lv >= n2) throw InputError("population detector level outside the density matrix");
        if (e.dtcTimeInt < 1) throw InputError("levDTC_timeInt must be positive");
        P.emitters.push_back(std::move(e));
    }
    if (!P.emitters.empty()) P.epsP.assign(epsOrDip, epsOrDip + D.cells());
}

}  // namespace chiml
