// Plan construction: a single-process restatement of the set-up work of chiML's
// field manager (FDTD_MANAGER/parallelFDTDField.hpp:214-1048,
// FDTD_MANAGER/parallelFDTDField.cpp:13-852) and CPML (PML/parallelPML.hpp:102-765).
//
// The reference builds lists of x-runs per update kind; here the same lists are
// generated (for one process: procLoc = 0, rank = size - 1 = 0), accumulated per
// cell, and compressed into the class-code form of plan.hpp. The compressed form
// is then checked cell by cell against the literal accumulation.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <functional>
#include <map>
#include <numeric>
#include <set>
#include <thread>
#include <tuple>
#include <utility>

#include <omp.h>

#include "plan.hpp"

namespace chiml {

bool ClassInfo::operator==(const ClassInfo& o) const {
    return toD == o.toD && lor == o.lor && ordip == o.ordip && obj == o.obj && eps == o.eps &&
           cint[0] == o.cint[0] && cint[1] == o.cint[1] && nplain[0] == o.nplain[0] && nplain[1] == o.nplain[1] &&
           kflag[0] == o.kflag[0] && kflag[1] == o.kflag[1] && npsi[0] == o.npsi[0] && npsi[1] == o.npsi[1] &&
           psiUpd[0] == o.psiUpd[0] && psiUpd[1] == o.psiUpd[1];
}

namespace {

// Host buffers of one value per grid cell: the vector leaves its elements uninitialised
// and filled() writes them in parallel (first touch spread over the threads).
template <typename T>
struct UninitAlloc : std::allocator<T> {
    template <typename U>
    struct rebind {
        typedef UninitAlloc<U> other;
    };
    UninitAlloc() = default;
    template <typename U>
    UninitAlloc(const UninitAlloc<U>&) {}
    template <typename U>
    void construct(U* p) noexcept {
        ::new (static_cast<void*>(p)) U;
    }
    template <typename U, typename... A>
    void construct(U* p, A&&... a) {
        ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
    }
};
template <typename T>
using Buf = std::vector<T, UninitAlloc<T>>;

template <typename T>
Buf<T> filled(std::size_t n, T init, int threads) {
    Buf<T> v(n);
    T* p = v.data();
    const long long m = static_cast<long long>(n);
#pragma omp parallel for schedule(static) num_threads(threads)
    for (long long i = 0; i < m; ++i) p[i] = init;
    return v;
}

template <typename T>
struct Field3 {
    Dims d;
    Buf<T> v;
    Field3() {}
    Field3(const Dims& dd, T init, int threads = 0)
        : d(dd), v(filled<T>(static_cast<std::size_t>(dd.cells()), init, threads > 0 ? threads : omp_get_max_threads())) {}
    T& at(int x, int y, int z) { return v[static_cast<std::size_t>(d.idx(x, y, z))]; }
    T at(int x, int y, int z) const { return v[static_cast<std::size_t>(d.idx(x, y, z))]; }
};

// Polarisation sets used by the CPML list builders: component c in 0..5
// (Ex,Ey,Ez,Hx,Hy,Hz) belongs to a set given as a bit mask.
constexpr int bEX = 1, bEY = 2, bEZ = 4, bHX = 8, bHY = 16, bHZ = 32;
inline bool inSet(int comp, int mask) { return (mask >> comp) & 1; }

// Nested OpenMP teams for the duration of a scope (an outer loop over independent parts,
// each with its own inner team). Both settings are read before either is changed: in
// libgomp omp_set_nested(1) raises max-active-levels to its maximum and omp_set_nested(0)
// drops it to 1, so the switch is set first and the level count after it, and on the way
// out the switch is restored first and the level count last. Older runtimes (a host
// application may bring its own) also gate nesting on the OpenMP 3 switch.
class NestedTeams {
public:
    NestedTeams() {
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wdeprecated-declarations"
        prevNested_ = omp_get_nested();
        prevLevels_ = omp_get_max_active_levels();
        omp_set_nested(1);
#pragma GCC diagnostic pop
        omp_set_max_active_levels(std::max(prevLevels_, 2));
    }
    ~NestedTeams() {
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wdeprecated-declarations"
        omp_set_nested(prevNested_);
#pragma GCC diagnostic pop
        omp_set_max_active_levels(prevLevels_);
    }

private:
    int prevNested_ = 0, prevLevels_ = 1;
};

struct Builder {
    const Inputs& in;
    Plan& P;
    Dims D;
    std::array<int, 3> nvec;        // physical points per axis (n_vec_)
    std::array<double, 3> d;
    double dt;
    std::vector<Object> objs;
    bool matInPML = false;
    // phys (object id) and eps maps per staggered grid: 0..2 E, 3..5 H, 6 POrDip, 7 MOrDip
    Field3<int> phys[8];
    Field3<double> epsRel[8];

    Builder(const Inputs& i, Plan& p) : in(i), P(p) {}

    // Radius of a sphere about o.loc that contains every point isObj accepts
    // (with geo or geoML), or 1e300 when no finite bound is known.
    double boundingRadius(const Object& o) const {
        double r = 0.0;
        switch (o.shape) {
            case Shape::SPHERE: r = std::max(o.geoML[0], o.geo[0]); break;
            case Shape::ELLIPSOID: r = 0.5 * std::max(std::max(std::abs(o.geoML[0]), std::abs(o.geoML[1])), std::abs(o.geoML[2])); break;
            case Shape::BLOCK: r = 0.5 * std::sqrt(o.geoML[0] * o.geoML[0] + o.geoML[1] * o.geoML[1] + o.geoML[2] * o.geoML[2]); break;
            case Shape::CYLINDER: r = std::sqrt(o.geoML[0] * o.geoML[0] + 0.25 * o.geoML[1] * o.geoML[1]); break;
            case Shape::HEMISPHERE: r = std::max(o.geoML[0], o.geo[0]); break;
            case Shape::HEMIELLIPSOID: r = 0.5 * std::max(std::max(std::abs(o.geoML[0]), std::abs(o.geoML[1])), std::abs(o.geoML[2])); break;
            case Shape::ROUNDED_BLOCK: r = 0.5 * std::sqrt(o.geoML[0] * o.geoML[0] + o.geoML[1] * o.geoML[1] + o.geoML[2] * o.geoML[2]); break;
            case Shape::TORUS: r = torusRadius(o); break;
            default: return 1e300;  // cone (unbounded along its axis), prism, tip, paraboloid, tetrahedron
        }
        r += 2.0 * std::max(std::max(d[0], d[1]), d[2]) + 1e-9 * std::abs(r);
        if (!(r < 1e300)) return 1e300;
        if ((o.shape == Shape::ELLIPSOID || o.shape == Shape::HEMIELLIPSOID) && o.geo[2] == 0.0 && D.threeD) return 1e300;
        if (o.shape != Shape::SPHERE)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double dot = 0.0;
                    for (int k = 0; k < 3; ++k) dot += o.coord[a * 3 + k] * o.coord[b * 3 + k];
                    if (!(std::abs(dot - (a == b ? 1.0 : 0.0)) < 1e-9)) return 1e300;
                }
        return r;
    }

    // Radius about o.loc of a torus: (rho - R)^2 <= r^2 - t_z^2 bounds rho by R + r and |t_z| by r.
    static double torusRadius(const Object& o) {
        const double R = std::max(std::abs(o.geo[0]), std::abs(o.geoML[0]));
        const double rc = std::max(std::abs(o.geo[1]), std::abs(o.geoML[1]));
        return std::sqrt((R + rc) * (R + rc) + rc * rc);
    }

    // Half extents h[q] about o.loc, along each grid axis, of every point isObj accepts with
    // geo or geoML (the object's axis box rotated into the grid frame); false when no bound
    // is known (axes that are not orthonormal, unbounded sizes).
    bool objectExtent(const Object& o, std::array<double, 3>& h) const {
        if (o.shape != Shape::SPHERE)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double dot = 0.0;
                    for (int k = 0; k < 3; ++k) dot += o.coord[a * 3 + k] * o.coord[b * 3 + k];
                    if (!(std::abs(dot - (a == b ? 1.0 : 0.0)) < 1e-9)) return false;
                }
        auto g = [&](int i) { return std::max(std::abs(o.geo[i]), std::abs(o.geoML[i])); };
        auto R = [&](int i, int q) { return o.coord[i * 3 + q]; };  // t_i = sum_q R(i, q) (p - loc)_q
        for (int q = 0; q < 3; ++q) {
            switch (o.shape) {
                case Shape::SPHERE: h[q] = std::max(o.geoML[0], o.geo[0]); break;
                case Shape::BLOCK: h[q] = 0.5 * (std::abs(R(0, q)) * g(0) + std::abs(R(1, q)) * g(1) + std::abs(R(2, q)) * g(2)); break;
                case Shape::ELLIPSOID:
                    h[q] = 0.5 * std::sqrt(std::pow(R(0, q) * g(0), 2) + std::pow(R(1, q) * g(1), 2) + std::pow(R(2, q) * g(2), 2));
                    break;
                case Shape::CYLINDER:
                    h[q] = 0.5 * std::abs(R(1, q)) * g(1) + g(0) * std::sqrt(R(0, q) * R(0, q) + R(2, q) * R(2, q));
                    break;
                case Shape::HEMISPHERE: h[q] = std::max(o.geoML[0], o.geo[0]); break;
                case Shape::ROUNDED_BLOCK: h[q] = 0.5 * (std::abs(R(0, q)) * g(0) + std::abs(R(1, q)) * g(1) + std::abs(R(2, q)) * g(2)); break;
                case Shape::HEMIELLIPSOID:
                    h[q] = 0.5 * std::sqrt(std::pow(R(0, q) * g(0), 2) + std::pow(R(1, q) * g(1), 2) + std::pow(R(2, q) * g(2), 2));
                    break;
                case Shape::TORUS: h[q] = torusRadius(o); break;
                default: return false;  // no bound kept: the whole grid is scanned
            }
            if (!(h[q] < 1e300)) return false;
        }
        return true;
    }

    // Objects of constant mu. Inside the interior regions the reference puts their H cells
    // on the U lists with the coefficient dt / (mu d) (fillBlasLists and populateUpLists,
    // parallelFDTDField.hpp:628-644, 751-780), which the material map above gives. Three
    // layouts take other paths there and are refused here, conservatively: mu reaching the
    // CPML (magMatInPML_ moves the H-side CPML onto B, parallelFDTDField.cpp:60-66), TFSF
    // surfaces (their H lines and surface terms would carry mu), and emitter objects.
    void checkMagnetic() const {
        for (std::size_t oo = 1; oo < objs.size(); ++oo) {
            const Object& o = objs[oo];
            if (o.muInf == 1.0) continue;
            if (!(o.muInf > 0.0)) throw InputError("an object's mu must be positive");
            if (o.ML) throw UnsupportedError("emitter objects with mu != 1 are not supported");
            if (!in.tfsf.empty()) throw UnsupportedError("TFSF surfaces with magnetic materials (mu != 1) are not supported");
            // per axis: the object's half extent (unbounded along an axis without a CPML, such
            // as z in 2-D, is fine) grown by two cells must stay inside the interior
            std::array<double, 3> h = {HUGE_VAL, HUGE_VAL, HUGE_VAL};  // unknown: unbounded
            objectExtent(o, h);
            for (int q = 0; q < 3; ++q) {
                const int t = in.pmlThickness[q];
                if (t <= 0 || nvec[q] <= 1 || d[q] <= 0) continue;
                const double inner = (nvec[q] / 2.0 - t) * d[q];  // distance of the CPML from the centre
                // the extent along the axis, else the bounding radius of the CPML scan
                const double hq = (h[q] < 1e300) ? h[q] : boundingRadius(o);
                const double reach = std::abs(o.loc[q]) + hq + 2.0 * d[q];
                if (!(hq < 1e300) || !(reach < inner))
                    throw UnsupportedError("magnetic materials (mu != 1) reaching the CPML are not supported");
            }
        }
    }

    // Index range [lo, hi) per axis that contains every cell whose sample point can
    // lie inside the object (isObj is only ever true within the object's extent).
    void objectIndexBox(const Object& o, std::array<double, 3> offPt, int lo[3], int hi[3]) const {
        std::array<double, 3> h;
        const bool bounded = objectExtent(o, h);
        for (int q = 0; q < 3; ++q) {
            if (d[q] <= 0 || !bounded) {
                lo[q] = -1;
                hi[q] = 1 << 30;
                continue;
            }
            const double pad = 2.0 * d[q] + 1e-9 * std::abs(h[q]);
            const double c0 = (nvec[q] - nvec[q] % 2) / 2.0 - offPt[q] + 1.0;  // index of the origin
            lo[q] = static_cast<int>(std::floor((o.loc[q] - h[q] - pad) / d[q] + c0)) - 1;
            hi[q] = static_cast<int>(std::ceil((o.loc[q] + h[q] + pad) / d[q] + c0)) + 2;
        }
    }

    // Narrows [a, b) to the x indices of one row (y, z fixed) that can lie in a sphere or
    // an ellipsoid: the row meets the shape grown by two cells on every semi-axis in an
    // interval of x found from a quadratic; cells farther out cannot pass isObj. Other
    // shapes keep the range (their bounding box only).
    void rowRange(const Object& o, const std::array<double, 3>& offPt, double py, double pz, int& a, int& b) const {
        if (o.shape != Shape::SPHERE && o.shape != Shape::ELLIPSOID) return;
        const double grow = 2.0 * std::max(std::max(d[0], d[1]), d[2]);
        double semi[3];
        int dims = 3;
        std::array<double, 9> R = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        if (o.shape == Shape::SPHERE) {
            const double r = std::max(o.geo[0], o.geoML[0]);
            semi[0] = semi[1] = semi[2] = r;
        } else {
            for (int i = 0; i < 3; ++i) semi[i] = 0.5 * std::max(std::abs(o.geo[i]), std::abs(o.geoML[i]));
            if (o.geo[2] == 0.0 || o.geoML[2] == 0.0) dims = 2;  // the test sums two terms
            R = o.coord;
        }
        // x of index ii: (ii + c) d0; t_i = R_i0 (x - loc0) + R_i1 (py - loc1) + R_i2 (pz - loc2)
        const double c = -1.0 + offPt[0] - (nvec[0] - nvec[0] % 2) / 2.0;
        double A = 0.0, B = 0.0, C = -1.0;
        for (int i = 0; i < dims; ++i) {
            const double s = semi[i] + grow + 1e-9 * semi[i];
            const double u = R[i * 3 + 0] / s;
            const double v = (R[i * 3 + 1] * (py - o.loc[1]) + R[i * 3 + 2] * (pz - o.loc[2]) - R[i * 3 + 0] * o.loc[0]) / s;
            A += u * u;
            B += 2.0 * u * v;
            C += v * v;
        }
        if (!(A > 1e-30)) return;  // x does not enter the test: keep the range
        const double disc = B * B - 4.0 * A * C;
        if (disc < 0.0) {
            b = a;  // the grown shape misses the row
            return;
        }
        const double r0 = (-B - std::sqrt(disc)) / (2.0 * A), r1 = (-B + std::sqrt(disc)) / (2.0 * A);
        // r0 <= x <= r1 (x in length units), as indices with one more cell of slack
        const double lo = std::floor(r0 / d[0] - c) - 1.0, hi = std::ceil(r1 / d[0] - c) + 2.0;
        if (lo > a) a = static_cast<int>(std::min(lo, static_cast<double>(b)));
        if (hi < b) b = static_cast<int>(std::max(hi, static_cast<double>(a)));
    }

    // setupPhysFields, parallelFDTDField.hpp:867-947
    void setupPhys(int g, bool E, std::array<double, 3> offPt, std::array<int, 3> endOff, int threads) {
        PhaseClock clk;
        Field3<int> ph(D, 0, threads);
        Field3<double> ep(D, 1.0, threads);
        clk.mark("mat-fill");
        const bool twoD = (D.lz == 1);
        int zmin = twoD ? 0 : 1;
        int zmax = twoD ? 1 : D.lz - 1;
        for (std::size_t oo = 1; oo < objs.size(); ++oo) {
            const Object& o = objs[oo];
            // the H grids also take objects of constant mu (parallelFDTDField.hpp:880-894); on
            // the E grids such an object is vacuum (eps 1, the same U-list coefficient)
            if (!(o.ML || o.gamma.size() > 0 || o.epsInf != 1.0 || (!E && o.muInf != 1.0))) continue;
            // Cells outside a generous bounding box of the object cannot pass isObj;
            // the box only narrows the loops, the test itself is unchanged.
            int lo[3], hi[3];
            objectIndexBox(o, offPt, lo, hi);
            const int i0 = std::max(1, lo[0]), i1 = std::min(D.lx - 1, hi[0]);
            const int j0 = std::max(1, lo[1]), j1 = std::min(D.ly - 1, hi[1]);
            const int k0 = twoD ? zmin : std::max(zmin, lo[2]), k1 = twoD ? zmax : std::min(zmax, hi[2]);
            // without an emitter buffer both tests are the same test
            const bool sameGeo = o.geoML == o.geo;
            const double epsHere = E ? o.epsInf : o.muInf;
            // Cells are tested in any order: each cell's value comes from the last object
            // that holds it, whatever the order of cells within one object.
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
            for (int jj = j0; jj < j1; ++jj)
                for (int kk = k0; kk < k1; ++kk) {
                    std::array<double, 3> pt;
                    pt[1] = ((jj - 1) + offPt[1] + 0 - (nvec[1] - nvec[1] % 2) / 2.0) * d[1];
                    pt[2] = ((kk - 1) + offPt[2] + 0 - (nvec[2] - nvec[2] % 2) / 2.0) * d[2];
                    int a = i0, b = i1;
                    rowRange(o, offPt, pt[1], pt[2], a, b);
                    for (int ii = a; ii < b; ++ii) {
                        pt[0] = ((ii - 1) + offPt[0] + 0 - (nvec[0] - nvec[0] % 2) / 2.0) * d[0];
                        const bool inML = o.isObj(pt, d[0], o.geoML);
                        if (inML) ph.at(ii, jj, kk) = static_cast<int>(oo);
                        if (sameGeo ? inML : o.isObj(pt, d[0], o.geo)) ep.at(ii, jj, kk) = epsHere;
                    }
                }
        }
        clk.mark("mat-objects");
        zmin = 0;
        zmax = twoD ? 1 : D.lz;
        if (!twoD) {
            for (int ii = 0; ii < D.lx; ++ii)
                for (int jj = 0; jj < D.ly; ++jj) {
                    ph.at(ii, jj, 0) = -1;
                    ph.at(ii, jj, zmax - 1) = -1;
                    if (endOff[2] == 1) {
                        ph.at(ii, jj, zmax - 2) = -1;
                        ep.at(ii, jj, zmax - 2) = 0.0;
                    }
                }
        }
        for (int ii = 0; ii < D.lx; ++ii)
            for (int kk = zmin; kk < zmax; ++kk) {
                ph.at(ii, 0, kk) = -1;
                ph.at(ii, D.ly - 1, kk) = -1;
                if (endOff[1] == 1 && D.ly > 3) {
                    ph.at(ii, D.ly - 2, kk) = -1;
                    ep.at(ii, D.ly - 2, kk) = 0.0;
                }
            }
        for (int kk = zmin; kk < zmax; ++kk)
            for (int jj = 0; jj < D.ly; ++jj) {
                ph.at(0, jj, kk) = -1;
                ph.at(D.lx - 1, jj, kk) = -1;
                if (endOff[0] == 1 && D.lx > 3) {
                    ph.at(D.lx - 2, jj, kk) = -1;
                    ep.at(D.lx - 2, jj, kk) = 0.0;
                }
            }
        phys[g] = std::move(ph);
        epsRel[g] = std::move(ep);
    }

    // Material-in-PML scan, parallelFDTDField.hpp:274-370 (including its loop-bound carry-over)
    void scanPML() {
        for (int pp = 0; pp < 3; ++pp) {
            int ci = pp, cj = (pp + 1) % 3, ck = (pp + 2) % 3;
            std::array<int, 3> mn, mx;
            for (int q = 0; q < 3; ++q) {
                mn[q] = static_cast<int>(-1 * static_cast<double>(nvec[q]) / 2);
                mx[q] = static_cast<int>(static_cast<double>(nvec[q]) / 2);
            }
            mx[ci] = static_cast<int>(in.pmlThickness[ci] - nvec[ci] / 2.0);
            bool carried = false;
            for (std::size_t oo = 0; oo < objs.size(); ++oo) {
                const Object& o = objs[oo];
                if (o.epsInf == 1.0 && o.gamma.size() < 1 && !o.ML) continue;
                bool dielc = !(o.epsInf == 1.0 && o.gamma.size() < 1);
                double rad = boundingRadius(o);
                auto maybeIn = [&](const std::array<double, 3>& pt) {
                    double s2 = 0.0;
                    for (int q = 0; q < 3; ++q) s2 += (pt[q] - o.loc[q]) * (pt[q] - o.loc[q]);
                    return s2 <= rad * rad;
                };
                // one (jj, kk) row of points over ii in [a, b): three staggered points each
                auto row = [&](int jj, int kk, int a, int b) {
                    for (int ii = a; ii < b && !matInPML; ++ii) {
                        std::array<double, 3> pt = {0, 0, 0};
                        pt[ci] = static_cast<double>(ii) * d[ci];
                        pt[cj] = static_cast<double>(jj) * d[cj];
                        pt[ck] = static_cast<double>(kk) * d[ck];
                        pt[0] += d[0] / 2.0;
                        if (!matInPML && maybeIn(pt) && o.isObj(pt, d[0], o.geo)) matInPML = dielc;
                        pt[1] += d[1] / 2.0;
                        pt[0] -= d[0] / 2.0;
                        if (!matInPML && maybeIn(pt) && o.isObj(pt, d[0], o.geo)) matInPML = dielc;
                        pt[2] += d[2] / 2.0;
                        pt[1] -= d[0] / 2.0;
                        if (!matInPML && maybeIn(pt) && o.isObj(pt, d[0], o.geo)) matInPML = dielc;
                    }
                };
                // The reference's loops reset the ii bounds to the plus-side slab in the second
                // pass of the first (jj, kk) iteration and never restore them: the first row's
                // first pass covers the minus-side slab, every later pass the plus side.
                if (mn[cj] >= mx[cj] || mn[ck] >= mx[ck]) continue;
                if (!carried) {
                    row(mn[cj], mn[ck], mn[ci], mx[ci]);
                    mn[ci] = nvec[ci] / 2 - in.pmlThickness[ci];
                    mx[ci] = nvec[ci] / 2;
                    carried = true;
                }
                // points outside the bounding sphere fail maybeIn and points outside the
                // object's extent fail isObj: scan only the index box of both (every
                // staggered point lies within half a cell of its row's point)
                std::array<double, 3> ext;
                const bool bounded = objectExtent(o, ext);
                auto box = [&](int ax, int m0, int m1, int& a, int& b) {
                    a = m0;
                    b = m1;
                    if (!(rad < 1e300) && !bounded) return;
                    const double r = bounded ? std::min(rad, ext[ax]) : rad;
                    const double reach = r + std::max(std::max(d[0], d[1]), d[2]);
                    a = std::max(m0, static_cast<int>(std::floor((o.loc[ax] - reach) / d[ax])) - 1);
                    b = std::min(m1, static_cast<int>(std::ceil((o.loc[ax] + reach) / d[ax])) + 2);
                };
                int ja, jb, ka, kb, ia, ib;
                box(cj, mn[cj], mx[cj], ja, jb);
                box(ck, mn[ck], mx[ck], ka, kb);
                box(ci, mn[ci], mx[ci], ia, ib);
                for (int jj = ja; jj < jb; ++jj)
                    for (int kk = ka; kk < kb; ++kk) row(jj, kk, ia, ib);
            }
        }
    }

    // ---- CPML (parallelPML.hpp) ----
    struct Pml {
        int comp;  // 0..5
        bool E;
        int ax_i, ax_j, ax_k;
        std::array<int, 3> T;          // thickness n_vec_
        std::array<int, 3> lnMn = {0, 0, 0}, lnPl = {0, 0, 0};
        std::vector<double> eta[3][2];  // [axis][pl]
        bool gridJ, gridK, psiJ, psiK;  // grid_j / grid_k exist, psi_j / psi_k exist
    };

    double sigmaMax(int ax) const { return in.pmlSigOptRat * 0.8 * (in.pmlM + 1) / d[ax]; }
    double kappaF(double ii, double iiMax) const {
        return (0.0 <= ii && ii <= iiMax) ? 1.0 + (in.pmlKappaMax - 1.0) * std::pow((iiMax - ii) / iiMax, in.pmlM) : 1.0;
    }
    double aValF(double ii, double iiMax) const {
        return (0.0 <= ii && ii <= iiMax) ? in.pmlAMax * std::pow(ii / iiMax, in.pmlMa) : 0.0;
    }
    double sigmaF(double ii, double iiMax, double eta, double sMax) const {
        return (0.0 <= ii && ii <= iiMax) ? sMax / eta * std::pow((iiMax - ii) / iiMax, in.pmlM) : 0.0;
    }
    double bF(double sig, double a, double kap) const { return std::exp(-1.0 * (sig / kap + a) * dt); }
    double cF(double sig, double a, double kap) const {
        return (sig == 0 && a == 0) ? 0 : sig * (bF(sig, a, kap) - 1.0) / (kap * (sig + kap * a));
    }
    int lnv(int ax) const { return ax == 0 ? D.lx : (ax == 1 ? D.ly : D.lz); }
    // parallelGrid n_vec_ (x, y include the halo; z is 1 in 2-D)
    int gnv(int ax) const { return ax == 0 ? D.lx : (ax == 1 ? D.ly : D.lz); }

    // genEtaEff (parallelPML.hpp:192-275) with the single-process plane getters
    void genEta(Pml& p, int g, int dir, bool pl, std::vector<double>& eta) {
        std::array<int, 3> pst = {D.lx - 2, D.ly - 2, D.lz - 2};
        int c = p.comp;
        if (inSet(c, bEX | bHY | bHZ)) pst[0] -= 1;
        if (inSet(c, bEY | bHX | bHZ)) pst[1] -= 1;
        if (inSet(c, bEZ | bHX | bHY)) pst[2] -= 1;
        if (D.lz == 1) pst[2] = 1;
        std::array<int, 2> psz;
        if (dir == 0) psz = {pst[2], pst[1]};
        else if (dir == 1) psz = {pst[0], pst[2]};
        else psz = {pst[0], pst[1]};
        int mn = pl ? gnv(dir) - 2 - p.T[dir] : 0;
        int mx = pl ? gnv(dir) - 2 : p.T[dir];
        const int zoff = (D.lz != 1) ? 1 : 0;
        const Field3<int>& ph = phys[g];
        // the planes are independent (each one's sum in its own order): computed in
        // parallel, kept in plane order
        std::vector<double> etaOf(static_cast<std::size_t>(std::max(0, mx - mn)), 0.0);
#pragma omp parallel for schedule(static) num_threads(innerThreads_)
        for (int ii = mn; ii < mx; ++ii) {
            std::vector<int> plane(static_cast<std::size_t>(std::max(0, psz[0] * psz[1])), 0);
            if (dir == 0) {
                int ySz = (D.ly - 2 > psz[1]) ? psz[1] : D.ly - 2;
                for (int yy = 0; yy < ySz; ++yy)
                    for (int zz = 0; zz < psz[0]; ++zz) plane[zz + yy * psz[0]] = ph.at(ii + 1, yy + 1, zz + zoff);
            } else if (dir == 1) {
                for (int zz = 0; zz < psz[1]; ++zz)
                    for (int x = 0; x < psz[0]; ++x) plane[zz * psz[0] + x] = ph.at(1 + x, ii + 1, zz + zoff);
            } else {
                int ySz = (D.ly - 2 > psz[1]) ? psz[1] : D.ly - 2;
                for (int yy = 0; yy < ySz; ++yy)
                    for (int x = 0; x < psz[0]; ++x) plane[psz[0] * yy + x] = ph.at(1 + x, yy + 1, ii + zoff);
            }
            double eps_sum = 0.0, mu_sum = 0.0;
            for (int val : plane)
                if (val != -1) {
                    eps_sum += objs[val].epsInf / static_cast<double>(plane.size());
                    mu_sum += 1.0 / static_cast<double>(plane.size());
                }
            double etaSum = eps_sum * mu_sum;
            etaOf[static_cast<std::size_t>(ii - mn)] = (etaSum != 0.00) ? etaSum : 0;
        }
        for (double etaVal : etaOf)
            if (static_cast<int>(eta.size()) < p.T[dir] && etaVal != 0.0) eta.push_back(etaVal);
    }

    struct PsiEntry {  // one run of the psi list
        long long ind, indOff;
        int n;
        long long stride;
        double b, c;
        int normCoord;  // coordinate along the normal axis
    };
    struct GridEntry {  // one run of the grid list
        long long ind, indOff;
        int n;
        long long stride;
        double Db, DbField;
        int startDeriv;  // coordinate of the run start along the derivative axis
        int slab;        // slab normal axis
        bool pl;
    };

    // getPsiUpList, parallelPML.hpp:321-451
    void psiList(const Pml& p, int dir, bool pl, int startPt, int nDir, int dirMax, std::vector<PsiEntry>& out) {
        const bool E = p.E;
        const int c = p.comp;
        int transSz2 = 1;
        int cn = -1, t1 = -1, t2 = -1, tr1Off = 0, tr2Off = 0, ccStart = 0;
        long long stride = 0;
        double sMax = sigmaMax(dir);
        const std::vector<double>* eta;
        if (dir == 0) {
            cn = 0;
            t1 = (D.lz == 1) ? 1 : 2;
            t2 = (D.lz == 1) ? 2 : 1;
            stride = D.lx;
            eta = &p.eta[0][pl ? 1 : 0];
            if (inSet(c, bEY | bHX | bHZ)) (D.lz == 1) ? tr1Off = 1 : tr2Off = 1;
            if (inSet(c, bHY | bHX | bEZ)) (D.lz == 1) ? tr2Off = 1 : tr1Off = 1;
            if (inSet(c, bHZ | bHY | bEX)) pl ? ccStart = 1 : dirMax -= 1;
        } else if (dir == 1) {
            cn = 1; t1 = 0; t2 = 2;
            stride = 1;
            eta = &p.eta[1][pl ? 1 : 0];
            if (inSet(c, bEX | bHY | bHZ)) tr1Off = 1;
            if (inSet(c, bHX | bHY | bEZ)) tr2Off = 1;
            if (pl && inSet(c, bHZ | bHX | bEY)) ccStart = 1;
            if (!pl && startPt + dirMax == nDir && inSet(c, bHZ | bHX | bEY)) dirMax -= 1;
        } else {
            cn = 2; t1 = 0; t2 = 1;
            stride = 1;
            eta = &p.eta[2][pl ? 1 : 0];
            if (inSet(c, bEX | bHY | bHZ)) tr1Off = 1;
            if (inSet(c, bHX | bHZ | bEY)) tr2Off = 1;
            if (inSet(c, bHX | bHY | bEZ)) pl ? ccStart = 1 : dirMax -= 1;
        }
        int transSz = lnv(t1) - 2 - tr1Off;
        transSz2 = lnv(t2) - 2 - tr2Off;
        if (D.lz == 1 && t2 == 2) transSz2 = 1;
        double distOff = E ? 0.0 : 0.5;
        std::array<int, 3> loc = {-1, -1, -1};
        loc[t1] = 1;
        for (int cc = ccStart; cc < dirMax; ++cc) {
            loc[cn] = pl ? lnv(cn) - 2 - cc : cc + 1;
            double dist = 0 + (loc[cn] - 1) + distOff;
            if (pl) dist = gnv(cn) - 2 - 1 - dist;
            if (dist < 0 || static_cast<std::size_t>(dist) >= eta->size())
                throw UnsupportedError("CPML eta profile index out of range (the reference aborts here)");
            double sig = sigmaF(dist, static_cast<double>(nDir - 1), eta->at(static_cast<std::size_t>(dist)), sMax);
            double kap = kappaF(dist, static_cast<double>(nDir - 1));
            double a = aValF(dist, static_cast<double>(nDir - 1));
            PsiEntry e;
            e.b = bF(sig, a, kap);
            e.c = cF(sig, a, kap) / d[cn];
            if (!E) e.c *= -1.0;
            e.n = transSz;
            e.stride = stride;
            e.normCoord = loc[cn];
            for (int jj = 0; jj < transSz2; ++jj) {
                loc[t2] = 1 + jj;
                if (D.lz == 1) loc[2] = 0;
                std::array<int, 3> lo = loc;
                lo[cn] += E ? -1 : 1;
                e.ind = D.idx(loc[0], loc[1], loc[2]);
                e.indOff = D.idx(lo[0], lo[1], lo[2]);
                out.push_back(e);
            }
        }
    }

    // getGridUpList, parallelPML.hpp:500-656
    void gridList(const Pml& p, int dir, int derivDir, bool pl, std::vector<GridEntry>& out) {
        const bool E = p.E;
        const int c = p.comp;
        std::array<int, 3> mn = {0, 0, 0}, mx = {0, 0, 0};
        int ci = 0, cj = 0, ck = 0, offii = 0;
        long long stride = 1;
        double Db = dt, DbBase = dt;
        std::array<int, 3> offset = {0, 0, 0};
        if (dir == 0) {
            ci = 0; cj = 1; ck = 2;
            stride = D.lx;
            if (pl && inSet(c, bHZ | bEX | bHY)) offii = -1;
            else if (!pl) offii = 1;
        } else if (dir == 1) {
            ci = 1; cj = 2; ck = 0;
            stride = 1;
            if (pl && inSet(c, bHZ | bHX | bEY)) offii = -1;
            if (!pl) offii = 1;
        } else {
            ci = 2; cj = 0; ck = 1;
            stride = 1;
            if (pl && inSet(c, bEZ | bHX | bHY)) offii = -1;
            else if (!pl) offii = 1;
        }
        int cd = derivDir;
        if (derivDir == 0) {
            if (inSet(c, bHZ | bEY)) Db *= -1.0;
            if (inSet(c, bHY | bEY)) DbBase *= -1.0;
        } else if (derivDir == 1) {
            if (inSet(c, bHX | bEZ)) Db *= -1.0;
            if (inSet(c, bHZ | bEZ)) DbBase *= -1.0;
        } else {
            if (inSet(c, bHY | bEX)) Db *= -1.0;
            if (inSet(c, bHX | bEX)) DbBase *= -1.0;
        }
        DbBase /= d[cd];
        offset[cd] = E ? -1 : 1;
        mn[ci] += pl ? lnv(ci) - p.lnPl[ci] - 1 : 1;
        mx[ci] += offii + (pl ? lnv(ci) - 1 : p.lnMn[ci]);
        mn[cj] = 1;
        mx[cj] = lnv(cj) - 1;
        mn[ck] = 1;
        mx[ck] = lnv(ck) - 1;
        if (dir == p.ax_i) {
            mn[cj] += p.lnMn[cj];
            mx[cj] -= p.lnPl[cj] - ((E || (cj == 1 && false)) ? 0 : 1);
            mn[ck] += p.lnMn[ck];
            mx[ck] -= p.lnPl[ck] - ((E || (ck == 1 && false)) ? 0 : 1);
        } else if (cd != ci) {
            mn[cd] += p.lnMn[cd];
            mx[cd] -= p.lnPl[cd] - ((E || (cd == 1 && false)) ? 0 : 1);
        }
        if (ci != 0 && inSet(c, bHZ | bEX | bHY)) mx[0] -= 1;
        if (ci != 1 && inSet(c, bHZ | bHX | bEY)) mx[1] -= 1;
        if (ci != 2 && D.lz != 1 && inSet(c, bHX | bHY | bEZ)) mx[2] -= 1;
        if (D.lz == 1) {
            mn[2] = 0;
            mx[2] = 1;
        }
        // getAxLists (parallelPML.hpp:462-489)
        std::vector<std::array<int, 5>> ax;
        if (stride == 1) {
            for (int kk = mn[2]; kk < mx[2]; ++kk)
                for (int jj = mn[1]; jj < mx[1]; ++jj) ax.push_back({mn[0], jj, kk, mx[0] - mn[0], 0});
        } else if (D.lz == 1) {
            for (int kk = mn[2]; kk < mx[2]; ++kk)
                for (int ii = mn[0]; ii < mx[0]; ++ii) ax.push_back({ii, mn[1], kk, mx[1] - mn[1], 0});
        } else {
            for (int jj = mn[1]; jj < mx[1]; ++jj)
                for (int ii = mn[0]; ii < mx[0]; ++ii) ax.push_back({ii, jj, mn[2], mx[2] - mn[2], 0});
        }
        double distOff = E ? 0.0 : 0.5;
        for (auto& a : ax) {
            double dist = 0 + a[cd] - 1 + distOff;
            if (pl) dist = gnv(cd) - 2 - 1 - dist;
            double kap = kappaF(dist, static_cast<double>(p.T[cd] - 1));
            GridEntry e;
            e.DbField = DbBase / kap;
            e.Db = Db;
            e.ind = D.idx(a[0], a[1], a[2]);
            e.indOff = D.idx(a[0] + offset[0], a[1] + offset[1], a[2] + offset[2]);
            e.n = a[3];
            e.stride = stride;
            e.startDeriv = a[cd];
            e.slab = dir;
            e.pl = pl;
            out.push_back(e);
        }
    }

    // The CPML of one component: ctor + initalizeLists (parallelPML.hpp:102-182, 669-689)
    void buildPml(int comp, bool gridJ, bool gridK, std::vector<PsiEntry> psi[2], std::vector<GridEntry> grid[2],
                  double dbBase[2], double dbPsi[2], bool hasPsi[2]) {
        Pml p;
        p.comp = comp;
        p.E = comp < 3;
        p.ax_i = comp % 3;
        p.ax_j = (p.ax_i + 1) % 3;
        p.ax_k = (p.ax_i + 2) % 3;
        p.T = in.pmlThickness;
        p.gridJ = gridJ;
        p.gridK = gridK;
        p.psiJ = gridK && (D.lz != 1 || p.ax_j != 2);  // psi_j_ (uses grid_k)
        p.psiK = gridJ && (D.lz != 1 || p.ax_k != 2);  // psi_k_ (uses grid_j)
        if (!p.psiJ && !p.psiK)
            throw InputError("Both PML auxiliary fields are undefined");
        // findLnVecs (single process)
        for (int q = 0; q < 3; ++q) {
            if (q == 2 && D.lz == 1) continue;
            int ln = lnv(q) - 2;
            if (0 < p.T[q]) p.lnMn[q] = (ln < p.T[q]) ? ln : p.T[q];
            if (ln > ln - p.T[q]) p.lnPl[q] = (0 > ln - p.T[q]) ? ln : ln - (ln - p.T[q]);
        }
        int g = comp;
        genEta(p, g, 0, false, p.eta[0][0]);
        genEta(p, g, 0, true, p.eta[0][1]);
        genEta(p, g, 1, false, p.eta[1][0]);
        genEta(p, g, 1, true, p.eta[1][1]);
        if (D.lz != 1) {
            genEta(p, g, 2, false, p.eta[2][0]);
            genEta(p, g, 2, true, p.eta[2][1]);
        }
        // term K: derivative along j_, field grid_k, psi_j ; term J: derivative along k_, field grid_j, psi_k
        auto init = [&](int lnPml, int dir, bool pl, int startPt, int nDir, int dirMax) {
            if (lnPml == 0) return;
            if (gridK) {
                if (dir == p.ax_j && p.psiJ) psiList(p, dir, pl, startPt, nDir, dirMax, psi[1]);
                gridList(p, dir, p.ax_j, pl, grid[1]);
            }
            if (gridJ) {
                if (dir == p.ax_k && p.psiK) psiList(p, dir, pl, startPt, nDir, dirMax, psi[0]);
                gridList(p, dir, p.ax_k, pl, grid[0]);
            }
        };
        init(p.lnMn[0], 0, false, 0, p.T[0], p.lnMn[0]);
        init(p.lnPl[0], 0, true, D.lx - 2, p.T[0], p.lnPl[0]);
        init(p.lnMn[1], 1, false, 0, p.T[1], p.lnMn[1]);
        init(p.lnPl[1], 1, true, D.ly - 2, p.T[1], p.lnPl[1]);
        init(p.lnMn[2], 2, false, 0, p.T[2], p.lnMn[2]);
        init(p.lnPl[2], 2, true, D.lz - 2, p.T[2], p.lnPl[2]);
        hasPsi[0] = p.psiK;
        hasPsi[1] = p.psiJ;
        for (int t = 0; t < 2; ++t) {
            dbBase[t] = 0.0;
            dbPsi[t] = 0.0;
            if (!grid[t].empty()) {
                dbPsi[t] = grid[t][0].Db;
            }
        }
        lnMnOut[comp] = p.lnMn;
        lnPlOut[comp] = p.lnPl;
    }
    std::array<int, 3> lnMnOut[6], lnPlOut[6];
    int innerThreads_ = 1;  // threads of each component's row loops
    std::function<void()> side;  // run concurrently with the component build

    // ---- update lists (parallelFDTDField.hpp:628-856) ----
    enum ListKind { L_NONE = 0, L_U = 1, L_D = 2 };

    void buildComp(int comp) {
        PhaseClock clk;
        CompPlan& cp = P.comp[comp];
        const bool E = comp < 3;
        const int i = comp % 3;
        const int jc = (i + 1) % 3, kc = (i + 2) % 3;
        const int other = E ? 3 : 0;
        const bool gridJ = P.comp[other + jc].present;
        const bool gridK = P.comp[other + kc].present;
        std::array<int, 3> fieldEnd = {0, 0, 0};
        if (E) fieldEnd[i] = 1;
        else {
            fieldEnd = {1, 1, 1};
            fieldEnd[i] = 0;
        }
        const Field3<int>& ph = phys[comp];
        const Field3<double>& ep = epsRel[comp];
        const double dj = d[jc], dk = d[kc];
        const bool twoD = (D.lz == 1);

        // CPML lists for this component
        std::vector<PsiEntry> psi[2];
        std::vector<GridEntry> grid[2];
        double dbBase[2], dbPsi[2];
        bool hasPsi[2] = {false, false};
        buildPml(comp, gridJ, gridK, psi, grid, dbBase, dbPsi, hasPsi);
        clk.mark("comp-pml");
        const std::array<int, 3> lnMn = lnMnOut[comp], lnPl = lnPlOut[comp];

        // initializeList ranges
        std::array<int, 3> mn = {1, 1, twoD ? 0 : 1};
        std::array<int, 3> mx = {D.lx - 1 - fieldEnd[0], D.ly - 1, twoD ? 1 : D.lz - 1 - fieldEnd[2]};
        mx[1] -= fieldEnd[1];

        // per-cell list membership
        const int nt = innerThreads_;
        // one byte per cell: the curl list kind (bits 0-1), the Lorentz list (bit 2) and the
        // oriented-dipole list (bit 3)
        Buf<uint8_t> cellLists = filled<uint8_t>(static_cast<std::size_t>(D.cells()), L_NONE, nt);
        clk.mark("comp-fill");

        // getBlasLists / fillBlasLists: seven regions partition the box [mn, mx) (the slabs
        // of the CPML thickness along y, then z, then x, and the interior); a cell of a slab
        // joins the U lists only when no material reaches into the CPML (incPML), one of the
        // interior always can. Cells of oriented-dipole objects go to that list (bit 3), other
        // cells that cannot join U to the Lorentz list (bit 2); the final fill over
        // [fmn, fmx) sets the curl list kind. One pass over the box applies all eight region
        // loops of the reference (their flags OR'ed where regions overlap).
        bool pmlMat = (E && matInPML);
        int xl = pmlMat ? lnMn[0] : 0, xr = pmlMat ? lnPl[0] : 0;
        if (xr != 0) xr -= fieldEnd[0];
        int yb = pmlMat ? lnMn[1] : 0, yt = pmlMat ? lnPl[1] : 0;
        if (yt != 0) yt -= fieldEnd[1];
        bool threeBoth = D.threeD;
        int zb = (threeBoth && pmlMat) ? lnPl[2] : 0, zf = (threeBoth && pmlMat) ? lnMn[2] : 0;
        if (zf != 0) zf -= fieldEnd[2];
        const bool incPML = !matInPML;
        std::array<int, 3> fmn = mn, fmx = mx;
        fmn[0] += lnMn[0];
        fmx[0] -= lnPl[0];
        if (lnPl[0] != 0) fmx[0] += fieldEnd[0];
        fmn[1] += lnMn[1];
        fmx[1] -= lnPl[1];
        if (lnPl[1] != 0) fmx[1] += fieldEnd[1];
        fmn[2] += lnPl[2];  // lnz_back() returns the plus-side thickness
        fmx[2] -= lnMn[2];  // lnz_front() returns the minus-side thickness
        if (lnMn[2] != 0) fmx[2] += fieldEnd[2];
        // per object: bit 0 an oriented-dipole cell, bit 1 a cell that may join U
        std::vector<uint8_t> objKind(objs.size());
        for (std::size_t o = 0; o < objs.size(); ++o) {
            const Object& ob = objs[o];
            const bool orDipCell = ob.orDip && (E && ob.gamma.size() > 0);
            const bool uAll = (!E) || (E && ob.gamma.size() < 1 && !ob.ML);
            objKind[o] = static_cast<uint8_t>((orDipCell ? 1 : 0) | (uAll ? 2 : 0));
        }
        auto inR = [](int v, int lo, int hi) { return v >= lo && v < hi; };
        const int y0 = std::min(mn[1], fmn[1]), y1 = std::max(mx[1], fmx[1]);
        const int z0 = std::min(mn[2], fmn[2]), z1 = std::max(mx[2], fmx[2]);
        const int x0 = std::min(mn[0], fmn[0]), x1 = std::max(mx[0], fmx[0]);
        int border = 0;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(| : border)
        for (int jj = y0; jj < y1; ++jj)
            for (int kk = z0; kk < z1; ++kk) {
                // the regions this row meets: y and z membership, x ranges
                const bool inY = inR(jj, mn[1], mx[1]), inZ = inR(kk, mn[2], mx[2]);
                const bool yMid = inR(jj, mn[1] + yb, mx[1] - yt), zMid = inR(kk, mn[2] + zb, mx[2] - zf);
                const bool rowSlab = inY && inZ &&
                                     (inR(jj, mn[1], mn[1] + yb) || inR(jj, mx[1] - yt, mx[1]) ||
                                      (yMid && (inR(kk, mn[2], mn[2] + zb) || inR(kk, mx[2] - zf, mx[2]))));
                const bool rowMid = inY && inZ && yMid && zMid;
                const bool rowF = inR(jj, fmn[1], fmx[1]) && inR(kk, fmn[2], fmx[2]);
                if (!rowSlab && !rowMid && !rowF) continue;
                const long long rowBase = D.idx(0, jj, kk);
                const int* const phR = ph.v.data() + rowBase;
                uint8_t* const clR = cellLists.data() + rowBase;
                // the row in segments of constant region membership
                int cut[8] = {x0, x1, mn[0], mn[0] + xl, mx[0] - xr, mx[0], fmn[0], fmx[0]};
                for (int& v : cut) v = std::min(std::max(v, x0), x1);
                std::sort(cut, cut + 8);
                for (int q = 0; q < 7; ++q) {
                    const int sa = cut[q], sb = cut[q + 1];
                    if (sa >= sb) continue;
                    const bool inX = inR(sa, mn[0], mx[0]);
                    const bool slab = inX && (rowSlab || (rowMid && (inR(sa, mn[0], mn[0] + xl) || inR(sa, mx[0] - xr, mx[0]))));
                    const bool mid = inX && rowMid && inR(sa, mn[0] + xl, mx[0] - xr);
                    const bool fin = rowF && inR(sa, fmn[0], fmx[0]);
                    if (!slab && !mid && !fin) continue;
                    // the list byte of each object kind in this segment
                    uint8_t byKind[4];
                    for (int k = 0; k < 4; ++k) {
                        const bool orDipCell = k & 1, uAll = (k & 2) != 0;
                        uint8_t cl = 0;
                        if (slab) cl |= orDipCell ? 8u : ((incPML && uAll) ? 0u : 4u);
                        if (mid) cl |= orDipCell ? 8u : (uAll ? 0u : 4u);
                        if (fin) cl = static_cast<uint8_t>((cl & ~3u) | ((!orDipCell && uAll) ? L_U : L_D));
                        byKind[k] = cl;
                    }
                    for (int ii = sa; ii < sb; ++ii) {
                        const int o = phR[ii];
                        if (o < 0) {
                            border = 1;
                            continue;
                        }
                        clR[ii] = byKind[objKind[static_cast<std::size_t>(o)]];
                    }
                }
            }
        if (border) throw InputError("update list reaches a border cell");
        clk.mark("comp-lists");

        // term geometry: J uses grid_j (derivative along k), K uses grid_k (derivative along j)
        TermPlan* tp = cp.term;
        const int sgn = E ? -1 : 1;
        for (int t = 0; t < 2; ++t) {
            TermPlan& T = tp[t];
            T.present = (t == 0) ? gridJ : gridK;
            T.field = other + ((t == 0) ? jc : kc);
            T.axis = (t == 0) ? kc : jc;
            std::array<int, 3> o = {0, 0, 0};
            o[T.axis] = sgn;
            if (twoD && T.axis == 2) {
                T.present = false;
            }
            T.off = o[0] + static_cast<long long>(D.lx) * (o[2] + static_cast<long long>(D.lz) * o[1]);
            T.hasPsi = hasPsi[t];
            T.dbpsi = dbPsi[t];
            int L = lnv(T.axis);
            T.kprof.assign(L, 0.0);
            T.b.assign(L, 0.0);
            T.cpsi.assign(L, 0.0);
            T.slabUse.assign(L, 0);
        }

        // Per cell and term, one byte of CPML list membership: the number of grid-list
        // entries on the cell (bits 0-1; the reference's npsi count), how many of them come
        // from slabs across the term's axis (bits 2-3), whether one comes from the slab along
        // it (bit 4), whether a psi entry updates the cell (bit 5) and whether any of its
        // grid-list coefficients is nonzero (bit 6). The compressed coefficient of a cell,
        // nplain * db + kflag * kprof[normal coordinate], equals the sum of its entries up
        // to rounding: every transverse entry carries db and the one entry along the axis
        // carries kprof at its coordinate (both checked per entry below), and the entries of
        // one component's term share the sign of (1/kappa - 1), so that their sum is nonzero
        // exactly when one of them is.
        const std::size_t N = static_cast<std::size_t>(D.cells());
        Buf<uint8_t> termBits[2] = {filled<uint8_t>(N, 0, nt), filled<uint8_t>(N, 0, nt)};
        auto coordOf = [&](long long id, int ax) {
            long long x = id % D.lx;
            long long r = id / D.lx;
            long long z = r % D.lz;
            long long y = r / D.lz;
            return static_cast<int>(ax == 0 ? x : (ax == 1 ? y : z));
        };
        // Per-entry checks and the coefficient profiles first (one value per entry, or per
        // step of an entry that runs along the term's axis, at most the slab thickness), then
        // the cell bytes of all entries in parallel: increments and flag bits commute, so the
        // bytes and the errors do not depend on the order (a byte is updated atomically).
        for (int t = 0; t < 2; ++t) {
            TermPlan& T = tp[t];
            uint8_t* tb = termBits[t].data();
            double base = 0.0;
            for (auto& e : grid[t]) {
                // a run moves along one grid axis: its coordinate along T.axis is c0 + q dq
                const int c0 = coordOf(e.ind, T.axis);
                const int dq = e.n > 1 ? coordOf(e.ind + e.stride, T.axis) - c0 : 0;
                if (e.n > 1 && coordOf(e.ind + (e.n - 1) * e.stride, T.axis) != c0 + (e.n - 1) * dq)
                    throw InputError("CPML run does not follow one grid axis");
                if (e.indOff - e.ind != T.off) throw InputError("CPML offset does not match the curl offset");
                const bool along = e.slab == T.axis;
                if (!along && e.n > 0) {
                    if (base == 0.0) base = e.DbField;
                    if (e.DbField != base) throw UnsupportedError("CPML transverse coefficient varies");
                }
                if (along)
                    for (int q = 0; q < (dq == 0 ? std::min(e.n, 1) : e.n); ++q) {
                        const int ac = c0 + q * dq;
                        if (T.kprof[ac] != 0.0 && T.kprof[ac] != e.DbField)
                            throw UnsupportedError("CPML coefficient is not a function of the normal coordinate");
                        T.kprof[ac] = e.DbField;
                        if (T.present) T.slabUse[ac] = 1;
                    }
            }
            T.db = base;
            for (auto& e : psi[t]) {
                if (e.indOff - e.ind != T.off) throw InputError("psi offset does not match the curl offset");
                if (e.n <= 0) continue;
                const int ac = e.normCoord;
                if ((T.b[ac] != 0.0 || T.cpsi[ac] != 0.0) && (T.b[ac] != e.b || T.cpsi[ac] != e.c))
                    throw UnsupportedError("psi coefficients are not a function of the normal coordinate");
                T.b[ac] = e.b;
                T.cpsi[ac] = e.c;
                if (T.present) {
                    const int p0 = coordOf(e.ind, T.axis);
                    const int dp = e.n > 1 ? coordOf(e.ind + e.stride, T.axis) - p0 : 0;
                    for (int q = 0; q < (dp == 0 ? 1 : e.n); ++q) T.slabUse[p0 + q * dp] = 1;
                }
            }
            // 1: more than three entries on a cell; 2: two slabs along the axis overlap;
            // 4: a psi cell updated twice. Each thread owns the cells of one band of y and
            // applies every entry's steps that fall in it (a run moves along one axis: its
            // y is constant or steps by one).
            int fault = 0;
            auto yStep = [&](long long ind, long long stride, int n, int& yFirst) {
                yFirst = coordOf(ind, 1);
                if (n < 2) return 0;
                const int dy = coordOf(ind + stride, 1) - yFirst;
                if (dy < -1 || dy > 1 || coordOf(ind + (n - 1) * stride, 1) != yFirst + (n - 1) * dy)
                    throw InputError("CPML run does not follow one grid axis");
                return dy;
            };
            auto qRange = [](int y0, int dy, int n, int ya, int yb, int& qa, int& qb) {
                if (dy == 0) {
                    qa = 0;
                    qb = (y0 >= ya && y0 < yb) ? n : 0;
                } else if (dy > 0) {
                    qa = std::max(0, ya - y0);
                    qb = std::min(n, yb - y0);
                } else {
                    qa = std::max(0, y0 - yb + 1);
                    qb = std::min(n, y0 - ya + 1);
                }
            };
            std::vector<std::array<int, 2>> gY(grid[t].size()), pY(psi[t].size());
            for (std::size_t q0 = 0; q0 < grid[t].size(); ++q0)
                gY[q0][1] = yStep(grid[t][q0].ind, grid[t][q0].stride, grid[t][q0].n, gY[q0][0]);
            for (std::size_t q0 = 0; q0 < psi[t].size(); ++q0)
                pY[q0][1] = yStep(psi[t][q0].ind, psi[t][q0].stride, psi[t][q0].n, pY[q0][0]);
#pragma omp parallel num_threads(nt) reduction(| : fault)
            {
                const int nth = omp_get_num_threads(), me = omp_get_thread_num();
                const int ya = static_cast<int>(static_cast<long long>(D.ly) * me / nth);
                const int yb = static_cast<int>(static_cast<long long>(D.ly) * (me + 1) / nth);
                for (std::size_t q0 = 0; q0 < grid[t].size(); ++q0) {
                    const auto& e = grid[t][q0];
                    int qa, qb;
                    qRange(gY[q0][0], gY[q0][1], e.n, ya, yb, qa, qb);
                    const bool along = e.slab == T.axis;
                    const uint8_t nz = (e.DbField != 0.0) ? 0x40 : 0;
                    for (int q = qa; q < qb; ++q) {
                        uint8_t& bt = tb[e.ind + q * e.stride];
                        if ((bt & 3u) == 3u) fault |= 1;
                        bt = static_cast<uint8_t>(static_cast<uint8_t>(bt + 1u) | nz);
                        if (along) {
                            if (bt & 0x10u) fault |= 2;
                            bt |= 0x10u;
                        } else {
                            bt = static_cast<uint8_t>(bt + 4u);
                        }
                    }
                }
                for (std::size_t q0 = 0; q0 < psi[t].size(); ++q0) {
                    const auto& e = psi[t][q0];
                    int qa, qb;
                    qRange(pY[q0][0], pY[q0][1], e.n, ya, yb, qa, qb);
                    for (int q = qa; q < qb; ++q) {
                        uint8_t& bt = tb[e.ind + q * e.stride];
                        if (bt & 0x20u) fault |= 4;
                        bt |= 0x20u;
                    }
                }
            }
            if (fault & 1) throw UnsupportedError("more than three CPML entries on one cell");
            if (fault & 2) throw UnsupportedError("overlapping CPML slabs along one axis");
            if (fault & 4) throw UnsupportedError("a psi cell is updated twice");
            if (!T.hasPsi) {
#pragma omp parallel for schedule(static) num_threads(nt)
                for (long long id = 0; id < static_cast<long long>(N); ++id) tb[id] &= static_cast<uint8_t>(~3u);
            }
        }
        clk.mark("comp-terms");
        // build classes: each cell's class (its update terms and coefficients) is looked up
        // by key; class ids are given in order of first appearance in the scan order
        // (y, z, x). Rows of y are scanned in parallel chunks with chunk-local ids, merged
        // in chunk order (which reproduces the scan order's first appearances) and remapped.
        cp.present = true;
        cp.isE = E;
        typedef std::array<double, 16> Key;
        cp.code.assign(N, 0);
        cp.classes.clear();
        std::map<Key, int> index;  // key -> class id
        {
            // class 0: cells no list updates (the halo and staggered borders); the
            // kernels skip them without touching any neighbour
            ClassInfo none;
            cp.classes.push_back(none);
            Key key;
            key.fill(0.0);
            key[4] = 1.0;  // eps as normalised below for non-dispersive classes
            index[key] = 0;
        }
        const int nChunks = std::max(1, std::min(D.ly, 64));
        std::vector<std::vector<std::pair<Key, ClassInfo>>> local(static_cast<std::size_t>(nChunks));
        std::vector<std::exception_ptr> chunkErr(static_cast<std::size_t>(nChunks));
        std::vector<char> chunkAnyD(static_cast<std::size_t>(nChunks), 0);
        auto chunkRows = [&](int ch, int& y0, int& y1) {
            y0 = static_cast<int>(static_cast<long long>(D.ly) * ch / nChunks);
            y1 = static_cast<int>(static_cast<long long>(D.ly) * (ch + 1) / nChunks);
        };
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
        for (int ch = 0; ch < nChunks; ++ch) {
            try {
                int y0, y1;
                chunkRows(ch, y0, y1);
                std::map<Key, int> lindex;
                std::vector<std::pair<Key, ClassInfo>>& lcls = local[ch];
                // A cell's class depends only on its object, permittivity, list byte and the
                // two term bytes; runs of cells with the same five reuse the last class id.
                uint64_t lastSig = ~0ull, lastEpsBits = 0;
                int lastId = -1;
                const uint8_t* tb0 = termBits[0].data();
                const uint8_t* tb1 = termBits[1].data();
                uint8_t* const codes = cp.code.data();
                for (int y = y0; y < y1; ++y)
                    for (int z = 0; z < D.lz; ++z) {
                        const std::size_t row = static_cast<std::size_t>(D.idx(0, y, z));
                        const int* const phR = ph.v.data() + row;
                        const double* const epR = ep.v.data() + row;
                        for (int x = 0; x < D.lx; ++x) {
                            std::size_t id = row + static_cast<std::size_t>(x);
                            // cells equal to the last one in all five take its class
                            if (static_cast<uint32_t>(phR[x]) == static_cast<uint32_t>(lastSig) &&
                                cellLists[id] == static_cast<uint8_t>(lastSig >> 32) && tb0[id] == static_cast<uint8_t>(lastSig >> 40) &&
                                tb1[id] == static_cast<uint8_t>(lastSig >> 48) && lastId >= 0) {
                                uint64_t eb;
                                std::memcpy(&eb, epR + x, sizeof eb);
                                if (eb == lastEpsBits) {
                                    codes[id] = static_cast<uint8_t>(lastId);
                                    continue;
                                }
                            }
                            const int o = phR[x];
                            const double cellEps = epR[x];
                            const uint8_t lists = cellLists[id];
                            const uint8_t tbit[2] = {tb0[id], tb1[id]};
                            const uint64_t sig = static_cast<uint64_t>(static_cast<uint32_t>(o)) |
                                                 (static_cast<uint64_t>(lists) << 32) |
                                                 (static_cast<uint64_t>(tbit[0]) << 40) |
                                                 (static_cast<uint64_t>(tbit[1]) << 48);
                            uint64_t epsBits;
                            std::memcpy(&epsBits, &cellEps, sizeof epsBits);
                            ClassInfo c;
                            c.obj = (o < 0) ? 0 : o;
                            const uint8_t kind = lists & 3u;
                            bool pmlCell = false;
                            for (int t = 0; t < 2; ++t) pmlCell = pmlCell || (tbit[t] & 3u) || (tbit[t] & 0x40u);
                            if (kind == L_U || kind == L_D) {
                                double em = (kind == L_U) ? cellEps : 1.0;
                                double pref1 = -1.0 * dt / (em * dj), pref2 = -1.0 * dt / (em * dk);
                                if (tp[0].present) c.cint[0] = pref2;
                                if (tp[1].present) c.cint[1] = -pref1;
                                c.toD = (kind == L_D) ? 1 : 0;
                            }
                            if (pmlCell) {
                                uint8_t pmlToD = (E && matInPML) ? 1 : 0;
                                if (kind != L_NONE && c.toD != pmlToD)
                                    throw UnsupportedError("a cell's interior and CPML updates target different fields");
                                c.toD = pmlToD;
                            }
                            c.lor = (lists >> 2) & 1u;
                            c.ordip = (lists >> 3) & 1u;
                            if (c.lor || c.ordip) c.eps = cellEps;
                            if (c.toD || c.lor || c.ordip) chunkAnyD[ch] = 1;
                            for (int t = 0; t < 2; ++t) {
                                if (!tp[t].present) {
                                    if (tbit[t] & 0x63u) throw InputError("CPML term without a neighbour field");
                                    continue;
                                }
                                c.nplain[t] = (tbit[t] >> 2) & 3u;
                                c.kflag[t] = (tbit[t] >> 4) & 1u;
                                c.npsi[t] = tbit[t] & 3u;
                                c.psiUpd[t] = (tbit[t] >> 5) & 1u;
                            }
                            Key key = {double(c.toD), double(c.lor), double(c.ordip), double(c.obj), c.eps,
                                       c.cint[0], c.cint[1], double(c.nplain[0]), double(c.nplain[1]),
                                       double(c.kflag[0]), double(c.kflag[1]), double(c.npsi[0]),
                                       double(c.npsi[1]), double(c.psiUpd[0]), double(c.psiUpd[1]), 0.0};
                            if (!(c.lor || c.ordip)) key[4] = 1.0, c.eps = 1.0;
                            if (!c.lor) key[3] = 0.0, c.obj = 0;
                            int lid;
                            auto it = lindex.find(key);
                            if (it == lindex.end()) {
                                lid = static_cast<int>(lcls.size());
                                // a chunk's classes are a subset of the whole component's
                                if (lid > 255) throw UnsupportedError("more than 255 distinct cell classes in one component");
                                lcls.emplace_back(key, c);
                                lindex[key] = lid;
                            } else {
                                lid = it->second;
                            }
                            lastSig = sig;
                            lastEpsBits = epsBits;
                            lastId = lid;
                            codes[id] = static_cast<uint8_t>(lid);
                        }
                    }
            } catch (...) {
                chunkErr[ch] = std::current_exception();
            }
        }
        for (int ch = 0; ch < nChunks; ++ch)
            if (chunkErr[ch]) std::rethrow_exception(chunkErr[ch]);
        clk.mark("comp-classes");
        bool anyD = false;
        std::vector<std::vector<uint8_t>> remap(static_cast<std::size_t>(nChunks));
        for (int ch = 0; ch < nChunks; ++ch) {
            anyD = anyD || chunkAnyD[ch];
            for (auto& kc : local[ch]) {
                auto it = index.find(kc.first);
                int cid;
                if (it == index.end()) {
                    cid = static_cast<int>(cp.classes.size());
                    if (cid > 255) throw UnsupportedError("more than 255 distinct cell classes in one component");
                    cp.classes.push_back(kc.second);
                    index[kc.first] = cid;
                } else {
                    cid = it->second;
                }
                remap[ch].push_back(static_cast<uint8_t>(cid));
            }
        }
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
        for (int ch = 0; ch < nChunks; ++ch) {
            int y0, y1;
            chunkRows(ch, y0, y1);
            const std::vector<uint8_t>& rm = remap[ch];
            const std::size_t b = static_cast<std::size_t>(D.idx(0, y0, 0)), e = static_cast<std::size_t>(D.idx(0, y1, 0));
            for (std::size_t id = b; id < e; ++id) cp.code[id] = rm[cp.code[id]];
        }
        clk.mark("comp-remap");
        for (std::size_t q = 1; q < cp.classes.size(); ++q) {
            const ClassInfo& k = cp.classes[q];
            bool acts = k.toD || k.lor || k.ordip;
            for (int t = 0; t < 2; ++t)
                acts = acts || k.cint[t] != 0.0 || k.nplain[t] || k.kflag[t] || k.npsi[t] || k.psiUpd[t];
            if (!acts) throw InputError("internal: a cell class with no update");
        }
        cp.hasD = anyD;
        int np = 0;
        for (auto& o : objs) np = std::max(np, static_cast<int>(o.gamma.size()));
        cp.nPoles = (E && P.disp) ? np : 0;
    }

    // Oriented-dipole polarisation cells (upOrDipP_): the cell-centred grid points whose
    // object has oriented-dipole poles, from initializeList on physPOrDip_
    // (parallelFDTDField.cpp:83-87 with getBlasLists / fillBlasLists), and the dipole
    // direction of every pole there (setupDipMoments, parallelFDTDField.hpp:960-1048:
    // isotropic 1, unidirectional the normalised direction).
    // getTangentDip (parallelFDTDField.hpp:1058-1091), 3-D form: the tangent rotated from the
    // normal by pi/2 in polar angle (longitudinal) and its cross product with the normal
    // (latitudinal), weighted.
    static std::array<double, 3> tangentDip(const std::array<double, 3>& n, double latF, double longF) {
        const double mag = std::sqrt(((0.0 + n[0] * n[0]) + n[1] * n[1]) + n[2] * n[2]);
        std::array<double, 3> sph = {mag, std::acos(n[2] / mag), std::atan(n[1] / n[0])};
        if (n[0] == 0.0) sph[2] = n[1] >= 0.0 ? M_PI / 2.0 : -1.0 * M_PI / 2.0;
        if (n[0] < 0) sph[2] += M_PI;
        if (mag < 1e-20) sph = {0.0, 0.0, 0.0};
        const double pol = sph[1] + M_PI / 2.0, az = sph[2];
        const std::array<double, 3> lng = {mag * std::sin(pol) * std::cos(az), mag * std::sin(pol) * std::sin(az), mag * std::cos(pol)};
        std::array<double, 3> out;
        for (int i = 0; i < 3; ++i) {
            const double lat = n[(i + 1) % 3] * lng[(i + 2) % 3] - n[(i + 2) % 3] * lng[(i + 1) % 3];
            out[i] = longF * lng[i] + latF * lat;
        }
        return out;
    }

    void buildOrDip() {
        OrDipPlan& od = P.ordip;
        od = OrDipPlan();
        int np = 0;
        for (auto& o : objs)
            if (o.orDip && o.gamma.size() > 0) np = std::max(np, static_cast<int>(o.gamma.size()));
        if (np == 0) return;
        od.present = true;
        od.nPoles = np;
        const Field3<int>& ph = phys[6];
        // rows of y in parallel, concatenated in y order (the reference's list order);
        // the first error in that order is the one reported
        const int rows = std::max(0, D.ly - 2);
        std::vector<std::vector<long long>> rCells(static_cast<std::size_t>(rows));
        std::vector<std::vector<int>> rObj(static_cast<std::size_t>(rows));
        std::vector<std::vector<std::array<double, 3>>> rDip(static_cast<std::size_t>(rows));
        std::vector<std::exception_ptr> rErr(static_cast<std::size_t>(rows));
#pragma omp parallel for schedule(dynamic, 4)
        for (int jj = 1; jj < D.ly - 1; ++jj) {
            const std::size_t r = static_cast<std::size_t>(jj - 1);
            try {
                for (int kk = 1; kk < D.lz - 1; ++kk)
                    for (int ii = 1; ii < D.lx - 1; ++ii) {
                        const int o = ph.at(ii, jj, kk);
                        if (o < 0) throw InputError("oriented-dipole list reaches a border cell");
                        const Object& ob = objs[o];
                        if (!(ob.orDip && ob.gamma.size() > 0)) continue;
                        rCells[r].push_back(D.idx(ii, jj, kk));
                        rObj[r].push_back(o);
                        for (int pp = 0; pp < np; ++pp) {
                            std::array<double, 3> dv = {0.0, 0.0, 0.0};
                            if (pp < static_cast<int>(ob.dipOr.size())) {
                                const DipOr dor = ob.dipOr[pp];
                                if (dor == DipOr::ISOTROPIC) {
                                    dv = {1.0, 1.0, 1.0};
                                } else if (dor == DipOr::UNIDIRECTIONAL) {
                                    dv = ob.dipE[pp];
                                } else if (dor == DipOr::REL_TO_NORM) {
                                    const std::array<double, 3> pt = {((ii - 1) - (nvec[0] - nvec[0] % 2) / 2.0) * d[0],
                                                                      ((jj - 1) - (nvec[1] - nvec[1] % 2) / 2.0) * d[1],
                                                                      ((kk - 1) - (nvec[2] - nvec[2] % 2) / 2.0) * d[2]};
                                    const std::array<double, 3> n = ob.gradient(pt);
                                    const std::array<double, 3>& w = ob.dipW[static_cast<std::size_t>(pp)];
                                    const std::array<double, 3> tan = tangentDip(n, w[1], w[2]);
                                    for (int c = 0; c < 3; ++c) dv[c] = w[0] * n[c] + tan[c];
                                }
                                // the lat_tangent and long_tangent forms leave the reference's
                                // dipole grid at zero (setupDipMoments has no branch for them)
                            }
                            rDip[r].push_back(dv);
                        }
                    }
            } catch (...) {
                rErr[r] = std::current_exception();
            }
        }
        for (int r = 0; r < rows; ++r) {
            if (rErr[static_cast<std::size_t>(r)]) std::rethrow_exception(rErr[static_cast<std::size_t>(r)]);
            const std::size_t q = static_cast<std::size_t>(r);
            od.cells.insert(od.cells.end(), rCells[q].begin(), rCells[q].end());
            od.obj.insert(od.obj.end(), rObj[q].begin(), rObj[q].end());
            od.dip.insert(od.dip.end(), rDip[q].begin(), rDip[q].end());
        }
        // E_c at the cell and one cell below along c enter the averaged dot product
        od.offA[0] = 1;
        od.offA[1] = static_cast<long long>(D.lx) * D.lz;
        od.offA[2] = D.lx;
    }

    void build() {
        PhaseClock clk;
        P.in = in;
        objs = in.objects;
        d = in.d;
        dt = in.dt;
        P.dt = dt;
        for (int q = 0; q < 3; ++q) nvec[q] = static_cast<int>(std::floor(in.size[q] / d[q] + 0.5)) + 1;
        for (auto& o : objs) o.setUpConsts(dt);
        D.nx = nvec[0];
        D.ny = nvec[1];
        D.nz = nvec[2];
        D.threeD = in.size[2] != 0;
        D.lx = nvec[0] + 2;
        D.ly = nvec[1] + 2;
        D.lz = D.threeD ? nvec[2] + 2 : 1;
        P.dims = D;
        P.nSteps = in.nSteps();
        P.tcur.resize(static_cast<std::size_t>(P.nSteps) + 1);
        double t = 0.0;
        for (int s = 0; s <= P.nSteps; ++s) {
            P.tcur[s] = t;
            t += dt;
        }
        // the seven material grids are independent: built concurrently, each with its
        // share of the threads
        {
            struct GridSpec {
                int g;
                bool E;
                std::array<double, 3> off;
                std::array<int, 3> end;
            };
            const GridSpec grids[7] = {{6, true, {0.0, 0.0, 0.0}, {0, 0, 0}}, {0, true, {0.5, 0.0, 0.0}, {1, 0, 0}},
                                       {1, true, {0.0, 0.5, 0.0}, {0, 1, 0}}, {2, true, {0.0, 0.0, 0.5}, {0, 0, 1}},
                                       {3, false, {0.0, 0.5, 0.5}, {0, 1, 1}}, {4, false, {0.5, 0.0, 0.5}, {1, 0, 1}},
                                       {5, false, {0.5, 0.5, 0.0}, {1, 1, 0}}};
            const int nThreads = omp_get_max_threads();
            const int outer = std::min(7, nThreads);
            const int inner = std::max(1, (nThreads + outer - 1) / outer);
            std::exception_ptr gErr[7];
            NestedTeams nest;
#pragma omp parallel for schedule(dynamic, 1) num_threads(outer)
            for (int q = 0; q < 7; ++q) {
                try {
                    setupPhys(grids[q].g, grids[q].E, grids[q].off, grids[q].end, inner);
                } catch (...) {
                    gErr[q] = std::current_exception();
                }
            }
            for (int q = 0; q < 7; ++q)
                if (gErr[q]) std::rethrow_exception(gErr[q]);
        }
        clk.mark("materials");
        // a barycentric test whose weights do not sum to one (Obj.cpp:485-489, 502-506)
        for (const auto& o : objs)
            if (o.baryFault->load())
                throw InputError(o.shape == Shape::TETRAHEDRON
                                     ? "The sum of the boundary checks for a tetrahedron does not equal the determinant of the verticies"
                                     : "The sum of the boundary checks for a triangular base does not equal the determinant of the verticies");
        scanPML();
        checkMagnetic();
        clk.mark("pml-scan");
        bool disp = false;
        for (auto& o : objs)
            if (o.gamma.size() > 0 || o.ML || o.epsInf > 1.0) disp = true;
        if (matInPML) disp = true;
        P.disp = disp;
        P.dielectricMatInPML = matInPML;
        bool te = D.threeD || in.pol == Pol::HZ || in.pol == Pol::EX || in.pol == Pol::EY;
        bool tm = D.threeD || in.pol == Pol::EZ || in.pol == Pol::HX || in.pol == Pol::HY;
        if (te) P.comp[EX].present = P.comp[EY].present = P.comp[HZ].present = true;
        if (tm) P.comp[HX].present = P.comp[HY].present = P.comp[EZ].present = true;
        for (auto& o : objs)
            if (o.orDip && o.gamma.size() > 0 && !D.threeD)
                throw UnsupportedError("oriented-dipole poles need a 3-D grid (the reference stops on a grid index "
                                       "assertion, GRID/parallelGrid.hpp:563, while it builds their 2-D lists)");
        // the reference's list order: TE (Hz, Ex, Ey) then TM (Ez, Hx, Hy)
        // Each component's lists depend only on the material maps and on which components
        // exist, so the components are built concurrently; the first error in the order
        // above is the one reported.
        const int order[6] = {HZ, EX, EY, EZ, HX, HY};
        bool present[6];
        for (int c = 0; c < 6; ++c) present[c] = P.comp[c].present;
        // Each component's row loops are parallel too (nested; the caller's setting is put back).
        std::exception_ptr err[6];
        int nComp = 0;
        for (int c = 0; c < 6; ++c) nComp += present[c] ? 1 : 0;
        const int nThreads = omp_get_max_threads();
        // every thread in some team (the last teams one thread larger than the fair share)
        innerThreads_ = std::max(1, (nThreads + std::max(1, nComp) - 1) / std::max(1, nComp));
        // the side work (emitter and TFSF set-up: it needs the material maps, not the lists)
        // runs on a thread of its own meanwhile; its errors come after the components'
        std::exception_ptr sideErr;
        std::thread sideThread;
        if (side)
            sideThread = std::thread([&] {
                try {
                    side();
                } catch (...) {
                    sideErr = std::current_exception();
                }
            });
        {
            NestedTeams nest;
#pragma omp parallel for schedule(dynamic, 1) num_threads(std::min(nThreads, std::max(1, nComp)))
            for (int q = 0; q < 6; ++q) {
                if (!present[order[q]]) continue;
                try {
                    buildComp(order[q]);
                } catch (...) {
                    err[q] = std::current_exception();
                }
            }
        }
        if (sideThread.joinable()) sideThread.join();
        for (int q = 0; q < 6; ++q)
            if (err[q]) std::rethrow_exception(err[q]);
        if (sideErr) std::rethrow_exception(sideErr);
        clk.mark("components");
        for (int c = 0; c < 3; ++c) P.comp[c].hasD = P.comp[c].present && disp;
        buildOrDip();
        P.alpha.clear();
        P.xi.clear();
        P.gamma.clear();
        P.alphaInc.clear();
        for (auto& o : objs) {
            P.alpha.push_back(o.alpha);
            P.xi.push_back(o.xi);
            P.gamma.push_back(o.gamma);
            P.alphaInc.push_back(o.alphaInc);
        }
        P.in.objects = objs;
        clk.mark("dipoles");
        buildSources();
        buildDetectors();
        buildFluxes();
        clk.mark("io");
    }

    // ---- sources (parallelFDTDField.cpp:455-620) ----
    // A source along a grid axis (phi a multiple of 90 degrees after rounding) is a normal
    // source (parallelSourceNormal.cpp:15-37): dt * Re(sum of pulses) on every cell of its
    // box. Any other phi is an oblique source (parallelSourceOblique.hpp:88-165), whose
    // cells each add scalefact * Re(sum of pulses at t - t_off) without the factor dt; an
    // oblique E_x/E_y (H_x/H_y) source acts on both in-plane components. A circularly
    // polarised source (L/R) is two normal sources on the two E components across the
    // source's thinnest axis (parallelFDTDField.cpp:548-618): the reference scales each
    // pulse by its polarisation prefactors and phase in a parameter slot past the one the
    // pulse functions read (UTIL/PulseFxn.hpp:19-89 read the amplitude at a fixed index), so
    // both components carry the unscaled pulse.
    void buildSources() {
        for (auto& s : in.sources) {
            if (s.pol == Pol::L || s.pol == Pol::R) {
                int amin = 0;  // isamin_: the first axis of the smallest size
                for (int ii = 1; ii < 3; ++ii)
                    if (s.sz[ii] < s.sz[amin]) amin = ii;
                const int pairs[3][2] = {{EY, EZ}, {EX, EZ}, {EX, EY}};
                for (int c : pairs[amin]) addNormalSource(s, c);
                continue;
            }
            int comp = EX;
            switch (s.pol) {
                case Pol::EX: comp = EX; break;
                case Pol::EY: comp = EY; break;
                case Pol::EZ: comp = EZ; break;
                case Pol::HX: comp = HX; break;
                case Pol::HY: comp = HY; break;
                case Pol::HZ: comp = HZ; break;
                default: throw UnsupportedError("source polarisation");
            }
            if (static_cast<int>(std::round(s.phi)) % 90 == 0) {
                addNormalSource(s, comp);
            } else if (comp == EX || comp == EY) {
                addObliqueSource(s, EX);
                addObliqueSource(s, EY);
            } else if (comp == HX || comp == HY) {
                // parallelFDTDField.cpp:523-536 builds the H_y part first for an H_x source
                addObliqueSource(s, comp == HX ? HY : HX);
                addObliqueSource(s, comp);
            } else {
                addObliqueSource(s, comp);
            }
        }
    }

    // One normal source of component comp: the box of the source (parallelSourceNormal.hpp:60-150).
    void addNormalSource(const SourceSpec& s, int comp) {
        if (!P.comp[comp].present) throw InputError("a source acts on a field that this polarisation does not have");
        SourcePlan sp;
        sp.comp = comp;
        std::array<int, 3> lloc, lsz = {0, 0, 0};
        bool inside = true;
        for (int ii = 0; ii < 3; ++ii) {
            int ln = lnv(ii);
            if (s.loc[ii] >= 0 && s.loc[ii] < ln - 2) lloc[ii] = s.loc[ii] + 1;
            else if (s.loc[ii] < 0 && s.loc[ii] + s.sz[ii] > 0) lloc[ii] = 1;
            else lloc[ii] = -1;
        }
        if (D.lz == 1) lloc[2] = 0;
        if (lloc[0] == -1 || lloc[1] == -1 || lloc[2] == -1) inside = false;
        if (inside) {
            for (int ii = 0; ii < 3; ++ii) {
                int ln = lnv(ii);
                lsz[ii] = (s.sz[ii] + s.loc[ii] > ln - 2) ? ln - lloc[ii] - 1 : s.loc[ii] + s.sz[ii] - (lloc[ii] - 1);
            }
            if (D.lz == 1) lsz[2] = 1;
            for (int z = 0; z < lsz[2]; ++z)
                for (int y = 0; y < lsz[1]; ++y)
                    for (int x = 0; x < lsz[0]; ++x) sp.cells.push_back(D.idx(lloc[0] + x, lloc[1] + y, lloc[2] + z));
        }
        sp.value.resize(static_cast<std::size_t>(P.nSteps));
        for (int st = 0; st < P.nSteps; ++st) {
            cplx v = 0.0;
            for (auto& pul : s.pulses) v += pul.value(P.tcur[st]);
            sp.value[st] = dt * std::real(v);
        }
        P.sources.push_back(std::move(sp));
    }

    // One oblique source acting on component comp (parallelSourceOblique.hpp:54-165): the
    // cells of the box around the source's centre whose offset from it lies within dx/sqrt(2)
    // of the plane normal to the propagation direction. The reference never reads a polar
    // angle for soft sources (srcTheta_ stays 90, parallelInputs.cpp:44), so in 3-D the
    // plane's normal is z and in 2-D (theta forced to 90 degrees) it lies in the xy plane
    // at phi. Cells with equal (scalefact, t_off) share one time series.
    void addObliqueSource(const SourceSpec& s, int comp) {
        if (!P.comp[comp].present) throw InputError("a source acts on a field that this polarisation does not have");
        const bool twoD = D.lz == 1;
        const double phiA = std::fmod(s.phi, 360.0) * M_PI / 180.0;
        double thetaA = std::fmod(90.0, 360.0) * M_PI / 180.0 - M_PI / 2.0;
        if (twoD) thetaA = M_PI / 2.0;
        const double phi = std::fmod(phiA + M_PI / 2.0, 2.0 * M_PI);
        const double theta = (thetaA >= M_PI / 2) ? thetaA - M_PI / 2.0 : thetaA + M_PI / 2.0;
        double nv[3] = {std::sin(thetaA) * std::cos(phiA), std::sin(thetaA) * std::sin(phiA), std::cos(thetaA)};
        const double nrm = 1.0 / std::sqrt(std::pow(nv[0], 2.0) + std::pow(nv[1], 2.0) + std::pow(nv[2], 2.0));
        for (double& v : nv) v *= nrm;
        const double dx = in.d[0], dy = in.d[1], dz = twoD ? 1.0 : in.d[2];
        const std::array<int, 3>& loc = s.loc;
        const std::array<int, 3>& sz = s.sz;
        auto half = [](double v) { return std::fabs(static_cast<int>(std::round(v / 2.0))); };
        auto tilt = [](int m, double v) { return static_cast<int>(std::fabs(std::round(m + v))); };
        int xMin = static_cast<int>(loc[0] - half(sz[0] * std::cos(phi)));
        xMin = std::min(xMin, tilt(xMin, sz[1] * std::cos(phi) * std::sin(theta)));
        int yMin = static_cast<int>(loc[1] - half(sz[0] * std::sin(phi)));
        yMin = std::min(yMin, tilt(yMin, sz[1] * std::sin(phi) * std::sin(theta)));
        int xMax = static_cast<int>(loc[0] + half(sz[0] * std::cos(phi)));
        xMax = std::min(xMax, tilt(xMax, sz[1] * std::cos(phi) * std::sin(theta)));
        int yMax = static_cast<int>(loc[1] + half(sz[0] * std::sin(phi)));
        yMax = std::min(yMax, tilt(yMax, sz[1] * std::sin(phi) * std::sin(theta)));
        int zMin = 0, zMax = 0;
        if (!twoD) {
            zMin = static_cast<int>(loc[2] - half(sz[1] * std::cos(theta)));
            zMax = static_cast<int>(loc[2] + half(sz[1] * std::cos(theta)));
        }
        double off[3] = {0.0, 0.0, 0.0};
        if (comp == EX || comp == HY || comp == HZ) off[0] = 0.5;
        if (comp == HX || comp == EY || comp == HZ) off[1] = 0.5;
        if (!twoD && (comp == HX || comp == HY || comp == EZ)) off[2] = 0.5;
        double scale;
        if (comp == EX || comp == HX) scale = std::cos(phi) * std::sin(thetaA);
        else if (comp == EY || comp == HY) scale = std::sin(phi) * std::sin(thetaA);
        else scale = std::cos(thetaA);
        const double reach = dx / std::sqrt(2.0);
        std::vector<double> offsets;           // distinct t_off, in the order first met
        std::vector<std::vector<long long>> cells;
        for (int xx = xMin; xx <= xMax; ++xx)
            for (int yy = yMin; yy <= yMax; ++yy)
                for (int zz = zMin; zz <= zMax; ++zz) {
                    const double pt[3] = {(xx - loc[0] + off[0]) * dx, (yy - loc[1] + off[1]) * dy, (zz - loc[2] + off[2]) * dz};
                    double dot = 0.0;  // the summation order of the one-process build's ddot_
                    for (int k = 0; k < 3; ++k) dot += pt[k] * nv[k];
                    if (std::fabs(dot) > reach) continue;
                    if (xx < 0 || xx >= D.nx || yy < 0 || yy >= D.ny || (!twoD && (zz < 0 || zz >= D.nz)))
                        throw InputError("An oblique source reaches outside the FDTD cell");
                    double toff = 0.0;
                    for (int k = 0; k < 3; ++k) toff += nv[k] * pt[k];
                    std::size_t g = 0;
                    while (g < offsets.size() && offsets[g] != toff) ++g;
                    if (g == offsets.size()) {
                        offsets.push_back(toff);
                        cells.emplace_back();
                    }
                    cells[g].push_back(D.idx(xx + 1, yy + 1, twoD ? 0 : zz + 1));
                }
        for (std::size_t g = 0; g < offsets.size(); ++g) {
            SourcePlan sp;
            sp.comp = comp;
            sp.cells = std::move(cells[g]);
            sp.value.resize(static_cast<std::size_t>(P.nSteps));
            for (int st = 0; st < P.nSteps; ++st) {
                cplx v = 0.0;
                for (auto& pul : s.pulses) v += pul.value(P.tcur[st] - offsets[g]);
                sp.value[st] = scale * std::real(v);
            }
            P.sources.push_back(std::move(sp));
        }
    }

    // ---- time-domain detectors (parallelDTC.hpp:40-120, parallelStorageDTC.hpp) ----
    void buildDetectors() {
        for (auto& ds : in.detectors) {
            DetectorPlan dp;
            dp.spec = ds;
            dp.sz = ds.sz;
            const bool freq = ds.cls == DtcClass::FREQ;
            // parallelFDTDField.cpp:1728 rounds a frequency detector's interval to the nearest step
            dp.timeInt = freq ? static_cast<int>(std::floor(ds.timeInt / dt + 0.5)) : static_cast<int>(std::floor(ds.timeInt / dt));
            if (dp.timeInt == 0) throw InputError("The time step of a detector is less than the main grid or set to 0.");
            std::vector<std::pair<int, std::array<int, 3>>> flds;
            auto need = [&](int c) {
                if (!P.comp[c].present) throw InputError("DTC TYPE IS NOT DEFINED for this polarisation");
            };
            switch (ds.type) {
                case DtcType::EX: need(EX); flds.push_back({EX, {0, 0, 0}}); break;
                case DtcType::EY: need(EY); flds.push_back({EY, {0, 0, 0}}); break;
                case DtcType::EZ: need(EZ); flds.push_back({EZ, {0, 0, 0}}); break;
                case DtcType::HX: need(HX); flds.push_back({HX, {0, 0, 0}}); break;
                case DtcType::HY: need(HY); flds.push_back({HY, {0, 0, 0}}); break;
                case DtcType::HZ: need(HZ); flds.push_back({HZ, {0, 0, 0}}); break;
                case DtcType::DX: case DtcType::DY: case DtcType::DZ: {
                    int c = static_cast<int>(ds.type) - static_cast<int>(DtcType::DX);
                    if (!P.comp[c].present || !P.disp) throw InputError("D detector without a D field");
                    flds.push_back({6 + c, {0, 0, 0}});
                    break;
                }
                case DtcType::EPOW:
                case DtcType::HPOW: {
                    bool e = ds.type == DtcType::EPOW;
                    bool h2 = P.comp[HZ].present, e2 = P.comp[EZ].present;
                    if (h2 && e2) {
                        if (e) flds = {{EX, {-1, 0, 0}}, {EY, {0, -1, 0}}, {EZ, {0, 0, -1}}};
                        else flds = {{HX, {1, 0, 0}}, {HY, {0, 1, 0}}, {HZ, {0, 0, 1}}};
                    } else if (h2) {
                        if (e) flds = {{EX, {-1, 0, 0}}, {EY, {0, -1, 0}}};
                        else flds = {{HZ, {0, 0, 0}}};
                    } else {
                        if (e) flds = {{EZ, {0, 0, 0}}};
                        else flds = {{HX, {1, 0, 0}}, {HY, {0, 1, 0}}};
                    }
                    break;
                }
                default: throw UnsupportedError("detector type needs polarisation or magnetic fields");
            }
            // conversions
            for (int ii = 0; ii < 3; ++ii) {
                int gn = gnv(ii);
                dp.realLoc[ii] = d[ii] * (ds.loc[ii] - (gn - 1 * 2 - gn % 2) / 2);
            }
            if (ds.SI) {
                dp.tConv *= in.a / kSpeedOfLight;
                for (auto& r : dp.realLoc) r *= in.a;
                dp.convFactor = (in.I0 / in.a);
                if (ds.type == DtcType::EX || ds.type == DtcType::EY || ds.type == DtcType::EZ)
                    dp.convFactor /= kEps0 * kSpeedOfLight;
                for (auto& r : dp.realLoc) r *= in.a;
            }
            dp.power = (ds.type == DtcType::EPOW || ds.type == DtcType::HPOW);
            if (dp.power) dp.convFactor *= dp.convFactor;
            if (freq) {
                freqDetector(dp, flds);
                P.freqDetectors.push_back(std::move(dp));
                continue;
            }
            for (auto& f : flds) {
                DetectorPlan::Field F;
                F.comp = f.first;
                F.off = f.second;
                std::array<int, 3> loc = ds.loc, sz = ds.sz;
                for (int oo = 0; oo < 3; ++oo) {
                    sz[oo] += (1 + std::abs(F.off[oo])) / 2;
                    loc[oo] -= (1 - F.off[oo]) / 2;
                }
                F.outSz = sz;
                F.cells.assign(static_cast<std::size_t>(sz[0]) * sz[1] * sz[2], -1);
                std::array<int, 3> ll, ls;
                bool inside = true;
                for (int ii = 0; ii < 3; ++ii) {
                    int ln = lnv(ii);
                    if (loc[ii] >= 0 && loc[ii] < ln - 2) ll[ii] = loc[ii] + 1;
                    else if (loc[ii] == -1) ll[ii] = 0;
                    else if (loc[ii] < 0 && loc[ii] + sz[ii] > 0) ll[ii] = 1;
                    else ll[ii] = -1;
                }
                if (D.lz == 1) ll[2] = 0;
                for (int ii = 0; ii < 3; ++ii)
                    if (ll[ii] == -1) inside = false;
                if (inside) {
                    for (int ii = 0; ii < 3; ++ii) {
                        int ln = lnv(ii);
                        ls[ii] = (sz[ii] + loc[ii] > ln - 2) ? ln - ll[ii] - 1 : loc[ii] + sz[ii] - (ll[ii] - 1);
                    }
                    if (D.lz == 1) ls[2] = 1;
                    std::array<int, 3> lo = {ll[0] - 1 - loc[0], ll[1] - 1 - loc[1], (D.lz == 1) ? 0 : ll[2] - 1 - loc[2]};
                    for (int y = 0; y < ls[1]; ++y)
                        for (int z = 0; z < ls[2]; ++z)
                            for (int x = 0; x < ls[0]; ++x) {
                                int ox = lo[0] + x, oy = lo[1] + y, oz = lo[2] + z;
                                if (ox < 0 || oy < 0 || oz < 0 || ox >= sz[0] || oy >= sz[1] || oz >= sz[2]) continue;
                                F.cells[static_cast<std::size_t>(ox + sz[0] * (oz + sz[2] * oy))] =
                                    D.idx(ll[0] + x, ll[1] + y, ll[2] + z);
                            }
                }
                dp.fields.push_back(std::move(F));
            }
            if (ds.cls == DtcClass::TXT) {
                // the text writer loops over the first field's enlarged box and reads box+offset
                const auto& F0 = dp.fields[0];
                for (auto& F : dp.fields)
                    for (int q = 0; q < 3; ++q)
                        if (F0.outSz[q] - 1 + std::abs(F.off[q]) >= F.outSz[q])
                            throw UnsupportedError("text detector of a staggered power field reads past its box (the reference aborts)");
            }
            P.detectors.push_back(std::move(dp));
        }
    }

    // A frequency-domain detector (parallelDetectorFREQ_Base constructor,
    // DTC/parallelDTC_FREQ.hpp:80-130): its own unit conversions, and per field the DFT box
    // of parallelStorageFreqDTC without a propagation direction (genDatStruct, getLocalLocEl,
    // getLocalSzEl: DTC/parallelStorageFreqDTC.hpp:168-320): points x fastest, then z, then
    // y, from the detector corner; the field offsets of power detectors are not applied.
    void freqDetector(DetectorPlan& dp, const std::vector<std::pair<int, std::array<int, 3>>>& flds) {
        const DetectorSpec& ds = dp.spec;
        dp.convFactor = 1.0;
        dp.freqConv = 1.0;
        if (ds.SI) {
            dp.convFactor = in.I0 / in.a;
            if (ds.type == DtcType::EX || ds.type == DtcType::EY || ds.type == DtcType::EZ)
                dp.convFactor /= kEps0 * kSpeedOfLight;
            dp.freqConv = kSpeedOfLight / in.a;
        }
        if (dp.power) dp.convFactor = std::pow(dp.convFactor, 2.0);
        dp.freqConv /= (M_PI * 2.0);
        dp.szFreq = static_cast<long long>(ds.sz[0]) * ds.sz[1] * ds.sz[2];
        for (auto& f : flds) {
            DetectorPlan::Field F;
            F.comp = f.first;
            F.off = f.second;
            std::array<int, 3> ll{}, ls{0, 0, 0};
            bool inside = true;
            for (int ii = 0; ii < 3; ++ii) {
                const int ln = lnv(ii);
                if (ds.loc[ii] >= 0 && ds.loc[ii] < ln - 2) ll[ii] = ds.loc[ii] + 1;
                else if (ds.loc[ii] == -1) ll[ii] = 0;
                else if (ds.loc[ii] < 0 && ds.loc[ii] + ds.sz[ii] > 0) ll[ii] = 1;
                else ll[ii] = -1;
            }
            if (D.lz == 1) ll[2] = 0;
            for (int ii = 0; ii < 3; ++ii)
                if (ll[ii] == -1) inside = false;
            if (inside)
                for (int ii = 0; ii < 3; ++ii) {
                    const int ln = lnv(ii);
                    ls[ii] = (ds.sz[ii] + ds.loc[ii] > ln - 2) ? ln - ll[ii] - 1 : ds.loc[ii] + ds.sz[ii] - (ll[ii] - 1);
                }
            F.outSz = ls;  // x, y, z sizes of the stored box
            for (int y = 0; y < ls[1]; ++y)
                for (int z = 0; z < ls[2]; ++z)
                    for (int x = 0; x < ls[0]; ++x) F.cells.push_back(D.idx(ll[0] + x, ll[1] + y, ll[2] + z));
            if (static_cast<long long>(F.cells.size()) > dp.szFreq) throw InputError("frequency detector box larger than the detector");
            dp.fields.push_back(std::move(F));
        }
    }

    // ---- DFT flux (parallelFlux.hpp:80-140, parallelFlux.cpp:13-70,338-542,
    //      parallelStorageFreqDTC.hpp:120-240) ----
    FreqStore makeStore(int comp, int propDir, std::array<int, 3> loc, std::array<int, 3> sz, int nfreq) {
        FreqStore st;
        st.comp = comp;
        st.loc = loc;
        st.sz = sz;
        st.propDir = propDir;
        std::array<int, 3> ll;
        for (int ii = 0; ii < 3; ++ii) {
            int ln = lnv(ii);
            if (loc[ii] >= 0 && loc[ii] < ln - 2) ll[ii] = loc[ii] + 1;
            else if (loc[ii] == -1) ll[ii] = 0;
            else if (loc[ii] < 0 && loc[ii] + sz[ii] > 0) ll[ii] = 1;
            else ll[ii] = -1;
        }
        if (D.lz == 1) ll[2] = 0;
        if (ll[0] == -1 || ll[1] == -1 || ll[2] == -1) {
            st.outN = {0, 0, 0};
            return st;
        }
        auto lsz = [&](int ind, int localLoc) {
            int ln = lnv(ind);
            return (sz[ind] + loc[ind] > ln - 2) ? ln - localLoc - 1 : loc[ind] + sz[ind] - (localLoc - 1);
        };
        std::array<int, 3> insz = {0, 0, 0}, add = {0, 0, 0};
        long long stride = 1;
        if (propDir == 0) {
            stride = D.lx;
            insz[2] = lsz(0, ll[0]);
            if (D.lz == 1) {
                insz[0] = lsz(1, ll[1]);
                insz[1] = 1;
                add = {0, 0, 1};
            } else {
                insz[0] = lsz(2, ll[2]);
                insz[1] = lsz(1, ll[1]);
                add = {0, 1, 0};
            }
        } else if (propDir == 1) {
            stride = 1;
            insz[0] = lsz(0, ll[0]);
            insz[1] = (D.lz == 1) ? 1 : lsz(2, ll[2]);
            insz[2] = lsz(1, ll[1]);
            add = {0, 0, 1};
        } else {
            stride = 1;
            insz[0] = lsz(0, ll[0]);
            insz[1] = lsz(1, ll[1]);
            insz[2] = lsz(2, ll[2]);
            add = {0, 1, 0};
        }
        st.inSz = insz;
        st.outN = {nfreq, insz[1], insz[0]};
        for (int ii = 0; ii < insz[1]; ++ii) {
            long long base = D.idx(ll[0] + ii * add[0], ll[1] + ii * add[1], ll[2] + ii * add[2]);
            for (int p = 0; p < insz[0]; ++p) st.cells.push_back(base + p * stride);
        }
        return st;
    }

    void buildFluxes() {
        for (auto& fs : in.fluxes) {
            FluxPlan fp;
            fp.spec = fs;
            const std::vector<double>& fl = fs.freqList;
            const int nfreq = static_cast<int>(fl.size());
            fp.dt = dt * static_cast<double>(fs.timeInt);
            fp.fluxConv = fs.weight;
            bool eq = (fl.size() > 1 && fl[1] - fl[0] == fl[2] - fl[1]);
            if (fl.size() < 3) throw UnsupportedError("flux regions need at least three frequencies (the reference reads freqList[2])");
            fp.dOmg = eq ? fl[1] - fl[0] : 0.0;
            fp.dLam = eq ? 0.0 : 1.0 / fl[1] - 1.0 / fl[0];
            if (fs.SI) {
                fp.freqConv = kSpeedOfLight / in.a;
                double cv = in.I0 / in.a * in.I0 / (kEps0 * in.a * kSpeedOfLight);
                fp.fluxConv = cv;
                for (auto& v : fp.incdConv) v = cv;
            }
            fp.real3D = P.comp[EZ].present && P.comp[HZ].present;
            fp.freqConv /= (M_PI * 2.0);
            // faces
            std::vector<std::pair<int, bool>> faces;
            const auto& sz = fs.sz;
            if (!fp.real3D) {
                if (sz[0] > 1 && sz[1] > 1) faces = {{1, false}, {1, true}, {0, false}, {0, true}};
                else if (sz[0] == 1 && (D.lx != 3)) faces = {{0, true}};
                else faces = {{1, true}};
            } else {
                if (sz[0] > 1 && sz[1] > 1 && sz[2] > 1) faces = {{0, true}, {0, false}, {1, true}, {1, false}, {2, true}, {2, false}};
                else if (sz[0] == 1) faces = {{0, true}};
                else if (sz[1] == 1) faces = {{1, true}};
                else if (sz[2] == 1) faces = {{2, true}};
            }
            for (auto& fc : faces) makeFace(fp, fc.first, fc.second, nfreq);
            long long off = 0;
            for (auto& st : fp.stores) {
                st.accOffset = off;
                off += static_cast<long long>(st.cells.size());
            }
            fp.npts = off;
            P.fluxes.push_back(std::move(fp));
        }
    }

    void makeFace(FluxPlan& fp, int dir, bool pl, int nfreq) {
        FluxFace f;
        const auto& loc_ = fp.spec.loc;
        const auto& sz_ = fp.spec.sz;
        int Ej, Ek, Hj, Hk;
        std::array<int, 3> sz;
        if (dir == 0) {
            Ej = EY; Hj = HY; Ek = EZ; Hk = HZ;
            bool z1 = (P.comp[Ej].present && D.lz == 1) || (P.comp[Ek].present && D.lz == 1);
            if (z1) { f.cor = 1; f.transCor1 = 2; f.transCor2 = 0; }
            else { f.cor = 2; f.transCor1 = 1; f.transCor2 = 0; }
            f.corI = 0; f.corJ = 1; f.corK = 2;
            sz = {1, sz_[1], sz_[2]};
        } else if (dir == 1) {
            Ej = EZ; Hj = HZ; Ek = EX; Hk = HX;
            f.cor = 0; f.transCor1 = 2; f.transCor2 = 1;
            f.corI = 1; f.corJ = 2; f.corK = 0;
            sz = {sz_[0], 1, sz_[2]};
        } else {
            Ej = EX; Hj = HX; Ek = EY; Hk = HY;
            f.cor = 0; f.transCor1 = 1; f.transCor2 = 2;
            f.corI = 2; f.corJ = 0; f.corK = 1;
            sz = {sz_[0], sz_[1], 1};
        }
        std::array<int, 3> loc = loc_;
        if (pl) loc[f.transCor2] = loc_[f.transCor2] + sz_[f.transCor2] - 1;
        std::array<int, 3> locOff = loc;
        f.sz = sz[f.cor] * sz[f.transCor1];
        f.faceSz = sz;
        auto add = [&](std::vector<int>& v, int comp, std::array<int, 3> l, std::array<int, 3> s) {
            v.push_back(static_cast<int>(fp.stores.size()));
            fp.stores.push_back(makeStore(comp, dir, l, s, nfreq));
        };
        bool e2 = P.comp[EZ].present, h2 = P.comp[HZ].present;
        if (e2 && h2) {
            std::array<int, 3> szOff = sz;
            locOff[f.corK] -= 1;
            szOff[f.corK] += 1;
            add(f.Ek, Ek, locOff, szOff);
            add(f.Hj, Hj, locOff, szOff);
            locOff[f.corI] -= 1;
            add(f.Hj, Hj, locOff, szOff);
            locOff[f.corK] += 1;
            szOff[f.corK] -= 1;
            locOff[f.corJ] -= 1;
            szOff[f.corJ] += 1;
            add(f.Hk, Hk, locOff, szOff);
            locOff[f.corI] += 1;
            add(f.Hk, Hk, locOff, szOff);
            add(f.Ej, Ej, locOff, szOff);
        } else if (e2) {
            if (P.comp[Ek].present) {
                locOff[f.corI] += -1;
                add(f.Ek, Ek, loc, sz);
                add(f.Hj, Hj, loc, sz);
                add(f.Hj, Hj, locOff, sz);
            } else {
                locOff[f.corI] += -1;
                add(f.Ej, Ej, loc, sz);
                add(f.Hk, Hk, loc, sz);
                add(f.Hk, Hk, locOff, sz);
            }
        } else {
            if (P.comp[Ej].present) {
                locOff[f.corI] += 1;
                add(f.Ej, Ej, loc, sz);
                add(f.Hk, Hk, loc, sz);
                add(f.Ej, Ej, locOff, sz);
            } else {
                locOff[f.corI] += 1;
                add(f.Ek, Ek, loc, sz);
                add(f.Hj, Hj, loc, sz);
                add(f.Ek, Ek, locOff, sz);
            }
        }
        f.weight = pl ? 1.0 : -1.0;
        bool any = false;
        for (auto* v : {&f.Ej, &f.Ek, &f.Hj, &f.Hk})
            for (int s : *v)
                if (fp.stores[s].outN[0] != 0) any = true;
        if (!any) throw InputError("One of the flux surfaces is outside the FDTD cell.");
        fp.faces.push_back(f);
    }
};

}  // namespace

Plan build_plan(const Inputs& in) {
    Plan P;
    Builder b(in, P);
    // The emitter and TFSF set-up read the material maps, the objects and which
    // components exist (all fixed before the component build) and write their own parts
    // of the plan: they run beside the component build.
    b.side = [&] {
        PhaseClock clk;
        if (!in.emitters.empty()) {
            const bool Ep[3] = {P.comp[EX].present, P.comp[EY].present, P.comp[EZ].present};
            build_emitters(in, P.dims, P.dt, Ep, b.epsRel[6].v.data(), P);
            clk.mark("emitters");
        }
        if (!in.tfsf.empty()) {
            const int* ph[6];
            for (int c = 0; c < 6; ++c) ph[c] = P.comp[c].present ? b.phys[c].v.data() : nullptr;
            build_tfsf(in, P.dims, P.dt, ph, b.objs, P);
            clk.mark("tfsf");
        }
    };
    b.build();
    // a surface term into D needs the D field of its component
    for (const TfsfPlan& T : P.tfsf)
        for (const TfsfAdds* a : {&T.addH, &T.addE})
            for (std::size_t q = 0; q < a->cells(); ++q)
                for (long long k = a->start[q]; k < a->start[q + 1]; ++k)
                    if (a->toD[static_cast<std::size_t>(k)] && (a->comp[q] > 2 || !P.comp[a->comp[q]].hasD))
                        throw UnsupportedError("TFSF correction into a D field the grid does not have");
    // incident-flux normalisation areas (parallelFlux.hpp:110-135)
    for (auto& fp : P.fluxes) {
        if (!fp.spec.crossSec) {
            auto simps = [](int n, double d) {
                std::vector<cplx> v(static_cast<std::size_t>(n), cplx(1.0, 0.0));
                if (n == 1) return v[0] * d;
                cplx r(0.0, 0.0);
                if (n % 2 == 0) {
                    for (int ii = 0; ii < (n - 2) / 2; ii++) r += d / 6.0 * (v[ii * 2] + 4.0 * v[ii * 2 + 1] + v[(ii + 1) * 2]);
                    for (int ii = 1; ii < n / 2; ii++) r += d / 6.0 * (v[ii * 2 - 1] + 4.0 * v[ii * 2] + v[ii * 2 + 1]);
                    r += d / 4.0 * (v[0] + v[1] + v[n - 1] + v[n - 2]);
                } else {
                    for (int ii = 0; ii < (n - 1) / 2; ii++) r += d / 3.0 * (v[ii * 2] + 4.0 * v[ii * 2 + 1] + v[(ii + 1) * 2]);
                }
                return r;
            };
            auto simps2DNorm = [&](int nx, int ny, double dx, double dy) {
                std::vector<cplx> res(static_cast<std::size_t>(ny), 0.0);
                for (auto& r : res) r = simps(nx, dx);
                // simps over a non-constant vector: re-implement on the values
                int n = ny;
                double d = dy;
                cplx r(0.0, 0.0);
                if (n == 1) return res[0] * d;
                if (n % 2 == 0) {
                    for (int ii = 0; ii < (n - 2) / 2; ii++) r += d / 6.0 * (res[ii * 2] + 4.0 * res[ii * 2 + 1] + res[(ii + 1) * 2]);
                    for (int ii = 1; ii < n / 2; ii++) r += d / 6.0 * (res[ii * 2 - 1] + 4.0 * res[ii * 2] + res[ii * 2 + 1]);
                    r += d / 4.0 * (res[0] + res[1] + res[n - 1] + res[n - 2]);
                } else {
                    for (int ii = 0; ii < (n - 1) / 2; ii++) r += d / 3.0 * (res[ii * 2] + 4.0 * res[ii * 2 + 1] + res[(ii + 1) * 2]);
                }
                return r;
            };
            const auto& sz = fp.spec.sz;
            const auto& d = P.in.d;
            if (fp.real3D) {
                fp.incdConv[0] *= (sz[2] > 1 && sz[1] > 1) ? std::real(simps2DNorm(sz[1], sz[2], d[1], d[2])) : 0.0;
                fp.incdConv[1] *= (sz[0] > 1 && sz[2] > 1) ? std::real(simps2DNorm(sz[0], sz[2], d[0], d[2])) : 0.0;
                fp.incdConv[2] *= (sz[0] > 1 && sz[1] > 1) ? std::real(simps2DNorm(sz[0], sz[1], d[0], d[1])) : 0.0;
            } else {
                fp.incdConv[1] *= std::real(simps(sz[0], d[0]));
                fp.incdConv[0] *= std::real(simps(sz[1], d[1]));
                fp.incdConv[2] = 0.0;
            }
        }
    }
    return P;
}

}  // namespace chiml
