#include "outputs.hpp"

#include <algorithm>
#include <cmath>
#include <complex>
#include <exception>
#include <fstream>
#include <iomanip>
#include <memory>
#include <sys/stat.h>

namespace chiml {

std::string out_path(const std::string& outDir, const std::string& name) {
    std::string full = (outDir.empty() || (!name.empty() && name[0] == '/')) ? name : outDir + "/" + name;
    // create the parent directories, as the reader does for every output name
    std::size_t slash = full.find_last_of('/');
    if (slash != std::string::npos && slash > 0) {
        std::string dir = full.substr(0, slash);
        for (std::size_t i = 1; i <= dir.size(); ++i)
            if (i == dir.size() || dir[i] == '/') ::mkdir(dir.substr(0, i).c_str(), 0755);
    }
    return full;
}

long long detector_event_values(const DetectorPlan& dp) {
    long long n = 0;
    for (auto& f : dp.fields) n += static_cast<long long>(f.cells.size());
    return n;
}

int detector_events(const DetectorPlan& dp, int nSteps) { return nSteps / dp.timeInt + 1; }

namespace {

// Field value accumulation of fieldOutputFunction / pwrOutputFunction
// (DTC/parallelDTCOutputFxn.hpp:22-40).
inline double accum(double cur, double pt, double conv, bool power) {
    return power ? cur + conv * std::pow(std::abs(pt), 2.0) : cur + conv * pt;
}

}  // namespace

void write_detectors(const Plan& P, const RunRecord& R, const std::string& outDir, int stepsDone) {
    for (std::size_t k = 0; k < P.detectors.size(); ++k) {
        const DetectorPlan& dp = P.detectors[k];
        const auto& ev = R.detectors[k];
        const int nev = std::min(static_cast<int>(ev.size()), stepsDone / dp.timeInt + 1);
        std::vector<long long> base(dp.fields.size(), 0);
        for (std::size_t f = 1; f < dp.fields.size(); ++f) base[f] = base[f - 1] + static_cast<long long>(dp.fields[f - 1].cells.size());
        const std::string path = out_path(outDir, dp.spec.name);
        const double half = dp.convFactor / 2.0;
        if (dp.spec.cls == DtcClass::TXT) {
            std::ofstream os(path);
            if (!os) throw InputError("cannot open detector output " + path);
            os << "# time\tx\ty\tz\tfield" << std::endl;
            const auto& o0 = dp.fields[0].outSz;
            for (int e = 0; e < nev; ++e) {
                const std::vector<double>& v = ev[e];
                double t = P.tcur[static_cast<std::size_t>(e) * dp.timeInt];
                os << std::setprecision(6) << t * dp.tConv << "\t" << dp.realLoc[0] << "\t" << dp.realLoc[1] << "\t"
                   << dp.realLoc[2];
                for (int jj = 0; jj < o0[1]; ++jj)
                    for (int kk = 0; kk < o0[2]; ++kk)
                        for (int ii = 0; ii < o0[0]; ++ii) {
                            double point = 0.0;
                            for (std::size_t f = 0; f < dp.fields.size(); ++f) {
                                const auto& F = dp.fields[f];
                                const auto& s = F.outSz;
                                long long i0 = ii + s[0] * (kk + s[2] * static_cast<long long>(jj));
                                long long i1 = (ii + std::abs(F.off[0])) + s[0] * ((kk + std::abs(F.off[2])) + s[2] * static_cast<long long>(jj + std::abs(F.off[1])));
                                point = accum(point, v[base[f] + i0], half, dp.power);
                                point = accum(point, v[base[f] + i1], half, dp.power);
                            }
                            os << "\t" << std::setw(24) << std::setprecision(18) << point;
                        }
                os << '\n';
            }
        } else {
            std::ofstream os(path, std::ios::out | std::ios::binary);
            if (!os) throw InputError("cannot open detector output " + path);
            os.write(reinterpret_cast<const char*>(dp.spec.sz.data()), 3 * sizeof(int));
            os.write(reinterpret_cast<const char*>(dp.spec.loc.data()), 3 * sizeof(int));
            const auto& sz = dp.spec.sz;
            std::vector<double> row(static_cast<std::size_t>(sz[0]), 0.0);
            for (int e = 0; e < nev; ++e) {
                const std::vector<double>& v = ev[e];
                double tt = P.tcur[static_cast<std::size_t>(e) * dp.timeInt] * dp.tConv;
                os.write(reinterpret_cast<const char*>(&tt), sizeof(tt));
                for (int kk = 0; kk < sz[2]; ++kk)
                    for (int jj = 0; jj < sz[1]; ++jj) {
                        std::fill(row.begin(), row.end(), 0.0);
                        for (std::size_t f = 0; f < dp.fields.size(); ++f) {
                            const auto& F = dp.fields[f];
                            const auto& s = F.outSz;
                            std::array<int, 3> ao = {std::abs(F.off[0]), std::abs(F.off[1]), std::abs(F.off[2])};
                            for (int x = 0; x < sz[0]; ++x) {
                                long long i0 = x + s[0] * (kk + s[2] * static_cast<long long>(jj));
                                row[x] = accum(row[x], v[base[f] + i0], half, dp.power);
                            }
                            for (int x = 0; x < sz[0]; ++x) {
                                long long i1 = (x + ao[0]) + s[0] * ((kk + ao[2]) + s[2] * static_cast<long long>(jj + ao[1]));
                                row[x] = accum(row[x], v[base[f] + i1], half, dp.power);
                            }
                        }
                        os.write(reinterpret_cast<const char*>(row.data()), static_cast<std::streamsize>(row.size() * sizeof(double)));
                    }
            }
        }
    }
}

namespace {

typedef std::complex<double> cx;

// simps (parallelFlux.hpp:548-576)
cx simps(const cx* v, int n, double d) {
    if (n == 1) return v[0] * d;
    cx r(0.0, 0.0);
    if (n % 2 == 0) {
        for (int ii = 0; ii < (n - 2) / 2; ii++) r += d / 6.0 * (v[ii * 2] + 4.0 * v[ii * 2 + 1] + v[(ii + 1) * 2]);
        for (int ii = 1; ii < (n) / 2; ii++) r += d / 6.0 * (v[ii * 2 - 1] + 4.0 * v[ii * 2] + v[ii * 2 + 1]);
        r += d / 4.0 * (v[0] + v[1] + v[n - 1] + v[n - 2]);
    } else {
        for (int ii = 0; ii < (n - 1) / 2; ii++) r += d / 3.0 * (v[ii * 2] + 4.0 * v[ii * 2 + 1] + v[(ii + 1) * 2]);
    }
    return r;
}

struct CGrid {  // Grid<cplx> with dims (x, y, z), index x + nx*(z + y*nz)
    int nx = 0, ny = 0, nz = 0;
    double dx = 0, dy = 0, dz = 0;
    std::vector<cx> v;
    CGrid(int x, int y, int z, double ddx, double ddy, double ddz)
        : nx(x), ny(y), nz(z), dx(ddx), dy(ddy), dz(ddz), v(static_cast<std::size_t>(x) * y * z, cx(0.0, 0.0)) {}
    cx& at(int x, int y, int z) {
        if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz)
            throw InputError("flux combination index out of range (the reference asserts here)");
        return v[static_cast<std::size_t>(x) + static_cast<std::size_t>(nx) * (z + static_cast<std::size_t>(nz) * y)];
    }
};

// simps2D (parallelFlux.hpp:578-597) on a (x, y) grid
cx simps2D(CGrid& g) {
    if (g.ny > 1 && g.nx > 1) {
        std::vector<cx> res(static_cast<std::size_t>(g.ny), 0.0);
        for (int jj = 0; jj < g.ny; ++jj) res[jj] = simps(&g.at(0, jj, 0), g.nx, g.dx);
        return simps(res.data(), static_cast<int>(res.size()), g.dy);
    } else if (g.nx > 1) {
        return simps(&g.at(0, 0, 0), g.nx, g.dx);
    } else if (g.ny > 1) {
        return simps(&g.at(0, 0, 0), g.ny, g.dy);
    }
    throw UnsupportedError("a single-point flux face has no defined integral in the reference");
}

}  // namespace

std::vector<double> simps_weights(int n, double d) {
    std::vector<double> w(static_cast<std::size_t>(std::max(n, 0)), 0.0);
    if (n == 1) {
        w[0] = d;
    } else if (n % 2 == 0) {
        for (int ii = 0; ii < (n - 2) / 2; ii++) {
            w[ii * 2] += d / 6.0;
            w[ii * 2 + 1] += d / 6.0 * 4.0;
            w[(ii + 1) * 2] += d / 6.0;
        }
        for (int ii = 1; ii < n / 2; ii++) {
            w[ii * 2 - 1] += d / 6.0;
            w[ii * 2] += d / 6.0 * 4.0;
            w[ii * 2 + 1] += d / 6.0;
        }
        for (int k : {0, 1, n - 1, n - 2}) w[k] += d / 4.0;
    } else {
        for (int ii = 0; ii < (n - 1) / 2; ii++) {
            w[ii * 2] += d / 3.0;
            w[ii * 2 + 1] += d / 3.0 * 4.0;
            w[(ii + 1) * 2] += d / 3.0;
        }
    }
    return w;
}

std::vector<FluxFaceMap> flux_face_maps(const Plan& P, std::size_t q) {
    const Dims& D = P.dims;
    auto lnv = [&](int ax) { return ax == 0 ? D.lx : (ax == 1 ? D.ly : D.lz); };
    const FluxPlan& fp = P.fluxes[q];
    const auto& loc_ = fp.spec.loc;
    // the faces are independent: built in parallel, kept in face order
    std::vector<FluxFaceMap> maps(fp.faces.size());
    std::vector<std::exception_ptr> faceErr(fp.faces.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (long long fi = 0; fi < static_cast<long long>(fp.faces.size()); ++fi) try {
        const FluxFace& f = fp.faces[static_cast<std::size_t>(fi)];
        FluxFaceMap& m = maps[static_cast<std::size_t>(fi)];
        // the face grids are (freq, y = faceSz[transCor1], z = faceSz[cor]); the product grid
        // of the integration is (x = faceSz[cor], y = faceSz[transCor1])
        m.nx = f.faceSz[f.cor];
        m.ny = f.faceSz[f.transCor1];
        m.dx = P.in.d[f.cor];
        m.dy = P.in.d[f.transCor1];
        m.sz = f.sz;
        m.pref = fp.fluxConv * f.weight;
        if (static_cast<long long>(m.sz) > static_cast<long long>(m.nx) * m.ny)
            throw InputError("flux face larger than its integration grid");
        const long long npt = static_cast<long long>(m.nx) * m.ny;
        std::array<int, 2> addIndex = {std::max(0, 0 - loc_[f.transCor1]), std::max(0, 0 - loc_[f.cor])};
        const std::vector<int>* lists[4] = {&f.Ej, &f.Ek, &f.Hj, &f.Hk};
        int ej, ek, hj, hk;
        if (f.corI == 0) { ej = EY; hj = HY; ek = EZ; hk = HZ; }
        else if (f.corI == 1) { ej = EZ; hj = HZ; ek = EX; hk = HX; }
        else { ej = EX; hj = HX; ek = EY; hk = HY; }
        const int comps[4] = {ej, ek, hj, hk};
        const int oth[4] = {1, 0, 3, 2};
        for (int w = 0; w < 4; ++w) {
            if (lists[w]->empty()) continue;
            m.has[w] = true;
            // act / trans fields and the J/K coordinate of constructSzProcOffsetLists (Real
            // flux): the complementary field exists when its component is present
            const int corJK = (w == 0 || w == 3) ? f.corJ : f.corK;
            const bool act = P.comp[comps[w]].present;
            const bool trans = P.comp[comps[oth[w]]].present;
            const std::vector<int>& lst = *lists[w];
            const double scaleDen = static_cast<double>(lst.size());
            // every (grid point, accumulator point, scale) term in the reference's order,
            // visited twice: to count the terms per grid point, then to place them
            auto visit = [&](auto&& fn) {
            for (std::size_t dd = 0; dd < lst.size(); ++dd) {
                const FreqStore& st = fp.stores[lst[dd]];
                if (st.outN[0] == 0) continue;  // outside the grid: no out grid
                std::vector<std::array<int, 9>> so;
                const int oy = st.outN[1], oz = st.outN[2];
                if (act && trans) {
                    so.assign(2, {0, oy, oz, 0, 0, 0, 0, 0, 0});
                    if (f.cor == corJK) {
                        if (addIndex[1] == 0) {
                            so[1][6] = 1;
                            so[1][4] = 1;
                        } else {
                            so[0][8] = 1;
                        }
                        if ((0 <= st.loc[corJK] + st.sz[corJK] - 1) && (st.loc[corJK] + st.sz[corJK] - 1 < lnv(corJK) - 2)) so[0][4] = 1;
                    } else if (f.transCor1 == corJK) {
                        if (addIndex[0] == 0) {
                            so[1][5] = 1;
                            so[1][3] = 1;
                        } else {
                            so[0][7] = 1;
                        }
                        if ((0 <= st.loc[corJK] + st.sz[corJK] - 1) && (st.loc[corJK] + st.sz[corJK] - 1 < lnv(corJK) - 2)) so[0][3] = 1;
                    }
                } else {
                    so.assign(1, {0, oy, oz, 0, 0, 0, 0, 0, 0});
                }
                const double scale = 1.0 / (scaleDen * static_cast<double>(so.size()));
                for (auto& o : so)
                    for (int jj = 0; jj < o[2] - o[4]; ++jj)
                        for (int ii = 0; ii < o[1] - o[3]; ++ii) {
                            const long long pt = st.accOffset + (jj + o[6]) + static_cast<long long>(ii + o[5]) * oz;
                            const int y = ii + addIndex[0] + o[7], z = jj + addIndex[1] + o[8];
                            if (y < 0 || z < 0 || y >= m.ny || z >= m.nx)
                                throw InputError("flux combination index out of range (the reference asserts here)");
                            fn(z + static_cast<long long>(m.nx) * y, pt, scale);
                        }
            }
            };
            std::vector<long long>& start = m.start[w];
            start.assign(static_cast<std::size_t>(npt) + 1, 0);
            visit([&](long long c, long long, double) { ++start[static_cast<std::size_t>(c) + 1]; });
            for (long long c = 0; c < npt; ++c) start[c + 1] += start[c];
            m.pt[w].resize(static_cast<std::size_t>(start[npt]));
            m.scale[w].resize(static_cast<std::size_t>(start[npt]));
            std::vector<long long> cursor(start.begin(), start.end() - 1);
            visit([&](long long c, long long pt, double scale) {
                const long long k = cursor[static_cast<std::size_t>(c)]++;
                m.pt[w][k] = pt;
                m.scale[w][k] = scale;
            });
        }
        // getFlux pairs the E grid with the complementary H grid: Ej with Hk, Ek with Hj
        if (!(m.has[0] || m.has[1]) || (m.has[0] && !m.has[3]) || (!m.has[0] && !m.has[2]) || (m.has[1] && !m.has[2]))
            throw InputError("flux face without field pairs");
        if (m.nx <= 1 && m.ny <= 1) throw UnsupportedError("a single-point flux face has no defined integral in the reference");
        m.wx = m.nx > 1 ? simps_weights(m.nx, m.dx) : std::vector<double>(1, 1.0);
        m.wy = m.ny > 1 ? simps_weights(m.ny, m.dy) : std::vector<double>(1, 1.0);
    } catch (...) {
        faceErr[static_cast<std::size_t>(fi)] = std::current_exception();
    }
    for (auto& e : faceErr)
        if (e) std::rethrow_exception(e);
    return maps;
}

std::vector<cplx> flux_face_values(const Plan& P, std::size_t q, const std::vector<FluxFaceMap>& maps,
                                   const std::vector<double>& re, const std::vector<double>& im, int nt,
                                   const FluxGrids* seed, FluxGrids* grids) {
    const FluxPlan& fp = P.fluxes[q];
    const int nfreq = static_cast<int>(fp.spec.freqList.size());
    const std::size_t nFaces = maps.size();
    std::vector<cplx> out(static_cast<std::size_t>(nfreq) * nFaces, cplx(0.0, 0.0));
    const double nt2 = std::pow(static_cast<double>(nt), 2.0);
    for (std::size_t vv = 0; vv < nFaces; ++vv) {
        const FluxFaceMap& m = maps[vv];
        const long long npt = static_cast<long long>(m.nx) * m.ny;
        // the face grids [point][freq], summed in the reference's order
        std::vector<cx> g[4];
        for (int w = 0; w < 4; ++w) {
            if (!m.has[w]) continue;
            if (seed) g[w] = (*seed)[vv][w];  // the grid starts from the loaded field (loadFields)
            else g[w].assign(static_cast<std::size_t>(npt) * nfreq, cx(0.0, 0.0));
#pragma omp parallel for schedule(static)
            for (long long c = 0; c < npt; ++c)
                for (long long k = m.start[w][c]; k < m.start[w][c + 1]; ++k) {
                    const std::size_t b = static_cast<std::size_t>(m.pt[w][k]) * nfreq;
                    for (int fq = 0; fq < nfreq; ++fq)
                        g[w][static_cast<std::size_t>(c) * nfreq + fq] += m.scale[w][k] * cx(re[b + fq], im[b + fq]);
                }
        }
        if (grids) {
            if (grids->size() < nFaces) grids->resize(nFaces);
            for (int w = 0; w < 4; ++w) (*grids)[vv][w] = g[w];
        }
        const cx* Ej = m.has[0] ? g[0].data() : nullptr;
        const cx* Ek = m.has[1] ? g[1].data() : nullptr;
        const cx* Hj = m.has[2] ? g[2].data() : nullptr;
        const cx* Hk = m.has[3] ? g[3].data() : nullptr;
#pragma omp parallel for schedule(dynamic, 1)
        for (int ff = 0; ff < nfreq; ++ff) {
            CGrid ijk(m.nx, m.ny, 1, m.dx, m.dy, 1.0);
            CGrid ikj(ijk.nx, ijk.ny, 1, ijk.dx, ijk.dy, 1.0);
            if (Ej)
                for (int s = 0; s < m.sz; ++s) {
                    cx e = Ej[static_cast<std::size_t>(ff) + static_cast<std::size_t>(nfreq) * s];
                    cx h = Hk[static_cast<std::size_t>(ff) + static_cast<std::size_t>(nfreq) * s];
                    ijk.v[s] = e * std::conj(h) / nt2;
                }
            if (Ek) {
                for (int s = 0; s < m.sz; ++s) {
                    cx e = Ek[static_cast<std::size_t>(ff) + static_cast<std::size_t>(nfreq) * s];
                    cx h = Hj[static_cast<std::size_t>(ff) + static_cast<std::size_t>(nfreq) * s];
                    ikj.v[s] = e * std::conj(h) / nt2;
                }
                for (std::size_t s = 0; s < ijk.v.size(); ++s) ijk.v[s] += cx(-1.0) * ikj.v[s];
            }
            out[static_cast<std::size_t>(ff) * nFaces + vv] = fp.fluxConv * fp.faces[vv].weight * simps2D(ijk);
        }
    }
    return out;
}

namespace {

// n_vec of a face grid as the reference's Grid holds it: {nfreq, transCor1 points, cor points}
std::array<int, 3> flux_grid_dims(int nfreq, const FluxFaceMap& m) { return {nfreq, m.ny, m.nx}; }

}  // namespace

void write_flux_fields(const Plan& P, std::size_t q, const std::vector<FluxFaceMap>& maps, const FluxGrids& grids,
                       const std::string& path) {
    const FluxPlan& fp = P.fluxes[q];
    const int nfreq = static_cast<int>(fp.spec.freqList.size());
    for (std::size_t vv = 0; vv < maps.size(); ++vv)
        for (int w = 0; w < 4; ++w)
            if (!maps[vv].has[w])
                throw UnsupportedError("saving the fields of a flux face without all four field grids (the reference "
                                       "dereferences the missing grid)");
    std::ofstream f(path, std::ios::binary | std::ios::out);
    if (!f) throw InputError("cannot open flux fields output " + path);
    auto put = [&](int v) { f.write(reinterpret_cast<const char*>(&v), sizeof(v)); };
    put(nfreq);
    for (int k = 0; k < 3; ++k) put(fp.spec.sz[k]);
    const int nFaces = static_cast<int>(maps.size());
    for (int w = 0; w < 4; ++w) put(nFaces);
    for (int w = 0; w < 4; ++w)
        for (std::size_t vv = 0; vv < maps.size(); ++vv) {
            const std::array<int, 3> n = flux_grid_dims(nfreq, maps[vv]);
            for (int k = 0; k < 3; ++k) put(n[k]);
            const std::vector<cplx>& g = grids[vv][w];
            f.write(reinterpret_cast<const char*>(g.data()), static_cast<std::streamsize>(g.size() * sizeof(cplx)));
        }
}

FluxGrids read_flux_fields(const Plan& P, std::size_t q, const std::vector<FluxFaceMap>& maps, const std::string& path,
                           double weight) {
    const FluxPlan& fp = P.fluxes[q];
    const int nfreq = static_cast<int>(fp.spec.freqList.size());
    std::ifstream f(path, std::ios::binary | std::ios::in);
    if (!f) throw InputError("cannot open the flux fields file " + path);
    auto get = [&]() {
        int v = 0;
        if (!f.read(reinterpret_cast<char*>(&v), sizeof(v))) throw InputError("flux fields file " + path + " is truncated");
        return v;
    };
    const int nf = get(), nx = get(), ny = get(), nz = get();
    int counts[4];
    for (int w = 0; w < 4; ++w) counts[w] = get();
    if (nf != nfreq || nx != fp.spec.sz[0] || ny != fp.spec.sz[1] || nz != fp.spec.sz[2])
        throw InputError("Given incident fields do not match size and frequency numbers for the current calculations");
    for (int w = 0; w < 4; ++w)
        if (counts[w] != static_cast<int>(maps.size()))
            throw InputError("The size of the field vectors of the saved fields are not the same as those in the current calculation");
    FluxGrids g(maps.size());
    static const char* names[4] = {"Ej_freq_", "Ek_freq_", "Hj_freq_", "Hk_freq_"};
    for (int w = 0; w < 4; ++w)
        for (std::size_t vv = 0; vv < maps.size(); ++vv) {
            const std::array<int, 3> n = flux_grid_dims(nfreq, maps[vv]);
            for (int k = 0; k < 3; ++k)
                if (get() != n[k])
                    throw InputError(std::string("When loading in a ") + names[w] +
                                     " field in a flux region, one of the size elements did not agree with the file.");
            std::vector<cplx>& v = g[vv][w];
            v.assign(static_cast<std::size_t>(n[0]) * n[1] * n[2], cplx(0.0, 0.0));
            if (!f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(cplx))))
                throw InputError("flux fields file " + path + " is truncated");
            for (cplx& x : v) x *= weight;
            if (!maps[vv].has[w]) v.clear();
        }
    return g;
}

void write_fluxes(const Plan& P, const RunRecord& R, const std::string& outDir) {
    for (std::size_t q = 0; q < P.fluxes.size(); ++q) {
        const FluxPlan& fp = P.fluxes[q];
        const int nfreq = static_cast<int>(fp.spec.freqList.size());
        const std::size_t nFaces = fp.faces.size();
        std::vector<cplx> faceVal;
        FluxGrids saved;
        if (fp.spec.save || fp.spec.load) {
            // the face grids start from minus the loaded incident field (parallelFlux.cpp:69-70,
            // loadFields(-1.0)) and are written after the flux (parallelFlux.hpp:535-536)
            if (q >= R.fluxRe.size() || R.fluxRe[q].empty())
                throw std::logic_error("flux save or load needs the accumulators on the host");
            const std::vector<FluxFaceMap> maps = flux_face_maps(P, q);
            FluxGrids seed;
            if (fp.spec.load) seed = read_flux_fields(P, q, maps, out_path(outDir, fp.spec.incdFile), -1.0);
            faceVal = flux_face_values(P, q, maps, R.fluxRe[q], R.fluxIm[q], R.fluxSamples[q], fp.spec.load ? &seed : nullptr,
                                       fp.spec.save ? &saved : nullptr);
        } else if (q < R.fluxFaces.size() && !R.fluxFaces[q].empty()) {
            faceVal = R.fluxFaces[q];
        } else {
            faceVal = flux_face_values(P, q, flux_face_maps(P, q), R.fluxRe[q], R.fluxIm[q], R.fluxSamples[q]);
        }
        if (faceVal.size() != static_cast<std::size_t>(nfreq) * nFaces) throw InputError("flux face values of the wrong size");
        const int nt = R.fluxSamples[q];
        // transform of the recorded incident fields (zero without a TFSF surface): the even
        // samples, then the odd ones, real parts only (parallelFlux.hpp:457-479)
        std::vector<cx> incd(static_cast<std::size_t>(nfreq));
        const std::vector<cplx>* incSer[6] = {&R.incE[0], &R.incE[1], &R.incE[2], &R.incH[0], &R.incH[1], &R.incH[2]};
        const std::size_t nInc = incSer[0]->size();
        const double tInt = static_cast<double>(fp.spec.timeInt);
#pragma omp parallel for schedule(dynamic, 1)
        for (int ff = 0; ff < nfreq; ++ff) {
            cx inc[6] = {0, 0, 0, 0, 0, 0};
            for (int start = 0; start < 2; ++start)
                for (std::size_t tt = start; tt < nInc; tt += 2) {
                    const cx ph = std::exp(cx(0.0, fp.spec.freqList.at(ff) * static_cast<double>(tt / 2) * (P.dt / tInt)));
                    for (int c = 0; c < 6; ++c) inc[c] += cx(std::real(0.5 * (*incSer[c])[tt]), 0.0) * ph;
                }
            cx flux_incd = std::pow(fp.incdConv[0] * (inc[1] * std::conj(inc[5]) - inc[2] * std::conj(inc[4])) /
                                        (std::pow(static_cast<double>(nt * fp.spec.timeInt), 2.0)), 2.0);
            flux_incd += std::pow(fp.incdConv[1] * (inc[2] * std::conj(inc[3]) - inc[0] * std::conj(inc[5])) /
                                      (std::pow(static_cast<double>(nt * fp.spec.timeInt), 2.0)), 2.0);
            flux_incd += std::pow(fp.incdConv[2] * (inc[0] * std::conj(inc[4]) - inc[1] * std::conj(inc[3])) /
                                      (std::pow(static_cast<double>(nt * fp.spec.timeInt), 2.0)), 2.0);
            incd[ff] = std::sqrt(flux_incd);
        }
        // getFlux output (parallelFlux.hpp:406-545)
        const std::string path = out_path(outDir, fp.spec.name + ".dat");
        std::ofstream f(path);
        if (!f) throw InputError("cannot open flux output " + path);
        f << "#" << std::setw(16) << "freq\tabs(incd)\treal(incd)\timag(incd)";
        if (nFaces > 1) {
            f << std::setw(16) << "\tabs(right)\treal(right)\timag(right)\tabs(left)\treal(left)\timag(left)\tabs(top)\treal(top)\timag(top)\tabs(bot)\treal(bot)\timag(bot)";
            if (fp.spec.sz[0] > 1 && fp.spec.sz[1] > 1 && fp.spec.sz[2] > 1)
                f << std::setw(16) << "\tabs(front)\treal(front)\timag(front)\tabs(back)\treal(back)\timag(back)";
        }
        f << std::setw(16) << "freq\tabs(total)\treal(total)\timag(total)\n";
        for (int ff = 0; ff < nfreq; ++ff) {
            const cx flux_incd = incd[ff];
            f << std::setw(18) << std::setprecision(15) << fp.freqConv * fp.spec.freqList[ff] << "\t" << std::setw(16)
              << std::setprecision(15) << std::abs(flux_incd) << "\t" << std::setw(16) << std::setprecision(15)
              << std::abs(std::real(flux_incd)) << "\t" << std::setw(16) << std::setprecision(15) << std::imag(flux_incd)
              << "\t";
            cx flux = 0.0;
            for (std::size_t vv = 0; vv < nFaces; ++vv) {
                const cx tempFlux = faceVal[static_cast<std::size_t>(ff) * nFaces + vv];
                flux += tempFlux;
                f << std::setw(16) << std::setprecision(15) << std::abs(tempFlux) << "\t" << std::setw(16)
                  << std::setprecision(15) << std::real(tempFlux) << "\t" << std::setw(16) << std::setprecision(15)
                  << std::imag(tempFlux) << "\t";
            }
            if (nFaces > 1)
                f << std::setw(16) << std::setprecision(15) << std::abs(flux) << "\t" << std::setw(16) << std::setprecision(15)
                  << std::real(flux) << "\t" << std::setw(16) << std::setprecision(15) << std::imag(flux) << std::endl;
            else
                f << std::endl;
        }
        f.close();
        if (fp.spec.save) write_flux_fields(P, q, flux_face_maps(P, q), saved, out_path(outDir, fp.spec.name + "_fields.dat"));
    }
}

void write_emitters(const Plan& P, const RunRecord& R, const std::string& outDir) {
    for (std::size_t q = 0; q < P.emitters.size(); ++q) {
        const EmitterPlan& e = P.emitters[q];
        if (e.outputPol && q < R.emitterP.size()) {
            const auto& tp = R.emitterP[q];
            std::ofstream f(out_path(outDir, e.polFile));
            if (!f) throw std::runtime_error("cannot open " + e.polFile);
            const std::size_t iterMax = std::max(tp[0].size(), tp[2].size());
            for (std::size_t ii = 0; ii < iterMax; ++ii) {
                f << e.dt * static_cast<double>(ii);
                double px = 0, py = 0, pz = 0;
                if (!tp[0].empty()) {
                    px += tp[0][ii];
                    py += tp[1][ii];
                    f << '\t' << px << '\t' << py;
                }
                if (!tp[2].empty()) {
                    pz += tp[2][ii];
                    f << '\t' << pz;
                }
                f << '\t' << std::sqrt(std::pow(px, 2) + std::pow(py, 2) + std::pow(pz, 2)) << '\n';
            }
        }
        for (std::size_t d = 0; d < e.dtcFiles.size() && q < R.emitterPop.size() && d < R.emitterPop[q].size(); ++d) {
            std::ofstream f(out_path(outDir, e.dtcFiles[d]));
            if (!f) throw std::runtime_error("cannot open " + e.dtcFiles[d]);
            const auto& pop = R.emitterPop[q][d];
            for (std::size_t tt = 0; tt < pop.size(); ++tt) {
                const cplx v = pop[tt];
                f << std::setw(9) << std::setprecision(9) << static_cast<double>(tt) * e.dtcTimeInt * e.dt << "\t"
                  << std::setw(16) << std::setprecision(16) << std::real(v) << "\t" << std::setw(16)
                  << std::setprecision(16) << std::imag(v) << "\t" << std::setw(16) << std::setprecision(16)
                  << std::abs(v) << std::endl;
            }
        }
    }
}

void write_freq_detectors(const Plan& P, const RunRecord& R, const std::string& outDir) {
    typedef std::complex<double> cx;
    for (std::size_t k = 0; k < P.freqDetectors.size(); ++k) {
        const DetectorPlan& dp = P.freqDetectors[k];
        const DetectorSpec& ds = dp.spec;
        const std::vector<double>& fl = ds.freqList;
        const int nfreq = static_cast<int>(fl.size());
        const long long szFreq = dp.szFreq;
        const int nt = R.freqSamples[k];
        const int ti = dp.timeInt;
        // the collected fields, transposed: [field][point][freq] (fieldTranspose)
        std::vector<std::vector<cx>> trans;
        long long off = 0;
        for (const auto& F : dp.fields) {
            std::vector<cx> g(static_cast<std::size_t>(szFreq) * nfreq, cx(0.0, 0.0));
            for (std::size_t p = 0; p < F.cells.size(); ++p)
                for (int f = 0; f < nfreq; ++f) {
                    const std::size_t a = static_cast<std::size_t>(off + static_cast<long long>(p)) * nfreq + f;
                    g[p + static_cast<std::size_t>(szFreq) * f] = cx(R.freqRe[k][a], R.freqIm[k][a]);
                }
            off += static_cast<long long>(F.cells.size());
            trans.push_back(std::move(g));
        }
        // the incident fields main.cpp passes for the detector type
        std::vector<const std::vector<cplx>*> incd;
        switch (ds.type) {
            case DtcType::HPOW: incd = {&R.incH[0], &R.incH[1], &R.incH[2]}; break;
            case DtcType::EPOW: incd = {&R.incE[0], &R.incE[1], &R.incE[2]}; break;
            case DtcType::EX: incd = {&R.incE[0]}; break;
            case DtcType::EY: incd = {&R.incE[1]}; break;
            case DtcType::EZ: incd = {&R.incE[2]}; break;
            case DtcType::HX: incd = {&R.incH[0]}; break;
            case DtcType::HY: incd = {&R.incH[1]}; break;
            case DtcType::HZ: incd = {&R.incH[2]}; break;
            default: break;
        }
        const double conv = dp.convFactor / 2.0;
        // toOutFile_: fieldOutFreqFunction / pwrOutFreqFunction (DTC/parallelDTCOutputFxn.cpp:9-18)
        auto out = [&](const cx* col, long long n) {
            cx sum(0.0, 0.0);
            if (dp.power) {
                for (long long p = 0; p < n; ++p) sum += col[p] * std::conj(col[p]);
                return conv * sum / std::pow(static_cast<double>(nt), 2.0);
            }
            for (long long p = 0; p < n; ++p) sum += col[p];
            return conv * sum / std::pow(static_cast<double>(nt), 1.0);
        };
        // incident spectra: even samples, then odd ones, real parts (parallelDTC_FREQ.hpp:416-428)
        auto incident = [&](int ii) {
            std::vector<cx> pts;
            for (const std::vector<cplx>* field : incd) {
                cx pt(0.0, 0.0);
                for (int start = 0; start < 2; ++start)
                    for (std::size_t tt = start; tt < field->size(); tt += 2)
                        pt += std::real(0.5 * (*field)[tt]) *
                              std::exp(cx(0.0, -1.0 * fl[ii] * static_cast<double>(tt / 2) * (P.dt / static_cast<double>(ti))));
                pt /= static_cast<double>(nt * ti);
                if (dp.power) pt *= std::conj(pt);
                pt *= dp.convFactor / 2.0;
                pts.push_back(pt);
            }
            return pts;
        };
        const std::size_t nField = trans.size();
        if (!ds.outputMaps) {
            const std::string path = out_path(outDir, ds.name);
            std::ofstream f(path);
            if (!f) throw InputError("cannot open detector output " + path);
            f << "#" << std::setw(16) << "freq\tabs(incd)\treal(incd)\timag(incd)";
            for (std::size_t nn = 1; nn < nField; ++nn) f << "\tabs(field " << nn << ")\treal(field " << nn << ")\timag(field " << nn << ")";
            if (nField > 1) f << "\tabs(total)\treal(total)\timag(total)";
            f << std::endl;
            for (int ii = 0; ii < nfreq; ++ii) {
                f << std::setw(16) << std::setprecision(12) << dp.freqConv * fl[ii];
                cx incdField(0.0, 0.0);
                for (const cx& pt : incident(ii)) {
                    f << "\t" << std::setw(16) << std::setprecision(12) << std::real(pt) << "\t" << std::setw(16)
                      << std::setprecision(12) << std::imag(pt) << "\t" << std::setw(16) << std::setprecision(12) << std::abs(pt);
                    incdField += pt;
                }
                if (incd.size() > 2)
                    f << "\t" << std::setw(16) << std::setprecision(12) << std::real(incdField) << "\t" << std::setw(16)
                      << std::setprecision(12) << std::imag(incdField) << "\t" << std::setw(16) << std::setprecision(12)
                      << std::abs(incdField);
                cx freq(0.0, 0.0);
                for (const auto& g : trans) {
                    const cx pt = out(&g[static_cast<std::size_t>(szFreq) * ii], szFreq);
                    f << "\t" << std::setw(16) << std::setprecision(12) << std::real(pt) << "\t" << std::setw(16)
                      << std::setprecision(12) << std::imag(pt) << "\t" << std::setw(16) << std::setprecision(12) << std::abs(pt);
                    freq += pt;
                }
                if (nField > 1)
                    f << '\t' << std::setw(16) << std::setprecision(12) << std::real(freq) << "\t" << std::setw(16)
                      << std::setprecision(12) << std::imag(freq) << "\t" << std::setw(16) << std::setprecision(12) << std::abs(freq)
                      << std::endl;
                else
                    f << "\n";
            }
        } else {
            for (int ii = 0; ii < nfreq; ++ii) {
                const std::string path = out_path(outDir, ds.name + "." + std::to_string(dp.freqConv * fl[ii]));
                std::ofstream f(path);
                if (!f) throw InputError("cannot open detector output " + path);
                f << "#" << std::setw(16) << "x\ty\tz\tabs(incd)\treal(incd)\timag(incd)";
                for (std::size_t nn = 1; nn < nField; ++nn) f << "\tabs(field " << nn << ")\treal(field " << nn << ")\timag(field " << nn << ")";
                if (nField > 1) f << "\tabs(total)\treal(total)\timag(total)";
                f << std::endl;
                std::vector<double> outIncd;
                cx incdField(0.0, 0.0);
                for (const cx& pt : incident(ii)) {
                    outIncd.push_back(std::real(pt));
                    outIncd.push_back(std::imag(pt));
                    outIncd.push_back(std::abs(pt));
                    incdField += pt;
                }
                if (incd.size() > 2) {
                    outIncd.push_back(std::real(incdField));
                    outIncd.push_back(std::imag(incdField));
                    outIncd.push_back(std::abs(incdField));
                }
                for (int yy = 0; yy < ds.sz[1]; ++yy)
                    for (int zz = 0; zz < ds.sz[2]; ++zz)
                        for (int xx = 0; xx < ds.sz[0]; ++xx) {
                            f << std::setw(16) << xx << '\t' << yy << '\t' << zz;
                            for (double v : outIncd) f << "\t" << std::setw(16) << std::setprecision(12) << v;
                            const long long jj = xx + static_cast<long long>(zz) * ds.sz[0] + static_cast<long long>(yy) * ds.sz[0] * ds.sz[2];
                            cx freq(0.0, 0.0);
                            for (const auto& g : trans) {
                                const cx pt = out(&g[static_cast<std::size_t>(szFreq) * ii + jj], 1);
                                f << "\t" << std::setw(16) << std::setprecision(12) << std::abs(pt) << "\t" << std::real(pt) << "\t"
                                  << std::imag(pt);
                                freq += pt;
                            }
                            if (nField > 1)
                                f << '\t' << std::setw(16) << std::setprecision(12) << std::real(freq) << "\t" << std::setw(16)
                                  << std::setprecision(12) << std::imag(freq) << "\t" << std::setw(16) << std::setprecision(12)
                                  << std::abs(freq) << std::endl;
                            else
                                f << "\n";
                        }
            }
        }
    }
}

}  // namespace chiml
