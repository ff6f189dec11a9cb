// The C ABI (include/chiml_gpu.h): builds the plan on the host, uploads it,
// drives the kernels per step (optionally as CUDA graphs of several steps),
// and writes the outputs at finalize.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/chiml_gpu.h"
#include "host/outputs.hpp"
#include "host/plan.hpp"
#include "kernels/fdtd_device.hpp"

using namespace chiml;

namespace {

thread_local std::string g_createError;

struct CudaError : public std::runtime_error {
    cudaError_t code;
    CudaError(cudaError_t c, const std::string& w) : std::runtime_error(w), code(c) {}
};

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(e, std::string(what) + ": " + cudaGetErrorString(e));
}

struct DevMem {
    std::vector<void*> ptrs;
    double bytes = 0;
    template <typename T>
    T* alloc(std::size_t n, bool zero = true) {
        if (n == 0) return nullptr;
        void* p = nullptr;
        ck(cudaMalloc(&p, n * sizeof(T)), "cudaMalloc");
        ptrs.push_back(p);
        bytes += static_cast<double>(n * sizeof(T));
        if (zero) ck(cudaMemset(p, 0, n * sizeof(T)), "cudaMemset");
        return static_cast<T*>(p);
    }
    template <typename T>
    T* upload(const std::vector<T>& v) {
        if (v.empty()) return nullptr;
        T* p = alloc<T>(v.size(), false);
        ck(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        h2d += static_cast<double>(v.size() * sizeof(T));
        return p;
    }
    double h2d = 0;
    ~DevMem() {
        for (void* p : ptrs) cudaFree(p);
    }
};

struct SimBase {
    virtual ~SimBase() {}
    virtual void step(long long n) = 0;
    virtual void finalize() = 0;
    virtual void getField(int comp, double* out) = 0;
    virtual void fillStats(chiml_stats* s) const = 0;
    virtual cudaStream_t stream() const = 0;
};

template <typename T>
class Sim : public SimBase {
public:
    Sim(Plan&& plan, const chiml_options& opt) : P(std::move(plan)), opt_(opt) {
        ck(cudaSetDevice(opt.device), "cudaSetDevice");
        ck(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        outDir_ = opt.out_dir ? opt.out_dir : "";
        upload();
    }
    ~Sim() override {
        if (graph_) cudaGraphExecDestroy(graph_);
        if (stream_) cudaStreamDestroy(stream_);
    }

    cudaStream_t stream() const override { return stream_; }

    void step(long long n) override {
        if (finalized_) throw std::logic_error("step after finalize");
        long long left = P.nSteps - stepsDone_;
        if (n > left) n = left;
        if (n <= 0) return;
        const int K = opt_.steps_per_graph;
        if (K > 0) {
            if (!graph_ && n >= K) buildGraph(K);
            while (n >= K && graph_) {
                ck(cudaGraphLaunch(graph_, stream_), "cudaGraphLaunch");
                n -= K;
                stepsDone_ += K;
            }
        }
        for (long long s = 0; s < n; ++s) {
            enqueueStep();
            ++stepsDone_;
        }
        ck(cudaGetLastError(), "kernel launch");
    }

    void finalize() override {
        ck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        RunRecord R;
        R.detectors.resize(P.detectors.size());
        std::vector<double> rec(recTotal_);
        if (recTotal_) ck(cudaMemcpy(rec.data(), dRec_, recTotal_ * sizeof(double), cudaMemcpyDeviceToHost), "D2H records");
        d2h_ += static_cast<double>(recTotal_ * sizeof(double));
        for (std::size_t k = 0; k < P.detectors.size(); ++k) {
            const DetectorPlan& dp = P.detectors[k];
            long long nv = detector_event_values(dp);
            int nev = std::min(detector_events(dp, P.nSteps), stepsDone_ / dp.timeInt + 1);
            for (int e = 0; e < nev; ++e) {
                const double* b = rec.data() + recBase_[k] + static_cast<long long>(e) * nv;
                R.detectors[k].emplace_back(b, b + nv);
            }
        }
        for (std::size_t q = 0; q < P.fluxes.size(); ++q) {
            const FluxPlan& fp = P.fluxes[q];
            std::size_t n = static_cast<std::size_t>(fp.npts) * fp.spec.freqList.size();
            std::vector<double> re(n), im(n);
            if (n) {
                ck(cudaMemcpy(re.data(), dft_[q].re, n * sizeof(double), cudaMemcpyDeviceToHost), "D2H flux");
                ck(cudaMemcpy(im.data(), dft_[q].im, n * sizeof(double), cudaMemcpyDeviceToHost), "D2H flux");
            }
            d2h_ += 2.0 * n * sizeof(double);
            R.fluxRe.push_back(std::move(re));
            R.fluxIm.push_back(std::move(im));
            R.fluxSamples.push_back(stepsDone_ / fp.spec.timeInt + 1);
        }
        write_detectors(P, R, outDir_, stepsDone_);
        write_fluxes(P, R, outDir_);
        finalized_ = true;
    }

    void getField(int comp, double* out) override {
        if (comp < 0 || comp > 8 || !fields_.f[comp]) throw std::invalid_argument("field not present");
        ck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        std::size_t N = static_cast<std::size_t>(P.dims.cells());
        if (std::is_same<T, double>::value) {
            ck(cudaMemcpy(out, fields_.f[comp], N * sizeof(double), cudaMemcpyDeviceToHost), "D2H field");
        } else {
            std::vector<T> tmp(N);
            ck(cudaMemcpy(tmp.data(), fields_.f[comp], N * sizeof(T), cudaMemcpyDeviceToHost), "D2H field");
            for (std::size_t i = 0; i < N; ++i) out[i] = static_cast<double>(tmp[i]);
        }
    }

    void fillStats(chiml_stats* s) const override {
        std::memset(s, 0, sizeof(*s));
        s->cells = P.dims.cells();
        s->cells_physical = static_cast<int64_t>(P.dims.nx) * P.dims.ny * P.dims.nz;
        s->nx = P.dims.nx;
        s->ny = P.dims.ny;
        s->nz = P.dims.nz;
        s->steps_total = P.nSteps;
        s->steps_done = stepsDone_;
        s->precision = std::is_same<T, double>::value ? CHIML_PREC_FP64 : CHIML_PREC_SPLIT;
        s->bytes_per_cell_update = bytesPerCell_;
        s->device_bytes = mem_.bytes;
        s->kernels_per_step = kernelsPerStep_;
    }

    double h2dBytes() const { return mem_.h2d; }
    double d2hBytes() const { return d2h_; }

private:
    Plan P;
    chiml_options opt_;
    std::string outDir_;
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
    DevMem mem_;
    dev::Pass<T> hPass_{}, ePass_{};
    dev::Fields<T> fields_{};
    dev::SourceTable src_{};
    dev::RecordTable recT_{};
    std::vector<dev::DftTable> dft_;
    std::vector<long long> recBase_;
    std::size_t recTotal_ = 0;
    double* dRec_ = nullptr;
    int* dStep_ = nullptr;
    int stepsDone_ = 0;
    bool finalized_ = false;
    double d2h_ = 0;
    double bytesPerCell_ = 0;
    int kernelsPerStep_ = 0;

    void enqueueStep() {
        void* s = stream_;
        dev::launch_pass<T>(hPass_, false, s);
        dev::launch_sources<T>(src_, fields_, dStep_, s);
        dev::launch_pass<T>(ePass_, true, s);
        dev::launch_increment(dStep_, s);
        dev::launch_record<T>(recT_, fields_, dStep_, s);
        for (auto& d : dft_) dev::launch_dft<T>(d, fields_, dStep_, s);
    }

    void buildGraph(int K) {
        cudaGraph_t g;
        ck(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        for (int k = 0; k < K; ++k) enqueueStep();
        ck(cudaStreamEndCapture(stream_, &g), "cudaStreamEndCapture");
        ck(cudaGraphInstantiate(&graph_, g, 0), "cudaGraphInstantiate");
        cudaGraphDestroy(g);
    }

    void upload() {
        const Dims& D = P.dims;
        const std::size_t N = static_cast<std::size_t>(D.cells());
        // fields
        for (int c = 0; c < 6; ++c)
            if (P.comp[c].present) fields_.f[c] = mem_.alloc<T>(N);
        for (int c = 0; c < 3; ++c)
            if (P.comp[c].present && P.comp[c].hasD) fields_.f[6 + c] = mem_.alloc<T>(N);
        // poles: per object start / count
        std::vector<int> pStart, pCount;
        std::vector<T> al, xi, ga;
        for (std::size_t o = 0; o < P.alpha.size(); ++o) {
            pStart.push_back(static_cast<int>(al.size()));
            pCount.push_back(static_cast<int>(P.alpha[o].size()));
            for (std::size_t q = 0; q < P.alpha[o].size(); ++q) {
                al.push_back(static_cast<T>(P.alpha[o][q]));
                xi.push_back(static_cast<T>(P.xi[o][q]));
                ga.push_back(static_cast<T>(P.gamma[o][q]));
            }
        }
        if (al.empty()) {
            al.push_back(0);
            xi.push_back(0);
            ga.push_back(0);
        }
        const int* dStart = mem_.upload(pStart);
        const int* dCount = mem_.upload(pCount);
        const T* dAl = mem_.upload(al);
        const T* dXi = mem_.upload(xi);
        const T* dGa = mem_.upload(ga);
        double bytes = 0;
        for (int half = 0; half < 2; ++half) {
            dev::Pass<T>& pass = half ? ePass_ : hPass_;
            pass.lx = D.lx;
            pass.ly = D.ly;
            pass.lz = D.lz;
            pass.poleStart = dStart;
            pass.poleCount = dCount;
            pass.alpha = dAl;
            pass.xi = dXi;
            pass.gamma = dGa;
            for (int ci = 0; ci < 3; ++ci) {
                const int c = (half ? 0 : 3) + ci;
                const CompPlan& cp = P.comp[c];
                dev::Comp<T>& dc = pass.c[ci];
                std::memset(&dc, 0, sizeof(dc));
                if (!cp.present) continue;
                dc.present = 1;
                dc.U = fields_.f[c];
                dc.D = (c < 3) ? fields_.f[6 + c] : nullptr;
                dc.code = mem_.upload(cp.code);
                std::vector<dev::Class<T>> cls(cp.classes.size());
                for (std::size_t q = 0; q < cp.classes.size(); ++q) {
                    const ClassInfo& k = cp.classes[q];
                    dev::Class<T>& o = cls[q];
                    std::memset(&o, 0, sizeof(o));
                    o.cint[0] = static_cast<T>(k.cint[0]);
                    o.cint[1] = static_cast<T>(k.cint[1]);
                    o.epsInv = static_cast<T>(1.0 / k.eps);
                    o.negEpsInv = static_cast<T>(-1.0 / k.eps);
                    o.obj = k.obj;
                    o.toD = k.toD;
                    o.lor = k.lor;
                    for (int t = 0; t < 2; ++t) {
                        o.nplain[t] = k.nplain[t];
                        o.kflag[t] = k.kflag[t];
                        o.npsi[t] = k.npsi[t];
                        o.psiUpd[t] = k.psiUpd[t];
                    }
                    if (k.ordip) throw UnsupportedError("oriented-dipole cells are not supported by the device engine");
                    if (k.lor && !cp.hasD) throw InputError("dispersive cell without a D field");
                }
                dc.cls = mem_.upload(cls);
                dc.nPoles = cp.nPoles;
                if (cp.nPoles > dev::kMaxPoles) throw UnsupportedError("more than 8 Lorentz poles on one component");
                for (int q = 0; q < cp.nPoles; ++q) {
                    dc.P[q] = mem_.alloc<T>(N);
                    dc.Pprev[q] = mem_.alloc<T>(N);
                }
                for (int t = 0; t < 2; ++t) {
                    const TermPlan& tp = cp.term[t];
                    dc.tpresent[t] = tp.present ? 1 : 0;
                    if (!tp.present) continue;
                    dc.axis[t] = tp.axis;
                    dc.off[t] = tp.off;
                    dc.G[t] = fields_.f[tp.field];
                    dc.db[t] = static_cast<T>(tp.db);
                    dc.dbpsi[t] = static_cast<T>(tp.dbpsi);
                    std::vector<T> kp(tp.kprof.begin(), tp.kprof.end()), b(tp.b.begin(), tp.b.end()), cpsi(tp.cpsi.begin(), tp.cpsi.end());
                    dc.kprof[t] = mem_.upload(kp);
                    dc.b[t] = mem_.upload(b);
                    dc.cpsi[t] = mem_.upload(cpsi);
                    dc.hasPsi[t] = tp.hasPsi ? 1 : 0;
                    if (tp.hasPsi) dc.psi[t] = mem_.alloc<T>(N);
                }
                bytes += 3.0 * sizeof(T) + 1.0;  // field read + write, neighbour read, code
            }
        }
        (void)bytes;
        bytesPerCell_ = algorithmicBytesPerCell();
        // sources
        {
            std::vector<int> comp, srcId;
            std::vector<long long> cell;
            std::vector<double> val;
            for (std::size_t s = 0; s < P.sources.size(); ++s) {
                const SourcePlan& sp = P.sources[s];
                for (long long c : sp.cells) {
                    comp.push_back(sp.comp);
                    cell.push_back(c);
                    srcId.push_back(static_cast<int>(s));
                }
                val.insert(val.end(), sp.value.begin(), sp.value.end());
            }
            src_.n = static_cast<int>(cell.size());
            src_.comp = mem_.upload(comp);
            src_.cell = mem_.upload(cell);
            src_.src = mem_.upload(srcId);
            src_.value = mem_.upload(val);
            src_.nSteps = P.nSteps;
        }
        // detector records
        {
            std::vector<int> det, comp, ti, nev;
            std::vector<long long> cell, outIdx, nvals;
            recBase_.clear();
            recTotal_ = 0;
            for (std::size_t k = 0; k < P.detectors.size(); ++k) {
                const DetectorPlan& dp = P.detectors[k];
                long long nv = detector_event_values(dp);
                int ne = detector_events(dp, P.nSteps);
                recBase_.push_back(static_cast<long long>(recTotal_));
                recTotal_ += static_cast<std::size_t>(nv) * ne;
                ti.push_back(dp.timeInt);
                nev.push_back(ne);
                nvals.push_back(nv);
                long long o = 0;
                for (auto& f : dp.fields) {
                    if (!fields_.f[f.comp]) throw InputError("detector field is not allocated");
                    for (long long c : f.cells) {
                        det.push_back(static_cast<int>(k));
                        comp.push_back(f.comp);
                        cell.push_back(c);
                        outIdx.push_back(o++);
                    }
                }
            }
            recT_.n = static_cast<int>(cell.size());
            recT_.det = mem_.upload(det);
            recT_.comp = mem_.upload(comp);
            recT_.cell = mem_.upload(cell);
            recT_.outIndex = mem_.upload(outIdx);
            recT_.timeInt = mem_.upload(ti);
            recT_.nvals = mem_.upload(nvals);
            recT_.recBase = mem_.upload(recBase_);
            recT_.nEvents = mem_.upload(nev);
            dRec_ = mem_.alloc<double>(recTotal_);
            recT_.rec = dRec_;
        }
        // DFT flux accumulators and phasor tables
        for (auto& fp : P.fluxes) {
            dev::DftTable d{};
            std::vector<int> comp;
            std::vector<long long> cell;
            for (auto& st : fp.stores)
                for (long long c : st.cells) {
                    comp.push_back(st.comp);
                    cell.push_back(c);
                }
            const int nf = static_cast<int>(fp.spec.freqList.size());
            std::vector<double> ph(static_cast<std::size_t>(P.nSteps + 1) * nf * 2);
            for (int s = 0; s <= P.nSteps; ++s)
                for (int f = 0; f < nf; ++f) {
                    std::complex<double> e = std::exp(std::complex<double>(0.0, -1.0 * P.tcur[s] * fp.spec.freqList[f]));
                    ph[(static_cast<std::size_t>(s) * nf + f) * 2 + 0] = e.real();
                    ph[(static_cast<std::size_t>(s) * nf + f) * 2 + 1] = e.imag();
                }
            d.npts = static_cast<long long>(cell.size());
            d.nfreq = nf;
            d.timeInt = fp.spec.timeInt;
            d.comp = mem_.upload(comp);
            d.cell = mem_.upload(cell);
            d.phasor = mem_.upload(ph);
            d.re = mem_.alloc<double>(cell.size() * nf);
            d.im = mem_.alloc<double>(cell.size() * nf);
            dft_.push_back(d);
        }
        dStep_ = mem_.alloc<int>(1);
        kernelsPerStep_ = 3 + (src_.n ? 1 : 0) + (recT_.n ? 1 : 0) + static_cast<int>(dft_.size());
        // t = 0 samples (parallelFDTDField.cpp:831-837)
        dev::launch_record<T>(recT_, fields_, dStep_, stream_);
        for (auto& d : dft_) dev::launch_dft<T>(d, fields_, dStep_, stream_);
        ck(cudaStreamSynchronize(stream_), "initial samples");
    }

    // Algorithmic HBM bytes per physical cell per step: each field array read
    // and written once, one class byte per component, CPML psi and dispersive
    // D/P arrays weighted by the fraction of cells that use them.
    double algorithmicBytesPerCell() const {
        const Dims& D = P.dims;
        double phys = static_cast<double>(D.nx) * D.ny * D.nz;
        double total = 0;
        for (int c = 0; c < 6; ++c) {
            const CompPlan& cp = P.comp[c];
            if (!cp.present) continue;
            total += phys * (2.0 * sizeof(T) + 1.0);
            long long psiCells[2] = {0, 0}, dCells = 0;
            std::vector<long long> classCount(cp.classes.size(), 0);
            for (uint8_t k : cp.code) classCount[k]++;
            for (std::size_t q = 0; q < cp.classes.size(); ++q) {
                const ClassInfo& k = cp.classes[q];
                for (int t = 0; t < 2; ++t)
                    if (k.psiUpd[t]) psiCells[t] += classCount[q];
                if (k.lor) dCells += classCount[q] * (2 + 4 * static_cast<long long>(P.alpha[k.obj].size()));
                else if (k.toD) dCells += classCount[q] * 2;
            }
            total += (psiCells[0] + psiCells[1]) * 2.0 * sizeof(T);
            total += dCells * static_cast<double>(sizeof(T));
        }
        return total / phys;
    }
};

struct Handle {
    std::unique_ptr<SimBase> sim;
    std::string err;
    double h2d = 0, d2h = 0;
};

chiml_status status_of(const std::exception& e) {
    if (dynamic_cast<const UnsupportedError*>(&e)) return CHIML_E_UNSUPPORTED;
    if (dynamic_cast<const InputError*>(&e)) return CHIML_E_INPUT;
    if (auto* c = dynamic_cast<const CudaError*>(&e))
        return c->code == cudaErrorMemoryAllocation ? CHIML_E_OOM : CHIML_E_CUDA;
    if (dynamic_cast<const std::bad_alloc*>(&e)) return CHIML_E_OOM;
    if (dynamic_cast<const std::logic_error*>(&e)) return CHIML_E_STATE;
    return CHIML_E_INPUT;
}

}  // namespace

struct chiml_sim {
    Handle h;
};

extern "C" {

chiml_status chiml_create(const char* json_path, const chiml_options* opt, chiml_sim** out) {
    if (!out) return CHIML_E_INPUT;
    *out = nullptr;
    chiml_options o{};
    o.precision = CHIML_PREC_FP64;
    o.device = 0;
    o.steps_per_graph = 0;
    o.out_dir = nullptr;
    if (opt) o = *opt;
    try {
        if (!json_path) throw InputError("no input file");
        Inputs in = read_inputs_file(json_path);
        Plan P = build_plan(in);
        std::unique_ptr<chiml_sim> s(new chiml_sim());
        if (o.precision == CHIML_PREC_FP64) s->h.sim.reset(new Sim<double>(std::move(P), o));
        else if (o.precision == CHIML_PREC_SPLIT) s->h.sim.reset(new Sim<float>(std::move(P), o));
        else throw InputError("unknown precision mode");
        *out = s.release();
        return CHIML_OK;
    } catch (const std::exception& e) {
        g_createError = e.what();
        return status_of(e);
    }
}

chiml_status chiml_step(chiml_sim* sim, int64_t nsteps) {
    if (!sim) return CHIML_E_STATE;
    try {
        sim->h.sim->step(nsteps);
        return CHIML_OK;
    } catch (const std::exception& e) {
        sim->h.err = e.what();
        return status_of(e);
    }
}

chiml_status chiml_sync(chiml_sim* sim) {
    if (!sim) return CHIML_E_STATE;
    cudaError_t e = cudaStreamSynchronize(sim->h.sim->stream());
    if (e != cudaSuccess) {
        sim->h.err = cudaGetErrorString(e);
        return CHIML_E_CUDA;
    }
    return CHIML_OK;
}

chiml_status chiml_finalize(chiml_sim* sim) {
    if (!sim) return CHIML_E_STATE;
    try {
        sim->h.sim->finalize();
        return CHIML_OK;
    } catch (const std::exception& e) {
        sim->h.err = e.what();
        return status_of(e);
    }
}

void chiml_destroy(chiml_sim* sim) { delete sim; }

const char* chiml_last_error(const chiml_sim* sim) {
    if (!sim) return g_createError.c_str();
    return sim->h.err.c_str();
}

chiml_status chiml_query(const chiml_sim* sim, chiml_stats* out) {
    if (!sim || !out) return CHIML_E_STATE;
    sim->h.sim->fillStats(out);
    return CHIML_OK;
}

chiml_status chiml_get_field(chiml_sim* sim, int comp, double* out) {
    if (!sim || !out) return CHIML_E_STATE;
    try {
        sim->h.sim->getField(comp, out);
        return CHIML_OK;
    } catch (const std::exception& e) {
        sim->h.err = e.what();
        return status_of(e);
    }
}

void* chiml_stream(chiml_sim* sim) { return sim ? static_cast<void*>(sim->h.sim->stream()) : nullptr; }

}  // extern "C"
