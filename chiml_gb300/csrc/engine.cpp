// The C ABI (include/chiml_gpu.h): builds the plan on the host, uploads it,
// drives the kernels per step (optionally as CUDA graphs of several steps),
// and writes the outputs at finalize.
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <exception>
#include <functional>
#include <future>
#include <map>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <parallel/algorithm>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "../../include/chiml_gpu.h"
#include "host/outputs.hpp"
#include "host/plan.hpp"
#include "kernels/box_noalloc.hpp"
#include "kernels/emitter_device.hpp"
#include "kernels/fdtd_device.hpp"
#include "kernels/flux_device.hpp"
#include "kernels/tfsf_device.hpp"

using namespace chiml;

namespace {

thread_local std::string g_createError;

struct DeviceStateError : public std::runtime_error {
    explicit DeviceStateError(const std::string& w) : std::runtime_error(w) {}
};

// A detector or DFT point read a NaN or Inf (the run has diverged).
struct NumericError : public std::runtime_error {
    explicit NumericError(const std::string& w) : std::runtime_error(w) {}
};

// A grid barrier of the persistent form gave up waiting.
struct TimeoutError : public std::runtime_error {
    explicit TimeoutError(const std::string& w) : std::runtime_error(w) {}
};

struct CudaError : public std::runtime_error {
    cudaError_t code;
    CudaError(cudaError_t c, const std::string& w) : std::runtime_error(w), code(c) {}
};

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(e, std::string(what) + ": " + cudaGetErrorString(e));
}

// Device allocations of a handle, freed together. The upload tasks of chiml_create run
// on several host threads at once, so the bookkeeping is guarded.
struct DevMem {
    std::vector<void*> ptrs;
    double bytes = 0;
    double allocSeconds = 0, copySeconds = 0;  // wall time in cudaMalloc + cudaMemset, and in copies
    double h2d = 0;
    std::mutex mu;
    template <typename T>
    T* alloc(std::size_t n, bool zero = true) {
        if (n == 0) return nullptr;
        const auto t0 = std::chrono::steady_clock::now();
        void* p = nullptr;
        ck(cudaMalloc(&p, n * sizeof(T)), "cudaMalloc");
        {
            std::lock_guard<std::mutex> g(mu);
            ptrs.push_back(p);
            bytes += static_cast<double>(n * sizeof(T));
        }
        if (zero) ck(cudaMemset(p, 0, n * sizeof(T)), "cudaMemset");
        addTime(allocSeconds, t0);
        return static_cast<T*>(p);
    }
    template <typename T>
    T* upload(const std::vector<T>& v) {
        if (v.empty()) return nullptr;
        T* p = alloc<T>(v.size(), false);
        const auto t0 = std::chrono::steady_clock::now();
        ck(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        addTime(copySeconds, t0);
        addCopied(static_cast<double>(v.size() * sizeof(T)));
        return p;
    }
    void addCopied(double b) {
        std::lock_guard<std::mutex> g(mu);
        h2d += b;
    }
    void addTime(double& acc, std::chrono::steady_clock::time_point t0) {
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::lock_guard<std::mutex> g(mu);
        acc += dt;
    }
    ~DevMem() {
        for (void* p : ptrs) cudaFree(p);
    }
};

// Runs the tasks on host threads of their own (each bound to the handle's device) and
// waits for all; the first failure in task order is rethrown.
void runConcurrently(int device, const std::vector<std::function<void()>>& tasks) {
    std::vector<std::exception_ptr> err(tasks.size());
    std::vector<std::thread> th;
    for (std::size_t k = 0; k < tasks.size(); ++k)
        th.emplace_back([&, k] {
            try {
                ck(cudaSetDevice(device), "cudaSetDevice");
                tasks[k]();
            } catch (...) {
                err[k] = std::current_exception();
            }
        });
    for (auto& t : th) t.join();
    for (auto& e : err)
        if (e) std::rethrow_exception(e);
}

struct SimBase {
    virtual ~SimBase() {}
    virtual void step(long long n) = 0;
    virtual void finalize() = 0;
    virtual void getField(int comp, double* out) = 0;
    virtual void fillStats(chiml_stats* s) const = 0;
    virtual cudaStream_t stream() const = 0;
    virtual int profile(int nsteps, double* ms, int maxSlots) = 0;
    virtual void checkDeviceErrors() = 0;
    virtual chiml_status getBoxNoAlloc(int comp, const int box[6], double* out, std::string& why) = 0;
};

template <typename T>
class Sim : public SimBase {
public:
    Sim(Plan&& plan, const chiml_options& opt) : P(std::move(plan)), opt_(opt) {
        PhaseClock clk;
        ck(cudaSetDevice(opt.device), "cudaSetDevice");
        // A blocking stream: ordered after the uploads and memsets that run on
        // the legacy default stream.
        ck(cudaStreamCreate(&stream_), "cudaStreamCreate");
        outDir_ = opt.out_dir ? opt.out_dir : "";
        // the fixed array of chiml_get_box_noalloc is placed on the device now, before
        // this handle's uploads, so that no read-back has to place it later
        ck(dev::box_noalloc_setup(opt.device), "chiml_get_box_noalloc set-up");
        clk.mark("device-setup");
        upload();
        clk.mark("upload");
        setupPersist();
        // the step graph is captured and instantiated here, so that no step call pays for it
        if (!persist_ && opt_.steps_per_graph > 0 && P.nSteps >= opt_.steps_per_graph) buildGraph(opt_.steps_per_graph);
        clk.mark("graph");
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
        if (persist_) {
            stepPersist(n);
            return;
        }
        const int K = opt_.steps_per_graph;
        if (K > 0) {
            if (!graph_ && n >= K) buildGraph(K);
            const long long period = foldPeriod();
            while (n >= K && graph_) {
                if (graphAligned_ && stepsDone_ % period != 0) {
                    // eager steps up to the next start of the fold period
                    while (n > 0 && stepsDone_ % period != 0) {
                        enqueueStep(stepsDone_, false);
                        ++stepsDone_;
                        --n;
                    }
                    continue;
                }
                ck(cudaGraphLaunch(graph_, stream_), "cudaGraphLaunch");
                n -= K;
                stepsDone_ += K;
            }
        }
        for (long long s = 0; s < n; ++s) {
            enqueueStep(stepsDone_, false);
            ++stepsDone_;
        }
        ck(cudaGetLastError(), "kernel launch");
    }

    // Raises when a kernel recorded a bounds error (it skipped the cell instead of faulting).
    void checkDeviceErrors() override {
        ck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        unsigned int e = 0;
        ck(cudaMemcpy(&e, dErr_, sizeof(e), cudaMemcpyDeviceToHost), "D2H error word");
        if (e & dev::kErrTimeout) throw TimeoutError("a grid barrier of the persistent step gave up waiting");
        if (e & ~dev::kErrNumeric) throw DeviceStateError("device bounds check failed (code " + std::to_string(e) + ")");
        if (e) throw NumericError("a detector or flux point sampled a NaN or Inf field value");
    }

    void finalize() override {
        PhaseClock clk;
        checkDeviceErrors();
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
        // fold every group's pending samples into the accumulators
        for (std::size_t q = 0; q < dft_.size(); ++q) {
            const dev::DftTable<T>& d = dft_[q];
            dev::launch_dft_flush<T>(d, stepsDone_ / d.timeInt + 1, stream_);
        }
        ck(cudaStreamSynchronize(stream_), "DFT flush");
        clk.mark("fin-records");
        for (std::size_t q = 0; q < P.fluxes.size(); ++q) {
            const int nt = stepsDone_ / P.fluxes[q].spec.timeInt + 1;
            R.fluxRe.emplace_back();
            R.fluxIm.emplace_back();
            if (P.fluxes[q].spec.save || P.fluxes[q].spec.load) {
                // saving or loading the face grids: combine and integrate on the host from
                // the accumulators (write_fluxes), which the grids are made from
                R.fluxFaces.emplace_back();
                downloadDft(q, P.fluxes[q].spec.freqList.size(), R.fluxRe.back(), R.fluxIm.back());
            } else {
                R.fluxFaces.push_back(fluxFacesOnDevice(q, nt));
            }
            R.fluxSamples.push_back(nt);
        }
        clk.mark("fin-flux");
        for (std::size_t k = 0; k < P.freqDetectors.size(); ++k) {
            std::vector<double> re, im;
            downloadDft(P.fluxes.size() + k, P.freqDetectors[k].spec.freqList.size(), re, im);
            R.freqRe.push_back(std::move(re));
            R.freqIm.push_back(std::move(im));
            R.freqSamples.push_back(stepsDone_ / P.freqDetectors[k].timeInt + 1);
        }
        for (std::size_t q = 0; q < emit_.size(); ++q) {
            const dev::EmitterDev& e = emit_[q];
            const EmitterPlan& ep = P.emitters[q];
            std::array<std::vector<double>, 3> tp;
            if (e.totP) {
                std::vector<double> all(3 * static_cast<std::size_t>(std::max(P.nSteps, 1)));
                ck(cudaMemcpy(all.data(), e.totP, all.size() * sizeof(double), cudaMemcpyDeviceToHost), "D2H emitter P");
                d2h_ += static_cast<double>(all.size() * sizeof(double));
                for (int c = 0; c < 3; ++c)
                    if (ep.comp[c])
                        tp[c].assign(all.begin() + static_cast<long long>(c) * P.nSteps,
                                     all.begin() + static_cast<long long>(c) * P.nSteps + stepsDone_);
            }
            R.emitterP.push_back(tp);
            std::vector<std::vector<cplx>> pops(ep.dtcLevs.size());
            if (e.nDtc > 0) {
                std::vector<double2> all(static_cast<std::size_t>(e.nDtc) * e.nEvents);
                ck(cudaMemcpy(all.data(), e.pop, all.size() * sizeof(double2), cudaMemcpyDeviceToHost), "D2H populations");
                d2h_ += static_cast<double>(all.size() * sizeof(double2));
                const int nev = stepsDone_ > 0 ? (stepsDone_ - 1) / ep.dtcTimeInt + 1 : 0;
                for (int d = 0; d < e.nDtc; ++d)
                    for (int v = 0; v < nev; ++v) {
                        const double2 x = all[static_cast<std::size_t>(d) * e.nEvents + v];
                        pops[d].emplace_back(x.x, x.y);
                    }
            }
            R.emitterPop.push_back(pops);
        }
        if (!tfsf_.empty()) {
            // incident values of the last surface (each surface overwrites them, parallelFDTDField.hpp:1238-1255)
            const std::size_t n = 2 * (static_cast<std::size_t>(P.nSteps) + 1);
            std::vector<double2> all(6 * n);
            ck(cudaMemcpy(all.data(), tfsf_.back().rec, all.size() * sizeof(double2), cudaMemcpyDeviceToHost), "D2H incident");
            d2h_ += static_cast<double>(all.size() * sizeof(double2));
            for (int c = 0; c < 6; ++c) {
                std::vector<cplx>& dst = c < 3 ? R.incE[c] : R.incH[c - 3];
                dst.resize(n);
                for (std::size_t k = 0; k < n; ++k) dst[k] = cplx(all[c * n + k].x, all[c * n + k].y);
            }
        }
        clk.mark("fin-downloads");
        write_detectors(P, R, outDir_, stepsDone_);
        write_fluxes(P, R, outDir_);
        write_freq_detectors(P, R, outDir_);
        write_emitters(P, R, outDir_);
        clk.mark("fin-writes");
        finalized_ = true;
    }

    // The accumulators of DFT table q (nf frequencies) in the plan's point order, [point][freq].
    void downloadDft(std::size_t q, std::size_t nf, std::vector<double>& re, std::vector<double>& im) {
        const dev::DftTable<T>& d = dft_[q];
        const std::size_t n = static_cast<std::size_t>(d.npts) * nf;
        std::vector<double> dre(n), dim(n);
        re.assign(n, 0.0);
        im.assign(n, 0.0);
        if (n) {
            ck(cudaMemcpy(dre.data(), d.re, n * sizeof(double), cudaMemcpyDeviceToHost), "D2H DFT accumulators");
            ck(cudaMemcpy(dim.data(), d.im, n * sizeof(double), cudaMemcpyDeviceToHost), "D2H DFT accumulators");
        }
        // the split form's float-float pairs become doubles (hi + lo is exact in FP64)
        auto value = [](const std::vector<double>& a, std::size_t i) {
            if (!dev::kFloatFloatAcc<T>) return a[i];
            float pr[2];
            std::memcpy(pr, &a[i], sizeof pr);
            return static_cast<double>(pr[0]) + static_cast<double>(pr[1]);
        };
        const std::vector<int>& pos = dftPos_[q];
        for (std::size_t p = 0; p < pos.size(); ++p)
            for (std::size_t f = 0; f < nf; ++f) {
                re[p * nf + f] = value(dre, static_cast<std::size_t>(pos[p]) * nf + f);
                im[p * nf + f] = value(dim, static_cast<std::size_t>(pos[p]) * nf + f);
            }
        d2h_ += 2.0 * n * sizeof(double);
    }

    // The integrated flux of every face of flux q, [freq * nFaces + face], evaluated from the
    // accumulators on the device; only these values are copied back.
    // The face maps of flux region q on the device, built at create (the integration
    // at finalize then only launches and reads back nfreq values per face).
    struct FluxFacesDev {
        bool ready = false;
        int nFaces = 0, nTiles = 0, nfreq = 0;
        const dev::FluxFaceDev* faces = nullptr;
        const int4* tiles = nullptr;
        double2* partial = nullptr;
        double2* out = nullptr;
    };
    std::vector<FluxFacesDev> fluxDev_;

    void prepareFluxFaces(std::size_t q, const std::vector<FluxFaceMap>& maps) {
        const FluxPlan& fp = P.fluxes[q];
        FluxFacesDev& fd = fluxDev_[q];
        fd.nfreq = static_cast<int>(fp.spec.freqList.size());
        fd.nFaces = static_cast<int>(maps.size());
        fd.ready = true;
        if (fd.nFaces == 0 || fd.nfreq == 0) return;
        std::vector<dev::FluxFaceDev> faces(static_cast<std::size_t>(fd.nFaces));
        std::vector<int4> tiles;
        for (int v = 0; v < fd.nFaces; ++v) {
            const FluxFaceMap& m = maps[v];
            dev::FluxFaceDev& F = faces[v];
            F.nx = m.nx;
            F.sz = m.sz;
            for (int w = 0; w < 4; ++w) {
                F.has[w] = m.has[w] ? 1 : 0;
                F.start[w] = m.has[w] ? mem_.upload(m.start[w]) : nullptr;
                std::vector<long long> devPt(m.pt[w].size());
                for (std::size_t k = 0; k < devPt.size(); ++k) {
                    const long long p = m.pt[w][k];
                    if (p < 0 || p >= fp.npts) throw std::logic_error("flux map point outside the accumulators");
                    devPt[k] = dftPos_[q][static_cast<std::size_t>(p)];
                }
                F.pt[w] = m.has[w] ? mem_.upload(devPt) : nullptr;
                F.scale[w] = m.has[w] ? mem_.upload(m.scale[w]) : nullptr;
            }
            F.wx = mem_.upload(m.wx);
            F.wy = mem_.upload(m.wy);
            F.pref = m.pref;
            F.firstTile = static_cast<int>(tiles.size());
            for (int s0 = 0; s0 < m.sz; s0 += dev::kFluxTile) tiles.push_back(make_int4(v, s0, std::min(m.sz, s0 + dev::kFluxTile), 0));
            F.nTiles = static_cast<int>(tiles.size()) - F.firstTile;
        }
        fd.faces = mem_.upload(faces);
        fd.tiles = mem_.upload(tiles);
        fd.nTiles = static_cast<int>(tiles.size());
        fd.partial = mem_.alloc<double2>(tiles.size() * static_cast<std::size_t>(fd.nfreq), false);
        fd.out = mem_.alloc<double2>(static_cast<std::size_t>(fd.nfreq) * fd.nFaces, false);
    }

    std::vector<cplx> fluxFacesOnDevice(std::size_t q, int nt) {
        const FluxFacesDev& fd = fluxDev_[q];
        if (!fd.ready) throw std::logic_error("flux face maps not prepared");
        std::vector<cplx> res(static_cast<std::size_t>(fd.nfreq) * fd.nFaces, cplx(0.0, 0.0));
        if (fd.nFaces == 0 || fd.nfreq == 0) return res;
        const double nt2 = std::pow(static_cast<double>(nt), 2.0);
        dev::launch_flux_faces(fd.faces, fd.nFaces, fd.tiles, fd.nTiles, fd.nfreq, dft_[q].re, dft_[q].im, dev::kFloatFloatAcc<T>, nt2,
                               fd.partial, fd.out, stream_);
        ck(cudaGetLastError(), "flux integration launch");
        std::vector<double2> h(res.size());
        ck(cudaMemcpyAsync(h.data(), fd.out, h.size() * sizeof(double2), cudaMemcpyDeviceToHost, stream_), "D2H flux faces");
        ck(cudaStreamSynchronize(stream_), "flux integration");
        d2h_ += static_cast<double>(h.size() * sizeof(double2));
        for (std::size_t i = 0; i < h.size(); ++i) res[i] = cplx(h[i].x, h[i].y);
        return res;
    }

    void getField(int comp, double* out) override {
        if (comp < 0 || comp > 8 || !fields_.f[comp]) throw std::invalid_argument("field not present");
        ck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        // the device rows are padded to pitch_ values: copy them out and drop the padding
        const Dims& D = P.dims;
        std::vector<T> tmp(static_cast<std::size_t>(cellsPad_));
        ck(cudaMemcpy(tmp.data(), fields_.f[comp], tmp.size() * sizeof(T), cudaMemcpyDeviceToHost), "D2H field");
        const long long rows = static_cast<long long>(D.ly) * D.lz;
        for (long long r = 0; r < rows; ++r)
            for (int x = 0; x < D.lx; ++x) out[r * D.lx + x] = static_cast<double>(tmp[static_cast<std::size_t>(r * pitch_ + x)]);
    }

    // Validates the box and reads it through the fixed device array; no allocation.
    chiml_status getBoxNoAlloc(int comp, const int box[6], double* out, std::string& why) override {
        const Dims& D = P.dims;
        if (comp < 0 || comp > 8 || !fields_.f[comp]) {
            why = "field not present";
            return CHIML_E_INPUT;
        }
        const int ext[3] = {D.lx, D.ly, D.lz};
        for (int a = 0; a < 3; ++a) {
            if (box[3 + a] < 1 || box[a] < 0 || box[a] > ext[a] - box[3 + a]) {
                why = "box outside the local grid (x0, y0, z0, nx, ny, nz against lx, ly, lz)";
                return CHIML_E_INPUT;
            }
        }
        const long long n = static_cast<long long>(box[3]) * box[4] * box[5];
        if (n > dev::kBoxScratchCells) {
            why = "box of " + std::to_string(n) + " cells exceeds the limit of " +
                  std::to_string(dev::kBoxScratchCells) + " cells of chiml_get_box_noalloc";
            return CHIML_E_INPUT;
        }
        cudaError_t e = dev::gather_box_noalloc<T>(opt_.device, fields_.f[comp], static_cast<int>(pitch_), D.lz, box, out, stream_);
        if (e == cudaSuccess) return CHIML_OK;
        why = std::string("chiml_get_box_noalloc: ") + cudaGetErrorString(e);
        return CHIML_E_CUDA;
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
        s->persistent = persist_ ? 1 : 0;
        s->bytes_h_pass = passBytes_[0];
        s->bytes_e_pass = passBytes_[1];
        s->bytes_dft = dftBytes_;
        s->h2d_bytes = mem_.h2d;
        s->d2h_bytes = d2h_;
        s->n_flux_regions = static_cast<int32_t>(dft_.size());
        s->n_emitters = static_cast<int32_t>(emit_.size());
        s->n_tfsf = static_cast<int32_t>(tfsf_.size());
    }

    int profile(int nsteps, double* ms, int maxSlots) override {
        if (finalized_) throw std::logic_error("step after finalize");
        const int nDft = static_cast<int>(dft_.size());
        const int nslots = 5 + 2 * nDft + static_cast<int>(emit_.size()) + static_cast<int>(tfsf_.size());
        // a start and an end event per slot, recorded around that slot's launches
        std::vector<cudaEvent_t> e0(static_cast<std::size_t>(nslots)), e1(static_cast<std::size_t>(nslots));
        for (auto& e : e0) ck(cudaEventCreate(&e), "cudaEventCreate");
        for (auto& e : e1) ck(cudaEventCreate(&e), "cudaEventCreate");
        std::vector<double> acc(static_cast<std::size_t>(nslots), 0.0);
        long long left = P.nSteps - stepsDone_;
        if (nsteps > left) nsteps = static_cast<int>(left);
        auto mark = [&](std::vector<cudaEvent_t>& v, int k) { ck(cudaEventRecord(v[k], stream_), "cudaEventRecord"); };
        for (int st = 0; st < nsteps; ++st) {
            void* s = stream_;
            mark(e0, 0);
            dev::launch_pass<T>(hPass_, false, s);
            mark(e1, 0);
            for (std::size_t q = 0; q < tfsf_.size(); ++q) {
                const int k = 5 + 2 * nDft + static_cast<int>(emit_.size() + q);
                mark(e0, k);
                launchTfsf(tfsf_[q], s);
                mark(e1, k);
            }
            mark(e0, 1);
            if (!srcInE_) dev::launch_sources<T>(src_, fields_, dStep_, s);  // else in the E pass
            mark(e1, 1);
            mark(e0, 2);
            dev::launch_pass<T>(ePass_, true, s);
            mark(e1, 2);
            T* const ef[3] = {fields_.f[0], fields_.f[1], fields_.f[2]};
            for (std::size_t q = 0; q < emit_.size(); ++q) {
                const int k = 5 + 2 * nDft + static_cast<int>(q);
                mark(e0, k);
                dev::launch_emitter_step<T>(emit_[q], ef, dStep_, s);
                mark(e1, k);
            }
            mark(e0, 3);
            dev::launch_increment(dStep_, s);
            mark(e1, 3);
            mark(e0, 4);
            dev::launch_record<T>(recT_, fields_, dStep_, s);
            mark(e1, 4);
            for (int q = 0; q < nDft; ++q) {
                mark(e0, 5 + 2 * q);
                dev::launch_dft_sample<T>(dft_[q], fields_, dStep_, s);
                mark(e1, 5 + 2 * q);
                mark(e0, 6 + 2 * q);
                dev::launch_dft_fold<T>(dft_[q], dStep_, s);
                mark(e1, 6 + 2 * q);
            }
            ck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
            for (int k = 0; k < nslots; ++k) {
                float m = 0.f;
                ck(cudaEventElapsedTime(&m, e0[k], e1[k]), "cudaEventElapsedTime");
                acc[k] += m;
            }
            ++stepsDone_;
        }
        for (auto& e : e0) cudaEventDestroy(e);
        for (auto& e : e1) cudaEventDestroy(e);
        int n = std::min(nslots, maxSlots);
        for (int k = 0; k < n; ++k) ms[k] = acc[k];
        return n;
    }

    double h2dBytes() const { return mem_.h2d; }
    double d2hBytes() const { return d2h_; }

    // ---- batched sweep: the device descriptors of this member, for packed launches ----
    const dev::Pass<T>& hPass() const { return hPass_; }
    const dev::Pass<T>& ePass() const { return ePass_; }
    const dev::Fields<T>& fields() const { return fields_; }
    const dev::SourceTable& sources() const { return src_; }
    const dev::RecordTable& records() const { return recT_; }
    const std::vector<dev::DftTable<T>>& dftTables() const { return dft_; }
    const std::vector<dev::EmitterDev>& emitters() const { return emit_; }
    int* stepCounter() const { return dStep_; }
    bool hasTfsf() const { return !tfsf_.empty(); }
    // The member's TFSF kernels on the given stream (packed steps launch them per member).
    void launchTfsfOn(void* s) {
        for (auto& t : tfsf_) launchTfsf(t, s);
    }
    long long stepsLeft() const { return finalized_ ? 0 : static_cast<long long>(P.nSteps) - stepsDone_; }
    bool fresh() const { return stepsDone_ == 0 && !finalized_; }  // no step has run: every field is still zero
    // Counts n steps that a packed launch sequence queued for this member.
    void stepsRunElsewhere(long long n) {
        if (finalized_) throw std::logic_error("step after finalize");
        if (n > stepsLeft()) throw std::logic_error("more steps than the member has left");
        stepsDone_ += static_cast<int>(n);
    }

private:
    // ---- persistent form of small 2-D grids (k_persist2d) ----
    bool persist_ = false;
    int persistBlocks_ = 0;
    dev::Persist2d<T> persistArgs_{};
    std::vector<uint32_t> classFlags_[6];  // FastClass flags of each component's classes

    // Whether this simulation runs in the persistent form (see dev::Persist2d for the
    // conditions). Opt-in, with CHIML_PERSIST2D=1 in the environment: on the 400^2 TMz
    // workload it measured 17.4 us per step against 13.8 us for the graph of per-kernel
    // launches (two grid barriers per step and a launch per four steps cost more than
    // the launches they replace), so the launch form stays the default.
    void setupPersist() {
        const char* env = std::getenv("CHIML_PERSIST2D");
        if (!env || std::string(env) != "1") return;
        const Dims& D = P.dims;
        if (D.lz != 1 || !hPass_.interior2d || !ePass_.interior2d) return;
        if (static_cast<long long>(D.lx) * D.ly > (1LL << 22)) return;  // larger grids fill the GPU per launch
        if (!tfsf_.empty() || !emit_.empty() || ePass_.od.n > 0) return;
        if (!dev::kInlineDispersive<T> && ePass_.nLor > 0) return;
        for (auto& d : dft_)
            if (d.timeInt != 1) return;
        if (src_.n > 0 && !sourcesInE()) return;
        int coop = 0;
        ck(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, opt_.device), "cudaDeviceGetAttribute");
        if (!coop) return;
        persistBlocks_ = dev::persist2d_blocks<T>(hPass_, ePass_, opt_.device);
        if (persistBlocks_ <= 0) return;
        // CHIML_PERSIST2D_BLOCKS caps the launch (fewer blocks: cheaper barriers, fewer warps)
        if (const char* nb = std::getenv("CHIML_PERSIST2D_BLOCKS")) {
            const int cap = std::atoi(nb);
            if (cap > 0) persistBlocks_ = std::min(persistBlocks_, cap);
        }
        dev::Persist2d<T>& a = persistArgs_;
        a.h = hPass_;
        a.e = ePass_;
        a.src = src_;
        a.rec = recT_;
        a.nDft = static_cast<int>(dft_.size());
        a.dft = mem_.upload(dft_);
        a.dftPoints = 0;
        for (auto& d : dft_) a.dftPoints += d.npts;
        a.f = fields_;
        a.step = dStep_;
        a.bar = mem_.alloc<unsigned int>(1);
        a.limitNs = 1000000000ull;  // one second per barrier
        persist_ = true;
    }

    // Whether the E pass can add the soft sources itself: at most kInlineMaxSrc entries, all
    // on E components, each on a cell whose update is the plain E = E + curl terms (where
    // adding the source to E first, as the source launch does, is the same operation).
    bool sourcesInE() const {
        if (src_.n > dev::kInlineMaxSrc) return false;
        for (const SourcePlan& sp : P.sources) {
            if (sp.comp > EZ) return false;  // H sources: after the H update, not in the E pass
            for (long long c : sp.cells) {
                const uint8_t k = P.comp[sp.comp].code[static_cast<std::size_t>(c)];
                const uint32_t fl = k < classFlags_[sp.comp].size() ? classFlags_[sp.comp][k] : 0u;
                if (k == 0 || !(fl & dev::kFcWrite) || (fl & (dev::kFcToD | dev::kFcLor | dev::kFcOrDip | dev::kFcDtoE)))
                    return false;
            }
        }
        return true;
    }

    // n steps in launches that end where a DFT group folds (every fourth sample) or after
    // kPersistChunk steps; the fold kernels run after a launch that ends at a fold.
    static constexpr long long kPersistChunk = 64;
    void stepPersist(long long n) {
        while (n > 0) {
            long long c = std::min(n, kPersistChunk);
            if (!dft_.empty()) {
                long long toFold = (3 - stepsDone_ % 4 + 4) % 4;  // steps until stepsDone = 3 (mod 4)
                if (toFold == 0) toFold = 4;
                c = std::min(c, toFold);
            }
            const int st = dev::launch_persist2d<T>(persistArgs_, persistBlocks_, stepsDone_, static_cast<int>(c), stream_);
            if (st != 0) ck(static_cast<cudaError_t>(st), "cooperative launch");
            stepsDone_ += static_cast<int>(c);
            n -= c;
            if (!dft_.empty() && stepsDone_ % 4 == 3)
                for (auto& d : dft_) dev::launch_dft_fold<T>(d, dStep_, stream_);
        }
        ck(cudaGetLastError(), "kernel launch");
    }

    Plan P;
    chiml_options opt_;
    std::string outDir_;
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
    bool srcInE_ = false;        // the E pass adds the soft sources (no source launch)
    bool graphAligned_ = false;  // the graph holds only the fold launches of a period-aligned replay
    DevMem mem_;
    dev::Pass<T> hPass_{}, ePass_{};
    dev::Fields<T> fields_{};
    dev::SourceTable src_{};
    dev::RecordTable recT_{};
    std::vector<dev::DftTable<T>> dft_;
    std::vector<dev::EmitterDev> emit_;
    std::vector<dev::TfsfDev> tfsf_;
    long long pitch_ = 0;     // device row length (values): lx rounded up to a multiple of 4
    long long cellsPad_ = 0;  // device grid size: pitch_ * ly * lz
    std::vector<long long> recBase_;
    std::size_t recTotal_ = 0;
    double* dRec_ = nullptr;
    int* dStep_ = nullptr;
    unsigned int* dErr_ = nullptr;
    int stepsDone_ = 0;
    bool finalized_ = false;
    double d2h_ = 0;
    double bytesPerCell_ = 0;
    double passBytes_[2] = {0, 0};
    double dftBytes_ = 0;
    int kernelsPerStep_ = 0;

    // The step with index st (steps done before it). A table's fold kernel runs at the steps
    // where one of its groups folds (foldsAfter); allFolds launches it every step, where
    // the kernel itself finds whether a group folds (a graph whose replays do not all start
    // at the same point of the fold period).
    void enqueueStep(long long st, bool allFolds) {
        void* s = stream_;
        dev::launch_pass<T>(hPass_, false, s);
        // TFSF after the H update, before the sources (parallelFDTDField.hpp:1237-1261)
        for (auto& t : tfsf_) launchTfsf(t, s);
        if (!srcInE_) dev::launch_sources<T>(src_, fields_, dStep_, s);
        dev::launch_pass<T>(ePass_, true, s);
        launchEmitters(s);
        // records, DFT samples and the step counter in one launch, then the folds
        dev::launch_step_tail<T>(tail_, s);
        for (auto& d : dft_)
            if (allFolds || foldsAfter(d, st + 1)) dev::launch_dft_fold<T>(d, dStep_, s);
    }

    // Whether a group of table d folds once the step counter reads `next` (the device's
    // foldGroupNow: a sample at `next` that is the last of a stagger period).
    static bool foldsAfter(const dev::DftTable<T>& d, long long next) {
        return next % d.timeInt == 0 && (next / d.timeInt + 1) % dev::kFoldStagger == 0;
    }

    // Steps after which the fold pattern of every table repeats.
    long long foldPeriod() const {
        long long p = 1;
        for (auto& d : dft_) p = std::lcm(p, static_cast<long long>(d.timeInt) * dev::kFoldStagger);
        return p;
    }

    // ---- the device layout: rows padded from lx to pitch_ values ----
    // Cell index of the device layout for a cell index of the plan (negative: unchanged).
    long long pad(long long i) const {
        if (i < 0) return i;
        const long long lx = P.dims.lx;
        return (i % lx) + pitch_ * (i / lx);
    }
    template <typename I>
    std::vector<I> padCells(const std::vector<I>& v) const {
        std::vector<I> o(v.size());
        for (std::size_t k = 0; k < v.size(); ++k) o[k] = static_cast<I>(pad(static_cast<long long>(v[k])));
        return o;
    }
    // A neighbour offset of the plan (dx + lx (dz + lz dy), |d*| <= 1) in the device layout.
    long long padOffset(long long off) const {
        const long long lx = P.dims.lx, lz = P.dims.lz;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz)
                for (int dx = -1; dx <= 1; ++dx)
                    if (dx + lx * (dz + lz * dy) == off) return dx + pitch_ * (dz + lz * dy);
        throw InputError("neighbour offset of more than one cell");
    }
    // A whole-grid byte array of the plan, copied row by row into the device layout (rows of
    // pitch_ values, the padding zero).
    const uint8_t* uploadPadded(const std::vector<uint8_t>& v) {
        const Dims& D = P.dims;
        if (static_cast<long long>(v.size()) != D.cells()) throw InputError("grid array of the wrong size");
        uint8_t* d = mem_.alloc<uint8_t>(static_cast<std::size_t>(cellsPad_));
        ck(cudaMemcpy2D(d, static_cast<std::size_t>(pitch_), v.data(), static_cast<std::size_t>(D.lx), static_cast<std::size_t>(D.lx),
                        static_cast<std::size_t>(D.ly) * D.lz, cudaMemcpyHostToDevice),
           "cudaMemcpy2D H2D");
        mem_.addCopied(static_cast<double>(v.size()));
        return d;
    }

    void launchTfsf(const dev::TfsfDev& t, void* s) {
        T* const f9[9] = {fields_.f[0], fields_.f[1], fields_.f[2], fields_.f[3], fields_.f[4],
                          fields_.f[5], fields_.f[6], fields_.f[7], fields_.f[8]};
        dev::launch_tfsf_step<T>(t, f9, dStep_, s);
    }

    // TFSF surfaces: the lines' two grids and psi lists (zeroed), the pulse table of
    // every step, the record array and the surface corrections as per-cell term lists.
    void uploadTfsf() {
        for (const TfsfPlan& tp : P.tfsf) {
            dev::TfsfDev t{};
            t.gridLen = tp.gridLen;
            t.pulseLen = tp.pulseLen;
            t.mTot = tp.mTot;
            t.pulAddStart = tp.pulAddStart;
            t.nSteps = P.nSteps;
            for (int c = 0; c < 6; ++c) {
                const TfsfLine& L = tp.line[c];
                dev::TfsfLineDev& d = t.line[c];
                d.present = L.present ? 1 : 0;
                if (!L.present) continue;
                if (L.runs.size() != 1 || L.pulseRuns.size() != 1) throw UnsupportedError("TFSF line with several materials");
                if (L.pml.size() > dev::kTfsfMaxPsi || L.pmlPulse.size() > dev::kTfsfMaxPsi)
                    throw UnsupportedError("TFSF line CPML with more than four psi lists");
                d.useJ = L.useJ ? 1 : 0;
                d.useK = L.useK ? 1 : 0;
                d.nbrJ = L.nbrJ;
                d.nbrK = L.nbrK;
                d.prefact = make_double2(L.prefact.real(), L.prefact.imag());
                d.U = mem_.alloc<double2>(static_cast<std::size_t>(tp.gridLen));
                d.pul = mem_.alloc<double2>(static_cast<std::size_t>(tp.pulseLen));
                const std::size_t len = static_cast<std::size_t>(tp.gridLen);
                if (L.epMu.size() != len || L.obj.size() != len || L.nPole < 0 ||
                    L.pa.size() != static_cast<std::size_t>(L.nPole) * len || L.px.size() != L.pa.size() ||
                    L.pg.size() != L.pa.size() || (L.nPole > 0 && !L.dLine))
                    throw InputError("TFSF line material set-up inconsistent");
                d.eps = mem_.upload(L.epMu);
                d.D = L.dLine ? mem_.alloc<double2>(len) : nullptr;
                if (L.dLine) t.layered = 1;
                d.nPole = L.nPole;
                if (L.nPole > 0) {
                    d.P = mem_.alloc<double2>(static_cast<std::size_t>(L.nPole) * len);
                    d.Pprev = mem_.alloc<double2>(static_cast<std::size_t>(L.nPole) * len);
                    d.pa = mem_.upload(L.pa);
                    d.px = mem_.upload(L.px);
                    d.pg = mem_.upload(L.pg);
                }
                auto run = [](const TfsfRun& r) {
                    return dev::TfsfRunDev{r.indI, r.n, r.posJ, r.negJ, r.posK, r.negK, r.pj, r.pk};
                };
                d.run = run(L.runs[0]);
                d.pulseRun = run(L.pulseRuns[0]);
                // every index a line element reads or writes stays inside its grid
                auto inRange = [](long long lo, long long n, long long len) { return lo >= 0 && n >= 0 && lo + n <= len; };
                const TfsfRun* rr[2] = {&L.runs[0], &L.pulseRuns[0]};
                const long long lens[2] = {tp.gridLen, tp.pulseLen};
                for (int g = 0; g < 2; ++g) {
                    const TfsfRun& r = *rr[g];
                    if (!inRange(r.indI, r.n, lens[g]) || !inRange(r.posJ, r.n, lens[g]) || !inRange(r.negJ, r.n, lens[g]) ||
                        !inRange(r.posK, r.n, lens[g]) || !inRange(r.negK, r.n, lens[g]))
                        throw InputError("TFSF run outside its line");
                    const std::vector<TfsfPsi>& pl = g == 0 ? L.pml : L.pmlPulse;
                    for (const TfsfPsi& q : pl)
                        if (!inRange(q.loc, q.n, lens[g]) || !inRange(q.locOff, q.n, lens[g]) || !inRange(q.gridLoc, q.n, lens[g]) ||
                            q.nbr < 0 || q.nbr > 5 || !tp.line[q.nbr].present || static_cast<int>(q.b.size()) != q.n ||
                            static_cast<int>(q.c.size()) != q.n || static_cast<int>(q.cOff.size()) != q.n)
                            throw InputError("TFSF CPML list outside its line");
                }
                if ((L.useJ && !tp.line[L.nbrJ].present) || (L.useK && !tp.line[L.nbrK].present) || L.recIdx < 0 ||
                    L.recIdx >= tp.pulseLen || L.recOffIdx < 0 || L.recOffIdx >= tp.pulseLen || tp.pulAddStart < 0 ||
                    tp.pulAddStart + tp.mTot > tp.pulseLen || static_cast<int>(L.dist.size()) != tp.mTot)
                    throw InputError("TFSF line set-up inconsistent");
                auto psiList = [&](const TfsfPsi& q) {
                    dev::TfsfPsiDev o{};
                    o.nbr = q.nbr;
                    o.loc = q.loc;
                    o.locOff = q.locOff;
                    o.gridLoc = q.gridLoc;
                    o.n = q.n;
                    o.Db = q.Db;
                    o.b = mem_.upload(q.b);
                    o.c = mem_.upload(q.c);
                    o.cOff = mem_.upload(q.cOff);
                    o.psi = mem_.alloc<double2>(static_cast<std::size_t>(q.n));
                    return o;
                };
                d.nPml = static_cast<int>(L.pml.size());
                for (int q = 0; q < d.nPml; ++q) d.pml[q] = psiList(L.pml[q]);
                d.nPmlPulse = static_cast<int>(L.pmlPulse.size());
                for (int q = 0; q < d.nPmlPulse; ++q) d.pmlPulse[q] = psiList(L.pmlPulse[q]);
                d.recIdx = L.recIdx;
                d.recOffIdx = L.recOffIdx;
            }
            // fillPulseVec for every step (SOURCE/parallelTFSF.cpp:76-81) at t = step * dt
            std::vector<double2> tab(static_cast<std::size_t>(std::max(P.nSteps, 1)) * 6 * tp.mTot, make_double2(0.0, 0.0));
            for (int st = 0; st < P.nSteps; ++st)
                for (int c = 0; c < 6; ++c) {
                    if (!tp.line[c].present) continue;
                    for (int r = 0; r < tp.mTot; ++r) {
                        cplx v = 0.0;
                        for (const PulseSpec& p : tp.pulses) v = v + p.value(static_cast<double>(st) * tp.dt - tp.line[c].dist[r]);
                        tab[(static_cast<std::size_t>(st) * 6 + c) * tp.mTot + r] = make_double2(v.real(), v.imag());
                    }
                }
            t.pulseTab = mem_.upload(tab);
            t.rec = mem_.alloc<double2>(6 * 2 * (static_cast<std::size_t>(P.nSteps) + 1));
            t.ticket = mem_.alloc<unsigned int>(1);
            const TfsfAdds* adds[2] = {&tp.addH, &tp.addE};
            const std::vector<TfsfSegment>* segs[2] = {&tp.segH, &tp.segE};
            for (int w = 0; w < 2; ++w) {
                // rows split into runs of single-term cells; the cells with several terms
                // (face edges, few) go to the per-cell list
                const TfsfAdds& a = *adds[w];
                long long nTerms = 0;
                for (const TfsfSegment& g : *segs[w]) nTerms += g.n;
                std::vector<long long> multiKeys;
                for (std::size_t q = 0; q < a.cells(); ++q)
                    if (a.start[q + 1] - a.start[q] > 1) multiKeys.push_back(a.comp[q] * P.dims.cells() + a.cell[q]);
                std::sort(multiKeys.begin(), multiKeys.end());
                auto multi = [&](long long key) { return std::binary_search(multiKeys.begin(), multiKeys.end(), key); };
                std::vector<dev::TfsfSegDev> sd;
                std::vector<int2> sw;
                for (const TfsfSegment& g : *segs[w]) {
                    int r = 0;
                    while (r < g.n) {
                        while (r < g.n && multi(g.comp * P.dims.cells() + g.cell0 + r * g.cellStride)) ++r;
                        const int r0 = r;
                        while (r < g.n && !multi(g.comp * P.dims.cells() + g.cell0 + r * g.cellStride)) ++r;
                        if (r == r0) continue;
                        dev::TfsfSegDev d{};
                        d.toD = g.toD ? 1 : 0;
                        d.div = g.div;
                        if (d.toD || d.div >= 0) t.layered = 1;
                        d.cell0 = pad(g.cell0 + r0 * g.cellStride);
                        d.cellStride = padOffset(g.cellStride);
                        d.incd0 = g.incd0 + r0 * g.incdStride;
                        d.incdStride = g.incdStride;
                        d.n = r - r0;
                        d.line = g.line;
                        d.comp = g.comp;
                        d.pref = g.pref;
                        const long long lastCell = d.cell0 + static_cast<long long>(d.n - 1) * d.cellStride;
                        const long long lastIncd = d.incd0 + static_cast<long long>(d.n - 1) * d.incdStride;
                        if (d.cell0 < 0 || lastCell >= cellsPad_ || d.incd0 < 0 || lastIncd >= tp.gridLen || d.cellStride < 0 ||
                            d.incdStride < 0 || !tp.line[d.line].present || !P.comp[d.comp].present ||
                            (d.div >= 0 && (d.div > 5 || !tp.line[d.div].present)))
                            throw InputError("TFSF surface row outside its grids");
                        if (d.toD && (d.comp > 2 || !fields_.f[6 + d.comp]))
                            throw UnsupportedError("TFSF correction into a D field the grid does not have");
                        for (int c = 0; c * dev::kTfsfRowChunk < d.n; ++c) sw.push_back(make_int2(static_cast<int>(sd.size()), c));
                        sd.push_back(d);
                    }
                }
                t.seg[w] = mem_.upload(sd);
                t.segWork[w] = mem_.upload(sw);
                t.segBlocks[w] = static_cast<int>(sw.size());
                std::vector<long long> cell;
                std::vector<int> comp, start, tl, ti, tf;
                std::vector<double> pref;
                if (static_cast<long long>(a.terms()) != nTerms) throw InputError("TFSF surface rows and cell lists disagree");
                for (std::size_t q = 0; q < a.cells(); ++q) {
                    if (a.start[q + 1] - a.start[q] < 2) continue;  // in a row
                    cell.push_back(pad(a.cell[q]));
                    comp.push_back(a.comp[q]);
                    start.push_back(static_cast<int>(tl.size()));
                    for (long long k = a.start[q]; k < a.start[q + 1]; ++k) {
                        if (!tp.line[a.line[k]].present || a.incd[k] < 0 || a.incd[k] >= tp.gridLen ||
                            a.cell[q] < 0 || a.cell[q] >= P.dims.cells() || !P.comp[a.comp[q]].present ||
                            (a.div[k] >= 0 && (a.div[k] > 5 || !tp.line[a.div[k]].present)))
                            throw InputError("TFSF correction outside its grids");
                        if (a.toD[k] && (a.comp[q] > 2 || !fields_.f[6 + a.comp[q]]))
                            throw UnsupportedError("TFSF correction into a D field the grid does not have");
                        tl.push_back(a.line[k]);
                        ti.push_back(a.incd[k]);
                        pref.push_back(a.pref[k]);
                        tf.push_back((a.toD[k] ? 1 : 0) | ((a.div[k] + 1) << 1));
                        if (tf.back() != 0) t.layered = 1;
                    }
                }
                start.push_back(static_cast<int>(tl.size()));
                t.nCell[w] = static_cast<int>(cell.size());
                t.cell[w] = mem_.upload(cell);
                t.comp[w] = mem_.upload(comp);
                t.start[w] = mem_.upload(start);
                t.termLine[w] = mem_.upload(tl);
                t.termIncd[w] = mem_.upload(ti);
                t.termPref[w] = mem_.upload(pref);
                t.termFlag[w] = mem_.upload(tf);
            }
            tfsf_.push_back(t);
        }
    }

    // emitters after D -> E, before the step counter moves (parallelFDTDField.hpp:1281-1287)
    void launchEmitters(void* s) {
        T* const ef[3] = {fields_.f[0], fields_.f[1], fields_.f[2]};
        for (auto& e : emit_) dev::launch_emitter_step<T>(e, ef, dStep_, s);
    }

    // Oriented-dipole polarisation entries, their dipole directions (entry-fastest per
    // pole and axis) and the full-grid P / P_prev arrays per component and pole.
    void uploadOrDip(dev::Pass<T>& pass) {
        const OrDipPlan& od = P.ordip;
        std::memset(&pass.od, 0, sizeof(pass.od));
        if (!od.present || od.cells.empty()) return;
        if (od.nPoles > dev::kMaxPoles) throw UnsupportedError("more than 8 oriented-dipole poles");
        const std::size_t N = static_cast<std::size_t>(cellsPad_);
        const long long n = static_cast<long long>(od.cells.size());
        pass.od.n = n;
        pass.od.nPoles = od.nPoles;
        pass.od.cell = mem_.upload(padCells(od.cells));
        pass.od.obj = mem_.upload(od.obj);
        std::vector<T> dip(static_cast<std::size_t>(od.nPoles) * 3 * n);
        for (long long j = 0; j < n; ++j)
            for (int pp = 0; pp < od.nPoles; ++pp)
                for (int a = 0; a < 3; ++a)
                    dip[(static_cast<std::size_t>(pp) * 3 + a) * n + j] = static_cast<T>(od.dip[j * od.nPoles + pp][a]);
        pass.od.dip = mem_.upload(dip);
        for (int c = 0; c < 3; ++c) {
            pass.od.off[c] = padOffset(od.offA[c]);
            for (int pp = 0; pp < od.nPoles; ++pp) {
                pass.od.P[c][pp] = mem_.alloc<T>(N);
                pass.od.Pprev[c][pp] = mem_.alloc<T>(N);
            }
        }
        for (long long j = 0; j < n; ++j) {
            const long long i = od.cells[j];
            if (i - od.offA[1] < 0 || i >= P.dims.cells()) throw InputError("oriented-dipole cell outside the grid");
        }
    }

    // Whether the density matrices stay Hermitian with a real symmetric Hamiltonian: every
    // dipole operator real and symmetric, and the relaxation rows map each element pair
    // (r, c), (c, r) onto conjugate pairs with equal rates (then the mirrored row of a
    // row holds the mirrored columns with the same values).
    static bool hermitianForm(const EmitterPlan& ep) {
        const int N = ep.nlevel;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < N; ++r)
                for (int k = 0; k < N; ++k) {
                    const std::complex<double> a = ep.mu[c][r + k * N], b = ep.mu[c][k + r * N];
                    if (a.imag() != 0.0 || b.imag() != 0.0 || a.real() != b.real()) return false;
                }
        auto mirror = [N](int i) { return (i / N) + (i % N) * N; };
        std::vector<std::vector<std::pair<int, double>>> rows(static_cast<std::size_t>(N) * N);
        for (std::size_t ii = 0; ii < ep.gam.size() && ii < rows.size(); ++ii) rows[ii] = ep.gam[ii];
        for (int ii = 0; ii < N * N; ++ii)
            for (const auto& g : rows[ii]) {
                bool found = false;
                for (const auto& h : rows[mirror(ii)])
                    if (h.first == mirror(g.first) && h.second == g.second) found = true;
                if (!found) return false;
            }
        return true;
    }

    // Device state of the emitter objects: FP64 density matrices (one per cell and
    // ensemble member) initialised to the member weight in rho[0], four zeroed derivative
    // slots, the P boxes, and the constants of the plan.
    void uploadEmitters() {
        const Dims& D = P.dims;
        for (const EmitterPlan& ep : P.emitters) {
            if (ep.nlevel > dev::kMaxEmitterLevels) throw UnsupportedError("emitters with more than 8 levels");
            if (ep.dtcLevs.size() > 8) throw UnsupportedError("more than 8 population detectors on one emitter");
            dev::EmitterDev e{};
            const int N = ep.nlevel, n2 = N * N;
            e.N = N;
            e.n2 = n2;
            e.nm = ep.nMembers;
            e.nc = static_cast<int>(ep.cellGrid.size());
            e.h0 = mem_.upload(ep.h0);
            std::vector<double2> mu(3 * n2), nmu(3 * n2);
            for (int c = 0; c < 3; ++c)
                for (int i = 0; i < n2; ++i) {
                    mu[c * n2 + i] = make_double2(ep.mu[c][i].real(), ep.mu[c][i].imag());
                    nmu[c * n2 + i] = make_double2(ep.negMu[c][i].real(), ep.negMu[c][i].imag());
                }
            e.mu = mem_.upload(mu);
            e.negMu = mem_.upload(nmu);
            for (int c = 0; c < 3; ++c) {
                e.addMu[c] = ep.addMu[c] ? 1 : 0;
                e.comp[c] = ep.comp[c] ? 1 : 0;
            }
            e.gatherZCopy = ep.gatherZCopy ? 1 : 0;
            std::vector<int> row(n2 + 1, 0), col;
            std::vector<double> val;
            for (int ii = 0; ii < n2; ++ii) {
                row[ii] = static_cast<int>(col.size());
                if (ii < static_cast<int>(ep.gam.size()))
                    for (auto& g : ep.gam[ii]) {
                        col.push_back(g.first);
                        val.push_back(g.second);
                    }
            }
            row[n2] = static_cast<int>(col.size());
            if (col.empty()) {
                col.push_back(0);
                val.push_back(0.0);
            }
            e.herm = hermitianForm(ep) ? 1 : 0;
            // H = h0 - E . mu: the diagonal and the nonzero elements of the coupled operators
            e.hmask = 0;
            for (int i = 0; i < n2 && i < 32; ++i) {
                bool nz = (i % N) == (i / N);
                for (int c = 0; c < 3; ++c)
                    if (ep.addMu[c] && ep.negMu[c][i] != std::complex<double>(0.0, 0.0)) nz = true;
                if (nz) e.hmask |= 1u << i;
            }
            if (n2 > 32) e.herm = 0;
            e.gamRow = mem_.upload(row);
            e.gamCol = mem_.upload(col);
            e.gamVal = mem_.upload(val);
            e.dt = ep.dt;
            e.hbar = ep.hbar;
            // PCABAM4 weights (parallelQE.hpp:727-770), as the device formed them
            e.abP[0] = 55.0 * ep.dt / 24.0;
            e.abP[1] = -59.0 * ep.dt / 24.0;
            e.abP[2] = 37.0 * ep.dt / 24.0;
            e.abP[3] = -9.0 * ep.dt / 24.0;
            e.abC[0] = 9.0 * ep.dt / 24.0;
            e.abC[1] = 19.0 * ep.dt / 24.0;
            e.abC[2] = -5.0 * ep.dt / 24.0;
            e.abC[3] = ep.dt / 24.0;
            e.invHbar = 1.0 / ep.hbar;
            e.na = ep.na;
            e.cellGrid = mem_.upload(padCells(ep.cellGrid));
            e.cellDip = nullptr;
            if (!ep.cellDip.empty()) {
                if (ep.cellDip.size() != ep.cellGrid.size()) throw InputError("per-cell dipoles do not match the emitter cells");
                std::vector<double> w(3 * ep.cellDip.size());
                for (std::size_t q = 0; q < ep.cellDip.size(); ++q)
                    for (int c = 0; c < 3; ++c) w[c * ep.cellDip.size() + q] = ep.cellDip[q][c];
                e.cellDip = mem_.upload(w);
            }
            e.cellP = mem_.upload(ep.cellP);
            e.unit[0] = 1;
            e.unit[1] = pitch_ * D.lz;
            e.unit[2] = pitch_;
            const std::size_t nstate = static_cast<std::size_t>(e.nm) * n2 * e.nc;
            std::vector<double2> rho(nstate, make_double2(0.0, 0.0));
            for (int m = 0; m < e.nm; ++m)
                for (int q = 0; q < e.nc; ++q) rho[static_cast<std::size_t>(m) * n2 * e.nc + q] = make_double2(ep.weight[m], 0.0);
            // FP32 fields with the Hermitian form: the split update (float-float state, FP32
            // histories; emitter_kernels.cu, memberHermSplit); otherwise FP64 state and histories
            e.split = (sizeof(T) == 4 && e.herm && N >= 2 && N <= 4) ? 1 : 0;
            if (e.split) {
                auto pair = [](double v) {
                    const float hi = static_cast<float>(v);
                    return std::make_pair(hi, static_cast<float>(v - static_cast<double>(hi)));
                };
                std::vector<float4> rf(nstate);
                for (std::size_t k = 0; k < nstate; ++k) {
                    const auto re = pair(rho[k].x), im = pair(rho[k].y);
                    rf[k] = make_float4(re.first, re.second, im.first, im.second);
                }
                e.rhoF = mem_.upload(rf);
                e.kdF = mem_.alloc<float2>(4 * nstate);
                std::vector<float2> dl(static_cast<std::size_t>(e.nm) * n2, make_float2(0.f, 0.f));
                for (int m = 0; m < e.nm; ++m)
                    for (int i = 0; i < N; ++i)
                        for (int j = 0; j < N; ++j) {
                            const double d = (ep.h0[static_cast<std::size_t>(m) * N + i] - ep.h0[static_cast<std::size_t>(m) * N + j]) / ep.hbar;
                            const auto pr = pair(d);
                            dl[static_cast<std::size_t>(m) * n2 + i + j * N] = make_float2(pr.first, pr.second);
                        }
                e.dlevF = mem_.upload(dl);
                std::vector<float> nmh(3 * n2), gv(val.size());
                for (int c = 0; c < 3; ++c)
                    for (int i = 0; i < n2; ++i) nmh[c * n2 + i] = static_cast<float>(ep.negMu[c][i].real() / ep.hbar);
                for (std::size_t k = 0; k < val.size(); ++k) gv[k] = static_cast<float>(val[k]);
                e.negMuHF = mem_.upload(nmh);
                e.gamValF = mem_.upload(gv);
                for (int k = 0; k < 4; ++k) {
                    e.abPf[k] = static_cast<float>(e.abP[k]);
                    e.abCf[k] = static_cast<float>(e.abC[k]);
                }
            } else {
                e.rho = static_cast<double2*>(mem_.upload(rho));
                e.kd = mem_.alloc<double2>(4 * nstate);
            }
            e.pBox = ep.pDims[0] * ep.pDims[1] * ep.pDims[2];
            e.P = mem_.alloc<double>(3 * static_cast<std::size_t>(e.pBox));
            std::vector<double> epsBox(e.pBox, 1.0);
            for (int j = 0; j < ep.pDims[1]; ++j)
                for (int k = 0; k < ep.pDims[2]; ++k)
                    for (int i = 0; i < ep.pDims[0]; ++i) {
                        const int gx = ep.boxBase[0] + i, gy = ep.boxBase[1] + j, gz = ep.boxBase[2] + k;
                        if (gx < D.lx && gy < D.ly && gz < D.lz)
                            epsBox[i + ep.pDims[0] * (k + ep.pDims[2] * j)] = P.epsP[static_cast<std::size_t>(D.idx(gx, gy, gz))];
                    }
            for (double& v : epsBox) v = -0.5 / v;
            e.negHalfInvEps = mem_.upload(epsBox);
            for (int k = 0; k < 3; ++k) {
                e.pDims[k] = ep.pDims[k];
                e.addN[k] = ep.addN[k];
                e.boxBase[k] = ep.boxBase[k];
            }
            e.zOff = ep.zOff;
            e.lx = static_cast<int>(pitch_);
            e.lz = D.lz;
            e.nDtc = static_cast<int>(ep.dtcLevs.size());
            std::vector<int> lev = ep.dtcLevs;
            if (lev.empty()) lev.push_back(0);
            e.dtcLev = mem_.upload(lev);
            e.dtcTimeInt = ep.dtcTimeInt;
            e.nPoints = static_cast<double>(ep.nPoints);
            e.partialBlocks = (e.nc + 127) / 128;
            e.popPartial = mem_.alloc<double2>(static_cast<std::size_t>(e.partialBlocks) * std::max(e.nDtc, 1));
            e.totPartial = mem_.alloc<double>(static_cast<std::size_t>(e.partialBlocks) * 3);
            e.nSteps = P.nSteps;
            e.nEvents = P.nSteps > 0 ? (P.nSteps - 1) / ep.dtcTimeInt + 1 : 1;
            e.pop = mem_.alloc<double2>(static_cast<std::size_t>(std::max(e.nDtc, 1)) * e.nEvents);
            e.totP = ep.outputPol ? mem_.alloc<double>(3 * static_cast<std::size_t>(std::max(P.nSteps, 1))) : nullptr;
            emit_.push_back(e);
        }
    }

    // The graph of K steps. When the fold period divides K, it holds only the fold launches of
    // a replay that starts at a multiple of the period (graphAligned_), and step() replays it
    // only from such steps; otherwise every step carries its fold launches.
    void buildGraph(int K) {
        cudaGraph_t g;
        graphAligned_ = K % foldPeriod() == 0;
        ck(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        for (int k = 0; k < K; ++k) enqueueStep(k, !graphAligned_);
        ck(cudaStreamEndCapture(stream_, &g), "cudaStreamEndCapture");
        ck(cudaGraphInstantiate(&graph_, g, 0), "cudaGraphInstantiate");
        cudaGraphDestroy(g);
    }

    // A dispersive class whose object has Lorentz poles (the others only divide D by eps_inf).
    bool lorHasPoles(const ClassInfo& k) const {
        return k.obj < 0 || k.obj >= static_cast<int>(P.alpha.size()) || !P.alpha[k.obj].empty();
    }

    // Per term, the coordinate bounds outside which no cell uses the term's CPML
    // profile or psi, and whether the 3-D interior kernel form applies.
    void setSlabsAndForm(dev::Pass<T>& pass, bool ePass) const {
        const Dims& D = P.dims;
        const bool twoD = D.lz == 1;
        bool interior = true;
        for (int ci = 0; ci < 3; ++ci) {
            const CompPlan& cp = P.comp[(ePass ? 0 : 3) + ci];
            dev::Comp<T>& dc = pass.c[ci];
            const int axes[2] = {(ci + 2) % 3, (ci + 1) % 3};
            if (!cp.present) {
                // a 2-D grid has one polarisation: the other components are absent
                if (!twoD) interior = false;
                continue;
            }
            for (int t = 0; t < 2; ++t) {
                const TermPlan& tp = cp.term[t];
                const int L = tp.axis == 0 ? D.lx : (tp.axis == 1 ? D.ly : D.lz);
                dc.slabLo[t] = 0;
                dc.slabHi[t] = L;
                if (twoD && axes[t] == 2) {
                    // the derivative along z of a 2-D grid: the term must be absent
                    dc.slabHi[t] = 1;
                    if (tp.present) interior = false;
                    continue;
                }
                const int field = (ePass ? 3 : 0) + (t == 0 ? (ci + 1) % 3 : (ci + 2) % 3);
                if (!tp.present || tp.axis != axes[t] || tp.field != field) {
                    interior = false;
                    continue;
                }
                const long long unit[3] = {1, static_cast<long long>(D.lx) * D.lz, D.lx};
                if (tp.off != (ePass ? -1 : 1) * unit[tp.axis]) interior = false;
                std::vector<uint8_t> uses(cp.classes.size(), 0);
                bool anyUse = false;
                for (std::size_t q = 0; q < cp.classes.size(); ++q) {
                    const ClassInfo& k = cp.classes[q];
                    // cells that only add psi without updating it add zero (their psi is never written)
                    uses[q] = (k.kflag[t] || k.psiUpd[t]) ? 1 : 0;
                    anyUse = anyUse || uses[q];
                }
                if (!anyUse) continue;  // empty slab: no a satisfies a < 0 or a >= L
                int lo = 0, hi = L;
                if (static_cast<int>(tp.slabUse.size()) == L) {
                    // the coordinates the plan marked: the same cells as the classes' flags
                    for (int a = 0; a < L; ++a) {
                        if (!tp.slabUse[a]) continue;
                        if (2 * a < L) lo = std::max(lo, a + 1);
                        else hi = std::min(hi, a);
                    }
                    dc.slabLo[t] = lo;
                    dc.slabHi[t] = hi;
                    continue;
                }
                const uint8_t* code = cp.code.data();
                const int ax = tp.axis;
#pragma omp parallel for schedule(static) reduction(max : lo) reduction(min : hi)
                for (int y = 0; y < D.ly; ++y)
                    for (int z = 0; z < D.lz; ++z) {
                        const long long row = static_cast<long long>(D.lx) * (z + static_cast<long long>(D.lz) * y);
                        for (int x = 0; x < D.lx; ++x) {
                            if (!uses[code[row + x]]) continue;
                            const int a = ax == 0 ? x : (ax == 1 ? y : z);
                            if (2 * a < L) lo = std::max(lo, a + 1);
                            else hi = std::min(hi, a);
                        }
                    }
                dc.slabLo[t] = lo;
                dc.slabHi[t] = hi;
            }
        }
        // the interior form never visits halo cells: all of them must be inactive
        if (interior) {
            for (int ci = 0; ci < 3 && interior; ++ci) {
                if (!P.comp[(ePass ? 0 : 3) + ci].present) continue;  // no code array
                const std::vector<uint8_t>& code = P.comp[(ePass ? 0 : 3) + ci].code;
                if (static_cast<long long>(code.size()) != D.cells()) {
                    interior = false;
                    break;
                }
                for (int y = 0; y < D.ly && interior; ++y)
                    for (int z = 0; z < D.lz && interior; ++z) {
                        const long long row = static_cast<long long>(D.lx) * (z + static_cast<long long>(D.lz) * y);
                        const bool edge = (y == 0 || y == D.ly - 1 || (!twoD && (z == 0 || z == D.lz - 1)));
                        if (edge) {
                            for (int x = 0; x < D.lx; ++x)
                                if (code[row + x]) interior = false;
                        } else if (code[row] || code[row + D.lx - 1]) {
                            interior = false;
                        }
                    }
            }
        }
        pass.interior3d = (interior && !twoD) ? 1 : 0;
        pass.interior2d = (interior && twoD) ? 1 : 0;
        pass.index64 = cellsPad_ + 2LL * pitch_ * D.lz >= (1LL << 31) ? 1 : 0;
    }

    // Host-side bounds validation of every index the kernels will dereference.
    void validatePlan() {
        const Dims& D = P.dims;
        const long long N = D.cells();
        for (int c = 0; c < 6; ++c) {
            const CompPlan& cp = P.comp[c];
            if (!cp.present) continue;
            if (static_cast<long long>(cp.code.size()) != N) throw InputError("class code array size");
            for (int t = 0; t < 2; ++t) {
                const TermPlan& tp = cp.term[t];
                if (!tp.present) continue;
                int L = tp.axis == 0 ? D.lx : (tp.axis == 1 ? D.ly : D.lz);
                if (static_cast<int>(tp.kprof.size()) != L || static_cast<int>(tp.b.size()) != L) throw InputError("profile size");
                if (!P.comp[tp.field].present) throw InputError("neighbour field absent");
            }
            // every code indexes the class table and every coded cell's neighbour stays
            // inside the grid (a cell farther than its offsets from either end of the
            // array always has its neighbours inside); the cells of each class are counted
            // on the way
            const int ncls = static_cast<int>(cp.classes.size());
            const long long off0 = cp.term[0].present ? cp.term[0].off : 0, off1 = cp.term[1].present ? cp.term[1].off : 0;
            const long long edge = std::max(std::abs(off0), std::abs(off1));
            std::vector<long long> count(256, 0);
            int bad = 0;
            const uint8_t* code = cp.code.data();
#pragma omp parallel
            {
                long long local[256] = {0};
#pragma omp for schedule(static)
                for (long long i = 0; i < N; ++i) ++local[code[i]];
#pragma omp critical
                for (int q = 0; q < 256; ++q) count[q] += local[q];
            }
            for (int q = ncls; q < 256; ++q)
                if (count[q]) bad |= 1;
            for (long long i = 0; i < std::min(edge, N); ++i)
                if (code[i] && (i + off0 < 0 || i + off0 >= N || i + off1 < 0 || i + off1 >= N)) bad |= 2;
            for (long long i = std::max(edge, N - edge); i < N; ++i)
                if (code[i] && (i + off0 < 0 || i + off0 >= N || i + off1 < 0 || i + off1 >= N)) bad |= 2;
            if (bad & 1) throw InputError("class code outside the class table");
            if (bad & 2) throw InputError("stencil neighbour outside the grid");
            classCount_[c].assign(count.begin(), count.begin() + ncls);
        }
        for (auto& s : P.sources)
            for (long long c : s.cells)
                if (c < 0 || c >= N) throw InputError("source cell outside the grid");
        for (auto& d : P.detectors)
            for (auto& f : d.fields)
                for (long long c : f.cells)
                    if (c >= N) throw InputError("detector cell outside the grid");
        for (auto& fp : P.fluxes)
            for (auto& st : fp.stores)
                for (long long c : st.cells)
                    if (c < 0 || c >= N) throw InputError("flux cell outside the grid");
    }

    void upload() {
        PhaseClock clk;
        const Dims& D = P.dims;
        // device rows of pitch_ >= lx values, a multiple of 4, so that every row starts on a
        // 16-byte boundary (32 bytes in FP64)
        pitch_ = (static_cast<long long>(D.lx) + 3) / 4 * 4;
        cellsPad_ = pitch_ * D.ly * D.lz;
        const std::size_t N = static_cast<std::size_t>(cellsPad_);
        // fields
        for (int c = 0; c < 6; ++c)
            if (P.comp[c].present) fields_.f[c] = mem_.alloc<T>(N);
        for (int c = 0; c < 3; ++c)
            if (P.comp[c].present && P.comp[c].hasD) fields_.f[6 + c] = mem_.alloc<T>(N);
        fluxDev_.assign(P.fluxes.size(), FluxFacesDev());
        std::vector<std::vector<FluxFaceMap>> maps(P.fluxes.size());
        clk.mark("up-fields");
        // independent parts, each on a host thread of its own: the plan's validation (its
        // failure is reported before any other; no kernel runs before it has passed), the
        // pass tables, the sources and detector records, the DFT tables and then the flux
        // face maps on the device, the emitters, the TFSF surfaces; the flux face maps are
        // built on the host meanwhile (the DFT task waits for them)
        std::shared_future<void> mapsReady = std::async(std::launch::async, [&] {
                                                 PhaseClock c;
                                                 buildFluxMaps(maps);
                                                 c.mark("task-flux-maps");
                                             }).share();
        auto timed = [](const char* what, const std::function<void()>& f) {
            return [what, f] {
                PhaseClock c;
                f();
                c.mark(what);
            };
        };
        runConcurrently(opt_.device, {timed("task-validate", [&] { validatePlan(); }), timed("task-passes", [&] { uploadPasses(); }),
                                      timed("task-src-rec", [&] { uploadSourcesRecords(); }),
                                      timed("task-dft-flux",
                                            [&] {
                                                uploadDftTables();
                                                mapsReady.get();
                                                for (std::size_t q = 0; q < P.fluxes.size(); ++q)
                                                    if (!P.fluxes[q].spec.save && !P.fluxes[q].spec.load) prepareFluxFaces(q, maps[q]);
                                            }),
                                      timed("task-emitters", [&] { uploadEmitters(); }), timed("task-tfsf", [&] { uploadTfsf(); })});
        mapsReady.wait();
        clk.mark("up-parts");
        uploadTail();
        clk.mark("up-tail");
        if (clk.on)
            std::fprintf(stderr, "host up: %.4f s in cudaMalloc + cudaMemset (%.0f MB), %.4f s in H2D copies (%.0f MB)\n",
                         mem_.allocSeconds, mem_.bytes / 1e6, mem_.copySeconds, mem_.h2d / 1e6);
    }

    // The face maps of every flux region (integration weights and accumulator points of
    // each face; the faces of a region are built on the host cores concurrently).
    void buildFluxMaps(std::vector<std::vector<FluxFaceMap>>& maps) {
        for (std::size_t k = 0; k < P.fluxes.size(); ++k)
            if (!P.fluxes[k].spec.save && !P.fluxes[k].spec.load) maps[k] = flux_face_maps(P, k);
    }

    // Pole coefficients, the class codes and tables, CPML profiles and psi arrays of both
    // passes, the oriented-dipole lists.
    void uploadPasses() {
        PhaseClock clk;
        const Dims& D = P.dims;
        const std::size_t N = static_cast<std::size_t>(cellsPad_);
        // poles: per object start / count
        std::vector<int> pStart, pCount;
        std::vector<T> al, xi, ga;
        for (std::size_t o = 0; o < P.alpha.size(); ++o) {
            pStart.push_back(static_cast<int>(al.size()));
            pCount.push_back(static_cast<int>(P.alpha[o].size()));
            for (std::size_t q = 0; q < P.alpha[o].size(); ++q) {
                // the FP32 kernels take the increment form's coefficients (kIncrementPoles)
                al.push_back(static_cast<T>(dev::kIncrementPoles<T> ? P.alphaInc[o][q] : P.alpha[o][q]));
                xi.push_back(static_cast<T>(dev::kIncrementPoles<T> ? -1.0 * P.xi[o][q] : P.xi[o][q]));
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
            pass.pitch = pitch_;
            pass.poleStart = dStart;
            pass.poleCount = dCount;
            pass.poleA = dAl;
            pass.poleB = dXi;
            pass.gamma = dGa;
            pass.nObj = static_cast<int>(pCount.size());
            for (int ci = 0; ci < 3; ++ci) {
                const int c = (half ? 0 : 3) + ci;
                const CompPlan& cp = P.comp[c];
                dev::Comp<T>& dc = pass.c[ci];
                std::memset(&dc, 0, sizeof(dc));
                if (!cp.present) continue;
                dc.present = 1;
                dc.U = fields_.f[c];
                dc.D = (c < 3) ? fields_.f[6 + c] : nullptr;
                dc.code = uploadPadded(cp.code);
                clk.mark("up-code");
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
                    o.ordip = k.ordip;
                    o.odCoef = static_cast<T>(-0.5 / k.eps);
                    if ((k.lor || k.toD || k.ordip) && !cp.hasD) throw InputError("dispersive cell without a D field");
                }
                dc.cls = mem_.upload(cls);
                std::vector<dev::FastClass<T>> fcls(cp.classes.size());
                for (std::size_t q = 0; q < cp.classes.size(); ++q) {
                    const ClassInfo& k = cp.classes[q];
                    dev::FastClass<T>& o = fcls[q];
                    std::memset(&o, 0, sizeof(o));
                    bool write = false;
                    for (int t = 0; t < 2; ++t) {
                        const TermPlan& tp = cp.term[t];
                        const double base = k.cint[t] + static_cast<double>(k.nplain[t]) * (tp.present ? tp.db : 0.0);
                        o.coef[t] = static_cast<T>(base);
                        if (k.kflag[t]) o.flags |= (t == 0 ? dev::kFcKp0 : dev::kFcKp1);
                        const bool psiUpd = k.psiUpd[t] && tp.present && tp.hasPsi;
                        o.psiCoef[t] = psiUpd ? static_cast<T>(static_cast<double>(k.npsi[t]) * tp.dbpsi) : T(0);
                        if (psiUpd) o.flags |= (t == 0 ? dev::kFcPsi0 : dev::kFcPsi1);
                        if (k.kflag[t] || k.psiUpd[t]) o.flags |= (t == 0 ? dev::kFcSlab0 : dev::kFcSlab1);
                        if (base != 0.0 || k.kflag[t] || (psiUpd && k.npsi[t])) write = true;
                    }
                    if (k.lor && lorHasPoles(k)) o.flags |= dev::kFcLor;
                    if (k.lor && !lorHasPoles(k)) o.flags |= dev::kFcDtoE;
                    if (k.ordip) o.flags |= dev::kFcOrDip;
                    o.epsInv = static_cast<T>(1.0 / k.eps);
                    o.obj = static_cast<uint32_t>(k.obj < 0 ? 0x7fffffff : k.obj);
                    if (k.toD) o.flags |= dev::kFcToD;
                    if (write) o.flags |= dev::kFcWrite;
                }
                dc.fcls = mem_.upload(fcls);
                classFlags_[c].clear();
                for (auto& fc : fcls) classFlags_[c].push_back(fc.flags);
                dc.ncls = static_cast<int>(cls.size());
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
                    dc.off[t] = padOffset(tp.off);
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
            clk.mark("up-classes");
            setSlabsAndForm(pass, half == 1);
            clk.mark("up-slabs");
            if (half == 1) uploadOrDip(pass);
            clk.mark("up-ordip");
            if (half == 1 && (pass.interior3d || pass.interior2d) && !dev::kInlineDispersive<T>) {
                // dispersive cells leave the interior form for their own list kernel
                std::vector<int> lc;
                std::vector<long long> li;
                for (int ci = 0; ci < 3; ++ci) {
                    const CompPlan& cp = P.comp[ci];
                    if (!cp.present) continue;
                    for (long long i = 0; i < static_cast<long long>(cp.code.size()); ++i) {
                        if (cp.code[i] >= cp.classes.size()) continue;  // rejected by validatePlan
                        if (cp.code[i] && ((cp.classes[cp.code[i]].lor && lorHasPoles(cp.classes[cp.code[i]])) ||
                                           cp.classes[cp.code[i]].ordip)) {
                            lc.push_back(ci);
                            li.push_back(i);
                        }
                    }
                }
                pass.nLor = static_cast<long long>(li.size());
                pass.lorComp = mem_.upload(lc);
                pass.lorCell = mem_.upload(padCells(li));
            }
        }
        (void)bytes;
    }

    void uploadSourcesRecords() {
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
            src_.cell = mem_.upload(padCells(cell));
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
            recT_.cell = mem_.upload(padCells(cell));
            recT_.outIndex = mem_.upload(outIdx);
            recT_.timeInt = mem_.upload(ti);
            recT_.nvals = mem_.upload(nvals);
            recT_.recBase = mem_.upload(recBase_);
            recT_.nEvents = mem_.upload(nev);
            dRec_ = mem_.alloc<double>(recTotal_);
            recT_.rec = dRec_;
        }
    }

    // DFT tables: the flux regions, then the frequency-domain detectors
    void uploadDftTables() {
        for (auto& fp : P.fluxes) {
            std::vector<int> comp, cell;
            for (auto& st : fp.stores)
                for (long long c : st.cells) {
                    const long long pc = pad(c);
                    if (pc > 0x7fffffffLL) throw UnsupportedError("grid too large for 32-bit flux point indices");
                    comp.push_back(st.comp);
                    cell.push_back(static_cast<int>(pc));
                }
            dft_.push_back(makeDft(comp, cell, fp.spec.freqList, fp.spec.timeInt));
        }
        for (auto& dp : P.freqDetectors) {
            std::vector<int> comp, cell;
            for (auto& F : dp.fields)
                for (long long c : F.cells) {
                    const long long pc = pad(c);
                    if (c < 0 || pc > 0x7fffffffLL) throw UnsupportedError("frequency detector point outside 32-bit indices");
                    comp.push_back(F.comp);
                    cell.push_back(static_cast<int>(pc));
                }
            dft_.push_back(makeDft(comp, cell, dp.spec.freqList, dp.timeInt));
        }
    }

    // One DFT table: point table (component, cell), phasors per sample from the accumulated
    // time, a ring of K samples and FP64 accumulators [point][frequency].
    // Position of each plan point of every DFT table in the device point order (points sorted
    // by component and cell, so that a warp's gathers share sectors: the two planes of a
    // face's averaged pair are neighbours in x). Accumulators, ring and tables are in the
    // device order; the flux maps and the frequency-detector downloads are translated.
    std::vector<std::vector<int>> dftPos_;

    dev::DftTable<T> makeDft(const std::vector<int>& comp0, const std::vector<int>& cell0, const std::vector<double>& freqs, int ti) {
        // (component, cell, plan index) keys: unique, so that the parallel sort gives the
        // order of a stable sort by (component, cell)
        const long long npt = static_cast<long long>(cell0.size());
        std::vector<std::pair<std::pair<int, int>, int>> key(cell0.size());
#pragma omp parallel for schedule(static)
        for (long long k = 0; k < npt; ++k) key[static_cast<std::size_t>(k)] = {{comp0[k], cell0[k]}, static_cast<int>(k)};
        __gnu_parallel::sort(key.begin(), key.end());
        std::vector<int> comp(cell0.size()), cell(cell0.size()), pos(cell0.size());
#pragma omp parallel for schedule(static)
        for (long long k = 0; k < npt; ++k) {
            const std::size_t q = static_cast<std::size_t>(k);
            comp[q] = key[q].first.first;
            cell[q] = key[q].first.second;
            pos[static_cast<std::size_t>(key[q].second)] = static_cast<int>(k);
        }
        dftPos_.push_back(std::move(pos));
        dev::DftTable<T> d{};
        {
            const int nf = static_cast<int>(freqs.size());
            const int nSamples = P.nSteps / ti + 1;
            const int nfPad = (nf + 31) / 32 * 32;
            std::vector<T> ph(static_cast<std::size_t>(nSamples) * nfPad * 2, T(0));
#pragma omp parallel for schedule(static)
            for (int n = 0; n < nSamples; ++n)
                for (int f = 0; f < nf; ++f) {
                    std::complex<double> e = std::exp(std::complex<double>(0.0, -1.0 * P.tcur[static_cast<std::size_t>(n) * ti] * freqs[f]));
                    ph[(static_cast<std::size_t>(n) * 2 + 0) * nfPad + f] = static_cast<T>(e.real());
                    ph[(static_cast<std::size_t>(n) * 2 + 1) * nfPad + f] = static_cast<T>(e.imag());
                }
            const int K = dftBlockLength(static_cast<long long>(cell.size()), nSamples);
            d.npts = static_cast<long long>(cell.size());
            d.stride = (d.npts + 127) / 128 * 128;
            d.nfreqPad = nfPad;
            d.nfreq = nf;
            d.timeInt = ti;
            d.K = K;
            d.nSamples = nSamples;
            d.comp = mem_.upload(comp);
            d.cell = mem_.upload(cell);
            d.phasor = mem_.upload(ph);
            d.ring = mem_.alloc<T>(static_cast<std::size_t>(d.stride) * static_cast<std::size_t>(K));
            d.re = mem_.alloc<double>(cell.size() * nf);
            d.im = mem_.alloc<double>(cell.size() * nf);
        }
        return d;
    }

    std::vector<long long> classCount_[6];  // cells of each class, per component
    dev::StepTail<T> tail_{};

    void uploadTail() {
        bytesPerCell_ = algorithmicBytesPerCell();
        dStep_ = mem_.alloc<int>(1);
        dErr_ = mem_.alloc<unsigned int>(1);
        hPass_.err = dErr_;
        ePass_.err = dErr_;
        recT_.err = dErr_;
        for (auto& d : dft_) d.err = dErr_;
        // a few soft sources on a 2-D grid: the E pass adds them (one launch less per step)
        srcInE_ = src_.n > 0 && ePass_.interior2d && sourcesInE();
        if (srcInE_) {
            ePass_.nSrcIn = src_.n;
            ePass_.srcComp = src_.comp;
            ePass_.srcCell = src_.cell;
            ePass_.srcId = src_.src;
            ePass_.srcValue = src_.value;
            ePass_.srcSteps = src_.nSteps;
            ePass_.step = dStep_;
        }
        // every copy and memset above has landed before the first kernel runs
        ck(cudaDeviceSynchronize(), "upload");
        kernelsPerStep_ = 3 + (src_.n && !srcInE_ ? 1 : 0) + static_cast<int>(dft_.size()) + (ePass_.nLor > 0 ? 1 : 0) + (ePass_.od.n > 0 ? 1 : 0) +
                          3 * static_cast<int>(emit_.size()) + 2 * static_cast<int>(tfsf_.size());
        // the step tail: record blocks, then each DFT table's sample blocks
        tail_ = dev::StepTail<T>{};
        tail_.rec = recT_;
        tail_.recBlocks = (recT_.n + 255) / 256;
        tail_.nDft = static_cast<int>(dft_.size());
        std::vector<int> start(1, 0);
        for (auto& d : dft_) start.push_back(start.back() + static_cast<int>((d.npts + 255) / 256));
        tail_.dft = mem_.upload(dft_);
        tail_.dftStart = mem_.upload(start);
        tail_.f = fields_;
        tail_.step = dStep_;
        tail_.ticket = mem_.alloc<unsigned int>(1);
        tail_.blocks = std::max(1, tail_.recBlocks + start.back());
        // t = 0 samples (parallelFDTDField.cpp:831-837)
        dev::launch_record<T>(recT_, fields_, dStep_, stream_);
        for (auto& d : dft_) dev::launch_dft_sample<T>(d, fields_, dStep_, stream_);
        ck(cudaStreamSynchronize(stream_), "initial samples");
    }

    // Samples per fold of a flux region: long blocks cut the accumulator
    // read-modify-write per step; the ring (K x points values) stays within 2 GB
    // and K stays near the run's sample count.
    static int dftBlockLength(long long npts, int nSamples) {
        int K = 256;
        while (K > 32 && static_cast<double>(K) * npts * sizeof(T) > 2.0e9) K /= 2;
        while (K > 32 && K / 2 >= nSamples) K /= 2;
        return K;
    }

    // Algorithmic HBM bytes of the passes: every array a pass touches is read
    // (and, if it is updated, written) once per launch -- the field components
    // of the pass, the neighbour components it reads, one class byte per
    // component and cell, and CPML psi (at the cells that update it), D and
    // Lorentz P/P_prev only at the cells whose class uses them. Per-step bytes per physical cell are the sum
    // of both passes over the physical cell count.
    double algorithmicBytesPerCell() {
        const Dims& D = P.dims;
        const double phys = static_cast<double>(D.nx) * D.ny * D.nz;
        const double cells = static_cast<double>(D.cells());
        const double t = static_cast<double>(sizeof(T));
        for (int half = 0; half < 2; ++half) {
            double b = 0.0;
            int own = 0, nbr = 0;
            for (int ci = 0; ci < 3; ++ci) {
                const int c = (half ? 0 : 3) + ci;
                if (P.comp[c].present) ++own;
                if (P.comp[(half ? 3 : 0) + ci].present) ++nbr;
            }
            b += cells * (own * (2.0 * t + 1.0) + nbr * t);
            for (int ci = 0; ci < 3; ++ci) {
                const int c = (half ? 0 : 3) + ci;
                const CompPlan& cp = P.comp[c];
                if (!cp.present) continue;
                const std::vector<long long>& count = classCount_[c];
                for (std::size_t q = 0; q < cp.classes.size(); ++q) {
                    const ClassInfo& k = cp.classes[q];
                    for (int tt = 0; tt < 2; ++tt)
                        if (k.psiUpd[tt]) b += count[q] * 2.0 * t;
                    if (k.lor) b += count[q] * t * (2.0 + 4.0 * P.alpha[k.obj].size());
                    else if (k.toD) b += count[q] * 2.0 * t;
                }
            }
            passBytes_[half] = b;  // [0] H pass, [1] E pass
        }
        // DFT per sampled step: gather (index 4 B + component 4 B + value read + ring write)
        // plus the fold's accumulator read-modify-write and ring read amortised over K
        dftBytes_ = 0.0;
        for (auto& d : dft_) {
            const double pts = static_cast<double>(d.npts);
            dftBytes_ += pts * (8.0 + 2.0 * t) + pts * (t + d.nfreq * 4.0 * sizeof(double)) / d.K;
        }
        return (passBytes_[0] + passBytes_[1]) / phys;
    }
};

// Independent simulations of one precision stepped by packed launches: per step one
// launch of each kind of work covers every member (H pass, sources, oriented-dipole P,
// E pass, emitters, step counters, detector records, DFT sample and fold), in the order
// of Sim::enqueueStep. The members' descriptors sit in device job arrays; a work table
// per launch maps each block to {job, block of that job}. 2-D members whose halo carries
// no update run the 2-D form of the passes (dispersive cells from their list), the
// others the generic form. The step is captured into a CUDA graph of `graphSteps` steps.
struct PackedBase {
    virtual ~PackedBase() {}
    virtual void run(long long n, int graphSteps) = 0;
};

template <typename T>
class PackedBatch : public PackedBase {
public:
    // march: the 2-D march depth per grid shape, chosen by the autotuner the first time
    // (all members fresh) and reused by later packings of the same batch.
    PackedBatch(const std::vector<Sim<T>*>& members, int device, int graphSteps, std::map<std::pair<int, int>, int>& march)
        : members_(members) {
        ck(cudaSetDevice(device), "cudaSetDevice");
        ck(cudaStreamCreate(&stream_), "cudaStreamCreate");
        std::vector<dev::Pass<T>> hp, ep;
        std::vector<dev::SrcJob<T>> src;
        std::vector<dev::RecJob<T>> rec;
        std::vector<dev::DftJob<T>> dft;
        std::vector<dev::EmitJob<T>> em;
        std::vector<int*> steps;
        std::vector<int2> passW, p2W[2], lorW, odW, srcW, recW, smpW, foldW, addW, updW[7];
        auto add = [](std::vector<int2>& w, int job, long long blocks) {
            for (long long b = 0; b < blocks; ++b) w.push_back(make_int2(job, static_cast<int>(b)));
        };
        for (Sim<T>* m : members) {
            const int j = static_cast<int>(hp.size());
            hp.push_back(m->hPass());
            ep.push_back(m->ePass());
            if (m->hPass().interior2d && m->ePass().interior2d) {
                // 2-D form: blocks of the present components only
                const dev::Pass<T>* ps[2] = {&m->hPass(), &m->ePass()};
                for (int h = 0; h < 2; ++h) {
                    const long long per = dev::pass2d_blocks_per_comp<T>(*ps[h]);
                    for (int ci = 0; ci < 3; ++ci)
                        if (ps[h]->c[ci].present)
                            for (long long b = 0; b < per; ++b) p2W[h].push_back(make_int2(j, static_cast<int>(ci * per + b)));
                }
                if (m->ePass().nLor > 0) add(lorW, j, dev::lorentz_blocks(m->ePass().nLor));
            } else {
                // generic form (its E pass runs the dispersive cells itself)
                add(passW, j, dev::pass_blocks<T>(m->hPass()));
                if (dev::pass_blocks<T>(m->ePass()) != dev::pass_blocks<T>(m->hPass()))
                    throw std::logic_error("H and E passes of a member differ in extent");
            }
            if (m->ePass().od.n > 0) add(odW, j, dev::ordip_blocks(m->ePass().od.n));
            if (m->sources().n > 0) {
                add(srcW, static_cast<int>(src.size()), dev::sources_blocks(m->sources().n));
                src.push_back(dev::SrcJob<T>{m->sources(), m->fields(), m->stepCounter()});
            }
            if (m->records().n > 0) {
                add(recW, static_cast<int>(rec.size()), dev::record_blocks(m->records().n));
                rec.push_back(dev::RecJob<T>{m->records(), m->fields(), m->stepCounter()});
            }
            for (const auto& d : m->dftTables()) {
                if (d.npts == 0) continue;
                const int q = static_cast<int>(dft.size());
                add(smpW, q, dev::dft_sample_blocks(d.npts));
                add(foldW, q, dev::dft_fold_blocks(d.npts, d.nfreq));
                dft.push_back(dev::DftJob<T>{d, m->fields(), m->stepCounter()});
            }
            for (const auto& e : m->emitters()) {
                const int q = static_cast<int>(em.size());
                const int bpc = dev::emitter_addp_blocks_per_comp(e);
                for (int c = 0; c < 3; ++c)
                    if (e.comp[c])
                        for (int b = 0; b < bpc; ++b) addW.push_back(make_int2(q, c * bpc + b));
                add(updW[dev::emitter_level_group(e.N, e.herm != 0)], q, dev::emitter_update_blocks(e));
                dev::EmitJob<T> jb{};
                jb.e = e;
                for (int c = 0; c < 3; ++c) jb.f[c] = m->fields().f[c];
                jb.step = m->stepCounter();
                em.push_back(jb);
            }
            steps.push_back(m->stepCounter());
        }
        auto map = [this](const std::vector<int2>& w) {
            if (w.size() > 0x7fffffffULL) throw UnsupportedError("a packed launch of more than 2^31 blocks");
            return dev::WorkMap{mem_.upload(w), static_cast<int>(w.size())};
        };
        dH_ = mem_.upload(hp);
        dE_ = mem_.upload(ep);
        dSrc_ = mem_.upload(src);
        dRec_ = mem_.upload(rec);
        dDft_ = mem_.upload(dft);
        dEm_ = mem_.upload(em);
        nEm_ = static_cast<int>(em.size());
        dSteps_ = mem_.upload(steps);
        nSteps_ = static_cast<int>(steps.size());
        passMap_ = map(passW);
        p2Map_[0] = map(p2W[0]);
        p2Map_[1] = map(p2W[1]);
        lorMap_ = map(lorW);
        odMap_ = map(odW);
        srcMap_ = map(srcW);
        recMap_ = map(recW);
        smpMap_ = map(smpW);
        foldMap_ = map(foldW);
        addMap_ = map(addW);
        for (int g = 0; g < 7; ++g) updMap_[g] = map(updW[g]);
        ck(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        autotune2d(hp, ep, march);
        // the packed step graph is made with the launches, not in the first run that uses it
        if (graphSteps > 0) buildGraph(graphSteps);
    }
    ~PackedBatch() {
        if (graph_) cudaGraphExecDestroy(graph_);
        if (stream_) {
            cudaStreamSynchronize(stream_);
            cudaStreamDestroy(stream_);
        }
    }

    // Queues n steps of every member and waits for them.
    void run(long long n, int graphSteps) override {
        for (Sim<T>* m : members_) ck(cudaStreamSynchronize(m->stream()), "cudaStreamSynchronize");
        if (graphSteps > 0 && n >= graphSteps) {
            if (!graph_ || graphSteps != graphSteps_) buildGraph(graphSteps);
            for (; n >= graphSteps; n -= graphSteps) ck(cudaGraphLaunch(graph_, stream_), "cudaGraphLaunch");
        }
        for (; n > 0; --n) enqueueStep();
        ck(cudaGetLastError(), "kernel launch");
        ck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    }

private:
    // The autotuner of the 2-D members: the march depth (rows per warp, the tile's extent
    // along y) is chosen per grid shape. Shapes in order of their total cells, each tries
    // the depths in kDepths with the others fixed, and keeps the one whose packed H and E
    // passes (all members) take least time, measured with CUDA events after one warm-up
    // launch. It runs only while every member is fresh: the fields are zero before the
    // first step and a pass maps zero fields to zero fields, so the trial launches leave
    // every member's state as it was. Later packings (members that finished leave the
    // batch) take the depths chosen then.
    void autotune2d(std::vector<dev::Pass<T>>& hp, std::vector<dev::Pass<T>>& ep, std::map<std::pair<int, int>, int>& chosen) {
        std::map<std::pair<int, int>, std::vector<int>> byShape;
        for (std::size_t j = 0; j < hp.size(); ++j)
            if (hp[j].interior2d && ep[j].interior2d) byShape[{hp[j].lx, hp[j].ly}].push_back(static_cast<int>(j));
        if (byShape.empty()) return;
        bool allFresh = true;
        for (Sim<T>* m : members_) allFresh = allFresh && m->fresh();
        // CHIML_BATCH_MARCH=2|4|8|16|32 fixes the depth of every shape instead of tuning
        if (const char* fixed = std::getenv("CHIML_BATCH_MARCH")) {
            const int v = std::atoi(fixed);
            if (v == 2 || v == 4 || v == 8 || v == 16 || v == 32)
                for (auto& g : byShape) chosen[g.first] = v;
        }
        bool known = true;
        for (auto& g : byShape) known = known && chosen.count(g.first) > 0;
        PhaseClock clk;
        static constexpr int kDepths[5] = {2, 4, 8, 16, 32};
        std::vector<std::pair<long long, std::vector<int>>> groups;
        for (auto& g : byShape) groups.push_back({static_cast<long long>(g.first.first) * g.first.second * g.second.size(), g.second});
        std::sort(groups.begin(), groups.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
        // work tables of both halves for the members' current depths, in buffers sized for
        // the shallowest depth (the most blocks)
        auto blocks2d = [&](int h, std::vector<int2>& w) {
            w.clear();
            const std::vector<dev::Pass<T>>& ps = h ? ep : hp;
            for (std::size_t j = 0; j < ps.size(); ++j) {
                if (!(hp[j].interior2d && ep[j].interior2d)) continue;
                const long long per = dev::pass2d_blocks_per_comp<T>(ps[j]);
                for (int ci = 0; ci < 3; ++ci)
                    if (ps[j].c[ci].present)
                        for (long long b = 0; b < per; ++b) w.push_back(make_int2(static_cast<int>(j), static_cast<int>(ci * per + b)));
            }
        };
        std::vector<int2> w[2];
        std::size_t cap = 0;
        for (auto& g : groups)
            for (int j : g.second) hp[j].march = ep[j].march = kDepths[0];
        for (int h = 0; h < 2; ++h) {
            blocks2d(h, w[h]);
            cap = std::max(cap, w[h].size());
        }
        int2* dW[2] = {mem_.alloc<int2>(cap, false), mem_.alloc<int2>(cap, false)};
        auto apply = [&] {
            ck(cudaMemcpy(dH_, hp.data(), hp.size() * sizeof(dev::Pass<T>), cudaMemcpyHostToDevice), "cudaMemcpy jobs");
            ck(cudaMemcpy(dE_, ep.data(), ep.size() * sizeof(dev::Pass<T>), cudaMemcpyHostToDevice), "cudaMemcpy jobs");
            for (int h = 0; h < 2; ++h) {
                blocks2d(h, w[h]);
                if (w[h].size() > cap) throw std::logic_error("packed work table larger than its buffer");
                ck(cudaMemcpy(dW[h], w[h].data(), w[h].size() * sizeof(int2), cudaMemcpyHostToDevice), "cudaMemcpy work");
                p2Map_[h] = dev::WorkMap{dW[h], static_cast<int>(w[h].size())};
            }
        };
        cudaEvent_t e0, e1;
        ck(cudaEventCreate(&e0), "cudaEventCreate");
        ck(cudaEventCreate(&e1), "cudaEventCreate");
        auto timePasses = [&] {
            apply();
            dev::launch_pass2d_packed<T>(dH_, p2Map_[0], false, stream_);
            dev::launch_pass2d_packed<T>(dE_, p2Map_[1], true, stream_);
            ck(cudaEventRecord(e0, stream_), "cudaEventRecord");
            for (int r = 0; r < 3; ++r) {
                dev::launch_pass2d_packed<T>(dH_, p2Map_[0], false, stream_);
                dev::launch_pass2d_packed<T>(dE_, p2Map_[1], true, stream_);
            }
            ck(cudaEventRecord(e1, stream_), "cudaEventRecord");
            ck(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float ms = 0.0f;
            ck(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
            return ms;
        };
        if (known || !allFresh) {
            // the depths chosen for the first packing (the default for a shape not tuned)
            for (auto& g : byShape) {
                const auto it = chosen.find(g.first);
                for (int j : g.second) hp[j].march = ep[j].march = it != chosen.end() ? it->second : dev::kP2CYDefault;
            }
            apply();
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            ck(cudaStreamSynchronize(stream_), "packed work tables");
            return;
        }
        for (auto& g : groups)
            for (int j : g.second) hp[j].march = ep[j].march = dev::kP2CYDefault;
        for (auto& g : groups) {
            int best = dev::kP2CYDefault;
            float bestMs = timePasses();
            for (int dpt : kDepths) {
                if (dpt == best) continue;
                for (int j : g.second) hp[j].march = ep[j].march = dpt;
                const float ms = timePasses();
                if (ms < 0.98f * bestMs) {
                    best = dpt;
                    bestMs = ms;
                }
            }
            for (int j : g.second) hp[j].march = ep[j].march = best;
            chosen[{hp[g.second[0]].lx, hp[g.second[0]].ly}] = best;
            if (clk.on)
                std::fprintf(stderr, "host tune %dx%d (%zu members): march %d\n", hp[g.second[0]].lx, hp[g.second[0]].ly,
                             g.second.size(), best);
        }
        apply();
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ck(cudaStreamSynchronize(stream_), "autotune");
        clk.mark("tune-2d");
    }

    void buildGraph(int graphSteps) {
        if (graph_) cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
        cudaGraph_t g;
        ck(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        for (int k = 0; k < graphSteps; ++k) enqueueStep();
        ck(cudaStreamEndCapture(stream_, &g), "cudaStreamEndCapture");
        ck(cudaGraphInstantiate(&graph_, g, 0), "cudaGraphInstantiate");
        cudaGraphDestroy(g);
        graphSteps_ = graphSteps;
    }

    std::vector<Sim<T>*> members_;
    int graphSteps_ = 0;
    DevMem mem_;
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
    dev::Pass<T>* dH_ = nullptr;
    dev::Pass<T>* dE_ = nullptr;
    dev::SrcJob<T>* dSrc_ = nullptr;
    dev::RecJob<T>* dRec_ = nullptr;
    dev::DftJob<T>* dDft_ = nullptr;
    dev::EmitJob<T>* dEm_ = nullptr;
    int nEm_ = 0;
    int** dSteps_ = nullptr;
    int nSteps_ = 0;
    dev::WorkMap passMap_{}, p2Map_[2]{}, lorMap_{}, odMap_{}, srcMap_{}, recMap_{}, smpMap_{}, foldMap_{}, addMap_{}, updMap_[7]{};

    void enqueueStep() {
        void* s = stream_;
        dev::launch_pass_packed<T>(dH_, passMap_, false, s);
        dev::launch_pass2d_packed<T>(dH_, p2Map_[0], false, s);
        for (Sim<T>* m : members_)
            if (m->hasTfsf()) m->launchTfsfOn(s);
        dev::launch_sources_packed<T>(dSrc_, srcMap_, s);
        dev::launch_ordip_packed<T>(dE_, odMap_, s);
        dev::launch_pass_packed<T>(dE_, passMap_, true, s);
        dev::launch_pass2d_packed<T>(dE_, p2Map_[1], true, s);
        dev::launch_lorentz_packed<T>(dE_, lorMap_, s);
        dev::launch_emitter_packed<T>(dEm_, nEm_, addMap_, updMap_, s);
        dev::launch_increment_packed(dSteps_, nSteps_, s);
        dev::launch_record_packed<T>(dRec_, recMap_, s);
        dev::launch_dft_sample_packed<T>(dDft_, smpMap_, s);
        dev::launch_dft_fold_packed<T>(dDft_, foldMap_, s);
    }
};

struct Handle {
    std::unique_ptr<SimBase> sim;
    std::string err;
    double h2d = 0, d2h = 0;
    double tPlan = 0, tUpload = 0, tFinalize = 0;  // wall seconds of create and finalize
};

double wall_seconds() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

chiml_status status_of(const std::exception& e) {
    if (dynamic_cast<const UnsupportedError*>(&e)) return CHIML_E_UNSUPPORTED;
    if (dynamic_cast<const InputError*>(&e)) return CHIML_E_INPUT;
    if (auto* c = dynamic_cast<const CudaError*>(&e))
        return c->code == cudaErrorMemoryAllocation ? CHIML_E_OOM : CHIML_E_CUDA;
    if (dynamic_cast<const std::bad_alloc*>(&e)) return CHIML_E_OOM;
    if (dynamic_cast<const NumericError*>(&e)) return CHIML_E_NUMERIC;
    if (dynamic_cast<const TimeoutError*>(&e)) return CHIML_E_TIMEOUT;
    if (dynamic_cast<const DeviceStateError*>(&e)) return CHIML_E_STATE;
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
        const double t0 = wall_seconds();
        PhaseClock clk;
        Inputs in = read_inputs_file(json_path);
        clk.mark("read-inputs");
        Plan P = build_plan(in);
        const double t1 = wall_seconds();
        std::unique_ptr<chiml_sim> s(new chiml_sim());
        if (o.precision == CHIML_PREC_FP64) s->h.sim.reset(new Sim<double>(std::move(P), o));
        else if (o.precision == CHIML_PREC_SPLIT) s->h.sim.reset(new Sim<float>(std::move(P), o));
        else throw InputError("unknown precision mode");
        s->h.tPlan = t1 - t0;
        s->h.tUpload = wall_seconds() - t1;
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

chiml_status chiml_barrier_selftest(int device, int blocks, int missing, double limit_seconds) {
    try {
        if (blocks < 1 || missing < 0) throw InputError("blocks must be positive and missing non-negative");
        // the caller's current device is put back on the way out
        struct Restore {
            int prev = 0;
            bool ok = false;
            ~Restore() {
                if (ok) cudaSetDevice(prev);
            }
        } restore;
        restore.ok = cudaGetDevice(&restore.prev) == cudaSuccess;
        ck(cudaSetDevice(device), "cudaSetDevice");
        int sms = 0, coop = 0;
        ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");
        ck(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device), "cudaDeviceGetAttribute");
        if (!coop) throw UnsupportedError("the device has no cooperative launch");
        if (blocks > sms) throw InputError("more blocks than SMs");
        const double lim = std::min(5.0, std::max(1e-3, limit_seconds));
        DevMem mem;
        unsigned int* bar = mem.alloc<unsigned int>(1);
        unsigned int* err = mem.alloc<unsigned int>(1);
        cudaStream_t s = nullptr;
        ck(cudaStreamCreate(&s), "cudaStreamCreate");
        const int st = dev::launch_barrier_selftest(blocks, missing, static_cast<unsigned long long>(lim * 1e9), bar, err, s);
        const cudaError_t se = cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
        if (st != 0) ck(static_cast<cudaError_t>(st), "cooperative launch");
        ck(se, "cudaStreamSynchronize");
        unsigned int e = 0;
        ck(cudaMemcpy(&e, err, sizeof(e), cudaMemcpyDeviceToHost), "D2H error word");
        return (e & dev::kErrTimeout) ? CHIML_E_TIMEOUT : CHIML_OK;
    } catch (const std::exception& e) {
        g_createError = e.what();
        return status_of(e);
    }
}

chiml_status chiml_sync(chiml_sim* sim) {
    if (!sim) return CHIML_E_STATE;
    try {
        sim->h.sim->checkDeviceErrors();
        return CHIML_OK;
    } catch (const std::exception& e) {
        sim->h.err = e.what();
        return status_of(e);
    }
}

chiml_status chiml_finalize(chiml_sim* sim) {
    if (!sim) return CHIML_E_STATE;
    try {
        const double t0 = wall_seconds();
        sim->h.sim->finalize();
        sim->h.tFinalize = wall_seconds() - t0;
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
    out->seconds_plan = sim->h.tPlan;
    out->seconds_upload = sim->h.tUpload;
    out->seconds_finalize = sim->h.tFinalize;
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

}  // extern "C"

struct chiml_batch {
    std::vector<chiml_sim*> members;
    int graphSteps = 0;
    int precision = CHIML_PREC_FP64;
    int device = 0;
    // packed launches of the current set of unfinished members, kept between calls
    std::unique_ptr<PackedBase> packed;
    std::vector<const void*> packedSet;
    std::map<std::pair<int, int>, int> march;  // 2-D march depth per grid shape (autotuned)
    ~chiml_batch() {
        packed.reset();  // waits for its stream before the members' memory goes
        for (chiml_sim* m : members) chiml_destroy(m);
    }
};

namespace {

// Up to maxSteps packed steps, in phases: each phase runs the unfinished members for the
// fewest steps any of them has left (or what remains of maxSteps), so members with
// different step counts each stop at their own. The packed launches are rebuilt only
// when the set of unfinished members changes.
template <typename T>
chiml_status batch_steps(chiml_batch* batch, long long maxSteps) {
    std::vector<Sim<T>*> all;
    for (chiml_sim* m : batch->members) {
        auto* s = dynamic_cast<Sim<T>*>(m->h.sim.get());
        if (!s) return CHIML_E_STATE;
        all.push_back(s);
    }
    try {
        while (maxSteps > 0) {
            std::vector<Sim<T>*> live;
            std::vector<const void*> set;
            long long n = maxSteps;
            for (Sim<T>* s : all)
                if (s->stepsLeft() > 0) {
                    live.push_back(s);
                    set.push_back(s);
                    n = std::min(n, s->stepsLeft());
                }
            if (live.empty()) break;
            if (!batch->packed || set != batch->packedSet) {
                batch->packed.reset();
                batch->packed.reset(new PackedBatch<T>(live, batch->device, batch->graphSteps, batch->march));
                batch->packedSet = set;
            }
            batch->packed->run(n, batch->graphSteps);
            for (Sim<T>* s : live) s->stepsRunElsewhere(n);
            maxSteps -= n;
        }
    } catch (const std::exception& e) {
        batch->members[0]->h.err = std::string("batched step: ") + e.what();
        return status_of(e);
    }
    return CHIML_OK;
}

}  // namespace

extern "C" {

chiml_status chiml_batch_create(const char* const* json_paths, int n, const chiml_options* opt, chiml_batch** out) {
    if (!out || !json_paths || n < 1) return CHIML_E_INPUT;
    *out = nullptr;
    std::unique_ptr<chiml_batch> b(new chiml_batch());
    // Members are created by a few host threads at once, each with its share of the
    // OpenMP threads (a small member's plan does not fill the host); the first failure in
    // member order is the one reported.
    std::vector<chiml_sim*> made(static_cast<std::size_t>(n), nullptr);
    std::vector<chiml_status> made_st(static_cast<std::size_t>(n), CHIML_OK);
    std::vector<std::string> why(static_cast<std::size_t>(n));
    std::atomic<int> next{0};
    const int workers = std::min(n, 8);
    const int hostThreads = omp_get_max_threads();
    auto createOne = [&](int i) {
        // without an output directory, a member writes beside its own input file
        chiml_options o = opt ? *opt : chiml_options{CHIML_PREC_FP64, 0, 0, nullptr};
        o.steps_per_graph = 0;  // members step through the batch's packed graph, not their own
        std::string dir;
        if (!o.out_dir && json_paths[i]) {
            dir = json_paths[i];
            const size_t slash = dir.find_last_of('/');
            dir = slash == std::string::npos ? std::string(".") : dir.substr(0, slash + 1);
            o.out_dir = dir.c_str();
        }
        made_st[static_cast<std::size_t>(i)] = chiml_create(json_paths[i], &o, &made[static_cast<std::size_t>(i)]);
        if (made_st[static_cast<std::size_t>(i)] != CHIML_OK) why[static_cast<std::size_t>(i)] = g_createError;
    };
    {
        std::vector<std::thread> pool;
        for (int w = 0; w < workers; ++w)
            pool.emplace_back([&] {
                omp_set_num_threads(std::max(1, hostThreads / workers));
                for (int i = next++; i < n; i = next++) createOne(i);
            });
        for (auto& t : pool) t.join();
    }
    for (int i = 0; i < n; ++i)
        if (made_st[static_cast<std::size_t>(i)] != CHIML_OK) {
            for (chiml_sim* m : made) chiml_destroy(m);
            g_createError = std::string("batch member ") + std::to_string(i) + " (" + (json_paths[i] ? json_paths[i] : "null") +
                            "): " + why[static_cast<std::size_t>(i)];
            return made_st[static_cast<std::size_t>(i)];
        }
    for (chiml_sim* m : made) b->members.push_back(m);
    b->graphSteps = opt ? opt->steps_per_graph : 0;
    b->precision = opt ? opt->precision : CHIML_PREC_FP64;
    b->device = opt ? opt->device : 0;
    *out = b.release();
    return CHIML_OK;
}

chiml_status chiml_batch_step(chiml_batch* batch, int64_t nsteps) {
    if (!batch) return CHIML_E_STATE;
    if (nsteps <= 0) return CHIML_OK;
    const chiml_status st =
        batch->precision == CHIML_PREC_SPLIT ? batch_steps<float>(batch, nsteps) : batch_steps<double>(batch, nsteps);
    if (st != CHIML_OK) return st;
    for (chiml_sim* m : batch->members) {
        try {
            m->h.sim->checkDeviceErrors();
        } catch (const std::exception& e) {
            m->h.err = e.what();
            return status_of(e);
        }
    }
    return CHIML_OK;
}

chiml_status chiml_batch_run(chiml_batch* batch) {
    if (!batch) return CHIML_E_STATE;
    long long most = 0;
    for (chiml_sim* m : batch->members) {
        chiml_stats st;
        m->h.sim->fillStats(&st);
        most = std::max<long long>(most, static_cast<long long>(st.steps_total) - st.steps_done);
    }
    return chiml_batch_step(batch, most);
}

chiml_status chiml_batch_finalize(chiml_batch* batch) {
    if (!batch) return CHIML_E_STATE;
    for (chiml_sim* m : batch->members) {
        const chiml_status s = chiml_finalize(m);
        if (s != CHIML_OK) return s;
    }
    return CHIML_OK;
}

chiml_sim* chiml_batch_member(chiml_batch* batch, int i) {
    if (!batch || i < 0 || i >= static_cast<int>(batch->members.size())) return nullptr;
    return batch->members[i];
}

void chiml_batch_destroy(chiml_batch* batch) { delete batch; }

chiml_status chiml_get_box_noalloc(chiml_sim* sim, int comp, const int32_t box[6], double* out) {
    if (!sim || !box || !out) return CHIML_E_STATE;
    const int b[6] = {box[0], box[1], box[2], box[3], box[4], box[5]};
    std::string why;
    const chiml_status st = sim->h.sim->getBoxNoAlloc(comp, b, out, why);
    if (st != CHIML_OK) sim->h.err = why;
    return st;
}

void* chiml_stream(chiml_sim* sim) { return sim ? static_cast<void*>(sim->h.sim->stream()) : nullptr; }

chiml_status chiml_profile_steps(chiml_sim* sim, int nsteps, double* ms_out, int max_slots, int* nslots) {
    if (!sim || !ms_out || !nslots) return CHIML_E_STATE;
    try {
        *nslots = sim->h.sim->profile(nsteps, ms_out, max_slots);
        return CHIML_OK;
    } catch (const std::exception& e) {
        sim->h.err = e.what();
        return status_of(e);
    }
}

}  // extern "C"
