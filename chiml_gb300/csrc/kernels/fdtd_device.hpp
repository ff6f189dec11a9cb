// Device-side descriptors of the time-step kernels, shared by the kernel
// translation unit (fdtd_kernels.cu) and the host engine (engine.cpp).
// Plain structs of device pointers and sizes; passed to kernels by value.
#pragma once

#include <cstdint>

namespace chiml {
namespace dev {

// Rows each warp of the 2-D pass form marches along y unless the batch autotuner chose
// another depth for the member's grid shape.
constexpr int kP2CYDefault = 16;

constexpr int kMaxPoles = 8;

// One cell class of a component (the compressed update lists, see plan.hpp).
template <typename T>
struct Class {
    T cint[2];       // interior curl coefficients of terms J, K
    T epsInv;        // 1 / eps_inf      (D -> E)
    T negEpsInv;     // -1 / eps_inf     (D -> E)
    int32_t obj;     // object whose Lorentz poles apply
    uint8_t toD;     // curl and CPML terms update D
    uint8_t lor;     // Lorentz P update before, D -> E after
    uint8_t nplain[2];
    uint8_t kflag[2];
    uint8_t npsi[2];
    uint8_t psiUpd[2];
    uint8_t ordip;   // oriented-dipole D -> E: P averaged over two cell-centred points
    uint8_t pad;
    T odCoef;        // -0.5 / eps_inf (orDipDtoU)
};

// The same class in the shape the interior form's arithmetic uses: per term
// the folded interior coefficient and the psi coefficient, plus flag bits. The
// first 16 bytes (coefficients and flags) are all a cell outside the CPML
// slabs needs.
template <typename T>
struct alignas(16) FastClass {
    T coef[2];     // cint + nplain * db
    uint32_t flags;
    uint32_t obj;  // object whose Lorentz poles apply (kFcLor)
    T psiCoef[2];  // npsi * dbpsi
    T epsInv;      // 1 / eps_inf of the D -> E cells (kFcDtoE, kFcLor, kFcOrDip)
};
constexpr uint32_t kFcPsi0 = 1u;     // term J updates psi
constexpr uint32_t kFcPsi1 = 2u;     // term K updates psi
constexpr uint32_t kFcLor = 4u;      // Lorentz ADE and D -> E (E pass)
constexpr uint32_t kFcToD = 8u;      // the update goes to D
constexpr uint32_t kFcWrite = 16u;   // the class changes the field
constexpr uint32_t kFcSlab0 = 32u;   // term J needs the slab (profile or psi)
constexpr uint32_t kFcSlab1 = 64u;   // term K needs the slab
constexpr uint32_t kFcKp0 = 128u;    // term J adds its normal-slab profile kprof
constexpr uint32_t kFcKp1 = 256u;    // term K adds its normal-slab profile kprof
constexpr uint32_t kFcOrDip = 512u;  // oriented-dipole D -> E (E pass)
constexpr uint32_t kFcDtoE = 1024u;  // D -> E of a cell whose object has no poles: E = D / eps_inf (E pass)

// Form of the Lorentz / Drude recursion (UpdateLorPol, UTIL/FDTD_up_eq.cpp:425-448).
// FP64 keeps the reference's form, P+ = alpha P + xi P- + gamma E, with Pprev holding P-.
// FP32 uses the increment form: Pprev holds J = P - P-, and
//   J+ = b J + a P + gamma E,  P+ = P + J+,  a = alpha + xi - 1 = -(w dt)^2 / (1 + g dt),  b = -xi,
// which is the same recursion without its cancellation: alpha ~ 2 and xi ~ -1, so alpha P
// + xi P- subtracts two nearly equal values, and in FP32 the rounding of that difference
// accumulates over the run (a Drude pole integrates it twice).
template <typename T>
constexpr bool kIncrementPoles = sizeof(T) == 4;

// The FP32 interior kernels update the dispersive (Lorentz, oriented-dipole) cells
// themselves; the FP64 ones, whose register budget the extra path would exceed, leave
// them to the list kernel (measured: FP32 E pass 0.25 ms inline vs 0.30 ms with the list
// at 256^3 with 16 uniaxial ellipsoids and the metal sphere).
template <typename T>
constexpr bool kInlineDispersive = sizeof(T) == 4;

template <typename T>
struct Comp {
    T* U;                  // field component
    T* D;                  // D component (E components of dispersive runs)
    const uint8_t* code;   // per-cell class code
    const Class<T>* cls;   // class table
    const FastClass<T>* fcls;  // the same table for the interior form
    int ncls;              // entries in cls
    int present;
    int nPoles;
    T* P[kMaxPoles];
    T* Pprev[kMaxPoles];   // P- (FP64 form) or J = P - P- (increment form)
    // neighbour terms J (uses grid_j) and K (uses grid_k)
    int tpresent[2];
    int axis[2];
    int hasPsi[2];
    long long off[2];
    const T* G[2];
    T* psi[2];
    const T* kprof[2];
    const T* b[2];
    const T* cpsi[2];
    T db[2];
    T dbpsi[2];
    // Coordinates along each term's axis outside which no cell uses that term's
    // CPML profile or psi: the slab is a < slabLo or a >= slabHi.
    int slabLo[2];
    int slabHi[2];
};

// Oriented-dipole polarisations (UpdateLorPolOrDip): one entry per cell-centred grid
// point inside an object with oriented-dipole poles. P and P_prev are full-grid arrays
// per component and pole; the dipole directions are stored per entry, pole and axis.
template <typename T>
struct OrDipDev {
    long long n;
    int nPoles;
    const long long* cell;
    const int* obj;
    const T* dip;                  // [(pole * 3 + axis) * n + entry]
    T* P[3][kMaxPoles];
    T* Pprev[3][kMaxPoles];        // P- (FP64 form) or J = P - P- (increment form)
    long long off[3];              // grid index step along x, y, z
};

template <typename T>
struct Pass {
    Comp<T> c[3];
    int lx, ly, lz;
    long long pitch;        // device row length: cell (x, y, z) is x + pitch (z + lz y), pitch >= lx
    const int* poleStart;   // per object: first pole in the coefficient arrays
    const int* poleCount;   // per object: number of poles
    const T* poleA;         // per pole: alpha (FP64 form) or a (increment form, kIncrementPoles)
    const T* poleB;         // per pole: xi (FP64 form) or b = -xi (increment form)
    const T* gamma;
    int nObj;
    unsigned int* err;      // device error word (kErr* bits); the kernel skips the cell instead of faulting
    // 3-D interior form usable: every halo cell has code 0, term j of component c
    // differentiates along (c+2)%3 / (c+1)%3 with offsets -1 (E) / +1 (H) cells.
    int interior3d;
    int interior2d;         // the same conditions on a 2-D grid (lz == 1; the z terms absent)
    int march;              // rows each warp marches in the packed 2-D form (0: kP2CYDefault)
    int index64;            // grid too large for 32-bit cell indices
    OrDipDev<T> od;         // oriented-dipole polarisations (E pass)
    // dispersive cells of the E pass, run by their own kernel in the interior form
    long long nLor;
    const int* lorComp;
    const long long* lorCell;
    // soft sources that the 2-D E pass adds itself (nSrcIn entries, at most kInlineMaxSrc;
    // 0: the source kernel runs): component, device cell, source id, the source table's
    // values [id * srcSteps + step] and the step counter
    int nSrcIn;
    const int* srcComp;
    const long long* srcCell;
    const int* srcId;
    const double* srcValue;
    int srcSteps;
    const int* step;
};
constexpr int kInlineMaxSrc = 64;

constexpr unsigned int kErrClassCode = 1u;   // a cell code outside its class table
constexpr unsigned int kErrPoleCount = 2u;   // a class asks for more poles than its component stores
constexpr unsigned int kErrSlab = 4u;        // a class uses a CPML term outside its term's slab bounds
constexpr unsigned int kErrNumeric = 8u;     // a sampled field value (detector or DFT point) is NaN or Inf
constexpr unsigned int kErrTimeout = 16u;    // a grid barrier of the persistent 2-D kernel gave up waiting

template <typename T>
struct Fields {
    T* f[9];  // Ex,Ey,Ez,Hx,Hy,Hz,Dx,Dy,Dz (null where absent)
};

struct SourceTable {
    int n;                    // source cells
    const int* comp;          // per cell: component
    const long long* cell;    // per cell: grid index
    const int* src;           // per cell: source id
    const double* value;      // [src * nSteps + step]
    int nSteps;
};

struct RecordTable {
    int n;                      // gathered values per event, summed over detectors
    const int* det;             // per entry: detector id
    const int* comp;            // per entry: component (0..8)
    const long long* cell;      // per entry: grid index or -1
    const long long* outIndex;  // per entry: index inside the detector event
    const int* timeInt;         // per detector
    const long long* nvals;     // per detector: values per event
    const long long* recBase;   // per detector: offset of event 0 in rec
    const int* nEvents;         // per detector
    double* rec;
    unsigned int* err;          // error word: kErrNumeric for a value that is not finite
};

// Time-blocked DFT of one flux region. Every sampled step gathers the field
// value of each accumulated point into a ring of K samples; every point folds the
// ring into the FP64 accumulators once per K samples (the point tiles in groups
// whose folds are staggered, one group every 4 samples):
//   re[pt][f] += sum_k cos(w_f t_k) F_k[pt],  im[pt][f] += sum_k -sin(w_f t_k) F_k[pt]
// which is the per-step update of parallelStorageFreqDTCReal::fieldIn
// (DTC/parallelStorageFreqDTC.cpp:21-30) regrouped over K steps.
// The split form's DFT accumulators are float-float pairs (48-bit significands): the fold
// adds its FP32 partial sums with FP32 TwoSum arithmetic instead of FP64 adds, which the
// GB300's FP64 rate (1/64 of FP32) made a third of the fold's issue time.
template <typename T>
constexpr bool kFloatFloatAcc = sizeof(T) == 4;

// The DFT fold is staggered: one group of point tiles folds every kFoldStagger samples
// (fdtd_kernels.cu, foldGroupNow).
constexpr int kFoldStagger = 4;

template <typename T>
struct DftTable {
    long long npts;
    int nfreq;
    int timeInt;
    int K;                      // samples per block
    int nSamples;               // samples a full run takes (phasor rows)
    int nfreqPad;               // frequencies per phasor row, a multiple of 32 (zero-filled past nfreq)
    long long stride;           // ring row pitch: points rounded up to a multiple of 128
    const int* comp;            // per point
    const int* cell;            // per point (grid index)
    const T* phasor;            // [(sample * 2 + {0: cos, 1: -sin}) * nfreqPad + f]
    T* ring;                    // [K][stride]
    // [pt * nfreq + f], 8 bytes per value: FP64 in the FP64 form; in the split form a
    // float-float pair (hi, lo) as a float2 (kFloatFloatAcc), summed on the FP32 pipe
    double* re;
    double* im;
    unsigned int* err;          // error word: kErrNumeric for a sample that is not finite
};

// Packed launches of the batched sweep: one launch runs one kind of work for many
// independent simulations (members). The job array holds each member's descriptor
// in device memory; work[b] = {job, block of that job} for block b of the launch,
// each job taking the blocks its own launch would have.
template <typename T>
struct SrcJob {
    SourceTable s;
    Fields<T> f;
    const int* step;
};
template <typename T>
struct RecJob {
    RecordTable r;
    Fields<T> f;
    const int* step;
};
template <typename T>
struct DftJob {
    DftTable<T> d;
    Fields<T> f;
    const int* step;
};
struct WorkMap {
    const int2* work;  // [blocks]
    int blocks;
};

// The end of a step in one launch: the detector records and the DFT samples of the
// step after the counter's increment, then the increment itself, done by the block that
// finishes last (a ticket counter, no waiting). Blocks [0, recBlocks) record, then the
// DFT tables' sample blocks follow in order, table q from dftStart[q].
template <typename T>
struct StepTail {
    RecordTable rec;
    int recBlocks;
    int nDft;
    const DftTable<T>* dft;  // [nDft] (device)
    const int* dftStart;     // [nDft + 1] block offsets after the record blocks (device)
    Fields<T> f;
    int* step;
    unsigned int* ticket;    // zero between launches
    int blocks;              // recBlocks + the sample blocks of every table (at least 1)
};

// Persistent form of a small 2-D grid: one cooperative launch runs several whole steps
// (H pass, E pass with the soft sources, detector records and DFT samples), the blocks
// meeting at a grid barrier between the passes. Eligible grids: the 2-D interior form,
// no TFSF, emitters or oriented dipoles, dispersive cells only where the pass updates them
// inline, soft sources only on E cells that the pass writes plainly (at most
// kPersistMaxSrc entries), DFT tables sampled every step (so that a group fold falls at
// the end of every fourth step, where the launch ends and the fold kernel runs).
constexpr int kPersistMaxSrc = kInlineMaxSrc;

template <typename T>
struct Persist2d {
    Pass<T> h, e;
    SourceTable src;         // E-component entries only
    RecordTable rec;
    const DftTable<T>* dft;  // [nDft] (device)
    int nDft;
    long long dftPoints;     // points over every table
    Fields<T> f;
    int* step;               // the step counter, written at the end of the launch
    unsigned int* bar;       // barrier arrivals, zero at launch
    unsigned long long limitNs;  // longest wait at a barrier
};

// Launchers (fdtd_kernels.cu). All run on the given stream.
template <typename T>
void launch_pass(const Pass<T>& p, bool ePass, void* stream);
template <typename T>
void launch_sources(const SourceTable& s, const Fields<T>& f, const int* step, void* stream);
template <typename T>
void launch_record(const RecordTable& r, const Fields<T>& f, const int* step, void* stream);
template <typename T>
void launch_dft_sample(const DftTable<T>& d, const Fields<T>& f, const int* step, void* stream);
// Folds the ring into the accumulators for the group of point tiles whose turn comes
// with the current sample (one group every 4 samples; nothing at the other steps).
template <typename T>
void launch_dft_fold(const DftTable<T>& d, const int* step, void* stream);
// End of a run: folds every group's pending samples, `samples` being the samples taken.
template <typename T>
void launch_dft_flush(const DftTable<T>& d, int samples, void* stream);
void launch_increment(int* step, void* stream);
template <typename T>
void launch_step_tail(const StepTail<T>& t, void* stream);

// Blocks each job of a packed launch takes (the grid of its own launch).
template <typename T>
long long pass_blocks(const Pass<T>& p);  // generic form
template <typename T>
long long pass2d_blocks_per_comp(const Pass<T>& p);  // 2-D form, per component
long long lorentz_blocks(long long n);
long long ordip_blocks(long long n);
int sources_blocks(int n);
int record_blocks(int n);
long long dft_sample_blocks(long long npts);
long long dft_fold_blocks(long long npts, int nfreq);

template <typename T>
void launch_pass_packed(const Pass<T>* jobs, WorkMap m, bool ePass, void* stream);
template <typename T>
void launch_pass2d_packed(const Pass<T>* jobs, WorkMap m, bool ePass, void* stream);
template <typename T>
void launch_lorentz_packed(const Pass<T>* jobs, WorkMap m, void* stream);
template <typename T>
void launch_ordip_packed(const Pass<T>* jobs, WorkMap m, void* stream);
template <typename T>
void launch_sources_packed(const SrcJob<T>* jobs, WorkMap m, void* stream);
template <typename T>
void launch_record_packed(const RecJob<T>* jobs, WorkMap m, void* stream);
template <typename T>
void launch_dft_sample_packed(const DftJob<T>* jobs, WorkMap m, void* stream);
template <typename T>
void launch_dft_fold_packed(const DftJob<T>* jobs, WorkMap m, void* stream);
void launch_increment_packed(int* const* steps, int n, void* stream);

// Blocks the persistent launch uses (resident on every SM at once), 0 when none fit.
template <typename T>
int persist2d_blocks(const Pass<T>& h, const Pass<T>& e, int device);
// nsteps steps from step0 in one cooperative launch of `blocks` blocks (barrier counter
// zeroed on the stream first). Returns the CUDA status of the launch.
template <typename T>
int launch_persist2d(const Persist2d<T>& a, int blocks, int step0, int nsteps, void* stream);
// The grid barrier on its own: `blocks` cooperative blocks wait for blocks + missing
// arrivals with the given limit; err receives kErrTimeout when the wait gives up.
int launch_barrier_selftest(int blocks, int missing, unsigned long long limitNs, unsigned int* bar, unsigned int* err,
                            void* stream);

}  // namespace dev
}  // namespace chiml
