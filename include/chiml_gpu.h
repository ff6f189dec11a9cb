/* chiml_gpu.h - C ABI of the GB300 time-step engine for chiML inputs.
 *
 * The boundary replaces the C++ class interface that chiML's driver uses:
 *   parallelFDTDFieldReal(parallelProgramInputs&, mpiInterface)  FDTD_MANAGER/parallelFDTDField.hpp:1793
 *   void step()                                                   FDTD_MANAGER/parallelFDTDField.hpp:1228
 *   final outputs (flux, detectors)                               src/main.cpp:67-118
 * A caller mirrors main.cpp: create from the JSON input, step ceil(tLim/dt)
 * times (main.cpp:54), finalize (writes the same files), destroy.
 *
 * Errors are integer status codes; no C++ exception crosses this boundary.
 * One handle owns one CUDA stream and all of its device memory; handles are
 * independent and each must be used from one host thread at a time.
 */
#ifndef CHIML_GPU_H
#define CHIML_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct chiml_sim chiml_sim;

typedef enum chiml_status {
    CHIML_OK = 0,
    CHIML_E_INPUT = 1,       /* malformed or inconsistent input (the reference throws std::logic_error) */
    CHIML_E_UNSUPPORTED = 2, /* a feature outside this engine (magnetic/chiral media, PBC, ...) */
    CHIML_E_CUDA = 3,        /* a CUDA runtime error */
    CHIML_E_OOM = 4,         /* device memory exhausted */
    CHIML_E_NUMERIC = 5,     /* a detector or flux/DFT point sampled a NaN or Inf field value */
    CHIML_E_TIMEOUT = 6,     /* a grid barrier of the persistent 2-D step gave up waiting */
    CHIML_E_STATE = 7        /* call out of order (e.g. step after finalize), or a device-side
                                bounds check of the plan failed */
} chiml_status;

typedef enum chiml_precision {
    CHIML_PREC_FP64 = 0,  /* every field, coefficient and accumulator in FP64 (the parity form) */
    CHIML_PREC_SPLIT = 1  /* fields, CPML and polarisations in FP32; DFT accumulators and emitter density matrices in FP64 */
} chiml_precision;

typedef struct chiml_options {
    int precision;        /* chiml_precision */
    int device;           /* CUDA device ordinal */
    int steps_per_graph;  /* steps captured per CUDA graph; 0 = launch kernels without graphs */
    const char* out_dir;  /* directory that relative output names resolve against; NULL = current directory */
} chiml_options;

typedef struct chiml_stats {
    int64_t cells;             /* grid cells including the halo */
    int64_t cells_physical;    /* nx * ny * nz */
    int32_t nx, ny, nz;
    int32_t steps_total;       /* ceil(tLim / dt) */
    int32_t steps_done;
    int32_t precision;
    double bytes_per_cell_update;  /* algorithmic HBM bytes per physical cell per step */
    double device_bytes;           /* device memory held by the handle */
    int32_t kernels_per_step;      /* kernel launches per step (of the launch-per-kernel form) */
    int32_t persistent;            /* 1: chiml_step runs the persistent 2-D form (cooperative launches
                                      of several steps; see chiml_barrier_selftest) */
    double bytes_h_pass;           /* algorithmic HBM bytes of one H-pass launch */
    double bytes_e_pass;           /* algorithmic HBM bytes of one E-pass launch */
    double bytes_dft;              /* algorithmic HBM bytes of the DFT launches of one sampled step */
    double h2d_bytes;              /* bytes copied host to device so far */
    double d2h_bytes;              /* bytes copied device to host so far */
    int32_t n_flux_regions;        /* DFT tables: flux regions, then frequency-domain detectors (two profile slots each) */
    int32_t n_emitters;            /* emitter objects (one profile slot each) */
    int32_t n_tfsf;                /* TFSF surfaces (one profile slot each) */
    int32_t reserved2;
    double seconds_plan;           /* chiml_create: reading the input and building the plan (host) */
    double seconds_upload;         /* chiml_create: device allocation and upload */
    double seconds_finalize;       /* chiml_finalize: flux integration, downloads and file writes */
} chiml_stats;

/* Reads the JSON input (chiML schema), builds the update plan and uploads it. */
chiml_status chiml_create(const char* json_path, const chiml_options* opt, chiml_sim** out);

/* Advances nsteps time steps (clamped to the steps left). Asynchronous with
 * respect to the host only inside the call: it returns after the work is queued
 * and checked for launch errors. */
chiml_status chiml_step(chiml_sim* sim, int64_t nsteps);

/* Waits for queued work. */
chiml_status chiml_sync(chiml_sim* sim);

/* Copies detector records, DFT accumulators and emitter outputs to the host and
 * writes the detector (time and frequency domain), flux, emitter polarisation and
 * population files in chiML's formats. */
chiml_status chiml_finalize(chiml_sim* sim);

void chiml_destroy(chiml_sim* sim);

/* Last error message of the handle; with sim == NULL, of the calling thread's last chiml_create. */
const char* chiml_last_error(const chiml_sim* sim);

chiml_status chiml_query(const chiml_sim* sim, chiml_stats* out);

/* Copies one field to host memory as FP64, in chiML's local grid layout
 * (x fastest, then z, then y, with a one-cell halo). comp: 0..2 Ex..Ez,
 * 3..5 Hx..Hz, 6..8 Dx..Dz. out holds stats.cells doubles. */
chiml_status chiml_get_field(chiml_sim* sim, int comp, double* out);

/* Device stream of the handle (a cudaStream_t), for callers that time kernels. */
void* chiml_stream(chiml_sim* sim);

/* Advances nsteps steps without graphs, timing every kernel launch with CUDA
 * events on the handle's stream. ms_out[k] receives the summed milliseconds of
 * kernel slot k: 0 H pass, 1 sources, 2 E pass, 3 step counter, 4 detector
 * records, 5 + 2q DFT sample gather and 6 + 2q DFT fold of DFT table q (flux
 * regions, then frequency-domain detectors), then
 * 5 + 2 * n_flux_regions + e the emitter step of emitter object e, then
 * 5 + 2 * n_flux_regions + n_emitters + k the step of TFSF surface k.
 * chiml_step runs the counter, the records and every table's sample gather as one
 * launch; here they run as separate launches so that each has its own time.
 * *nslots receives the number of slots written (at most max_slots). */
chiml_status chiml_profile_steps(chiml_sim* sim, int nsteps, double* ms_out, int max_slots, int* nslots);

/* A batch of independent simulations stepped together (a parameter sweep), of
 * uneven sizes: each member keeps its own plan and device state, and each kind of
 * per-step work of all members runs as one packed launch, driven by a table that maps
 * every block to a member and a block of that member's own launch. The reference runs
 * such sweeps as separate processes. */
typedef struct chiml_batch chiml_batch;

/* Creates one member per input file, all with the same options, except that with
 * opt->out_dir NULL each member's relative output names resolve against the
 * directory of its own input file (one directory per sweep point, as separate
 * reference runs would use). On failure no batch is returned and
 * chiml_last_error(NULL) names the failing input; after a failed run or finalize,
 * chiml_last_error of the failing member (chiml_batch_member) holds the reason. */
chiml_status chiml_batch_create(const char* const* json_paths, int n, const chiml_options* opt, chiml_batch** out);

/* Advances every unfinished member by nsteps steps (each stops at its own last
 * step, ceil(tLim/dt)) and waits: per step, one packed launch of each kind of work
 * covers all members, the steps captured as CUDA graphs of opt->steps_per_graph steps. */
chiml_status chiml_batch_step(chiml_batch* batch, int64_t nsteps);

/* Advances every member to its last step and waits. */
chiml_status chiml_batch_run(chiml_batch* batch);

/* Writes every member's output files (as chiml_finalize). */
chiml_status chiml_batch_finalize(chiml_batch* batch);

/* Member i of the batch (owned by the batch), or NULL when i is out of range. */
chiml_sim* chiml_batch_member(chiml_batch* batch, int i);

void chiml_batch_destroy(chiml_batch* batch);

/* Largest box, in cells, that chiml_get_box_noalloc reads in one call. */
#define CHIML_BOX_NOALLOC_MAX_CELLS 1048576

/* Copies the box {x0, y0, z0, nx, ny, nz} of one field (local grid, halo
 * included, as chiml_get_field) to host memory as FP64, x fastest, then z, then
 * y; out holds nx*ny*nz doubles. No counterpart in the reference: chiML has no
 * device memory to read back.
 *
 * It allocates nothing, on the device or through any library: it is for
 * callers that cannot allocate device memory when they read a field, such as a
 * run that fills HBM and has no room for a temporary, or a host application
 * whose own memory pool must not see cudaMalloc/cudaFree (which also stall the
 * device) from a library. The values pass through one fixed device array of
 * CHIML_BOX_NOALLOC_MAX_CELLS doubles (8 MiB) per device; a larger box, or one
 * outside the grid, returns CHIML_E_INPUT with the reason in chiml_last_error.
 * The array is placed on a device, and its address looked up, when the first
 * handle on that device is created (chiml_create, before the handle's own
 * uploads), so a read places nothing and loads no code. Every call shares the
 * array and leaves its values there; each call writes every value it returns
 * before copying, so nothing needs clearing. The call waits for its copy, and
 * leaves the calling thread's current device as it found it. Calls that
 * overlap on the GPU (handles of one device used from several host threads at
 * once) race on the array. */
chiml_status chiml_get_box_noalloc(chiml_sim* sim, int comp, const int32_t box[6], double* out);

/* Small 2-D grids can step in a persistent form (opt-in: CHIML_PERSIST2D=1 in the
 * environment at chiml_create): one cooperative launch runs several steps, its blocks
 * meeting at grid barriers whose waits are limited to one second; a wait that gives up
 * ends the launch and the next chiml_sync / chiml_finalize returns CHIML_E_TIMEOUT. This diagnostic runs that barrier alone: `blocks` cooperative blocks
 * of 32 threads on `device` (at most one per SM) wait for blocks + missing arrivals, each
 * wait limited to limit_seconds (clamped to 1 ms .. 5 s). CHIML_OK when every block
 * arrived; CHIML_E_TIMEOUT when the wait gave up (missing > 0). The device stays usable
 * either way; chiml_last_error(NULL) holds the reason of any other failure. */
chiml_status chiml_barrier_selftest(int device, int blocks, int missing, double limit_seconds);

#ifdef __cplusplus
}
#endif

#endif /* CHIML_GPU_H */
