/*
 * pic_gb300.h -- C ABI of the GB300-native 2D electrostatic PIC deposition path.
 *
 * This ABI is the drop-in boundary for the hot path of ehocine/pic-deposition.
 * Each entry point names the reference interface it replaces (file:line in that
 * project). The reference's own GPU entry points are
 *   void pic::depositChargeCudaSoA(const ParticlesSoA&, FieldGrid&, const DepositionConfig&)
 *   (src/deposition/cuda/deposition_cuda.hpp:11-12, deposition_cuda.cu:288-337),
 * which copy host arrays to the device on every call; here particle and grid
 * state stays resident in a context between calls and host copies happen only
 * in the upload/download calls and in calls given a non-NULL host pointer.
 *
 * Conventions
 *  - Every function returns an int status: PIC_OK (0) or a negative PIC_ERR_*.
 *    No C++ exception crosses the ABI. pic_gpu_last_error() gives the message of
 *    the calling thread's last failure.
 *  - A context is bound to one CUDA device and one stream; it is not thread-safe
 *    (the caller serialises calls), like the reference's single-threaded API.
 *  - Host pointers are plain arrays; lengths are element counts. Device state is
 *    opaque.
 *  - Particles are stored on the device as FP32 offsets inside their cell plus a
 *    u32 cell key iy*Nx+ix; the key is computed from the FP64 host position with
 *    the reference's Domain::cellCoords (src/pic/domain.hpp:34-43), so keys are
 *    bit-identical to pic::particleCellIndex (src/sorting/cell_sort.cpp:8-13).
 *  - Charge is deposited in fixed point. The resident charge is stored as
 *    qn = q/max|q| (FP32) and a particle carries A = rint(qn*2^24) units; each
 *    stencil value qn*2^24*w is rounded to the nearest integer, the node of
 *    largest weight takes the remainder so the particle deposits exactly A
 *    units, and the grid sums in int64. rho is therefore independent of
 *    summation order, bit-identical run to run, and conserves total charge
 *    exactly for a uniform |q|. One unit of the int64 grid is
 *    max|q| * inv_vol * 2^-24 (returned by pic_gpu_get_rho_fixed).
 */
#ifndef PIC_GB300_H
#define PIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PIC_OK 0
#define PIC_ERR_ARG (-1)         /* bad argument (NULL, size, scheme, ...)              */
#define PIC_ERR_CUDA (-2)        /* a CUDA runtime / cuFFT call failed                  */
#define PIC_ERR_NOMEM (-3)       /* device or pinned allocation failed                  */
#define PIC_ERR_STATE (-4)       /* call out of order (e.g. deposit before upload)      */
#define PIC_ERR_OVERFLOW (-5)    /* fixed-point headroom would be exceeded              */
#define PIC_ERR_COURANT (-6)     /* Esirkepov current needs |v|*dt < cell size          */
#define PIC_ERR_TIMEOUT (-7)     /* a bounded device-side wait gave up                  */
#define PIC_ERR_UNSUPPORTED (-8) /* valid request the library does not support         */
#define PIC_ERR_DEVICE (-9)      /* a kernel reported bad data (non-finite position ...) */

/* ---- schemes: values of pic::DepositionScheme (src/deposition/deposition.hpp:11) ---- */
#define PIC_SCHEME_NGP 0
#define PIC_SCHEME_CIC 1
#define PIC_SCHEME_TSC 2
#define PIC_SCHEME_ESIRKEPOV 3 /* the reference's trajectory-averaged rho (ngp.cpp:13-84) */

/* ---- deposit ordering modes ---- */
/* PIC_ORDER_AUTO: the tiled kernel when cell-sorted; between sorts (particles
 * pushed since) the tiled kernel that also finds the particles that left their
 * cell, until one deposit finds more than 40 % of them moved, then the
 * run-aggregating kernel until the next sort (chosen on the device); otherwise
 * the run-aggregating kernel. Every choice gives the same grid bit for bit. */
#define PIC_ORDER_AUTO 0
#define PIC_ORDER_SORTED 1   /* tiled kernel; PIC_ERR_STATE unless sorted (or only pushed since) */
#define PIC_ORDER_UNSORTED 2 /* run-aggregating kernel (any order; fast when nearly sorted)      */
#define PIC_ORDER_ATOMIC 3   /* one thread per particle, one int64 atomic per stencil node       */

/* Mirrors pic::Domain (src/pic/domain.hpp:7-44): periodic box [0,Lx)x[0,Ly),
 * Nx x Ny cells, dx = Lx/Nx, dy = Ly/Ny. */
typedef struct pic_domain {
    double Lx;
    double Ly;
    int32_t Nx;
    int32_t Ny;
} pic_domain;

typedef struct pic_ctx pic_ctx;

/* Mirrors pic::Diagnostics (src/pic/diagnostics.hpp:8-15), FP64 sums on the GPU. */
typedef struct pic_diag {
    double charge_error;
    double total_charge;
    double integrated_rho;
    double kinetic_energy;
    double field_energy;
    double total_energy;
} pic_diag;

/* ---- context ---- */

/* Creates a context on `device` for up to `capacity` particles. Replaces the
 * reference's static never-freed device pool (deposition_cuda.cu:243-273). */
int pic_gpu_create(const pic_domain* domain, size_t capacity, int device, pic_ctx** out);
int pic_gpu_destroy(pic_ctx* ctx);
const char* pic_gpu_last_error(void);
int pic_gpu_synchronize(pic_ctx* ctx);
/* Number of kernels this library launched on the context since creation. */
int pic_gpu_launch_count(pic_ctx* ctx, long long* out);
/* The context's CUDA stream (cudaStream_t), for callers that time on it. */
int pic_gpu_get_stream(pic_ctx* ctx, void** stream_out);
/* CUDA-event timing of the library's dominant kernels on the context stream.
 * While enabled, every launch of a named kernel ("deposit", "sort", ...) is
 * bracketed by two events; pic_gpu_profile_read synchronises, returns the summed
 * milliseconds and launch count for `kernel` and forgets those records. The
 * reference times whole calls with std::chrono (deposition.cpp:257-310). */
int pic_gpu_profile_enable(pic_ctx* ctx, int enable);
int pic_gpu_profile_read(pic_ctx* ctx, const char* kernel, double* total_ms, long long* launches);

/* Page-locked host buffers for fast uploads/downloads (cudaHostAlloc / cudaFreeHost). */
int pic_gpu_host_alloc(size_t bytes, void** out);
int pic_gpu_host_free(void* p);

/* ---- particles ---- */

/* Uploads FP64 SoA particles (layout of pic::ParticlesSoA, src/pic/particles.hpp:45-83)
 * and converts them to the device layout. vx, vy, m may be NULL (0, 0, 1).
 * Replaces the per-call H2D copies of deposition_cuda.cu:296-303. Marks the
 * particles unsorted. */
int pic_gpu_upload_particles(pic_ctx* ctx, const double* x, const double* y, const double* vx, const double* vy,
                             const double* q, const double* m, size_t n);
/* Generates particles on the device (no counterpart in the reference; for synthetic
 * workloads too large to build on the host): x from the density
 * 1 + amplitude*cos(2*pi*mode*x/Lx) (mode 0: uniform), y uniform, Maxwellian
 * velocities of thermal speed vth per component, plus +v0 in x for the first
 * half and -v0 for the second (two beams, as ParticlesSoA::initializeTwoStream,
 * src/pic/particles_aos.cpp:142-160, when v0 != 0); every particle has the given
 * charge and mass. Philox4x32-10 random numbers, so the set depends only on seed
 * and n. Replaces the resident particles (n <= capacity); marks them unsorted. */
typedef struct pic_gen_config {
    size_t n;
    double amplitude;
    int mode;
    double vth;
    double v0;
    double charge;
    double mass;
    unsigned seed;
} pic_gen_config;
int pic_gpu_generate(pic_ctx* ctx, const pic_gen_config* cfg);
/* Downloads particles back to FP64 SoA (positions rebuilt as (ix+xr)*dx). Any pointer may be NULL.
 * The reference keeps its particles in host memory (pic::ParticlesSoA, src/pic/particles.hpp:45-83);
 * this returns the resident ones there. */
int pic_gpu_download_particles(pic_ctx* ctx, double* x, double* y, double* vx, double* vy, double* q, double* m);
/* Raw device layout, for bit-exact parity checks: any pointer may be NULL (no counterpart
 * in the reference). */
int pic_gpu_download_device_layout(pic_ctx* ctx, uint32_t* cell, float* xr, float* yr, float* vx, float* vy,
                                   float* q);
/* ParticlesSoA::size (src/pic/particles.hpp:45-83) of the resident set. */
int pic_gpu_num_particles(pic_ctx* ctx, size_t* n_out);
/* 1 when the resident particles are in cell order with valid per-cell offsets
 * (after pic_gpu_sort, or after an upload whose keys were already non-decreasing).
 * No counterpart: the reference sorts a copy on every sorted deposit
 * (src/deposition/deposition.cpp:181-200). */
int pic_gpu_is_sorted(pic_ctx* ctx, int* sorted_out);
/* The stored charge q/max|q| shared by every resident particle (+-1), or 0 when
 * the charges differ. With one charge the kernels do not read the charge stream.
 * No counterpart in the reference. */
int pic_gpu_charge_uniform(pic_ctx* ctx, float* qn_out);

/* ---- cell sort: replaces pic::sortParticlesByCell(ParticlesSoA&, const Domain&)
 *      (src/sorting/cell_sort.hpp:8-11, cell_sort.cpp:22-46) ---- */

/* Stable LSD radix sort of the resident particles by cell key, in place.
 * Optional host outputs: sorted keys (n), permutation (n; perm[i] = pre-sort
 * index of the particle now at i) and per-cell offsets (Nx*Ny+1). */
int pic_gpu_sort(pic_ctx* ctx, uint32_t* keys_out, uint32_t* perm_out, uint32_t* offsets_out);

/* ---- deposition: replaces pic::depositChargeSoA / depositKernelSoA's backend
 *      dispatch (src/deposition/deposition.cpp:120-132,181-200) ---- */

int pic_gpu_set_deposit_order(pic_ctx* ctx, int order);
/* Tile of the sorted kernel, in cells (tile_w <= 64, tile_h <= 32). Without
 * this call the tile is chosen per deposit for about 8192 particles per tile. */
int pic_gpu_set_tile(pic_ctx* ctx, int tile_w, int tile_h);
/* Deposits rho for `scheme` (PIC_SCHEME_*) into the context's grid, adds
 * `background` to every node, and copies rho to `rho_out` (Nx*Ny doubles)
 * when non-NULL. `dt` is DepositionConfig::esirkepov_dt (deposition.hpp:23). */
int pic_gpu_deposit(pic_ctx* ctx, int scheme, double dt, double background, double* rho_out);
/* The int64 fixed-point grid of the last deposit and its unit (rho = acc*unit + background). */
int pic_gpu_get_rho_fixed(pic_ctx* ctx, int64_t* acc_out, double* unit_out);
int pic_gpu_get_rho(pic_ctx* ctx, double* rho_out);

/* ---- Esirkepov current (new; the reference's "Esirkepov" deposits charge only,
 *      src/deposition/ngp.cpp:13-84) ----
 * First-order charge-conserving current (Esirkepov 2001) of the move x -> x + v*dt
 * of every resident particle: Jx[iy*Nx+ix] on the edge from node (ix,iy) to
 * (ix+1,iy), Jy[iy*Nx+ix] on the edge to (ix,iy+1). Needs |v|*dt < cell size on
 * each axis (PIC_ERR_COURANT). In the int64 grids, the CIC charge after
 * pic_gpu_push(dt) minus the charge before plus the integer divergence of J is
 * exactly zero at every node. J unit = max|q|*inv_vol*2^-24*dx/dt (x), dy/dt (y). */
int pic_gpu_deposit_current(pic_ctx* ctx, double dt, double* jx_out, double* jy_out);
int pic_gpu_get_current_fixed(pic_ctx* ctx, int64_t* jx, int64_t* jy, double* unit_x, double* unit_y);

/* ---- fields: pic::FieldGrid (src/pic/field_grid.hpp:9-39) ---- */

/* Replaces FieldGrid::rho() with caller data (Nx*Ny doubles). */
int pic_gpu_set_rho(pic_ctx* ctx, const double* rho);
/* Sets phi, Ex, Ey (any may be NULL) and refreshes the FP32 copies the gather reads. */
int pic_gpu_set_fields(pic_ctx* ctx, const double* phi, const double* Ex, const double* Ey);
int pic_gpu_get_fields(pic_ctx* ctx, double* phi, double* Ex, double* Ey);

/* ---- Poisson: replaces pic::PoissonSolverFFT::solve (src/pic/poisson_fft.cpp:45-94) ----
 * phi = IFFT(FFT(rho*dV) / k^2) with the continuous k^2 and DC set to 0, then
 * E = -(phi[i+1]-phi[i])/dx. FP64 cuFFT (D2Z/Z2D) plus this library's kernels. */
int pic_gpu_poisson_fft(pic_ctx* ctx);

/* ---- Poisson by red-black Gauss-Seidel (new; the reference's PoissonSolverGS,
 *      src/pic/poisson_gs.cpp:11-61, is lexicographic with a max|dphi| stop) ----
 * Same 5-point stencil and sign; right-hand side rho*dV minus its mean; starts
 * from the context's phi when warm_start != 0 (the previous solve's, or one set
 * with pic_gpu_set_fields), else from 0; stops when ||b - A phi||_2/||b||_2 <= tol
 * (checked every check_every sweeps) or after max_iters sweeps; removes the mean
 * of phi and computes E. FP64. Needs even Nx and Ny (PIC_ERR_UNSUPPORTED). */
int pic_gpu_poisson_rbgs(pic_ctx* ctx, double tol, int max_iters, int warm_start, int check_every, int* iters_out,
                         double* resid_out);

/* Arithmetic of the red-black Gauss-Seidel sweeps (this context, all later solves; no
 * counterpart: the reference's PoissonSolverGS, src/pic/poisson_gs.cpp:11-61, is FP64 only):
 * 0 (default) FP64 sweeps; 1 FP32 sweeps on a correction equation, refined in FP64
 * (r = b - A phi in FP64, A e = r relaxed in FP32, phi += e, until the FP64
 * relative residual meets tol). Both stop on the same FP64 test; mode 1 needs a
 * grid that tiles into 64x32 (or smaller power-of-two) tiles, else it runs mode 0. */
int pic_gpu_set_rbgs_precision(pic_ctx* ctx, int mixed);

/* Test hook of the bounded device waits (no counterpart in the reference): runs
 * the one-launch FP64 red-black solve on the context's rho (phi from 0, 64
 * sweeps) with CTA absent_block leaving before its first grid barrier (-1: none)
 * and every barrier wait limited to wait_ms (0 < wait_ms <= 1000). The other
 * CTAs give up, set the error flag and return; the call returns PIC_ERR_TIMEOUT
 * and the context stays usable. PIC_ERR_UNSUPPORTED when the grid does not fit
 * one cooperative launch. */
int pic_gpu_test_rbgs_barrier_timeout(pic_ctx* ctx, int absent_block, double wait_ms);

/* ---- particle motion ---- */

/* pic::gatherFieldsSoA (src/deposition/deposition.cpp:335-356): v += -(q/m)*E*dt. */
int pic_gpu_gather(pic_ctx* ctx, double dt);
/* pic::pushParticlesSoA (deposition.cpp:367-374): x += v*dt, periodic wrap. Marks particles unsorted. */
int pic_gpu_push(pic_ctx* ctx, double dt);
/* gather then push in one pass over the particles (44 B per particle). */
int pic_gpu_gather_push(pic_ctx* ctx, double dt);

/* ---- diagnostics: pic::computeDiagnostics (src/pic/diagnostics.cpp:42-51), FP64 sums
 *      in a fixed order (bit-identical run to run) ---- */
int pic_gpu_diagnostics(pic_ctx* ctx, pic_diag* out);

/* ---- time stepping: replaces pic::Simulation::run's loop (src/pic/simulation.cpp:69-145) ----
 * NGP/CIC/TSC: push -> [sort] -> deposit -> +background -> Poisson -> gather -> diagnostics;
 * Esirkepov rho: deposit -> +background -> Poisson -> push -> gather -> diagnostics. */
typedef struct pic_run_config {
    int scheme;            /* PIC_SCHEME_* of the charge deposit */
    int poisson;           /* 0: FFT (PoissonSolverFFT), 1: red-black Gauss-Seidel warm-started from phi */
    double dt;             /* Domain::dt; also the Esirkepov path length v*dt */
    double background;     /* added to rho after each deposit (applyBackgroundIfNeeded, simulation.cpp:52-59) */
    int sort_interval;     /* in-place cell sort every k steps (0: never); results do not depend on it */
    int use_graph;         /* replay the step as a CUDA graph (FFT Poisson only) */
    double rbgs_tol;       /* poisson == 1: relative residual target */
    int rbgs_max_iters;    /* poisson == 1: sweep limit per solve */
    int rbgs_check_every;  /* poisson == 1: sweeps between residual checks */
    int rbgs_warm;         /* poisson == 1: starting guess of each solve: 0 the previous step's phi;
                              1 cubic extrapolation of the last three solutions; 2 extrapolation plus
                              the trained network's correction (pic_gpu_ws_*). Modes 1 and 2 need
                              pic_gpu_ws_init; until three solutions exist they start from phi. */
    double sort_moved_fraction; /* 0: sorts follow sort_interval alone. > 0: also sort when the
                              deposit of step s-2 found more than this fraction of the particles
                              outside their cell of the last sort (read two steps behind, so the
                              GPU never waits for the host); the interval, if > 0, still bounds
                              the steps between sorts, and step 0 sorts unless the particles are
                              already in cell order. Results do not depend on it. */
} pic_run_config;
/* Advances `steps` steps; history (steps entries, may be NULL) receives every
 * step's diagnostics (SimulationResult::*_history, simulation.hpp:49-60). */
int pic_gpu_run(pic_ctx* ctx, const pic_run_config* cfg, int steps, pic_diag* history);
/* Cell sorts performed on this context so far (pic_gpu_sort, and the sorts of pic_gpu_run). */
int pic_gpu_sort_count(pic_ctx* ctx, long long* n);

/* ---- deposit for callers that cannot allocate device memory ----
 *
 * No counterpart in the reference: it exists for hosts that own the whole
 * device-memory budget (a particle code that fills the GPU from its own pool)
 * or that must not pay the device-wide synchronisation of cudaMalloc/cudaFree
 * inside their time-step loop. It needs no context and allocates nothing: the
 * caller passes device arrays in this library's particle layout (cell key
 * iy*Nx+ix, in-cell offsets xr, yr in [0,1], charge qn = q/max_abs_q) and a
 * device output grid rho of Nx*Ny doubles; the int64 scratch grid lives in a
 * fixed device array of PIC_NOALLOC_MAX_CELLS cells (8 MiB) that every GPU
 * loading this library holds until the process exits.
 *  - Grids above PIC_NOALLOC_MAX_CELLS cells are rejected with PIC_ERR_ARG.
 *  - Schemes NGP, CIC and TSC; max_abs_q must be finite and >= 0 (|qn| <= 1 is
 *    the caller's contract). The result equals pic_gpu_deposit's bit for bit on
 *    particles with more than one charge value (with one shared charge,
 *    pic_gpu_deposit's TSC uses exact integer weights: both within the stated
 *    1e-5 relative L2 of the FP64 deposit). Particles whose key is not below
 *    Nx*Ny are skipped.
 *  - The first call in a CUDA context looks up the scratch array's device
 *    address in that context (once per context, with it current); make that
 *    first call before any stream capture.
 *  - All calls share the one scratch array, which keeps the last call's sums;
 *    each call clears the part it uses. Calls whose work overlaps on the GPU
 *    (different streams or host threads) race and corrupt each other.
 *  - Work is queued on `stream` (a cudaStream_t; NULL = the default stream);
 *    the call does not synchronise. */
#define PIC_NOALLOC_MAX_CELLS (1024 * 1024)
int pic_gpu_deposit_noalloc(const pic_domain* domain, int scheme, const uint32_t* cell, const float* xr,
                            const float* yr, const float* qn, size_t n, float max_abs_q, double background,
                            double* rho, void* stream);

/* ---- learned warm start for the red-black Gauss-Seidel solve ----
 *
 * No counterpart in the reference (its PoissonSolverGS, src/pic/poisson_gs.cpp:11-61,
 * starts from zero every call). Three starting guesses for the same solve, each
 * iterated to the same relative residual:
 *   0  the previous step's phi (the plain method and the fallback),
 *   1  the cubic extrapolation E = 3 phi[n-1] - 3 phi[n-2] + phi[n-3],
 *   2  E + s * sigma * net(r / sigma), r = b - A E, sigma = rms(r): a 6-layer 3x3
 *      convolutional network (32 channels, BF16 on the tensor cores, FP32
 *      accumulation) trained on the run's own converged solutions.
 * Needs Nx a multiple of 128 and even Ny. Parameters: one FP32 array, per layer
 * w[9][cout][cin] then bias[cout], channels (16,32),(32,32)x4,(32,16) of which
 * the first layer's input and the last layer's output use channel 0 only. */
typedef struct pic_ws_stats {
    int iters[3];          /* sweeps from guesses 0, 1, 2 */
    double ms[3];          /* device time of each solve: guess + sweeps + checks */
    double resid[3];       /* final relative residual */
    double guess_resid[3]; /* relative residual of the guess itself */
    double phi_diff;       /* rms difference of the guess-2 solution from the guess-0 one */
} pic_ws_stats;

size_t pic_gpu_ws_param_count(void);
/* Creates the network (He-normal initialisation from `seed`) and a device
 * dataset of up to `dataset_capacity` (input, target) pairs of Nx*Ny BF16 each. */
int pic_gpu_ws_init(pic_ctx* ctx, unsigned seed, size_t dataset_capacity);
int pic_gpu_ws_get_params(pic_ctx* ctx, float* params, size_t n);
int pic_gpu_ws_set_params(pic_ctx* ctx, const float* params, size_t n);
/* Advances the resident particles `steps` steps (gather+push, cell sort every
 * sort_interval steps, CIC deposit + background, exact solve of the 5-point
 * system) and appends one training pair per step once three solutions exist. */
int pic_gpu_ws_generate(pic_ctx* ctx, int steps, double dt, double background, int sort_interval);
int pic_gpu_ws_dataset_size(pic_ctx* ctx, size_t* n);
/* Adam (beta 0.9, 0.999) on the mean squared error over shuffled batches;
 * loss_per_epoch[epochs] (may be NULL) gets each epoch's mean loss. */
int pic_gpu_ws_train(pic_ctx* ctx, int epochs, int batch, float lr, unsigned seed, double* loss_per_epoch);
/* Loss and gradient of one batch (inputs, targets: batch*Nx*Ny floats, rounded to
 * BF16 on the device), for checking the backward pass. */
int pic_gpu_ws_loss_grad(pic_ctx* ctx, int batch, const float* inputs, const float* targets, double* loss,
                         float* grad);
/* Network output (Nx*Ny floats) for one input field. */
int pic_gpu_ws_predict(pic_ctx* ctx, const float* input, float* output);
/* Advances `steps` steps as pic_gpu_ws_generate does, but solves each step's
 * system by red-black Gauss-Seidel three times, from guesses 0, 1 and 2, to
 * `tol` (checked every check_every sweeps, at most max_iters), timing each on
 * the device; the run continues with the guess-0 solution. */
int pic_gpu_ws_study(pic_ctx* ctx, int steps, double dt, double background, int sort_interval, double tol,
                     int check_every, int max_iters, pic_ws_stats* stats);

/* ---- batched ensemble of independent runs ----
 *
 * No counterpart in the reference (it runs one Simulation at a time,
 * src/pic/simulation.cpp:69-145). Many Langmuir-oscillation runs with uneven
 * grids (N x N cells, dx = dy = 1) and particle counts advance together: per
 * step every run does gather + push, [cell sort every sort_interval steps], CIC
 * deposit in fixed point + background 1, FFT Poisson (continuous k^2, as
 * PoissonSolverFFT) and E, with the particle work of a step in one persistent
 * cooperative launch and, with use_graph, the whole step one CUDA graph.
 * Particles are generated on the device (counter-based random numbers, seed per
 * run): x from the density 1 + amplitude*cos(2*pi*x/N), y uniform, Maxwellian v
 * of thermal speed vth; charge -1/ppc and mass 1/ppc per particle (mean charge
 * density -1, omega_p = 1). Each run's state equals that of the same run
 * advanced alone through pic_gpu_run (scheme CIC, FFT Poisson, background 1). */
typedef struct pic_ens pic_ens;
typedef struct pic_ens_member {
    int N;          /* grid N x N (even) */
    int ppc;        /* particles per cell */
    unsigned seed;  /* per-run seed (mixed with pic_ens_config.seed); a run's initial state
                     * depends on its N, ppc, seed and the config only, not on the other
                     * runs of the batch, so a batch can be split over GPUs */
} pic_ens_member;
typedef struct pic_ens_config {
    double dt;
    double amplitude;   /* density perturbation on mode 1 */
    double vth;         /* thermal speed per component */
    int sort_interval;  /* cell sort every this many steps (0 = never) */
    int use_graph;
    unsigned seed;
    double sort_disorder; /* 0: sorts follow sort_interval alone. > 0: also sort when, two steps
                             earlier, more than this fraction of adjacent particle pairs were out
                             of cell order after the push (read two steps behind, so the GPU
                             never waits for the host). Results do not depend on it. */
} pic_ens_config;
typedef struct pic_ens_run_info {
    int N, ppc;
    size_t particles;
    int tile_w, tile_h; /* deposit tile chosen by the autotuner (after the first sorted step) */
} pic_ens_run_info;

/* Runs are reordered by grid size (stable); pic_ens_info gives run r's setup in that order. */
int pic_ens_create(const pic_ens_member* runs, int nruns, const pic_ens_config* cfg, int device, pic_ens** out);
int pic_ens_destroy(pic_ens* ens);
/* Advances every run `steps` steps; field_energy and kinetic_energy (steps x nruns,
 * may be NULL) get each run's 0.5*sum(E^2)*dV after the solve and 0.5*m*sum(v^2).
 * PIC_ERR_TIMEOUT: a grid-wide barrier of the step kernel gave up (about one second);
 * that step is incomplete, the error stays set, and the ensemble is to be destroyed. */
int pic_ens_run(pic_ens* ens, int steps, double* field_energy, double* kinetic_energy);
int pic_ens_num_runs(pic_ens* ens, int* n);
int pic_ens_info(pic_ens* ens, int run, pic_ens_run_info* info);
int pic_ens_launch_count(pic_ens* ens, long long* n);
int pic_ens_get_stream(pic_ens* ens, void** stream_out);
/* Cell sorts the ensemble has done. */
int pic_ens_sort_count(pic_ens* ens, long long* n);
/* Run `run`'s particles (positions in cell units, velocities; any pointer may be
 * NULL) in their device order, and its rho and phi (N*N each). */
int pic_ens_download_run(pic_ens* ens, int run, double* x, double* y, double* vx, double* vy, double* rho,
                         double* phi);

/* ---- 3x3 periodic convolution layers on the tensor cores (BF16, FP32 accumulate) ----
 *
 * No counterpart in the reference: the layers of the learned warm start for the
 * red-black Gauss-Seidel solve. This entry runs one layer on host buffers, on
 * the current device, synchronously (it allocates and frees device memory).
 * Tensors are NHWC with BF16 bit patterns; weights FP32 w[tap][cout][cin] with
 * tap = (dy+1)*3 + (dx+1), rounded to BF16 on the device. W must be a multiple
 * of 128 (op 3: of 64); cin, cout in {16, 32}.
 *   op 0: out(BF16, cout ch) = relu(conv(x) + bias)            x: cin channels
 *   op 1: out(FP32, 1 ch)    = conv(x)[channel 0] + bias[0]     x: cin channels
 *   op 2: out(BF16, cin ch)  = conv^T(x) * (aux > 0)            x: cout channels (the
 *         output gradient), aux: cin channels (the layer input, its ReLU mask)
 *   op 3: out(FP32)          = dL/dw [9][cout][cin] then dL/dbias [cout],
 *         x: the layer input (cin ch), aux: the output gradient (cout ch) */
int pic_nn_conv3x3(int op, int batch, int H, int W, int cin, int cout, const uint16_t* x, const float* weight,
                   const float* bias, const uint16_t* aux, void* out);

#ifdef __cplusplus
}
#endif

#endif
