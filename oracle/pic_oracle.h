/*
 * CPU oracle for the GB300 PIC deposition path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
 * load liboracle.so, and only as the checker or as the timed CPU baseline.
 * The product (libpicgb300.so and its host adapter) never links or calls it.
 *
 * Two families of functions:
 *  1. FP64 restatements of the reference algorithms of ehocine/pic-deposition
 *     (each cites the reference file:line it follows). These are checked
 *     against the reference itself (oracle/_ref, built from the reference
 *     sources) and against the reference's archived golden CSVs.
 *  2. Exact restatements of the GPU arithmetic (FP32 cell-relative positions,
 *     int32 fixed-point stencil contributions summed in int64, each particle's
 *     contributions adding up exactly to its integer charge), used for
 *     bit-exact parity of the CUDA kernels.
 *
 * Compiled with -ffp-contract=off: no multiply-add is fused, matching the CUDA
 * kernels, which are compiled with --fmad=false.
 */
#ifndef PIC_ORACLE_H
#define PIC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double Lx, Ly;
    int32_t Nx, Ny;
} orc_domain;

enum { ORC_NGP = 0, ORC_CIC = 1, ORC_TSC = 2, ORC_ESIRKEPOV = 3 };

/* ---- geometry (src/pic/domain.hpp) ---- */
void orc_cell_coords(const orc_domain* d, double x, double y, int* ix, int* iy, double* wx, double* wy);
int orc_particle_cell_index(const orc_domain* d, double x, double y);

/* ---- reference RNG and initialisers (src/pic/particles_aos.cpp) ---- */
int orc_init_particles(int kind, const orc_domain* d, size_t n, double p0, double p1, int mode, uint32_t seed,
                       double* x, double* y, double* vx, double* vy, double* q, double* m);

/* ---- FP64 reference deposits (src/deposition/ngp.cpp, deposition_parallel.cpp) ---- */
int orc_deposit_ref(const orc_domain* d, int scheme, size_t n, const double* x, const double* y, const double* vx,
                    const double* vy, const double* q, double esirkepov_dt, int threads, double* rho);
int orc_deposit_timed(const orc_domain* d, int scheme, size_t n, const double* x, const double* y, const double* vx,
                      const double* vy, const double* q, double esirkepov_dt, int threads, int warmups, int repeats,
                      double* rho, double* mean_ms);

/* ---- stable cell sort (keys bit-exact with src/sorting/cell_sort.cpp:8-13) ---- */
int orc_stable_cell_sort(const orc_domain* d, size_t n, const double* x, const double* y, uint32_t* keys_sorted,
                         uint32_t* perm, uint32_t* offsets);
/* sortParticlesByCell (src/sorting/cell_sort.cpp:22-46), in place (cell_sort_port.cpp) */
int orc_sort_particles_by_cell(const orc_domain* d, size_t n, double* x, double* y, double* vx, double* vy,
                               double* q, double* m);
int orc_stable_sort_keys(size_t n, uint32_t nkeys, const uint32_t* keys, uint32_t* keys_sorted, uint32_t* perm,
                         uint32_t* offsets);

/* ---- FP64 gather / push (src/deposition/deposition.cpp:335-374) ---- */
void orc_gather_ref(const orc_domain* d, size_t n, const double* x, const double* y, double* vx, double* vy,
                    const double* q, const double* m, const double* ex, const double* ey, double dt);
void orc_push_ref(const orc_domain* d, size_t n, double* x, double* y, const double* vx, const double* vy, double dt);

/* ---- Poisson (src/pic/poisson_gs.cpp) ---- */
int orc_gs_ref(const orc_domain* d, const double* rho, int max_iters, double tol, double* phi, double* ex, double* ey);
void orc_efield(const orc_domain* d, const double* phi, double* ex, double* ey);
int orc_rbgs(const orc_domain* d, const double* rho, double* phi, double tol, int max_iters, int check_every,
             int* iters_out, double* resid_out);
double orc_rbgs_residual(const orc_domain* d, const double* b, const double* phi);

/* ---- FP64 sums (src/pic/field_grid.cpp:24-38, particles_aos.cpp:182-196, diagnostics.cpp:26-29) ---- */
double orc_integrated_rho(const orc_domain* d, const double* rho);
double orc_field_energy(const orc_domain* d, const double* ex, const double* ey);
double orc_kinetic_energy(size_t n, const double* vx, const double* vy, const double* m);
double orc_charge_error(double integrated_rho, double total_charge, double abs_charge_sum);

/* ---- restatement of the GPU data layout and fixed-point deposit ---- */
void orc_to_device(const orc_domain* d, size_t n, const double* x, const double* y, uint32_t* cell, float* xr,
                   float* yr);
void orc_normalize_charge(size_t n, const double* q, float* qn, float* maxq_out);
int orc_charge_uniform(size_t n, const float* qn);
int orc_deposit_fixed(const orc_domain* d, int scheme, size_t n, const uint32_t* cell, const float* xr,
                      const float* yr, const float* vx, const float* vy, const float* qn, float maxq, double dt,
                      int64_t* acc, double* unit_out);
void orc_fixed_to_rho(size_t g, const int64_t* acc, double unit, double background, double* rho);
int orc_esirkepov_j_ref(const orc_domain* d, size_t n, const double* x, const double* y, const double* vx,
                        const double* vy, const double* q, double dt, double* jx, double* jy);
int orc_esirkepov_j_fixed(const orc_domain* d, size_t n, const uint32_t* cell, const float* xr, const float* yr,
                          const float* vx, const float* vy, const float* qn, float maxq, double dt, int64_t* jx,
                          int64_t* jy, double* unit_x, double* unit_y);
void orc_move_f32(const orc_domain* d, size_t n, uint32_t* cell, float* xr, float* yr, float* vx, float* vy,
                  const float* qn, float maxq, const float* m, const double* Ex, const double* Ey, double dt,
                  int gather, int push);

#ifdef __cplusplus
}
#endif

#endif
