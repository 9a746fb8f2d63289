/*
 * Minimal FFTW3-API shim, written for this project from FFTW's public
 * documentation (halfcomplex r2r layout, "What FFTW Really Computes").
 *
 * Test infrastructure only: it lets the reference's own FFT users
 * (src/pic/poisson_fft.cpp, src/pic/diagnostics.cpp) compile into the CPU
 * oracle library oracle/_ref, because FFTW3 itself is not installed here.
 *
 * Only the calls the reference makes are provided:
 *   fftw_alloc_real, fftw_free, fftw_plan_r2r_2d (R2HC / HC2R),
 *   fftw_execute, fftw_destroy_plan, and the planner flag constants.
 * Transforms are unnormalised, like FFTW's.
 */
#ifndef PIC_ORACLE_FFTW3_SHIM_H
#define PIC_ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { FFTW_R2HC = 0, FFTW_HC2R = 1 } fftw_r2r_kind;

typedef struct pic_shim_fftw_plan_s* fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

double* fftw_alloc_real(size_t n);
void fftw_free(void* p);
fftw_plan fftw_plan_r2r_2d(int n0, int n1, double* in, double* out, fftw_r2r_kind kind0, fftw_r2r_kind kind1,
                           unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);

#ifdef __cplusplus
}
#endif

#endif
