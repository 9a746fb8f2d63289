// Fields: FFT Poisson solve (cuFFT), forward-difference E, FP64 diagnostics.
//
// PoissonSolverFFT::solve (src/pic/poisson_fft.cpp:45-94) in the reference runs
// FFTW's R2HC x R2HC transform of rho*dV, divides by the continuous k^2
// (k = 2*pi*m/L, m folded to [-N/2, N/2], poisson_fft.cpp:23-35) with the DC term
// set to zero, transforms back, scales by 1/(Nx*Ny) and takes the forward
// difference E = -(phi[i+1] - phi[i]) / dx (poisson_fft.cpp:77-93). The
// separable halfcomplex basis and the complex basis diagonalise the same
// operator with the same eigenvalue k^2 per frequency, so here the transform is
// cuFFT's D2Z / Z2D in FP64 with this library's own k-divide and E kernels.
//
// Diagnostics (src/pic/field_grid.cpp:24-38, particles_aos.cpp:182-196,
// diagnostics.cpp:26-51) are FP64 sums computed with a fixed two-level tree
// (fixed block partition, then one block over the partials), so every run
// gives the same bits.
#include <cufft.h>

#include <cmath>

#include "pic_internal.cuh"

namespace picgb {

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 1024;  // fixed partition: results do not depend on the device

// ---- deterministic FP64 sums --------------------------------------------
__device__ __forceinline__ double block_sum(double v) {
    __shared__ double ws[RED_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) ws[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < RED_THREADS / 32; ++w) s = __dadd_rn(s, ws[w]);
    __syncthreads();
    return s;
}

// Per-item quantities summed by the diagnostics.
enum SumKind : int {
    SUM_GRID = 0,      // sum x[i]
    SUM_GRID_SQ2 = 1,  // sum x[i]^2 + y[i]^2
    SUM_Q = 2,         // sum qn[i]*maxq
    SUM_ABS_Q = 3,     // sum |qn[i]*maxq|
    SUM_KE = 4,        // sum 0.5*m*(vx^2+vy^2)
};

struct SumArgs {
    int kind;
    const double* x;
    const double* y;
    const float* q;
    const float* vx;
    const float* vy;
    const float* m;
    const DevStats* st;
    size_t n;
};

__device__ __forceinline__ double sum_item(const SumArgs& a, size_t i) {
    switch (a.kind) {
        case SUM_GRID:
            return a.x[i];
        case SUM_GRID_SQ2:
            return __dadd_rn(__dmul_rn(a.x[i], a.x[i]), __dmul_rn(a.y[i], a.y[i]));
        case SUM_Q:
            return (double)(a.q[i] * load_maxq(a.st));
        case SUM_ABS_Q:
            return fabs((double)(a.q[i] * load_maxq(a.st)));
        default: {
            const double vx = a.vx[i], vy = a.vy[i];
            const double m = a.m ? (double)a.m[i] : 1.0;
            return __dmul_rn(__dmul_rn(0.5, m), __dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)));
        }
    }
}

__global__ void __launch_bounds__(RED_THREADS) sum_partials(SumArgs a, double* __restrict__ partial) {
    const size_t chunk = (a.n + RED_BLOCKS - 1) / RED_BLOCKS;
    const size_t b = (size_t)blockIdx.x * chunk;
    const size_t e = b + chunk < a.n ? b + chunk : a.n;
    double s = 0.0;
    for (size_t i = b + threadIdx.x; i < e; i += RED_THREADS) s = __dadd_rn(s, sum_item(a, i));
    const double t = block_sum(s);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// Sum of vx^2 + vy^2 over the particles with no FP64 arithmetic per particle
// (FP64 is slow on this part): each square is formed exactly as an FP32 pair
// (product and its fused-multiply-add error), each thread accumulates in
// double-FP32 (Knuth's two-sum keeps the running sum's rounding errors; ke_add),
// and the threads' totals enter the same deterministic FP64 block and grid sums.
// Agrees with an FP64 sum of the squares to about 1e-14 relative.

__global__ void __launch_bounds__(RED_THREADS) sum_v2_partials(const float* __restrict__ vx,
                                                              const float* __restrict__ vy, size_t n,
                                                              double* __restrict__ partial) {
    const size_t chunk = (n + RED_BLOCKS - 1) / RED_BLOCKS;
    const size_t b = (size_t)blockIdx.x * chunk;
    const size_t e = b + chunk < n ? b + chunk : n;
    float hi = 0.0f, lo = 0.0f;
    for (size_t i = b + threadIdx.x; i < e; i += RED_THREADS) {
        ke_add(hi, lo, vx[i], vy[i]);
    }
    const double t = block_sum(__dadd_rn((double)hi, (double)lo));
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void __launch_bounds__(RED_THREADS) sum_final(const double* __restrict__ partial, double scale,
                                                        double* out, int count = RED_BLOCKS) {
    double s = 0.0;
    for (int i = threadIdx.x; i < count; i += RED_THREADS) s = __dadd_rn(s, partial[i]);
    const double t = block_sum(s);
    if (threadIdx.x == 0) *out = __dmul_rn(t, scale);
}

// Queues one deterministic sum into slot `out` (device), times `scale`.
int device_sum(pic_ctx* c, const SumArgs& a, double* out, double scale) {
    sum_partials<<<RED_BLOCKS, RED_THREADS, 0, c->stream>>>(a, c->red_partials);
    PIC_TRY(check_launch(c, "sum_partials"));
    sum_final<<<1, RED_THREADS, 0, c->stream>>>(c->red_partials, scale, out);
    return check_launch(c, "sum_final");
}
int device_sum(pic_ctx* c, const SumArgs& a, double* out) { return device_sum(c, a, out, 1.0); }

__global__ void copy_charge_sums(double* r) {
    r[1] = r[8];
    r[6] = r[9];
}

// ---- Poisson ---------------------------------------------------------------
__global__ void rhs_from_rho(const double* __restrict__ rho, double vol, size_t g, double* __restrict__ rhs) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g) rhs[i] = __dmul_rn(rho[i], vol);  // poisson_fft.cpp:51-55
}

// spectrum /= k^2 (continuous k, poisson_fft.cpp:23-35), DC = 0 (poisson_fft.cpp:59-62)
__global__ void k_divide(cufftDoubleComplex* __restrict__ spec, int Nx, int Ny, double Lx, double Ly) {
    const int nh = Nx / 2 + 1;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)nh * Ny) return;
    const int i = (int)(t % nh), j = (int)(t / nh);
    if (i == 0 && j == 0) {
        spec[t].x = 0.0;
        spec[t].y = 0.0;
        return;
    }
    const double twopi = 2.0 * 3.14159265358979323846;
    const int mx = (i <= Nx / 2) ? i : i - Nx;
    const int my = (j <= Ny / 2) ? j : j - Ny;
    const double kx = __ddiv_rn(__dmul_rn(twopi, (double)mx), Lx);
    const double ky = __ddiv_rn(__dmul_rn(twopi, (double)my), Ly);
    const double k2 = __dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky));
    spec[t].x = __ddiv_rn(spec[t].x, k2);
    spec[t].y = __ddiv_rn(spec[t].y, k2);
}

__global__ void scale_phi(double* __restrict__ phi, size_t g, double norm) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g) phi[i] = __dmul_rn(phi[i], norm);  // poisson_fft.cpp:66-75
}

// E = -(phi[i+1] - phi[i]) / d (poisson_fft.cpp:77-93, poisson_gs.cpp:48-60); FP32 copies for gather.
__global__ void efield(const double* __restrict__ phi, int Nx, int Ny, double idx_dx, double idx_dy,
                       double* __restrict__ Ex, double* __restrict__ Ey, float* __restrict__ Exf,
                       float* __restrict__ Eyf) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)Nx * Ny) return;
    const int i = (int)(t % Nx), j = (int)(t / Nx);
    const int ip = (i + 1) % Nx, jp = (j + 1) % Ny;
    const double p = phi[t];
    const double ex = -__dmul_rn(__dsub_rn(phi[(size_t)j * Nx + ip], p), idx_dx);
    const double ey = -__dmul_rn(__dsub_rn(phi[(size_t)jp * Nx + i], p), idx_dy);
    Ex[t] = ex;
    Ey[t] = ey;
    Exf[t] = __double2float_rn(ex);
    Eyf[t] = __double2float_rn(ey);
}

__global__ void fields_to_f32(const double* __restrict__ Ex, const double* __restrict__ Ey, size_t g,
                              float* __restrict__ Exf, float* __restrict__ Eyf) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g) {
        Exf[i] = __double2float_rn(Ex[i]);
        Eyf[i] = __double2float_rn(Ey[i]);
    }
}

static const char* cufft_name(cufftResult r) {
    switch (r) {
        case CUFFT_SUCCESS:
            return "CUFFT_SUCCESS";
        case CUFFT_ALLOC_FAILED:
            return "CUFFT_ALLOC_FAILED";
        case CUFFT_INVALID_VALUE:
            return "CUFFT_INVALID_VALUE";
        case CUFFT_EXEC_FAILED:
            return "CUFFT_EXEC_FAILED";
        case CUFFT_SETUP_FAILED:
            return "CUFFT_SETUP_FAILED";
        case CUFFT_INVALID_SIZE:
            return "CUFFT_INVALID_SIZE";
        default:
            return "cuFFT error";
    }
}

#define PIC_CUFFT_TRY(call)                                                              \
    do {                                                                                 \
        cufftResult r__ = (call);                                                        \
        if (r__ != CUFFT_SUCCESS) return fail(PIC_ERR_CUDA, std::string(#call) + ": " + cufft_name(r__)); \
    } while (0)

int ensure_fields(pic_ctx* c) {
    int rc = PIC_OK;
    const size_t g = c->G;
    if (!c->phi) c->phi = (double*)dalloc(g * 8, &rc);
    if (rc) return rc;
    if (!c->Ex) c->Ex = (double*)dalloc(g * 8, &rc);
    if (rc) return rc;
    if (!c->Ey) c->Ey = (double*)dalloc(g * 8, &rc);
    if (rc) return rc;
    if (!c->Exf) c->Exf = (float*)dalloc(g * 4, &rc);
    if (rc) return rc;
    if (!c->Eyf) c->Eyf = (float*)dalloc(g * 4, &rc);
    if (rc) return rc;
    if (!c->red_partials) c->red_partials = (double*)dalloc(RED_BLOCKS * 8, &rc);
    if (!rc && !c->ke_partials) c->ke_partials = (double*)dalloc(MOVE_KE_BLOCKS * 8, &rc);
    if (rc) return rc;
    if (!c->red_out) c->red_out = (double*)dalloc(16 * 8, &rc);
    if (rc) return rc;
    if (!c->fields_init) {
        PIC_CUDA_TRY(cudaMemsetAsync(c->phi, 0, g * 8, c->stream));
        PIC_CUDA_TRY(cudaMemsetAsync(c->Ex, 0, g * 8, c->stream));
        PIC_CUDA_TRY(cudaMemsetAsync(c->Ey, 0, g * 8, c->stream));
        PIC_CUDA_TRY(cudaMemsetAsync(c->Exf, 0, g * 4, c->stream));
        PIC_CUDA_TRY(cudaMemsetAsync(c->Eyf, 0, g * 4, c->stream));
        c->fields_init = 1;
    }
    return PIC_OK;
}

static int ensure_fft(pic_ctx* c) {
    PIC_TRY(ensure_fields(c));
    if (c->fft_ready) return PIC_OK;
    int rc = PIC_OK;
    const size_t nh = (size_t)(c->Nx / 2 + 1);
    c->spec = dalloc(nh * (size_t)c->Ny * sizeof(cufftDoubleComplex), &rc);
    if (rc) return rc;
    c->fft_rhs = (double*)dalloc(c->G * 8, &rc);
    if (rc) return rc;
    cufftHandle f, b;
    PIC_CUFFT_TRY(cufftPlan2d(&f, c->Ny, c->Nx, CUFFT_D2Z));
    PIC_CUFFT_TRY(cufftPlan2d(&b, c->Ny, c->Nx, CUFFT_Z2D));
    PIC_CUFFT_TRY(cufftSetStream(f, c->stream));
    PIC_CUFFT_TRY(cufftSetStream(b, c->stream));
    c->fft_fwd = (int)f;
    c->fft_inv = (int)b;
    c->fft_ready = 1;
    return PIC_OK;
}

void release_fields(pic_ctx* c) {
    if (c->fft_ready) {
        cufftDestroy((cufftHandle)c->fft_fwd);
        cufftDestroy((cufftHandle)c->fft_inv);
        c->fft_ready = 0;
    }
    void* ptrs[] = {c->phi, c->Ex, c->Ey, c->Exf, c->Eyf, c->spec, c->fft_rhs, c->red_partials, c->red_out,
                    c->ke_partials};
    for (void* p : ptrs) dfree(p);
}

int efield_from_phi(pic_ctx* c) {
    const unsigned blocks = (unsigned)((c->G + 255) / 256);
    efield<<<blocks, 256, 0, c->stream>>>(c->phi, c->Nx, c->Ny, 1.0 / c->dx, 1.0 / c->dy, c->Ex, c->Ey, c->Exf,
                                          c->Eyf);
    return check_launch(c, "efield");
}

int poisson_fft(pic_ctx* c) {
    PIC_TRY(ensure_fft(c));
    const unsigned blocks = (unsigned)((c->G + 255) / 256);
    rhs_from_rho<<<blocks, 256, 0, c->stream>>>(c->rho, c->dx * c->dy, c->G, c->fft_rhs);
    PIC_TRY(check_launch(c, "rhs_from_rho"));
    prof_begin(c, "poisson_fft");
    PIC_CUFFT_TRY(cufftExecD2Z((cufftHandle)c->fft_fwd, c->fft_rhs, (cufftDoubleComplex*)c->spec));
    const size_t ns = (size_t)(c->Nx / 2 + 1) * c->Ny;
    k_divide<<<(unsigned)((ns + 255) / 256), 256, 0, c->stream>>>((cufftDoubleComplex*)c->spec, c->Nx, c->Ny, c->Lx,
                                                                   c->Ly);
    PIC_TRY(check_launch(c, "k_divide"));
    PIC_CUFFT_TRY(cufftExecZ2D((cufftHandle)c->fft_inv, (cufftDoubleComplex*)c->spec, c->phi));
    prof_end(c);
    scale_phi<<<blocks, 256, 0, c->stream>>>(c->phi, c->G, 1.0 / (double)c->G);
    PIC_TRY(check_launch(c, "scale_phi"));
    return efield_from_phi(c);
}

// spectrum /= eigenvalue of the 5-point operator
//   denom - 2*ix2*cos(2*pi*mx/Nx) - 2*iy2*cos(2*pi*my/Ny), DC = 0
__global__ void k_divide_discrete(cufftDoubleComplex* __restrict__ spec, int Nx, int Ny, double ix2, double iy2,
                                  double denom) {
    const int nh = Nx / 2 + 1;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)nh * Ny) return;
    const int i = (int)(t % nh), j = (int)(t / nh);
    if (i == 0 && j == 0) {
        spec[t].x = 0.0;
        spec[t].y = 0.0;
        return;
    }
    const double twopi = 2.0 * 3.14159265358979323846;
    const double cx = cos(twopi * (double)i / (double)Nx), cy = cos(twopi * (double)j / (double)Ny);
    const double lam = denom - 2.0 * ix2 * cx - 2.0 * iy2 * cy;
    spec[t].x = spec[t].x / lam;
    spec[t].y = spec[t].y / lam;
}

int solve_discrete_fft(pic_ctx* c, const double* b, double* phi) {
    PIC_TRY(ensure_fft(c));
    double ix2, iy2, denom;
    rbgs_operator(c, &ix2, &iy2, &denom);
    PIC_CUDA_TRY(cudaMemcpyAsync(c->fft_rhs, b, c->G * 8, cudaMemcpyDeviceToDevice, c->stream));
    PIC_CUFFT_TRY(cufftExecD2Z((cufftHandle)c->fft_fwd, c->fft_rhs, (cufftDoubleComplex*)c->spec));
    const size_t ns = (size_t)(c->Nx / 2 + 1) * c->Ny;
    k_divide_discrete<<<(unsigned)((ns + 255) / 256), 256, 0, c->stream>>>((cufftDoubleComplex*)c->spec, c->Nx,
                                                                            c->Ny, ix2, iy2, denom);
    PIC_TRY(check_launch(c, "k_divide_discrete"));
    PIC_CUFFT_TRY(cufftExecZ2D((cufftHandle)c->fft_inv, (cufftDoubleComplex*)c->spec, phi));
    scale_phi<<<(unsigned)((c->G + 255) / 256), 256, 0, c->stream>>>(phi, c->G, 1.0 / (double)c->G);
    return check_launch(c, "scale_phi");
}

// Queues the six diagnostics into c->red_out[0..5] (pic_diag order).
int diagnostics_async(pic_ctx* c) {
    PIC_TRY(ensure_fields(c));
    SumArgs a{};
    a.st = c->dstats;
    a.q = c->q;
    a.vx = c->vx;
    a.vy = c->vy;
    a.m = c->has_mass ? c->m : nullptr;
    a.n = c->n;
    if (!c->qsum_valid) {  // total charge and sum |q| change only with the particle set
        a.kind = SUM_Q;
        PIC_TRY(device_sum(c, a, c->red_out + 8));
        a.kind = SUM_ABS_Q;
        PIC_TRY(device_sum(c, a, c->red_out + 9));
        c->qsum_valid = 1;
    }
    copy_charge_sums<<<1, 1, 0, c->stream>>>(c->red_out);  // total_charge, sum |q|
    PIC_TRY(check_launch(c, "copy_charge_sums"));
    // kinetic: sum 0.5*m*v^2 in FP64 per particle when masses differ from 1;
    // with unit masses 0.5 * sum v^2 (double-FP32 per thread, FP64 across threads)
    if (a.m) {
        a.kind = SUM_KE;
        PIC_TRY(device_sum(c, a, c->red_out + 3));
    } else if (c->n > 0 && c->ke_ready) {  // left by the gather that produced these velocities
        c->ke_ready = 0;                     // used once: the next diagnostics recompute unless a gather refills it
        sum_final<<<1, RED_THREADS, 0, c->stream>>>(c->ke_partials, 0.5, c->red_out + 3, c->ke_count);
        PIC_TRY(check_launch(c, "sum_final"));
    } else if (c->n > 0) {
        sum_v2_partials<<<RED_BLOCKS, RED_THREADS, 0, c->stream>>>(c->vx, c->vy, c->n, c->red_partials);
        PIC_TRY(check_launch(c, "sum_v2_partials"));
        sum_final<<<1, RED_THREADS, 0, c->stream>>>(c->red_partials, 0.5, c->red_out + 3);
        PIC_TRY(check_launch(c, "sum_final"));
    } else {
        PIC_CUDA_TRY(cudaMemsetAsync(c->red_out + 3, 0, sizeof(double), c->stream));
    }
    SumArgs g{};
    g.n = c->G;
    g.kind = SUM_GRID;
    g.x = c->rho;
    PIC_TRY(device_sum(c, g, c->red_out + 2));  // sum rho
    g.kind = SUM_GRID_SQ2;
    g.x = c->Ex;
    g.y = c->Ey;
    return device_sum(c, g, c->red_out + 4);  // sum Ex^2+Ey^2
}

int read_diagnostics(pic_ctx* c, pic_diag* d) {
    double r[8];
    PIC_CUDA_TRY(cudaMemcpyAsync(r, c->red_out, sizeof(r), cudaMemcpyDeviceToHost, c->stream));
    PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    const double vol = c->dx * c->dy;
    d->total_charge = r[1];
    d->integrated_rho = r[2] * vol;                       // field_grid.cpp:24-30
    const double den = r[6] > 1e-12 ? r[6] : 1e-12;       // diagnostics.cpp:26-29
    d->charge_error = std::fabs(d->integrated_rho - d->total_charge) / den;
    d->kinetic_energy = r[3];
    d->field_energy = 0.5 * r[4] * vol;                   // field_grid.cpp:32-38
    d->total_energy = d->kinetic_energy + d->field_energy;
    return PIC_OK;
}

}  // namespace picgb

using namespace picgb;

extern "C" {

int pic_gpu_set_rho(pic_ctx* c, const double* rho) {
    if (!c || !rho) return fail(PIC_ERR_ARG, "NULL argument");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    PIC_CUDA_TRY(cudaMemcpyAsync(c->rho, rho, c->G * 8, cudaMemcpyHostToDevice, c->stream));
    return pic_gpu_synchronize(c);
}

int pic_gpu_set_fields(pic_ctx* c, const double* phi, const double* Ex, const double* Ey) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    PIC_TRY(ensure_fields(c));
    if (phi) PIC_CUDA_TRY(cudaMemcpyAsync(c->phi, phi, c->G * 8, cudaMemcpyHostToDevice, c->stream));
    if (Ex) PIC_CUDA_TRY(cudaMemcpyAsync(c->Ex, Ex, c->G * 8, cudaMemcpyHostToDevice, c->stream));
    if (Ey) PIC_CUDA_TRY(cudaMemcpyAsync(c->Ey, Ey, c->G * 8, cudaMemcpyHostToDevice, c->stream));
    fields_to_f32<<<(unsigned)((c->G + 255) / 256), 256, 0, c->stream>>>(c->Ex, c->Ey, c->G, c->Exf, c->Eyf);
    PIC_TRY(check_launch(c, "fields_to_f32"));
    return pic_gpu_synchronize(c);
}

int pic_gpu_get_fields(pic_ctx* c, double* phi, double* Ex, double* Ey) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_TRY(ensure_fields(c));
    if (phi) PIC_CUDA_TRY(cudaMemcpyAsync(phi, c->phi, c->G * 8, cudaMemcpyDeviceToHost, c->stream));
    if (Ex) PIC_CUDA_TRY(cudaMemcpyAsync(Ex, c->Ex, c->G * 8, cudaMemcpyDeviceToHost, c->stream));
    if (Ey) PIC_CUDA_TRY(cudaMemcpyAsync(Ey, c->Ey, c->G * 8, cudaMemcpyDeviceToHost, c->stream));
    return pic_gpu_synchronize(c);
}

int pic_gpu_poisson_fft(pic_ctx* c) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    return poisson_fft(c);
}

int pic_gpu_diagnostics(pic_ctx* c, pic_diag* out) {
    if (!c || !out) return fail(PIC_ERR_ARG, "NULL argument");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    PIC_TRY(diagnostics_async(c));
    PIC_TRY(read_diagnostics(c, out));
    return check_device_status(c);
}

}  // extern "C"
