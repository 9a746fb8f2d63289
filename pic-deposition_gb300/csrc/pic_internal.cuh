// Internal definitions shared by the translation units of libpicgb300.so.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "pic_gb300.h"

namespace picgb {

// Device-side status block. The error fields are written with atomicCAS so the
// first failure wins; maxima of |q|, |vx|, |vy| are kept as the bit patterns of
// non-negative floats, whose unsigned order equals their float order.
struct DevStats {
    unsigned int maxq_bits;
    unsigned int maxvx_bits;
    unsigned int maxvy_bits;
    int err;
    unsigned int err_info;
    unsigned int order_breaks;  // uploads: count of i with cell[i] < cell[i-1]
    unsigned int q_mixed;       // uploads: nonzero when the stored charges differ
    float q_first;              // uploads: the first particle's stored charge
    float q_raw0;               // uploads: the first particle's charge before normalisation
    unsigned int any_order;     // between sorts: 1 once most particles have left their sorted cell
    unsigned long long moved;   // deposits between sorts: particles found outside their sorted cell
    unsigned long long moved_dep;  // the same, for the any_order decision after each deposit
};

enum DevErr : int {
    DEV_OK = 0,
    DEV_BAD_POSITION = 1,   // non-finite or out-of-range position on upload
    DEV_BAD_CELL = 3,       // cell key >= Nx*Ny
    DEV_MOVE_TOO_LARGE = 4, // trajectory longer than the general Esirkepov loop allows
    DEV_COURANT = 5,        // Esirkepov current with |v|*dt >= cell size
};

// Particle arrays are allocated this many elements longer than the capacity:
// the sorted deposit reads four consecutive particles with one 128-bit load
// from a 4-aligned index below n, which may reach up to 3 elements past n.
constexpr size_t PARTICLE_PAD = 32;
constexpr int MOVE_KE_BLOCKS = 4096;  // fixed grid of a gather that sums the kinetic energy

struct WsState;

struct ScanScratch {
    unsigned int* partials = nullptr;  // per-level block sums
    size_t capacity = 0;               // elements in partials
};

}  // namespace picgb

struct pic_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;

    // domain (pic::Domain, src/pic/domain.hpp)
    double Lx = 1.0, Ly = 1.0, dx = 1.0, dy = 1.0;
    int Nx = 1, Ny = 1;
    size_t G = 1;

    // particles, device SoA
    size_t n = 0, cap = 0;
    uint32_t* cell = nullptr;
    float *xr = nullptr, *yr = nullptr, *vx = nullptr, *vy = nullptr, *q = nullptr, *m = nullptr;
    int has_mass = 0;
    // Nonzero when every particle's stored charge q/max|q| equals it (one
    // species; set by an upload that finds it so, and by a generate): the
    // kernels then use the value instead of reading the charge stream (the
    // array stays valid, the sort leaves it in place).
    float qn_uniform = 0.0f;
    int sorted = 0;  // particles are in stable cell order and `offsets` is valid
    // `offsets` (from the last sort) still cut the particle array into the cells'
    // ranges of that sort: kept by the push, which moves particles without
    // reordering them; cleared when particles are replaced or reordered
    int part_valid = 0;

    // sort scratch
    uint32_t *cell_alt = nullptr, *idx_a = nullptr, *idx_b = nullptr;
    float *alt[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    uint32_t* counts = nullptr;  // radix histograms, digit-major
    size_t counts_cap = 0;
    uint32_t* offsets = nullptr;  // G+1
    uint32_t* cellcount = nullptr;  // G+1
    picgb::ScanScratch scan;

    // upload staging (device FP64, two slots) and its copy stream
    double* stage = nullptr;
    size_t stage_elems = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_converted[2] = {nullptr, nullptr};

    // grid
    long long* acc = nullptr;  // fixed-point rho accumulator (G)
    double* rho = nullptr;     // FP64 rho (G)
    double* unitbuf = nullptr; // device copy of the last fixed-point unit
    int last_scheme = -1;

    // fields (FieldGrid phi/Ex/Ey, src/pic/field_grid.hpp) + FP32 copies for the gather
    double *phi = nullptr, *Ex = nullptr, *Ey = nullptr;
    float *Exf = nullptr, *Eyf = nullptr;
    int fields_init = 0;
    // cuFFT Poisson
    void* spec = nullptr;  // Ny x (Nx/2+1) complex
    double* fft_rhs = nullptr;
    int fft_fwd = 0, fft_inv = 0, fft_ready = 0;
    // deterministic FP64 reductions
    double* red_partials = nullptr;
    double* red_out = nullptr;
    // per-block sums of vx^2 + vy^2 left by a time step's gather (MOVE_KE_BLOCKS
    // entries); ke_ready: they belong to the current velocities
    double* ke_partials = nullptr;
    int ke_ready = 0;
    int ke_count = 0;  // entries the last gather filled
    // red_out[8], red_out[9] hold sum(q) and sum(|q|) of the current particle set:
    // charges do not change while particles move or are sorted
    int qsum_valid = 0;
    // red-black Gauss-Seidel
    double *rb_b = nullptr, *rb_partial = nullptr, *rb_scalars = nullptr;
    double* rb_ps = nullptr;   // persistent solve: partial sums, barrier, results
    int rbgs_persistent = 1;   // use the one-launch solve where it applies
    int rbgs_mixed = 0;        // FP32 sweeps on FP64-refined corrections (pic_gpu_set_rbgs_precision)
    double* rb_mix = nullptr;  // mixed solve: FP64 residual, FP32 rhs and correction
    int last_rbgs_iters = 0;
    double last_rbgs_resid = 0.0, first_rbgs_resid = 0.0;
    // learned warm start (warmstart.cu)
    picgb::WsState* ws = nullptr;
    // Esirkepov current: int64 edge grids, FP64 copies, units (x, y)
    long long *accjx = nullptr, *accjy = nullptr;
    double *jx = nullptr, *jy = nullptr, *junits = nullptr;
    int has_current = 0;
    // kernels inside the captured time-step graphs (for the launch counter)
    long long graph_launches_sort = 0, graph_launches_plain = 0;

    picgb::DevStats* dstats = nullptr;

    // tuning
    int order_mode = PIC_ORDER_AUTO;
    int tile_w = 32, tile_h = 8;
    int tile_user = 0;  // tile shape set by pic_gpu_set_tile (else chosen per deposit)

    long long launches = 0;
    long long sorts = 0;  // cell sorts performed (pic_gpu_sort and the time step's)

    // optional CUDA-event records around named kernels (pic_gpu_profile_*)
    int prof_enabled = 0;
    struct ProfRec {
        const char* name;
        cudaEvent_t a, b;
    };
    std::vector<ProfRec>* prof = nullptr;
};

namespace picgb {

// Records a failure message for pic_gpu_last_error and returns `code`.
int fail(int code, const std::string& msg);
// Checks a CUDA call; on failure records the message and returns PIC_ERR_CUDA.
int cuda_fail(cudaError_t e, const char* what);
// Reads back the device status block; maps a device error to PIC_ERR_*.
int check_device_status(pic_ctx* ctx);
// Launch-configuration error check after a kernel launch.
int check_launch(pic_ctx* ctx, const char* what);
// Raises `kernel`'s dynamic shared-memory limit on the current device to at least
// `bytes` (the attribute is per device; recorded per kernel and device, thread-safe).
int opt_in_dynamic_smem(const void* kernel, size_t bytes);

void* dalloc(size_t bytes, int* rc);
void dfree(void* p);

// Device-wide exclusive scan of n u32 values in place (any n >= 0).
int exclusive_scan_u32(pic_ctx* ctx, unsigned int* data, size_t n);

// Ensures sort/offset scratch sized for the context's capacity and grid.
int ensure_sort_scratch(pic_ctx* ctx);
// Per-cell offsets of cell-ordered keys (histogram + scan into ctx->offsets).
int build_offsets(pic_ctx* ctx, const uint32_t* keys);
// perm: also build the permutation (idx_a) that pic_gpu_sort returns; the
// library's own sorts (time step, ensemble, warm start) do not read it
int sort_particles(pic_ctx* ctx, bool perm = false);

// Fields, Poisson and diagnostics (fields.cu).
int ensure_fields(pic_ctx* ctx);
int poisson_fft(pic_ctx* ctx);
int efield_from_phi(pic_ctx* ctx);
int diagnostics_async(pic_ctx* ctx);
int read_diagnostics(pic_ctx* ctx, pic_diag* d);
void release_fields(pic_ctx* ctx);
void release_rbgs(pic_ctx* ctx);
void release_current(pic_ctx* ctx);
// Deposit (deposit.cu).
int deposit_rho(pic_ctx* ctx, int scheme, double dt, double background);
// Red-black Gauss-Seidel pieces (rbgs.cu): right-hand side b = rho*dV - mean into
// the solver's buffer; r = b - A phi; the 5-point operator's coefficients; a
// solve from the phi in the context.
int rbgs_prepare(pic_ctx* ctx);
int rbgs_residual_field(pic_ctx* ctx, const double* phi, double* r);
void rbgs_operator(pic_ctx* ctx, double* ix2, double* iy2, double* denom);
int rbgs_solve(pic_ctx* ctx, double tol, int max_iters, int check_every, int* iters_out, double* resid_out);
// Exact solution of the 5-point system A phi = b (b with zero mean), by FFT with
// the operator's own eigenvalues (fields.cu).
int solve_discrete_fft(pic_ctx* ctx, const double* b, double* phi);
// Particle motion (push.cu).
int move(pic_ctx* ctx, double dt, bool gather, bool push);
void release_ws(pic_ctx* ctx);
// 1/d when d is a power of two (then x * (1/d) == x / d exactly), else 0.
double exact_reciprocal(double d);

// Brackets a kernel launch with profiling events when enabled.
void prof_begin(pic_ctx* ctx, const char* name);
void prof_end(pic_ctx* ctx);

}  // namespace picgb

#define PIC_CUDA_TRY(call)                                         \
    do {                                                           \
        cudaError_t e__ = (call);                                  \
        if (e__ != cudaSuccess) return picgb::cuda_fail(e__, #call); \
    } while (0)

#define PIC_TRY(expr)              \
    do {                           \
        int rc__ = (expr);         \
        if (rc__ != PIC_OK) return rc__; \
    } while (0)

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
namespace picgb {

__device__ __forceinline__ int wrap_i(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

// i mod n without a division when i lies within one period of [0, n) (a
// neighbour node or a move of at most one grid length); wrap_i otherwise.
__device__ __forceinline__ int wrap_near(int i, int n) {
    if (i >= n)
        i -= n;
    else if (i < 0)
        i += n;
    return (unsigned)i < (unsigned)n ? i : wrap_i(i, n);
}

// key = iy * n + ix split without an integer division: for key < 2^24 the FP32
// quotient key * (1/n) is within one of floor(key / n), and one correction
// step makes it exact; larger keys divide.
__device__ __forceinline__ void split_key(uint32_t key, int n, float inv_n, int& iy, int& ix) {
    if (key < (1u << 24)) {
        int q = (int)((float)key * inv_n);
        int r = (int)key - q * n;
        if (r < 0) {
            --q;
            r += n;
        } else if (r >= n) {
            ++q;
            r -= n;
        }
        iy = q;
        ix = r;
    } else {
        iy = (int)(key / (uint32_t)n);
        ix = (int)(key - (uint32_t)iy * (uint32_t)n);
    }
}

__device__ __forceinline__ void set_dev_error(DevStats* st, int code, unsigned int info) {
    if (atomicCAS(&st->err, 0, code) == 0) st->err_info = info;
}

__device__ __forceinline__ float load_maxq(const DevStats* st) { return __uint_as_float(st->maxq_bits); }

// CIC interpolation of a node field at cell offsets (wx, wy), in the
// reference's operation order (deposition.cpp:335-356); the build uses
// --fmad=false, so the oracle reproduces every bit.
__device__ __forceinline__ float interp_nodes(float e00, float e10, float e01, float e11, float wx, float wy) {
    const float omx = 1.0f - wx, omy = 1.0f - wy;
    return (((e00 * omx) * omy + (e10 * wx) * omy) + (e01 * omx) * wy) + (e11 * wx) * wy;
}
__device__ __forceinline__ float interp(const float* __restrict__ E, size_t i00, size_t i10, size_t i01, size_t i11,
                                        float wx, float wy) {
    return interp_nodes(__ldg(E + i00), __ldg(E + i10), __ldg(E + i01), __ldg(E + i11), wx, wy);
}

// x += v*dt/dx in cell-relative form: the integer part moves the cell index (wrapped).
__device__ __forceinline__ void drift(float& r, int& i, float v, float dtd, int n) {
    const float x = r + v * dtd;
    const float s = floorf(x);
    r = x - s;
    i = wrap_near(i + (int)s, n);
}

// Running double-FP32 sum (Knuth's two-sum) of the kinetic-energy partials.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float t) {
    const float s = __fadd_rn(hi, t);
    const float v = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, v)), __fsub_rn(t, v));
    hi = s;
    lo = __fadd_rn(lo, err);
}
// Adds vx^2 + vy^2 to a double-FP32 sum: exact FP32 squares (product and FMA error).
__device__ __forceinline__ void ke_add(float& hi, float& lo, float vx, float vy) {
    const float px = __fmul_rn(vx, vx), py = __fmul_rn(vy, vy);
    const float ex = __fmaf_rn(vx, vx, -px), ey = __fmaf_rn(vy, vy, -py);
    two_sum_acc(hi, lo, px);
    two_sum_acc(hi, lo, py);
    lo = __fadd_rn(lo, __fadd_rn(ex, ey));
}

// Domain::cellCoords (src/pic/domain.hpp:34-43) in FP64: w = x/dx, i = floor(w),
// frac = w - i, i wrapped. When dx is a power of two, x * (1/dx) equals the
// correctly rounded x/dx exactly and replaces the (slow) FP64 division. The
// FP32 offset keeps the NGP choice frac >= 0.5 (ngp.cpp:116-117) exact: a frac
// below 0.5 that rounds up to 0.5f is stored as the float just below 0.5.
__device__ __forceinline__ bool cell_coord(double x, double d, double inv_d, int n, int* idx, float* off) {
    const double w = inv_d != 0.0 ? __dmul_rn(x, inv_d) : __ddiv_rn(x, d);
    if (!(fabs(w) < 1073741824.0)) return false;  // also rejects NaN/inf
    const double f = floor(w);
    int i = (int)f;
    const double frac = __dsub_rn(w, (double)i);
    float r = __double2float_rn(frac);
    if (frac < 0.5 && r >= 0.5f) r = 0.49999997f;
    *idx = wrap_i(i, n);
    *off = r;
    return true;
}


// One unit of the int64 charge grid: max|q| * inv_vol * 2^-24 (FP64). The
// resident charge is stored normalised, qn = q / max|q|, and a particle carries
// rint(qn * 2^24) units.
__device__ __forceinline__ double charge_unit(const DevStats* st, double inv_vol) {
    return __dmul_rn(__dmul_rn((double)load_maxq(st), inv_vol), 5.9604644775390625e-08);
}

}  // namespace picgb
