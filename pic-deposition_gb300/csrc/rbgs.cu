// Red-black Gauss-Seidel Poisson solve (FP64).
//
// PoissonSolverGS::solve (src/pic/poisson_gs.cpp:11-61) is lexicographic,
// zeroes phi on every call and stops on max|dphi| < 1e-6. This solver keeps its
// 5-point stencil and sign, phi = ((phiW+phiE)/dx^2 + (phiS+phiN)/dy^2 + rho*dV)
// / (2(1/dx^2+1/dy^2)) (poisson_gs.cpp:32-38), and changes what a data-parallel
// solve with a learned warm start needs: red-black ordering (all points with (i+j) even, then odd; each
// colour is one data-parallel kernel), the right-hand side rho*dV with its mean
// removed (the periodic problem is singular), a warm start from the phi already
// in the context (the previous step's, or a learned guess), and the stop
// ||b - A phi||_2 / ||b||_2 <= tol checked every `check_every` sweeps. On exit
// phi has its mean removed and E is the forward difference of phi
// (poisson_gs.cpp:48-60). Multiplications by 1/dx^2, 1/dy^2 and 1/denom
// replace the reference's divisions (FP64 division is slow on this part); the
// oracle's restatement uses the same order of operations.
//
// Sums (mean, residual norms) use a fixed two-level tree, so results are
// identical run to run. Odd Nx or Ny is rejected: the colouring would not be a
// valid red-black split across the periodic seam.
#include <cstring>

#include "pic_internal.cuh"

namespace picgb {

constexpr int RB_THREADS = 256;
constexpr int RB_RED_BLOCKS = 1024;

struct RbArgs {
    double* phi;
    const double* b;
    int Nx, Ny;
    double ix2, iy2, inv_denom, denom;
};

__global__ void rbgs_half(RbArgs a, int color) {
    const int hx = a.Nx >> 1;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)hx * a.Ny) return;
    const int j = (int)(t / hx);
    const int i = 2 * (int)(t - (size_t)j * hx) + ((j + color) & 1);
    const int im = i == 0 ? a.Nx - 1 : i - 1, ip = i == a.Nx - 1 ? 0 : i + 1;
    const int jm = j == 0 ? a.Ny - 1 : j - 1, jp = j == a.Ny - 1 ? 0 : j + 1;
    const size_t id = (size_t)j * a.Nx + i;
    const double we = __dadd_rn(a.phi[(size_t)j * a.Nx + im], a.phi[(size_t)j * a.Nx + ip]);
    const double sn = __dadd_rn(a.phi[(size_t)jm * a.Nx + i], a.phi[(size_t)jp * a.Nx + i]);
    a.phi[id] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(we, a.ix2), __dmul_rn(sn, a.iy2)), a.b[id]), a.inv_denom);
}

__device__ __forceinline__ double rb_block_sum(double v) {
    __shared__ double ws[RB_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) ws[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < RB_THREADS / 32; ++w) s = __dadd_rn(s, ws[w]);
    __syncthreads();
    return s;
}

// partial[blk] = sum of rho*vol over a fixed chunk
__global__ void rb_sum_rhs(const double* __restrict__ rho, double vol, size_t g, double* __restrict__ partial) {
    const size_t chunk = (g + RB_RED_BLOCKS - 1) / RB_RED_BLOCKS;
    const size_t b = (size_t)blockIdx.x * chunk, e = b + chunk < g ? b + chunk : g;
    double s = 0.0;
    for (size_t i = b + threadIdx.x; i < e; i += RB_THREADS) s = __dadd_rn(s, __dmul_rn(rho[i], vol));
    const double t = rb_block_sum(s);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// partial[2*blk] = sum r^2, partial[2*blk+1] = sum b^2 with r = b - A phi
__global__ void rb_resid_partials(RbArgs a, double* __restrict__ partial) {
    const size_t g = (size_t)a.Nx * a.Ny;
    const size_t chunk = (g + RB_RED_BLOCKS - 1) / RB_RED_BLOCKS;
    const size_t b0 = (size_t)blockIdx.x * chunk, e = b0 + chunk < g ? b0 + chunk : g;
    double rr = 0.0, bb = 0.0;
    for (size_t id = b0 + threadIdx.x; id < e; id += RB_THREADS) {
        const int j = (int)(id / a.Nx), i = (int)(id - (size_t)j * a.Nx);
        const int im = i == 0 ? a.Nx - 1 : i - 1, ip = i == a.Nx - 1 ? 0 : i + 1;
        const int jm = j == 0 ? a.Ny - 1 : j - 1, jp = j == a.Ny - 1 ? 0 : j + 1;
        const double we = __dadd_rn(a.phi[(size_t)j * a.Nx + im], a.phi[(size_t)j * a.Nx + ip]);
        const double sn = __dadd_rn(a.phi[(size_t)jm * a.Nx + i], a.phi[(size_t)jp * a.Nx + i]);
        const double ap = __dsub_rn(__dsub_rn(__dmul_rn(a.denom, a.phi[id]), __dmul_rn(we, a.ix2)), __dmul_rn(sn, a.iy2));
        const double r = __dsub_rn(a.b[id], ap);
        rr = __dadd_rn(rr, __dmul_rn(r, r));
        bb = __dadd_rn(bb, __dmul_rn(a.b[id], a.b[id]));
    }
    const double t1 = rb_block_sum(rr);
    const double t2 = rb_block_sum(bb);
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = t1;
        partial[2 * blockIdx.x + 1] = t2;
    }
}

// out[0] = sum of partial[0..n) (stride `stride`, offset `off`)
__global__ void rb_final(const double* __restrict__ partial, int n, int stride, int off, double* out) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += RB_THREADS) s = __dadd_rn(s, partial[(size_t)i * stride + off]);
    const double t = rb_block_sum(s);
    if (threadIdx.x == 0) *out = t;
}

// b = rho*vol - mean, mean = sum / g
__global__ void rb_make_rhs(const double* __restrict__ rho, double vol, size_t g, const double* __restrict__ sum,
                            double* __restrict__ b) {
    const double mean = __ddiv_rn(*sum, (double)g);
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g) b[i] = __dsub_rn(__dmul_rn(rho[i], vol), mean);
}

__global__ void rb_sub_mean(double* __restrict__ phi, size_t g, const double* __restrict__ sum) {
    const double mean = __ddiv_rn(*sum, (double)g);
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g) phi[i] = __dsub_rn(phi[i], mean);
}

static int ensure_rbgs(pic_ctx* c) {
    PIC_TRY(ensure_fields(c));
    int rc = PIC_OK;
    if (!c->rb_b) c->rb_b = (double*)dalloc(c->G * 8, &rc);
    if (rc) return rc;
    if (!c->rb_partial) c->rb_partial = (double*)dalloc(2 * RB_RED_BLOCKS * 8, &rc);
    if (rc) return rc;
    if (!c->rb_scalars) c->rb_scalars = (double*)dalloc(8 * 8, &rc);
    return rc;
}

static RbArgs rb_args(pic_ctx* c) {
    RbArgs a;
    a.phi = c->phi;
    a.b = c->rb_b;
    a.Nx = c->Nx;
    a.Ny = c->Ny;
    const double dx2 = c->dx * c->dx, dy2 = c->dy * c->dy;
    a.ix2 = 1.0 / dx2;
    a.iy2 = 1.0 / dy2;
    a.denom = 2.0 * (1.0 / dx2 + 1.0 / dy2);
    a.inv_denom = 1.0 / a.denom;
    return a;
}

static int rb_sweeps(pic_ctx* c, const RbArgs& a, int n) {
    const size_t half = (size_t)(c->Nx / 2) * c->Ny;
    const unsigned blocks = (unsigned)((half + RB_THREADS - 1) / RB_THREADS);
    for (int s = 0; s < n; ++s) {
        rbgs_half<<<blocks, RB_THREADS, 0, c->stream>>>(a, 0);
        PIC_TRY(check_launch(c, "rbgs_half"));
        rbgs_half<<<blocks, RB_THREADS, 0, c->stream>>>(a, 1);
        PIC_TRY(check_launch(c, "rbgs_half"));
    }
    return PIC_OK;
}

static int rb_residual_async(pic_ctx* c, const RbArgs& a) {
    rb_resid_partials<<<RB_RED_BLOCKS, RB_THREADS, 0, c->stream>>>(a, c->rb_partial);
    PIC_TRY(check_launch(c, "rb_resid_partials"));
    rb_final<<<1, RB_THREADS, 0, c->stream>>>(c->rb_partial, RB_RED_BLOCKS, 2, 0, c->rb_scalars + 1);
    PIC_TRY(check_launch(c, "rb_final"));
    rb_final<<<1, RB_THREADS, 0, c->stream>>>(c->rb_partial, RB_RED_BLOCKS, 2, 1, c->rb_scalars + 2);
    return check_launch(c, "rb_final");
}

// rhs b = rho*dV - mean into c->rb_b (queued).
static int rb_prepare(pic_ctx* c) {
    const unsigned blocks = (unsigned)((c->G + 255) / 256);
    rb_sum_rhs<<<RB_RED_BLOCKS, RB_THREADS, 0, c->stream>>>(c->rho, c->dx * c->dy, c->G, c->rb_partial);
    PIC_TRY(check_launch(c, "rb_sum_rhs"));
    rb_final<<<1, RB_THREADS, 0, c->stream>>>(c->rb_partial, RB_RED_BLOCKS, 1, 0, c->rb_scalars);
    PIC_TRY(check_launch(c, "rb_final"));
    rb_make_rhs<<<blocks, 256, 0, c->stream>>>(c->rho, c->dx * c->dy, c->G, c->rb_scalars, c->rb_b);
    return check_launch(c, "rb_make_rhs");
}

static int rb_finish(pic_ctx* c) {
    const unsigned blocks = (unsigned)((c->G + 255) / 256);
    rb_sum_rhs<<<RB_RED_BLOCKS, RB_THREADS, 0, c->stream>>>(c->phi, 1.0, c->G, c->rb_partial);
    PIC_TRY(check_launch(c, "rb_sum_rhs"));
    rb_final<<<1, RB_THREADS, 0, c->stream>>>(c->rb_partial, RB_RED_BLOCKS, 1, 0, c->rb_scalars + 3);
    PIC_TRY(check_launch(c, "rb_final"));
    rb_sub_mean<<<blocks, 256, 0, c->stream>>>(c->phi, c->G, c->rb_scalars + 3);
    PIC_TRY(check_launch(c, "rb_sub_mean"));
    return efield_from_phi(c);
}

// ---- one cooperative launch per solve ---------------------------------------
// Each CTA owns a tw x th tile of phi and keeps it, with a halo of PS_HALO
// cells and the matching piece of b, in shared memory. Between two exchanges it
// performs PS_HALO half-sweeps (two full red-black sweeps) on its extended
// tile, the updated region shrinking by one cell per half-sweep, so the owned
// cells end with exactly the values the one-launch-per-colour path computes
// (same update, same operation order, same colour order). Then it writes its
// owned cells back, waits at a grid-wide barrier and reloads its halo. The
// residual is checked every check_every sweeps: per-CTA sums of r^2 and b^2,
// a barrier, and every CTA adds the partials in index order and takes the
// same decision. Barriers give up after about one second (PIC_ERR_TIMEOUT).
constexpr int PS_THREADS = RB_THREADS;
constexpr int PS_HALO = 4;
constexpr int PS_MAX_BLOCKS = 4096;
constexpr unsigned long long PS_WAIT_NS = 1000000000ull;

struct PsArgs {
    RbArgs a;
    int tw, th, tiles_x, ew, eh;
    double tol;
    int max_iters, check_every;
    double* partial;  // [2 * blocks]
    unsigned* bar;    // [0] arrivals, [1] generation
    int* err;
    double* out;      // [0] sweeps, [1] residual, [2] first residual
    int absent_block; // -1, or a CTA that leaves at once (the timeout test hook)
    unsigned long long wait_ns;  // limit of one barrier wait
};

__device__ __forceinline__ uint64_t ps_time_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ bool ps_barrier(unsigned* bar, int* err, unsigned long long wait_ns = PS_WAIT_NS) {
    __syncthreads();
    __shared__ int ok;
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned* vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const uint64_t t0 = ps_time_ns();
            while (*vgen == gen)
                if (ps_time_ns() - t0 > wait_ns) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ int ps_wrap(int i, int n) {
    const int r = i % n;
    return r < 0 ? r + n : r;
}

__global__ void __launch_bounds__(PS_THREADS) rbgs_persistent(PsArgs p) {
    extern __shared__ double psm[];
    const int E = p.ew * p.eh;
    double* sphi = psm;
    double* sb = psm + E;
    __shared__ double tot[2];
    const RbArgs& a = p.a;
    if ((int)blockIdx.x == p.absent_block) return;
    const int tx = blockIdx.x % p.tiles_x, ty = blockIdx.x / p.tiles_x;
    const int ox = tx * p.tw - PS_HALO, oy = ty * p.th - PS_HALO;
    for (int i = threadIdx.x; i < E; i += PS_THREADS) {
        const int ly = i / p.ew, lx = i - ly * p.ew;
        const size_t g = (size_t)ps_wrap(oy + ly, a.Ny) * a.Nx + ps_wrap(ox + lx, a.Nx);
        sb[i] = a.b[g];
        sphi[i] = a.phi[g];
    }
    __syncthreads();
    const int nown = p.tw * p.th;
    double bb = 0.0;
    for (int t = threadIdx.x; t < nown; t += PS_THREADS) {
        const int i = (PS_HALO + t / p.tw) * p.ew + PS_HALO + t % p.tw;
        bb = __dadd_rn(bb, __dmul_rn(sb[i], sb[i]));
    }
    bb = rb_block_sum(bb);
    if (threadIdx.x == 0) p.partial[2 * blockIdx.x + 1] = bb;
    int it = 0;
    double res = 0.0, res0 = -1.0;
    for (;;) {
        if (it % p.check_every == 0 || it >= p.max_iters) {
            double rr = 0.0;
            for (int t = threadIdx.x; t < nown; t += PS_THREADS) {
                const int i = (PS_HALO + t / p.tw) * p.ew + PS_HALO + t % p.tw;
                const double we = __dadd_rn(sphi[i - 1], sphi[i + 1]);
                const double sn = __dadd_rn(sphi[i - p.ew], sphi[i + p.ew]);
                const double ap = __dsub_rn(__dsub_rn(__dmul_rn(a.denom, sphi[i]), __dmul_rn(we, a.ix2)),
                                            __dmul_rn(sn, a.iy2));
                const double r = __dsub_rn(sb[i], ap);
                rr = __dadd_rn(rr, __dmul_rn(r, r));
            }
            rr = rb_block_sum(rr);
            if (threadIdx.x == 0) p.partial[2 * blockIdx.x] = rr;
            if (!ps_barrier(p.bar, p.err, p.wait_ns)) break;
            if (threadIdx.x == 0) {
                double s1 = 0.0, s2 = 0.0;
                for (unsigned k = 0; k < gridDim.x; ++k) {
                    s1 = __dadd_rn(s1, p.partial[2 * k]);
                    s2 = __dadd_rn(s2, p.partial[2 * k + 1]);
                }
                tot[0] = s1;
                tot[1] = s2;
            }
            __syncthreads();
            res = tot[1] > 0.0 ? sqrt(tot[0] / tot[1]) : sqrt(tot[0]);
            if (res0 < 0.0) res0 = res;
            if (res <= p.tol || it >= p.max_iters) break;
        }
        for (int k = 0; k < PS_HALO; ++k) {
            const int color = k & 1;
            const int lo = k + 1;
            const int rows = p.eh - 2 * lo, cols = p.ew - 2 * lo;
            const int half = (cols + 1) >> 1;
            for (int t = threadIdx.x; t < rows * half; t += PS_THREADS) {
                const int r = t / half, m = t - r * half;
                const int ly = lo + r;
                const int lx = lo + (((ox + lo + oy + ly) & 1) ^ color) + 2 * m;
                if (lx >= p.ew - lo) continue;
                const int i = ly * p.ew + lx;
                const double we = __dadd_rn(sphi[i - 1], sphi[i + 1]);
                const double sn = __dadd_rn(sphi[i - p.ew], sphi[i + p.ew]);
                sphi[i] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(we, a.ix2), __dmul_rn(sn, a.iy2)), sb[i]),
                                    a.inv_denom);
            }
            __syncthreads();
        }
        it += PS_HALO / 2;
        for (int t = threadIdx.x; t < nown; t += PS_THREADS) {
            const int ly = PS_HALO + t / p.tw, lx = PS_HALO + t % p.tw;
            a.phi[(size_t)(oy + ly) * a.Nx + (ox + lx)] = sphi[ly * p.ew + lx];
        }
        if (!ps_barrier(p.bar, p.err, p.wait_ns)) break;
        for (int i = threadIdx.x; i < E; i += PS_THREADS) {
            const int ly = i / p.ew, lx = i - ly * p.ew;
            if (ly >= PS_HALO && ly < PS_HALO + p.th && lx >= PS_HALO && lx < PS_HALO + p.tw) continue;
            sphi[i] = a.phi[(size_t)ps_wrap(oy + ly, a.Ny) * a.Nx + ps_wrap(ox + lx, a.Nx)];
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        p.out[0] = (double)it;
        p.out[1] = res;
        p.out[2] = res0;
    }
}

static int largest_divisor_tile(int n, const int* cand, int ncand) {
    for (int k = 0; k < ncand; ++k)
        if (cand[k] <= n && n % cand[k] == 0) return cand[k];
    return 0;
}

// Solves in one cooperative launch when the grid tiles evenly and every CTA can
// be resident; returns PIC_ERR_UNSUPPORTED (nothing queued) otherwise.
// absent_block >= 0 makes that CTA leave before its first barrier, so that every
// other CTA's wait runs out after wait_ns (the timeout test hook; -1 in solves).
static int rbgs_solve_persistent(pic_ctx* c, const RbArgs& a, double tol, int max_iters, int check_every, int* it,
                                 double* res, int absent_block = -1, unsigned long long wait_ns = PS_WAIT_NS) {
    if ((check_every & 1) || (max_iters & 1)) return PIC_ERR_UNSUPPORTED;
    static const int cw[] = {64, 32, 16, 8, 4, 2};
    static const int ch[] = {32, 16, 8, 4, 2};
    const int tw = largest_divisor_tile(c->Nx, cw, 6), th = largest_divisor_tile(c->Ny, ch, 5);
    if (!tw || !th) return PIC_ERR_UNSUPPORTED;
    const int tiles_x = c->Nx / tw, blocks = tiles_x * (c->Ny / th);
    const int ew = tw + 2 * PS_HALO, eh = th + 2 * PS_HALO;
    const size_t smem = (size_t)2 * ew * eh * sizeof(double);
    if (blocks > PS_MAX_BLOCKS || smem > 200 * 1024) return PIC_ERR_UNSUPPORTED;
    if (smem > 48 * 1024 && opt_in_dynamic_smem((const void*)rbgs_persistent, smem) != PIC_OK)
        return PIC_ERR_UNSUPPORTED;
    int per_sm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rbgs_persistent, PS_THREADS, smem);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    if (per_sm * sms < blocks) return PIC_ERR_UNSUPPORTED;
    int rc = PIC_OK;
    if (!c->rb_ps) c->rb_ps = (double*)dalloc((2 * PS_MAX_BLOCKS + 8) * sizeof(double), &rc);
    if (rc) return rc;
    double* out = c->rb_ps + 2 * PS_MAX_BLOCKS;
    unsigned* bar = reinterpret_cast<unsigned*>(out + 4);
    int* err = reinterpret_cast<int*>(out + 5);
    PIC_CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), c->stream));
    PIC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
    PsArgs p{a,   tw,  th,  tiles_x, ew,  eh,           tol,    max_iters,
             check_every, c->rb_ps, bar, err,     out, absent_block, wait_ns};
    cudaLaunchConfig_t lc{};
    lc.gridDim = dim3(blocks);
    lc.blockDim = dim3(PS_THREADS);
    lc.dynamicSmemBytes = smem;
    lc.stream = c->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    PIC_CUDA_TRY(cudaLaunchKernelEx(&lc, rbgs_persistent, p));
    c->launches++;
    double h[6];
    PIC_CUDA_TRY(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    int herr = 0;
    std::memcpy(&herr, &h[5], sizeof(int));
    if (herr) return fail(PIC_ERR_TIMEOUT, "red-black Gauss-Seidel: a grid-wide barrier timed out");
    *it = (int)h[0];
    *res = h[1];
    c->first_rbgs_resid = h[2];
    return PIC_OK;
}

// ---- mixed precision: FP32 sweeps on the correction, FP64 residual --------
// Iterative refinement: r = b - A phi in FP64; A e = r is relaxed in FP32 by the
// same red-black sweeps (one cooperative launch, 8-cell halo, 4 sweeps per grid
// barrier) until ||r - A e|| <= itol ||r||; phi += e in FP64; repeat until the
// FP64 relative residual meets tol. The answer meets the same FP64 test as the
// FP64 solve; sweeps are counted over all corrections.
constexpr int PF_HALO = 8;

__global__ void rb_residual_field(RbArgs a, const double* __restrict__ phi, double* __restrict__ r);

struct PsArgsF {
    float* e;        // correction (in/out)
    const float* r;  // right-hand side of the correction
    int Nx, Ny;
    float ix2, iy2, inv_denom, denom;
    int tw, th, tiles_x, ew, eh;
    float itol;
    int max_sweeps, check_every;
    double* partial;
    unsigned* bar;
    int* err;
    double* out;  // [0] sweeps
};

__global__ void __launch_bounds__(PS_THREADS) rbgs_persistent_f32(PsArgsF p) {
    extern __shared__ float pfm[];
    const int E = p.ew * p.eh;
    float* se = pfm;
    float* sr = pfm + E;
    __shared__ double tot[2];
    const int tx = blockIdx.x % p.tiles_x, ty = blockIdx.x / p.tiles_x;
    const int ox = tx * p.tw - PF_HALO, oy = ty * p.th - PF_HALO;
    for (int i = threadIdx.x; i < E; i += PS_THREADS) {
        const int ly = i / p.ew, lx = i - ly * p.ew;
        const size_t g = (size_t)ps_wrap(oy + ly, p.Ny) * p.Nx + ps_wrap(ox + lx, p.Nx);
        sr[i] = p.r[g];
        se[i] = p.e[g];
    }
    __syncthreads();
    const int nown = p.tw * p.th;
    double rr0 = 0.0;
    for (int t = threadIdx.x; t < nown; t += PS_THREADS) {
        const int i = (PF_HALO + t / p.tw) * p.ew + PF_HALO + t % p.tw;
        rr0 += (double)sr[i] * (double)sr[i];
    }
    rr0 = rb_block_sum(rr0);
    if (threadIdx.x == 0) p.partial[2 * blockIdx.x + 1] = rr0;
    int it = 0;
    double prev = 1e300;
    for (;;) {
        if (it % p.check_every == 0 || it >= p.max_sweeps) {
            double rr = 0.0;
            for (int t = threadIdx.x; t < nown; t += PS_THREADS) {
                const int i = (PF_HALO + t / p.tw) * p.ew + PF_HALO + t % p.tw;
                const float ae = p.denom * se[i] - p.ix2 * (se[i - 1] + se[i + 1]) - p.iy2 * (se[i - p.ew] + se[i + p.ew]);
                const double q = (double)(sr[i] - ae);
                rr += q * q;
            }
            rr = rb_block_sum(rr);
            if (threadIdx.x == 0) p.partial[2 * blockIdx.x] = rr;
            if (!ps_barrier(p.bar, p.err)) break;
            if (threadIdx.x == 0) {
                double s1 = 0.0, s2 = 0.0;
                for (unsigned k = 0; k < gridDim.x; ++k) {
                    s1 += p.partial[2 * k];
                    s2 += p.partial[2 * k + 1];
                }
                tot[0] = s1;
                tot[1] = s2;
            }
            __syncthreads();
            const double res = tot[1] > 0.0 ? sqrt(tot[0] / tot[1]) : 0.0;
            // stop at the tolerance, the sweep limit, or when FP32 rounding stalls the residual
            if (res <= (double)p.itol || it >= p.max_sweeps || res > 0.999 * prev) break;
            prev = res;
        }
        for (int k = 0; k < PF_HALO; ++k) {
            const int color = k & 1;
            const int lo = k + 1;
            const int rows = p.eh - 2 * lo, cols = p.ew - 2 * lo;
            const int half = (cols + 1) >> 1;
            for (int t = threadIdx.x; t < rows * half; t += PS_THREADS) {
                const int rw = t / half, m = t - rw * half;
                const int ly = lo + rw;
                const int lx = lo + (((ox + lo + oy + ly) & 1) ^ color) + 2 * m;
                if (lx >= p.ew - lo) continue;
                const int i = ly * p.ew + lx;
                se[i] = ((se[i - 1] + se[i + 1]) * p.ix2 + (se[i - p.ew] + se[i + p.ew]) * p.iy2 + sr[i]) * p.inv_denom;
            }
            __syncthreads();
        }
        it += PF_HALO / 2;
        for (int t = threadIdx.x; t < nown; t += PS_THREADS) {
            const int ly = PF_HALO + t / p.tw, lx = PF_HALO + t % p.tw;
            p.e[(size_t)(oy + ly) * p.Nx + (ox + lx)] = se[ly * p.ew + lx];
        }
        if (!ps_barrier(p.bar, p.err)) break;
        for (int i = threadIdx.x; i < E; i += PS_THREADS) {
            const int ly = i / p.ew, lx = i - ly * p.ew;
            if (ly >= PF_HALO && ly < PF_HALO + p.th && lx >= PF_HALO && lx < PF_HALO + p.tw) continue;
            se[i] = p.e[(size_t)ps_wrap(oy + ly, p.Ny) * p.Nx + ps_wrap(ox + lx, p.Nx)];
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) p.out[0] = (double)it;
}

__global__ void rb_to_f32(const double* __restrict__ r, size_t n, float* __restrict__ r32, float* __restrict__ e) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        r32[i] = __double2float_rn(r[i]);
        e[i] = 0.0f;
    }
}

__global__ void rb_add_correction(double* __restrict__ phi, const float* __restrict__ e, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) phi[i] = __dadd_rn(phi[i], (double)e[i]);
}

// The mixed-precision solve; PIC_ERR_UNSUPPORTED (nothing queued) when the
// grid does not tile evenly or the tiles cannot all be resident.
static int rbgs_solve_mixed(pic_ctx* c, const RbArgs& a, double tol, int max_iters, int check_every, int* it_out,
                            double* res_out) {
    static const int cw[] = {64, 32, 16, 8, 4, 2};
    static const int ch[] = {32, 16, 8, 4, 2};
    const int tw = largest_divisor_tile(c->Nx, cw, 6), th = largest_divisor_tile(c->Ny, ch, 5);
    if (!tw || !th) return PIC_ERR_UNSUPPORTED;
    const int tiles_x = c->Nx / tw, blocks = tiles_x * (c->Ny / th);
    const int ew = tw + 2 * PF_HALO, eh = th + 2 * PF_HALO;
    const size_t smem = (size_t)2 * ew * eh * sizeof(float);
    if (blocks > PS_MAX_BLOCKS || smem > 48 * 1024) return PIC_ERR_UNSUPPORTED;
    int per_sm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rbgs_persistent_f32, PS_THREADS, smem);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    if (per_sm * sms < blocks) return PIC_ERR_UNSUPPORTED;
    int rc = PIC_OK;
    if (!c->rb_ps) c->rb_ps = (double*)dalloc((2 * PS_MAX_BLOCKS + 8) * sizeof(double), &rc);
    if (rc) return rc;
    if (!c->rb_mix) c->rb_mix = (double*)dalloc(c->G * (8 + 4 + 4), &rc);
    if (rc) return rc;
    double* r64 = c->rb_mix;
    float* r32 = reinterpret_cast<float*>(r64 + c->G);
    float* e32 = r32 + c->G;
    double* out = c->rb_ps + 2 * PS_MAX_BLOCKS;
    unsigned* bar = reinterpret_cast<unsigned*>(out + 4);
    int* err = reinterpret_cast<int*>(out + 5);
    PIC_CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), c->stream));
    PIC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
    const unsigned gb = (unsigned)((c->G + 255) / 256);
    const int ce = check_every < 4 ? 4 : (check_every / 4) * 4;
    int it = 0;
    double res = 0.0, prev_res = 0.0;
    for (int outer = 0;; ++outer) {
        PIC_TRY(rb_residual_async(c, a));
        double s[3];
        PIC_CUDA_TRY(cudaMemcpyAsync(s, c->rb_scalars, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
        PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        res = s[2] > 0.0 ? std::sqrt(s[1] / s[2]) : std::sqrt(s[1]);
        if (outer == 0) c->first_rbgs_resid = res;
        if (res <= tol || it >= max_iters) break;
        rb_residual_field<<<gb, 256, 0, c->stream>>>(a, c->phi, r64);
        PIC_TRY(check_launch(c, "rb_residual_field"));
        rb_to_f32<<<gb, 256, 0, c->stream>>>(r64, c->G, r32, e32);
        PIC_TRY(check_launch(c, "rb_to_f32"));
        // reduce the residual by what is left to reach tol; FP32 rounding of the
        // correction limits one pass to about cond(A) * 2^-24 of the residual, so a
        // pass aims at 1e-2 at most and the passes repeat
        double itol = 0.5 * tol / res;
        if (itol < 1e-2) itol = 1e-2;
        if (itol > 0.5) itol = 0.5;
        if (outer > 0 && res > 0.5 * prev_res) {  // a pass that no longer helps: finish in FP64
            int it64 = 0;
            double r64v = 0.0;
            const double first = c->first_rbgs_resid;
            const int prc = rbgs_solve_persistent(c, a, tol, (max_iters - it) & ~1, check_every & ~1 ? check_every & ~1 : 2,
                                                  &it64, &r64v);
            c->first_rbgs_resid = first;
            if (prc == PIC_OK) {
                it += it64;
                res = r64v;
                break;
            }
            if (prc != PIC_ERR_UNSUPPORTED) return prc;
        }
        prev_res = res;
        PsArgsF p{e32, r32, c->Nx, c->Ny, (float)a.ix2, (float)a.iy2, (float)a.inv_denom, (float)a.denom,
                  tw, th, tiles_x, ew, eh, (float)itol, max_iters - it, ce, c->rb_ps, bar, err, out};
        cudaLaunchConfig_t lc{};
        lc.gridDim = dim3(blocks);
        lc.blockDim = dim3(PS_THREADS);
        lc.dynamicSmemBytes = smem;
        lc.stream = c->stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        lc.attrs = at;
        lc.numAttrs = 1;
        PIC_CUDA_TRY(cudaLaunchKernelEx(&lc, rbgs_persistent_f32, p));
        c->launches += 3;
        rb_add_correction<<<gb, 256, 0, c->stream>>>(c->phi, e32, c->G);
        PIC_TRY(check_launch(c, "rb_add_correction"));
        double h[6];
        PIC_CUDA_TRY(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        int herr = 0;
        std::memcpy(&herr, &h[5], sizeof(int));
        if (herr) return fail(PIC_ERR_TIMEOUT, "red-black Gauss-Seidel: a grid-wide barrier timed out");
        const int sw = (int)h[0];
        it += sw > 0 ? sw : 1;  // a pass that made no sweep still counts, so the loop ends
    }
    *it_out = it;
    *res_out = res;
    return PIC_OK;
}

// Solves with the residual checked every `check_every` sweeps: in one
// cooperative launch where possible, else one launch per colour with the
// residual read on the host; with the mixed-precision option, FP32 sweeps on
// FP64-refined corrections.
int rbgs_solve(pic_ctx* c, double tol, int max_iters, int check_every, int* iters_out, double* resid_out) {
    if ((c->Nx & 1) || (c->Ny & 1)) return fail(PIC_ERR_UNSUPPORTED, "red-black Gauss-Seidel needs even Nx and Ny");
    if (max_iters < 0) return fail(PIC_ERR_ARG, "max_iters < 0");
    if (check_every < 1) check_every = 1;
    PIC_TRY(ensure_rbgs(c));
    PIC_TRY(rb_prepare(c));
    const RbArgs a = rb_args(c);
    int it = 0;
    double res = 0.0;
    prof_begin(c, "rbgs");
    int prc = PIC_ERR_UNSUPPORTED;
    if (c->rbgs_mixed) prc = rbgs_solve_mixed(c, a, tol, max_iters, check_every, &it, &res);
    if (prc == PIC_ERR_UNSUPPORTED && c->rbgs_persistent)
        prc = rbgs_solve_persistent(c, a, tol, max_iters, check_every, &it, &res);
    if (prc != PIC_OK && prc != PIC_ERR_UNSUPPORTED) {
        prof_end(c);
        return prc;
    }
    for (; prc == PIC_ERR_UNSUPPORTED;) {
        PIC_TRY(rb_residual_async(c, a));
        double s[3];
        PIC_CUDA_TRY(cudaMemcpyAsync(s, c->rb_scalars, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
        PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        res = s[2] > 0.0 ? std::sqrt(s[1] / s[2]) : std::sqrt(s[1]);
        if (it == 0) c->first_rbgs_resid = res;
        if (res <= tol || it >= max_iters) break;
        const int n = (max_iters - it) < check_every ? (max_iters - it) : check_every;
        PIC_TRY(rb_sweeps(c, a, n));
        it += n;
    }
    prof_end(c);
    PIC_TRY(rb_finish(c));
    if (iters_out) *iters_out = it;
    if (resid_out) *resid_out = res;
    c->last_rbgs_iters = it;
    c->last_rbgs_resid = res;
    return PIC_OK;
}

// r = b - A phi for the right-hand side prepared by rbgs_prepare.
__global__ void rb_residual_field(RbArgs a, const double* __restrict__ phi, double* __restrict__ r) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)a.Nx * a.Ny) return;
    const int j = (int)(id / a.Nx), i = (int)(id - (size_t)j * a.Nx);
    const int im = i == 0 ? a.Nx - 1 : i - 1, ip = i == a.Nx - 1 ? 0 : i + 1;
    const int jm = j == 0 ? a.Ny - 1 : j - 1, jp = j == a.Ny - 1 ? 0 : j + 1;
    const double we = __dadd_rn(phi[(size_t)j * a.Nx + im], phi[(size_t)j * a.Nx + ip]);
    const double sn = __dadd_rn(phi[(size_t)jm * a.Nx + i], phi[(size_t)jp * a.Nx + i]);
    const double ap = __dsub_rn(__dsub_rn(__dmul_rn(a.denom, phi[id]), __dmul_rn(we, a.ix2)), __dmul_rn(sn, a.iy2));
    r[id] = __dsub_rn(a.b[id], ap);
}

int rbgs_prepare(pic_ctx* c) {
    if ((c->Nx & 1) || (c->Ny & 1)) return fail(PIC_ERR_UNSUPPORTED, "red-black Gauss-Seidel needs even Nx and Ny");
    PIC_TRY(ensure_rbgs(c));
    return rb_prepare(c);
}

int rbgs_residual_field(pic_ctx* c, const double* phi, double* r) {
    const RbArgs a = rb_args(c);
    rb_residual_field<<<(unsigned)((c->G + 255) / 256), 256, 0, c->stream>>>(a, phi, r);
    return check_launch(c, "rb_residual_field");
}

void rbgs_operator(pic_ctx* c, double* ix2, double* iy2, double* denom) {
    const RbArgs a = rb_args(c);
    *ix2 = a.ix2;
    *iy2 = a.iy2;
    *denom = a.denom;
}

int rbgs_solve_async(pic_ctx* c, double tol, int max_iters, int check_every) {
    return rbgs_solve(c, tol, max_iters, check_every, nullptr, nullptr);
}

void release_rbgs(pic_ctx* c) {
    dfree(c->rb_mix);
    dfree(c->rb_ps);
    dfree(c->rb_b);
    dfree(c->rb_partial);
    dfree(c->rb_scalars);
}

}  // namespace picgb

using namespace picgb;

extern "C" int pic_gpu_set_rbgs_precision(pic_ctx* c, int mixed) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    if (mixed != 0 && mixed != 1) return fail(PIC_ERR_ARG, "precision must be 0 (FP64) or 1 (mixed)");
    c->rbgs_mixed = mixed;
    return PIC_OK;
}

// Runs the persistent FP64 solve on the context's rho with CTA `absent_block`
// leaving at once and every barrier wait limited to wait_ms: the other CTAs give
// up, set the error flag and return, and the call reports PIC_ERR_TIMEOUT.
extern "C" int pic_gpu_test_rbgs_barrier_timeout(pic_ctx* c, int absent_block, double wait_ms) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    if (absent_block < -1) return fail(PIC_ERR_ARG, "absent_block < -1");
    if (!(wait_ms > 0.0 && wait_ms <= 1000.0)) return fail(PIC_ERR_ARG, "wait_ms must be in (0, 1000]");
    if ((c->Nx & 1) || (c->Ny & 1)) return fail(PIC_ERR_UNSUPPORTED, "red-black Gauss-Seidel needs even Nx and Ny");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    PIC_TRY(ensure_fields(c));
    PIC_TRY(ensure_rbgs(c));
    PIC_TRY(rb_prepare(c));
    PIC_CUDA_TRY(cudaMemsetAsync(c->phi, 0, c->G * 8, c->stream));
    const RbArgs a = rb_args(c);
    int it = 0;
    double res = 0.0;
    const int rc = rbgs_solve_persistent(c, a, 0.0, 64, 2, &it, &res, absent_block,
                                         (unsigned long long)(wait_ms * 1e6));
    if (rc == PIC_ERR_UNSUPPORTED) return fail(rc, "the grid does not fit one cooperative launch");
    if (rc != PIC_OK) return rc;
    return pic_gpu_synchronize(c);
}

extern "C" int pic_gpu_poisson_rbgs(pic_ctx* c, double tol, int max_iters, int warm_start, int check_every,
                                    int* iters_out, double* resid_out) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    PIC_TRY(ensure_fields(c));
    if (!warm_start) PIC_CUDA_TRY(cudaMemsetAsync(c->phi, 0, c->G * 8, c->stream));
    PIC_TRY(rbgs_solve(c, tol, max_iters, check_every, iters_out, resid_out));
    return pic_gpu_synchronize(c);
}
