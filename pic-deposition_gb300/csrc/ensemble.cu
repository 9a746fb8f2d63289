// Batched ensemble: many independent electrostatic runs with uneven grid sizes
// and particle counts advanced together.
//
// Layout. The runs' grids are laid end to end in one global cell space: run r
// owns keys [cell_base_r, cell_base_r + N_r^2), row-major inside (key =
// cell_base_r + iy*N_r + ix, unit cells, dx = dy = 1). All particles live in one
// SoA set (a pic_ctx whose "grid" is the global cell space, so the library's
// radix sort and per-cell offsets work unchanged); a run's particles occupy a
// fixed index range because keys of different runs never interleave and the
// sort is stable. Fields (rho, phi, E, the int64 charge grid) are global arrays
// over the same cell space.
//
// One step (every run): gather + push, [cell sort], CIC deposit in fixed point,
// + background, FFT Poisson per run, E. The particle work of a step is ONE
// persistent cooperative launch (ens_step_kernel): phase 1 moves every particle
// of every run, a grid-wide barrier, phase 2 deposits them (the run-aggregating
// warp step: 4 consecutive particles per lane, register sums per cell,
// segmented warp scan, one int64 atomic per run of equal cells), a barrier,
// phase 3 turns the int64 grid into rho (+ background) and clears it. The
// Poisson solves are one batched cuFFT plan per grid size (runs sorted by
// size, so equal sizes are contiguous) plus two small kernels. With use_graph
// the whole step is one CUDA graph. Steps with a cell sort run the move, the
// sort, a tiled deposit and the conversion as separate launches; the tiled
// deposit's tile shape per (grid size, particles per cell) class is picked by
// timing candidate shapes on the first sorted step (the autotuner).
//
// Every arithmetic operation on a particle or a cell is the one the single-run
// path performs (push.cu, deposit.cu, fields.cu), so each run's particles and
// fields equal, bit for bit, those of the same run advanced alone.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

#include "philox.cuh"
#include "pic_internal.cuh"

namespace picgb {

int ensure_fields(pic_ctx* c);

namespace {

constexpr int ENS_THREADS = 256;
constexpr int ENS_WARPS = ENS_THREADS / 32;
constexpr int MAX_RUNS = 256;
constexpr unsigned FULLM = 0xffffffffu;
constexpr uint32_t NO_KEY = 0xffffffffu;

struct RunDesc {
    uint32_t cell_base;  // first global key
    uint32_t cells;      // N*N
    uint32_t pbase;      // first particle
    uint32_t np;         // particles
    uint32_t tile_base;  // first CTA of the run in the tiled deposit
    uint32_t en_base;    // first block of the run in the energy sums
    uint32_t en_blocks;  // blocks of the run in the energy sums
    int N;
    int tile_w, tile_h, tiles_x;
    float maxq;          // |q| of the run's particles
    float coef;          // -(q/m) of the run's particles, FP32 as the gather computes it
    double unit;         // one int64 unit: maxq * inv_vol * 2^-24
    double background;
};

struct StepArgs {
    const RunDesc* runs;
    int nruns;
    uint32_t* cell;
    float *xr, *yr, *vx, *vy;
    const float* q;
    const float* Exf;
    const float* Eyf;
    unsigned long long* acc;
    double* rho;
    size_t n;
    uint32_t G;
    float dtf, dtd;
    unsigned* bar;   // [0] arrivals, [1] generation
    int* err;
    int do_move, do_deposit, do_convert;
    unsigned long long* breaks;  // moved particles out of cell order (adjacent pairs), or null
};

__device__ __forceinline__ uint64_t gtime_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for a cooperative launch (all CTAs resident). Gives up
// after about one second and records an error; returns false then.
__device__ bool grid_barrier(unsigned* bar, int* err) {
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
            const uint64_t t0 = gtime_ns();
            while (*vgen == gen) {
                if (gtime_ns() - t0 > 1000000000ull) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Index of the run whose range [base[i], base[i+1]) holds v (binary search over
// `nruns` sorted bases held in shared memory).
__device__ __forceinline__ int find_run(const uint32_t* base, int nruns, uint32_t v) {
    int lo = 0, hi = nruns - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ float interp_f(const float* __restrict__ E, size_t i00, size_t i10, size_t i01, size_t i11,
                                          float wx, float wy) {
    const float omx = 1.0f - wx, omy = 1.0f - wy;
    return (((__ldg(E + i00) * omx) * omy + (__ldg(E + i10) * wx) * omy) + (__ldg(E + i01) * omx) * wy) +
           (__ldg(E + i11) * wx) * wy;
}

__device__ __forceinline__ void drift_f(float& r, int& i, float v, float dtd, int n) {
    const float x = r + v * dtd;
    const float s = floorf(x);
    r = x - s;
    i = wrap_i(i + (int)s, n);
}

// CIC stencil values of one particle (deposit.cu's stencil_values<CIC>):
// val[j*2+i] = rint((aq*Y[j])*X[i]), the first largest weight takes the remainder.
__device__ __forceinline__ void cic_values(float rx, float ry, float qn, int (&val)[4]) {
    const float aq = qn * 16777216.0f;
    const int A = __float2int_rn(aq);
    const float X[2] = {1.0f - rx, rx}, Y[2] = {1.0f - ry, ry};
    int sum = 0;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float ay = aq * Y[j];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            val[j * 2 + i] = __float2int_rn(ay * X[i]);
            sum += val[j * 2 + i];
        }
    }
    const int kmaj = (Y[1] > Y[0] ? 2 : 0) + (X[1] > X[0] ? 1 : 0);
    val[kmaj] += A - sum;
}

__device__ __forceinline__ void flush_cic(const StepArgs& a, const RunDesc* runs, const uint32_t* cbase, int nruns,
                                          uint32_t key, const int (&acc)[4]) {
    const RunDesc& r = runs[find_run(cbase, nruns, key)];
    const uint32_t local = key - r.cell_base;
    const int iy = (int)(local / (uint32_t)r.N), ix = (int)(local - (uint32_t)iy * (uint32_t)r.N);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const size_t row = (size_t)r.cell_base + (size_t)wrap_i(iy + j, r.N) * r.N;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int v = acc[j * 2 + i];
            if (v != 0) atomicAdd(a.acc + row + wrap_i(ix + i, r.N), (unsigned long long)(long long)v);
        }
    }
}

__device__ __forceinline__ uint32_t u4k(const uint4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
__device__ __forceinline__ float f4k(const float4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }

struct Quad4 {
    uint4 cell;
    float4 xr, yr, q;
};

__device__ __forceinline__ void load_quad4(const StepArgs& a, size_t p0, bool ok, Quad4& d) {
    if (ok) {
        d.cell = __ldcs(reinterpret_cast<const uint4*>(a.cell + p0));
        d.xr = __ldcs(reinterpret_cast<const float4*>(a.xr + p0));
        d.yr = __ldcs(reinterpret_cast<const float4*>(a.yr + p0));
        d.q = make_float4(-1.0f, -1.0f, -1.0f, -1.0f);  // every stored charge is -1 (ens_init_run)
    }
}

// The step's particle work in one launch (see the file header).
__global__ void __launch_bounds__(ENS_THREADS, 4) ens_step_kernel(StepArgs a) {
    __shared__ uint32_t cbase[MAX_RUNS];
    for (int i = threadIdx.x; i < a.nruns; i += ENS_THREADS) cbase[i] = a.runs[i].cell_base;
    __syncthreads();
    const size_t nthreads = (size_t)gridDim.x * ENS_THREADS;
    const size_t tid = (size_t)blockIdx.x * ENS_THREADS + threadIdx.x;

    // With both the move and the deposit, the moved quads are deposited straight
    // from registers (the deposit phase's run sums and segmented warp scan over
    // the same 128-particle warp layout): the deposit does not read the particles again.
    const bool fused = a.do_move && a.do_deposit;
    unsigned brk = 0;  // fused: this thread's order breaks
    if (a.do_move) {  // gather + push (push.cu move_particles<true, true>), 4 particles per thread
        const int lane = threadIdx.x & 31;
        const unsigned upto = (lane == 31) ? FULLM : ((2u << lane) - 1u);
        const size_t wfirst = tid - (size_t)lane;  // this warp's first thread
        for (int ri = 0; ri < a.nruns; ++ri) {
            const RunDesc& r = a.runs[ri];
            const int N = r.N;
            const size_t b0 = r.cell_base;
            const size_t nq = r.np / 4, q0 = r.pbase / 4;  // particle counts and bases are multiples of 4
            // the next quad's cell keys are loaded before this quad is used, so its
            // field gathers can start with the other fields' loads
            uint4 ncl = make_uint4(0, 0, 0, 0);
            if (tid < nq) ncl = *reinterpret_cast<const uint4*>(a.cell + (q0 + tid) * 4);
            // warp-uniform loop: lanes past the run's end sit out (their quads do not exist)
            for (size_t qb = wfirst; qb < nq; qb += nthreads) {
                const size_t qi = qb + (size_t)lane;
                const bool act = qi < nq;
                const size_t p0 = (q0 + qi) * 4;
                uint4 cl = ncl;
                if (qi + nthreads < nq) ncl = *reinterpret_cast<const uint4*>(a.cell + (q0 + qi + nthreads) * 4);
                float4 fx = make_float4(0.0f, 0.0f, 0.0f, 0.0f), fy = fx, gx = fx, gy = fx;
                uint32_t* pc = reinterpret_cast<uint32_t*>(&cl);
                float *px = reinterpret_cast<float*>(&fx), *py = reinterpret_cast<float*>(&fy);
                float *pvx = reinterpret_cast<float*>(&gx), *pvy = reinterpret_cast<float*>(&gy);
                if (act) {
                    fx = *reinterpret_cast<const float4*>(a.xr + p0);
                    fy = *reinterpret_cast<const float4*>(a.yr + p0);
                    gx = *reinterpret_cast<const float4*>(a.vx + p0);
                    gy = *reinterpret_cast<const float4*>(a.vy + p0);
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const uint32_t local = pc[k] - r.cell_base;
                        int iy = (int)(local / (uint32_t)N);
                        int ix = (int)(local - (uint32_t)iy * (uint32_t)N);
                        float rx = px[k], ry = py[k];
                        float vxx = pvx[k], vyy = pvy[k];
                        const int ixp = (ix + 1) % N, iyp = (iy + 1) % N;
                        const size_t i00 = b0 + (size_t)iy * N + ix, i10 = b0 + (size_t)iy * N + ixp;
                        const size_t i01 = b0 + (size_t)iyp * N + ix, i11 = b0 + (size_t)iyp * N + ixp;
                        const float ex = interp_f(a.Exf, i00, i10, i01, i11, rx, ry);
                        const float ey = interp_f(a.Eyf, i00, i10, i01, i11, rx, ry);
                        vxx = vxx + (r.coef * ex) * a.dtf;
                        vyy = vyy + (r.coef * ey) * a.dtf;
                        drift_f(rx, ix, vxx, a.dtd, N);
                        drift_f(ry, iy, vyy, a.dtd, N);
                        pvx[k] = vxx;
                        pvy[k] = vyy;
                        px[k] = rx;
                        py[k] = ry;
                        pc[k] = r.cell_base + (uint32_t)iy * (uint32_t)N + (uint32_t)ix;
                    }
                    *reinterpret_cast<uint4*>(a.cell + p0) = cl;
                    *reinterpret_cast<float4*>(a.xr + p0) = fx;
                    *reinterpret_cast<float4*>(a.yr + p0) = fy;
                    *reinterpret_cast<float4*>(a.vx + p0) = gx;
                    *reinterpret_cast<float4*>(a.vy + p0) = gy;
                }
                if (fused) {  // deposit.cu deposit_runs<CIC> on the moved quads (charge -1)
                    // disorder: adjacent pairs whose cell key decreases (within the run's range;
                    // inactive lanes are the warp's last ones, so lane - 1 is active with lane)
                    const uint32_t prev3 = __shfl_up_sync(FULLM, pc[3], 1);
                    if (act)
                        brk += (pc[1] < pc[0]) + (pc[2] < pc[1]) + (pc[3] < pc[2]) +
                               ((lane > 0 && qi > 0 && pc[0] < prev3) ? 1u : 0u);
                    uint32_t ckey = NO_KEY;
                    int acc[4] = {0, 0, 0, 0};
                    if (act) {
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            int val[4];
                            cic_values(px[k], py[k], -1.0f, val);
                            if (pc[k] != ckey) {
                                if (ckey != NO_KEY) flush_cic(a, a.runs, cbase, a.nruns, ckey, acc);
                                ckey = pc[k];
#pragma unroll
                                for (int q = 0; q < 4; ++q) acc[q] = val[q];
                            } else {
#pragma unroll
                                for (int q = 0; q < 4; ++q) acc[q] += val[q];
                            }
                        }
                    }
                    const uint32_t kprev = __shfl_up_sync(FULLM, ckey, 1);
                    // segments stop at lane 16: a run total covers <= 64 particles and fits int32
                    const unsigned H = __ballot_sync(FULLM, lane == 0 || lane == 16 || ckey != kprev);
                    const int segstart = 31 - __clz(H & upto);
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const bool take = lane - d >= segstart;
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int o = __shfl_up_sync(FULLM, acc[q], d);
                            if (take) acc[q] += o;
                        }
                    }
                    const bool tail = (lane == 31) || ((H >> (lane + 1)) & 1u);
                    if (tail && ckey != NO_KEY) flush_cic(a, a.runs, cbase, a.nruns, ckey, acc);
                }
            }
        }
        if (fused && a.breaks) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) brk += __shfl_xor_sync(FULLM, brk, o);
            if (lane == 0 && brk) atomicAdd(a.breaks, (unsigned long long)brk);
        }
        if (fused ? a.do_convert : (a.do_deposit || a.do_convert))
            if (!grid_barrier(a.bar, a.err)) return;
    }
    if (a.do_deposit && !fused) {  // deposit.cu deposit_runs<CIC>, per-run wrap
        const int lane = threadIdx.x & 31;
        const size_t gw = (size_t)blockIdx.x * ENS_WARPS + (threadIdx.x >> 5);
        const size_t stride = (size_t)gridDim.x * ENS_WARPS * 128;
        const unsigned upto = (lane == 31) ? FULLM : ((2u << lane) - 1u);
        size_t base = gw * 128;
        Quad4 cur, nxt;
        load_quad4(a, base + 4u * lane, base + 4u * lane < a.n, cur);
        for (; base < a.n; base += stride) {
            const size_t nbase = base + stride;
            if (nbase < a.n) load_quad4(a, nbase + 4u * lane, nbase + 4u * lane < a.n, nxt);
            uint32_t ckey = NO_KEY;
            int acc[4] = {0, 0, 0, 0};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const size_t p = base + 4u * lane + (size_t)k;
                if (p < a.n) {
                    const uint32_t key = u4k(cur.cell, k);
                    if (key >= a.G) continue;
                    int val[4];
                    cic_values(f4k(cur.xr, k), f4k(cur.yr, k), f4k(cur.q, k), val);
                    if (key != ckey) {
                        if (ckey != NO_KEY) flush_cic(a, a.runs, cbase, a.nruns, ckey, acc);
                        ckey = key;
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[q] = val[q];
                    } else {
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[q] += val[q];
                    }
                }
            }
            const uint32_t kprev = __shfl_up_sync(FULLM, ckey, 1);
            // segments stop at lane 16: a run total covers <= 64 particles and fits int32
            const unsigned H = __ballot_sync(FULLM, lane == 0 || lane == 16 || ckey != kprev);
            const int segstart = 31 - __clz(H & upto);
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const bool take = lane - d >= segstart;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int o = __shfl_up_sync(FULLM, acc[q], d);
                    if (take) acc[q] += o;
                }
            }
            const bool tail = (lane == 31) || ((H >> (lane + 1)) & 1u);
            if (tail && ckey != NO_KEY) flush_cic(a, a.runs, cbase, a.nruns, ckey, acc);
            cur = nxt;
        }
        if (a.do_convert)
            if (!grid_barrier(a.bar, a.err)) return;
    }
    if (a.do_convert) {  // deposit.cu fixed_to_rho per run; clears the int64 grid
        for (int ri = 0; ri < a.nruns; ++ri) {
            const RunDesc& r = a.runs[ri];
            for (size_t i = tid; i < r.cells; i += nthreads) {
                const size_t g = r.cell_base + i;
                const long long v = (long long)a.acc[g];
                a.rho[g] = __dadd_rn(__dmul_rn((double)v, r.unit), r.background);
                a.acc[g] = 0ull;
            }
        }
    }
}

// Tiled CIC deposit over cell-sorted particles (deposit.cu deposit_tiled<CIC>
// with one tile table over all runs; tile shape per run).
__global__ void __launch_bounds__(ENS_THREADS) ens_deposit_tiled(StepArgs a, const uint32_t* __restrict__ offsets,
                                                                int first_run, int last_run) {
    extern __shared__ long long sacc[];
    __shared__ uint32_t tbase[MAX_RUNS];
    for (int i = threadIdx.x; i < a.nruns; i += ENS_THREADS) tbase[i] = a.runs[i].tile_base;
    __syncthreads();
    const uint32_t cta = blockIdx.x + a.runs[first_run].tile_base;
    int ri = find_run(tbase, a.nruns, cta);
    if (ri < first_run || ri > last_run) return;
    const RunDesc& R = a.runs[ri];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int t = (int)(cta - R.tile_base);
    const int SW = R.tile_w + 3;
    const int tx = t % R.tiles_x, ty = t / R.tiles_x;
    const int x0 = tx * R.tile_w, y0 = ty * R.tile_h;
    const int tw = min(R.tile_w, R.N - x0), th = min(R.tile_h, R.N - y0);
    const int nloc = (th + 3) * SW;
    for (int i = threadIdx.x; i < nloc; i += ENS_THREADS) sacc[i] = 0;
    __syncthreads();
    const unsigned upto = (lane == 31) ? FULLM : ((2u << lane) - 1u);
    for (int r = warp; r < th; r += ENS_WARPS) {
        const int iy = y0 + r;
        const uint32_t rowbase = R.cell_base + (uint32_t)iy * (uint32_t)R.N;
        const uint32_t c0 = rowbase + (uint32_t)x0;
        const uint32_t pbeg = offsets[c0], pend = offsets[c0 + tw];
        const int lrow = r + 1;
        const int lcol = 1 - x0;
        uint32_t base = pbeg & ~3u;
        Quad4 cur, nxt;
        load_quad4(a, base + 4u * lane, base + 4u * lane < pend, cur);
        while (base < pend) {
            const uint32_t nbase = base + 128u;
            if (nbase < pend) load_quad4(a, nbase + 4u * lane, nbase + 4u * lane < pend, nxt);
            uint32_t ckey = NO_KEY;
            int acc[4] = {0, 0, 0, 0};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t p = base + 4u * lane + (uint32_t)k;
                if (p >= pbeg && p < pend) {
                    const uint32_t key = u4k(cur.cell, k);
                    if (key - c0 >= (uint32_t)tw) continue;
                    int val[4];
                    cic_values(f4k(cur.xr, k), f4k(cur.yr, k), f4k(cur.q, k), val);
                    if (key != ckey) {
                        if (ckey != NO_KEY) {
                            const int lx = (int)(ckey - rowbase) + lcol;
#pragma unroll
                            for (int q = 0; q < 4; ++q)
                                if (acc[q] != 0)
                                    atomicAdd(reinterpret_cast<unsigned long long*>(sacc + (lrow + q / 2) * SW + lx + (q % 2)),
                                              (unsigned long long)(long long)acc[q]);
                        }
                        ckey = key;
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[q] = val[q];
                    } else {
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[q] += val[q];
                    }
                }
            }
            const uint32_t kprev = __shfl_up_sync(FULLM, ckey, 1);
            // segments stop at lane 16: a run total covers <= 64 particles and fits int32
            const unsigned H = __ballot_sync(FULLM, lane == 0 || lane == 16 || ckey != kprev);
            const int segstart = 31 - __clz(H & upto);
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const bool take = lane - d >= segstart;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int o = __shfl_up_sync(FULLM, acc[q], d);
                    if (take) acc[q] += o;
                }
            }
            const bool tail = (lane == 31) || ((H >> (lane + 1)) & 1u);
            if (tail && ckey != NO_KEY) {
                const int lx = (int)(ckey - rowbase) + lcol;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (acc[q] != 0)
                        atomicAdd(reinterpret_cast<unsigned long long*>(sacc + (lrow + q / 2) * SW + lx + (q % 2)),
                                  (unsigned long long)(long long)acc[q]);
            }
            cur = nxt;
            base = nbase;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nloc; i += ENS_THREADS) {
        const long long v = sacc[i];
        if (v != 0) {
            const int ly = i / SW, lx = i % SW;
            const int gx = wrap_i(x0 - 1 + lx, R.N), gy = wrap_i(y0 - 1 + ly, R.N);
            atomicAdd(a.acc + R.cell_base + (size_t)gy * R.N + gx, (unsigned long long)v);
        }
    }
}

struct InitArgs {
    const RunDesc* runs;
    int run;
    uint32_t seed;
    uint32_t member_seed;  // the member's own seed: its stream does not depend on its place in the batch
    double amp, vth;
    uint32_t* cell;
    float *xr, *yr, *vx, *vy, *q;
};

// x from the density 1 + amp*cos(2*pi*x/L) by Newton on its CDF, y uniform,
// v Maxwellian (Box-Muller), charge qn = -1 (the run's |q| is in its descriptor).
__global__ void ens_init_run(InitArgs a) {
    const RunDesc& R = a.runs[a.run];
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R.np) return;
    const size_t p = R.pbase + i;
    U4 c;
    c.v[0] = (uint32_t)i;
    c.v[1] = (uint32_t)((uint64_t)i >> 32);
    c.v[2] = a.member_seed;
    c.v[3] = 0x5EED0001u;
    const U4 u = philox(c, a.seed, 0x7A3C91E5u);
    c.v[3] = 0x5EED0002u;
    const U4 w = philox(c, a.seed, 0x7A3C91E5u);
    const double L = (double)R.N;
    const double k = 2.0 * 3.14159265358979323846 / L;
    const double target = unit_open0(u.v[0], u.v[1]) * L;
    double x = target;
    for (int it = 0; it < 8; ++it) {
        const double f = x + (a.amp / k) * sin(k * x) - target;
        x -= f / (1.0 + a.amp * cos(k * x));
    }
    double y = unit_open0(u.v[2], u.v[3]) * L;
    const double r1 = sqrt(-2.0 * log(unit_open0(w.v[0], w.v[1])));
    const double t1 = 2.0 * unit_open0(w.v[2], w.v[3]);
    const double gx = r1 * cospi(t1), gy = r1 * sinpi(t1);
    // cell coordinates as the upload computes them (context.cu cell_coord), no
    // offset equal to 1.0f
    int cx[2];
    float off[2];
    const double pos[2] = {x, y};
    for (int d = 0; d < 2; ++d) {
        double v = pos[d];
        if (v >= L) v -= L;
        if (v < 0.0) v += L;
        const double f = floor(v);
        int ii = (int)f;
        const double frac = v - (double)ii;
        float r = __double2float_rn(frac);
        if (frac < 0.5 && r >= 0.5f) r = 0.49999997f;
        if (r >= 1.0f) {
            r = 0.0f;
            ii += 1;
        }
        cx[d] = wrap_i(ii, R.N);
        off[d] = r;
    }
    a.cell[p] = R.cell_base + (uint32_t)cx[1] * (uint32_t)R.N + (uint32_t)cx[0];
    a.xr[p] = off[0];
    a.yr[p] = off[1];
    a.vx[p] = __double2float_rn(gx * a.vth);
    a.vy[p] = __double2float_rn(gy * a.vth);
    a.q[p] = -1.0f;
}

// fields.cu k_divide for a batch of equal-size runs: spec /= k^2 (continuous k,
// L = N), DC = 0.
__global__ void ens_k_divide(cufftDoubleComplex* __restrict__ spec, int N, int count) {
    const int nh = N / 2 + 1;
    const size_t per = (size_t)nh * N;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= per * count) return;
    const size_t s = t % per;
    const int i = (int)(s % nh), j = (int)(s / nh);
    if (i == 0 && j == 0) {
        spec[t].x = 0.0;
        spec[t].y = 0.0;
        return;
    }
    const double twopi = 2.0 * 3.14159265358979323846;
    const int mx = (i <= N / 2) ? i : i - N;
    const int my = (j <= N / 2) ? j : j - N;
    const double L = (double)N;
    const double kx = __ddiv_rn(__dmul_rn(twopi, (double)mx), L);
    const double ky = __ddiv_rn(__dmul_rn(twopi, (double)my), L);
    const double k2 = __dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky));
    spec[t].x = __ddiv_rn(spec[t].x, k2);
    spec[t].y = __ddiv_rn(spec[t].y, k2);
}

// rhs = rho * dV (dV = 1) for the batch's cells
__global__ void ens_copy_rhs(const double* __restrict__ rho, size_t n, double* __restrict__ rhs) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rhs[i] = __dmul_rn(rho[i], 1.0);
}

// phi *= 1/G_run, then E = forward difference (fields.cu scale_phi + efield), per run
__global__ void ens_scale_efield(const RunDesc* __restrict__ runs, int nruns, uint32_t G, double* __restrict__ phi,
                                 double* __restrict__ Ex, double* __restrict__ Ey, float* __restrict__ Exf,
                                 float* __restrict__ Eyf, int phase) {
    __shared__ uint32_t cbase[MAX_RUNS];
    for (int i = threadIdx.x; i < nruns; i += blockDim.x) cbase[i] = runs[i].cell_base;
    __syncthreads();
    const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    const RunDesc& r = runs[find_run(cbase, nruns, (uint32_t)g)];
    if (phase == 0) {
        phi[g] = __dmul_rn(phi[g], 1.0 / (double)r.cells);
        return;
    }
    const uint32_t local = (uint32_t)g - r.cell_base;
    const int j = (int)(local / (uint32_t)r.N), i = (int)(local - (uint32_t)j * (uint32_t)r.N);
    const int ip = (i + 1) % r.N, jp = (j + 1) % r.N;
    const double p = phi[g];
    const double ex = -__dmul_rn(__dsub_rn(phi[r.cell_base + (size_t)j * r.N + ip], p), 1.0);
    const double ey = -__dmul_rn(__dsub_rn(phi[r.cell_base + (size_t)jp * r.N + i], p), 1.0);
    Ex[g] = ex;
    Ey[g] = ey;
    Exf[g] = __double2float_rn(ex);
    Eyf[g] = __double2float_rn(ey);
}

// Per-run energies of the step into hist[step*nruns + r]: field energy
// 0.5*sum(Ex^2+Ey^2) (FP64) and kinetic 0.5*m*sum(vx^2+vy^2), summed in FP32
// per thread (a few thousand particles) and in FP64 across threads (FP64
// arithmetic per particle would cost more than the step's particle work). Blocks are given to runs in
// proportion to their particles (EN_CHUNK per block); a run's blocks are added
// in index order, so the result does not depend on the launch.
constexpr size_t EN_CHUNK = 1 << 20;
__global__ void ens_energy_partials(const RunDesc* __restrict__ runs, int nruns, const double* __restrict__ Ex,
                                    const double* __restrict__ Ey, const float* __restrict__ vx,
                                    const float* __restrict__ vy, double* __restrict__ partial) {
    __shared__ uint32_t ebase[MAX_RUNS];
    __shared__ double ws[2][ENS_THREADS / 32];
    for (int i = threadIdx.x; i < nruns; i += ENS_THREADS) ebase[i] = runs[i].en_base;
    __syncthreads();
    const int r = find_run(ebase, nruns, blockIdx.x);
    const RunDesc& R = runs[r];
    const int b = (int)(blockIdx.x - R.en_base), nb = (int)R.en_blocks;
    double fe = 0.0, ke = 0.0;
    {
        const size_t n = R.cells, chunk = (n + nb - 1) / nb;
        const size_t s = (size_t)b * chunk, e = s + chunk < n ? s + chunk : n;
        for (size_t i = s + threadIdx.x; i < e; i += ENS_THREADS) {
            const double ex = Ex[R.cell_base + i], ey = Ey[R.cell_base + i];
            fe = __dadd_rn(fe, __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)));
        }
    }
    {
        const size_t n = R.np, chunk = (n + nb - 1) / nb;
        const size_t s = (size_t)b * chunk, e = s + chunk < n ? s + chunk : n;
        float kf = 0.0f;
        for (size_t i = s + threadIdx.x; i < e; i += ENS_THREADS) {
            const float a = vx[R.pbase + i], c = vy[R.pbase + i];
            kf += a * a + c * c;
        }
        ke = (double)kf;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        fe = __dadd_rn(fe, __shfl_down_sync(FULLM, fe, o));
        ke = __dadd_rn(ke, __shfl_down_sync(FULLM, ke, o));
    }
    if (lane == 0) {
        ws[0][warp] = fe;
        ws[1][warp] = ke;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int w = 0; w < ENS_THREADS / 32; ++w) {
            a = __dadd_rn(a, ws[0][w]);
            c = __dadd_rn(c, ws[1][w]);
        }
        partial[2 * blockIdx.x] = a;
        partial[2 * blockIdx.x + 1] = c;
    }
}

__global__ void ens_energy_final(const RunDesc* __restrict__ runs, const float* __restrict__ mass,
                                 const double* __restrict__ partial, int nruns, const int* __restrict__ step,
                                 int max_steps, double* __restrict__ fe_hist, double* __restrict__ ke_hist) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = *step;
    if (r < nruns && s < max_steps) {
        const RunDesc& R = runs[r];
        double a = 0.0, c = 0.0;
        for (uint32_t b = R.en_base; b < R.en_base + R.en_blocks; ++b) {
            a = __dadd_rn(a, partial[2 * b]);
            c = __dadd_rn(c, partial[2 * b + 1]);
        }
        fe_hist[(size_t)s * nruns + r] = __dmul_rn(0.5, a);
        ke_hist[(size_t)s * nruns + r] = __dmul_rn(__dmul_rn(0.5, (double)mass[r]), c);
    }
}

__global__ void bump_step(int* step) { *step += 1; }

// ring[step] = the order breaks the step's kernel counted; the counter restarts
__global__ void take_breaks(unsigned long long* counter, unsigned long long* ring, const int* step, int cap) {
    const int s = *step;
    if (s < cap) ring[s] = *counter;
    *counter = 0;
}

}  // namespace

}  // namespace picgb

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
using namespace picgb;

struct pic_ens {
    pic_ctx* c = nullptr;  // particles (global cell space) + sort + fields
    std::vector<RunDesc> runs;
    std::vector<int> ppc;
    RunDesc* druns = nullptr;
    float* dmass = nullptr;  // per-run mass (FP32), for the kinetic energy
    unsigned* bar = nullptr;
    int* err = nullptr;
    int* step_ctr = nullptr;
    double *fe_hist = nullptr, *ke_hist = nullptr, *en_partial = nullptr;
    int hist_cap = 0;
    double dt = 0.1, amp = 0.01, vth = 0.05;
    int sort_interval = 0, use_graph = 1;
    double sort_disorder = 0.0;   // > 0: also sort on the measured order breaks
    unsigned long long* breaks = nullptr;       // counter of the step kernel
    unsigned long long* breaks_ring = nullptr;  // per step of a pic_ens_run call (hist_cap entries)
    long long sorts = 0;
    long long steps_done = 0;
    int coop_blocks = 0;
    uint32_t en_blocks = 0;  // blocks of the energy sums (all runs)
    bool tuned = false;
    // batched FFT per grid size
    struct Batch {
        int N, first_run, count;
        uint32_t cell_base;
        cufftHandle fwd, inv;
        cufftDoubleComplex* spec;
        double* rhs;
    };
    std::vector<Batch> batches;
    double* rhs_all = nullptr;
    cufftDoubleComplex* spec_all = nullptr;
    // graphs keyed by the particle buffers
    struct G {
        float* key;
        cudaGraphExec_t exec;
    };
    std::vector<G> graphs;
    long long graph_kernels = 0;
};

namespace {

int ens_fail_cufft(cufftResult r, const char* what) {
    return r == CUFFT_SUCCESS ? PIC_OK : fail(PIC_ERR_CUDA, std::string(what) + " failed");
}

StepArgs step_args(pic_ens* e) {
    pic_ctx* c = e->c;
    StepArgs a{};
    a.runs = e->druns;
    a.nruns = (int)e->runs.size();
    a.cell = c->cell;
    a.xr = c->xr;
    a.yr = c->yr;
    a.vx = c->vx;
    a.vy = c->vy;
    a.q = c->q;
    a.Exf = c->Exf;
    a.Eyf = c->Eyf;
    a.acc = reinterpret_cast<unsigned long long*>(c->acc);
    a.rho = c->rho;
    a.n = c->n;
    a.G = (uint32_t)c->G;
    a.dtf = (float)e->dt;
    a.dtd = (float)(e->dt / 1.0);
    a.bar = e->bar;
    a.err = e->err;
    a.breaks = e->sort_disorder > 0.0 ? e->breaks : nullptr;
    return a;
}

int launch_step_kernel(pic_ens* e, int move, int deposit, int convert) {
    StepArgs a = step_args(e);
    a.do_move = move;
    a.do_deposit = deposit;
    a.do_convert = convert;
    // cooperative: every CTA resident at once (the grid barriers rely on it)
    cudaLaunchConfig_t lc{};
    lc.gridDim = dim3(e->coop_blocks);
    lc.blockDim = dim3(ENS_THREADS);
    lc.dynamicSmemBytes = 0;
    lc.stream = e->c->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    const cudaError_t r = cudaLaunchKernelEx(&lc, ens_step_kernel, a);
    if (r != cudaSuccess) return cuda_fail(r, "cudaLaunchKernelEx(ens_step_kernel, cooperative)");
    e->c->launches++;
    return PIC_OK;
}

int launch_tiled(pic_ens* e, int first_run, int last_run) {
    pic_ctx* c = e->c;
    const RunDesc& f = e->runs[first_run];
    const RunDesc& l = e->runs[last_run];
    const uint32_t ntiles = l.tile_base + (uint32_t)(l.tiles_x * ((l.N + l.tile_h - 1) / l.tile_h)) - f.tile_base;
    int smem = 0;
    for (int r = first_run; r <= last_run; ++r)
        smem = std::max(smem, (e->runs[r].tile_h + 3) * (e->runs[r].tile_w + 3) * 8);
    StepArgs a = step_args(e);
    ens_deposit_tiled<<<ntiles, ENS_THREADS, smem, c->stream>>>(a, c->offsets, first_run, last_run);
    c->launches++;
    return check_launch(c, "ens_deposit_tiled");
}

// Re-lays the tile table after tile shapes change.
int upload_runs(pic_ens* e) {
    uint32_t tb = 0;
    for (auto& r : e->runs) {
        r.tiles_x = (r.N + r.tile_w - 1) / r.tile_w;
        r.tile_base = tb;
        tb += (uint32_t)(r.tiles_x * ((r.N + r.tile_h - 1) / r.tile_h));
    }
    PIC_CUDA_TRY(cudaMemcpyAsync(e->druns, e->runs.data(), e->runs.size() * sizeof(RunDesc), cudaMemcpyHostToDevice,
                                 e->c->stream));
    return PIC_OK;
}

int poisson(pic_ens* e) {
    pic_ctx* c = e->c;
    for (auto& b : e->batches) {
        const size_t cells = (size_t)b.count * b.N * b.N;
        ens_copy_rhs<<<(unsigned)((cells + 255) / 256), 256, 0, c->stream>>>(c->rho + b.cell_base, cells, b.rhs);
        PIC_TRY(check_launch(c, "ens_copy_rhs"));
        PIC_TRY(ens_fail_cufft(cufftExecD2Z(b.fwd, b.rhs, b.spec), "cufftExecD2Z"));
        const size_t ns = (size_t)b.count * b.N * (b.N / 2 + 1);
        ens_k_divide<<<(unsigned)((ns + 255) / 256), 256, 0, c->stream>>>(b.spec, b.N, b.count);
        PIC_TRY(check_launch(c, "ens_k_divide"));
        PIC_TRY(ens_fail_cufft(cufftExecZ2D(b.inv, b.spec, c->phi + b.cell_base), "cufftExecZ2D"));
        c->launches += 2;
    }
    const unsigned blocks = (unsigned)((c->G + 255) / 256);
    for (int phase = 0; phase < 2; ++phase) {
        ens_scale_efield<<<blocks, 256, 0, c->stream>>>(e->druns, (int)e->runs.size(), (uint32_t)c->G, c->phi, c->Ex,
                                                        c->Ey, c->Exf, c->Eyf, phase);
        PIC_TRY(check_launch(c, "ens_scale_efield"));
        c->launches++;
    }
    return PIC_OK;
}

int energies(pic_ens* e) {
    pic_ctx* c = e->c;
    const int nr = (int)e->runs.size();
    ens_energy_partials<<<e->en_blocks, ENS_THREADS, 0, c->stream>>>(e->druns, nr, c->Ex, c->Ey, c->vx, c->vy,
                                                                    e->en_partial);
    PIC_TRY(check_launch(c, "ens_energy_partials"));
    ens_energy_final<<<(nr + 127) / 128, 128, 0, c->stream>>>(e->druns, e->dmass, e->en_partial, nr, e->step_ctr,
                                                              e->hist_cap, e->fe_hist, e->ke_hist);
    PIC_TRY(check_launch(c, "ens_energy_final"));
    bump_step<<<1, 1, 0, c->stream>>>(e->step_ctr);
    c->launches += 3;
    return check_launch(c, "bump_step");
}

// The step without a sort: persistent kernel, Poisson, energies.
int take_step_breaks(pic_ens* e) {
    if (e->sort_disorder <= 0.0) return PIC_OK;
    take_breaks<<<1, 1, 0, e->c->stream>>>(e->breaks, e->breaks_ring, e->step_ctr, e->hist_cap);
    e->c->launches++;
    return check_launch(e->c, "take_breaks");
}

int plain_step(pic_ens* e) {
    PIC_TRY(launch_step_kernel(e, 1, 1, 1));
    PIC_TRY(take_step_breaks(e));
    PIC_TRY(poisson(e));
    return energies(e);
}

// Autotuner: for each class of runs with equal (N, particles per cell), time
// the tiled deposit with each candidate tile shape on the current (sorted)
// particles and keep the fastest. Leaves the int64 grid cleared.
int autotune(pic_ens* e) {
    pic_ctx* c = e->c;
    static const int cand[][2] = {{32, 8}, {64, 4}, {16, 16}, {32, 16}, {64, 8}, {128, 2}};
    cudaEvent_t a, b;
    PIC_CUDA_TRY(cudaEventCreate(&a));
    PIC_CUDA_TRY(cudaEventCreate(&b));
    size_t i = 0;
    int out = PIC_OK;
    while (i < e->runs.size() && out == PIC_OK) {
        size_t j = i;
        while (j + 1 < e->runs.size() && e->runs[j + 1].N == e->runs[i].N && e->ppc[j + 1] == e->ppc[i]) ++j;
        float best = 1e30f;
        int bw = e->runs[i].tile_w, bh = e->runs[i].tile_h;
        for (const auto& t : cand) {
            if (t[0] > e->runs[i].N || t[1] > e->runs[i].N) continue;
            for (size_t r = i; r <= j; ++r) {
                e->runs[r].tile_w = t[0];
                e->runs[r].tile_h = t[1];
            }
            if ((out = upload_runs(e)) != PIC_OK) break;
            float ms = 0.0f;
            for (int rep = 0; rep < 3 && out == PIC_OK; ++rep) {
                cudaEventRecord(a, c->stream);
                out = launch_tiled(e, (int)i, (int)j);
                cudaEventRecord(b, c->stream);
                cudaEventSynchronize(b);
                float t1 = 0.0f;
                cudaEventElapsedTime(&t1, a, b);
                if (rep > 0) ms += t1;
            }
            if (ms < best) {
                best = ms;
                bw = t[0];
                bh = t[1];
            }
        }
        for (size_t r = i; r <= j; ++r) {
            e->runs[r].tile_w = bw;
            e->runs[r].tile_h = bh;
        }
        i = j + 1;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    PIC_TRY(out);
    PIC_TRY(upload_runs(e));
    PIC_CUDA_TRY(cudaMemsetAsync(c->acc, 0, c->G * 8, c->stream));
    e->tuned = true;
    return PIC_OK;
}

int sorted_step(pic_ens* e) {
    pic_ctx* c = e->c;
    PIC_TRY(launch_step_kernel(e, 1, 0, 0));
    PIC_TRY(sort_particles(c));
    e->sorts++;
    if (!e->tuned) PIC_TRY(autotune(e));
    PIC_TRY(launch_tiled(e, 0, (int)e->runs.size() - 1));
    PIC_TRY(launch_step_kernel(e, 0, 0, 1));
    PIC_TRY(take_step_breaks(e));  // zero: the step's deposit ran on sorted particles
    PIC_TRY(poisson(e));
    return energies(e);
}

int graph_step(pic_ens* e) {
    pic_ctx* c = e->c;
    for (auto& g : e->graphs)
        if (g.key == c->xr) {
            PIC_CUDA_TRY(cudaGraphLaunch(g.exec, c->stream));
            c->launches += e->graph_kernels;
            return PIC_OK;
        }
    cudaGraph_t graph;
    const long long before = c->launches;
    PIC_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = plain_step(e);
    const cudaError_t ec = cudaStreamEndCapture(c->stream, &graph);
    PIC_TRY(rc);
    if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture");
    e->graph_kernels = c->launches - before;
    c->launches = before;
    cudaGraphExec_t exec;
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return cuda_fail(ei, "cudaGraphInstantiate");
    e->graphs.push_back({c->xr, exec});
    PIC_CUDA_TRY(cudaGraphLaunch(exec, c->stream));
    c->launches += e->graph_kernels;
    return PIC_OK;
}

}  // namespace

extern "C" {

int pic_ens_create(const pic_ens_member* runs_in, int nruns, const pic_ens_config* cfg, int device, pic_ens** out) {
    if (!runs_in || nruns <= 0 || nruns > MAX_RUNS || !cfg || !out) return fail(PIC_ERR_ARG, "bad ensemble argument");
    *out = nullptr;
    if (!(cfg->sort_disorder >= 0.0 && cfg->sort_disorder <= 1.0))
        return fail(PIC_ERR_ARG, "ensemble sort_disorder must be in [0, 1]");
    std::vector<int> order(nruns);
    for (int i = 0; i < nruns; ++i) {
        const int N = runs_in[i].N, ppc = runs_in[i].ppc;
        if (N < 2 || (N & 1) || ppc <= 0) return fail(PIC_ERR_ARG, "ensemble runs need even N >= 2 and ppc > 0");
        order[i] = i;
    }
    // runs sorted by grid size (stable), so equal sizes share one batched FFT
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return runs_in[a].N < runs_in[b].N; });
    size_t G = 0, n = 0;
    for (int i = 0; i < nruns; ++i) {
        const pic_ens_member& r = runs_in[order[i]];
        G += (size_t)r.N * r.N;
        n += (size_t)r.N * r.N * r.ppc;
    }
    if (G >= (1ull << 31) || n > (1ull << 32) - 4096) return fail(PIC_ERR_ARG, "ensemble too large for 32-bit keys");
    pic_ens* e = new pic_ens();
    e->dt = cfg->dt;
    e->amp = cfg->amplitude;
    e->vth = cfg->vth;
    e->sort_interval = cfg->sort_interval;
    e->sort_disorder = cfg->sort_disorder;
    e->use_graph = cfg->use_graph;
    pic_domain d{(double)G, 1.0, (int32_t)G, 1};
    int rc = pic_gpu_create(&d, n, device, &e->c);
    if (rc != PIC_OK) {
        delete e;
        return rc;
    }
    pic_ctx* c = e->c;
    size_t cb = 0, pb = 0;
    std::vector<float> mass(nruns);
    for (int i = 0; i < nruns; ++i) {
        const pic_ens_member& in = runs_in[order[i]];
        RunDesc r{};
        r.cell_base = (uint32_t)cb;
        r.cells = (uint32_t)((size_t)in.N * in.N);
        r.pbase = (uint32_t)pb;
        r.np = (uint32_t)((size_t)in.N * in.N * in.ppc);
        r.N = in.N;
        r.tile_w = std::min(32, in.N);
        r.tile_h = std::min(8, in.N);
        // charge -1/ppc and mass 1/ppc per particle: mean charge density -1, q/m = -1, omega_p = 1
        r.maxq = 1.0f / (float)in.ppc;
        const float m = 1.0f / (float)in.ppc;
        const float qf = -1.0f * r.maxq;
        r.coef = (-qf) / m;  // push.cu: __fdiv_rn(-q*maxq, m)
        r.unit = ((double)r.maxq * 1.0) * 5.9604644775390625e-08;
        r.background = 1.0;
        e->runs.push_back(r);
        e->ppc.push_back(in.ppc);
        mass[i] = m;
        cb += r.cells;
        pb += r.np;
    }
    c->n = n;
    for (auto& r : e->runs) {
        r.en_base = e->en_blocks;
        r.en_blocks = (uint32_t)std::max<size_t>(1, (r.np + EN_CHUNK - 1) / EN_CHUNK);
        e->en_blocks += r.en_blocks;
    }
    int out_rc = PIC_OK;
    auto A = [&](size_t bytes) { return out_rc ? nullptr : dalloc(bytes, &out_rc); };
    e->druns = (RunDesc*)A(sizeof(RunDesc) * nruns);
    e->dmass = (float*)A(sizeof(float) * nruns);
    e->bar = (unsigned*)A(2 * sizeof(unsigned));
    e->err = (int*)A(sizeof(int));
    e->step_ctr = (int*)A(sizeof(int));
    e->breaks = (unsigned long long*)A(sizeof(unsigned long long));
    e->en_partial = (double*)A(sizeof(double) * 2 * e->en_blocks);
    if (out_rc == PIC_OK) out_rc = ensure_fields(c);
    if (out_rc == PIC_OK) out_rc = upload_runs(e);
    if (out_rc == PIC_OK && (cudaMemcpyAsync(e->dmass, mass.data(), sizeof(float) * nruns, cudaMemcpyHostToDevice,
                                             c->stream) != cudaSuccess ||
                             cudaMemsetAsync(e->bar, 0, 2 * sizeof(unsigned), c->stream) != cudaSuccess ||
                             cudaMemsetAsync(e->err, 0, sizeof(int), c->stream) != cudaSuccess ||
                             cudaMemsetAsync(e->step_ctr, 0, sizeof(int), c->stream) != cudaSuccess ||
                             cudaMemsetAsync(c->acc, 0, G * 8, c->stream) != cudaSuccess))
        out_rc = fail(PIC_ERR_CUDA, "ensemble setup copy");
    // particles
    for (int i = 0; i < nruns && out_rc == PIC_OK; ++i) {
        InitArgs ia{e->druns, i, cfg->seed ^ (uint32_t)(runs_in[order[i]].seed * 2654435761u),
                    runs_in[order[i]].seed, e->amp, e->vth, c->cell, c->xr, c->yr, c->vx, c->vy, c->q};
        const size_t np = e->runs[i].np;
        ens_init_run<<<(unsigned)((np + 255) / 256), 256, 0, c->stream>>>(ia);
        out_rc = check_launch(c, "ens_init_run");
    }
    if (out_rc == PIC_OK) {
        // the context's charge normalisation (used by nothing but the sort's
        // bookkeeping) and the particles' sortedness
        c->has_mass = 0;
        c->sorted = 0;
        c->part_valid = 0;
        c->qsum_valid = 0;
        c->qn_uniform = -1.0f;
    }
    // batched FFT plans per grid size
    size_t spec_total = 0;
    for (int i = 0; i < nruns && out_rc == PIC_OK;) {
        int j = i;
        while (j + 1 < nruns && e->runs[j + 1].N == e->runs[i].N) ++j;
        pic_ens::Batch b{};
        b.N = e->runs[i].N;
        b.first_run = i;
        b.count = j - i + 1;
        b.cell_base = e->runs[i].cell_base;
        int nn[2] = {b.N, b.N};
        if (cufftPlanMany(&b.fwd, 2, nn, nullptr, 1, b.N * b.N, nullptr, 1, b.N * (b.N / 2 + 1), CUFFT_D2Z, b.count) !=
                CUFFT_SUCCESS ||
            cufftPlanMany(&b.inv, 2, nn, nullptr, 1, b.N * (b.N / 2 + 1), nullptr, 1, b.N * b.N, CUFFT_Z2D, b.count) !=
                CUFFT_SUCCESS) {
            out_rc = fail(PIC_ERR_CUDA, "cufftPlanMany");
            break;
        }
        cufftSetStream(b.fwd, c->stream);
        cufftSetStream(b.inv, c->stream);
        spec_total += (size_t)b.count * b.N * (b.N / 2 + 1);
        e->batches.push_back(b);
        i = j + 1;
    }
    if (out_rc == PIC_OK) {
        e->rhs_all = (double*)A(G * 8);
        e->spec_all = (cufftDoubleComplex*)A(spec_total * sizeof(cufftDoubleComplex));
        size_t so = 0;
        for (auto& b : e->batches) {
            b.rhs = e->rhs_all ? e->rhs_all + b.cell_base : nullptr;
            b.spec = e->spec_all ? e->spec_all + so : nullptr;
            so += (size_t)b.count * b.N * (b.N / 2 + 1);
        }
    }
    if (out_rc == PIC_OK) {
        int per_sm = 0, sms = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ens_step_kernel, ENS_THREADS, 0);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
        e->coop_blocks = std::max(1, per_sm * sms);
        // fields start at zero, as in a single run (the first gather adds nothing)
        out_rc = pic_gpu_synchronize(c);
    }
    if (out_rc != PIC_OK) {
        pic_ens_destroy(e);
        return out_rc;
    }
    *out = e;
    return PIC_OK;
}

int pic_ens_destroy(pic_ens* e) {
    if (!e) return PIC_OK;
    if (e->c) cudaStreamSynchronize(e->c->stream);
    for (auto& g : e->graphs) cudaGraphExecDestroy(g.exec);
    for (auto& b : e->batches) {
        cufftDestroy(b.fwd);
        cufftDestroy(b.inv);
    }
    void* ptrs[] = {e->druns, e->dmass, e->bar, e->err, e->step_ctr, e->fe_hist, e->ke_hist, e->en_partial,
                    e->rhs_all, e->spec_all, e->breaks, e->breaks_ring};
    for (void* p : ptrs) dfree(p);
    if (e->c) pic_gpu_destroy(e->c);
    delete e;
    return PIC_OK;
}

int pic_ens_run(pic_ens* e, int steps, double* field_energy, double* kinetic_energy) {
    if (!e || steps < 0) return fail(PIC_ERR_ARG, "bad argument");
    pic_ctx* c = e->c;
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    const int nr = (int)e->runs.size();
    if (steps > e->hist_cap) {
        dfree(e->fe_hist);
        dfree(e->ke_hist);
        dfree(e->breaks_ring);
        int rc = PIC_OK;
        e->fe_hist = (double*)dalloc((size_t)steps * nr * 8, &rc);
        if (!rc) e->ke_hist = (double*)dalloc((size_t)steps * nr * 8, &rc);
        if (!rc) e->breaks_ring = (unsigned long long*)dalloc((size_t)steps * 8, &rc);
        if (rc) {
            e->hist_cap = 0;
            return rc;
        }
        e->hist_cap = steps;
        for (auto& g : e->graphs) cudaGraphExecDestroy(g.exec);
        e->graphs.clear();
    }
    // sorts on measured disorder: the breaks of step s - 2 decide step s (copied to
    // page-locked memory after each step; the host waits for a step two behind)
    const bool by_disorder = e->sort_disorder > 0.0;
    unsigned long long* brk_h = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    auto release = [&]() {
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        if (brk_h) cudaFreeHost(brk_h);
    };
    if (by_disorder && steps > 0) {
        if (cudaHostAlloc((void**)&brk_h, (size_t)steps * 8, 0) != cudaSuccess) {
            brk_h = nullptr;
            return fail(PIC_ERR_NOMEM, "pinned allocation");
        }
        for (int i = 0; i < 3; ++i)
            if (cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess) {
                release();
                return fail(PIC_ERR_CUDA, "cudaEventCreate");
            }
    }
    const int loop_rc = [&]() -> int {
        PIC_CUDA_TRY(cudaMemsetAsync(e->step_ctr, 0, sizeof(int), c->stream));
        if (by_disorder) PIC_CUDA_TRY(cudaMemsetAsync(e->breaks, 0, sizeof(unsigned long long), c->stream));
        const double limit = e->sort_disorder * (double)c->n;
        int last_sort = -1;
        for (int s = 0; s < steps; ++s) {
            bool sort = e->sort_interval > 0 && (e->steps_done % e->sort_interval) == 0;
            const int m = s - 2;
            if (by_disorder && !sort && m >= 0 && m > last_sort) {
                PIC_CUDA_TRY(cudaEventSynchronize(ev[m % 3]));
                sort = (double)brk_h[m] > limit;
            }
            if (sort) {
                last_sort = s;
                PIC_TRY(sorted_step(e));
            } else if (e->use_graph) {
                PIC_TRY(graph_step(e));
            } else {
                PIC_TRY(plain_step(e));
            }
            if (by_disorder) {
                PIC_CUDA_TRY(cudaMemcpyAsync(brk_h + s, e->breaks_ring + s, 8, cudaMemcpyDeviceToHost, c->stream));
                PIC_CUDA_TRY(cudaEventRecord(ev[s % 3], c->stream));
            }
            e->steps_done++;
        }
        return PIC_OK;
    }();
    const cudaError_t se = cudaStreamSynchronize(c->stream);
    release();
    PIC_TRY(loop_rc);
    if (se != cudaSuccess) return cuda_fail(se, "cudaStreamSynchronize");
    int herr = 0;
    PIC_CUDA_TRY(cudaMemcpyAsync(&herr, e->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if (field_energy)
        PIC_CUDA_TRY(cudaMemcpyAsync(field_energy, e->fe_hist, (size_t)steps * nr * 8, cudaMemcpyDeviceToHost,
                                     c->stream));
    if (kinetic_energy)
        PIC_CUDA_TRY(cudaMemcpyAsync(kinetic_energy, e->ke_hist, (size_t)steps * nr * 8, cudaMemcpyDeviceToHost,
                                     c->stream));
    PIC_TRY(pic_gpu_synchronize(c));
    if (herr) return fail(PIC_ERR_TIMEOUT, "ensemble: a grid-wide barrier timed out");
    return PIC_OK;
}

int pic_ens_sort_count(pic_ens* e, long long* n) {
    if (!e || !n) return fail(PIC_ERR_ARG, "bad argument");
    *n = e->sorts;
    return PIC_OK;
}

int pic_ens_info(pic_ens* e, int r, pic_ens_run_info* info) {
    if (!e || !info || r < 0 || r >= (int)e->runs.size()) return fail(PIC_ERR_ARG, "bad argument");
    const RunDesc& d = e->runs[r];
    info->N = d.N;
    info->ppc = e->ppc[r];
    info->particles = d.np;
    info->tile_w = d.tile_w;
    info->tile_h = d.tile_h;
    return PIC_OK;
}

int pic_ens_num_runs(pic_ens* e, int* n) {
    if (!e || !n) return fail(PIC_ERR_ARG, "bad argument");
    *n = (int)e->runs.size();
    return PIC_OK;
}

int pic_ens_launch_count(pic_ens* e, long long* n) {
    if (!e || !n) return fail(PIC_ERR_ARG, "bad argument");
    *n = e->c->launches;
    return PIC_OK;
}

int pic_ens_get_stream(pic_ens* e, void** s) {
    if (!e || !s) return fail(PIC_ERR_ARG, "bad argument");
    *s = (void*)e->c->stream;
    return PIC_OK;
}

int pic_ens_download_run(pic_ens* e, int r, double* x, double* y, double* vx, double* vy, double* rho, double* phi) {
    if (!e || r < 0 || r >= (int)e->runs.size()) return fail(PIC_ERR_ARG, "bad argument");
    pic_ctx* c = e->c;
    const RunDesc& d = e->runs[r];
    std::vector<uint32_t> cell(d.np);
    std::vector<float> f(d.np);
    PIC_CUDA_TRY(cudaMemcpyAsync(cell.data(), c->cell + d.pbase, d.np * 4, cudaMemcpyDeviceToHost, c->stream));
    PIC_TRY(pic_gpu_synchronize(c));
    auto get = [&](const float* src, double* dst, int axis) -> int {
        if (!dst) return PIC_OK;
        PIC_CUDA_TRY(cudaMemcpyAsync(f.data(), src + d.pbase, d.np * 4, cudaMemcpyDeviceToHost, c->stream));
        PIC_TRY(pic_gpu_synchronize(c));
        for (size_t i = 0; i < d.np; ++i) {
            const uint32_t local = cell[i] - d.cell_base;
            const uint32_t iy = local / (uint32_t)d.N, ix = local - iy * (uint32_t)d.N;
            dst[i] = axis == 0 ? (double)ix + (double)f[i] : axis == 1 ? (double)iy + (double)f[i] : (double)f[i];
        }
        return PIC_OK;
    };
    PIC_TRY(get(c->xr, x, 0));
    PIC_TRY(get(c->yr, y, 1));
    PIC_TRY(get(c->vx, vx, 2));
    PIC_TRY(get(c->vy, vy, 2));
    if (rho) PIC_CUDA_TRY(cudaMemcpyAsync(rho, c->rho + d.cell_base, (size_t)d.cells * 8, cudaMemcpyDeviceToHost, c->stream));
    if (phi) PIC_CUDA_TRY(cudaMemcpyAsync(phi, c->phi + d.cell_base, (size_t)d.cells * 8, cudaMemcpyDeviceToHost, c->stream));
    return pic_gpu_synchronize(c);
}

}  // extern "C"
