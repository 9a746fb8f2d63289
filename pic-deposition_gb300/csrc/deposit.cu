// Charge deposition: NGP / CIC / TSC / trajectory-averaged ("Esirkepov") rho.
//
// Replaces the reference's CPU kernels (src/deposition/ngp.cpp:108-228) and its
// CUDA backend (src/deposition/cuda/deposition_cuda.cu:205-241: one thread per
// particle with FP64 global atomics, or one block per tile scanning all
// particles). Design:
//
//  * Fixed point. The resident charge is qn = q/max|q|; a particle carries
//    A = rint(qn*2^24) units. Each stencil value (qn*2^24*Y[j])*X[i] (FP32) is
//    rounded to the nearest int32, and one node takes A - (sum of the others)
//    (TSC: the particle's own cell node, weight >= 1/64; NGP/CIC/ESK: the node
//    of largest weight), so every particle deposits exactly A units and
//    total charge is exact. Sums are int64, so the result does not depend on
//    summation order: the sorted, any-order, atomic and oracle paths agree bit
//    for bit. TSC with one charge for every particle uses exact integer
//    weights instead (2^30 units per particle, see tsci_weights).
//  * Sorted path (deposit_cells). One CTA per tile of tile_w x tile_h cells;
//    one lane per cell of a 32-cell unit of a tile row walks the cell's
//    contiguous range of the cell-sorted stream (staged into shared memory with
//    cp.async), sums its particles' stencil values in registers and adds the
//    cell's totals to the tile's accumulators in shared memory once (split
//    into two native 32-bit atomics); at the end the tile is flushed to the
//    global int64 grid once. A freshly sorted stream needs no cell keys: the
//    offsets name every particle's cell. Details at the kernel.
//  * Any-order path (deposit_runs): a warp handles 128 consecutive particles
//    at a time, lane l taking particles 4l..4l+3 (one 128-bit streaming load
//    per field, the next step's loads issued first); a lane sums its
//    particles' values while they share a cell, then a segmented warp scan over
//    the lanes' (cell, sums) leaves each run's total in the run's last lane,
//    which adds it to the global int64 grid (L2-resident). Needs no offsets;
//    fast when particles are nearly cell-ordered (between sorts). The scan's
//    segments stop at lane 16, so a run total covers at most 64 particles and
//    fits int32 (|value| <= 2^24 + 3 per particle and entry).
//  * Naive path (deposit_atomic): one thread per particle, one int64 atomic
//    per stencil node into the global grid.
//
// Stencil frames (weights relative to the particle's own cell, identical to the
// oracle's restatement):
//   NGP   2 nodes (0..1)  one-hot at offset (r >= 0.5)             ngp.cpp:108-120
//   CIC   2 nodes (0..1)  (1-r, r)                                 ngp.cpp:140-157
//   TSC   4 nodes (-1..2) tscWeights written in cell-relative form ngp.cpp:28-34,181-202
//   ESK   3 nodes (-1..1) path r -> r + v*dt/dx split at cell     ngp.cpp:36-84,216-228
//         boundaries, weights = piece / path; static (|v*dt| < 1e-15) -> CIC.
//         Moves of a cell or more go through a general per-lane loop with
//         global atomics.
//
// Compiled with --fmad=false: no multiply-add is fused, so every FP32 result
// equals the oracle's (compiled with -ffp-contract=off).
#include "pic_internal.cuh"

namespace picgb {

enum { S_NGP = 0, S_CIC = 1, S_TSC = 2, S_ESK = 3 };

template <int S>
struct Frame;
template <>
struct Frame<S_NGP> {
    static constexpr int NX = 2, LO = 0, V = 4;
};
template <>
struct Frame<S_CIC> {
    static constexpr int NX = 2, LO = 0, V = 4;
};
template <>
struct Frame<S_TSC> {
    static constexpr int NX = 4, LO = -1, V = 16;
};
template <>
struct Frame<S_ESK> {
    static constexpr int NX = 3, LO = -1, V = 16;
};

constexpr int DEP_THREADS = 256;
constexpr int DEP_WARPS = DEP_THREADS / 32;
constexpr unsigned FULL = 0xffffffffu;
constexpr int ESK_GEN_CAP = 256;

struct DepArgs {
    const uint32_t* cell;
    const float* xr;
    const float* yr;
    const float* vx;
    const float* vy;
    const float* q;
    const uint32_t* offsets;
    unsigned long long* acc;
    size_t n;
    int Nx, Ny;
    float dtf, dtdx, dtdy;
    int tile_w, tile_h, tiles_x;
    float qc;  // nonzero: every particle's stored charge (the charge stream is not read)
    DevStats* st;
    // non-null: the kernel deposits only when *gate == gate_when (the choice
    // between the cell kernel and the any-order kernel between sorts is made on
    // the device, so a captured step keeps one shape)
    const unsigned int* gate;
    unsigned int gate_when;
};

__device__ __forceinline__ bool gated_off(const DepArgs& a) { return a.gate && *a.gate != a.gate_when; }

// ---- one axis of a frame. Returns false when an Esirkepov move needs the general loop.
template <int S>
__device__ __forceinline__ bool axis_frame(float r, float v, float dtf, float dtd, float (&X)[Frame<S>::NX]) {
    if constexpr (S == S_NGP) {
        X[0] = r >= 0.5f ? 0.0f : 1.0f;
        X[1] = r >= 0.5f ? 1.0f : 0.0f;
        return true;
    } else if constexpr (S == S_CIC) {
        X[0] = 1.0f - r;
        X[1] = r;
        return true;
    } else if constexpr (S == S_TSC) {
        if (r < 0.5f) {
            const float d0 = 0.5f - r, d2 = 0.5f + r;
            X[0] = 0.5f * (d0 * d0);
            X[1] = 0.75f - r * r;
            X[2] = 0.5f * (d2 * d2);
            X[3] = 0.0f;
        } else {
            const float d0 = 1.5f - r, d1 = r - 1.0f, d2 = r - 0.5f;
            X[0] = 0.0f;
            X[1] = 0.5f * (d0 * d0);
            X[2] = 0.75f - d1 * d1;
            X[3] = 0.5f * (d2 * d2);
        }
        return true;
    } else {
        if (fabsf(v * dtf) < 1e-15f) {
            X[0] = 0.0f;
            X[1] = 1.0f - r;
            X[2] = r;
            return true;
        }
        const float dc = v * dtd;
        if (!(fabsf(dc) < 1.0f)) return false;
        const float e = r + dc;
        X[0] = 0.0f;
        X[1] = 1.0f;
        X[2] = 0.0f;
        if (dc > 0.0f) {
            if (e > 1.0f) {
                const float wb = __fdiv_rn(e - 1.0f, e - r);
                X[1] = 1.0f - wb;
                X[2] = wb;
            }
        } else if (e < 0.0f) {
            const float wl = __fdiv_rn(0.0f - e, r - e);
            X[0] = wl;
            X[1] = 1.0f - wl;
        }
        return true;
    }
}

// General trajectory split (moves of one cell or more), one piece per call.
struct SegIter {
    float r, e, tot, s;
    int c, dir, k;
    __device__ void init(float r0, float v, float dtf, float dtd) {
        r = r0;
        k = 0;
        if (fabsf(v * dtf) < 1e-15f) {
            dir = 0;
            return;
        }
        const float dc = v * dtd;
        e = r0 + dc;
        dir = dc > 0.0f ? 1 : -1;
        tot = dir > 0 ? e - r0 : r0 - e;
        s = r0;
        c = 0;
    }
    __device__ bool next(int& off, float& w) {
        if (dir == 0) {
            if (k == 0) {
                off = 0;
                w = 1.0f - r;
                k = 1;
                return true;
            }
            if (k == 1) {
                off = 1;
                w = r;
                k = 2;
                return true;
            }
            return false;
        }
        if (dir > 0) {
            if (!(s < e)) return false;
            const float b = (float)(c + 1);
            const float nx = e < b ? e : b;
            off = c;
            w = __fdiv_rn(nx - s, tot);
            s = nx;
            ++c;
        } else {
            if (!(s > e)) return false;
            const float b = (float)c;
            const float nx = e > b ? e : b;
            off = c;
            w = __fdiv_rn(s - nx, tot);
            s = nx;
            --c;
        }
        ++k;
        return true;
    }
};

// Index of the first largest weight (the node that takes a particle's rounding remainder).
template <int N>
__device__ __forceinline__ int first_max(const float (&X)[N]) {
    int m = 0;
    float mv = X[0];
#pragma unroll
    for (int i = 1; i < N; ++i)
        if (X[i] > mv) {
            mv = X[i];
            m = i;
        }
    return m;
}

// Index of the first largest piece of a general trajectory split.
__device__ int seg_first_max(float r, float v, float dtf, float dtd) {
    SegIter it;
    it.init(r, v, dtf, dtd);
    int off, k = 0, m = 0;
    float w, mv = -1.0f;
    while (it.next(off, w) && k <= ESK_GEN_CAP) {
        if (w > mv) {
            mv = w;
            m = k;
        }
        ++k;
    }
    return m;
}

// Moves of one cell or more: deposits straight to the global grid. The piece of
// largest weight on each axis takes the particle's rounding remainder, as in
// the frame path, so the particle deposits exactly A units.
__device__ __noinline__ void esk_general_deposit(const DepArgs& a, int ix, int iy, float aq, long long A, float rx,
                                                 float ry, float vxx, float vyy, size_t pidx) {
    const int mx = seg_first_max(rx, vxx, a.dtf, a.dtdx);
    const int my = seg_first_max(ry, vyy, a.dtf, a.dtdy);
    long long others = 0;
    for (int pass = 0; pass < 2; ++pass) {
        SegIter yi;
        yi.init(ry, vyy, a.dtf, a.dtdy);
        int oy, ox, j = 0;
        float wy, wx;
        while (yi.next(oy, wy)) {
            if (j >= ESK_GEN_CAP) {
                set_dev_error(a.st, DEV_MOVE_TOO_LARGE, (unsigned)pidx);
                return;
            }
            const float ay = aq * wy;
            const int gy = wrap_i(iy + oy, a.Ny);
            SegIter xi;
            xi.init(rx, vxx, a.dtf, a.dtdx);
            int i = 0;
            while (xi.next(ox, wx)) {
                if (i >= ESK_GEN_CAP) {
                    set_dev_error(a.st, DEV_MOVE_TOO_LARGE, (unsigned)pidx);
                    return;
                }
                const bool major = (i == mx && j == my);
                const long long v = major ? 0 : (long long)__float2int_rn(ay * wx);
                if (pass == 0) {
                    others += v;
                } else {
                    const long long out = major ? A - others : v;
                    if (out) atomicAdd(a.acc + (size_t)gy * a.Nx + wrap_i(ix + ox, a.Nx), (unsigned long long)out);
                }
                ++i;
            }
            ++j;
        }
    }
}

// Stencil values of one particle into val[0 .. NX*NX) (row-major j, i), zeros
// elsewhere; the values add up exactly to the particle's A = rint(qn * 2^24)
// units (the largest-weight node takes the rounding remainder). Returns false
// if the particle took the general Esirkepov path (already deposited, val all
// zero).
template <int S>
__device__ __forceinline__ bool stencil_values(const DepArgs& a, float rx, float ry, float qn, float vxx, float vyy,
                                               int ix, int iy, size_t p, int (&val)[Frame<S>::V]) {
    constexpr int NX = Frame<S>::NX, V = Frame<S>::V;
    const float aq = qn * 16777216.0f;
    const int A = __float2int_rn(aq);
    float X[NX], Y[NX];
    const bool okx = axis_frame<S>(rx, vxx, a.dtf, a.dtdx, X);
    const bool oky = axis_frame<S>(ry, vyy, a.dtf, a.dtdy, Y);
#pragma unroll
    for (int k = 0; k < V; ++k) val[k] = 0;
    if (!(okx && oky)) {
        esk_general_deposit(a, ix, iy, aq, A, rx, ry, vxx, vyy, p);
        return false;
    }
    int sum = 0;
#pragma unroll
    for (int j = 0; j < NX; ++j) {
        const float ay = aq * Y[j];
#pragma unroll
        for (int i = 0; i < NX; ++i) {
            val[j * NX + i] = __float2int_rn(ay * X[i]);
            sum += val[j * NX + i];
        }
    }
    // TSC: the particle's own cell node (frame entry (1,1)); else the first largest weight
    const int kmaj = S == S_TSC ? NX + 1 : first_max(Y) * NX + first_max(X);
    const int rem = A - sum;
#pragma unroll
    for (int k = 0; k < NX * NX; ++k) val[k] += (k == kmaj) ? rem : 0;
    return true;
}

template <int S>
__device__ __forceinline__ bool particle_values(const DepArgs& a, size_t p, int ix, int iy,
                                                int (&val)[Frame<S>::V]) {
    const float rx = __ldcs(a.xr + p), ry = __ldcs(a.yr + p);
    const float qn = a.qc != 0.0f ? a.qc : __ldcs(a.q + p);
    float vxx = 0.0f, vyy = 0.0f;
    if constexpr (S == S_ESK) {
        vxx = __ldcs(a.vx + p);
        vyy = __ldcs(a.vy + p);
    }
    return stencil_values<S>(a, rx, ry, qn, vxx, vyy, ix, iy, p, val);
}

constexpr uint32_t NO_CELL = 0xffffffffu;

// Four consecutive particles of each field, one 128-bit streaming load per field.
template <int S>
struct Quad {
    uint4 cell;
    float4 xr, yr, q, vx, vy;
};

template <int S>
__device__ __forceinline__ void load_quad(const DepArgs& a, uint32_t p0, bool ok, Quad<S>& d) {
    if (ok) {
        d.cell = __ldcs(reinterpret_cast<const uint4*>(a.cell + p0));
        d.xr = __ldcs(reinterpret_cast<const float4*>(a.xr + p0));
        d.yr = __ldcs(reinterpret_cast<const float4*>(a.yr + p0));
        d.q = a.qc != 0.0f ? make_float4(a.qc, a.qc, a.qc, a.qc) : __ldcs(reinterpret_cast<const float4*>(a.q + p0));
        if constexpr (S == S_ESK) {
            d.vx = __ldcs(reinterpret_cast<const float4*>(a.vx + p0));
            d.vy = __ldcs(reinterpret_cast<const float4*>(a.vy + p0));
        }
    }
}

__device__ __forceinline__ uint32_t u4(const uint4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
__device__ __forceinline__ float f4(const float4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }

// Adds a lane's sums for cell `key` straight to the global grid.
template <int S>
__device__ __forceinline__ void flush_global(const DepArgs& a, uint32_t key, const int (&acc)[Frame<S>::NX * Frame<S>::NX]) {
    constexpr int NX = Frame<S>::NX, LO = Frame<S>::LO;
    const int iy = (int)(key / (uint32_t)a.Nx), ix = (int)(key - (uint32_t)iy * (uint32_t)a.Nx);
#pragma unroll
    for (int j = 0; j < NX; ++j) {
        const size_t row = (size_t)wrap_i(iy + LO + j, a.Ny) * a.Nx;
#pragma unroll
        for (int i = 0; i < NX; ++i) {
            const int v = acc[j * NX + i];
            if (v != 0) atomicAdd(a.acc + row + wrap_i(ix + LO + i, a.Nx), (unsigned long long)(long long)v);
        }
    }
}

// flush_global without integer division (the any-order kernels flush once per
// run of a warp step; measured faster there, while the tiled kernel keeps the
// plain form above).
template <int S>
__device__ __forceinline__ void flush_global_nd(const DepArgs& a, uint32_t key, float inv_nx,
                                                const int (&acc)[Frame<S>::NX * Frame<S>::NX]) {
    constexpr int NX = Frame<S>::NX, LO = Frame<S>::LO;
    int iy, ix;
    split_key(key, a.Nx, inv_nx, iy, ix);
#pragma unroll
    for (int j = 0; j < NX; ++j) {
        const size_t row = (size_t)wrap_near(iy + LO + j, a.Ny) * a.Nx;
#pragma unroll
        for (int i = 0; i < NX; ++i) {
            const int v = acc[j * NX + i];
            if (v != 0) atomicAdd(a.acc + row + wrap_near(ix + LO + i, a.Nx), (unsigned long long)(long long)v);
        }
    }
}

// Any-order path with run aggregation: a warp step of 128 consecutive particles
// (4 per lane, register sums per cell, segmented warp scan) over the whole
// particle array, with the run totals added straight to the global int64 grid. It needs no per-cell offsets and is correct for any order;
// runs are long when the particles are nearly cell-ordered, as between the
// sorts of a time-stepping loop.
template <int S>
__global__ void __launch_bounds__(DEP_THREADS) deposit_runs(DepArgs a) {
    if (gated_off(a)) return;
    constexpr int NX = Frame<S>::NX, V = Frame<S>::V;
    constexpr int NV = NX * NX;
    const int lane = threadIdx.x & 31;
    const size_t gw = (size_t)blockIdx.x * DEP_WARPS + (threadIdx.x >> 5);
    const size_t stride = (size_t)gridDim.x * DEP_WARPS * 128;
    const uint32_t G = (uint32_t)a.Nx * (uint32_t)a.Ny;
    const float inv_nx = 1.0f / (float)a.Nx;
    const unsigned upto = (lane == 31) ? FULL : ((2u << lane) - 1u);
    size_t base = gw * 128;
    Quad<S> cur, nxt;
    load_quad<S>(a, (uint32_t)(base + 4u * lane), base + 4u * lane < a.n, cur);
    for (; base < a.n; base += stride) {
        const size_t nbase = base + stride;
        if (nbase < a.n) load_quad<S>(a, (uint32_t)(nbase + 4u * lane), nbase + 4u * lane < a.n, nxt);
        uint32_t ckey = NO_CELL;
        int acc[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const size_t p = base + 4u * lane + (size_t)k;
            if (p < a.n) {
                const uint32_t key = u4(cur.cell, k);
                if (key >= G) {
                    set_dev_error(a.st, DEV_BAD_CELL, (unsigned)p);
                    continue;
                }
                int iy, ixk;
                split_key(key, a.Nx, inv_nx, iy, ixk);
                int val[V];
                float vxx = 0.0f, vyy = 0.0f;
                if constexpr (S == S_ESK) {
                    vxx = f4(cur.vx, k);
                    vyy = f4(cur.vy, k);
                }
                if (!stencil_values<S>(a, f4(cur.xr, k), f4(cur.yr, k), f4(cur.q, k), vxx, vyy,
                                       ixk, iy, p, val))
                    continue;
                if (key != ckey) {
                    if (ckey != NO_CELL) flush_global_nd<S>(a, ckey, inv_nx, acc);
                    ckey = key;
#pragma unroll
                    for (int q = 0; q < NV; ++q) acc[q] = val[q];
                } else {
#pragma unroll
                    for (int q = 0; q < NV; ++q) acc[q] += val[q];
                }
            }
        }
        const uint32_t kprev = __shfl_up_sync(FULL, ckey, 1);
        // a segment never spans lanes 15|16: a run total covers at most 64
        // particles, |total| <= 64 * (2^24 + 3) < 2^31
        const unsigned H = __ballot_sync(FULL, lane == 0 || lane == 16 || ckey != kprev);
        const int segstart = 31 - __clz(H & upto);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const bool take = lane - d >= segstart;
#pragma unroll
            for (int q = 0; q < NV; ++q) {
                const int o = __shfl_up_sync(FULL, acc[q], d);
                if (take) acc[q] += o;
            }
        }
        const bool tail = (lane == 31) || ((H >> (lane + 1)) & 1u);
        if (tail && ckey != NO_CELL) flush_global_nd<S>(a, ckey, inv_nx, acc);
        cur = nxt;
    }
}

__device__ __forceinline__ void tsci_particle_to_global(const DepArgs& a, uint32_t key, float rx, float ry);

template <int S>
__global__ void __launch_bounds__(DEP_THREADS) deposit_atomic(DepArgs a) {
    constexpr int NX = Frame<S>::NX, LO = Frame<S>::LO, V = Frame<S>::V;
    const uint32_t G = (uint32_t)a.Nx * (uint32_t)a.Ny;
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += (size_t)gridDim.x * blockDim.x) {
        const uint32_t key = __ldcs(a.cell + p);
        if (key >= G) {
            set_dev_error(a.st, DEV_BAD_CELL, (unsigned)p);
            continue;
        }
        if constexpr (S == S_TSC) {
            if (a.qc != 0.0f) {  // one charge for all particles: exact integer weights
                tsci_particle_to_global(a, key, __ldcs(a.xr + p), __ldcs(a.yr + p));
                continue;
            }
        }
        const int iy = (int)(key / (uint32_t)a.Nx), ix = (int)(key - (uint32_t)iy * (uint32_t)a.Nx);
        int val[V];
        if (!particle_values<S>(a, p, ix, iy, val)) continue;
#pragma unroll
        for (int j = 0; j < NX; ++j) {
            const size_t row = (size_t)wrap_i(iy + LO + j, a.Ny) * a.Nx;
#pragma unroll
            for (int i = 0; i < NX; ++i) {
                const int v = val[j * NX + i];
                if (v != 0)
                    atomicAdd(a.acc + row + wrap_i(ix + LO + i, a.Nx), (unsigned long long)(long long)v);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// TSC fast paths. Same values as stencil_values<TSC> bit for bit, fewer
// instructions:
//  * the weights are computed without branching on r < 0.5: with t = r (r < 0.5)
//    or t = r - 1 (r >= 0.5), the three non-zero weights are 0.5*(0.5-t)^2,
//    0.75-t^2, 0.5*(0.5+t)^2 at frame columns 0..2 or 1..3 (each operation gives
//    the bits the branchy form gives: r - 1, 0.5 - t and 0.5 + t are exact there);
//  * the remainder goes to frame entry (1,1), the particle's own cell node;
//  * the 12 entries outside rows and columns 1..2 involve an outer weight <= 1/8,
//    so |value| < 2^22 and rint is one FP32 add of 1.5*2^23 (round to nearest
//    even on the integer grid): the accumulators keep those entries with the
//    constant's bits added once per particle, and the per-run particle count
//    removes them when a total is written out. The 4 central entries use F2I.
// ---------------------------------------------------------------------------
constexpr float TSC_MAGIC = 12582912.0f;     // 1.5 * 2^23
constexpr uint32_t TSC_MAGIC_BITS = 0x4B400000u;

__host__ __device__ constexpr bool tsc_central(int k) { return ((k >> 2) == 1 || (k >> 2) == 2) && ((k & 3) == 1 || (k & 3) == 2); }

// Paired FP32 arithmetic (two lanes of a 64-bit register, each IEEE
// round-to-nearest like the scalar instruction): the x and y axes, or two
// frame entries, in one instruction. A paired multiply is never followed by a
// paired add or subtract of its result: the assembler fuses such a pair into
// one multiply-add (one rounding) even with explicit .rn, which would change
// the bits; those adds are scalar (add.rn.f32, never contracted).
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f32x2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// ---------------------------------------------------------------------------
// TSC with one charge for every particle: exact integer weights.
// Per axis, with t = r (r < 0.5) or r - 1 (r >= 0.5) as above, the outer
// weights are WL = rint(2^14 (0.5 - t)^2) and WR = rint(2^14 (0.5 + t)^2),
// each one FP32 fma (d * (d * 2^14) + 1.5*2^23: the product is exact, the sum
// rounds once to the nearest even integer), and WC = 2^15 - WL - WR, so an
// axis' three weights sum to 2^15 exactly (tscWeights, ngp.cpp:28-34, at
// 2^-15 resolution: rho within about 2.3e-6 relative L2 of the FP64 deposit at
// 64 particles per cell). A frame value WX[i] * WY[j] is an exact integer
// product (no rounding, no remainder step) and a particle deposits exactly
// 2^30 units; the charge and its sign sit in the unit, qn * max|q| * inv_vol *
// 2^-30. Bounds: the 12 frame entries outside the central 2x2 are at most
// 2^12 * 24576 < 2^26.6 per particle (32-bit sums for runs of up to 32
// particles); the central 4 at most 24576^2 = 0.5625 * 2^30 (64-bit sums).
// ---------------------------------------------------------------------------
constexpr uint32_t TSCI_ONE = 1u << 15;

__device__ __forceinline__ void tsci_weights(float rx, float ry, uint32_t (&X)[4], uint32_t (&Y)[4]) {
    const bool sx = rx >= 0.5f, sy = ry >= 0.5f;
    float mx, my;
    f2_unpack(f2_add(f2_pack(rx, ry), f2_pack(-1.0f, -1.0f)), mx, my);
    const f32x2 t = f2_pack(sx ? mx : rx, sy ? my : ry);
    const f32x2 half = f2_pack(0.5f, 0.5f);
    const f32x2 dl = f2_sub(half, t), dr = f2_add(half, t);
    const f32x2 s14 = f2_pack(16384.0f, 16384.0f), mag = f2_pack(TSC_MAGIC, TSC_MAGIC);
    const f32x2 wl = f2_fma(dl, f2_mul(dl, s14), mag), wr = f2_fma(dr, f2_mul(dr, s14), mag);
    float lx, ly, rxw, ryw;
    f2_unpack(wl, lx, ly);
    f2_unpack(wr, rxw, ryw);
    const uint32_t WLx = __float_as_uint(lx) - TSC_MAGIC_BITS, WLy = __float_as_uint(ly) - TSC_MAGIC_BITS;
    const uint32_t WRx = __float_as_uint(rxw) - TSC_MAGIC_BITS, WRy = __float_as_uint(ryw) - TSC_MAGIC_BITS;
    const uint32_t WCx = TSCI_ONE - WLx - WRx, WCy = TSCI_ONE - WLy - WRy;
    X[0] = sx ? 0u : WLx;
    X[1] = sx ? WLx : WCx;
    X[2] = sx ? WCx : WRx;
    X[3] = sx ? WRx : 0u;
    Y[0] = sy ? 0u : WLy;
    Y[1] = sy ? WLy : WCy;
    Y[2] = sy ? WCy : WRy;
    Y[3] = sy ? WRy : 0u;
}

// c + a * b in 64 bits, one multiply-add (a widening multiply followed by a
// separate 64-bit add takes three instructions)
__device__ __forceinline__ unsigned long long mad_wide(uint32_t a, uint32_t b, unsigned long long c) {
    unsigned long long d;
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
}

// Frame entry q (row-major j*4+i) -> slot among the 12 outer or the 4 central entries.
__host__ __device__ constexpr int tsci_outer_slot(int q) { return q < 5 ? q : q < 7 ? 4 : q < 8 ? 5 : q < 9 ? 6 : q < 11 ? 7 : q - 4; }
__host__ __device__ constexpr int tsci_central_slot(int q) { return q == 5 ? 0 : q == 6 ? 1 : q == 9 ? 2 : 3; }

// The frame sums of a run of particles of one cell (exact).
struct TscIntSums {
    uint32_t o[12];
    unsigned long long c[4];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int k = 0; k < 12; ++k) o[k] = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) c[k] = 0;
    }
    __device__ __forceinline__ void add(float rx, float ry) {
        uint32_t X[4], Y[4];
        tsci_weights(rx, ry, X, Y);
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int q = j * 4 + i;
                if (tsc_central(q))
                    c[tsci_central_slot(q)] = mad_wide(X[i], Y[j], c[tsci_central_slot(q)]);
                else
                    o[tsci_outer_slot(q)] += X[i] * Y[j];
            }
    }
    __device__ __forceinline__ long long get(int q) const {
        return tsc_central(q) ? (long long)c[tsci_central_slot(q)] : (long long)o[tsci_outer_slot(q)];
    }
};

// Frame values: central entries exact, the others biased by TSC_MAGIC_BITS.
// Both axes' weights are computed as pairs (x, y) and the products of a frame
// row as pairs of columns.
__device__ __forceinline__ void tsc_accumulate(float rx, float ry, float qn, uint32_t (&acc)[16]) {
    const float aq = qn * 16777216.0f;
    const int A = __float2int_rn(aq);
    const bool sx = rx >= 0.5f, sy = ry >= 0.5f;
    float mx, my;
    f2_unpack(f2_add(f2_pack(rx, ry), f2_pack(-1.0f, -1.0f)), mx, my);
    const f32x2 t = f2_pack(sx ? mx : rx, sy ? my : ry);
    const f32x2 half = f2_pack(0.5f, 0.5f);
    const f32x2 dl = f2_sub(half, t), dr = f2_add(half, t);
    const f32x2 L2 = f2_mul(half, f2_mul(dl, dl));
    float ttx, tty;
    f2_unpack(f2_mul(t, t), ttx, tty);
    const f32x2 C2 = f2_pack(0.75f - ttx, 0.75f - tty);
    const f32x2 R2 = f2_mul(half, f2_mul(dr, dr));
    float Lx, Ly, Cx, Cy, Rx, Ry;
    f2_unpack(L2, Lx, Ly);
    f2_unpack(C2, Cx, Cy);
    f2_unpack(R2, Rx, Ry);
    const float X0 = sx ? 0.0f : Lx, X1 = sx ? Lx : Cx, X2 = sx ? Cx : Rx, X3 = sx ? Rx : 0.0f;
    const float Y0 = sy ? 0.0f : Ly, Y1 = sy ? Ly : Cy, Y2 = sy ? Cy : Ry, Y3 = sy ? Ry : 0.0f;
    const f32x2 aq2 = f2_pack(aq, aq);
    float ay[4];
    f2_unpack(f2_mul(aq2, f2_pack(Y0, Y1)), ay[0], ay[1]);
    f2_unpack(f2_mul(aq2, f2_pack(Y2, Y3)), ay[2], ay[3]);
    const f32x2 x01 = f2_pack(X0, X1), x23 = f2_pack(X2, X3);
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const f32x2 ayj = f2_pack(ay[j], ay[j]);
        const f32x2 p01 = f2_mul(ayj, x01), p23 = f2_mul(ayj, x23);
        float v0, v1, v2, v3;
        f2_unpack(p01, v0, v1);
        f2_unpack(p23, v2, v3);
        uint32_t e0, e1, e2, e3;
        if (j == 0 || j == 3) {
            e0 = __float_as_uint(v0 + TSC_MAGIC);
            e1 = __float_as_uint(v1 + TSC_MAGIC);
            e2 = __float_as_uint(v2 + TSC_MAGIC);
            e3 = __float_as_uint(v3 + TSC_MAGIC);
        } else {
            e0 = __float_as_uint(v0 + TSC_MAGIC);
            e1 = (uint32_t)__float2int_rn(v1);
            e2 = (uint32_t)__float2int_rn(v2);
            e3 = __float_as_uint(v3 + TSC_MAGIC);
        }
        acc[j * 4 + 0] += e0;
        acc[j * 4 + 1] += e1;
        acc[j * 4 + 2] += e2;
        acc[j * 4 + 3] += e3;
        sum += e0 + e1 + e2 + e3;
    }
    acc[5] += (uint32_t)A - (sum - 12u * TSC_MAGIC_BITS);  // the remainder: own cell node
}

// One particle's frame values (tsc_accumulate into zeros).
__device__ __forceinline__ void tsc_values(float rx, float ry, float qn, uint32_t (&val)[16]) {
#pragma unroll
    for (int q = 0; q < 16; ++q) val[q] = 0;
    tsc_accumulate(rx, ry, qn, val);
}

// True total of entry q of a run of `cnt` particles.
__device__ __forceinline__ int tsc_true(int q, uint32_t acc, uint32_t cnt) {
    return tsc_central(q) ? (int)acc : (int)(acc - cnt * TSC_MAGIC_BITS);
}

// Adds one particle's exact integer TSC values (one charge for all particles)
// straight to the global grid.
__device__ __forceinline__ void tsci_particle_to_global(const DepArgs& a, uint32_t key, float rx, float ry) {
    const int iy = (int)(key / (uint32_t)a.Nx), ix = (int)(key - (uint32_t)iy * (uint32_t)a.Nx);
    uint32_t X[4], Y[4];
    tsci_weights(rx, ry, X, Y);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const size_t row = (size_t)wrap_i(iy - 1 + j, a.Ny) * a.Nx;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const unsigned long long v = (unsigned long long)X[i] * Y[j];
            if (v != 0) atomicAdd(a.acc + row + wrap_i(ix - 1 + i, a.Nx), v);
        }
    }
}

// A particle outside the tile row whose slice of the stream holds it (the cell
// ranges are those of an earlier sort and the particle has moved since): its
// values go straight to the global int64 grid.
template <int S, bool QC>
__device__ __forceinline__ void particle_to_global(const DepArgs& a, uint32_t key, float rx, float ry, float qn,
                                                float vxx, float vyy, uint32_t p) {
    constexpr int NV = Frame<S>::NX * Frame<S>::NX;
    if (key >= (uint32_t)a.Nx * (uint32_t)a.Ny) {
        set_dev_error(a.st, DEV_BAD_CELL, p);
        return;
    }
    if constexpr (S == S_TSC && QC) {
        tsci_particle_to_global(a, key, rx, ry);
        return;
    }
    const int iy = (int)(key / (uint32_t)a.Nx), ix = (int)(key - (uint32_t)iy * (uint32_t)a.Nx);
    int tv[NV];
    if constexpr (S == S_TSC) {
        uint32_t val[16];
        tsc_values(rx, ry, qn, val);
#pragma unroll
        for (int q = 0; q < 16; ++q) tv[q] = tsc_true(q, val[q], 1u);
    } else {
        int iv[Frame<S>::V];
        if (!stencil_values<S>(a, rx, ry, qn, vxx, vyy, ix, iy, p, iv)) return;
#pragma unroll
        for (int q = 0; q < NV; ++q) tv[q] = iv[q];
    }
    flush_global<S>(a, key, tv);
}

// Adds a lane's run totals for cell `key` (64-bit values) straight to the global grid.
template <int NX, int LO, int NV>
__device__ __forceinline__ void flush_global_ll(const DepArgs& a, uint32_t key, const long long (&tv)[NV]) {
    const int iy = (int)(key / (uint32_t)a.Nx), ix = (int)(key - (uint32_t)iy * (uint32_t)a.Nx);
#pragma unroll
    for (int j = 0; j < NX; ++j) {
        const size_t row = (size_t)wrap_i(iy + LO + j, a.Ny) * a.Nx;
#pragma unroll
        for (int i = 0; i < NX; ++i) {
            const long long v = tv[j * NX + i];
            if (v != 0) atomicAdd(a.acc + row + wrap_i(ix + LO + i, a.Nx), (unsigned long long)v);
        }
    }
}

// Fields of a particle staged by the sorted kernel: cell, xr, yr, q (not when
// one charge is shared), vx, vy (Esirkepov).
template <int S, bool QC>
struct StageFields {
    static constexpr int NF = (S == S_ESK ? 6 : 4) - (QC ? 1 : 0);
};

// Tile accumulators: 64-bit shared atomics are not native (they compile to
// compare-and-swap loops), so a cell's total v is added as two native 32-bit
// shared atomics, v & (2^15-1) to an unsigned low word and v >> 15 to a high
// word; the node's total is hi * 2^15 + lo. A node receives at most 16
// additions per cell (one per neighbouring cell), so the low words stay exact;
// the high words stay exact while the tile holds fewer than 2^17 particles
// (signed, |value| <= 2^24 + 3 per particle and node in the general form;
// unsigned in the exact integer TSC form, at most 0.5625 * 2^30 per particle).
// Denser tiles add their cells' totals straight to the global int64 grid.
constexpr int TILE_SPLIT = 15;
constexpr uint32_t TILE_SPLIT_MAX = 1u << 17;  // particles per tile for the split accumulators

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Adds a run's exact integer TSC totals for cell `key` straight to the global
// grid, without integer division (as flush_global_nd).
__device__ __forceinline__ void tsci_flush_global_nd(const DepArgs& a, uint32_t key, float inv_nx, const TscIntSums& s) {
    int iy, ix;
    split_key(key, a.Nx, inv_nx, iy, ix);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const size_t row = (size_t)wrap_near(iy - 1 + j, a.Ny) * a.Nx;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const unsigned long long v = (unsigned long long)s.get(j * 4 + i);
            if (v != 0) atomicAdd(a.acc + row + wrap_near(ix - 1 + i, a.Nx), v);
        }
    }
}

// Any-order path for TSC with one charge for all particles (exact integer
// weights): the warp step of deposit_runs with the run sums of TscIntSums. The
// scan's segments stop at lanes 8, 16 and 24, so a run total covers at most 32
// particles and the 12 outer entries stay below 32 * 2^26.6 < 2^32.
__global__ void __launch_bounds__(DEP_THREADS, 4) deposit_runs_tsci(DepArgs a) {
    if (gated_off(a)) return;
    const int lane = threadIdx.x & 31;
    const size_t gw = (size_t)blockIdx.x * DEP_WARPS + (threadIdx.x >> 5);
    const size_t stride = (size_t)gridDim.x * DEP_WARPS * 128;
    const uint32_t G = (uint32_t)a.Nx * (uint32_t)a.Ny;
    const float inv_nx = 1.0f / (float)a.Nx;
    const unsigned upto = (lane == 31) ? FULL : ((2u << lane) - 1u);
    size_t base = gw * 128;
    Quad<S_TSC> cur, nxt;
    load_quad<S_TSC>(a, (uint32_t)(base + 4u * lane), base + 4u * lane < a.n, cur);
    for (; base < a.n; base += stride) {
        const size_t nbase = base + stride;
        if (nbase < a.n) load_quad<S_TSC>(a, (uint32_t)(nbase + 4u * lane), nbase + 4u * lane < a.n, nxt);
        uint32_t ckey = NO_CELL;
        TscIntSums s;
        s.zero();
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const size_t p = base + 4u * lane + (size_t)k;
            if (p < a.n) {
                const uint32_t key = u4(cur.cell, k);
                if (key >= G) {
                    set_dev_error(a.st, DEV_BAD_CELL, (unsigned)p);
                    continue;
                }
                if (key != ckey) {
                    if (ckey != NO_CELL) tsci_flush_global_nd(a, ckey, inv_nx, s);
                    ckey = key;
                    s.zero();
                }
                s.add(f4(cur.xr, k), f4(cur.yr, k));
            }
        }
        const uint32_t kprev = __shfl_up_sync(FULL, ckey, 1);
        const unsigned H = __ballot_sync(FULL, (lane & 7) == 0 || ckey != kprev);
        const int segstart = 31 - __clz(H & upto);
#pragma unroll
        for (int d = 1; d < 8; d <<= 1) {
            const bool take = lane - d >= segstart;
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                const uint32_t o = __shfl_up_sync(FULL, s.o[k], d);
                if (take) s.o[k] += o;
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned long long o = __shfl_up_sync(FULL, s.c[k], d);
                if (take) s.c[k] += o;
            }
        }
        const bool tail = (lane == 31) || ((H >> (lane + 1)) & 1u);
        if (tail && ckey != NO_CELL) tsci_flush_global_nd(a, ckey, inv_nx, s);
        cur = nxt;
    }
}

// Any-order path for TSC (deposit_runs with the values above). Capped at 64
// registers (4 CTAs per SM, a few spilled words): latency-bound, it measured 7 %
// faster per 2048^2 time step than with 80 registers and 3 CTAs.
__global__ void __launch_bounds__(DEP_THREADS, 4) deposit_runs_tsc(DepArgs a) {
    if (gated_off(a)) return;
    const int lane = threadIdx.x & 31;
    const size_t gw = (size_t)blockIdx.x * DEP_WARPS + (threadIdx.x >> 5);
    const size_t stride = (size_t)gridDim.x * DEP_WARPS * 128;
    const uint32_t G = (uint32_t)a.Nx * (uint32_t)a.Ny;
    const float inv_nx = 1.0f / (float)a.Nx;
    const unsigned upto = (lane == 31) ? FULL : ((2u << lane) - 1u);
    size_t base = gw * 128;
    Quad<S_TSC> cur, nxt;
    load_quad<S_TSC>(a, (uint32_t)(base + 4u * lane), base + 4u * lane < a.n, cur);
    for (; base < a.n; base += stride) {
        const size_t nbase = base + stride;
        if (nbase < a.n) load_quad<S_TSC>(a, (uint32_t)(nbase + 4u * lane), nbase + 4u * lane < a.n, nxt);
        uint32_t ckey = NO_CELL, cnt = 0;
        uint32_t acc[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const size_t p = base + 4u * lane + (size_t)k;
            if (p < a.n) {
                const uint32_t key = u4(cur.cell, k);
                if (key >= G) {
                    set_dev_error(a.st, DEV_BAD_CELL, (unsigned)p);
                    continue;
                }
                if (key != ckey) {
                    if (ckey != NO_CELL) {
                        int t[16];
#pragma unroll
                        for (int q = 0; q < 16; ++q) t[q] = tsc_true(q, acc[q], cnt);
                        flush_global_nd<S_TSC>(a, ckey, inv_nx, t);
                    }
                    ckey = key;
                    cnt = 0;
#pragma unroll
                    for (int q = 0; q < 16; ++q) acc[q] = 0;
                }
                tsc_accumulate(f4(cur.xr, k), f4(cur.yr, k), f4(cur.q, k), acc);
                ++cnt;
            }
        }
        const uint32_t kprev = __shfl_up_sync(FULL, ckey, 1);
        // a segment never spans lanes 15|16: a run total covers at most 64
        // particles, |total| <= 64 * (2^24 + 3) < 2^31
        const unsigned H = __ballot_sync(FULL, lane == 0 || lane == 16 || ckey != kprev);
        const int segstart = 31 - __clz(H & upto);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const bool take = lane - d >= segstart;
            const uint32_t oc = __shfl_up_sync(FULL, cnt, d);
            if (take) cnt += oc;
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const uint32_t o = __shfl_up_sync(FULL, acc[q], d);
                if (take) acc[q] += o;
            }
        }
        const bool tail = (lane == 31) || ((H >> (lane + 1)) & 1u);
        if (tail && ckey != NO_CELL) {
            int t[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) t[q] = tsc_true(q, acc[q], cnt);
            flush_global_nd<S_TSC>(a, ckey, inv_nx, t);
        }
        cur = nxt;
    }
}

// ---------------------------------------------------------------------------
// Sorted path, cell form (deposit_cells). One CTA of NW warps per tile of
// tile_w x tile_h cells; the tile's rows are cut into units of up to 32
// consecutive cells and warp w walks units w, w+NW, ... Lane l of a unit owns
// one cell: the contiguous range [offsets[c], offsets[c+1]) of the cell-sorted
// stream, which it walks in stages of LPP particles.
//  * Staging: each stage's quads (4 particles, from the 16-byte boundary at or
//    below the cell's first particle) are copied global -> shared with
//    cp.async, 16 bytes per lane, field and quad, into [field][quad][lane]
//    slots (the copies and the lanes' 128-bit reads are conflict-free); two
//    stage buffers per warp, the next stage -- or the next unit's first -- in
//    flight while this one is used. A unit takes as many stages as its fullest
//    cell; lanes whose cell is done idle.
//  * A lane's particles all belong to its cell, so there are no runs to detect
//    and no cell keys to read: the offsets name every particle's cell (KEYS =
//    false, a fresh sort). After particles have moved since the sort (KEYS =
//    true, between the sorts of a time-stepping loop) the keys are read;
//    particles that left their cell are queued per warp (ballot compaction
//    into shared memory) and, after the stage, all lanes deposit them straight
//    to the global grid, one per lane (no divergent per-particle path).
//  * Sums: per stage in 32 bits (at most LPP particles), added to 64-bit cell
//    totals at the end of each stage (CellRun); the exact integer TSC form
//    keeps 9 of its 16 entries and 6 axis sums (see CellRun<S_TSC, true>).
//  * Each lane writes its cell's totals out once: to the tile's split 32-bit
//    shared accumulators (adjacent lanes hit different nodes: no same-address
//    conflicts), or, in a tile of 2^17 particles or more, to the global grid.
// At the end the tile is added to the global int64 grid once.
// ---------------------------------------------------------------------------
template <int S, bool QC>
struct CellRun {
    static constexpr int NV = Frame<S>::NX * Frame<S>::NX;
    uint32_t v[NV];   // this stage's sums (TSC: outer entries biased, see tsc_accumulate)
    long long T[NV];  // the cell's totals
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            v[q] = 0;
            T[q] = 0;
        }
    }
    __device__ __forceinline__ void end_quad() {}
    __device__ __forceinline__ void finish() {}
    // adds the sums of a stage (`cnt` particles) to the totals
    __device__ __forceinline__ void end_stage(uint32_t cnt, bool) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            if constexpr (S == S_TSC)
                T[q] += tsc_true(q, v[q], cnt);
            else
                T[q] += (int)v[q];
            v[q] = 0;
        }
    }
    __device__ __forceinline__ void totals(uint32_t, long long (&A)[NV]) const {
#pragma unroll
        for (int q = 0; q < NV; ++q) A[q] = T[q];
    }
};

// TSC with one charge for all particles. Every particle's frame is X (x) Y
// with sum_i X[i] = sum_j Y[j] = 2^15, so a cell's 4x4 sums A[j][i] have row
// sums 2^15 * SY[j] and column sums 2^15 * SX[i] (SX, SY: the sums of each
// axis' weights). The lane keeps the 9 entries A[j][i] with i, j in {0, 1, 3}
// and the axis sums SX[0,1,3], SY[0,1,3]; row 2, column 2 and SX[2], SY[2]
// follow exactly (integer identities) when the cell is written out. Per
// particle: 9 32-bit multiply-adds and 6 adds. Bounds: the 8 entries other than
// A[1][1] are at most 2^12 * 24576 < 2^26.6 per particle, summed in 32 bits for
// at most 32 particles (32/LPP stages) and then added to 64-bit totals; A[1][1] <=
// 24576^2 < 2^29.2 per particle is summed in 32 bits for a quad (4 particles);
// the axis sums are 64-bit totals of 32-bit sums of as many stages.
template <>
struct CellRun<S_TSC, true> {
    static constexpr int NV = 16;
    uint32_t e[8], c11;            // partial sums of the current stage / quad
    unsigned long long E[8], C11;  // A00 A01 A03 A10 A13 A30 A31 A33, A11
    uint32_t sx0, sx1, sx3, sy0, sy1, sy3;
    unsigned long long SX0, SX1, SX3, SY0, SY1, SY3;
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            e[k] = 0;
            E[k] = 0;
        }
        c11 = 0;
        C11 = 0;
        sx0 = sx1 = sx3 = sy0 = sy1 = sy3 = 0;
        SX0 = SX1 = SX3 = SY0 = SY1 = SY3 = 0;
    }
    __device__ __forceinline__ void add(float rx, float ry) {
        uint32_t X[4], Y[4];
        tsci_weights(rx, ry, X, Y);
        e[0] += X[0] * Y[0];
        e[1] += X[1] * Y[0];
        e[2] += X[3] * Y[0];
        e[3] += X[0] * Y[1];
        e[4] += X[3] * Y[1];
        e[5] += X[0] * Y[3];
        e[6] += X[1] * Y[3];
        e[7] += X[3] * Y[3];
        c11 += X[1] * Y[1];
        sx0 += X[0];
        sx1 += X[1];
        sx3 += X[3];
        sy0 += Y[0];
        sy1 += Y[1];
        sy3 += Y[3];
    }
    __device__ __forceinline__ void end_quad() {
        C11 += c11;
        c11 = 0;
    }
    // partial sums -> 64-bit totals (every 4 stages: at most 32 particles, 2^31.6)
    __device__ __forceinline__ void fold() {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            E[k] += e[k];
            e[k] = 0;
        }
        SX0 += sx0;
        SX1 += sx1;
        SX3 += sx3;
        SY0 += sy0;
        SY1 += sy1;
        SY3 += sy3;
        sx0 = sx1 = sx3 = sy0 = sy1 = sy3 = 0;
    }
    __device__ __forceinline__ void end_stage(uint32_t, bool fold_now) {
        if (fold_now) fold();
    }
    __device__ __forceinline__ void finish() { fold(); }
    // the 16 totals of n particles, row-major A[j][i] (after finish)
    __device__ __forceinline__ void totals(uint32_t n, long long (&A)[16]) const {
        const long long one = (long long)TSCI_ONE;
        A[0] = (long long)E[0];
        A[1] = (long long)E[1];
        A[3] = (long long)E[2];
        A[4] = (long long)E[3];
        A[5] = (long long)C11;
        A[7] = (long long)E[4];
        A[12] = (long long)E[5];
        A[13] = (long long)E[6];
        A[15] = (long long)E[7];
        const long long sy2 = (long long)n * one - (long long)(SY0 + SY1 + SY3);
        A[2] = one * (long long)SY0 - A[0] - A[1] - A[3];
        A[6] = one * (long long)SY1 - A[4] - A[5] - A[7];
        A[14] = one * (long long)SY3 - A[12] - A[13] - A[15];
        A[8] = one * (long long)SX0 - A[0] - A[4] - A[12];
        A[9] = one * (long long)SX1 - A[1] - A[5] - A[13];
        A[11] = one * (long long)SX3 - A[3] - A[7] - A[15];
        A[10] = one * sy2 - A[8] - A[9] - A[11];
    }
};

// NGP with one charge for all particles: every particle deposits exactly
// A = rint(qn * 2^24) units to its nearest node (ngp.cpp:108-120, ties go up),
// so a cell's four node sums are A times the counts of its particles in each
// quarter of the cell: the general form's values bit for bit, from two
// comparisons and three counts per particle.
template <>
struct CellRun<S_NGP, true> {
    static constexpr int NV = 4;
    int A;                 // the units of one particle
    uint32_t nx, ny, nxy;  // particles with rx >= 0.5, ry >= 0.5, both
    __device__ __forceinline__ void zero() { nx = ny = nxy = 0; }
    __device__ __forceinline__ void add(float rx, float ry) {
        const uint32_t sx = rx >= 0.5f ? 1u : 0u, sy = ry >= 0.5f ? 1u : 0u;
        nx += sx;
        ny += sy;
        nxy += sx & sy;
    }
    __device__ __forceinline__ void end_quad() {}
    __device__ __forceinline__ void end_stage(uint32_t, bool) {}
    __device__ __forceinline__ void finish() {}
    __device__ __forceinline__ void totals(uint32_t n, long long (&T)[4]) const {
        const long long a = A;
        T[0] = a * ((long long)n - nx - ny + nxy);
        T[1] = a * ((long long)nx - nxy);
        T[2] = a * ((long long)ny - nxy);
        T[3] = a * (long long)nxy;
    }
};

// A particle that left its cell since the sort (out of line: rare).
template <int S, bool QC>
__device__ __noinline__ void stale_to_global(const DepArgs& a, uint32_t key, float rx, float ry, float qn, float vxx,
                                             float vyy, uint32_t p) {
    particle_to_global<S, QC>(a, key, rx, ry, qn, vxx, vyy, p);
}

// A particle that left its cell since the sort, added to the CTA's tile
// accumulators when its frame lies within them: its cell at most one cell
// outside the tile (the accumulators have a halo one cell wider than the
// tile's own frames need, between sorts). The same values as particle_to_global,
// split into the low and high words. False: not in reach (the caller goes global).
template <int S, bool QC>
__device__ __noinline__ bool stale_to_tile(const DepArgs& a, uint32_t key, float rx, float ry, float qn, int x0, int y0,
                                           int tw, int th, int SW, uint32_t* slo, int* shi) {
    constexpr int NX = Frame<S>::NX, LO = Frame<S>::LO, NV = NX * NX;
    static_assert(S != S_ESK, "trajectory frames stay on the global path");
    if (key >= (uint32_t)a.Nx * (uint32_t)a.Ny) return false;
    const int iy = (int)(key / (uint32_t)a.Nx), ix = (int)(key - (uint32_t)iy * (uint32_t)a.Nx);
    int cx = ix - x0, cy = iy - y0;
    // the periodic image nearest the tile (any image maps back to the same node)
    if (cx > a.Nx / 2) cx -= a.Nx;
    if (cx < -(a.Nx / 2)) cx += a.Nx;
    if (cy > a.Ny / 2) cy -= a.Ny;
    if (cy < -(a.Ny / 2)) cy += a.Ny;
    if (cx < -1 || cx > tw || cy < -1 || cy > th) return false;
    const int lx0 = cx + 2 + LO, ly0 = cy + 2 + LO;  // local node of frame entry (0, 0)
    long long tv[NV];
    if constexpr (S == S_TSC && QC) {
        uint32_t X[4], Y[4];
        tsci_weights(rx, ry, X, Y);
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int i = 0; i < 4; ++i) tv[j * 4 + i] = (long long)((unsigned long long)X[i] * Y[j]);
    } else if constexpr (S == S_TSC) {
        uint32_t val[16];
        tsc_values(rx, ry, qn, val);
#pragma unroll
        for (int q = 0; q < 16; ++q) tv[q] = tsc_true(q, val[q], 1u);
    } else {
        int iv[Frame<S>::V];
        stencil_values<S>(a, rx, ry, qn, 0.0f, 0.0f, ix, iy, 0, iv);
#pragma unroll
        for (int q = 0; q < NV; ++q) tv[q] = iv[q];
    }
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const long long x = tv[q];
        if (x != 0) {
            const int i = (ly0 + q / NX) * SW + lx0 + (q % NX);
            atomicAdd(slo + i, (uint32_t)x & ((1u << TILE_SPLIT) - 1u));
            atomicAdd(shi + i, (int)(x >> TILE_SPLIT));
        }
    }
    return true;
}

// Shared memory: [stage buffers: NW warps x NBUF x NF fields x LPP/4 quads x
// 32 lanes x 16 bytes][tile accumulators: low, high words][the tile rows' cell
// offsets].
template <int S, int LPP, int NW, bool QC, bool KEYS, int NBUF>
__host__ __device__ constexpr size_t cells_fixed_bytes() {
    return (size_t)NW * NBUF * (StageFields<S, QC>::NF - (KEYS ? 0 : 1)) * (LPP / 4) * 512;
}

template <int S, int LPP, int NW, int MINB, bool QC, bool KEYS, int NBUF>
__global__ void __launch_bounds__(NW * 32, MINB) deposit_cells(DepArgs a) {
    if (gated_off(a)) return;
    constexpr int NX = Frame<S>::NX, LO = Frame<S>::LO, V = Frame<S>::V;
    constexpr int NV = NX * NX;
    constexpr int NF = StageFields<S, QC>::NF - (KEYS ? 0 : 1);  // the cell key is staged only with KEYS
    constexpr int FX = KEYS ? 1 : 0;                            // stage field of xr
    constexpr int FQ = FX + 2;                                  // of q (not QC)
    constexpr int FV = FX + (QC ? 2 : 3);                       // of vx (ESK)
    constexpr int QL = LPP / 4;                                 // quads per lane per stage
    constexpr int BUFB = NF * QL * 512;                         // bytes of one stage buffer of a warp
    constexpr bool TSCI = S == S_TSC && QC;                     // exact integer TSC weights
    static_assert(LPP % 4 == 0 && LPP <= 16, "stage sums of LPP particles stay in 32 bits");
    constexpr uint32_t FOLD = 32 / LPP;  // stages per fold of the exact TSC partial sums (32 particles)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t s_count;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // between sorts the accumulators get one more halo cell on each side, where
    // the particles that moved to a neighbouring cell of the tile land
    constexpr int PAD = (KEYS && S != S_ESK) ? 1 : 0;
    const int SW = a.tile_w + 3 + 2 * PAD;
    const int tx = blockIdx.x % a.tiles_x, ty = blockIdx.x / a.tiles_x;
    const int x0 = tx * a.tile_w, y0 = ty * a.tile_h;
    const int tw = min(a.tile_w, a.Nx - x0), th = min(a.tile_h, a.Ny - y0);
    const int nloc = (th + 3 + 2 * PAD) * SW;
    const int nch = (tw + 31) >> 5;  // units of up to 32 cells per tile row
    unsigned char* swarp = smem_raw + (size_t)warp * NBUF * BUFB;
    const uint32_t stage0 = (uint32_t)__cvta_generic_to_shared(swarp) + (uint32_t)(lane * 16);
    uint32_t* slo = reinterpret_cast<uint32_t*>(smem_raw + cells_fixed_bytes<S, LPP, NW, QC, KEYS, NBUF>());
    int* shi = reinterpret_cast<int*>(slo + nloc);
    uint32_t* soff = reinterpret_cast<uint32_t*>(shi + nloc);  // the tile rows' offsets, th x (tw + 1)
    const int ow = tw + 1;
    // KEYS: this warp's queue of particles that left their cell (at most a stage)
    uint32_t* squeue = soff + a.tile_h * (a.tile_w + 1) + warp * 32 * LPP;
    if (threadIdx.x == 0) s_count = 0;
    for (int i = threadIdx.x; i < nloc; i += NW * 32) {
        slo[i] = 0;
        shi[i] = 0;
    }
    for (int i = threadIdx.x; i < th * ow; i += NW * 32) {
        const int r = i / ow;
        soff[i] = a.offsets[(uint32_t)(y0 + r) * (uint32_t)a.Nx + (uint32_t)x0 + (uint32_t)(i - r * ow)];
    }
    __syncthreads();
    if (threadIdx.x < th) atomicAdd(&s_count, soff[threadIdx.x * ow + tw] - soff[threadIdx.x * ow]);
    __syncthreads();
    const bool dense = s_count >= TILE_SPLIT_MAX;

    const uint32_t* fptr[NF];
    if constexpr (KEYS) fptr[0] = a.cell;
    fptr[FX] = reinterpret_cast<const uint32_t*>(a.xr);
    fptr[FX + 1] = reinterpret_cast<const uint32_t*>(a.yr);
    if constexpr (!QC) fptr[FQ] = reinterpret_cast<const uint32_t*>(a.q);
    if constexpr (S == S_ESK) {
        fptr[FV] = reinterpret_cast<const uint32_t*>(a.vx);
        fptr[FV + 1] = reinterpret_cast<const uint32_t*>(a.vy);
    }
    // unit u = (tile row, 32-cell chunk); this lane's cell range and quads
    struct Unit {
        uint32_t beg, end, q0, q1, nst;  // particles [beg, end), quads [q0, q1), stages of the unit
        int r, col;                     // tile row, this lane's column in the tile (-1: no cell)
    };
    const int nunits = th * nch;
    auto unit_of = [&](int u) {
        Unit w;
        w.r = u / nch;
        const int col = (u - w.r * nch) * 32 + lane;
        w.col = col < tw ? col : -1;
        w.beg = w.end = 0;
        if (w.col >= 0) {
            w.beg = soff[w.r * ow + w.col];
            w.end = soff[w.r * ow + w.col + 1];
        }
        w.q0 = w.beg >> 2;
        w.q1 = w.end > w.beg ? (w.end + 3u) >> 2 : w.q0;
        const uint32_t st = (w.q1 - w.q0 + QL - 1) / QL;
        w.nst = __reduce_max_sync(FULL, st);
        return w;
    };
    auto issue = [&](const Unit& w, uint32_t t, int buf) {
        const uint32_t dst = stage0 + (uint32_t)(buf * BUFB);
#pragma unroll
        for (int h = 0; h < QL; ++h) {
            const uint32_t qd = w.q0 + t * QL + (uint32_t)h;
            if (qd < w.q1) {
#pragma unroll
                for (int f = 0; f < NF; ++f) cp_async16(dst + (uint32_t)((f * QL + h) * 512), fptr[f] + 4u * qd);
            }
        }
        cp_async_commit();
    };

    // the first non-empty unit at or after u (nunits: none)
    auto next_unit = [&](int u, Unit& w) {
        for (; u < nunits; u += NW) {
            w = unit_of(u);
            if (w.nst) break;
        }
        return u;
    };
    // prefetch cursor (stage pt of unit pu), NBUF - 1 stages ahead of the consumer
    Unit pw{};
    int pu = next_unit(warp, pw);
    uint32_t pt = 0;
    auto issue_next = [&](int buf) {
        if (pu < nunits) {
            issue(pw, pt, buf);
            if (++pt >= pw.nst) {
                pt = 0;
                pu = next_unit(pu + NW, pw);
            }
        } else {
            cp_async_commit();  // an empty group keeps the wait counts uniform
        }
    };
#pragma unroll
    for (int k = 0; k < NBUF - 1; ++k) issue_next(k);
    Unit cw{};
    int u = next_unit(warp, cw);
    uint32_t t = 0;
    int buf = 0;
    uint32_t cnt = 0;  // particles of the cell summed (KEYS: those still in it)
    uint32_t moved = 0;  // KEYS: particles of this warp's cells that left them (warp-uniform)
    CellRun<S, QC> run;
    if constexpr (S == S_NGP && QC) run.A = __float2int_rn(a.qc * 16777216.0f);
    run.zero();
    while (u < nunits) {
        issue_next(buf == 0 ? NBUF - 1 : buf - 1);  // the buffer consumed last
        cp_async_wait<NBUF - 1>();
        __syncwarp();
        const bool unit_end = t + 1 >= cw.nst;

        const int iy = y0 + cw.r;
        const uint32_t rowbase = (uint32_t)iy * (uint32_t)a.Nx;
        const uint32_t mykey = rowbase + (uint32_t)(x0 + cw.col);
        const unsigned char* sb = swarp + (size_t)buf * BUFB + lane * 16;
        uint32_t scnt = 0;  // particles summed in this stage
        uint32_t qn = 0;  // particles of this stage that left their cell (KEYS), queued in squeue
#pragma unroll
        for (int h = 0; h < QL; ++h) {
            const uint32_t qd = cw.q0 + t * QL + (uint32_t)h;
            const bool qok = qd < cw.q1;
            if (KEYS || qok) {
                Quad<S> d;
                if constexpr (KEYS) d.cell = qok ? *reinterpret_cast<const uint4*>(sb + h * 512) : make_uint4(0, 0, 0, 0);
                d.xr = *reinterpret_cast<const float4*>(sb + (FX * QL + h) * 512);
                d.yr = *reinterpret_cast<const float4*>(sb + ((FX + 1) * QL + h) * 512);
                if constexpr (QC)
                    d.q = make_float4(a.qc, a.qc, a.qc, a.qc);
                else
                    d.q = *reinterpret_cast<const float4*>(sb + (FQ * QL + h) * 512);
                if constexpr (S == S_ESK) {
                    d.vx = *reinterpret_cast<const float4*>(sb + (FV * QL + h) * 512);
                    d.vy = *reinterpret_cast<const float4*>(sb + ((FV + 1) * QL + h) * 512);
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t p = 4u * qd + (uint32_t)k;
                    bool valid = qok && p - cw.beg < cw.end - cw.beg;
                    if constexpr (KEYS) {
                        // a particle that left its cell since the last sort is queued and
                        // deposited after the stage by all lanes together (no divergent path)
                        const bool stale = valid && u4(d.cell, k) != mykey;
                        const unsigned sb_mask = __ballot_sync(FULL, stale);
                        if (sb_mask) {
                            if (stale) squeue[qn + __popc(sb_mask & ((1u << lane) - 1u))] = p;
                            qn += __popc(sb_mask);
                            valid = valid && !stale;
                        }
                    }
                    if (valid) {
                        float vxx = 0.0f, vyy = 0.0f;
                        if constexpr (S == S_ESK) {
                            vxx = f4(d.vx, k);
                            vyy = f4(d.vy, k);
                        }
                        if constexpr (TSCI || (S == S_NGP && QC)) {
                            run.add(f4(d.xr, k), f4(d.yr, k));
                        } else if constexpr (S == S_TSC) {
                            tsc_accumulate(f4(d.xr, k), f4(d.yr, k), f4(d.q, k), run.v);
                        } else {
                            int iv[V];
                            if (!stencil_values<S>(a, f4(d.xr, k), f4(d.yr, k), f4(d.q, k), vxx, vyy,
                                                   (int)(mykey - rowbase), iy, p, iv))
                                continue;  // deposited by the general trajectory path
#pragma unroll
                            for (int q = 0; q < NV; ++q) run.v[q] += (uint32_t)iv[q];
                        }
                        ++scnt;
                    }
                }
                run.end_quad();
            }
        }
        if constexpr (KEYS) {
            moved += qn;
            if (qn) {  // the stage's particles that left their cell, one per lane
                __syncwarp();
                for (uint32_t i = (uint32_t)lane; i < qn; i += 32) {
                    const uint32_t p = squeue[i];
                    float vxx = 0.0f, vyy = 0.0f;
                    if constexpr (S == S_ESK) {
                        vxx = a.vx[p];
                        vyy = a.vy[p];
                    }
                    const uint32_t key = a.cell[p];
                    const float rx = a.xr[p], ry = a.yr[p], qn = QC ? a.qc : a.q[p];
                    if constexpr (PAD > 0) {
                        if (!dense && stale_to_tile<S, QC>(a, key, rx, ry, qn, x0, y0, tw, th, SW, slo, shi)) continue;
                    }
                    stale_to_global<S, QC>(a, key, rx, ry, qn, vxx, vyy, p);
                }
                __syncwarp();
            }
        }
        run.end_stage(scnt, (t + 1u) % FOLD == 0u);
        cnt += scnt;
        if (unit_end) {  // the end of the unit: write out this lane's cell
            if (cnt) {
                long long tv[NV];
                run.finish();
                run.totals(cnt, tv);
                if (dense) {
                    flush_global_ll<NX, LO, NV>(a, mykey, tv);
                } else {
                    const int lx = cw.col + 1 + LO + PAD;
                    const int lrow = cw.r + 1 + LO + PAD;
#pragma unroll
                    for (int q = 0; q < NV; ++q) {
                        const long long x = tv[q];
                        if (x != 0) {
                            const int i = (lrow + q / NX) * SW + lx + (q % NX);
                            atomicAdd(slo + i, (uint32_t)x & ((1u << TILE_SPLIT) - 1u));
                            atomicAdd(shi + i, (int)(x >> TILE_SPLIT));
                        }
                    }
                }
            }
            run.zero();
            cnt = 0;
        }
        __syncwarp();
        if (unit_end) {
            t = 0;
            u = next_unit(u + NW, cw);
        } else {
            ++t;
        }
        buf = buf + 1 == NBUF ? 0 : buf + 1;
    }
    cp_async_wait<0>();
    if constexpr (KEYS) {
        if (lane == 0 && moved) {
            atomicAdd(&a.st->moved, (unsigned long long)moved);
            atomicAdd(&a.st->moved_dep, (unsigned long long)moved);
        }
    }
    __syncthreads();
    if (dense) return;
    for (int i = threadIdx.x; i < nloc; i += NW * 32) {
        // the high word is signed in the general form, unsigned in the exact integer TSC form
        const long long hi = TSCI ? (long long)(uint32_t)shi[i] : (long long)shi[i];
        const long long v = hi * (1ll << TILE_SPLIT) + (long long)slo[i];
        if (v != 0) {
            const int ly = i / SW, lx = i % SW;
            const int gx = wrap_i(x0 - 1 - PAD + lx, a.Nx), gy = wrap_i(y0 - 1 - PAD + ly, a.Ny);
            atomicAdd(a.acc + (size_t)gy * a.Nx + gx, (unsigned long long)v);
        }
    }
}

// One unit of the int64 grid (FP64): max|q| * inv_vol * 2^-24, or, for the
// exact integer TSC form, max|q| * inv_vol * (qn * 2^-30) (scale != 0).
__global__ void fixed_unit(double inv_vol, double scale, const DevStats* st, double* unit_out) {
    *unit_out = scale == 0.0 ? charge_unit(st, inv_vol) : __dmul_rn(__dmul_rn((double)load_maxq(st), inv_vol), scale);
}

__global__ void fixed_to_rho(const long long* __restrict__ acc, size_t g, double background,
                             const double* __restrict__ unitp, double* __restrict__ rho) {
    const double unit = *unitp;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g) rho[i] = __dadd_rn(__dmul_rn((double)acc[i], unit), background);
}

#ifndef CELLS_LPP
#define CELLS_LPP 8
#endif

#ifndef CELLS_NBUF
#define CELLS_NBUF 2
#endif
template <int S, int LPP, int NW, int MINB, bool QC, bool KEYS>
static int launch_cells(pic_ctx* c, const DepArgs& a, unsigned tiles) {
    constexpr int NBUF = CELLS_NBUF;
    constexpr int PAD = (KEYS && S != S_ESK) ? 1 : 0;  // the kernel's extra halo between sorts
    const size_t smem = cells_fixed_bytes<S, LPP, NW, QC, KEYS, NBUF>() +
                        (size_t)(a.tile_h + 3 + 2 * PAD) * (a.tile_w + 3 + 2 * PAD) * 2 * sizeof(uint32_t) +
                        (size_t)a.tile_h * (a.tile_w + 1) * sizeof(uint32_t) +
                        (KEYS ? (size_t)NW * 32 * LPP * sizeof(uint32_t) : 0);
    const int rc = opt_in_dynamic_smem((const void*)deposit_cells<S, LPP, NW, MINB, QC, KEYS, NBUF>, smem);
    if (rc != PIC_OK) return rc;
    deposit_cells<S, LPP, NW, MINB, QC, KEYS, NBUF><<<tiles, NW * 32, smem, c->stream>>>(a);
    return PIC_OK;
}

// After a deposit between sorts whose kernel was chosen on the device: once the
// cell kernel has found more than `limit` particles outside their sorted cell,
// the any-order kernel takes the following deposits (it is faster when most
// particles have moved: every mover is a separate frame of atomics in the cell
// kernel) until the next sort clears the flag. A deposit made in any order
// counts every particle as moved, so a sort triggered by the moved fraction
// still follows.
__global__ void choose_any_order(DevStats* st, unsigned long long limit, unsigned long long n) {
    if (st->any_order)
        st->moved += n;
    else if (st->moved_dep > limit)
        st->any_order = 1u;
    st->moved_dep = 0;
}

// The fraction of the particles above which deposits between sorts switch to
// the any-order kernel (measured crossover at 1024^2, TSC: the cell kernel takes
// about 6.7 ms with every particle moved, the any-order kernel 3.0 ms).
constexpr double ANY_ORDER_FRACTION = 0.4;

template <int S>
static int launch_runs(pic_ctx* c, const DepArgs& a) {
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    size_t blocks = (a.n + DEP_THREADS * 4 - 1) / (DEP_THREADS * 4);
    const size_t cap = (size_t)sms * 8;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    if constexpr (S == S_TSC) {
        if (a.qc != 0.0f)
            deposit_runs_tsci<<<(unsigned)blocks, DEP_THREADS, 0, c->stream>>>(a);
        else
            deposit_runs_tsc<<<(unsigned)blocks, DEP_THREADS, 0, c->stream>>>(a);
    } else {
        deposit_runs<S><<<(unsigned)blocks, DEP_THREADS, 0, c->stream>>>(a);
    }
    return check_launch(c, "deposit_runs");
}

template <int S>
// kernel choice: 0 tiled (cell-sorted), 1 run-aggregating (any order), 2 one thread per particle;
// `adaptive`: between sorts, the device picks the tiled or the any-order kernel (choose_any_order)
static int launch_deposit(pic_ctx* c, const DepArgs& a, int kind, bool adaptive) {
    if (kind == 0 && adaptive && !c->sorted) {
        DepArgs ak = a, ar = a;
        ak.gate = ar.gate = &c->dstats->any_order;
        ak.gate_when = 0;
        ar.gate_when = 1;
        const unsigned tiles = (unsigned)(a.tiles_x * ((c->Ny + a.tile_h - 1) / a.tile_h));
        prof_begin(c, "deposit");
        int rc = a.qc != 0.0f ? launch_cells<S, CELLS_LPP, 4, 4, true, true>(c, ak, tiles)
                              : launch_cells<S, CELLS_LPP, 4, 4, false, true>(c, ak, tiles);
        if (rc == PIC_OK) rc = check_launch(c, "deposit_cells");
        if (rc == PIC_OK) rc = launch_runs<S>(c, ar);
        if (rc == PIC_OK) {
            choose_any_order<<<1, 1, 0, c->stream>>>(c->dstats,
                                                     (unsigned long long)(ANY_ORDER_FRACTION * (double)a.n),
                                                     (unsigned long long)a.n);
            rc = check_launch(c, "choose_any_order");
        }
        prof_end(c);
        return rc;
    }
    if (kind == 0) {
        const unsigned tiles = (unsigned)(a.tiles_x * ((c->Ny + a.tile_h - 1) / a.tile_h));
        prof_begin(c, "deposit");
        // 8 particles per lane and stage, 4 warps per tile; TSC capped at 96
        // registers (5 CTAs per SM), measured fastest at 1024^2 x 64 particles/cell.
        // cp.async staging measured 10 % faster than TMA tensor copies of the
        // same stages (128-byte swizzle, one lane issuing, mbarrier completion)
        // freshly sorted: the offsets name every particle's cell and the keys are not read
        const bool keys = !c->sorted;
        int rc;
        if (a.qc != 0.0f) {  // one charge for all particles: the charge stream is not staged
            rc = keys ? launch_cells<S, CELLS_LPP, 4, 4, true, true>(c, a, tiles)
                      : launch_cells<S, CELLS_LPP, 4, 4, true, false>(c, a, tiles);
        } else {
            rc = keys ? launch_cells<S, CELLS_LPP, 4, 4, false, true>(c, a, tiles)
                      : launch_cells<S, CELLS_LPP, 4, 4, false, false>(c, a, tiles);
        }
        prof_end(c);
        if (rc != PIC_OK) return rc;
        return check_launch(c, "deposit_cells");
    }
    if (kind == 1) {
        prof_begin(c, "deposit");
        const int rc = launch_runs<S>(c, a);
        prof_end(c);
        return rc;
    }
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    size_t blocks = (a.n + DEP_THREADS - 1) / DEP_THREADS;
    const size_t cap = (size_t)sms * 16;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    prof_begin(c, "deposit");
    deposit_atomic<S><<<(unsigned)blocks, DEP_THREADS, 0, c->stream>>>(a);
    prof_end(c);
    return check_launch(c, "deposit_atomic");
}

int deposit_rho(pic_ctx* c, int scheme, double dt, double background) {
    if (scheme < PIC_SCHEME_NGP || scheme > PIC_SCHEME_ESIRKEPOV) return fail(PIC_ERR_ARG, "unknown scheme");
    int tiled;  // kernel kind, see launch_deposit
    if (c->order_mode == PIC_ORDER_SORTED) {
        if (!c->sorted && !c->part_valid)
            return fail(PIC_ERR_STATE, "deposit: PIC_ORDER_SORTED needs cell-sorted particles");
        tiled = 0;
    } else if (c->order_mode == PIC_ORDER_UNSORTED) {
        tiled = 1;
    } else if (c->order_mode == PIC_ORDER_ATOMIC) {
        tiled = 2;
    } else {
        // between sorts (the last sort's cell ranges still index the particles) the
        // cell kernel walks those ranges and deposits the particles that moved to
        // another cell on their own; otherwise the run-aggregating kernel
        tiled = (c->sorted || c->part_valid) ? 0 : 1;
    }
    PIC_CUDA_TRY(cudaMemsetAsync(c->acc, 0, c->G * sizeof(long long), c->stream));
    DepArgs a;
    a.cell = c->cell;
    a.xr = c->xr;
    a.yr = c->yr;
    a.vx = c->vx;
    a.vy = c->vy;
    a.q = c->q;
    a.offsets = c->offsets;
    a.acc = reinterpret_cast<unsigned long long*>(c->acc);
    a.n = c->n;
    a.Nx = c->Nx;
    a.Ny = c->Ny;
    a.dtf = (float)dt;
    a.dtdx = (float)(dt / c->dx);
    a.dtdy = (float)(dt / c->dy);
    if (!c->tile_user) {
        // rows of 32 cells (one per lane) and about 8K particles per tile, at
        // least as many rows as the 4 warps of a CTA
        const double ppc = (double)c->n / (double)c->G;
        const double cells = ppc > 0.0 ? 8192.0 / ppc : 2048.0;
        c->tile_w = 32;
        int h = 4;
        while (h < 32 && (double)(c->tile_w * h * 2) <= cells) h *= 2;
        c->tile_h = h;
    }
    a.tile_w = c->tile_w;
    a.tile_h = c->tile_h;
    a.tiles_x = (c->Nx + c->tile_w - 1) / c->tile_w;
    a.qc = c->qn_uniform;
    a.st = c->dstats;
    a.gate = nullptr;
    a.gate_when = 0;
    const bool adaptive = c->order_mode == PIC_ORDER_AUTO;
    if (c->n > 0) {
        switch (scheme) {
            case PIC_SCHEME_NGP:
                PIC_TRY(launch_deposit<S_NGP>(c, a, tiled, adaptive));
                break;
            case PIC_SCHEME_CIC:
                PIC_TRY(launch_deposit<S_CIC>(c, a, tiled, adaptive));
                break;
            case PIC_SCHEME_TSC:
                PIC_TRY(launch_deposit<S_TSC>(c, a, tiled, adaptive));
                break;
            default:
                PIC_TRY(launch_deposit<S_ESK>(c, a, tiled, adaptive));
                break;
        }
    }
    const double inv_vol = 1.0 / (c->dx * c->dy);
    // TSC with one charge for all particles deposits exact integer weights (2^30 units per particle)
    const double scale = (scheme == PIC_SCHEME_TSC && c->n > 0 && c->qn_uniform != 0.0f)
                             ? (double)c->qn_uniform * 0x1p-30
                             : 0.0;
    fixed_unit<<<1, 1, 0, c->stream>>>(inv_vol, scale, c->dstats, c->unitbuf);
    PIC_TRY(check_launch(c, "fixed_unit"));
    fixed_to_rho<<<(unsigned)((c->G + 255) / 256), 256, 0, c->stream>>>(c->acc, c->G, background, c->unitbuf,
                                                                         c->rho);
    PIC_TRY(check_launch(c, "fixed_to_rho"));
    c->last_scheme = scheme;
    return PIC_OK;
}

}  // namespace picgb

using namespace picgb;

extern "C" {

int pic_gpu_set_deposit_order(pic_ctx* c, int order) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    if (order < PIC_ORDER_AUTO || order > PIC_ORDER_ATOMIC) return fail(PIC_ERR_ARG, "unknown order mode");
    c->order_mode = order;
    return PIC_OK;
}

int pic_gpu_set_tile(pic_ctx* c, int tile_w, int tile_h) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    if (tile_w < 1 || tile_w > 64 || tile_h < 1 || tile_h > 32)
        return fail(PIC_ERR_ARG, "tile must be 1..64 x 1..32 cells");
    c->tile_w = tile_w;
    c->tile_h = tile_h;
    c->tile_user = 1;
    return PIC_OK;
}

int pic_gpu_deposit(pic_ctx* c, int scheme, double dt, double background, double* rho_out) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    PIC_TRY(deposit_rho(c, scheme, dt, background));
    if (rho_out) {
        PIC_CUDA_TRY(cudaMemcpyAsync(rho_out, c->rho, c->G * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        return pic_gpu_synchronize(c);
    }
    return PIC_OK;
}

int pic_gpu_get_rho_fixed(pic_ctx* c, int64_t* acc_out, double* unit_out) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    if (c->last_scheme < 0) return fail(PIC_ERR_STATE, "no deposit has run");
    if (acc_out)
        PIC_CUDA_TRY(cudaMemcpyAsync(acc_out, c->acc, c->G * sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    if (unit_out) PIC_CUDA_TRY(cudaMemcpyAsync(unit_out, c->unitbuf, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return pic_gpu_synchronize(c);
}

int pic_gpu_get_rho(pic_ctx* c, double* rho_out) {
    if (!c || !rho_out) return fail(PIC_ERR_ARG, "NULL argument");
    PIC_CUDA_TRY(cudaMemcpyAsync(rho_out, c->rho, c->G * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return pic_gpu_synchronize(c);
}

}  // extern "C"
