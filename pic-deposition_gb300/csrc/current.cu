// Esirkepov current deposition (Jx, Jy) -- new; the reference's "Esirkepov"
// deposits trajectory-averaged charge only (src/deposition/ngp.cpp:13-84).
//
// First-order (CIC-shape) charge-conserving current, Esirkepov, Comput. Phys.
// Commun. 135 (2001) 144, in 2D. For a particle moving by (dx_c, dy_c) cells
// (|d| < 1 on each axis, else PIC_ERR_COURANT), with S0/S1 the CIC weights of
// the old/new positions and DS = S1 - S0 on a 4-node frame (cell offsets -1..2
// around the old cell):
//     W1[j][i] = DSx[i] (S0y[j] + DSy[j]/2),  W2[j][i] = DSy[j] (S0x[i] + DSx[i]/2)
//     Jx(i+1/2, j) = -(q/dV)(dx/dt) sum_{i'<=i} W1[j][i'], Jy likewise along j.
// Jx[k] is stored at the node k of the cell edge's lower (left) end: the edge
// from node (i, j) to (i+1, j); Jy[k] at the edge from (i, j) to (i, j+1).
//
// Integer form (exact discrete continuity). A particle's old and new integer
// CIC charges R0, R1 use the charge deposit's rounding and remainder rule, W1 is
// rounded with row sums forced to 0 and column sums forced to those of R1 - R0,
// and W2 = (R1 - R0) - W1. Then (R1 - R0) + div J = 0 holds exactly in the
// int64 grids: the CIC charge of the pushed particles minus that of the old ones
// plus the integer divergence of J is zero at every node. J unit =
// max|q| inv_vol 2^-24 dx/dt (x), dy/dt (y). DS entries are formed from
// quantities of their own size (no S1 - S0 cancellation): no crossing
// DS = (0,-d,d,0); crossing up DS = (0, r-1, (1-r)-fr, fr); down DS = (-e, r+e, -r, 0).
//
// Kernels: cell-sorted particles, one lane per cell (current_cells); any order,
// the deposit's warp step (128 particles, 4 consecutive per lane via 128-bit
// loads), each lane summing its particles' 24 edge values while they share a
// cell (one rolled copy of the particle body), a segmented warp scan, and int64
// atomics from the run tails (deposit_current).
#include "pic_internal.cuh"

namespace picgb {

constexpr int J_THREADS = 256;
constexpr int J_WARPS = J_THREADS / 32;
constexpr int NJ = 24;  // 12 Jx edges (rows j=0..3, i=0..2) + 12 Jy edges (j=0..2, i=0..3)
constexpr uint32_t J_NO_CELL = 0xffffffffu;

struct JArgs {
    const uint32_t* cell;
    const float *xr, *yr, *vx, *vy, *q;
    size_t n;
    int Nx, Ny;
    float dtdx, dtdy;
    float qc;  // nonzero: every particle's stored charge (the charge stream is not read)
    unsigned long long *jx, *jy;
    DevStats* st;
};

__device__ __forceinline__ void esk_ds(float r, float d, float (&s0)[4], float (&ds)[4]) {
    const float e = r + d;
    const float f = floorf(e);
    const float fr = e - f;
    s0[0] = 0.0f;
    s0[1] = 1.0f - r;
    s0[2] = r;
    s0[3] = 0.0f;
    if (f == 0.0f) {
        ds[0] = 0.0f;
        ds[1] = -d;
        ds[2] = d;
        ds[3] = 0.0f;
    } else if (f > 0.0f) {
        ds[0] = 0.0f;
        ds[1] = r - 1.0f;
        ds[2] = (1.0f - r) - fr;
        ds[3] = fr;
    } else {
        ds[0] = -e;
        ds[1] = r + e;
        ds[2] = -r;
        ds[3] = 0.0f;
    }
}

// The particle's integer CIC charges (a 2x2 block at frame offset (kx, ky)),
// exactly as the charge deposit rounds them.
__device__ __forceinline__ void cic_int(float a, int A, float rx, float ry, int (&v)[4]) {
    const float X0 = 1.0f - rx, X1 = rx, Y0 = 1.0f - ry, Y1 = ry;
    const float a0 = a * Y0, a1 = a * Y1;
    v[0] = __float2int_rn(a0 * X0);
    v[1] = __float2int_rn(a0 * X1);
    v[2] = __float2int_rn(a1 * X0);
    v[3] = __float2int_rn(a1 * X1);
    const int mx = X1 > X0 ? 1 : 0, my = Y1 > Y0 ? 1 : 0;
    const int rem = A - (v[0] + v[1] + v[2] + v[3]);
    const int km = my * 2 + mx;
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] += (k == km) ? rem : 0;
}

// 24 integer edge values of one particle (see the file header). Returns false
// (and flags PIC_ERR_COURANT) when the move is a cell or more.
__device__ __forceinline__ bool edge_values(const JArgs& a, float rx, float ry, float vxx, float vyy, float qn,
                                            size_t p, int (&out)[NJ]) {
    const float ddx = vxx * a.dtdx, ddy = vyy * a.dtdy;
    if (!(fabsf(ddx) < 1.0f && fabsf(ddy) < 1.0f)) {
        set_dev_error(a.st, DEV_COURANT, (unsigned)p);
        return false;
    }
    float s0x[4], dsx[4], s0y[4], dsy[4];
    esk_ds(rx, ddx, s0x, dsx);
    esk_ds(ry, ddy, s0y, dsy);
    const float aq = qn * 16777216.0f;
    const int A = __float2int_rn(aq);
    int r0[4], r1[4];
    cic_int(aq, A, rx, ry, r0);
    const float ex = rx + ddx, ey = ry + ddy;
    const float fx = floorf(ex), fy = floorf(ey);
    cic_int(aq, A, ex - fx, ey - fy, r1);
    const int kx = (int)fx + 1, ky = (int)fy + 1;
    // dR = R1 - R0 on the 4x4 frame; R0 sits at offset (1, 1)
    int dR[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) dR[k] = 0;
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int i = 0; i < 2; ++i) dR[(1 + j) * 4 + (1 + i)] -= r0[j * 2 + i];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int jj = j - ky, ii = i - kx;
            const bool in = jj >= 0 && jj < 2 && ii >= 0 && ii < 2;
            dR[j * 4 + i] += in ? r1[(jj & 1) * 2 + (ii & 1)] : 0;
        }
    int W1[16];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const float ay = aq * (s0y[j] + 0.5f * dsy[j]);
        int row = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            W1[j * 4 + i] = __float2int_rn(ay * dsx[i]);
            row += W1[j * 4 + i];
        }
        W1[j * 4 + 3] = -row;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int col = 0, colR = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j) col += W1[j * 4 + i];
#pragma unroll
        for (int j = 0; j < 4; ++j) colR += dR[j * 4 + i];
        W1[12 + i] = colR - col;
    }
    // Jx edges: out[j*3 + i] = -sum_{i'<=i} W1[j][i'], i = 0..2
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        int cum = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            cum += W1[j * 4 + i];
            out[j * 3 + i] = -cum;
        }
    }
    // Jy edges: out[12 + j*4 + i] = -sum_{j'<=j} (dR - W1)[j'][i], j = 0..2
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int cum = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            cum += dR[j * 4 + i] - W1[j * 4 + i];
            out[12 + j * 4 + i] = -cum;
        }
    }
    return true;
}

__device__ __forceinline__ void flush_edges(const JArgs& a, uint32_t key, const int (&acc)[NJ]) {
    const int iy = (int)(key / (uint32_t)a.Nx), ix = (int)(key - (uint32_t)iy * (uint32_t)a.Nx);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const size_t row = (size_t)wrap_i(iy - 1 + j, a.Ny) * a.Nx;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int v = acc[j * 3 + i];
            if (v) atomicAdd(a.jx + row + wrap_i(ix - 1 + i, a.Nx), (unsigned long long)(long long)v);
        }
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const size_t row = (size_t)wrap_i(iy - 1 + j, a.Ny) * a.Nx;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int v = acc[12 + j * 4 + i];
            if (v) atomicAdd(a.jy + row + wrap_i(ix - 1 + i, a.Nx), (unsigned long long)(long long)v);
        }
    }
}

__device__ __forceinline__ float f4(const float4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
__device__ __forceinline__ uint32_t u4(const uint4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }

__global__ void __launch_bounds__(J_THREADS) deposit_current(JArgs a) {
    const int lane = threadIdx.x & 31;
    const size_t gw = (size_t)blockIdx.x * J_WARPS + (threadIdx.x >> 5);
    const size_t stride = (size_t)gridDim.x * J_WARPS * 128;
    const uint32_t G = (uint32_t)a.Nx * (uint32_t)a.Ny;
    const unsigned upto = (lane == 31) ? 0xffffffffu : ((2u << lane) - 1u);
    for (size_t base = gw * 128; base < a.n; base += stride) {
        const size_t p0 = base + 4u * lane;
        uint4 cell = make_uint4(0, 0, 0, 0);
        float4 xr = make_float4(0, 0, 0, 0), yr = xr, vx = xr, vy = xr, q = xr;
        if (p0 < a.n) {
            cell = __ldcs(reinterpret_cast<const uint4*>(a.cell + p0));
            xr = __ldcs(reinterpret_cast<const float4*>(a.xr + p0));
            yr = __ldcs(reinterpret_cast<const float4*>(a.yr + p0));
            vx = __ldcs(reinterpret_cast<const float4*>(a.vx + p0));
            vy = __ldcs(reinterpret_cast<const float4*>(a.vy + p0));
            q = a.qc != 0.0f ? make_float4(a.qc, a.qc, a.qc, a.qc) : __ldcs(reinterpret_cast<const float4*>(a.q + p0));
        }
        uint32_t ckey = J_NO_CELL;
        int acc[NJ];
#pragma unroll
        for (int k = 0; k < NJ; ++k) acc[k] = 0;
        // rolled loops (one copy of the particle body and of the scan step): the
        // unrolled kernel thrashed the instruction cache (ncu: 18 cycles per issue
        // waiting for instructions; rolled, 2.1x faster)
#pragma unroll 1
        for (int k = 0; k < 4; ++k) {
            const size_t p = p0 + (size_t)k;
            if (p >= a.n) continue;
            const uint32_t key = u4(cell, k);
            if (key >= G) {
                set_dev_error(a.st, DEV_BAD_CELL, (unsigned)p);
                continue;
            }
            int v[NJ];
            if (!edge_values(a, f4(xr, k), f4(yr, k), f4(vx, k), f4(vy, k), f4(q, k), p, v)) continue;
            if (key != ckey) {
                if (ckey != J_NO_CELL) flush_edges(a, ckey, acc);
                ckey = key;
#pragma unroll
                for (int t = 0; t < NJ; ++t) acc[t] = v[t];
            } else {
#pragma unroll
                for (int t = 0; t < NJ; ++t) acc[t] += v[t];
            }
        }
        const uint32_t kprev = __shfl_up_sync(0xffffffffu, ckey, 1);
        // segments stop at lane 16: a run total covers <= 64 particles and fits int32
        const unsigned H = __ballot_sync(0xffffffffu, lane == 0 || lane == 16 || ckey != kprev);
        const int segstart = 31 - __clz(H & upto);
#pragma unroll 1
        for (int d = 1; d < 32; d <<= 1) {
            const bool take = lane - d >= segstart;
#pragma unroll
            for (int t = 0; t < NJ; ++t) {
                const int o = __shfl_up_sync(0xffffffffu, acc[t], d);
                if (take) acc[t] += o;
            }
        }
        const bool tail = (lane == 31) || ((H >> (lane + 1)) & 1u);
        if (tail && ckey != J_NO_CELL) flush_edges(a, ckey, acc);
    }
}

// Cell-sorted particles: one lane per cell. A CTA owns a 32 x 8 tile of cells;
// warp w takes the tile rows w, w + 4, and lane l the cell in column l, walking
// that cell's range of the sorted stream (16-byte loads of 4 particles) and
// summing its particles' 24 edge values in 32-bit registers (at most 64
// particles per sum: |sum| <= 64 * 2^24). Each sum goes to the tile's Jx and Jy
// accumulators in shared memory (low 15 bits and the rest in two 32-bit words,
// a halo of one node left and below and two right and above), and the tile to
// the int64 grids once. Integer sums, so the grids equal those of
// deposit_current bit for bit.
constexpr int JC_TW = 32, JC_TH = 8, JC_WARPS = 4;
constexpr int JC_SW = JC_TW + 3, JC_SH = JC_TH + 3, JC_N = JC_SW * JC_SH;
constexpr int JC_RUN = 64;
constexpr int JC_SPLIT = 15;

template <bool QC>
__global__ void __launch_bounds__(JC_WARPS * 32) current_cells(JArgs a, const uint32_t* __restrict__ offsets,
                                                                int tiles_x) {
    __shared__ uint32_t slo[2 * JC_N];
    __shared__ int shi[2 * JC_N];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int x0 = tx * JC_TW, y0 = ty * JC_TH;
    const int tw = min(JC_TW, a.Nx - x0), th = min(JC_TH, a.Ny - y0);
    for (int i = threadIdx.x; i < 2 * JC_N; i += JC_WARPS * 32) {
        slo[i] = 0;
        shi[i] = 0;
    }
    __syncthreads();
    int acc[NJ];
    // adds acc (the cell in column `lane`, tile row r) to the tile accumulators
    auto flush = [&](int r) {
#pragma unroll
        for (int t = 0; t < NJ; ++t) {
            const int v = acc[t];
            if (v != 0) {
                // Jx edge (j, i) = t (j * 3 + i), Jy edge (j, i) = t - 12 (j * 4 + i): local node (lane + i, r + j)
                const int j = t < 12 ? t / 3 : (t - 12) / 4, i = t < 12 ? t % 3 : (t - 12) % 4;
                const int idx = (t < 12 ? 0 : JC_N) + (r + j) * JC_SW + lane + i;
                atomicAdd(slo + idx, (uint32_t)v & ((1u << JC_SPLIT) - 1u));
                atomicAdd(shi + idx, v >> JC_SPLIT);
            }
            acc[t] = 0;
        }
    };
    for (int r = warp; r < th; r += JC_WARPS) {
        uint32_t beg = 0, end = 0;
        if (lane < tw) {
            const uint32_t cell = (uint32_t)(y0 + r) * (uint32_t)a.Nx + (uint32_t)(x0 + lane);
            beg = offsets[cell];
            end = offsets[cell + 1];
        }
#pragma unroll
        for (int t = 0; t < NJ; ++t) acc[t] = 0;
        int cnt = 0;
        const uint32_t q0 = beg >> 2, q1 = end > beg ? (end + 3u) >> 2 : q0;
#pragma unroll 1
        for (uint32_t qd = q0; qd < q1; ++qd) {
            const float4 xr = __ldg(reinterpret_cast<const float4*>(a.xr) + qd);
            const float4 yr = __ldg(reinterpret_cast<const float4*>(a.yr) + qd);
            const float4 vx = __ldg(reinterpret_cast<const float4*>(a.vx) + qd);
            const float4 vy = __ldg(reinterpret_cast<const float4*>(a.vy) + qd);
            const float4 q = QC ? make_float4(a.qc, a.qc, a.qc, a.qc) : __ldg(reinterpret_cast<const float4*>(a.q) + qd);
#pragma unroll 1
            for (int k = 0; k < 4; ++k) {
                const uint32_t p = 4u * qd + (uint32_t)k;
                if (p < beg || p >= end) continue;
                int v[NJ];
                if (edge_values(a, f4(xr, k), f4(yr, k), f4(vx, k), f4(vy, k), f4(q, k), p, v)) {
#pragma unroll
                    for (int t = 0; t < NJ; ++t) acc[t] += v[t];
                }
                if (++cnt == JC_RUN) {
                    flush(r);
                    cnt = 0;
                }
            }
        }
        if (cnt) flush(r);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * JC_N; i += JC_WARPS * 32) {
        const long long v = (long long)shi[i] * (1ll << JC_SPLIT) + (long long)slo[i];
        if (v != 0) {
            const int li = i < JC_N ? i : i - JC_N;
            const int ly = li / JC_SW, lx = li - ly * JC_SW;
            const size_t g = (size_t)wrap_i(y0 - 1 + ly, a.Ny) * a.Nx + wrap_i(x0 - 1 + lx, a.Nx);
            atomicAdd((i < JC_N ? a.jx : a.jy) + g, (unsigned long long)v);
        }
    }
}

__global__ void current_to_f64(const long long* __restrict__ jx, const long long* __restrict__ jy, size_t g,
                               const double* __restrict__ units, double* __restrict__ ox, double* __restrict__ oy) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g) {
        ox[i] = __dmul_rn((double)jx[i], units[0]);
        oy[i] = __dmul_rn((double)jy[i], units[1]);
    }
}

__global__ void current_units(double inv_vol, double dxdt, double dydt, const DevStats* st, double* units) {
    const double u = charge_unit(st, inv_vol);
    units[0] = __dmul_rn(u, dxdt);
    units[1] = __dmul_rn(u, dydt);
}

static int ensure_current(pic_ctx* c) {
    int rc = PIC_OK;
    if (!c->accjx) c->accjx = (long long*)dalloc(c->G * 8, &rc);
    if (rc) return rc;
    if (!c->accjy) c->accjy = (long long*)dalloc(c->G * 8, &rc);
    if (rc) return rc;
    if (!c->jx) c->jx = (double*)dalloc(c->G * 8, &rc);
    if (rc) return rc;
    if (!c->jy) c->jy = (double*)dalloc(c->G * 8, &rc);
    if (rc) return rc;
    if (!c->junits) c->junits = (double*)dalloc(2 * 8, &rc);
    return rc;
}

int deposit_current_async(pic_ctx* c, double dt) {
    if (!(dt > 0.0)) return fail(PIC_ERR_ARG, "deposit_current: dt must be > 0");
    PIC_TRY(ensure_current(c));
    PIC_CUDA_TRY(cudaMemsetAsync(c->accjx, 0, c->G * 8, c->stream));
    PIC_CUDA_TRY(cudaMemsetAsync(c->accjy, 0, c->G * 8, c->stream));
    JArgs a;
    a.cell = c->cell;
    a.xr = c->xr;
    a.yr = c->yr;
    a.vx = c->vx;
    a.vy = c->vy;
    a.q = c->q;
    a.n = c->n;
    a.Nx = c->Nx;
    a.Ny = c->Ny;
    a.dtdx = (float)(dt / c->dx);
    a.dtdy = (float)(dt / c->dy);
    a.qc = c->qn_uniform;
    a.jx = reinterpret_cast<unsigned long long*>(c->accjx);
    a.jy = reinterpret_cast<unsigned long long*>(c->accjy);
    a.st = c->dstats;
    if (c->n && c->sorted) {
        // cell-sorted: one lane per cell over the sort's ranges
        const int tiles_x = (c->Nx + JC_TW - 1) / JC_TW, tiles_y = (c->Ny + JC_TH - 1) / JC_TH;
        prof_begin(c, "current");
        if (a.qc != 0.0f)
            current_cells<true><<<(unsigned)(tiles_x * tiles_y), JC_WARPS * 32, 0, c->stream>>>(a, c->offsets, tiles_x);
        else
            current_cells<false><<<(unsigned)(tiles_x * tiles_y), JC_WARPS * 32, 0, c->stream>>>(a, c->offsets, tiles_x);
        prof_end(c);
        PIC_TRY(check_launch(c, "current_cells"));
    } else if (c->n) {
        int sms = 148;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
        size_t blocks = (c->n + J_THREADS * 4 - 1) / (J_THREADS * 4);
        if (blocks > (size_t)sms * 8) blocks = (size_t)sms * 8;
        prof_begin(c, "current");
        deposit_current<<<(unsigned)blocks, J_THREADS, 0, c->stream>>>(a);
        prof_end(c);
        PIC_TRY(check_launch(c, "deposit_current"));
    }
    current_units<<<1, 1, 0, c->stream>>>(1.0 / (c->dx * c->dy), c->dx / dt, c->dy / dt, c->dstats, c->junits);
    PIC_TRY(check_launch(c, "current_units"));
    current_to_f64<<<(unsigned)((c->G + 255) / 256), 256, 0, c->stream>>>(c->accjx, c->accjy, c->G, c->junits, c->jx,
                                                                           c->jy);
    PIC_TRY(check_launch(c, "current_to_f64"));
    c->has_current = 1;
    return PIC_OK;
}

void release_current(pic_ctx* c) {
    void* ptrs[] = {c->accjx, c->accjy, c->jx, c->jy, c->junits};
    for (void* p : ptrs) dfree(p);
}

}  // namespace picgb

using namespace picgb;

extern "C" {

int pic_gpu_deposit_current(pic_ctx* c, double dt, double* jx_out, double* jy_out) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    PIC_TRY(deposit_current_async(c, dt));
    if (jx_out) PIC_CUDA_TRY(cudaMemcpyAsync(jx_out, c->jx, c->G * 8, cudaMemcpyDeviceToHost, c->stream));
    if (jy_out) PIC_CUDA_TRY(cudaMemcpyAsync(jy_out, c->jy, c->G * 8, cudaMemcpyDeviceToHost, c->stream));
    if (jx_out || jy_out) return pic_gpu_synchronize(c);
    return PIC_OK;
}

int pic_gpu_get_current_fixed(pic_ctx* c, int64_t* jx, int64_t* jy, double* unit_x, double* unit_y) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    if (!c->has_current) return fail(PIC_ERR_STATE, "no current deposit has run");
    if (jx) PIC_CUDA_TRY(cudaMemcpyAsync(jx, c->accjx, c->G * 8, cudaMemcpyDeviceToHost, c->stream));
    if (jy) PIC_CUDA_TRY(cudaMemcpyAsync(jy, c->accjy, c->G * 8, cudaMemcpyDeviceToHost, c->stream));
    double u[2];
    PIC_CUDA_TRY(cudaMemcpyAsync(u, c->junits, sizeof(u), cudaMemcpyDeviceToHost, c->stream));
    PIC_TRY(pic_gpu_synchronize(c));
    if (unit_x) *unit_x = u[0];
    if (unit_y) *unit_y = u[1];
    return PIC_OK;
}

}  // extern "C"
