// Stable LSD radix cell sort of the resident particles.
//
// Replaces pic::sortParticlesByCell (src/sorting/cell_sort.cpp:22-46), which
// sorts an index array with the unstable std::sort on particleCellIndex
// (cell_sort.cpp:8-13) and then gathers the six arrays. Here:
//   * the key is the stored cell key iy*Nx+ix (computed at upload with the
//     reference's cellCoords, so keys are identical to particleCellIndex);
//   * the sort is stable, 8-bit digits, ceil(log2(Nx*Ny)/8) passes over
//     (key, index) pairs; each pass = per-tile digit histogram, device scan of
//     the digit-major histogram table, and a scatter that ranks keys stably
//     inside the tile with warp match/ballot ranks and writes them out through
//     shared memory in digit runs;
//   * the payload (offsets, velocities, charge, mass) is gathered once through
//     the final permutation;
//   * per-cell offsets[Nx*Ny+1] come from a cell histogram and a scan.
#include "pic_internal.cuh"

namespace picgb {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;                        // per thread
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;      // 4096 keys per tile
constexpr int RS_WARP_ITEMS = RS_TILE / RS_WARPS;   // 512 keys per warp
constexpr int RS_RADIX = 256;

__global__ void __launch_bounds__(RS_THREADS) radix_histogram(const uint32_t* __restrict__ keys, size_t n,
                                                              int shift, uint32_t mask, uint32_t* __restrict__ counts,
                                                              unsigned num_tiles) {
    __shared__ uint32_t hist[RS_WARPS][RS_RADIX];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < RS_WARPS * RS_RADIX; i += RS_THREADS) (&hist[0][0])[i] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * RS_TILE + (size_t)warp * RS_WARP_ITEMS;
#pragma unroll 4
    for (int r = 0; r < RS_WARP_ITEMS / 32; ++r) {
        const size_t i = base + (size_t)r * 32 + lane;
        if (i < n) atomicAdd(&hist[warp][(keys[i] >> shift) & mask], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_RADIX; d += RS_THREADS) {
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) s += hist[w][d];
        counts[(size_t)d * num_tiles + blockIdx.x] = s;
    }
}

// Scatter of one radix pass. Tile order = (warp, round, lane) = input order, so
// ranks built warp by warp and round by round are stable.
__global__ void __launch_bounds__(RS_THREADS) radix_scatter(const uint32_t* __restrict__ keys_in,
                                                            const uint32_t* __restrict__ vals_in, int iota_vals,
                                                            uint32_t* __restrict__ keys_out,
                                                            uint32_t* __restrict__ vals_out, size_t n, int shift,
                                                            uint32_t mask, const uint32_t* __restrict__ offsets,
                                                            unsigned num_tiles) {
    __shared__ uint32_t wcnt[RS_WARPS][RS_RADIX];
    __shared__ uint32_t bstart[RS_RADIX];
    __shared__ uint32_t gstart[RS_RADIX];
    __shared__ uint32_t skeys[RS_TILE];
    __shared__ uint32_t svals[RS_TILE];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int i = threadIdx.x; i < RS_WARPS * RS_RADIX; i += RS_THREADS) (&wcnt[0][0])[i] = 0;
    for (int d = threadIdx.x; d < RS_RADIX; d += RS_THREADS) gstart[d] = offsets[(size_t)d * num_tiles + blockIdx.x];
    __syncthreads();

    const size_t tile_base = (size_t)blockIdx.x * RS_TILE;
    const size_t base = tile_base + (size_t)warp * RS_WARP_ITEMS;
    uint32_t k[RS_ITEMS], v[RS_ITEMS], rank[RS_ITEMS];
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const size_t i = base + (size_t)r * 32 + lane;
        const bool ok = i < n;
        k[r] = ok ? keys_in[i] : 0u;
        v[r] = ok ? (iota_vals ? (uint32_t)i : vals_in[i]) : 0u;
        // lanes with the same digit form one group; its lowest lane advances the
        // warp's counter for that digit by the group size and broadcasts the old value
        const uint32_t d = ok ? ((k[r] >> shift) & mask) : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        uint32_t basev = 0;
        if (ok && lane == leader) {
            basev = wcnt[warp][d];
            wcnt[warp][d] = basev + (uint32_t)__popc(peers);
        }
        basev = __shfl_sync(0xffffffffu, basev, leader);
        rank[r] = ok ? basev + (uint32_t)__popc(peers & lt_mask) : 0xffffffffu;
        __syncwarp();
    }
    __syncthreads();
    // per-digit warp prefix and tile-local digit starts
    if (threadIdx.x < RS_RADIX) {
        const int d = threadIdx.x;
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) {
            const uint32_t c = wcnt[w][d];
            wcnt[w][d] = s;
            s += c;
        }
        bstart[d] = s;  // total for now
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        // exclusive scan of 256 totals by one warp (8 per lane)
        uint32_t t[8];
        uint32_t s = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            t[j] = bstart[lane * 8 + j];
            s += t[j];
        }
        uint32_t inc = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        uint32_t run = inc - s;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            bstart[lane * 8 + j] = run;
            run += t[j];
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        if (rank[r] != 0xffffffffu) {
            const uint32_t d = (k[r] >> shift) & mask;
            const uint32_t lp = bstart[d] + wcnt[warp][d] + rank[r];
            skeys[lp] = k[r];
            svals[lp] = v[r];
        }
    }
    __syncthreads();
    const size_t rem = n - tile_base;
    const int tile_n = rem < (size_t)RS_TILE ? (int)rem : RS_TILE;
    for (int i = threadIdx.x; i < tile_n; i += RS_THREADS) {
        const uint32_t kk = skeys[i];
        const uint32_t d = (kk >> shift) & mask;
        const size_t g = (size_t)gstart[d] + (size_t)(i - (int)bstart[d]);
        keys_out[g] = kk;
        vals_out[g] = svals[i];
    }
}

__global__ void iota_u32(uint32_t* __restrict__ out, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint32_t)i;
}

struct GatherArgs {
    const uint32_t* perm;
    size_t n;
    const float* src[6];
    float* dst[6];
    int count;
};

__global__ void gather_payload(GatherArgs a) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const uint32_t p = a.perm[i];
#pragma unroll
    for (int k = 0; k < 6; ++k)
        if (k < a.count) a.dst[k][i] = __ldg(a.src[k] + p);
}

// Per-cell counts of the sorted keys; runs of equal keys inside a warp are
// aggregated (sorted input => one atomic per run).
__global__ void cell_histogram(const uint32_t* __restrict__ keys, size_t n, uint32_t G, uint32_t* __restrict__ cnt,
                               DevStats* st) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = i < n;
    uint32_t k = ok ? keys[i] : 0xffffffffu;
    if (ok && k >= G) {
        set_dev_error(st, DEV_BAD_CELL, (unsigned int)i);
        k = 0xfffffffeu;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    const int lane = threadIdx.x & 31;
    if (ok && k < G && lane == __ffs(peers) - 1) atomicAdd(&cnt[k], (uint32_t)__popc(peers));
}

int ensure_sort_scratch(pic_ctx* c) {
    const size_t cp = (c->cap ? c->cap : 1) + PARTICLE_PAD;
    int rc = PIC_OK;
    if (!c->cell_alt) c->cell_alt = (uint32_t*)dalloc(cp * 4, &rc);
    if (rc) return rc;
    if (!c->idx_a) c->idx_a = (uint32_t*)dalloc(cp * 4, &rc);
    if (rc) return rc;
    if (!c->idx_b) c->idx_b = (uint32_t*)dalloc(cp * 4, &rc);
    if (rc) return rc;
    for (int k = 0; k < 6; ++k) {
        if (k == 5 && !c->m) continue;
        if (!c->alt[k]) c->alt[k] = (float*)dalloc(cp * 4, &rc);
        if (rc) return rc;
    }
    if (!c->offsets) c->offsets = (uint32_t*)dalloc((c->G + 1) * 4, &rc);
    if (rc) return rc;
    if (!c->cellcount) c->cellcount = (uint32_t*)dalloc((c->G + 1) * 4, &rc);
    if (rc) return rc;
    const size_t tiles = (cp + RS_TILE - 1) / RS_TILE;
    const size_t need = tiles * RS_RADIX;
    if (c->counts_cap < need) {
        dfree(c->counts);
        c->counts = (uint32_t*)dalloc(need * 4, &rc);
        if (rc) {
            c->counts_cap = 0;
            return rc;
        }
        c->counts_cap = need;
    }
    return PIC_OK;
}

// Offsets of the (sorted) keys: histogram + exclusive scan over G+1 entries.
int build_offsets(pic_ctx* c, const uint32_t* keys) {
    PIC_CUDA_TRY(cudaMemsetAsync(c->offsets, 0, (c->G + 1) * 4, c->stream));
    if (c->n) {
        cell_histogram<<<(unsigned)((c->n + 255) / 256), 256, 0, c->stream>>>(keys, c->n, (uint32_t)c->G, c->offsets,
                                                                              c->dstats);
        PIC_TRY(check_launch(c, "cell_histogram"));
    }
    return exclusive_scan_u32(c, c->offsets, c->G + 1);
}

int sort_particles(pic_ctx* c) {
    PIC_TRY(ensure_sort_scratch(c));
    const size_t n = c->n;
    if (n == 0) {
        c->sorted = 1;
        c->part_valid = 1;
        return build_offsets(c, c->cell);
    }
    const unsigned tiles = (unsigned)((n + RS_TILE - 1) / RS_TILE);
    int bits = 0;
    while (bits < 32 && ((c->G - 1) >> bits) != 0) ++bits;
    uint32_t* kin = c->cell;
    uint32_t* kout = c->cell_alt;
    uint32_t* vin = c->idx_a;
    uint32_t* vout = c->idx_b;
    if (bits == 0) {
        iota_u32<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->idx_a, n);
        PIC_TRY(check_launch(c, "iota_u32"));
    }
    int pass = 0;
    for (int shift = 0; shift < bits; shift += 8, ++pass) {
        const int w = (bits - shift) < 8 ? (bits - shift) : 8;
        const uint32_t mask = (1u << w) - 1u;
        radix_histogram<<<tiles, RS_THREADS, 0, c->stream>>>(kin, n, shift, mask, c->counts, tiles);
        PIC_TRY(check_launch(c, "radix_histogram"));
        PIC_TRY(exclusive_scan_u32(c, c->counts, (size_t)RS_RADIX * tiles));
        radix_scatter<<<tiles, RS_THREADS, 0, c->stream>>>(kin, vin, pass == 0 ? 1 : 0, kout, vout, n, shift, mask,
                                                           c->counts, tiles);
        PIC_TRY(check_launch(c, "radix_scatter"));
        uint32_t* t = kin;
        kin = kout;
        kout = t;
        t = vin;
        vin = vout;
        vout = t;
    }
    // kin = sorted keys, vin = permutation
    if (kin != c->cell) {
        uint32_t* t = c->cell;
        c->cell = kin;
        c->cell_alt = t;
    }
    if (vin != c->idx_a) {
        uint32_t* t = c->idx_a;
        c->idx_a = vin;
        c->idx_b = t;
    }
    GatherArgs g;
    g.perm = c->idx_a;
    g.n = n;
    // the payload: offsets, velocities, charges (not when uniform: any order of
    // equal values is the same array) and masses (when stored)
    float** slots[6] = {&c->xr, &c->yr, &c->vx, &c->vy, &c->q, &c->m};
    int fields[6], nf = 0;
    for (int k = 0; k < 6; ++k)
        if ((k != 4 || c->qn_uniform == 0.0f) && (k != 5 || c->has_mass)) fields[nf++] = k;
    g.count = nf;
    for (int j = 0; j < nf; ++j) {
        g.src[j] = *slots[fields[j]];
        g.dst[j] = c->alt[fields[j]];
    }
    gather_payload<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(g);
    PIC_TRY(check_launch(c, "gather_payload"));
    for (int j = 0; j < nf; ++j) {
        const int k = fields[j];
        float* t = *slots[k];
        *slots[k] = c->alt[k];
        c->alt[k] = t;
    }
    PIC_TRY(build_offsets(c, c->cell));
    c->sorted = 1;
    c->part_valid = 1;
    return PIC_OK;
}

}  // namespace picgb

using namespace picgb;

extern "C" int pic_gpu_sort(pic_ctx* c, uint32_t* keys_out, uint32_t* perm_out, uint32_t* offsets_out) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    prof_begin(c, "sort");
    const int rc = sort_particles(c);
    prof_end(c);
    PIC_TRY(rc);
    if (keys_out && c->n)
        PIC_CUDA_TRY(cudaMemcpyAsync(keys_out, c->cell, c->n * 4, cudaMemcpyDeviceToHost, c->stream));
    if (perm_out && c->n)
        PIC_CUDA_TRY(cudaMemcpyAsync(perm_out, c->idx_a, c->n * 4, cudaMemcpyDeviceToHost, c->stream));
    if (offsets_out)
        PIC_CUDA_TRY(cudaMemcpyAsync(offsets_out, c->offsets, (c->G + 1) * 4, cudaMemcpyDeviceToHost, c->stream));
    if (keys_out || perm_out || offsets_out) return pic_gpu_synchronize(c);
    return PIC_OK;
}
