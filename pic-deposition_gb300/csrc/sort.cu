// Stable LSD radix cell sort of the resident particles.
//
// Replaces pic::sortParticlesByCell (src/sorting/cell_sort.cpp:22-46), which
// sorts an index array with the unstable std::sort on particleCellIndex
// (cell_sort.cpp:8-13) and then gathers the six arrays. Here:
//   * the key is the stored cell key iy*Nx+ix (computed at upload with the
//     reference's cellCoords, so keys are identical to particleCellIndex);
//   * the sort is stable and least-significant digit first, with digits of up
//     to 10 bits: ceil(bits/10) passes (two at 1024^2 cells, three at 2048^2). A
//     pass is a per-tile digit histogram, a device scan of the digit-major
//     histogram table, and a scatter that ranks the tile's keys stably with
//     warp match/ballot ranks and moves the keys and the whole payload
//     (offsets, velocities, charge and mass where stored, and the permutation)
//     through shared memory to the output in digit runs: every global read
//     and write is coalesced, and no random gather follows the last pass;
//   * per-cell offsets[Nx*Ny+1] are written from the sorted keys: where the key
//     changes between i-1 and i, offsets of the cells in between are i.
#include <utility>

#include "pic_internal.cuh"

namespace picgb {

constexpr int RS_THREADS = 512;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;                        // per thread
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;      // 8192 keys per tile: a 10-bit digit's run fills a sector
constexpr int RS_WARP_ITEMS = RS_TILE / RS_WARPS;   // 512 keys per warp
constexpr int RS_MAX_BITS = 10;                     // widest digit (wider ones spill, one CTA per SM)
constexpr int RS_MAX_PAYLOAD = 7;                   // xr yr vx vy q m perm

// Digit histogram of one tile. Each thread counts 16 consecutive keys (four
// 16-byte loads, all issued before the first count) and adds each run of equal
// digits with one shared atomic: about one atomic per thread for cell-ordered
// input. Keys are read with the streaming (evict-first) policy.
template <int BITS>
__global__ void __launch_bounds__(RS_THREADS) radix_histogram(const uint32_t* __restrict__ keys, size_t n,
                                                              int shift, uint32_t mask, uint32_t* __restrict__ counts,
                                                              unsigned num_tiles) {
    constexpr int RADIX = 1 << BITS;
    static_assert(RS_ITEMS % 4 == 0, "whole 16-byte loads");
    __shared__ uint32_t hist[RADIX];
    for (int i = threadIdx.x; i < RADIX; i += RS_THREADS) hist[i] = 0;
    // key arrays hold PARTICLE_PAD words past the last particle and start 16-byte
    // aligned, so a thread's four loads stay inside the allocation
    const size_t base = (size_t)blockIdx.x * RS_TILE + (size_t)threadIdx.x * RS_ITEMS;
    uint4 v[RS_ITEMS / 4];
    if (base < n) {
#pragma unroll
        for (int j = 0; j < RS_ITEMS / 4; ++j) v[j] = __ldcs(reinterpret_cast<const uint4*>(keys + base) + j);
    }
    __syncthreads();
    if (base < n) {
        const int cnt = (n - base) < (size_t)RS_ITEMS ? (int)(n - base) : RS_ITEMS;
        uint32_t run_d = (v[0].x >> shift) & mask, run_n = 0;
#pragma unroll
        for (int j = 0; j < RS_ITEMS; ++j) {
            if (j < cnt) {
                const uint4& w = v[j >> 2];
                const uint32_t kj = (j & 3) == 0 ? w.x : (j & 3) == 1 ? w.y : (j & 3) == 2 ? w.z : w.w;
                const uint32_t d = (kj >> shift) & mask;
                if (d != run_d) {
                    atomicAdd(&hist[run_d], run_n);
                    run_d = d;
                    run_n = 0;
                }
                ++run_n;
            }
        }
        atomicAdd(&hist[run_d], run_n);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += RS_THREADS) counts[(size_t)d * num_tiles + blockIdx.x] = hist[d];
}

// The fields moved with the keys by a scatter pass: 32-bit words per particle.
struct Payload {
    const uint32_t* src[RS_MAX_PAYLOAD];  // NULL with iota: the field is the particle's input index
    uint32_t* dst[RS_MAX_PAYLOAD];
    int count;
};

// Shared memory of the scatter: per-warp 16-bit digit counters (a warp ranks at
// most 512 keys), tile digit starts, global digit starts, the tile's keys (then
// each tile slot's output index) and one staged payload field.
template <int BITS>
__host__ __device__ constexpr size_t scatter_smem_bytes() {
    return (size_t)RS_WARPS * (1 << BITS) * 2 + (2 * (size_t)(1 << BITS) + 2 * (size_t)RS_TILE) * 4;
}

// Scatter of one radix pass. Tile order = (warp, round, lane) = input order, so
// ranks built warp by warp and round by round are stable.
template <int BITS>
__global__ void __launch_bounds__(RS_THREADS, 2) radix_scatter(const uint32_t* __restrict__ keys_in,
                                                               uint32_t* __restrict__ keys_out, size_t n, int shift,
                                                               uint32_t mask, const uint32_t* __restrict__ offsets,
                                                               unsigned num_tiles, Payload pay) {
    constexpr int RADIX = 1 << BITS;
    extern __shared__ uint32_t rs_smem[];
    uint32_t* bstart = rs_smem;                     // [RADIX]
    uint32_t* gstart = bstart + RADIX;              // [RADIX]
    uint32_t* skeys = gstart + RADIX;               // [RS_TILE]: keys, then output indices
    uint32_t* sval = skeys + RS_TILE;               // [RS_TILE]
    uint16_t* wcnt = reinterpret_cast<uint16_t*>(sval + RS_TILE);  // [RS_WARPS][RADIX]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int i = threadIdx.x; i < RS_WARPS * RADIX; i += RS_THREADS) wcnt[i] = 0;
    for (int d = threadIdx.x; d < RADIX; d += RS_THREADS) gstart[d] = offsets[(size_t)d * num_tiles + blockIdx.x];
    __syncthreads();

    const size_t tile_base = (size_t)blockIdx.x * RS_TILE;
    const size_t base = tile_base + (size_t)warp * RS_WARP_ITEMS;
    uint32_t k[RS_ITEMS], rank[RS_ITEMS];
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const size_t i = base + (size_t)r * 32 + lane;
        const bool ok = i < n;
        k[r] = ok ? __ldcs(keys_in + i) : 0u;
        // lanes with the same digit form one group; its lowest lane advances the
        // warp's counter for that digit by the group size and broadcasts the old value
        const uint32_t d = ok ? ((k[r] >> shift) & mask) : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        uint32_t basev = 0;
        if (ok && lane == leader) {
            basev = wcnt[warp * RADIX + d];
            wcnt[warp * RADIX + d] = (uint16_t)(basev + (uint32_t)__popc(peers));
        }
        basev = __shfl_sync(0xffffffffu, basev, leader);
        rank[r] = ok ? basev + (uint32_t)__popc(peers & lt_mask) : 0xffffffffu;
        __syncwarp();
    }
    __syncthreads();
    // per-digit warp prefix and the tile's digit totals
    for (int d = threadIdx.x; d < RADIX; d += RS_THREADS) {
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) {
            const uint32_t c = wcnt[w * RADIX + d];
            wcnt[w * RADIX + d] = (uint16_t)s;  // a tile holds at most 8192 keys
            s += c;
        }
        bstart[d] = s;  // total for now
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        // exclusive scan of the RADIX totals by one warp (RADIX/32 per lane)
        constexpr int PER = RADIX / 32 > 0 ? RADIX / 32 : 1;
        uint32_t s = 0;
        for (int j = 0; j < PER; ++j) s += lane * PER + j < RADIX ? bstart[lane * PER + j] : 0u;
        uint32_t inc = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        uint32_t run = inc - s;
        for (int j = 0; j < PER; ++j)
            if (lane * PER + j < RADIX) {
                const uint32_t t = bstart[lane * PER + j];
                bstart[lane * PER + j] = run;
                run += t;
            }
    }
    __syncthreads();
    // tile slot of every item
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        if (rank[r] != 0xffffffffu) {
            const uint32_t d = (k[r] >> shift) & mask;
            rank[r] = bstart[d] + wcnt[warp * RADIX + d] + rank[r];
            skeys[rank[r]] = k[r];
        }
    }
    __syncthreads();
    const size_t rem = n - tile_base;
    const int tile_n = rem < (size_t)RS_TILE ? (int)rem : RS_TILE;
    // the first payload field, read in input order while the keys are written out
    uint32_t pv[RS_ITEMS];
    auto load_field = [&](int f) {
        const uint32_t* src = pay.src[f];
#pragma unroll
        for (int r = 0; r < RS_ITEMS; ++r) {
            const size_t i = base + (size_t)r * 32 + lane;
            pv[r] = rank[r] == 0xffffffffu ? 0u : (src ? __ldcs(src + i) : (uint32_t)i);
        }
    };
    if (pay.count > 0) load_field(0);
    // tile slot i goes to gstart[d] + (i - bstart[d]): consecutive slots of a digit are
    // consecutive outputs; each slot's output index replaces its key in skeys
    for (int i = threadIdx.x; i < tile_n; i += RS_THREADS) {
        const uint32_t kk = skeys[i];
        const uint32_t d = (kk >> shift) & mask;
        const uint32_t g = gstart[d] + (uint32_t)(i - (int)bstart[d]);
        keys_out[g] = kk;
        skeys[i] = g;
    }
    // the payload, one field at a time through the staging buffer; the next
    // field's loads are issued before this one is written out
    for (int f = 0; f < pay.count; ++f) {
#pragma unroll
        for (int r = 0; r < RS_ITEMS; ++r)
            if (rank[r] != 0xffffffffu) sval[rank[r]] = pv[r];
        __syncthreads();
        if (f + 1 < pay.count) load_field(f + 1);
        uint32_t* dst = pay.dst[f];
        for (int i = threadIdx.x; i < tile_n; i += RS_THREADS) dst[skeys[i]] = sval[i];
        __syncthreads();
    }
}

__global__ void iota_u32(uint32_t* __restrict__ out, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint32_t)i;
}

// offsets[c] = the first index whose key is >= c, from cell-ordered keys: index
// i writes i into offsets[keys[i-1]+1 .. keys[i]] (index 0 from cell 0), the
// last index also offsets[keys[n-1]+1 .. G]. Every entry is written once. Four
// keys per thread (one 16-byte load; the key before them comes from the
// previous lane, lane 0 loads it). A range of more than OFS_SHORT cells (empty
// cells between two particles) is left to the whole warp, 32 entries per store
// instruction, so a sparse or lopsided distribution costs no long serial loop.
constexpr uint32_t OFS_SHORT = 16;

// Range j of a thread's four keys k (j = 4: the cells after the last particle):
// cells [from, end) get val; false when there is none.
__device__ __forceinline__ bool offsets_range(int j, const uint32_t (&k)[4], uint32_t before, size_t i0, int cnt,
                                              size_t n, uint32_t G, uint32_t& from, uint32_t& end, uint32_t& val) {
    if (j < 4) {
        if (j >= cnt) return false;
        const uint32_t prev = j == 0 ? before : k[j - 1];
        from = (j == 0 && i0 == 0) ? 0u : (prev >= G ? G : prev + 1u);
        end = k[j] < G ? k[j] + 1u : G;
        val = (uint32_t)(i0 + j);
        return true;
    }
    if (cnt == 0 || i0 + (size_t)cnt != n || k[cnt - 1] >= G) return false;
    from = k[cnt - 1] + 1u;
    end = G + 1u;
    val = (uint32_t)n;
    return true;
}

__global__ void offsets_from_sorted(const uint32_t* __restrict__ keys, size_t n, uint32_t G,
                                    uint32_t* __restrict__ offsets, DevStats* st) {
    const int lane = threadIdx.x & 31;
    const size_t i0 = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    const bool act = i0 < n;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (act) v = __ldcs(reinterpret_cast<const uint4*>(keys + i0));  // padded, 16-byte aligned array
    uint32_t before = __shfl_up_sync(0xffffffffu, v.w, 1);
    if (act && lane == 0 && i0 > 0) before = keys[i0 - 1];
    const uint32_t k[4] = {v.x, v.y, v.z, v.w};
    const int cnt = act ? ((n - i0) < 4 ? (int)(n - i0) : 4) : 0;
    for (int j = 0; j < cnt; ++j)
        if (k[j] >= G) set_dev_error(st, DEV_BAD_CELL, (unsigned int)(i0 + j));
    unsigned longs = 0;  // ranges left to the warp
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        uint32_t from, end, val;
        if (offsets_range(j, k, before, i0, cnt, n, G, from, end, val)) {
            if (end > from + OFS_SHORT)
                longs |= 1u << j;
            else
                for (uint32_t c = from; c < end; ++c) offsets[c] = val;
        }
    }
    unsigned m = __ballot_sync(0xffffffffu, longs != 0);
    while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1u;
        const unsigned sl = __shfl_sync(0xffffffffu, longs, src);
        const uint32_t sk[4] = {__shfl_sync(0xffffffffu, k[0], src), __shfl_sync(0xffffffffu, k[1], src),
                                __shfl_sync(0xffffffffu, k[2], src), __shfl_sync(0xffffffffu, k[3], src)};
        const uint32_t sb = __shfl_sync(0xffffffffu, before, src);
        const int sc = __shfl_sync(0xffffffffu, cnt, src);
        const size_t si = i0 + 4 * (size_t)(src - lane);
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            uint32_t from, end, val;
            if (((sl >> j) & 1u) && offsets_range(j, sk, sb, si, sc, n, G, from, end, val))
                for (uint32_t c = from + (uint32_t)lane; c < end; c += 32u) offsets[c] = val;
        }
    }
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
    const size_t need = tiles * ((size_t)1 << RS_MAX_BITS);
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

// Offsets of cell-ordered keys (every caller's keys are: a sort's output, an
// upload found in order, a one-cell grid).
int build_offsets(pic_ctx* c, const uint32_t* keys) {
    if (c->n == 0) {
        PIC_CUDA_TRY(cudaMemsetAsync(c->offsets, 0, (c->G + 1) * 4, c->stream));
        return PIC_OK;
    }
    offsets_from_sorted<<<(unsigned)((c->n + 1023) / 1024), 256, 0, c->stream>>>(keys, c->n, (uint32_t)c->G,
                                                                                  c->offsets, c->dstats);
    return check_launch(c, "offsets_from_sorted");
}

template <int BITS>
static int launch_pass(pic_ctx* c, const uint32_t* kin, uint32_t* kout, size_t n, int shift, uint32_t mask,
                       unsigned tiles, const Payload& pay) {
    radix_histogram<BITS><<<tiles, RS_THREADS, 0, c->stream>>>(kin, n, shift, mask, c->counts, tiles);
    PIC_TRY(check_launch(c, "radix_histogram"));
    PIC_TRY(exclusive_scan_u32(c, c->counts, ((size_t)1 << BITS) * tiles));
    const size_t smem = scatter_smem_bytes<BITS>();
    PIC_TRY(opt_in_dynamic_smem((const void*)radix_scatter<BITS>, smem));
    radix_scatter<BITS><<<tiles, RS_THREADS, smem, c->stream>>>(kin, kout, n, shift, mask, c->counts, tiles, pay);
    return check_launch(c, "radix_scatter");
}

int sort_particles(pic_ctx* c, bool perm) {
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
    if (bits == 0) {  // one cell: already in order; the permutation is the identity
        if (perm) {
            iota_u32<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->idx_a, n);
            PIC_TRY(check_launch(c, "iota_u32"));
        }
        PIC_TRY(build_offsets(c, c->cell));
        c->sorted = 1;
        c->part_valid = 1;
        return PIC_OK;
    }
    const int passes = (bits + RS_MAX_BITS - 1) / RS_MAX_BITS;
    const int width = (bits + passes - 1) / passes;
    // the payload: offsets, velocities, charges (not when uniform: any order of
    // equal values is the same array), masses (when stored) and, when asked for,
    // the permutation
    float** slots[6] = {&c->xr, &c->yr, &c->vx, &c->vy, &c->q, &c->m};
    int fields[6], nf = 0;
    for (int k = 0; k < 6; ++k)
        if ((k != 4 || c->qn_uniform == 0.0f) && (k != 5 || c->has_mass)) fields[nf++] = k;
    for (int pass = 0, shift = 0; pass < passes; ++pass, shift += width) {
        const int w = (bits - shift) < width ? (bits - shift) : width;
        const uint32_t mask = (1u << w) - 1u;
        Payload pay;
        pay.count = nf + (perm ? 1 : 0);
        for (int j = 0; j < nf; ++j) {
            pay.src[j] = reinterpret_cast<const uint32_t*>(*slots[fields[j]]);
            pay.dst[j] = reinterpret_cast<uint32_t*>(c->alt[fields[j]]);
        }
        if (perm) {
            pay.src[nf] = pass == 0 ? nullptr : c->idx_a;  // the first pass starts from the identity
            pay.dst[nf] = c->idx_b;
        }
        int rc;
        if (width <= 8)
            rc = launch_pass<8>(c, c->cell, c->cell_alt, n, shift, mask, tiles, pay);
        else if (width <= 9)
            rc = launch_pass<9>(c, c->cell, c->cell_alt, n, shift, mask, tiles, pay);
        else
            rc = launch_pass<10>(c, c->cell, c->cell_alt, n, shift, mask, tiles, pay);
        PIC_TRY(rc);
        std::swap(c->cell, c->cell_alt);
        if (perm) std::swap(c->idx_a, c->idx_b);
        for (int j = 0; j < nf; ++j) std::swap(*slots[fields[j]], c->alt[fields[j]]);
    }
    PIC_TRY(build_offsets(c, c->cell));
    // deposits between the sorts start again with the cell kernel
    PIC_CUDA_TRY(cudaMemsetAsync(&c->dstats->any_order, 0, sizeof(unsigned int), c->stream));
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
    const int rc = sort_particles(c, true);
    prof_end(c);
    PIC_TRY(rc);
    c->sorts++;
    if (keys_out && c->n)
        PIC_CUDA_TRY(cudaMemcpyAsync(keys_out, c->cell, c->n * 4, cudaMemcpyDeviceToHost, c->stream));
    if (perm_out && c->n)
        PIC_CUDA_TRY(cudaMemcpyAsync(perm_out, c->idx_a, c->n * 4, cudaMemcpyDeviceToHost, c->stream));
    if (offsets_out)
        PIC_CUDA_TRY(cudaMemcpyAsync(offsets_out, c->offsets, (c->G + 1) * 4, cudaMemcpyDeviceToHost, c->stream));
    if (keys_out || perm_out || offsets_out) return pic_gpu_synchronize(c);
    return PIC_OK;
}
