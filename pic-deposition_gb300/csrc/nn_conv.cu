// 3x3 periodic convolutions as implicit GEMMs on the 5th-generation tensor cores.
//
// Forward / input-gradient kernel (conv3x3_kernel): one CTA owns a 128-pixel
// segment of a run of image rows. The GEMM per output row is
//     D[128 px][cout] = sum over 9 taps of A_tap[128 px][cin] * B_tap[cin][cout]
// with D in tensor memory (FP32), issued as tcgen05.mma kind::f16 (BF16 x BF16,
// M = 128, N = cout, K = 16) by one thread. The input rows are staged in shared
// memory as "planes" of 8 channels: pixel slot s of plane j holds the 16 bytes of
// channels 8j..8j+7 of pixel x0-1+s. In the K-major no-swizzle operand layout
// (8-row core matrices of 16-byte rows, stride between row groups SBO = 128 B,
// between the two K halves LBO = one plane) row r of A sits at r*16 bytes, so
// the operand of tap dx is the same staged row with its start moved by
// (dx+1)*16 bytes: im2col costs nothing. Warp-specialised: one warp stages rows
// into a ring of 6 slots, one thread issues the MMAs of row y into one TMEM
// buffer while four warps drain row y-1 from the other (bias + ReLU, or the
// ReLU mask of the backward pass), handing over through mbarriers.
//
// Weight-gradient kernel (wgrad_kernel): D[(dy, ci)][(dx, co)] = sum over pixels
// of x[p + (dy, dx)][ci] * dy[p][co], K = pixels, both operands MN-major as they
// sit in NHWC memory (see the kernel's comment); the bias gradient is one more
// MMA per K step against an all-ones operand. Each CTA accumulates its blocks
// of pixels in TMEM and writes one partial sum; reduce_wgrad adds the partials
// in a fixed order, so gradients are identical run to run.
//
// Every wait on the tensor cores is bounded (about one second of %globaltimer);
// on expiry the kernel records an error, skips the remaining work, frees its
// tensor memory and returns.
#include <cuda_bf16.h>

#include "nn_conv.cuh"
#include "pic_internal.cuh"

namespace picnn {

namespace {

constexpr int SLOTS = 130;             // pixels x0-1 .. x0+128
constexpr int PLANE = SLOTS * 16;      // bytes per 8-channel plane
constexpr int THREADS = 128;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Waits for phase `parity` of the barrier; false after about one second.
__device__ bool mbar_wait(uint32_t a, uint32_t parity) {
    if (mbar_try(a, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try(a, parity))
        if (globaltimer_ns() - t0 > 1000000000ull) return false;
    return true;
}

__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void tmem_load(uint32_t taddr, float* v) {
    uint32_t r[N];
#pragma unroll
    for (int c = 0; c < N; c += 16) tmem_ld16(taddr + c, r + c);
    tmem_wait_ld();
#pragma unroll
    for (int c = 0; c < N; ++c) v[c] = __uint_as_float(r[c]);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__host__ __device__ constexpr uint32_t tmem_cols(int n) { return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : 256u; }

// ---------------------------------------------------------------------------
// forward / input gradient
// ---------------------------------------------------------------------------
template <int COUT, int EPI>
__device__ __forceinline__ void conv_epilogue(const ConvLaunch& a, int b, int y, int x0, uint32_t taddr,
                                              const float* sbias, int warp, int lane) {
    float v[COUT];
    tmem_load<COUT>(taddr, v);
    const int px = x0 + warp * 32 + lane;
    const size_t pix = ((size_t)b * a.H + y) * a.W + px;
    if (EPI == EPI_BIAS_OUT) {
        reinterpret_cast<float*>(a.y)[pix] = v[0] + sbias[0];
        return;
    }
    if (EPI == EPI_BIAS_RELU) {
#pragma unroll
        for (int c = 0; c < COUT; ++c) v[c] = fmaxf(v[c] + sbias[c], 0.0f);
    } else {
        const uint4* m = reinterpret_cast<const uint4*>(a.mask + pix * COUT);
#pragma unroll
        for (int q = 0; q < COUT / 8; ++q) {
            const uint4 mm = m[q];
            const uint32_t w[4] = {mm.x, mm.y, mm.z, mm.w};
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int16_t bits = (int16_t)((w[e >> 1] >> ((e & 1) * 16)) & 0xFFFFu);
                if (!(bits > 0)) v[q * 8 + e] = 0.0f;
            }
        }
    }
    uint4* out = reinterpret_cast<uint4*>(reinterpret_cast<uint16_t*>(a.y) + pix * COUT);
#pragma unroll
    for (int q = 0; q < COUT / 8; ++q) {
        uint4 o;
        o.x = pack_bf16x2(v[q * 8 + 0], v[q * 8 + 1]);
        o.y = pack_bf16x2(v[q * 8 + 2], v[q * 8 + 3]);
        o.z = pack_bf16x2(v[q * 8 + 4], v[q * 8 + 5]);
        o.w = pack_bf16x2(v[q * 8 + 6], v[q * 8 + 7]);
        out[q] = o;
    }
}

template <int CIN, int COUT>
struct ConvSmem {
    static constexpr int PLANES = CIN / 8;
    static constexpr int SLOT = PLANES * PLANE;
    static constexpr int WBYTES = 9 * CIN * COUT * 2;
    static constexpr int OFF_BIAS = WBYTES;
    static constexpr int OFF_RING = ((WBYTES + COUT * 4) + 127) / 128 * 128;
    static constexpr int BYTES = OFF_RING + 6 * SLOT;
};

__device__ __forceinline__ void mbar_arrive_cta(uint32_t a) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}

// Warp-specialised: warp 4 stages input rows into the ring (cp.async), lane 0
// of warp 5 issues each output row's MMAs, warps 0-3 (one TMEM lane quarter
// each) run the epilogue of the previous row from the other TMEM buffer.
// Barriers: full[s] (32 producer arrivals: the row in slot s has landed),
// rowfree[s] (an MMA commit: the last output row that reads slot s is done),
// tfull[b] (an MMA commit: accumulator b holds a row), tempty[b] (128
// epilogue arrivals: accumulator b has been read). Every wait is bounded and
// no role waits at a CTA barrier inside the loop.
constexpr int CONV_THREADS = 192;
constexpr int NRING = 6;

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(CONV_THREADS) conv3x3_kernel(ConvLaunch a) {
    using L = ConvSmem<CIN, COUT>;
    constexpr int KSTEPS = CIN / 16;
    constexpr uint32_t IDESC = idesc_bf16(128, COUT);
    constexpr uint32_t TCOLS = tmem_cols(2 * COUT);
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[NRING], rowfree[NRING], tfull[2], tempty[2];
    __shared__ uint32_t tmem_slot;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int x0 = blockIdx.x * 128;
    const int b = blockIdx.z;
    const int y_begin = blockIdx.y * a.rows_per_cta;
    const int y_end = min(a.H, y_begin + a.rows_per_cta);
    if (y_begin >= y_end) return;
    const int nout = y_end - y_begin, nrows = nout + 2;  // output rows; staged rows y_begin-1 .. y_end
    const uint32_t s_w = smem_addr(smem);
    const uint32_t s_ring = s_w + L::OFF_RING;
    float* sbias = reinterpret_cast<float*>(smem + L::OFF_BIAS);

    for (int i = tid; i < L::WBYTES / 16; i += CONV_THREADS)
        cp_async16(s_w + i * 16, reinterpret_cast<const uint8_t*>(a.wimg) + (size_t)i * 16);
    if (EPI != EPI_MASK && tid < COUT) sbias[tid] = a.bias[tid];
    cp_async_wait_all();
    fence_async_smem();
    if (tid == 0) {
        for (int i = 0; i < NRING; ++i) {
            mbar_init(smem_addr(&full[i]), 32);
            mbar_init(smem_addr(&rowfree[i]), 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_addr(&tfull[i]), 1);
            mbar_init(smem_addr(&tempty[i]), 128);
        }
    }
    if (warp == 0) tmem_alloc(smem_addr(&tmem_slot), TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    auto slot_addr = [&](int rr) { return s_ring + (uint32_t)((rr % NRING) * L::SLOT); };

    int ok = 1;
    if (warp == 4) {
        // producer: staged row rr (input row y_begin - 1 + rr) into slot rr % NRING
        for (int rr = 0; rr < nrows; ++rr) {
            if (rr >= NRING &&
                !mbar_wait(smem_addr(&rowfree[rr % NRING]), ((rr / NRING) - 1) & 1)) {
                ok = 0;
                break;
            }
            constexpr int PLANES = CIN / 8;
            const int yy = (((y_begin - 1 + rr) % a.H) + a.H) % a.H;
            const uint16_t* row = a.x + ((size_t)b * a.H + yy) * (size_t)a.W * CIN;
            const uint32_t dst = slot_addr(rr);
            for (int t = lane; t < SLOTS * PLANES; t += 32) {
                const int sl = t / PLANES, j = t - sl * PLANES;
                int xx = x0 - 1 + sl;
                if (xx < 0) xx += a.W;
                if (xx >= a.W) xx -= a.W;
                cp_async16(dst + (uint32_t)(j * PLANE + sl * 16), row + (size_t)xx * CIN + j * 8);
            }
            cp_async_commit();
            if (rr >= 1) {  // the previous row's copies have landed: hand it over
                cp_async_wait_group<1>();
                fence_async_smem();
                mbar_arrive_cta(smem_addr(&full[(rr - 1) % NRING]));
            }
        }
        if (ok) {
            cp_async_wait_group<0>();
            fence_async_smem();
            mbar_arrive_cta(smem_addr(&full[(nrows - 1) % NRING]));
        }
    } else if (warp == 5) {
        if (lane == 0) {
            // MMA issuer: output row i reads staged rows i, i+1, i+2
            for (int i = 0; i < nout && ok; ++i) {
                for (int rr = (i == 0 ? 0 : i + 2); rr <= i + 2; ++rr)
                    if (!mbar_wait(smem_addr(&full[rr % NRING]), (rr / NRING) & 1)) ok = 0;
                if (ok && i >= 2 && !mbar_wait(smem_addr(&tempty[i & 1]), ((i >> 1) - 1) & 1)) ok = 0;
                if (!ok) break;
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)((i & 1) * COUT);
                int k = 0;
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    const int dy = t / 3, dx = t % 3;  // staged row i + dy, pixel offset dx
                    const uint32_t arow = slot_addr(i + dy) + dx * 16;
#pragma unroll
                    for (int s = 0; s < KSTEPS; ++s, ++k) {
                        const uint64_t ad = umma_desc(arow + 2 * s * PLANE, PLANE, 128);
                        const uint64_t bd = umma_desc(s_w + (t * L::PLANES + 2 * s) * COUT * 16, COUT * 16, 128);
                        mma_bf16(d, ad, bd, IDESC, k > 0 ? 1u : 0u);
                    }
                }
                mma_commit(smem_addr(&tfull[i & 1]));
                mma_commit(smem_addr(&rowfree[i % NRING]));  // staged row i: its last reader
            }
        }
        __syncwarp();
    } else {
        // epilogue warps 0-3: TMEM lanes 32*warp .. 32*warp + 31 = pixels
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        for (int i = 0; i < nout; ++i) {
            // the TMEM load below is warp-aligned: the warp decides together
            if (!__all_sync(0xffffffffu, mbar_wait(smem_addr(&tfull[i & 1]), (i >> 1) & 1))) {
                ok = 0;
                break;
            }
            tc_fence_after();
            conv_epilogue<COUT, EPI>(a, b, y_begin + i, x0, lane_base + (i & 1) * COUT, sbias, warp, lane);
            tc_fence_before();
            mbar_arrive_cta(smem_addr(&tempty[i & 1]));
        }
    }
    cp_async_wait_all();
    ok = __syncthreads_and(ok);
    if (!ok && tid == 0) atomicExch(a.err, 1);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TCOLS);
    }
}

// ---------------------------------------------------------------------------
// weight gradient
// ---------------------------------------------------------------------------
// Both operands are MN-major: A[m][k] = x with m = (row offset, channel) and
// k = pixel, B[k][n] = dy with n = output channel. Staged as 8-channel planes
// (16 bytes per pixel slot) they are the canonical MN-major no-swizzle layout:
// a core matrix is 8 pixels (K, 16 B apart) of 8 channels (MN, contiguous); K
// core matrices are 128 B apart (LBO), MN core matrices one plane apart (SBO).
// With the staged x rows of a block one after the other, the 16 MN core
// matrices of an M = 128 operand starting at row i are rows i .. i + 128/CIN - 1:
// rows i, i+1, i+2 are the taps dy = -1, 0, 1 of output row i (the rest is
// discarded), and the tap dx moves the start by one 16-byte pixel slot. The
// bias gradient is one more MMA per K step, of a constant all-ones A.
//
// Staging: a row of a block is one TMA copy (cp.async.bulk.tensor) of a box of
// 8 channels x 34 (or 40) pixels x planes through a 5-D view of the NHWC tensor whose
// pixel stride is the pixel's size and whose plane stride is 16 bytes, so the
// box lands plane by plane; the periodic row wrap is the row coordinate. The two
// segments at the ends of an image row, whose pixel halo wraps around, are
// staged with cp.async by three warps instead.
constexpr int WG_ROWS = 8;    // output rows per block
constexpr int WG_PX = 32;     // output pixels per block (one K segment)
constexpr int WG_SLOTS = 34;  // x pixels used: x0-1 .. x0+32
constexpr int WG_DPLANE = WG_PX * 16;
constexpr int WG_NBUF = 2;    // blocks in the shared-memory ring
constexpr int WG_ONES = 16 * 256;  // all-ones A operand: 16 MN x 2 K core matrices

template <int CIN, int COUT>
struct WgSmem {
    static constexpr int G = 128 / CIN;                 // x rows spanned by one M = 128 operand
    static constexpr int XROWS = WG_ROWS + G - 1;       // staged x rows per block
    // x pixels per TMA box: the 34 used, or 40 where 34 would leave the rows off
    // the 128-byte alignment of a TMA destination
    static constexpr int XBOX = ((CIN / 8) * 34 * 16) % 128 == 0 ? 34 : 40;
    static constexpr int XPLANE = XBOX * 16;
    static constexpr int XROW = (CIN / 8) * XPLANE;     // bytes per staged x row
    static constexpr int DROW = (COUT / 8) * WG_DPLANE;
    static constexpr int XBYTES = XROWS * XROW;
    static constexpr int DBYTES = WG_ROWS * DROW;
    static constexpr int BUF = (XBYTES + DBYTES + 127) / 128 * 128;
    static constexpr int OFF_ONES = WG_NBUF * BUF;
    static constexpr int BYTES = OFF_ONES + WG_ONES;
};

__device__ __forceinline__ void cp_async_wait_all_groups() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint32_t a, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, int c1, int c2, int c3, int c4,
                                            uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(mbar)
        : "memory");
}

// Instruction descriptor of kind::f16 with both operands MN-major.
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int m, int n) {
    return idesc_bf16(m, n) | (1u << 15) | (1u << 16);
}

struct WgBlock {
    int b, y0, x0, rows;
    bool edge;  // the x halo wraps around the image row: staged with cp.async
};

__device__ __forceinline__ WgBlock wg_block(const WgradLaunch& a, long long blk) {
    const int segs = a.W / WG_PX, yblocks = (a.H + WG_ROWS - 1) / WG_ROWS;
    WgBlock k;
    const int seg = (int)(blk % segs);
    const long long r2 = blk / segs;
    k.y0 = (int)(r2 % yblocks) * WG_ROWS;
    k.b = (int)(r2 / yblocks);
    k.x0 = seg * WG_PX;
    k.rows = min(WG_ROWS, a.H - k.y0);
    k.edge = seg == 0 || seg == segs - 1;
    return k;
}

// cp.async staging of a block by the 96 producer threads (pt = 0..95): the same
// layout as the TMA boxes (slots past 33 of a plane, if any, are not written or read).
template <int CIN, int COUT>
__device__ __forceinline__ void wg_stage_cp(const WgradLaunch& a, const WgBlock& k, uint32_t buf, int pt) {
    using L = WgSmem<CIN, COUT>;
    constexpr int XP = CIN / 8, DP = COUT / 8;
    const size_t img = (size_t)k.b * a.H;
    int ystart = (k.y0 - 1) % a.H;
    if (ystart < 0) ystart += a.H;
    for (int u = pt; u < XP * WG_SLOTS; u += 96) {
        const int sl = u / XP, j = u % XP;
        int xx = k.x0 - 1 + sl;
        if (xx < 0) xx += a.W;
        if (xx >= a.W) xx -= a.W;
        const uint16_t* col = a.x + (size_t)xx * CIN + j * 8;
        int yy = ystart;
#pragma unroll
        for (int r = 0; r < L::XROWS; ++r) {
            cp_async16(buf + (uint32_t)(r * L::XROW + j * L::XPLANE + sl * 16), col + (img + yy) * (size_t)a.W * CIN);
            if (++yy == a.H) yy = 0;
        }
    }
    for (int u = pt; u < DP * WG_PX; u += 96) {
        const int sl = u / DP, j = u % DP;
        const uint16_t* col = a.dy + ((img + k.y0) * a.W + k.x0 + sl) * COUT + j * 8;
        for (int r = 0; r < k.rows; ++r)
            cp_async16(buf + (uint32_t)(L::XBYTES + r * L::DROW + j * WG_DPLANE + sl * 16), col + (size_t)r * a.W * COUT);
    }
}

// Warp-specialised pipeline over a ring of WG_NBUF buffers. Warps 1-3 are the
// producers (lane 0 of warp 1 issues the TMA copies; all three warps stage the
// edge blocks with cp.async); lane 0 of warp 0 issues the MMAs. full[b] takes one
// arrival from every producer thread for every block (after its cp.async copies
// landed; the TMA issuer's arrival carries the expected bytes) and says buffer b
// holds a block; empty[b] (the MMAs' commit) says the tensor cores are done with
// it. Every producer thread waits on empty and arrives on full for every block,
// so no thread is ever more than one phase away from a barrier it waits on (a
// parity wait needs that), and no producer waits for another, so a wait that
// runs out cannot strand the rest.
template <int CIN, int COUT>
__global__ void __launch_bounds__(THREADS) wgrad_kernel(const __grid_constant__ WgradLaunch a) {
    using L = WgSmem<CIN, COUT>;
    constexpr uint32_t IDESC = idesc_bf16_mn(128, COUT);
    constexpr uint32_t TCOLS = tmem_cols(4 * COUT);
    constexpr int MPAD = 9 * CIN + 1;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[WG_NBUF], empty[WG_NBUF];
    __shared__ uint32_t tmem_slot;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long total = (long long)a.batch * ((a.H + WG_ROWS - 1) / WG_ROWS) * (a.W / WG_PX);
    const long long k_begin = (long long)blockIdx.x * a.units_per_cta;
    const int nk = (int)max(0ll, min(total, k_begin + a.units_per_cta) - k_begin);
    const uint32_t s0 = smem_addr(smem);
    float* part = a.partials + (size_t)blockIdx.x * MPAD * COUT;

    {  // the all-ones operand of the bias MMAs (BF16 1.0)
        uint4* o = reinterpret_cast<uint4*>(smem + L::OFF_ONES);
        for (int i = tid; i < WG_ONES / 16; i += THREADS) o[i] = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
    }
    fence_async_smem();
    if (tid == 0) {
        for (int i = 0; i < WG_NBUF; ++i) {
            mbar_init(smem_addr(&full[i]), 96);
            mbar_init(smem_addr(&empty[i]), 1);
        }
    }
    if (warp == 0) tmem_alloc(smem_addr(&tmem_slot), TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    int ok = 1;
    if (warp > 0) {
        const int pt = tid - 32;
        for (int k = 0; k < nk; ++k) {
            const int bsel = k % WG_NBUF;
            const uint32_t buf = s0 + (uint32_t)(bsel * L::BUF);
            const uint32_t fb = smem_addr(&full[bsel]);
            const WgBlock blk = wg_block(a, k_begin + k);
            if (k >= WG_NBUF && !mbar_wait(smem_addr(&empty[bsel]), ((k / WG_NBUF) - 1) & 1)) {
                ok = 0;
                break;
            }
            if (blk.edge) {
                wg_stage_cp<CIN, COUT>(a, blk, buf, pt);
                cp_async_commit();
                cp_async_wait_all_groups();
                fence_async_smem();
                mbar_arrive(fb);
            } else if (pt != 0) {
                mbar_arrive(fb);
            } else {
                mbar_arrive_tx(fb, (uint32_t)(L::XROWS * L::XROW + blk.rows * L::DROW));
                int yy = (blk.y0 - 1) % a.H;
                if (yy < 0) yy += a.H;
                for (int r = 0; r < L::XROWS; ++r) {
                    tma_load_5d(buf + (uint32_t)(r * L::XROW), &a.tmx, blk.x0 - 1, 0, yy, blk.b, fb);
                    if (++yy == a.H) yy = 0;
                }
                for (int r = 0; r < blk.rows; ++r)
                    tma_load_5d(buf + (uint32_t)(L::XBYTES + r * L::DROW), &a.tmdy, blk.x0, 0, blk.y0 + r, blk.b, fb);
            }
        }
    } else if (lane == 0) {
        bool first = true;
        const uint64_t ones = umma_desc(s0 + (uint32_t)L::OFF_ONES, 128, 256);
        for (int k = 0; k < nk; ++k) {
            const int bsel = k % WG_NBUF;
            const uint32_t buf = s0 + (uint32_t)(bsel * L::BUF);
            if (!mbar_wait(smem_addr(&full[bsel]), (k / WG_NBUF) & 1)) {
                ok = 0;
                break;
            }
            tc_fence_after();
            const int rows = wg_block(a, k_begin + k).rows;
            // descriptors advance by (bytes >> 4) in their start-address field
            const uint64_t a0 = umma_desc(buf, 128, L::XPLANE);
            const uint64_t b0 = umma_desc(buf + (uint32_t)L::XBYTES, 128, WG_DPLANE);
            for (int i = 0; i < rows; ++i) {
#pragma unroll
                for (int kk = 0; kk < WG_PX / 16; ++kk) {
                    const uint64_t bd = b0 + (uint64_t)((i * L::DROW + 16 * kk * 16) >> 4);
                    const uint32_t acc = (first && kk == 0) ? 0u : 1u;
#pragma unroll
                    for (int dx = 0; dx < 3; ++dx) {
                        const uint64_t ad = a0 + (uint64_t)((i * L::XROW + (16 * kk + dx) * 16) >> 4);
                        mma_bf16(tmem + (uint32_t)(dx * COUT), ad, bd, IDESC, acc);
                    }
                    mma_bf16(tmem + (uint32_t)(3 * COUT), ones, bd, IDESC, acc);
                }
                first = false;
            }
            mma_commit(smem_addr(&empty[bsel]));
        }
    }
    cp_async_wait_all_groups();
    __syncwarp();
    ok = __syncthreads_and(ok);
    if (ok && nk > 0) {
        const int last = nk - 1;
        ok = __syncthreads_and(mbar_wait(smem_addr(&empty[last % WG_NBUF]), (last / WG_NBUF) & 1));
        if (ok) {
            tc_fence_after();
            // TMEM lane m = (row offset dyi, channel ci); column dx * COUT + co;
            // columns 3 * COUT + co: the bias gradient (every lane the same)
            if (warp * 32 < 3 * CIN) {
                const int m = warp * 32 + lane, dyi = m / CIN, ci = m % CIN;
#pragma unroll
                for (int dx = 0; dx < 3; ++dx) {
                    float v[COUT];
                    tmem_load<COUT>(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(dx * COUT), v);
                    if (dyi < 3) {
                        float* row = part + (size_t)((dyi * 3 + dx) * CIN + ci) * COUT;
#pragma unroll
                        for (int c = 0; c < COUT; ++c) row[c] = v[c];
                    }
                }
            }
            if (warp == 0) {
                float v[COUT];
                tmem_load<COUT>(tmem + (uint32_t)(3 * COUT), v);
                if (lane == 0) {
#pragma unroll
                    for (int c = 0; c < COUT; ++c) part[(size_t)9 * CIN * COUT + c] = v[c];
                }
            }
        }
    } else if (ok) {
        for (int i = tid; i < MPAD * COUT; i += THREADS) part[i] = 0.0f;
    }
    if (!ok && tid == 0) atomicExch(a.err, 1);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TCOLS);
    }
}

__global__ void weight_image_kernel(const float* __restrict__ w, int cin, int cout, int transpose,
                                    uint16_t* __restrict__ img) {
    const int kcin = transpose ? cout : cin, kcout = transpose ? cin : cout;
    const int total = 9 * kcin * kcout;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    // img[((tap*(kcin/8) + j)*kcout + n)*8 + e] holds kernel weight (tap, out n, in 8j+e)
    const int e = i & 7;
    const int r = i >> 3;
    const int n = r % kcout;
    const int r2 = r / kcout;
    const int j = r2 % (kcin / 8);
    const int tap = r2 / (kcin / 8);
    const int kc = 8 * j + e;
    const float v = transpose ? w[((size_t)(8 - tap) * cout + kc) * cin + n] : w[((size_t)tap * cout + n) * cin + kc];
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    img[i] = *reinterpret_cast<const uint16_t*>(&h);
}

__global__ void reduce_wgrad_kernel(const float* __restrict__ partials, int grid, int cin, int cout, int mpad,
                                    float* __restrict__ dw, float* __restrict__ db) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nw = 9 * cin * cout;
    if (i >= nw + cout) return;
    int m, co;
    if (i < nw) {  // dw[tap][co][ci]
        const int ci = i % cin, r = i / cin;
        co = r % cout;
        const int tap = r / cout;
        m = tap * cin + ci;
    } else {
        co = i - nw;
        m = 9 * cin;
    }
    float s = 0.0f;
    for (int g = 0; g < grid; ++g) s += partials[((size_t)g * mpad + m) * cout + co];
    if (i < nw)
        dw[i] = s;
    else
        db[co] = s;
}

template <int CIN, int COUT, int EPI>
int launch_conv_t(const ConvLaunch& a, cudaStream_t s) {
    using L = ConvSmem<CIN, COUT>;
    const int attr = picgb::opt_in_dynamic_smem((const void*)conv3x3_kernel<CIN, COUT, EPI>, L::BYTES);
    if (attr != PIC_OK) return attr;
    const dim3 grid(a.W / 128, (a.H + a.rows_per_cta - 1) / a.rows_per_cta, a.batch);
    conv3x3_kernel<CIN, COUT, EPI><<<grid, CONV_THREADS, L::BYTES, s>>>(a);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PIC_OK : picgb::cuda_fail(e, "conv3x3_kernel launch");
}

typedef CUresult (*TensorMapEncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                           const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                           CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int tensor_map_encoder(TensorMapEncodeTiledFn* out) {
    static TensorMapEncodeTiledFn fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        const cudaError_t e =
            cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void**)&fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
            fn = nullptr;
            return picgb::fail(PIC_ERR_UNSUPPORTED, "the driver does not provide cuTensorMapEncodeTiled");
        }
    }
    *out = fn;
    return PIC_OK;
}

// 5-D view of an NHWC BF16 tensor with C channels: (8 channels, pixel, 8-channel
// plane, row, image), pixel stride C * 2 bytes and plane stride 16 bytes, and a
// box of 8 channels x `px` pixels x all planes of one row, which lands in shared
// memory as planes of `px` 16-byte pixel slots.
int encode_planes_map(CUtensorMap* m, const uint16_t* base, int C, int batch, int H, int W, int px) {
    TensorMapEncodeTiledFn enc;
    PIC_TRY(tensor_map_encoder(&enc));
    const cuuint64_t dims[5] = {8, (cuuint64_t)W, (cuuint64_t)(C / 8), (cuuint64_t)H, (cuuint64_t)batch};
    const cuuint64_t strides[4] = {(cuuint64_t)C * 2, 16, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    const cuuint32_t box[5] = {8, (cuuint32_t)px, (cuuint32_t)(C / 8), 1, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<uint16_t*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return picgb::fail(PIC_ERR_CUDA, "cuTensorMapEncodeTiled failed for the weight gradient");
    return PIC_OK;
}

template <int CIN, int COUT>
int launch_wgrad_t(const WgradLaunch& a0, int grid, cudaStream_t s) {
    using L = WgSmem<CIN, COUT>;
    const int attr = picgb::opt_in_dynamic_smem((const void*)wgrad_kernel<CIN, COUT>, L::BYTES);
    if (attr != PIC_OK) return attr;
    WgradLaunch a = a0;
    PIC_TRY(encode_planes_map(&a.tmx, a.x, CIN, a.batch, a.H, a.W, L::XBOX));
    PIC_TRY(encode_planes_map(&a.tmdy, a.dy, COUT, a.batch, a.H, a.W, WG_PX));
    wgrad_kernel<CIN, COUT><<<grid, THREADS, L::BYTES, s>>>(a);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PIC_OK : picgb::cuda_fail(e, "wgrad_kernel launch");
}

template <int CIN, int COUT>
int launch_conv_epi(const ConvLaunch& a, int epi, cudaStream_t s) {
    switch (epi) {
        case EPI_BIAS_RELU:
            return launch_conv_t<CIN, COUT, EPI_BIAS_RELU>(a, s);
        case EPI_BIAS_OUT:
            return launch_conv_t<CIN, COUT, EPI_BIAS_OUT>(a, s);
        case EPI_MASK:
            return launch_conv_t<CIN, COUT, EPI_MASK>(a, s);
    }
    return picgb::fail(PIC_ERR_ARG, "unknown convolution epilogue");
}

}  // namespace

int build_weight_image(const float* w_math, int cin, int cout, int transpose, uint16_t* img, cudaStream_t s) {
    const int total = 9 * cin * cout;
    weight_image_kernel<<<(total + 255) / 256, 256, 0, s>>>(w_math, cin, cout, transpose, img);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PIC_OK : picgb::cuda_fail(e, "weight_image_kernel launch");
}

int launch_conv(const ConvLaunch& a, int kcin, int kcout, int epi, cudaStream_t s) {
    if (a.W % 128 != 0 || a.W <= 0 || a.H <= 0 || a.batch <= 0 || a.rows_per_cta <= 0)
        return picgb::fail(PIC_ERR_ARG, "convolution needs W a multiple of 128 and H, batch, rows > 0");
    if (kcin == 16 && kcout == 16) return launch_conv_epi<16, 16>(a, epi, s);
    if (kcin == 16 && kcout == 32) return launch_conv_epi<16, 32>(a, epi, s);
    if (kcin == 32 && kcout == 16) return launch_conv_epi<32, 16>(a, epi, s);
    if (kcin == 32 && kcout == 32) return launch_conv_epi<32, 32>(a, epi, s);
    return picgb::fail(PIC_ERR_ARG, "convolution channels must be 16 or 32");
}

int wgrad_grid(long long units) {
    const long long g = units < 2 * 152 ? units : 2 * 152;
    return (int)(g < 1 ? 1 : g);
}

int launch_wgrad(const WgradLaunch& a, int cin, int cout, int grid, cudaStream_t s) {
    if (a.W % WG_PX != 0 || a.W <= 0 || a.H <= 0 || a.batch <= 0 || grid <= 0)
        return picgb::fail(PIC_ERR_ARG, "weight gradient needs W a multiple of 32");
    if (cin == 16 && cout == 16) return launch_wgrad_t<16, 16>(a, grid, s);
    if (cin == 16 && cout == 32) return launch_wgrad_t<16, 32>(a, grid, s);
    if (cin == 32 && cout == 16) return launch_wgrad_t<32, 16>(a, grid, s);
    if (cin == 32 && cout == 32) return launch_wgrad_t<32, 32>(a, grid, s);
    return picgb::fail(PIC_ERR_ARG, "convolution channels must be 16 or 32");
}

int reduce_wgrad(const float* partials, int grid, int cin, int cout, float* dw, float* db, cudaStream_t s) {
    const int total = 9 * cin * cout + cout;
    reduce_wgrad_kernel<<<(total + 255) / 256, 256, 0, s>>>(partials, grid, cin, cout, wgrad_mpad(cin), dw, db);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PIC_OK : picgb::cuda_fail(e, "reduce_wgrad_kernel launch");
}

}  // namespace picnn
