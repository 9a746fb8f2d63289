// 3x3 periodic convolutions as implicit GEMMs on the 5th-generation tensor cores.
//
// Forward / input-gradient kernel (conv3x3_kernel): one CTA of 4 warps owns a
// 128-pixel segment of a run of image rows. The GEMM per output row is
//     D[128 px][cout] = sum over 9 taps of A_tap[128 px][cin] * B_tap[cin][cout]
// with D in tensor memory (FP32), issued as tcgen05.mma kind::f16 (BF16 x BF16,
// M = 128, N = cout, K = 16) by one thread. The input rows are staged in shared
// memory as "planes" of 8 channels: pixel slot s of plane j holds the 16 bytes of
// channels 8j..8j+7 of pixel x0-1+s. In the K-major no-swizzle operand layout
// (8-row core matrices of 16-byte rows, stride between row groups SBO = 128 B,
// between the two K halves LBO = one plane) row r of A sits at r*16 bytes, so
// the operand of tap dx is the same staged row with its start moved by
// (dx+1)*16 bytes: im2col costs nothing. Rows y-1, y, y+1 live in a ring of 4
// slots; while the MMAs of row y run, the CTA drains row y-1 from the other
// TMEM buffer (bias + ReLU, or the ReLU mask of the backward pass) and stages
// row y+2 with cp.async.
//
// Weight-gradient kernel (wgrad_kernel): D[(tap,ci)][co] = sum over pixels of
// x[p+tap][ci] * dy[p][co], K = pixels. Per 64-pixel half row the CTA writes
// the K-major operands explicitly (A: 9*cin rows plus one row of ones whose
// product is the bias gradient; B: dy transposed) into one of two buffers and
// issues 3 x 4 (cin 32) MMAs while it fills the other. Each CTA accumulates its
// share of the pixels in TMEM and writes one partial sum; reduce_wgrad adds the
// partials in a fixed order, so gradients are identical run to run.
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
template <int CIN>
__device__ __forceinline__ void stage_row(const ConvLaunch& a, int b, int yraw, int x0, uint32_t slot, int tid) {
    constexpr int PLANES = CIN / 8;
    const int yy = ((yraw % a.H) + a.H) % a.H;
    const uint16_t* row = a.x + ((size_t)b * a.H + yy) * (size_t)a.W * CIN;
    for (int t = tid; t < SLOTS * PLANES; t += THREADS) {
        const int s = t / PLANES, j = t - s * PLANES;
        int xx = x0 - 1 + s;
        if (xx < 0) xx += a.W;
        if (xx >= a.W) xx -= a.W;
        cp_async16(slot + (uint32_t)(j * PLANE + s * 16), row + (size_t)xx * CIN + j * 8);
    }
}

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
    static constexpr int BYTES = OFF_RING + 4 * SLOT;
};

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(THREADS) conv3x3_kernel(ConvLaunch a) {
    using L = ConvSmem<CIN, COUT>;
    constexpr int KSTEPS = CIN / 16;
    constexpr uint32_t IDESC = idesc_bf16(128, COUT);
    constexpr uint32_t TCOLS = tmem_cols(2 * COUT);
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int x0 = blockIdx.x * 128;
    const int b = blockIdx.z;
    const int y_begin = blockIdx.y * a.rows_per_cta;
    const int y_end = min(a.H, y_begin + a.rows_per_cta);
    if (y_begin >= y_end) return;
    const uint32_t s_w = smem_addr(smem);
    const uint32_t s_ring = s_w + L::OFF_RING;
    float* sbias = reinterpret_cast<float*>(smem + L::OFF_BIAS);

    for (int i = tid; i < L::WBYTES / 16; i += THREADS)
        cp_async16(s_w + i * 16, reinterpret_cast<const uint8_t*>(a.wimg) + (size_t)i * 16);
    if (EPI != EPI_MASK && tid < COUT) sbias[tid] = a.bias[tid];
    for (int r = -1; r <= 1; ++r) stage_row<CIN>(a, b, y_begin + r, x0, s_ring + ((y_begin + r + 4) & 3) * L::SLOT, tid);
    cp_async_wait_all();
    fence_async_smem();
    if (tid == 0) {
        mbar_init(smem_addr(&mbar[0]), 1);
        mbar_init(smem_addr(&mbar[1]), 1);
    }
    if (warp == 0) tmem_alloc(smem_addr(&tmem_slot), TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);

    bool ok = true;
    int i = 0;
    for (int y = y_begin; y < y_end; ++y, ++i) {
        if (tid == 0) {
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)((i & 1) * COUT);
            int k = 0;
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                const int dy = t / 3 - 1, dx = t % 3 - 1;
                const uint32_t arow = s_ring + ((y + dy + 4) & 3) * L::SLOT + (dx + 1) * 16;
#pragma unroll
                for (int s = 0; s < KSTEPS; ++s, ++k) {
                    const uint64_t ad = umma_desc(arow + 2 * s * PLANE, PLANE, 128);
                    const uint64_t bd = umma_desc(s_w + (t * L::PLANES + 2 * s) * COUT * 16, COUT * 16, 128);
                    mma_bf16(d, ad, bd, IDESC, k > 0 ? 1u : 0u);
                }
            }
            mma_commit(smem_addr(&mbar[i & 1]));
        }
        if (i > 0) {
            ok = __syncthreads_and(mbar_wait(smem_addr(&mbar[(i - 1) & 1]), ((i - 1) >> 1) & 1));
            if (!ok) break;
            tc_fence_after();
            conv_epilogue<COUT, EPI>(a, b, y - 1, x0, lane_base + ((i - 1) & 1) * COUT, sbias, warp, lane);
            tc_fence_before();
        }
        if (y + 1 < y_end) stage_row<CIN>(a, b, y + 2, x0, s_ring + ((y + 2 + 4) & 3) * L::SLOT, tid);
        cp_async_wait_all();
        fence_async_smem();
        __syncthreads();
    }
    if (ok) {
        const int last = i - 1;
        ok = __syncthreads_and(mbar_wait(smem_addr(&mbar[last & 1]), (last >> 1) & 1));
        if (ok) {
            tc_fence_after();
            conv_epilogue<COUT, EPI>(a, b, y_end - 1, x0, lane_base + (last & 1) * COUT, sbias, warp, lane);
        }
    }
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
template <int CIN, int COUT>
struct WgSmem {
    static constexpr int MPAD = ((9 * CIN + 1 + 127) / 128) * 128;
    static constexpr int MT = MPAD / 128;
    static constexpr int LBO_A = MPAD * 16;
    static constexpr int ABYTES = 8 * LBO_A;
    static constexpr int BBYTES = 8 * COUT * 16;
    static constexpr int OFF_B = 2 * ABYTES;
    static constexpr int OFF_RAWX = OFF_B + 2 * BBYTES;
    static constexpr int RAWX = 3 * 66 * CIN * 2;
    static constexpr int OFF_RAWD = OFF_RAWX + RAWX;
    static constexpr int BYTES = OFF_RAWD + 64 * COUT * 2;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(THREADS) wgrad_kernel(WgradLaunch a) {
    using L = WgSmem<CIN, COUT>;
    constexpr uint32_t IDESC = idesc_bf16(128, COUT);
    constexpr uint32_t TCOLS = tmem_cols(L::MT * COUT);
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int halves = a.W / 64;
    const long long total = (long long)a.batch * a.H * halves;
    const long long u_begin = (long long)blockIdx.x * a.units_per_cta;
    const long long u_end = min(total, u_begin + a.units_per_cta);
    const uint32_t s_a = smem_addr(smem);
    const uint32_t s_b = s_a + L::OFF_B;
    const uint16_t* rawx = reinterpret_cast<const uint16_t*>(smem + L::OFF_RAWX);
    const uint16_t* rawd = reinterpret_cast<const uint16_t*>(smem + L::OFF_RAWD);
    float* part = a.partials + (size_t)blockIdx.x * L::MPAD * COUT;

    {  // zero both A buffers once: rows past the bias row stay zero
        uint4* z = reinterpret_cast<uint4*>(smem);
        for (int i = tid; i < 2 * L::ABYTES / 16; i += THREADS) z[i] = make_uint4(0, 0, 0, 0);
    }
    if (tid == 0) {
        mbar_init(smem_addr(&mbar[0]), 1);
        mbar_init(smem_addr(&mbar[1]), 1);
    }
    if (warp == 0) tmem_alloc(smem_addr(&tmem_slot), TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    bool ok = true;
    int k = 0;
    for (long long u = u_begin; u < u_end; ++u, ++k) {
        const int half = (int)(u % halves);
        const long long rest = u / halves;
        const int y = (int)(rest % a.H);
        const int b = (int)(rest / a.H);
        const int x0 = half * 64;
        // raw rows: x at y-1..y+1, pixels x0-1..x0+64; dy at y, pixels x0..x0+63
        for (int t = tid; t < 3 * 66 * (CIN / 8); t += THREADS) {
            const int j = t % (CIN / 8), rs = t / (CIN / 8), s = rs % 66, r = rs / 66;
            const int yy = ((y + r - 1) % a.H + a.H) % a.H;
            int xx = x0 - 1 + s;
            if (xx < 0) xx += a.W;
            if (xx >= a.W) xx -= a.W;
            cp_async16(s_a + L::OFF_RAWX + (uint32_t)(((r * 66 + s) * CIN + j * 8) * 2),
                       a.x + (((size_t)b * a.H + yy) * a.W + xx) * CIN + j * 8);
        }
        for (int t = tid; t < 64 * (COUT / 8); t += THREADS) {
            const int j = t % (COUT / 8), s = t / (COUT / 8);
            cp_async16(s_a + L::OFF_RAWD + (uint32_t)((s * COUT + j * 8) * 2),
                       a.dy + (((size_t)b * a.H + y) * a.W + x0 + s) * COUT + j * 8);
        }
        cp_async_wait_all();
        const int buf = k & 1;
        bool w = true;
        if (k >= 2) w = mbar_wait(smem_addr(&mbar[buf]), ((k - 2) >> 1) & 1);
        ok = __syncthreads_and(w);
        if (!ok) break;
        tc_fence_after();
        uint8_t* abuf = smem + buf * L::ABYTES;
        for (int t = tid; t < 9 * CIN * 8 + 8; t += THREADS) {
            uint32_t p[4];
            int m, kc;
            if (t < 9 * CIN * 8) {
                const int ci = t % CIN, rest2 = t / CIN;
                kc = rest2 % 8;
                const int tap = rest2 / 8;
                m = tap * CIN + ci;
                const int r = tap / 3, dx = tap % 3;
                const uint16_t* src = rawx + (r * 66 + kc * 8 + dx) * CIN + ci;
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    p[e] = (uint32_t)src[(2 * e) * CIN] | ((uint32_t)src[(2 * e + 1) * CIN] << 16);
            } else {
                kc = t - 9 * CIN * 8;
                m = 9 * CIN;
#pragma unroll
                for (int e = 0; e < 4; ++e) p[e] = 0x3F803F80u;  // BF16 1.0, 1.0
            }
            *reinterpret_cast<uint4*>(abuf + kc * L::LBO_A + m * 16) = make_uint4(p[0], p[1], p[2], p[3]);
        }
        uint8_t* bbuf = smem + L::OFF_B + buf * L::BBYTES;
        for (int t = tid; t < 8 * COUT; t += THREADS) {
            const int co = t % COUT, kc = t / COUT;
            const uint16_t* src = rawd + (kc * 8) * COUT + co;
            uint32_t p[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) p[e] = (uint32_t)src[(2 * e) * COUT] | ((uint32_t)src[(2 * e + 1) * COUT] << 16);
            *reinterpret_cast<uint4*>(bbuf + kc * COUT * 16 + co * 16) = make_uint4(p[0], p[1], p[2], p[3]);
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = s_a + buf * L::ABYTES, b0 = s_b + buf * L::BBYTES;
#pragma unroll
            for (int mt = 0; mt < L::MT; ++mt)
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    const uint64_t ad = umma_desc(a0 + mt * 128 * 16 + s * 2 * L::LBO_A, L::LBO_A, 128);
                    const uint64_t bd = umma_desc(b0 + s * 2 * COUT * 16, COUT * 16, 128);
                    mma_bf16(tmem + mt * COUT, ad, bd, IDESC, (k > 0 || s > 0) ? 1u : 0u);
                }
            mma_commit(smem_addr(&mbar[buf]));
        }
    }
    if (ok && k > 0) {
        const int last = k - 1;
        ok = __syncthreads_and(mbar_wait(smem_addr(&mbar[last & 1]), (last >> 1) & 1));
        if (ok) {
            tc_fence_after();
            for (int mt = 0; mt < L::MT; ++mt) {
                float v[COUT];
                tmem_load<COUT>(tmem + ((uint32_t)(warp * 32) << 16) + mt * COUT, v);
                float* row = part + (size_t)(mt * 128 + warp * 32 + lane) * COUT;
#pragma unroll
                for (int c = 0; c < COUT; ++c) row[c] = v[c];
            }
        }
    } else if (ok) {
        for (int i = tid; i < L::MPAD * COUT; i += THREADS) part[i] = 0.0f;
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
    conv3x3_kernel<CIN, COUT, EPI><<<grid, THREADS, L::BYTES, s>>>(a);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PIC_OK : picgb::cuda_fail(e, "conv3x3_kernel launch");
}

template <int CIN, int COUT>
int launch_wgrad_t(const WgradLaunch& a, int grid, cudaStream_t s) {
    using L = WgSmem<CIN, COUT>;
    const int attr = picgb::opt_in_dynamic_smem((const void*)wgrad_kernel<CIN, COUT>, L::BYTES);
    if (attr != PIC_OK) return attr;
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
    if (a.W % 64 != 0 || a.W <= 0 || a.H <= 0 || a.batch <= 0 || grid <= 0)
        return picgb::fail(PIC_ERR_ARG, "weight gradient needs W a multiple of 64");
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
