// Context lifecycle, errors, particle upload/download and the device-wide scan.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "pic_internal.cuh"

namespace picgb {

static thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return PIC_ERR_CUDA;
}

int opt_in_dynamic_smem(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> done;
    int dev = 0;
    PIC_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    size_t& have = done[std::make_pair(kernel, dev)];
    if (bytes <= have) return PIC_OK;
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return cuda_fail(e, "cudaFuncSetAttribute(MaxDynamicSharedMemorySize)");
    }
    have = bytes;
    return PIC_OK;
}

int check_launch(pic_ctx* ctx, const char* what) {
    ctx->launches++;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    return PIC_OK;
}

void* dalloc(size_t bytes, int* rc) {
    void* p = nullptr;
    if (bytes == 0) bytes = 16;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        *rc = fail(PIC_ERR_NOMEM, std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
        (void)cudaGetLastError();
        return nullptr;
    }
    *rc = PIC_OK;
    return p;
}

void dfree(void* p) {
    if (p) cudaFree(p);
}

void prof_begin(pic_ctx* ctx, const char* name) {
    if (!ctx->prof_enabled) return;
    if (!ctx->prof) ctx->prof = new std::vector<pic_ctx::ProfRec>();
    pic_ctx::ProfRec r;
    r.name = name;
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, ctx->stream);
    ctx->prof->push_back(r);
}

void prof_end(pic_ctx* ctx) {
    if (!ctx->prof_enabled || !ctx->prof || ctx->prof->empty()) return;
    cudaEventRecord(ctx->prof->back().b, ctx->stream);
}

static void prof_clear(pic_ctx* ctx, const char* name) {
    if (!ctx->prof) return;
    std::vector<pic_ctx::ProfRec> keep;
    for (auto& r : *ctx->prof) {
        if (!name || std::strcmp(r.name, name) == 0) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        } else {
            keep.push_back(r);
        }
    }
    *ctx->prof = keep;
}

int check_device_status(pic_ctx* ctx) {
    DevStats st;
    PIC_CUDA_TRY(cudaMemcpyAsync(&st, ctx->dstats, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
    PIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (st.err == DEV_OK) return PIC_OK;
    // clear so that the context stays usable after the caller handles the error
    PIC_CUDA_TRY(cudaMemsetAsync(&ctx->dstats->err, 0, sizeof(int), ctx->stream));
    switch (st.err) {
        case DEV_BAD_POSITION:
            return fail(PIC_ERR_DEVICE, "non-finite or out-of-range particle position (particle " +
                                            std::to_string(st.err_info) + ")");
        case DEV_BAD_CELL:
            return fail(PIC_ERR_DEVICE, "cell key out of range (particle " + std::to_string(st.err_info) + ")");
        case DEV_MOVE_TOO_LARGE:
            return fail(PIC_ERR_ARG, "trajectory longer than 256 cells in one step (particle " +
                                         std::to_string(st.err_info) + ")");
        case DEV_COURANT:
            return fail(PIC_ERR_COURANT, "Esirkepov current needs |v|*dt < cell size (particle " +
                                             std::to_string(st.err_info) + ")");
        default:
            return fail(PIC_ERR_DEVICE, "device error " + std::to_string(st.err));
    }
}

// ---------------------------------------------------------------------------
// exclusive scan (three phases: block sums, recursive scan of sums, add-back)
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ unsigned int block_exclusive_scan(unsigned int v, unsigned int* total) {
    __shared__ unsigned int warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        unsigned int s = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s;  // inclusive
    }
    __syncthreads();
    const unsigned int warp_prefix = warp > 0 ? warp_sums[warp - 1] : 0u;
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    const unsigned int r = warp_prefix + x - v;
    __syncthreads();
    return r;
}

__global__ void scan_block_sums(const unsigned int* __restrict__ data, size_t n, unsigned int* __restrict__ sums) {
    const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    unsigned int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) s += data[base + k];
    unsigned int total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_apply(unsigned int* __restrict__ data, size_t n, const unsigned int* __restrict__ offs) {
    const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    unsigned int v[SCAN_ITEMS];
    unsigned int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (base + k < n) ? data[base + k] : 0u;
        s += v[k];
    }
    unsigned int run = block_exclusive_scan(s, nullptr) + (offs ? offs[blockIdx.x] : 0u);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) data[base + k] = run;
        run += v[k];
    }
}

static size_t scan_partials_needed(size_t n) {
    size_t total = 0;
    while (n > (size_t)SCAN_TILE) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        total += n;
    }
    return total + 1;
}

static int scan_rec(pic_ctx* ctx, unsigned int* data, size_t n, unsigned int* scratch) {
    if (n == 0) return PIC_OK;
    if (n <= (size_t)SCAN_TILE) {
        scan_apply<<<1, SCAN_THREADS, 0, ctx->stream>>>(data, n, nullptr);
        return check_launch(ctx, "scan_apply");
    }
    const size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    scan_block_sums<<<(unsigned)nb, SCAN_THREADS, 0, ctx->stream>>>(data, n, scratch);
    PIC_TRY(check_launch(ctx, "scan_block_sums"));
    PIC_TRY(scan_rec(ctx, scratch, nb, scratch + nb));
    scan_apply<<<(unsigned)nb, SCAN_THREADS, 0, ctx->stream>>>(data, n, scratch);
    return check_launch(ctx, "scan_apply");
}

int exclusive_scan_u32(pic_ctx* ctx, unsigned int* data, size_t n) {
    const size_t need = scan_partials_needed(n);
    if (ctx->scan.capacity < need) {
        dfree(ctx->scan.partials);
        int rc;
        ctx->scan.partials = (unsigned int*)dalloc(need * sizeof(unsigned int), &rc);
        if (!ctx->scan.partials) {
            ctx->scan.capacity = 0;
            return rc;
        }
        ctx->scan.capacity = need;
    }
    return scan_rec(ctx, data, n, ctx->scan.partials);
}

// ---------------------------------------------------------------------------
// upload: FP64 host SoA -> device cell key + FP32 in-cell offsets
// ---------------------------------------------------------------------------
struct ConvertArgs {
    const double *x, *y, *vx, *vy, *q, *m;  // chunk (device staging or pinned host); vx/vy/m may be null
    size_t count, first;                    // chunk size and global index of its first particle
    double dx, dy;
    double inv_dx, inv_dy;                  // exact reciprocals when dx / dy are powers of two, else 0
    int Nx, Ny;
    uint32_t* cell;
    float *xr, *yr, *fvx, *fvy, *fq, *fm;
    DevStats* st;
};

__global__ void convert_particles(ConvertArgs a) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float aq = 0.0f, avx = 0.0f, avy = 0.0f;
    if (i < a.count) {
        int ix = 0, iy = 0;
        float rx = 0.0f, ry = 0.0f;
        const bool okx = cell_coord(a.x[i], a.dx, a.inv_dx, a.Nx, &ix, &rx);
        const bool oky = cell_coord(a.y[i], a.dy, a.inv_dy, a.Ny, &iy, &ry);
        if (!(okx && oky)) set_dev_error(a.st, DEV_BAD_POSITION, (unsigned int)(a.first + i));
        const size_t o = a.first + i;
        a.cell[o] = (uint32_t)iy * (uint32_t)a.Nx + (uint32_t)ix;
        a.xr[o] = rx;
        a.yr[o] = ry;
        const float fvx = a.vx ? __double2float_rn(a.vx[i]) : 0.0f;
        const float fvy = a.vy ? __double2float_rn(a.vy[i]) : 0.0f;
        const float fq = __double2float_rn(a.q[i]);
        a.fvx[o] = fvx;
        a.fvy[o] = fvy;
        a.fq[o] = fq;
        if (a.fm) a.fm[o] = a.m ? __double2float_rn(a.m[i]) : 1.0f;
        if (o == 0) a.st->q_raw0 = fq;
        aq = fabsf(fq);
        avx = fabsf(fvx);
        avy = fabsf(fvy);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        aq = fmaxf(aq, __shfl_xor_sync(0xffffffffu, aq, o));
        avx = fmaxf(avx, __shfl_xor_sync(0xffffffffu, avx, o));
        avy = fmaxf(avy, __shfl_xor_sync(0xffffffffu, avy, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&a.st->maxq_bits, __float_as_uint(aq));
        atomicMax(&a.st->maxvx_bits, __float_as_uint(avx));
        atomicMax(&a.st->maxvy_bits, __float_as_uint(avy));
    }
}

// 1/d when d is a power of two (then x * (1/d) == x / d exactly), else 0.
double exact_reciprocal(double d) {
    int e = 0;
    const double mant = std::frexp(d, &e);
    return mant == 0.5 ? std::ldexp(1.0, 1 - e) : 0.0;
}

static int ensure_copy_stream(pic_ctx* c) {
    if (c->copy_stream) return PIC_OK;
    PIC_CUDA_TRY(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
        PIC_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_copied[k], cudaEventDisableTiming));
        PIC_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_converted[k], cudaEventDisableTiming));
    }
    return PIC_OK;
}

// One pass over the stored charges and keys after the conversion, four
// particles per thread (16-byte loads and stores; the arrays are padded past the
// last particle and 16-byte aligned):
//  * q <- q / max|q| (FP32 IEEE division): a uniform |q| becomes exactly +-1;
//  * a flag when a normalised charge differs (bitwise) from the first
//    particle's (normalised from its charge as converted, which every thread
//    reads before any store);
//  * the count of adjacent pairs out of cell order (0: the upload is already
//    sorted): per thread, the key before its four from the previous lane (lane
//    0 loads it), summed per block, one global atomic per block.
__global__ void finish_upload(float* __restrict__ q, const uint32_t* __restrict__ cell, size_t n, DevStats* st) {
    __shared__ unsigned s_breaks;
    if (threadIdx.x == 0) s_breaks = 0;
    __syncthreads();
    const float mq = load_maxq(st);
    const float q0 = mq > 0.0f ? __fdiv_rn(st->q_raw0, mq) : 0.0f;
    const size_t i0 = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    const bool act = i0 < n;
    uint4 kv = make_uint4(0u, 0u, 0u, 0u);
    float4 qv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (act) {
        kv = *reinterpret_cast<const uint4*>(cell + i0);
        qv = *reinterpret_cast<const float4*>(q + i0);
    }
    uint32_t before = __shfl_up_sync(0xffffffffu, kv.w, 1);
    bool diff = false;
    unsigned brk = 0;
    if (act) {
        if ((threadIdx.x & 31) == 0 && i0 > 0) before = cell[i0 - 1];
        const int cnt = (n - i0) < 4 ? (int)(n - i0) : 4;
        float w[4] = {qv.x, qv.y, qv.z, qv.w};
        const uint32_t k[4] = {kv.x, kv.y, kv.z, kv.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j < cnt) {
                w[j] = mq > 0.0f ? __fdiv_rn(w[j], mq) : 0.0f;
                diff |= __float_as_uint(w[j]) != __float_as_uint(q0);
                brk += (j == 0 ? (i0 > 0 && k[0] < before) : (k[j] < k[j - 1])) ? 1u : 0u;
            }
        }
        *reinterpret_cast<float4*>(q + i0) = make_float4(w[0], w[1], w[2], w[3]);
        if (i0 == 0) st->q_first = q0;
    }
    if (__any_sync(0xffffffffu, diff) && (threadIdx.x & 31) == 0) atomicOr(&st->q_mixed, 1u);
    brk = __reduce_add_sync(0xffffffffu, brk);
    if ((threadIdx.x & 31) == 0 && brk) atomicAdd(&s_breaks, brk);
    __syncthreads();
    if (threadIdx.x == 0 && s_breaks) atomicAdd(&st->order_breaks, s_breaks);
}

}  // namespace picgb

using namespace picgb;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* pic_gpu_last_error(void) { return g_last_error.c_str(); }

int pic_gpu_create(const pic_domain* dom, size_t capacity, int device, pic_ctx** out) {
    if (!dom || !out) return fail(PIC_ERR_ARG, "pic_gpu_create: NULL argument");
    *out = nullptr;
    if (dom->Nx < 1 || dom->Ny < 1 || !(dom->Lx > 0.0) || !(dom->Ly > 0.0))
        return fail(PIC_ERR_ARG, "pic_gpu_create: grid must be Nx,Ny >= 1 and Lx,Ly > 0");
    if ((size_t)dom->Nx * (size_t)dom->Ny > (size_t)1 << 30)
        return fail(PIC_ERR_ARG, "pic_gpu_create: more than 2^30 cells");
    // particle indices are 32-bit on the device; int64 cell sums hold 2^39 particles of 2^24 units
    if (capacity > ((size_t)1 << 32) - 4096) return fail(PIC_ERR_ARG, "pic_gpu_create: capacity above 2^32-4096");
    int ndev = 0;
    PIC_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(PIC_ERR_ARG, "pic_gpu_create: no such device");
    PIC_CUDA_TRY(cudaSetDevice(device));

    pic_ctx* c = new pic_ctx();
    c->device = device;
    c->Lx = dom->Lx;
    c->Ly = dom->Ly;
    c->Nx = dom->Nx;
    c->Ny = dom->Ny;
    c->dx = dom->Lx / dom->Nx;  // Domain::updateDerived, domain.hpp:17-20
    c->dy = dom->Ly / dom->Ny;
    c->G = (size_t)dom->Nx * (size_t)dom->Ny;
    c->cap = capacity;
    int rc = PIC_OK;
    auto A = [&](size_t bytes) -> void* {
        if (rc != PIC_OK) return nullptr;
        return dalloc(bytes, &rc);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaStreamCreate");
    }
    const size_t cp = (capacity ? capacity : 1) + PARTICLE_PAD;
    c->cell = (uint32_t*)A(cp * 4);
    c->xr = (float*)A(cp * 4);
    c->yr = (float*)A(cp * 4);
    c->vx = (float*)A(cp * 4);
    c->vy = (float*)A(cp * 4);
    c->q = (float*)A(cp * 4);
    c->acc = (long long*)A(c->G * 8);
    c->rho = (double*)A(c->G * 8);
    c->unitbuf = (double*)A(64);
    c->dstats = (DevStats*)A(sizeof(DevStats));
    if (rc != PIC_OK) {
        pic_gpu_destroy(c);
        return rc;
    }
    cudaMemsetAsync(c->dstats, 0, sizeof(DevStats), c->stream);
    cudaMemsetAsync(c->rho, 0, c->G * 8, c->stream);
    cudaMemsetAsync(c->acc, 0, c->G * 8, c->stream);
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        pic_gpu_destroy(c);
        return cuda_fail(e, "pic_gpu_create init");
    }
    *out = c;
    return PIC_OK;
}

int pic_gpu_destroy(pic_ctx* c) {
    if (!c) return PIC_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    void* ptrs[] = {c->cell, c->xr, c->yr, c->vx, c->vy, c->q, c->m, c->cell_alt, c->idx_a, c->idx_b,
                    c->alt[0], c->alt[1], c->alt[2], c->alt[3], c->alt[4], c->alt[5], c->counts, c->offsets,
                    c->cellcount, c->scan.partials, c->stage, c->acc, c->rho, c->unitbuf, c->dstats};
    for (void* p : ptrs) dfree(p);
    release_fields(c);
    release_rbgs(c);
    release_current(c);
    release_ws(c);
    prof_clear(c, nullptr);
    delete c->prof;
    for (int k = 0; k < 2; ++k) {
        if (c->ev_copied[k]) cudaEventDestroy(c->ev_copied[k]);
        if (c->ev_converted[k]) cudaEventDestroy(c->ev_converted[k]);
    }
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return PIC_OK;
}

int pic_gpu_synchronize(pic_ctx* c) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return check_device_status(c);
}

int pic_gpu_launch_count(pic_ctx* c, long long* out) {
    if (!c || !out) return fail(PIC_ERR_ARG, "NULL argument");
    *out = c->launches;
    return PIC_OK;
}

int pic_gpu_get_stream(pic_ctx* c, void** out) {
    if (!c || !out) return fail(PIC_ERR_ARG, "NULL argument");
    *out = (void*)c->stream;
    return PIC_OK;
}

int pic_gpu_num_particles(pic_ctx* c, size_t* out) {
    if (!c || !out) return fail(PIC_ERR_ARG, "NULL argument");
    *out = c->n;
    return PIC_OK;
}

int pic_gpu_upload_particles(pic_ctx* c, const double* x, const double* y, const double* vx, const double* vy,
                             const double* q, const double* m, size_t n) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    if (n > c->cap) return fail(PIC_ERR_ARG, "pic_gpu_upload_particles: n exceeds context capacity");
    if (n > 0 && (!x || !y || !q)) return fail(PIC_ERR_ARG, "pic_gpu_upload_particles: x, y, q are required");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    bool need_m = false;
    if (m) {
        for (size_t i = 0; i < n; ++i)
            if (m[i] != 1.0) {
                need_m = true;
                break;
            }
    }
    if (need_m && !c->m) {
        int rc;
        c->m = (float*)dalloc(((c->cap ? c->cap : 1) + PARTICLE_PAD) * 4, &rc);
        if (!c->m) return rc;
    }
    c->has_mass = need_m ? 1 : 0;

    const double* src[6] = {x, y, vx, vy, q, need_m ? m : nullptr};
    ConvertArgs a{};
    a.dx = c->dx;
    a.dy = c->dy;
    a.inv_dx = exact_reciprocal(c->dx);
    a.inv_dy = exact_reciprocal(c->dy);
    a.Nx = c->Nx;
    a.Ny = c->Ny;
    a.cell = c->cell;
    a.xr = c->xr;
    a.yr = c->yr;
    a.fvx = c->vx;
    a.fvy = c->vy;
    a.fq = c->q;
    a.fm = need_m ? c->m : nullptr;
    a.st = c->dstats;
    PIC_CUDA_TRY(cudaMemsetAsync(c->dstats, 0, sizeof(DevStats), c->stream));

    // Page-locked inputs are read by the conversion kernel itself over the
    // host link (one pass, no staging copy); other inputs go through two device
    // staging slots, the copy of chunk i+1 overlapping the conversion of chunk i.
    const double* dev_src[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool direct = n > 0;
    for (int k = 0; k < 6 && direct; ++k) {
        if (!src[k]) continue;
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, src[k]) != cudaSuccess || at.type != cudaMemoryTypeHost ||
            !at.devicePointer) {
            (void)cudaGetLastError();
            direct = false;
        } else {
            dev_src[k] = (const double*)at.devicePointer;
        }
    }
    if (direct) {
        a.x = dev_src[0];
        a.y = dev_src[1];
        a.vx = dev_src[2];
        a.vy = dev_src[3];
        a.q = dev_src[4];
        a.m = dev_src[5];
        a.count = n;
        a.first = 0;
        convert_particles<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(a);
        PIC_TRY(check_launch(c, "convert_particles"));
    } else if (n > 0) {
        const size_t chunk = n < ((size_t)1 << 22) ? n : ((size_t)1 << 22);
        if (c->stage_elems < chunk * 12) {
            dfree(c->stage);
            int rc;
            c->stage = (double*)dalloc(chunk * 12 * sizeof(double), &rc);
            if (!c->stage) {
                c->stage_elems = 0;
                return rc;
            }
            c->stage_elems = chunk * 12;
        }
        PIC_TRY(ensure_copy_stream(c));
        int i = 0;
        for (size_t first = 0; first < n; first += chunk, ++i) {
            const int slot = i & 1;
            const size_t cnt = (n - first) < chunk ? (n - first) : chunk;
            double* s = c->stage + (size_t)slot * chunk * 6;
            if (i >= 2) PIC_CUDA_TRY(cudaStreamWaitEvent(c->copy_stream, c->ev_converted[slot], 0));
            double* dst[6];
            for (int k = 0; k < 6; ++k) {
                dst[k] = s + (size_t)k * chunk;
                if (src[k])
                    PIC_CUDA_TRY(cudaMemcpyAsync(dst[k], src[k] + first, cnt * sizeof(double),
                                                 cudaMemcpyHostToDevice, c->copy_stream));
            }
            PIC_CUDA_TRY(cudaEventRecord(c->ev_copied[slot], c->copy_stream));
            PIC_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->ev_copied[slot], 0));
            a.x = dst[0];
            a.y = dst[1];
            a.vx = vx ? dst[2] : nullptr;
            a.vy = vy ? dst[3] : nullptr;
            a.q = dst[4];
            a.m = need_m ? dst[5] : nullptr;
            a.count = cnt;
            a.first = first;
            convert_particles<<<(unsigned)((cnt + 255) / 256), 256, 0, c->stream>>>(a);
            PIC_TRY(check_launch(c, "convert_particles"));
            PIC_CUDA_TRY(cudaEventRecord(c->ev_converted[slot], c->stream));
        }
    }
    c->n = n;
    c->sorted = 0;
    c->part_valid = 0;
    c->qsum_valid = 0;
    c->qn_uniform = 0.0f;
    if (n > 0) {
        finish_upload<<<(unsigned)((n + 1023) / 1024), 256, 0, c->stream>>>(c->q, c->cell, n, c->dstats);
        PIC_TRY(check_launch(c, "finish_upload"));
    }
    PIC_TRY(pic_gpu_synchronize(c));
    DevStats st;
    PIC_CUDA_TRY(cudaMemcpy(&st, c->dstats, sizeof(st), cudaMemcpyDeviceToHost));
    c->qn_uniform = (n > 0 && st.q_mixed == 0 && st.q_first != 0.0f && std::isfinite(st.q_first)) ? st.q_first : 0.0f;
    if (st.order_breaks == 0) {
        // already in cell order: offsets make it usable by the tiled kernel without a sort
        PIC_TRY(ensure_sort_scratch(c));
        PIC_TRY(build_offsets(c, c->cell));
        PIC_TRY(pic_gpu_synchronize(c));
        c->sorted = 1;
        c->part_valid = 1;
    }
    return PIC_OK;
}

int pic_gpu_download_device_layout(pic_ctx* c, uint32_t* cell, float* xr, float* yr, float* vx, float* vy,
                                   float* q) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    const size_t n = c->n;
    if (n) {
        if (cell) PIC_CUDA_TRY(cudaMemcpyAsync(cell, c->cell, n * 4, cudaMemcpyDeviceToHost, c->stream));
        if (xr) PIC_CUDA_TRY(cudaMemcpyAsync(xr, c->xr, n * 4, cudaMemcpyDeviceToHost, c->stream));
        if (yr) PIC_CUDA_TRY(cudaMemcpyAsync(yr, c->yr, n * 4, cudaMemcpyDeviceToHost, c->stream));
        if (vx) PIC_CUDA_TRY(cudaMemcpyAsync(vx, c->vx, n * 4, cudaMemcpyDeviceToHost, c->stream));
        if (vy) PIC_CUDA_TRY(cudaMemcpyAsync(vy, c->vy, n * 4, cudaMemcpyDeviceToHost, c->stream));
        if (q) PIC_CUDA_TRY(cudaMemcpyAsync(q, c->q, n * 4, cudaMemcpyDeviceToHost, c->stream));
    }
    return pic_gpu_synchronize(c);
}

int pic_gpu_download_particles(pic_ctx* c, double* x, double* y, double* vx, double* vy, double* q, double* m) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    const size_t n = c->n;
    if (n == 0) return PIC_OK;
    uint32_t* cell = new uint32_t[n];
    float* f = new float[n];
    int rc = pic_gpu_download_device_layout(c, cell, nullptr, nullptr, nullptr, nullptr, nullptr);
    auto fetch = [&](const float* src, double* dst) -> int {
        if (!dst || rc != PIC_OK) return rc;
        cudaError_t e = cudaMemcpy(f, src, n * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "download");
        for (size_t i = 0; i < n; ++i) dst[i] = (double)f[i];
        return PIC_OK;
    };
    if (rc == PIC_OK && (x || y)) {
        cudaError_t e = cudaMemcpy(f, c->xr, n * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail(e, "download");
        if (rc == PIC_OK && x)
            for (size_t i = 0; i < n; ++i) x[i] = ((double)(cell[i] % (uint32_t)c->Nx) + (double)f[i]) * c->dx;
        if (rc == PIC_OK && y) {
            e = cudaMemcpy(f, c->yr, n * 4, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) rc = cuda_fail(e, "download");
            for (size_t i = 0; rc == PIC_OK && i < n; ++i)
                y[i] = ((double)(cell[i] / (uint32_t)c->Nx) + (double)f[i]) * c->dy;
        }
    }
    rc = fetch(c->vx, vx);
    rc = fetch(c->vy, vy);
    rc = fetch(c->q, q);
    if (rc == PIC_OK && q) {
        // resident charge is q / max|q|
        DevStats st;
        cudaError_t e = cudaMemcpy(&st, c->dstats, sizeof(st), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail(e, "download");
        float mq;
        std::memcpy(&mq, &st.maxq_bits, sizeof(float));
        for (size_t i = 0; rc == PIC_OK && i < n; ++i) q[i] = (double)((float)q[i] * mq);
    }
    if (rc == PIC_OK && m) {
        if (c->has_mass && c->m) {
            rc = fetch(c->m, m);
        } else {
            for (size_t i = 0; i < n; ++i) m[i] = 1.0;
        }
    }
    delete[] cell;
    delete[] f;
    return rc;
}

int pic_gpu_host_alloc(size_t bytes, void** out) {
    if (!out) return fail(PIC_ERR_ARG, "NULL argument");
    *out = nullptr;
    const cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 16, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(PIC_ERR_NOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    }
    return PIC_OK;
}

int pic_gpu_host_free(void* p) {
    if (p) PIC_CUDA_TRY(cudaFreeHost(p));
    return PIC_OK;
}

int pic_gpu_is_sorted(pic_ctx* c, int* out) {
    if (!c || !out) return fail(PIC_ERR_ARG, "NULL argument");
    *out = c->sorted;
    return PIC_OK;
}

int pic_gpu_charge_uniform(pic_ctx* c, float* out) {
    if (!c || !out) return fail(PIC_ERR_ARG, "NULL argument");
    *out = c->qn_uniform;
    return PIC_OK;
}

int pic_gpu_profile_enable(pic_ctx* c, int enable) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    c->prof_enabled = enable ? 1 : 0;
    if (!enable) prof_clear(c, nullptr);
    return PIC_OK;
}

int pic_gpu_profile_read(pic_ctx* c, const char* kernel, double* total_ms, long long* launches) {
    if (!c || !kernel || !total_ms || !launches) return fail(PIC_ERR_ARG, "NULL argument");
    PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    double tot = 0.0;
    long long cnt = 0;
    if (c->prof) {
        for (auto& r : *c->prof) {
            if (std::strcmp(r.name, kernel) != 0) continue;
            float ms = 0.0f;
            PIC_CUDA_TRY(cudaEventElapsedTime(&ms, r.a, r.b));
            tot += ms;
            ++cnt;
        }
    }
    prof_clear(c, kernel);
    *total_ms = tot;
    *launches = cnt;
    return PIC_OK;
}

}  // extern "C"
