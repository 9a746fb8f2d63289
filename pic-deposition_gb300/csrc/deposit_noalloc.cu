// Charge deposition for callers that cannot allocate device memory.
//
// Some hosts of this library own the whole device-memory budget and do not let
// a library allocate behind their back: a particle-in-cell code that sizes its
// particle arrays to fill the GPU and hands out every buffer from its own pool,
// or a time-step loop that must never pay the device-wide synchronisation a
// cudaMalloc/cudaFree can cause. Such a caller already owns the particle
// arrays and the output grid; what it cannot provide is the int64 accumulator
// grid the deposit needs as scratch. pic_gpu_deposit_noalloc therefore keeps
// that scratch in a fixed array in this library's device image, sized for up to
// PIC_NOALLOC_MAX_CELLS grid cells; each GPU that loads the library holds that
// array (8 MiB) until the process exits.
//
// The arithmetic is the general form of the context deposit: the same FP32
// stencil frames, the same rounding to int32 units with the same node taking
// each particle's remainder, and the same FP64 conversion, so the result equals
// pic_gpu_deposit's bit for bit on particles with more than one charge value.
// (For a set with one shared charge the context deposit's TSC uses exact
// integer weights at 2^-15 resolution; both stay within the 1e-5 relative L2
// bound of the FP64 deposit there.)
#include <cuda.h>  // driver types only: the two driver calls are resolved at run time

#include <cmath>
#include <mutex>

#include "pic_internal.cuh"

namespace picgb {
namespace noalloc {

static __device__ __align__(256) unsigned long long g_scratch[PIC_NOALLOC_MAX_CELLS];

constexpr int THREADS = 256;
constexpr int MAX_CONTEXTS = 64;

// A __device__ array's address belongs to a CUDA context, not to a device: a
// host that makes its own driver context current gets a different address
// than the device's primary context. The address is therefore looked up once
// per context (keyed by the context's unique id, which is never reused) with
// that context current, and kept in a small table.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

static std::mutex g_mutex;
static CtxGetCurrentFn g_get_current = nullptr;
static CtxGetIdFn g_get_id = nullptr;
static unsigned long long g_ctx_id[MAX_CONTEXTS] = {};
static void* g_scratch_addr[MAX_CONTEXTS] = {};
static int g_entries = 0;

static int resolve_driver_calls() {
    if (g_get_current && g_get_id) return PIC_OK;
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = cudaDriverEntryPointSymbolNotFound;
    PIC_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void**)&g_get_current, 12000, cudaEnableDefault, &q1));
    PIC_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetId", (void**)&g_get_id, 12000, cudaEnableDefault, &q2));
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !g_get_current || !g_get_id)
        return fail(PIC_ERR_UNSUPPORTED, "pic_gpu_deposit_noalloc: driver does not provide cuCtxGetCurrent/cuCtxGetId");
    return PIC_OK;
}

// The scratch array's device address in the current context.
static int scratch_for_current_context(void** out) {
    std::lock_guard<std::mutex> lock(g_mutex);
    PIC_TRY(resolve_driver_calls());
    CUcontext ctx = nullptr;
    if (g_get_current(&ctx) != CUDA_SUCCESS) return fail(PIC_ERR_CUDA, "pic_gpu_deposit_noalloc: cuCtxGetCurrent failed");
    void* p = nullptr;
    if (!ctx) {
        // no context is current yet: this runtime call makes the device's primary context current
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
        if (g_get_current(&ctx) != CUDA_SUCCESS || !ctx)
            return fail(PIC_ERR_CUDA, "pic_gpu_deposit_noalloc: no current CUDA context");
    }
    unsigned long long id = 0;
    if (g_get_id(ctx, &id) != CUDA_SUCCESS) return fail(PIC_ERR_CUDA, "pic_gpu_deposit_noalloc: cuCtxGetId failed");
    for (int i = 0; i < g_entries; ++i)
        if (g_ctx_id[i] == id) {
            *out = g_scratch_addr[i];
            return PIC_OK;
        }
    if (!p) {
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
    }
    if (g_entries < MAX_CONTEXTS) {
        g_ctx_id[g_entries] = id;
        g_scratch_addr[g_entries] = p;
        ++g_entries;
    }
    *out = p;
    return PIC_OK;
}

struct Args {
    const uint32_t* cell;
    const float* xr;
    const float* yr;
    const float* qn;
    size_t n;
    int Nx, Ny;
    unsigned long long* acc;
};

template <int NX>
__device__ __forceinline__ int first_max(const float (&X)[NX]) {
    int m = 0;
    float mv = X[0];
#pragma unroll
    for (int i = 1; i < NX; ++i)
        if (X[i] > mv) {
            mv = X[i];
            m = i;
        }
    return m;
}

// Weights of one axis relative to the particle's cell; frame node i sits at
// cell offset i + LO. NGP/CIC: offsets 0..1; TSC: -1..2.
template <int S, int NX>
__device__ __forceinline__ void frame(float r, float (&X)[NX]) {
    if constexpr (S == PIC_SCHEME_NGP) {
        X[0] = r >= 0.5f ? 0.0f : 1.0f;
        X[1] = r >= 0.5f ? 1.0f : 0.0f;
    } else if constexpr (S == PIC_SCHEME_CIC) {
        X[0] = 1.0f - r;
        X[1] = r;
    } else {
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
    }
}

template <int S>
__global__ void __launch_bounds__(THREADS) deposit_kernel(Args a) {
    constexpr int NX = (S == PIC_SCHEME_TSC) ? 4 : 2;
    constexpr int LO = (S == PIC_SCHEME_TSC) ? -1 : 0;
    const uint32_t G = (uint32_t)a.Nx * (uint32_t)a.Ny;
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += (size_t)gridDim.x * blockDim.x) {
        const uint32_t key = a.cell[p];
        if (key >= G) continue;  // not a cell of this grid: skipped
        const int iy = (int)(key / (uint32_t)a.Nx), ix = (int)(key - (uint32_t)iy * (uint32_t)a.Nx);
        const float aq = a.qn[p] * 16777216.0f;
        const int A = __float2int_rn(aq);
        float X[NX], Y[NX];
        frame<S>(a.xr[p], X);
        frame<S>(a.yr[p], Y);
        int val[NX * NX];
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
        const int kmaj = S == PIC_SCHEME_TSC ? NX + 1 : first_max(Y) * NX + first_max(X);
#pragma unroll
        for (int j = 0; j < NX; ++j) {
            const size_t row = (size_t)wrap_i(iy + LO + j, a.Ny) * a.Nx;
#pragma unroll
            for (int i = 0; i < NX; ++i) {
                const int k = j * NX + i;
                const int v = val[k] + (k == kmaj ? A - sum : 0);
                if (v != 0) atomicAdd(a.acc + row + wrap_i(ix + LO + i, a.Nx), (unsigned long long)(long long)v);
            }
        }
    }
}

__global__ void to_rho(const unsigned long long* __restrict__ acc, size_t g, double unit, double background,
                       double* __restrict__ rho) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g) rho[i] = __dadd_rn(__dmul_rn((double)(long long)acc[i], unit), background);
}

}  // namespace noalloc
}  // namespace picgb

using namespace picgb;

extern "C" int pic_gpu_deposit_noalloc(const pic_domain* dom, int scheme, const uint32_t* cell, const float* xr,
                                       const float* yr, const float* qn, size_t n, float max_abs_q,
                                       double background, double* rho, void* stream) {
    if (!dom) return fail(PIC_ERR_ARG, "pic_gpu_deposit_noalloc: NULL domain");
    if (dom->Nx < 1 || dom->Ny < 1 || !(dom->Lx > 0.0) || !(dom->Ly > 0.0))
        return fail(PIC_ERR_ARG, "pic_gpu_deposit_noalloc: grid must be Nx,Ny >= 1 and Lx,Ly > 0");
    const size_t G = (size_t)dom->Nx * (size_t)dom->Ny;
    if (G > (size_t)PIC_NOALLOC_MAX_CELLS)
        return fail(PIC_ERR_ARG, "pic_gpu_deposit_noalloc: grid of " + std::to_string(G) +
                                     " cells exceeds the fixed scratch of " + std::to_string(PIC_NOALLOC_MAX_CELLS) +
                                     " cells; use pic_gpu_deposit for larger grids");
    if (scheme != PIC_SCHEME_NGP && scheme != PIC_SCHEME_CIC && scheme != PIC_SCHEME_TSC)
        return fail(PIC_ERR_ARG, "pic_gpu_deposit_noalloc: scheme must be NGP, CIC or TSC");
    if (!rho) return fail(PIC_ERR_ARG, "pic_gpu_deposit_noalloc: NULL output grid");
    if (n > 0 && (!cell || !xr || !yr || !qn)) return fail(PIC_ERR_ARG, "pic_gpu_deposit_noalloc: NULL particle array");
    if (n > ((size_t)1 << 31) - 1) return fail(PIC_ERR_ARG, "pic_gpu_deposit_noalloc: n above 2^31-1");
    if (!(max_abs_q >= 0.0f) || !std::isfinite(max_abs_q))
        return fail(PIC_ERR_ARG, "pic_gpu_deposit_noalloc: max_abs_q must be finite and >= 0");

    void* scratch = nullptr;
    PIC_TRY(noalloc::scratch_for_current_context(&scratch));
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long* acc = (unsigned long long*)scratch;
    // the scratch keeps the previous call's sums: clear the part this grid uses
    PIC_CUDA_TRY(cudaMemsetAsync(acc, 0, G * sizeof(unsigned long long), s));

    noalloc::Args a;
    a.cell = cell;
    a.xr = xr;
    a.yr = yr;
    a.qn = qn;
    a.n = n;
    a.Nx = dom->Nx;
    a.Ny = dom->Ny;
    a.acc = acc;
    if (n > 0) {
        int dev = 0, sms = 0;
        PIC_CUDA_TRY(cudaGetDevice(&dev));
        PIC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        size_t blocks = (n + noalloc::THREADS - 1) / noalloc::THREADS;
        if (blocks > (size_t)sms * 16) blocks = (size_t)sms * 16;
        switch (scheme) {
            case PIC_SCHEME_NGP:
                noalloc::deposit_kernel<PIC_SCHEME_NGP><<<(unsigned)blocks, noalloc::THREADS, 0, s>>>(a);
                break;
            case PIC_SCHEME_CIC:
                noalloc::deposit_kernel<PIC_SCHEME_CIC><<<(unsigned)blocks, noalloc::THREADS, 0, s>>>(a);
                break;
            default:
                noalloc::deposit_kernel<PIC_SCHEME_TSC><<<(unsigned)blocks, noalloc::THREADS, 0, s>>>(a);
                break;
        }
        PIC_CUDA_TRY(cudaGetLastError());
    }
    const double inv_vol = 1.0 / ((dom->Lx / dom->Nx) * (dom->Ly / dom->Ny));
    const double unit = ((double)max_abs_q * inv_vol) * 5.9604644775390625e-08;
    noalloc::to_rho<<<(unsigned)((G + 255) / 256), 256, 0, s>>>(acc, G, unit, background, rho);
    PIC_CUDA_TRY(cudaGetLastError());
    return PIC_OK;
}
