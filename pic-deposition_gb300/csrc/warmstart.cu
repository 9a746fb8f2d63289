// Learned warm start for the red-black Gauss-Seidel Poisson solve.
//
// The solve A phi = b (5-point operator, b = rho*dV - mean, periodic) is run to
// a relative residual ||b - A phi|| / ||b|| <= tol from one of three starting
// guesses:
//   0  phi of the previous step (the plain method, and the fallback),
//   1  the cubic extrapolation E = 3 phi[n-1] - 3 phi[n-2] + phi[n-3],
//   2  E plus a correction predicted by a convolutional network from the
//      residual of E:  phi0 = E + s * sigma * net(r / sigma),
//      r = b - A E,  sigma = rms(r),  s a fixed output scale.
// Every guess is iterated to the same tolerance, so the guess changes the
// number of sweeps, never the answer.
//
// The network is six 3x3 periodic convolutions with 32 channels (1 -> 32,
// 4 x 32 -> 32, 32 -> 1; the single input and output channels are carried in
// 16-channel tensors whose other channels are zero), ReLU between layers, BF16
// weights and activations with FP32 accumulation on the tensor cores
// (nn_conv.cu). It is trained with Adam on pairs (r / sigma, (phi - E) / (s * sigma))
// produced by the run itself: phi is the exact solution of the same 5-point
// system (FFT with the operator's eigenvalues, i.e. what the iteration
// converges to), E and r as above. Loss: mean squared error.
//
// Layouts: the grid (Ny rows of Nx cells, row-major) is the image (H = Ny,
// W = Nx); Nx must be a multiple of 128 and Ny even. Parameters are one FP32
// array, per layer w[9][cout][cin] then b[cout], in the order of the layers.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "nn_conv.cuh"
#include "pic_internal.cuh"

namespace picgb {

namespace {

constexpr int NL = 6;
constexpr int CIN[NL] = {16, 32, 32, 32, 32, 32};
constexpr int COUT[NL] = {32, 32, 32, 32, 32, 16};
constexpr int RED_T = 256;
constexpr int RED_B = 512;

__global__ void extrapolate3(const double* __restrict__ p1, const double* __restrict__ p2,
                             const double* __restrict__ p3, size_t g, double* __restrict__ e) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g) e[i] = __dadd_rn(__dmul_rn(3.0, __dsub_rn(p1[i], p2[i])), p3[i]);
}

__device__ __forceinline__ double block_sum_d(double v) {
    __shared__ double ws[RED_T / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) ws[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < RED_T / 32; ++w) s = __dadd_rn(s, ws[w]);
    __syncthreads();
    return s;
}

// partial[blk] = sum over a fixed chunk of x[i]^2 (x FP64) or (x[i]-y[i])^2
__global__ void sumsq_partials(const double* __restrict__ x, const double* __restrict__ y, size_t n,
                               double* __restrict__ partial) {
    const size_t chunk = (n + RED_B - 1) / RED_B;
    const size_t b = (size_t)blockIdx.x * chunk, e = b + chunk < n ? b + chunk : n;
    double s = 0.0;
    for (size_t i = b + threadIdx.x; i < e; i += RED_T) {
        const double d = y ? __dsub_rn(x[i], y[i]) : x[i];
        s = __dadd_rn(s, __dmul_rn(d, d));
    }
    const double t = block_sum_d(s);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void sum_final_d(const double* __restrict__ partial, int n, double* __restrict__ out) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += RED_T) s = __dadd_rn(s, partial[i]);
    const double t = block_sum_d(s);
    if (threadIdx.x == 0) *out = t;
}

__device__ __forceinline__ uint16_t to_bf16(float f) {
    const __nv_bfloat16 h = __float2bfloat16_rn(f);
    return *reinterpret_cast<const uint16_t*>(&h);
}
__device__ __forceinline__ float from_bf16(uint16_t u) { return __uint_as_float((uint32_t)u << 16); }

// act0[p] = (bf16(r[p] / sigma), 0 x 15), sigma = sqrt(sumsq / n)
__global__ void pack_residual(const double* __restrict__ r, const double* __restrict__ sumsq, size_t n,
                              uint16_t* __restrict__ act0) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double sig = sqrt(*sumsq / (double)n);
    const float v = sig > 0.0 ? (float)(r[i] / sig) : 0.0f;
    uint4* o = reinterpret_cast<uint4*>(act0 + i * 16);
    o[0] = make_uint4((uint32_t)to_bf16(v), 0u, 0u, 0u);
    o[1] = make_uint4(0u, 0u, 0u, 0u);
}

// dataset row: in[p] = bf16(r/sigma), tgt[p] = bf16((phi - e) / (scale * sigma))
__global__ void make_pair(const double* __restrict__ r, const double* __restrict__ phi, const double* __restrict__ e,
                          const double* __restrict__ sumsq, const double* __restrict__ scale, size_t n,
                          uint16_t* __restrict__ in, uint16_t* __restrict__ tgt) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double sig = sqrt(*sumsq / (double)n);
    const double s = sig > 0.0 ? sig : 1.0;
    in[i] = to_bf16((float)(r[i] / s));
    tgt[i] = to_bf16((float)(__dsub_rn(phi[i], e[i]) / (s * *scale)));
}

// phi[p] = e[p] + out[p] * scale * sigma
__global__ void apply_correction(const double* __restrict__ e, const float* __restrict__ out,
                                 const double* __restrict__ sumsq, const double* __restrict__ scale, size_t n,
                                 double* __restrict__ phi) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double sig = sqrt(*sumsq / (double)n);
    phi[i] = e[i] + (double)out[i] * *scale * sig;
}

// act0 for a training batch: sample s of the batch is dataset row idx[s]
__global__ void pack_batch(const uint16_t* __restrict__ ds_in, const int* __restrict__ idx, int nb, size_t P,
                           uint16_t* __restrict__ act0) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)nb * P) return;
    const int s = (int)(t / P);
    const size_t p = t - (size_t)s * P;
    const uint16_t v = ds_in[(size_t)idx[s] * P + p];
    uint4* o = reinterpret_cast<uint4*>(act0 + t * 16);
    o[0] = make_uint4((uint32_t)v, 0u, 0u, 0u);
    o[1] = make_uint4(0u, 0u, 0u, 0u);
}

// dz16[p] = (bf16(scale * (out - target)), 0 x 15); partial sums of (out - target)^2
__global__ void loss_grad(const float* __restrict__ out, const uint16_t* __restrict__ ds_tgt,
                          const int* __restrict__ idx, int nb, size_t P, float scale, uint16_t* __restrict__ dz16,
                          double* __restrict__ partial) {
    const size_t n = (size_t)nb * P;
    const size_t chunk = (n + RED_B - 1) / RED_B;
    const size_t b = (size_t)blockIdx.x * chunk, e = b + chunk < n ? b + chunk : n;
    double s = 0.0;
    for (size_t t = b + threadIdx.x; t < e; t += RED_T) {
        const int smp = (int)(t / P);
        const size_t p = t - (size_t)smp * P;
        const float d = out[t] - from_bf16(ds_tgt[(size_t)idx[smp] * P + p]);
        s = __dadd_rn(s, (double)d * (double)d);
        uint4* o = reinterpret_cast<uint4*>(dz16 + t * 16);
        o[0] = make_uint4((uint32_t)to_bf16(scale * d), 0u, 0u, 0u);
        o[1] = make_uint4(0u, 0u, 0u, 0u);
    }
    const double tot = block_sum_d(s);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

__global__ void adam_step(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                          float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1,
                          float c2) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void f32_to_bf16_rows(const float* __restrict__ x, size_t n, uint16_t* __restrict__ y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = to_bf16(x[i]);
}

unsigned blocks_for(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

struct WsState {
    int H = 0, W = 0, batch_cap = 0;
    size_t P = 0;
    size_t nparams = 0, off_w[NL] = {}, off_b[NL] = {};
    float *params = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    long long adam_t = 0;
    uint16_t* img_f[NL] = {};
    uint16_t* img_b[NL] = {};
    uint16_t* act[NL] = {};
    float* out = nullptr;
    uint16_t *dz16 = nullptr, *dza = nullptr, *dzb = nullptr;
    float* partials = nullptr;
    double* red = nullptr;      // reduction partials (RED_B)
    double* scalars = nullptr;  // [0] sumsq of r, [1] output scale, [2] loss, [3..] scratch
    double* losses = nullptr;   // per training step
    int* err = nullptr;
    int* idx = nullptr;         // sample indices (dataset rows)
    size_t idx_cap = 0;
    // dataset
    uint16_t *ds_in = nullptr, *ds_tgt = nullptr;
    size_t ds_cap = 0, ds_n = 0;
    bool scale_set = false;
    // phi history, newest first, and work fields
    double* hist[3] = {};
    int hist_n = 0;
    double *e = nullptr, *r = nullptr, *phi_new = nullptr;
};

namespace {

int ws_sumsq(pic_ctx* c, const double* x, const double* y, size_t n, double* out) {
    WsState* s = c->ws;
    sumsq_partials<<<RED_B, RED_T, 0, c->stream>>>(x, y, n, s->red);
    PIC_TRY(check_launch(c, "sumsq_partials"));
    sum_final_d<<<1, RED_T, 0, c->stream>>>(s->red, RED_B, out);
    return check_launch(c, "sum_final_d");
}

int ws_images(pic_ctx* c) {
    WsState* s = c->ws;
    for (int l = 0; l < NL; ++l) {
        PIC_TRY(picnn::build_weight_image(s->params + s->off_w[l], CIN[l], COUT[l], 0, s->img_f[l], c->stream));
        if (l > 0)
            PIC_TRY(picnn::build_weight_image(s->params + s->off_w[l], CIN[l], COUT[l], 1, s->img_b[l], c->stream));
    }
    return PIC_OK;
}

// Network forward on act[0] for nb samples -> s->out (FP32, nb*P).
int ws_forward(pic_ctx* c, int nb) {
    WsState* s = c->ws;
    const int rows = nb >= 4 ? 16 : 8;
    for (int l = 0; l < NL; ++l) {
        picnn::ConvLaunch a{s->act[l], s->img_f[l], s->params + s->off_b[l], nullptr,
                            l < NL - 1 ? (void*)s->act[l + 1] : (void*)s->out, nb, s->H, s->W, rows, s->err};
        prof_begin(c, "conv_fwd");
        const int rc = picnn::launch_conv(a, CIN[l], COUT[l], l < NL - 1 ? picnn::EPI_BIAS_RELU : picnn::EPI_BIAS_OUT,
                                          c->stream);
        prof_end(c);
        PIC_TRY(rc);
        c->launches++;
    }
    return PIC_OK;
}

// Backward from dz16 (gradient at the output) into s->grad.
int ws_backward(pic_ctx* c, int nb) {
    WsState* s = c->ws;
    const int rows = nb >= 4 ? 16 : 8;
    const long long units = picnn::wgrad_units(nb, s->H, s->W);
    const int grid0 = picnn::wgrad_grid(units);
    const int upc = (int)((units + grid0 - 1) / grid0);
    const int grid = (int)((units + upc - 1) / upc);
    const uint16_t* g = s->dz16;
    uint16_t* bufs[2] = {s->dza, s->dzb};
    for (int l = NL - 1; l >= 0; --l) {
        picnn::WgradLaunch w{s->act[l], g, s->partials, nb, s->H, s->W, upc, s->err};
        prof_begin(c, "conv_wgrad");
        const int rw = picnn::launch_wgrad(w, CIN[l], COUT[l], grid, c->stream);
        prof_end(c);
        PIC_TRY(rw);
        PIC_TRY(picnn::reduce_wgrad(s->partials, grid, CIN[l], COUT[l], s->grad + s->off_w[l], s->grad + s->off_b[l],
                                    c->stream));
        c->launches += 2;
        if (l > 0) {
            uint16_t* next = bufs[l & 1];
            picnn::ConvLaunch a{g, s->img_b[l], nullptr, s->act[l], next, nb, s->H, s->W, rows, s->err};
            prof_begin(c, "conv_dgrad");
            const int rd = picnn::launch_conv(a, COUT[l], CIN[l], picnn::EPI_MASK, c->stream);
            prof_end(c);
            PIC_TRY(rd);
            c->launches++;
            g = next;
        }
    }
    return PIC_OK;
}

int ws_check_err(pic_ctx* c) {
    int e = 0;
    PIC_CUDA_TRY(cudaMemcpyAsync(&e, c->ws->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (e) return fail(PIC_ERR_TIMEOUT, "warm-start network: a wait on the tensor cores timed out");
    return check_device_status(c);
}

int ensure_batch(pic_ctx* c, int nb) {
    WsState* s = c->ws;
    if (nb <= s->batch_cap) return PIC_OK;
    for (int l = 0; l < NL; ++l) dfree(s->act[l]);
    dfree(s->out);
    dfree(s->dz16);
    dfree(s->dza);
    dfree(s->dzb);
    dfree(s->partials);
    int rc = PIC_OK;
    const size_t P = s->P;
    for (int l = 0; l < NL; ++l) {
        s->act[l] = (uint16_t*)dalloc((size_t)nb * P * CIN[l] * 2, &rc);
        if (rc) return rc;
    }
    s->out = (float*)dalloc((size_t)nb * P * 4, &rc);
    if (!rc) s->dz16 = (uint16_t*)dalloc((size_t)nb * P * 16 * 2, &rc);
    if (!rc) s->dza = (uint16_t*)dalloc((size_t)nb * P * 32 * 2, &rc);
    if (!rc) s->dzb = (uint16_t*)dalloc((size_t)nb * P * 32 * 2, &rc);
    if (!rc)
        s->partials = (float*)dalloc((size_t)picnn::wgrad_grid(picnn::wgrad_units(nb, s->H, s->W)) *
                                         picnn::wgrad_mpad(32) * 32 * 4,
                                     &rc);
    if (rc) return rc;
    s->batch_cap = nb;
    return PIC_OK;
}

int ensure_idx(pic_ctx* c, size_t n) {
    WsState* s = c->ws;
    if (n <= s->idx_cap) return PIC_OK;
    dfree(s->idx);
    int rc = PIC_OK;
    s->idx = (int*)dalloc(n * sizeof(int), &rc);
    if (rc) return rc;
    s->idx_cap = n;
    return PIC_OK;
}

int ws_require(pic_ctx* c) {
    if (!c->ws) return fail(PIC_ERR_STATE, "learned warm start not initialised (pic_gpu_ws_init)");
    return PIC_OK;
}

// Guess for `mode` into c->phi (history must hold 3 solutions for modes 1, 2;
// the right-hand side must be prepared).
int ws_guess(pic_ctx* c, int mode) {
    WsState* s = c->ws;
    const size_t g = c->G;
    if (mode == 0) {
        PIC_CUDA_TRY(cudaMemcpyAsync(c->phi, s->hist[0], g * 8, cudaMemcpyDeviceToDevice, c->stream));
        return PIC_OK;
    }
    extrapolate3<<<blocks_for(g), 256, 0, c->stream>>>(s->hist[0], s->hist[1], s->hist[2], g,
                                                       mode == 1 ? c->phi : s->e);
    PIC_TRY(check_launch(c, "extrapolate3"));
    if (mode == 1) return PIC_OK;
    PIC_TRY(rbgs_residual_field(c, s->e, s->r));
    PIC_TRY(ws_sumsq(c, s->r, nullptr, g, s->scalars));
    pack_residual<<<blocks_for(g), 256, 0, c->stream>>>(s->r, s->scalars, g, s->act[0]);
    PIC_TRY(check_launch(c, "pack_residual"));
    PIC_TRY(ws_forward(c, 1));
    apply_correction<<<blocks_for(g), 256, 0, c->stream>>>(s->e, s->out, s->scalars, s->scalars + 1, g, c->phi);
    return check_launch(c, "apply_correction");
}

// Rotates the history: hist[0] <- phi (copied), older entries shift down.
int ws_push_history(pic_ctx* c, const double* phi) {
    WsState* s = c->ws;
    double* oldest = s->hist[2];
    s->hist[2] = s->hist[1];
    s->hist[1] = s->hist[0];
    s->hist[0] = oldest;
    PIC_CUDA_TRY(cudaMemcpyAsync(s->hist[0], phi, c->G * 8, cudaMemcpyDeviceToDevice, c->stream));
    if (s->hist_n < 3) s->hist_n++;
    return PIC_OK;
}

// One simulation step up to the right-hand side: gather+push, optional sort, CIC deposit + background.
int ws_advance(pic_ctx* c, double dt, double background, bool sort) {
    PIC_TRY(move(c, dt, true, true));
    if (sort) PIC_TRY(sort_particles(c));
    PIC_TRY(deposit_rho(c, PIC_SCHEME_CIC, 0.0, background));
    return rbgs_prepare(c);
}

// Sets the phi the next gather uses.
int ws_set_phi(pic_ctx* c, const double* phi) {
    if (phi != c->phi) PIC_CUDA_TRY(cudaMemcpyAsync(c->phi, phi, c->G * 8, cudaMemcpyDeviceToDevice, c->stream));
    return efield_from_phi(c);
}

}  // namespace

// Starting guess of a time-step solve (pic_run_config::rbgs_warm): mode 1 the
// extrapolation, mode 2 extrapolation + network; the previous phi (already in
// the context) until three solutions have been recorded.
int ws_warm_guess(pic_ctx* c, int mode) {
    if (!c->ws || c->ws->hist_n < 3 || mode <= 0) return PIC_OK;
    PIC_TRY(rbgs_prepare(c));
    return ws_guess(c, mode);
}

int ws_record_solution(pic_ctx* c) {
    if (!c->ws) return PIC_OK;
    return ws_push_history(c, c->phi);
}

void release_ws(pic_ctx* c) {
    WsState* s = c->ws;
    if (!s) return;
    void* ptrs[] = {s->params, s->grad, s->adam_m, s->adam_v, s->out, s->dz16, s->dza, s->dzb, s->partials,
                    s->red, s->scalars, s->losses, s->err, s->idx, s->ds_in, s->ds_tgt, s->hist[0], s->hist[1],
                    s->hist[2], s->e, s->r, s->phi_new};
    for (void* p : ptrs) dfree(p);
    for (int l = 0; l < NL; ++l) {
        dfree(s->img_f[l]);
        dfree(s->img_b[l]);
        dfree(s->act[l]);
    }
    delete s;
    c->ws = nullptr;
}

}  // namespace picgb

using namespace picgb;

extern "C" {

size_t pic_gpu_ws_param_count(void) {
    size_t n = 0;
    for (int l = 0; l < NL; ++l) n += (size_t)9 * CIN[l] * COUT[l] + COUT[l];
    return n;
}

int pic_gpu_ws_init(pic_ctx* c, unsigned seed, size_t dataset_capacity) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    if (c->Nx % 128 != 0 || (c->Ny & 1))
        return fail(PIC_ERR_UNSUPPORTED, "learned warm start needs Nx a multiple of 128 and even Ny");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    release_ws(c);
    PIC_TRY(ensure_fields(c));
    WsState* s = new WsState();
    c->ws = s;
    s->H = c->Ny;
    s->W = c->Nx;
    s->P = c->G;
    size_t off = 0;
    for (int l = 0; l < NL; ++l) {
        s->off_w[l] = off;
        off += (size_t)9 * CIN[l] * COUT[l];
        s->off_b[l] = off;
        off += COUT[l];
    }
    s->nparams = off;
    int rc = PIC_OK;
    auto A = [&](size_t bytes) { return rc ? nullptr : dalloc(bytes, &rc); };
    s->params = (float*)A(off * 4);
    s->grad = (float*)A(off * 4);
    s->adam_m = (float*)A(off * 4);
    s->adam_v = (float*)A(off * 4);
    for (int l = 0; l < NL; ++l) {
        s->img_f[l] = (uint16_t*)A(picnn::wimg_bytes(CIN[l], COUT[l]));
        s->img_b[l] = (uint16_t*)A(picnn::wimg_bytes(CIN[l], COUT[l]));
    }
    s->red = (double*)A(RED_B * 8);
    s->scalars = (double*)A(16 * 8);
    s->err = (int*)A(sizeof(int));
    for (int k = 0; k < 3; ++k) s->hist[k] = (double*)A(c->G * 8);
    s->e = (double*)A(c->G * 8);
    s->r = (double*)A(c->G * 8);
    s->phi_new = (double*)A(c->G * 8);
    if (dataset_capacity) {
        s->ds_in = (uint16_t*)A(dataset_capacity * c->G * 2);
        s->ds_tgt = (uint16_t*)A(dataset_capacity * c->G * 2);
        s->ds_cap = dataset_capacity;
    }
    if (rc) {
        release_ws(c);
        return rc;
    }
    PIC_TRY(ensure_batch(c, 1));
    // He-normal initialisation of the used channels; padded channels stay zero
    std::vector<float> h(off, 0.0f);
    std::mt19937 rng(seed);
    for (int l = 0; l < NL; ++l) {
        const int ci_used = l == 0 ? 1 : CIN[l];
        const int co_used = l == NL - 1 ? 1 : COUT[l];
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (9.0f * ci_used)) * (l == NL - 1 ? 0.1f : 1.0f));
        for (int t = 0; t < 9; ++t)
            for (int co = 0; co < co_used; ++co)
                for (int ci = 0; ci < ci_used; ++ci) h[s->off_w[l] + ((size_t)t * COUT[l] + co) * CIN[l] + ci] = nd(rng);
    }
    PIC_CUDA_TRY(cudaMemcpyAsync(s->params, h.data(), off * 4, cudaMemcpyHostToDevice, c->stream));
    PIC_CUDA_TRY(cudaMemsetAsync(s->adam_m, 0, off * 4, c->stream));
    PIC_CUDA_TRY(cudaMemsetAsync(s->adam_v, 0, off * 4, c->stream));
    PIC_CUDA_TRY(cudaMemsetAsync(s->err, 0, sizeof(int), c->stream));
    PIC_CUDA_TRY(cudaMemsetAsync(s->scalars, 0, 16 * 8, c->stream));
    const double one = 1.0;
    PIC_CUDA_TRY(cudaMemcpyAsync(s->scalars + 1, &one, 8, cudaMemcpyHostToDevice, c->stream));
    PIC_TRY(ws_images(c));
    return pic_gpu_synchronize(c);
}

int pic_gpu_ws_get_params(pic_ctx* c, float* params, size_t n) {
    if (!c || !params) return fail(PIC_ERR_ARG, "NULL argument");
    PIC_TRY(ws_require(c));
    if (n != c->ws->nparams) return fail(PIC_ERR_ARG, "parameter count mismatch");
    PIC_CUDA_TRY(cudaMemcpyAsync(params, c->ws->params, n * 4, cudaMemcpyDeviceToHost, c->stream));
    return pic_gpu_synchronize(c);
}

int pic_gpu_ws_set_params(pic_ctx* c, const float* params, size_t n) {
    if (!c || !params) return fail(PIC_ERR_ARG, "NULL argument");
    PIC_TRY(ws_require(c));
    if (n != c->ws->nparams) return fail(PIC_ERR_ARG, "parameter count mismatch");
    PIC_CUDA_TRY(cudaMemcpyAsync(c->ws->params, params, n * 4, cudaMemcpyHostToDevice, c->stream));
    PIC_TRY(ws_images(c));
    return pic_gpu_synchronize(c);
}

int pic_gpu_ws_loss_grad(pic_ctx* c, int batch, const float* inputs, const float* targets, double* loss, float* grad) {
    if (!c || !inputs || !targets || batch <= 0) return fail(PIC_ERR_ARG, "bad argument");
    PIC_TRY(ws_require(c));
    WsState* s = c->ws;
    const size_t P = s->P, n = (size_t)batch * P;
    PIC_TRY(ensure_batch(c, batch));
    PIC_TRY(ensure_idx(c, batch));
    int rc = PIC_OK;
    float* f = (float*)dalloc(n * 4, &rc);
    uint16_t* bin = rc ? nullptr : (uint16_t*)dalloc(n * 2, &rc);
    uint16_t* btg = rc ? nullptr : (uint16_t*)dalloc(n * 2, &rc);
    if (rc) {
        dfree(f);
        dfree(bin);
        dfree(btg);
        return rc;
    }
    std::vector<int> ident(batch);
    for (int i = 0; i < batch; ++i) ident[i] = i;
    int out = PIC_OK;
    do {
        if (cudaMemcpyAsync(s->idx, ident.data(), batch * sizeof(int), cudaMemcpyHostToDevice, c->stream) ||
            cudaMemcpyAsync(f, inputs, n * 4, cudaMemcpyHostToDevice, c->stream)) {
            out = fail(PIC_ERR_CUDA, "copy");
            break;
        }
        f32_to_bf16_rows<<<blocks_for(n), 256, 0, c->stream>>>(f, n, bin);
        if (cudaMemcpyAsync(f, targets, n * 4, cudaMemcpyHostToDevice, c->stream)) {
            out = fail(PIC_ERR_CUDA, "copy");
            break;
        }
        f32_to_bf16_rows<<<blocks_for(n), 256, 0, c->stream>>>(f, n, btg);
        pack_batch<<<blocks_for(n), 256, 0, c->stream>>>(bin, s->idx, batch, P, s->act[0]);
        if ((out = ws_forward(c, batch)) != PIC_OK) break;
        loss_grad<<<RED_B, RED_T, 0, c->stream>>>(s->out, btg, s->idx, batch, P, 2.0f / (float)n, s->dz16, s->red);
        sum_final_d<<<1, RED_T, 0, c->stream>>>(s->red, RED_B, s->scalars + 2);
        if ((out = ws_backward(c, batch)) != PIC_OK) break;
        double l = 0.0;
        if (cudaMemcpyAsync(&l, s->scalars + 2, 8, cudaMemcpyDeviceToHost, c->stream) ||
            cudaMemcpyAsync(grad, s->grad, s->nparams * 4, cudaMemcpyDeviceToHost, c->stream)) {
            out = fail(PIC_ERR_CUDA, "copy");
            break;
        }
        if ((out = ws_check_err(c)) != PIC_OK) break;
        if (loss) *loss = l / (double)n;
    } while (0);
    cudaStreamSynchronize(c->stream);
    dfree(f);
    dfree(bin);
    dfree(btg);
    return out;
}

int pic_gpu_ws_predict(pic_ctx* c, const float* input, float* output) {
    if (!c || !input || !output) return fail(PIC_ERR_ARG, "NULL argument");
    PIC_TRY(ws_require(c));
    WsState* s = c->ws;
    int rc = PIC_OK;
    float* f = (float*)dalloc(s->P * 4, &rc);
    uint16_t* b = rc ? nullptr : (uint16_t*)dalloc(s->P * 2, &rc);
    if (rc) {
        dfree(f);
        return rc;
    }
    const int zero = 0;
    int out = PIC_OK;
    PIC_TRY(ensure_idx(c, 1));
    if (cudaMemcpyAsync(s->idx, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream) ||
        cudaMemcpyAsync(f, input, s->P * 4, cudaMemcpyHostToDevice, c->stream))
        out = fail(PIC_ERR_CUDA, "copy");
    if (!out) {
        f32_to_bf16_rows<<<blocks_for(s->P), 256, 0, c->stream>>>(f, s->P, b);
        pack_batch<<<blocks_for(s->P), 256, 0, c->stream>>>(b, s->idx, 1, s->P, s->act[0]);
        out = ws_forward(c, 1);
    }
    if (!out && cudaMemcpyAsync(output, s->out, s->P * 4, cudaMemcpyDeviceToHost, c->stream))
        out = fail(PIC_ERR_CUDA, "copy");
    if (!out) out = ws_check_err(c);
    cudaStreamSynchronize(c->stream);
    dfree(f);
    dfree(b);
    return out;
}

int pic_gpu_ws_generate(pic_ctx* c, int steps, double dt, double background, int sort_interval) {
    if (!c || steps < 0) return fail(PIC_ERR_ARG, "bad argument");
    PIC_TRY(ws_require(c));
    WsState* s = c->ws;
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    for (int k = 0; k < steps; ++k) {
        PIC_TRY(ws_advance(c, dt, background, sort_interval > 0 && k % sort_interval == 0));
        PIC_TRY(solve_discrete_fft(c, c->rb_b, s->phi_new));
        if (s->hist_n >= 3 && s->ds_n < s->ds_cap) {
            extrapolate3<<<blocks_for(c->G), 256, 0, c->stream>>>(s->hist[0], s->hist[1], s->hist[2], c->G, s->e);
            PIC_TRY(check_launch(c, "extrapolate3"));
            PIC_TRY(rbgs_residual_field(c, s->e, s->r));
            PIC_TRY(ws_sumsq(c, s->r, nullptr, c->G, s->scalars));
            if (!s->scale_set) {  // output scale: rms((phi - E)/sigma) of the first pair
                PIC_TRY(ws_sumsq(c, s->phi_new, s->e, c->G, s->scalars + 3));
                double h[4];
                PIC_CUDA_TRY(cudaMemcpyAsync(h, s->scalars, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
                PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
                const double sc = h[0] > 0.0 ? std::sqrt(h[3] / h[0]) : 1.0;
                const double v = sc > 0.0 ? sc : 1.0;
                PIC_CUDA_TRY(cudaMemcpyAsync(s->scalars + 1, &v, 8, cudaMemcpyHostToDevice, c->stream));
                PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
                s->scale_set = true;
            }
            make_pair<<<blocks_for(c->G), 256, 0, c->stream>>>(s->r, s->phi_new, s->e, s->scalars, s->scalars + 1,
                                                               c->G, s->ds_in + s->ds_n * c->G,
                                                               s->ds_tgt + s->ds_n * c->G);
            PIC_TRY(check_launch(c, "make_pair"));
            s->ds_n++;
        }
        PIC_TRY(ws_push_history(c, s->phi_new));
        PIC_TRY(ws_set_phi(c, s->phi_new));
    }
    return pic_gpu_synchronize(c);
}

int pic_gpu_ws_dataset_size(pic_ctx* c, size_t* n) {
    if (!c || !n) return fail(PIC_ERR_ARG, "NULL argument");
    PIC_TRY(ws_require(c));
    *n = c->ws->ds_n;
    return PIC_OK;
}

int pic_gpu_ws_train(pic_ctx* c, int epochs, int batch, float lr, unsigned seed, double* loss_per_epoch) {
    if (!c || epochs < 0 || batch <= 0) return fail(PIC_ERR_ARG, "bad argument");
    PIC_TRY(ws_require(c));
    WsState* s = c->ws;
    if (s->ds_n < (size_t)batch) return fail(PIC_ERR_STATE, "dataset smaller than one batch");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    PIC_TRY(ensure_batch(c, batch));
    const size_t nsteps = s->ds_n / batch;
    PIC_TRY(ensure_idx(c, nsteps * batch));
    int rc = PIC_OK;
    dfree(s->losses);
    s->losses = (double*)dalloc(nsteps * 8, &rc);
    if (rc) return rc;
    std::mt19937 rng(seed);
    std::vector<int> perm(s->ds_n);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const size_t n = (size_t)batch * s->P;
    for (int ep = 0; ep < epochs; ++ep) {
        for (size_t i = 0; i < perm.size(); ++i) perm[i] = (int)i;
        std::shuffle(perm.begin(), perm.end(), rng);
        PIC_CUDA_TRY(cudaMemcpyAsync(s->idx, perm.data(), nsteps * batch * sizeof(int), cudaMemcpyHostToDevice,
                                     c->stream));
        for (size_t st = 0; st < nsteps; ++st) {
            const int* idx = s->idx + st * batch;
            pack_batch<<<blocks_for(n), 256, 0, c->stream>>>(s->ds_in, idx, batch, s->P, s->act[0]);
            PIC_TRY(check_launch(c, "pack_batch"));
            PIC_TRY(ws_forward(c, batch));
            loss_grad<<<RED_B, RED_T, 0, c->stream>>>(s->out, s->ds_tgt, idx, batch, s->P, 2.0f / (float)n, s->dz16,
                                                      s->red);
            PIC_TRY(check_launch(c, "loss_grad"));
            sum_final_d<<<1, RED_T, 0, c->stream>>>(s->red, RED_B, s->losses + st);
            PIC_TRY(check_launch(c, "sum_final_d"));
            PIC_TRY(ws_backward(c, batch));
            s->adam_t++;
            const float c1 = 1.0f - std::pow(b1, (float)s->adam_t), c2 = 1.0f - std::pow(b2, (float)s->adam_t);
            adam_step<<<blocks_for(s->nparams), 256, 0, c->stream>>>(s->params, s->grad, s->adam_m, s->adam_v,
                                                                    s->nparams, lr, b1, b2, eps, c1, c2);
            PIC_TRY(check_launch(c, "adam_step"));
            PIC_TRY(ws_images(c));
            c->launches += 4 + 11;
        }
        std::vector<double> h(nsteps);
        PIC_CUDA_TRY(cudaMemcpyAsync(h.data(), s->losses, nsteps * 8, cudaMemcpyDeviceToHost, c->stream));
        PIC_TRY(ws_check_err(c));
        double tot = 0.0;
        for (double v : h) tot += v;
        if (loss_per_epoch) loss_per_epoch[ep] = tot / ((double)nsteps * (double)n);
    }
    return pic_gpu_synchronize(c);
}

int pic_gpu_ws_study(pic_ctx* c, int steps, double dt, double background, int sort_interval, double tol,
                     int check_every, int max_iters, pic_ws_stats* stats) {
    if (!c || steps < 0 || !stats) return fail(PIC_ERR_ARG, "bad argument");
    PIC_TRY(ws_require(c));
    WsState* s = c->ws;
    if (s->hist_n < 3) return fail(PIC_ERR_STATE, "the study needs three previous solutions (run pic_gpu_ws_generate)");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    cudaEvent_t ev[2];
    PIC_CUDA_TRY(cudaEventCreate(&ev[0]));
    PIC_CUDA_TRY(cudaEventCreate(&ev[1]));
    int out = PIC_OK;
    for (int k = 0; k < steps && out == PIC_OK; ++k) {
        pic_ws_stats& st = stats[k];
        if ((out = ws_advance(c, dt, background, sort_interval > 0 && k % sort_interval == 0)) != PIC_OK) break;
        for (int mode = 0; mode < 3 && out == PIC_OK; ++mode) {
            cudaEventRecord(ev[0], c->stream);
            if ((out = ws_guess(c, mode)) != PIC_OK) break;
            int it = 0;
            double res = 0.0;
            if ((out = rbgs_solve(c, tol, max_iters, check_every, &it, &res)) != PIC_OK) break;
            cudaEventRecord(ev[1], c->stream);
            if (cudaEventSynchronize(ev[1]) != cudaSuccess) {
                out = fail(PIC_ERR_CUDA, "cudaEventSynchronize");
                break;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ev[0], ev[1]);
            st.iters[mode] = it;
            st.ms[mode] = ms;
            st.resid[mode] = res;
            st.guess_resid[mode] = c->first_rbgs_resid;
            if (mode == 0)
                out = cudaMemcpyAsync(s->phi_new, c->phi, c->G * 8, cudaMemcpyDeviceToDevice, c->stream) == cudaSuccess
                          ? PIC_OK
                          : fail(PIC_ERR_CUDA, "copy");
            else if (mode == 2)
                out = ws_sumsq(c, c->phi, s->phi_new, c->G, s->scalars + 4);
            if (out == PIC_OK && mode == 2) {
                double d[2];
                if (cudaMemcpyAsync(d, s->scalars + 4, 8, cudaMemcpyDeviceToHost, c->stream) ||
                    cudaStreamSynchronize(c->stream)) {
                    out = fail(PIC_ERR_CUDA, "copy");
                    break;
                }
                st.phi_diff = std::sqrt(d[0] / (double)c->G);
            }
        }
        if (out == PIC_OK) out = ws_push_history(c, s->phi_new);
        if (out == PIC_OK) out = ws_set_phi(c, s->phi_new);
    }
    if (out == PIC_OK) out = ws_check_err(c);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (out != PIC_OK) return out;
    return pic_gpu_synchronize(c);
}

}  // extern "C"
