// Field gather and leapfrog push on the resident particles.
//
//  gather   = pic::gatherFieldsSoA (src/deposition/deposition.cpp:335-356): CIC
//             interpolation of Ex, Ey at the particle with the deposit's
//             weights, then v += -(q/m) * E * dt.
//  push     = pic::pushParticlesSoA (deposition.cpp:367-374): x += v * dt with
//             periodic wrap (Domain::wrapPosition, src/pic/domain.hpp:27-32).
//  fused    = gather then push in one pass over the particles (kick of step n
//             and drift of step n+1 in the reference's loop order,
//             src/pic/simulation.cpp:82-131): reads cell, offsets, v, q
//             (24 B) and writes cell, offsets, v (20 B) per particle.
//
// Positions stay cell-relative in FP32: r' = r + v*dt/dx, the integer part moves
// the cell key (wrapped) and the fraction stays in [0,1]. Operation order
// follows the reference:
//   e  = ((E00*(1-wx))*(1-wy) + (E10*wx)*(1-wy)) + (E01*(1-wx))*wy + (E11*wx)*wy
//   v  = v + ((-q/m)*e)*dt
// with E the FP32 copies of the FP64 fields. Compiled with --fmad=false, so the
// oracle reproduces every bit.
#include "pic_internal.cuh"

namespace picgb {

struct MoveArgs {
    double* ke_partial;  // KE: per-block sums of vx^2 + vy^2 after the gather
    uint32_t* cell;
    float *xr, *yr, *vx, *vy;
    const float* q;
    const float* m;  // null when every mass is 1
    const float* Exf;
    const float* Eyf;
    size_t n;
    int Nx, Ny;
    float dtf, dtdx, dtdy;
    float qc;  // nonzero: every particle's stored charge (the charge stream is not read)
    const DevStats* st;
};


// KE (with GATHER, every mass 1): the sum of vx^2 + vy^2 of the updated
// velocities in the arithmetic of fields.cu's sum_v2_partials (exact FP32
// squares, double-FP32 per thread, FP64 across the block in a fixed order),
// one partial per block of a fixed grid: the time step's kinetic energy
// without another pass over the velocities.
template <bool GATHER, bool PUSH, bool KE = false>
__global__ void __launch_bounds__(256) move_particles(MoveArgs a) {
    float ke_hi = 0.0f, ke_lo = 0.0f;
    const float maxq = load_maxq(a.st);
    const float inv_nx = 1.0f / (float)a.Nx;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    // the next particle's key, offsets and velocities are loaded before this one is
    // used: only the field gather's round trip stays on the critical path
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t key = 0;
    float rx = 0.0f, ry = 0.0f, vxx = 0.0f, vyy = 0.0f;
    if (p < a.n) {
        key = a.cell[p];
        rx = a.xr[p];
        ry = a.yr[p];
        vxx = a.vx[p];
        vyy = a.vy[p];
    }
    for (; p < a.n; p += stride) {
        const size_t pn = p + stride;
        uint32_t nkey = 0;
        float nrx = 0.0f, nry = 0.0f, nvx = 0.0f, nvy = 0.0f;
        if (pn < a.n) {
            nkey = a.cell[pn];
            nrx = a.xr[pn];
            nry = a.yr[pn];
            nvx = a.vx[pn];
            nvy = a.vy[pn];
        }
        int iy, ix;
        split_key(key, a.Nx, inv_nx, iy, ix);
        if constexpr (GATHER) {
            const int ixp = ix + 1 == a.Nx ? 0 : ix + 1, iyp = iy + 1 == a.Ny ? 0 : iy + 1;
            const size_t i00 = (size_t)iy * a.Nx + ix, i10 = (size_t)iy * a.Nx + ixp;
            const size_t i01 = (size_t)iyp * a.Nx + ix, i11 = (size_t)iyp * a.Nx + ixp;
            const float ex = interp(a.Exf, i00, i10, i01, i11, rx, ry);
            const float ey = interp(a.Eyf, i00, i10, i01, i11, rx, ry);
            const float qf = (a.qc != 0.0f ? a.qc : a.q[p]) * maxq;
            const float coef = a.m ? __fdiv_rn(-qf, a.m[p]) : -qf;
            vxx = vxx + (coef * ex) * a.dtf;
            vyy = vyy + (coef * ey) * a.dtf;
            a.vx[p] = vxx;
            a.vy[p] = vyy;
            if constexpr (KE) ke_add(ke_hi, ke_lo, vxx, vyy);
        }
        if constexpr (PUSH) {
            drift(rx, ix, vxx, a.dtdx, a.Nx);
            drift(ry, iy, vyy, a.dtdy, a.Ny);
            a.xr[p] = rx;
            a.yr[p] = ry;
            a.cell[p] = (uint32_t)iy * (uint32_t)a.Nx + (uint32_t)ix;
        }
        key = nkey;
        rx = nrx;
        ry = nry;
        vxx = nvx;
        vyy = nvy;
    }
    if constexpr (KE) {
        __shared__ double ws[8];
        double v = __dadd_rn((double)ke_hi, (double)ke_lo);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
        if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < 8; ++w) t = __dadd_rn(t, ws[w]);
            a.ke_partial[blockIdx.x] = t;
        }
    }
}

// ke: with the gather and unit masses, also leave the kinetic sums of the
// updated velocities in c->ke_partials (fixed grid of MOVE_KE_BLOCKS blocks).
int move(pic_ctx* c, double dt, bool gather, bool push, bool ke) {
    c->ke_ready = 0;
    if (c->n == 0) return PIC_OK;
    if (gather) PIC_TRY(ensure_fields(c));
    ke = ke && gather && !c->has_mass;
    MoveArgs a;
    a.ke_partial = c->ke_partials;
    a.cell = c->cell;
    a.xr = c->xr;
    a.yr = c->yr;
    a.vx = c->vx;
    a.vy = c->vy;
    a.q = c->q;
    a.m = c->has_mass ? c->m : nullptr;
    a.Exf = c->Exf;
    a.Eyf = c->Eyf;
    a.n = c->n;
    a.Nx = c->Nx;
    a.Ny = c->Ny;
    a.dtf = (float)dt;
    a.dtdx = (float)(dt / c->dx);
    a.dtdy = (float)(dt / c->dy);
    a.qc = c->qn_uniform;
    a.st = c->dstats;
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    size_t blocks = (c->n + 255) / 256;
    if (blocks > (size_t)sms * 32) blocks = (size_t)sms * 32;
    if (ke) blocks = MOVE_KE_BLOCKS;  // the partition of the sums does not depend on the device
    prof_begin(c, gather && push ? "gather_push" : gather ? "gather" : "push");
    if (gather && push)
        ke ? move_particles<true, true, true><<<(unsigned)blocks, 256, 0, c->stream>>>(a)
           : move_particles<true, true><<<(unsigned)blocks, 256, 0, c->stream>>>(a);
    else if (gather)
        ke ? move_particles<true, false, true><<<(unsigned)blocks, 256, 0, c->stream>>>(a)
           : move_particles<true, false><<<(unsigned)blocks, 256, 0, c->stream>>>(a);
    else
        move_particles<false, true><<<(unsigned)blocks, 256, 0, c->stream>>>(a);
    prof_end(c);
    PIC_TRY(check_launch(c, "move_particles"));
    if (push) c->sorted = 0;
    c->ke_ready = ke ? 1 : 0;
    c->ke_count = MOVE_KE_BLOCKS;
    return PIC_OK;
}

int move(pic_ctx* c, double dt, bool gather, bool push) { return move(c, dt, gather, push, false); }

}  // namespace picgb

using namespace picgb;

extern "C" {

int pic_gpu_gather(pic_ctx* c, double dt) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    return move(c, dt, true, false);
}

int pic_gpu_push(pic_ctx* c, double dt) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    return move(c, dt, false, true);
}

int pic_gpu_gather_push(pic_ctx* c, double dt) {
    if (!c) return fail(PIC_ERR_ARG, "NULL context");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    return move(c, dt, true, true);
}

}  // extern "C"
