// Device-side particle generation for the large synthetic workloads (hundreds
// of millions of particles, where building FP64 host arrays and uploading them
// would dominate): x from the density 1 + a*cos(2*pi*mode*x/Lx) by Newton's
// method on its cumulative distribution, y uniform, Maxwellian velocities
// (Box-Muller) of thermal speed vth, and optionally two equal counter-streaming
// beams +-v0 in x (first half +v0, second half -v0, as the reference's
// ParticlesSoA::initializeTwoStream, src/pic/particles_aos.cpp:142-160). Random
// numbers are Philox4x32-10, counter = particle index, so the set depends only
// on the seed. Positions are converted to the device layout exactly as an
// upload of the same FP64 positions would be (cell_coord).
#include <cmath>
#include <cstring>

#include "philox.cuh"
#include "pic_internal.cuh"

namespace picgb {

namespace {

struct GenArgs {
    size_t n;
    double Lx, Ly, dx, dy, inv_dx, inv_dy;
    int Nx, Ny;
    double amp, k, vth, v0;
    float qn;
    uint32_t seed;
    uint32_t* cell;
    float *xr, *yr, *vx, *vy, *q, *m;
    float mass;
    DevStats* st;
};

__global__ void generate_particles(GenArgs a) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float avx = 0.0f, avy = 0.0f;
    if (i < a.n) {
        U4 c;
        c.v[0] = (uint32_t)i;
        c.v[1] = (uint32_t)((uint64_t)i >> 32);
        c.v[2] = 0x47454E31u;
        c.v[3] = 1u;
        const U4 u = philox(c, a.seed, 0x2F6B3C1Du);
        c.v[3] = 2u;
        const U4 w = philox(c, a.seed, 0x2F6B3C1Du);
        const double target = unit_open0(u.v[0], u.v[1]) * a.Lx;
        double x = target;
        if (a.amp != 0.0)
            for (int it = 0; it < 8; ++it) x -= (x + (a.amp / a.k) * sin(a.k * x) - target) / (1.0 + a.amp * cos(a.k * x));
        if (x >= a.Lx) x -= a.Lx;
        const double y = unit_open0(u.v[2], u.v[3]) * a.Ly;
        const double r1 = sqrt(-2.0 * log(unit_open0(w.v[0], w.v[1])));
        const double t1 = 2.0 * unit_open0(w.v[2], w.v[3]);
        double vxx = r1 * cospi(t1) * a.vth, vyy = r1 * sinpi(t1) * a.vth;
        if (a.v0 != 0.0) vxx += (i < a.n / 2) ? a.v0 : -a.v0;
        int ix, iy;
        float rx, ry;
        if (!cell_coord(x, a.dx, a.inv_dx, a.Nx, &ix, &rx) || !cell_coord(y, a.dy, a.inv_dy, a.Ny, &iy, &ry))
            set_dev_error(a.st, DEV_BAD_POSITION, (unsigned)i);
        a.cell[i] = (uint32_t)iy * (uint32_t)a.Nx + (uint32_t)ix;
        a.xr[i] = rx;
        a.yr[i] = ry;
        const float fvx = __double2float_rn(vxx), fvy = __double2float_rn(vyy);
        a.vx[i] = fvx;
        a.vy[i] = fvy;
        a.q[i] = a.qn;
        if (a.m) a.m[i] = a.mass;
        avx = fabsf(fvx);
        avy = fabsf(fvy);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        avx = fmaxf(avx, __shfl_xor_sync(0xffffffffu, avx, o));
        avy = fmaxf(avy, __shfl_xor_sync(0xffffffffu, avy, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&a.st->maxvx_bits, __float_as_uint(avx));
        atomicMax(&a.st->maxvy_bits, __float_as_uint(avy));
    }
}

}  // namespace

}  // namespace picgb

using namespace picgb;

extern "C" int pic_gpu_generate(pic_ctx* c, const pic_gen_config* g) {
    if (!c || !g) return fail(PIC_ERR_ARG, "NULL argument");
    if (g->n > c->cap) return fail(PIC_ERR_ARG, "pic_gpu_generate: n above the context capacity");
    if (!(g->charge != 0.0) || !(g->mass > 0.0) || g->vth < 0.0 || g->mode < 0)
        return fail(PIC_ERR_ARG, "pic_gpu_generate: bad charge, mass, vth or mode");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    GenArgs a{};
    a.n = g->n;
    a.Lx = c->Lx;
    a.Ly = c->Ly;
    a.dx = c->dx;
    a.dy = c->dy;
    a.inv_dx = exact_reciprocal(c->dx);
    a.inv_dy = exact_reciprocal(c->dy);
    a.Nx = c->Nx;
    a.Ny = c->Ny;
    a.amp = g->mode ? g->amplitude : 0.0;
    a.k = 2.0 * 3.14159265358979323846 * (double)(g->mode ? g->mode : 1) / c->Lx;
    a.vth = g->vth;
    a.v0 = g->v0;
    a.qn = g->charge > 0.0 ? 1.0f : -1.0f;
    a.seed = g->seed;
    a.cell = c->cell;
    a.xr = c->xr;
    a.yr = c->yr;
    a.vx = c->vx;
    a.vy = c->vy;
    a.q = c->q;
    a.mass = (float)g->mass;
    if (a.mass != 1.0f && !c->m) {  // masses are stored only when some mass is not 1 (as an upload does)
        int rc = PIC_OK;
        c->m = (float*)dalloc(((c->cap ? c->cap : 1) + PARTICLE_PAD) * 4, &rc);
        if (!c->m) return rc;
    }
    a.m = a.mass != 1.0f ? c->m : nullptr;
    a.st = c->dstats;
    // the stored charge is q / max|q| = +-1; max|q| = |charge| (FP32), as an upload computes it
    DevStats st{};
    st.maxq_bits = 0;
    const float aq = (float)std::fabs(g->charge);
    std::memcpy(&st.maxq_bits, &aq, 4);
    PIC_CUDA_TRY(cudaMemcpyAsync(c->dstats, &st, sizeof(st), cudaMemcpyHostToDevice, c->stream));
    if (g->n) {
        generate_particles<<<(unsigned)((g->n + 255) / 256), 256, 0, c->stream>>>(a);
        PIC_TRY(check_launch(c, "generate_particles"));
    }
    c->n = g->n;
    c->has_mass = a.m ? 1 : 0;
    c->sorted = 0;
    c->part_valid = 0;
    c->qsum_valid = 0;
    c->qn_uniform = g->n ? a.qn : 0.0f;
    c->launches++;
    return pic_gpu_synchronize(c);
}
