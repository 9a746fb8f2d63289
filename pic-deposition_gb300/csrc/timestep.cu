// Time stepping on the resident particles: pic::Simulation::run's loop
// (src/pic/simulation.cpp:69-145) with the deposit, Poisson solve, gather and
// push on the GPU.
//
// Per step, for NGP/CIC/TSC (simulation.cpp:94-98, 101-105, 120-131):
//     push(dt) -> [cell sort, every sort_interval steps] -> deposit -> + background
//     -> Poisson -> gather(dt) -> diagnostics
// and for the trajectory-averaged ("Esirkepov") rho:
//     deposit(dt) -> + background -> Poisson -> push(dt) -> gather(dt) -> diagnostics.
// The reference sorts a copy of the particles inside every deposit
// (deposition.cpp:185-188); here the sort is in place and persists, and between
// sorts the deposit uses the run-aggregating kernel on the nearly ordered
// particles. Because the deposit is fixed point (order independent), the sort
// interval does not change any result bit.
//
// Diagnostics of every step (pic::computeDiagnostics, diagnostics.cpp:42-51)
// are reduced and finalised on the device into a history buffer, read back once
// at the end. With use_graph, one eager step warms every allocation, then the
// step with and without the sort are captured as CUDA graphs and replayed.
#include "pic_internal.cuh"

namespace picgb {

int move(pic_ctx* c, double dt, bool gather, bool push);
int rbgs_solve_async(pic_ctx* c, double tol, int max_iters, int check_every);

// pic_diag from the raw sums in red_out (same formulas as read_diagnostics).
__global__ void finalize_diag(const double* __restrict__ r, double vol, double* __restrict__ hist,
                              int* __restrict__ step, int steps) {
    const int s = *step;
    if (s < steps) {
        double* d = hist + (size_t)s * 6;
        const double total_charge = r[1];
        const double integrated = __dmul_rn(r[2], vol);
        const double den = r[6] > 1e-12 ? r[6] : 1e-12;
        const double ke = r[3];
        const double fe = __dmul_rn(__dmul_rn(0.5, r[4]), vol);
        d[0] = __ddiv_rn(fabs(__dsub_rn(integrated, total_charge)), den);
        d[1] = total_charge;
        d[2] = integrated;
        d[3] = ke;
        d[4] = fe;
        d[5] = __dadd_rn(ke, fe);
    }
    *step = s + 1;
}

static int solve(pic_ctx* c, const pic_run_config* cfg) {
    if (cfg->poisson == 1) return rbgs_solve_async(c, cfg->rbgs_tol, cfg->rbgs_max_iters, cfg->rbgs_check_every);
    return poisson_fft(c);
}

// One step; `do_sort` selects the variant with the cell sort.
static int one_step(pic_ctx* c, const pic_run_config* cfg, bool do_sort, double* hist, int* step_ctr, int steps) {
    const bool esk = cfg->scheme == PIC_SCHEME_ESIRKEPOV;
    if (!esk) PIC_TRY(move(c, cfg->dt, false, true));
    if (do_sort) PIC_TRY(sort_particles(c));
    PIC_TRY(deposit_rho(c, cfg->scheme, cfg->dt, cfg->background));
    PIC_TRY(solve(c, cfg));
    if (esk) PIC_TRY(move(c, cfg->dt, false, true));
    PIC_TRY(move(c, cfg->dt, true, false));
    PIC_TRY(diagnostics_async(c));
    finalize_diag<<<1, 1, 0, c->stream>>>(c->red_out, c->dx * c->dy, hist, step_ctr, steps);
    return check_launch(c, "finalize_diag");
}

static int capture(pic_ctx* c, const pic_run_config* cfg, bool do_sort, double* hist, int* ctr, int steps,
                   cudaGraphExec_t* out) {
    const int prof = c->prof_enabled;
    c->prof_enabled = 0;
    cudaGraph_t g = nullptr;
    const long long l0 = c->launches;
    PIC_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = one_step(c, cfg, do_sort, hist, ctr, steps);
    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->prof_enabled = prof;
    (do_sort ? c->graph_launches_sort : c->graph_launches_plain) = c->launches - l0;
    c->launches = l0;  // capturing launches nothing
    if (rc != PIC_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    const cudaError_t e2 = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaGraphInstantiate");
    return PIC_OK;
}

int run_steps(pic_ctx* c, const pic_run_config* cfg, int steps, pic_diag* history) {
    if (cfg->scheme < PIC_SCHEME_NGP || cfg->scheme > PIC_SCHEME_ESIRKEPOV) return fail(PIC_ERR_ARG, "unknown scheme");
    if (cfg->poisson != 0 && cfg->poisson != 1) return fail(PIC_ERR_ARG, "poisson must be 0 (FFT) or 1 (RBGS)");
    if (steps < 0) return fail(PIC_ERR_ARG, "steps < 0");
    if (steps == 0) return PIC_OK;
    int rc = PIC_OK;
    double* hist = (double*)dalloc((size_t)steps * 6 * sizeof(double), &rc);
    if (!hist) return rc;
    int* ctr = (int*)dalloc(sizeof(int), &rc);
    if (!ctr) {
        dfree(hist);
        return rc;
    }
    cudaGraphExec_t gsort = nullptr, gplain = nullptr;
    auto cleanup = [&]() {
        if (gsort) cudaGraphExecDestroy(gsort);
        if (gplain) cudaGraphExecDestroy(gplain);
        cudaStreamSynchronize(c->stream);
        dfree(hist);
        dfree(ctr);
    };
    rc = [&]() -> int {
        PIC_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(int), c->stream));
        PIC_TRY(ensure_fields(c));
        const int k = cfg->sort_interval;
        // the Gauss-Seidel stop is decided on the host, so those steps run eagerly
        const bool graph = cfg->use_graph && cfg->poisson == 0;
        for (int s = 0; s < steps; ++s) {
            const bool do_sort = k > 0 && (s % k) == 0;
            if (!graph || s == 0) {
                PIC_TRY(one_step(c, cfg, do_sort, hist, ctr, steps));
                continue;
            }
            cudaGraphExec_t& g = do_sort ? gsort : gplain;
            if (!g) PIC_TRY(capture(c, cfg, do_sort, hist, ctr, steps, &g));
            PIC_CUDA_TRY(cudaGraphLaunch(g, c->stream));
            c->launches += do_sort ? c->graph_launches_sort : c->graph_launches_plain;
        }
        if (history)
            PIC_CUDA_TRY(cudaMemcpyAsync(history, hist, (size_t)steps * 6 * sizeof(double), cudaMemcpyDeviceToHost,
                                         c->stream));
        PIC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        c->sorted = 0;  // conservative: the last step pushed the particles
        return check_device_status(c);
    }();
    cleanup();
    return rc;
}

}  // namespace picgb

using namespace picgb;

extern "C" int pic_gpu_run(pic_ctx* c, const pic_run_config* cfg, int steps, pic_diag* history) {
    if (!c || !cfg) return fail(PIC_ERR_ARG, "NULL argument");
    PIC_CUDA_TRY(cudaSetDevice(c->device));
    return run_steps(c, cfg, steps, history);
}
