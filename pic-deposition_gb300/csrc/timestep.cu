// Time stepping on the resident particles: pic::Simulation::run's loop
// (src/pic/simulation.cpp:69-145) with the deposit, Poisson solve, gather and
// push on the GPU.
//
// Per step, for NGP/CIC/TSC (simulation.cpp:94-98, 101-105, 120-131):
//     push(dt) -> [cell sort, every sort_interval steps] -> deposit -> + background
//     -> Poisson -> gather(dt) -> diagnostics
// where a step's gather runs in one pass with the next step's push (same
// arithmetic, one read and write of the particles fewer) and its diagnostics
// right after that pass.
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
#include <vector>

#include "pic_internal.cuh"

namespace picgb {

int move(pic_ctx* c, double dt, bool gather, bool push);
int move(pic_ctx* c, double dt, bool gather, bool push, bool ke);
int rbgs_solve_async(pic_ctx* c, double tol, int max_iters, int check_every);
int ws_warm_guess(pic_ctx* c, int mode);
int ws_record_solution(pic_ctx* c);

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

// moved[s] = the particles the step's deposit found outside their sorted cell
// (step s = the diagnostics counter: the previous step's diagnostics are done)
__global__ void take_moved(DevStats* st, unsigned long long* __restrict__ moved, const int* __restrict__ step,
                           int steps) {
    const int s = *step;
    if (s < steps) moved[s] = st->moved;
    st->moved = 0;
}

static int solve(pic_ctx* c, const pic_run_config* cfg) {
    if (cfg->poisson != 1) return poisson_fft(c);
    if (cfg->rbgs_warm > 0) PIC_TRY(ws_warm_guess(c, cfg->rbgs_warm));
    PIC_TRY(rbgs_solve_async(c, cfg->rbgs_tol, cfg->rbgs_max_iters, cfg->rbgs_check_every));
    return cfg->rbgs_warm > 0 ? ws_record_solution(c) : PIC_OK;
}

// The diagnostics of the step whose gather has just run.
static int record_step(pic_ctx* c, double* hist, int* step_ctr, int steps) {
    PIC_TRY(diagnostics_async(c));
    finalize_diag<<<1, 1, 0, c->stream>>>(c->red_out, c->dx * c->dy, hist, step_ctr, steps);
    return check_launch(c, "finalize_diag");
}

// One step; `do_sort` selects the variant with the cell sort. For NGP/CIC/TSC
// the step ends after its Poisson solve with its gather pending: with `head`,
// the previous step's gather runs fused with this step's push (kick of step
// s-1 and drift of step s in one pass over the particles, push.cu's fused
// kernel), then the previous step's diagnostics (the push leaves the velocities
// unchanged); the last step's gather runs after the loop.
static int one_step(pic_ctx* c, const pic_run_config* cfg, bool do_sort, double* hist, int* step_ctr, int steps,
                    bool head, unsigned long long* moved) {
    auto count_moved = [&]() -> int {
        if (!moved) return PIC_OK;
        take_moved<<<1, 1, 0, c->stream>>>(c->dstats, moved, step_ctr, steps);
        return check_launch(c, "take_moved");
    };
    if (cfg->scheme == PIC_SCHEME_ESIRKEPOV) {
        PIC_TRY(deposit_rho(c, cfg->scheme, cfg->dt, cfg->background));
        PIC_TRY(count_moved());
        PIC_TRY(solve(c, cfg));
        PIC_TRY(move(c, cfg->dt, false, true));
        PIC_TRY(move(c, cfg->dt, true, false, true));
        return record_step(c, hist, step_ctr, steps);
    }
    if (head) {
        PIC_TRY(move(c, cfg->dt, true, true, true));
        PIC_TRY(record_step(c, hist, step_ctr, steps));
    } else {
        PIC_TRY(move(c, cfg->dt, false, true));
    }
    if (do_sort) PIC_TRY(sort_particles(c));
    PIC_TRY(deposit_rho(c, cfg->scheme, cfg->dt, cfg->background));
    PIC_TRY(count_moved());
    return solve(c, cfg);
}

// The cell sort ping-pongs the particle arrays with their scratch copies by
// swapping the context's pointers on the host. A captured graph keeps the
// pointers of its capture, so each graph is keyed by the buffer assignment it
// starts from and records the assignment it leaves; after a replay the host
// pointers are set to that assignment. Assignments alternate between two
// states, so at most four graphs exist.
struct Buffers {
    uint32_t *cell, *cell_alt, *idx_a, *idx_b;
    float *xr, *yr, *vx, *vy, *q, *m;
    float* alt[6];
    int sorted, part_valid;
    bool operator==(const Buffers& o) const {
        return cell == o.cell && cell_alt == o.cell_alt && idx_a == o.idx_a && xr == o.xr && yr == o.yr &&
               vx == o.vx && vy == o.vy && q == o.q && m == o.m;
    }
};

static Buffers buffers_of(const pic_ctx* c) {
    Buffers b;
    b.cell = c->cell;
    b.cell_alt = c->cell_alt;
    b.idx_a = c->idx_a;
    b.idx_b = c->idx_b;
    b.xr = c->xr;
    b.yr = c->yr;
    b.vx = c->vx;
    b.vy = c->vy;
    b.q = c->q;
    b.m = c->m;
    for (int k = 0; k < 6; ++k) b.alt[k] = c->alt[k];
    b.sorted = c->sorted;
    b.part_valid = c->part_valid;
    return b;
}

static void set_buffers(pic_ctx* c, const Buffers& b) {
    c->cell = b.cell;
    c->cell_alt = b.cell_alt;
    c->idx_a = b.idx_a;
    c->idx_b = b.idx_b;
    c->xr = b.xr;
    c->yr = b.yr;
    c->vx = b.vx;
    c->vy = b.vy;
    c->q = b.q;
    c->m = b.m;
    for (int k = 0; k < 6; ++k) c->alt[k] = b.alt[k];
    c->sorted = b.sorted;
    c->part_valid = b.part_valid;
}

struct StepGraph {
    bool do_sort;
    Buffers before, after;
    cudaGraphExec_t exec;
    long long kernels;
};

static int capture(pic_ctx* c, const pic_run_config* cfg, bool do_sort, double* hist, int* ctr, int steps,
                   bool head, unsigned long long* moved, cudaGraphExec_t* out) {
    const int prof = c->prof_enabled;
    c->prof_enabled = 0;
    cudaGraph_t g = nullptr;
    const long long l0 = c->launches;
    PIC_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = one_step(c, cfg, do_sort, hist, ctr, steps, head, moved);
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
    if (cfg->poisson == 1 && (cfg->rbgs_warm < 0 || cfg->rbgs_warm > 2))
        return fail(PIC_ERR_ARG, "rbgs_warm must be 0, 1 or 2");
    if (cfg->poisson == 1 && cfg->rbgs_warm > 0 && !c->ws)
        return fail(PIC_ERR_STATE, "rbgs_warm 1 and 2 need pic_gpu_ws_init");
    if (steps < 0) return fail(PIC_ERR_ARG, "steps < 0");
    if (cfg->sort_interval < 0) return fail(PIC_ERR_ARG, "sort_interval < 0");
    if (!(cfg->sort_moved_fraction >= 0.0 && cfg->sort_moved_fraction <= 1.0))
        return fail(PIC_ERR_ARG, "sort_moved_fraction must be in [0, 1]");
    if (steps == 0) return PIC_OK;
    int rc = PIC_OK;
    const bool by_moved = cfg->sort_moved_fraction > 0.0;
    double* hist = (double*)dalloc((size_t)steps * 6 * sizeof(double), &rc);
    if (!hist) return rc;
    int* ctr = (int*)dalloc(sizeof(int), &rc);
    unsigned long long* moved = nullptr;     // per step, on the device
    unsigned long long* moved_h = nullptr;   // the same, page-locked, copied after each step
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    if (ctr && by_moved) {
        moved = (unsigned long long*)dalloc((size_t)steps * sizeof(unsigned long long), &rc);
        if (moved && cudaHostAlloc((void**)&moved_h, (size_t)steps * sizeof(unsigned long long), 0) != cudaSuccess) {
            moved_h = nullptr;
            rc = fail(PIC_ERR_NOMEM, "pinned allocation");
        }
        for (int i = 0; i < 3 && rc == PIC_OK; ++i)
            if (cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess)
                rc = fail(PIC_ERR_CUDA, "cudaEventCreate");
    }
    std::vector<StepGraph> graphs;
    auto cleanup = [&]() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.exec);
        cudaStreamSynchronize(c->stream);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        if (moved_h) cudaFreeHost(moved_h);
        dfree(moved);
        dfree(hist);
        dfree(ctr);
    };
    if (rc != PIC_OK) {
        cleanup();
        return rc;
    }
    rc = [&]() -> int {
        PIC_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(int), c->stream));
        PIC_CUDA_TRY(cudaMemsetAsync(&c->dstats->moved, 0, sizeof(unsigned long long), c->stream));
        PIC_TRY(ensure_fields(c));
        const int k = cfg->sort_interval;
        // the Gauss-Seidel stop is decided on the host, so those steps run eagerly
        const bool graph = cfg->use_graph && cfg->poisson == 0;
        const bool esk = cfg->scheme == PIC_SCHEME_ESIRKEPOV;
        const double limit = cfg->sort_moved_fraction * (double)c->n;
        int last_sort = -1;
        for (int s = 0; s < steps; ++s) {
            bool do_sort = k > 0 && (s % k) == 0;
            if (by_moved) {
                // interval: steps since the last sort; step 0 sorts unless already in order
                do_sort = (s == 0 && !c->sorted) || (k > 0 && last_sort >= 0 && s - last_sort >= k);
                const int m = s - 2;  // the newest count the host may wait for without draining the GPU
                if (!do_sort && m >= 0 && m > last_sort) {
                    PIC_CUDA_TRY(cudaEventSynchronize(ev[m % 3]));
                    do_sort = (double)moved_h[m] > limit;
                }
            }
            if (do_sort) {
                last_sort = s;
                c->sorts++;
            }
            const bool head = s > 0;  // the previous step's gather is pending (NGP/CIC/TSC)
            auto after_step = [&]() -> int {
                if (!by_moved) return PIC_OK;
                PIC_CUDA_TRY(cudaMemcpyAsync(moved_h + s, moved + s, sizeof(unsigned long long),
                                             cudaMemcpyDeviceToHost, c->stream));
                PIC_CUDA_TRY(cudaEventRecord(ev[s % 3], c->stream));
                return PIC_OK;
            };
            if (!graph || s == 0) {
                PIC_TRY(one_step(c, cfg, do_sort, hist, ctr, steps, head, moved));
                PIC_TRY(after_step());
                continue;
            }
            const Buffers now = buffers_of(c);
            StepGraph* g = nullptr;
            for (auto& sg : graphs)
                if (sg.do_sort == do_sort && sg.before == now && sg.before.sorted == now.sorted) g = &sg;
            if (!g) {
                StepGraph sg;
                sg.do_sort = do_sort;
                sg.before = now;
                PIC_TRY(capture(c, cfg, do_sort, hist, ctr, steps, head, moved, &sg.exec));
                sg.after = buffers_of(c);  // the capture ran the host side: pointers as the graph leaves them
                sg.kernels = do_sort ? c->graph_launches_sort : c->graph_launches_plain;
                graphs.push_back(sg);
                g = &graphs.back();
            }
            PIC_CUDA_TRY(cudaGraphLaunch(g->exec, c->stream));
            set_buffers(c, g->after);
            c->launches += g->kernels;
            PIC_TRY(after_step());
        }
        if (!esk) {  // the last step's gather and diagnostics
            PIC_TRY(move(c, cfg->dt, true, false, true));
            PIC_TRY(record_step(c, hist, ctr, steps));
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

extern "C" int pic_gpu_sort_count(pic_ctx* c, long long* n) {
    if (!c || !n) return fail(PIC_ERR_ARG, "NULL argument");
    *n = c->sorts;
    return PIC_OK;
}
