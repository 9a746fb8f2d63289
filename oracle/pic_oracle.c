/*
 * CPU oracle for the GB300 PIC deposition path -- TEST INFRASTRUCTURE ONLY.
 * See pic_oracle.h for who may call it. Every function cites the reference
 * (ehocine/pic-deposition) file:line it restates, or says that it restates
 * the GPU arithmetic of this project.
 */
#include "pic_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ======================================================================= */
/* geometry                                                                 */
/* ======================================================================= */

/* wrapIndex, src/deposition/ngp.cpp:9 */
static inline int wrap_index(int i, int n) { return (i % n + n) % n; }

static inline double dom_dx(const orc_domain* d) { return d->Lx / d->Nx; } /* domain.hpp:17-20 */
static inline double dom_dy(const orc_domain* d) { return d->Ly / d->Ny; }

/* Domain::cellCoords, src/pic/domain.hpp:34-43, with dx = Lx/Nx, dy = Ly/Ny precomputed */
static inline void cell_coords(double dx, double dy, int Nx, int Ny, double x, double y, int* ix, int* iy, double* wx,
                               double* wy) {
    double fx = x / dx;
    double fy = y / dy;
    int i = (int)floor(fx);
    int j = (int)floor(fy);
    fx -= i;
    fy -= j;
    *ix = wrap_index(i, Nx);
    *iy = wrap_index(j, Ny);
    *wx = fx;
    *wy = fy;
}

void orc_cell_coords(const orc_domain* d, double x, double y, int* ix, int* iy, double* wx, double* wy) {
    cell_coords(dom_dx(d), dom_dy(d), d->Nx, d->Ny, x, y, ix, iy, wx, wy);
}

/* particleCellIndex, src/sorting/cell_sort.cpp:8-13 (cellIndex = iy*Nx+ix, domain.hpp:25) */
int orc_particle_cell_index(const orc_domain* d, double x, double y) {
    int ix, iy;
    double wx, wy;
    orc_cell_coords(d, x, y, &ix, &iy, &wx, &wy);
    return iy * d->Nx + ix;
}

/* ======================================================================= */
/* reference RNG: std::mt19937 (Matsumoto & Nishimura 1998), the 53-bit    */
/* canonical double made from two 32-bit draws, and the Marsaglia polar    */
/* normal method, as libstdc++ applies them. A fresh normal distribution   */
/* is built for every draw (sampleNormal, particles_aos.cpp:11-14), so the */
/* second polar variate is always discarded.                               */
/* ======================================================================= */

typedef struct {
    uint32_t mt[624];
    int idx;
} mt19937;

static void mt_seed(mt19937* g, uint32_t seed) {
    g->mt[0] = seed;
    for (int i = 1; i < 624; ++i) g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->idx = 624;
}

static uint32_t mt_next(mt19937* g) {
    if (g->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            const uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
            g->mt[i] = g->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        g->idx = 0;
    }
    uint32_t y = g->mt[g->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* canonical double in [0,1) from two draws: (g1 + g2 * 2^32) / 2^64 */
static double mt_canonical(mt19937* g) {
    double sum = 0.0, tmp = 1.0;
    for (int k = 0; k < 2; ++k) {
        sum += (double)mt_next(g) * tmp;
        tmp *= 4294967296.0;
    }
    double r = sum / tmp;
    if (r >= 1.0) r = nextafter(1.0, 0.0);
    return r;
}

static double mt_uniform(mt19937* g, double a, double b) { return (b - a) * mt_canonical(g) + a; }

static double mt_normal(mt19937* g, double stddev) {
    double x, y, r2;
    do {
        x = 2.0 * mt_canonical(g) - 1.0;
        y = 2.0 * mt_canonical(g) - 1.0;
        r2 = x * x + y * y;
    } while (r2 > 1.0 || r2 == 0.0);
    const double mult = sqrt(-2 * log(r2) / r2);
    const double ret = y * mult;
    return ret * stddev + 0.0;
}

/* ParticlesSoA initialisers, src/pic/particles_aos.cpp:
 *   kind 0 initializeUniformMaxwellian  :67-81  (p0 = T)
 *   kind 1 initializeLangmuirWave       :83-96  (p0 = amplitude)
 *   kind 2 initializeWarmLangmuirWave   :98-113 (p0 = amplitude, p1 = temperature)
 *   kind 3 initializeTwoStream          :142-160 (p0 = beam velocity, p1 = perturbation)
 *   kind 4 initializeTwoStreamQuasi1D   :162-180 */
int orc_init_particles(int kind, const orc_domain* d, size_t n, double p0, double p1, int mode, uint32_t seed,
                       double* x, double* y, double* vx, double* vy, double* q, double* m) {
    mt19937* g = (mt19937*)malloc(sizeof(mt19937));
    mt_seed(g, seed);
    const double Lx = d->Lx, Ly = d->Ly;
    if (kind == 0) {
        const double stdv = sqrt(p0);
        for (size_t i = 0; i < n; ++i) {
            x[i] = mt_uniform(g, 0.0, Lx);
            y[i] = mt_uniform(g, 0.0, Ly);
            vx[i] = mt_normal(g, stdv);
            vy[i] = mt_normal(g, stdv);
            m[i] = 1.0;
            q[i] = (i % 2 == 0) ? 1.0 : -1.0;
        }
    } else if (kind == 1 || kind == 2) {
        const double k = 2.0 * M_PI * (double)mode / Lx;
        const double qp = -1.0 / (double)n;
        const double stdv = sqrt(p1);
        for (size_t i = 0; i < n; ++i) {
            x[i] = Lx * (double)i / (double)n;
            y[i] = 0.5 * Ly;
            if (kind == 1) {
                vx[i] = p0 * sin(k * x[i]);
                vy[i] = 0.0;
            } else {
                vx[i] = p0 * sin(k * x[i]) + mt_normal(g, stdv);
                vy[i] = mt_normal(g, stdv);
            }
            m[i] = 1.0;
            q[i] = qp;
        }
    } else if (kind == 3 || kind == 4) {
        const double qp = -1.0 / (double)n;
        const double k = 2.0 * M_PI / Lx;
        for (size_t i = 0; i < n; ++i) {
            x[i] = mt_uniform(g, 0.0, Lx);
            y[i] = (kind == 3) ? mt_uniform(g, 0.0, Ly) : 0.5 * Ly;
            const double sign = (i < n / 2) ? 1.0 : -1.0;
            const double pert = p1 * sin(k * x[i]);
            vx[i] = sign * p0 + pert;
            vy[i] = 0.0;
            m[i] = 1.0;
            q[i] = qp;
        }
    } else {
        free(g);
        return -1;
    }
    free(g);
    return 0;
}

/* ======================================================================= */
/* FP64 reference deposits                                                  */
/* ======================================================================= */

/* tscWeights, src/deposition/ngp.cpp:28-34 */
static void tsc_weights(double xi, double w[3], int* i0) {
    *i0 = (int)floor(xi - 0.5);
    const double x = xi - (double)(*i0);
    w[0] = 0.5 * (1.5 - x) * (1.5 - x);
    w[1] = 0.75 - (x - 1.0) * (x - 1.0);
    w[2] = 0.5 * (x - 0.5) * (x - 0.5);
}

typedef struct {
    int index;
    double weight;
} esk_weight;

/* esirkepovWeights1DSparse, src/deposition/ngp.cpp:36-84. Returns the count;
 * `cap` bounds the list (the reference uses a growable vector). */
static int esirkepov_weights_1d(double x0, double x1, double dx, int n, esk_weight* w, int cap) {
    int cnt = 0;
    if (fabs(x1 - x0) < 1e-15) {
        const int ix = (int)floor(x0 / dx);
        const double xi = x0 / dx - (double)ix;
        w[0].index = wrap_index(ix, n);
        w[0].weight = 1.0 - xi;
        w[1].index = wrap_index(ix + 1, n);
        w[1].weight = xi;
        return 2;
    }
    const double inv_dx = 1.0 / dx;
    double x_curr = x0;
    const double x_end = x1;
    int cell = (int)floor(x_curr * inv_dx);
    if (x_end > x0) {
        while (x_curr < x_end - 1e-15 && cnt < cap) {
            const double b = (cell + 1) * dx;
            const double x_next = x_end < b ? x_end : b;
            w[cnt].index = wrap_index(cell, n);
            w[cnt].weight = (x_next - x_curr) * inv_dx;
            ++cnt;
            x_curr = x_next;
            cell++;
        }
    } else {
        while (x_curr > x_end + 1e-15 && cnt < cap) {
            const double b = cell * dx;
            const double x_next = x_end > b ? x_end : b;
            w[cnt].index = wrap_index(cell, n);
            w[cnt].weight = (x_curr - x_next) * inv_dx;
            ++cnt;
            x_curr = x_next;
            cell--;
        }
    }
    double total = 0.0;
    for (int k = 0; k < cnt; ++k) total += w[k].weight;
    if (total > 1e-300) {
        const double inv_total = 1.0 / total;
        for (int k = 0; k < cnt; ++k) w[k].weight *= inv_total;
    }
    return cnt;
}

#define ESK_CAP 4096

/* One particle range [b, e) into rho, serial reference order:
 *   NGP        ngp.cpp:108-120 (q / cellVolume) or deposition_parallel.cpp:51-66 (q * inv_vol)
 *   CIC        ngp.cpp:140-157, deposition_parallel.cpp:68-87
 *   TSC        ngp.cpp:181-202, deposition_parallel.cpp:89-116 (indices wrapped correctly here)
 *   Esirkepov  ngp.cpp:13-24,216-228, deposition_parallel.cpp:118-144 */
static void deposit_range(const orc_domain* d, int scheme, size_t b, size_t e, const double* x, const double* y,
                          const double* vx, const double* vy, const double* q, double dt, int parallel_form,
                          double* rho, esk_weight* xs, esk_weight* ys) {
    const double dx = dom_dx(d), dy = dom_dy(d);
    const double vol = dx * dy;
    const double inv_vol = 1.0 / vol;
    const int Nx = d->Nx, Ny = d->Ny;
    if (scheme == ORC_NGP) {
        for (size_t idx = b; idx < e; ++idx) {
            int ix, iy;
            double wx, wy;
            cell_coords(dx, dy, Nx, Ny, x[idx], y[idx], &ix, &iy, &wx, &wy);
            const int jx = wx >= 0.5 ? wrap_index(ix + 1, Nx) : ix;
            const int jy = wy >= 0.5 ? wrap_index(iy + 1, Ny) : iy;
            rho[(size_t)jy * Nx + jx] += parallel_form ? q[idx] * inv_vol : q[idx] / vol;
        }
    } else if (scheme == ORC_CIC) {
        for (size_t idx = b; idx < e; ++idx) {
            int ix, iy;
            double wx, wy;
            cell_coords(dx, dy, Nx, Ny, x[idx], y[idx], &ix, &iy, &wx, &wy);
            const double qq = q[idx] * inv_vol;
            const int ixp = wrap_index(ix + 1, Nx);
            const int iyp = wrap_index(iy + 1, Ny);
            rho[(size_t)iy * Nx + ix] += qq * (1.0 - wx) * (1.0 - wy);
            rho[(size_t)iy * Nx + ixp] += qq * wx * (1.0 - wy);
            rho[(size_t)iyp * Nx + ix] += qq * (1.0 - wx) * wy;
            rho[(size_t)iyp * Nx + ixp] += qq * wx * wy;
        }
    } else if (scheme == ORC_TSC) {
        for (size_t idx = b; idx < e; ++idx) {
            const double fx = x[idx] / dx;
            const double fy = y[idx] / dy;
            int ix0, iy0;
            double wx[3], wy[3];
            tsc_weights(fx, wx, &ix0);
            tsc_weights(fy, wy, &iy0);
            const double qq = q[idx] * inv_vol;
            for (int oy = 0; oy < 3; ++oy) {
                const int jy = wrap_index(iy0 + oy, Ny);
                for (int ox = 0; ox < 3; ++ox) {
                    const int jx = wrap_index(ix0 + ox, Nx);
                    rho[(size_t)jy * Nx + jx] += qq * wx[ox] * wy[oy];
                }
            }
        }
    } else {
        for (size_t idx = b; idx < e; ++idx) {
            const int nxs = esirkepov_weights_1d(x[idx], x[idx] + vx[idx] * dt, dx, Nx, xs, ESK_CAP);
            const int nys = esirkepov_weights_1d(y[idx], y[idx] + vy[idx] * dt, dy, Ny, ys, ESK_CAP);
            for (int a = 0; a < nxs; ++a)
                for (int c = 0; c < nys; ++c)
                    rho[(size_t)ys[c].index * Nx + xs[a].index] += q[idx] * xs[a].weight * ys[c].weight * inv_vol;
        }
    }
}

/* depositCpuSoA dispatch (src/deposition/deposition.cpp:60-91) with the
 * privatised OpenMP form of parallelDepositPrivatized
 * (src/deposition/deposition_parallel.cpp:19-47): contiguous particle chunks,
 * one private full grid per thread, merged into rho. The merge runs in thread
 * order here so the result is reproducible (the reference merges in
 * `omp critical` arrival order). rho is cleared first (clearRho). */
int orc_deposit_ref(const orc_domain* d, int scheme, size_t n, const double* x, const double* y, const double* vx,
                    const double* vy, const double* q, double esirkepov_dt, int threads, double* rho) {
    const size_t g = (size_t)d->Nx * (size_t)d->Ny;
    memset(rho, 0, g * sizeof(double));
    if (threads <= 1) {
        esk_weight* xs = (esk_weight*)malloc(sizeof(esk_weight) * ESK_CAP);
        esk_weight* ys = (esk_weight*)malloc(sizeof(esk_weight) * ESK_CAP);
        deposit_range(d, scheme, 0, n, x, y, vx, vy, q, esirkepov_dt, 0, rho, xs, ys);
        free(xs);
        free(ys);
        return 0;
    }
#ifdef _OPENMP
    double** priv = (double**)calloc((size_t)threads, sizeof(double*));
    int used = threads;
#pragma omp parallel num_threads(threads)
    {
        const int tid = omp_get_thread_num();
        const int nth = omp_get_num_threads();
#pragma omp single
        used = nth;
        const size_t chunk = (n + (size_t)nth - 1) / (size_t)nth;
        const size_t b = (size_t)tid * chunk;
        const size_t e = b + chunk < n ? b + chunk : n;
        double* local = (double*)malloc(g * sizeof(double));
        for (size_t i = 0; i < g; ++i) local[i] = 0.0;
        esk_weight* xs = (esk_weight*)malloc(sizeof(esk_weight) * ESK_CAP);
        esk_weight* ys = (esk_weight*)malloc(sizeof(esk_weight) * ESK_CAP);
        if (b < e) deposit_range(d, scheme, b, e, x, y, vx, vy, q, esirkepov_dt, 1, local, xs, ys);
        free(xs);
        free(ys);
        priv[tid] = local;
#pragma omp barrier
#pragma omp for schedule(static)
        for (size_t i = 0; i < g; ++i) {
            double s = rho[i];
            for (int t = 0; t < nth; ++t) s += priv[t][i];
            rho[i] = s;
        }
    }
    for (int t = 0; t < used; ++t) free(priv[t]);
    free(priv);
    return 0;
#else
    (void)threads;
    return orc_deposit_ref(d, scheme, n, x, y, vx, vy, q, esirkepov_dt, 1, rho);
#endif
}

/* ======================================================================= */
/* stable cell sort: key = particleCellIndex (cell_sort.cpp:8-13). The     */
/* reference sorts with the unstable std::sort (cell_sort.cpp:22-46); the   */
/* GPU sort is stable, so its permutation is pinned by a stable counting    */
/* sort on the same keys, and the per-cell offsets by histogram + scan.     */
/* ======================================================================= */
/* depositChargeTimedSoA's timer (src/deposition/deposition.cpp:257-310): `warmups`
 * untimed deposits, then `repeats` timed ones (each clears rho and deposits, as
 * depositKernelSoA does); returns the mean deposit time in ms in *mean_ms. */
int orc_deposit_timed(const orc_domain* d, int scheme, size_t n, const double* x, const double* y, const double* vx,
                      const double* vy, const double* q, double esirkepov_dt, int threads, int warmups, int repeats,
                      double* rho, double* mean_ms) {
    for (int i = 0; i < warmups; ++i)
        if (orc_deposit_ref(d, scheme, n, x, y, vx, vy, q, esirkepov_dt, threads, rho) != 0) return -1;
    double sum = 0.0;
    for (int i = 0; i < repeats; ++i) {
        struct timespec a, b;
        clock_gettime(CLOCK_MONOTONIC, &a);
        if (orc_deposit_ref(d, scheme, n, x, y, vx, vy, q, esirkepov_dt, threads, rho) != 0) return -1;
        clock_gettime(CLOCK_MONOTONIC, &b);
        sum += (double)(b.tv_sec - a.tv_sec) * 1e3 + (double)(b.tv_nsec - a.tv_nsec) * 1e-6;
    }
    if (mean_ms) *mean_ms = repeats > 0 ? sum / repeats : 0.0;
    return 0;
}

int orc_stable_sort_keys(size_t n, uint32_t nkeys, const uint32_t* keys, uint32_t* keys_sorted, uint32_t* perm,
                         uint32_t* offsets) {
    uint32_t* cursor = (uint32_t*)calloc((size_t)nkeys + 1, sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) {
        if (keys[i] >= nkeys) {
            free(cursor);
            return -1;
        }
        cursor[keys[i] + 1]++;
    }
    for (uint32_t c = 0; c < nkeys; ++c) cursor[c + 1] += cursor[c];
    if (offsets) memcpy(offsets, cursor, ((size_t)nkeys + 1) * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) {
        const uint32_t pos = cursor[keys[i]]++;
        if (perm) perm[pos] = (uint32_t)i;
        if (keys_sorted) keys_sorted[pos] = keys[i];
    }
    free(cursor);
    return 0;
}

int orc_stable_cell_sort(const orc_domain* d, size_t n, const double* x, const double* y, uint32_t* keys_sorted,
                         uint32_t* perm, uint32_t* offsets) {
    uint32_t* keys = (uint32_t*)malloc((n ? n : 1) * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) keys[i] = (uint32_t)orc_particle_cell_index(d, x[i], y[i]);
    const int rc = orc_stable_sort_keys(n, (uint32_t)d->Nx * (uint32_t)d->Ny, keys, keys_sorted, perm, offsets);
    free(keys);
    return rc;
}

/* ======================================================================= */
/* FP64 gather / push                                                       */
/* ======================================================================= */

/* gatherFieldsSoA, src/deposition/deposition.cpp:335-356 */
void orc_gather_ref(const orc_domain* d, size_t n, const double* x, const double* y, double* vx, double* vy,
                    const double* q, const double* m, const double* Ex, const double* Ey, double dt) {
    const int Nx = d->Nx, Ny = d->Ny;
    for (size_t i = 0; i < n; ++i) {
        int ix, iy;
        double wx, wy;
        orc_cell_coords(d, x[i], y[i], &ix, &iy, &wx, &wy);
        const int ixp = (ix + 1) % Nx;
        const int iyp = (iy + 1) % Ny;
        const size_t i00 = (size_t)iy * Nx + ix, i10 = (size_t)iy * Nx + ixp;
        const size_t i01 = (size_t)iyp * Nx + ix, i11 = (size_t)iyp * Nx + ixp;
        const double ex = Ex[i00] * (1.0 - wx) * (1.0 - wy) + Ex[i10] * wx * (1.0 - wy) + Ex[i01] * (1.0 - wx) * wy +
                          Ex[i11] * wx * wy;
        const double ey = Ey[i00] * (1.0 - wx) * (1.0 - wy) + Ey[i10] * wx * (1.0 - wy) + Ey[i01] * (1.0 - wx) * wy +
                          Ey[i11] * wx * wy;
        const double mm = m ? m[i] : 1.0;
        vx[i] += -q[i] / mm * ex * dt;
        vy[i] += -q[i] / mm * ey * dt;
    }
}

/* pushParticlesSoA + Domain::wrapPosition, deposition.cpp:367-374, domain.hpp:27-32 */
void orc_push_ref(const orc_domain* d, size_t n, double* x, double* y, const double* vx, const double* vy, double dt) {
    for (size_t i = 0; i < n; ++i) {
        x[i] += vx[i] * dt;
        y[i] += vy[i] * dt;
        x[i] = fmod(x[i], d->Lx);
        if (x[i] < 0.0) x[i] += d->Lx;
        y[i] = fmod(y[i], d->Ly);
        if (y[i] < 0.0) y[i] += d->Ly;
    }
}

/* ======================================================================= */
/* Poisson                                                                  */
/* ======================================================================= */

/* forward-difference E, src/pic/poisson_gs.cpp:48-60 (same as poisson_fft.cpp:77-93) */
void orc_efield(const orc_domain* d, const double* phi, double* Ex, double* Ey) {
    const int nx = d->Nx, ny = d->Ny;
    const double idx_dx = 1.0 / dom_dx(d);
    const double idx_dy = 1.0 / dom_dy(d);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int ip = (i + 1) % nx;
            const int jp = (j + 1) % ny;
            const size_t id = (size_t)j * nx + i;
            Ex[id] = -(phi[(size_t)j * nx + ip] - phi[id]) * idx_dx;
            Ey[id] = -(phi[(size_t)jp * nx + i] - phi[id]) * idx_dy;
        }
}

/* PoissonSolverGS::solve, src/pic/poisson_gs.cpp:11-61: lexicographic,
 * phi zeroed each call, stop on max|dphi| < tol. Returns the sweep count. */
int orc_gs_ref(const orc_domain* d, const double* rho, int max_iters, double tol, double* phi, double* Ex,
               double* Ey) {
    const int nx = d->Nx, ny = d->Ny;
    const double dx = dom_dx(d), dy = dom_dy(d);
    const double dx2 = dx * dx, dy2 = dy * dy;
    const double denom = 2.0 * (1.0 / dx2 + 1.0 / dy2);
    const double scale = dx * dy;
    memset(phi, 0, (size_t)nx * ny * sizeof(double));
    int it = 0;
    for (; it < max_iters; ++it) {
        double max_delta = 0.0;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int im = (i - 1 + nx) % nx, ip = (i + 1) % nx;
                const int jm = (j - 1 + ny) % ny, jp = (j + 1) % ny;
                const size_t id = (size_t)j * nx + i;
                const double nphi = ((phi[(size_t)j * nx + im] + phi[(size_t)j * nx + ip]) / dx2 +
                                     (phi[(size_t)jm * nx + i] + phi[(size_t)jp * nx + i]) / dy2 + rho[id] * scale) /
                                    denom;
                const double dd = fabs(nphi - phi[id]);
                if (dd > max_delta) max_delta = dd;
                phi[id] = nphi;
            }
        if (max_delta < tol) {
            ++it;
            break;
        }
    }
    orc_efield(d, phi, Ex, Ey);
    return it;
}

/* Red-black Gauss-Seidel (new; no reference implementation). The stencil and
 * sign are those of poisson_gs.cpp:32-38 with right-hand side b = rho*dV - mean.
 * A sweep updates all points with (i+j) even, then all with (i+j) odd.
 * ||b - A phi||_2 / ||b||_2 is checked every `check_every` sweeps; on exit phi
 * has its mean removed. Requires even Nx and Ny. */
static double* rbgs_rhs(const orc_domain* d, const double* rho) {
    const size_t g = (size_t)d->Nx * d->Ny;
    const double scale = dom_dx(d) * dom_dy(d);
    double* b = (double*)calloc(g ? g : 1, sizeof(double));
    if (!b) return NULL;
    double s = 0.0;
    for (size_t i = 0; i < g; ++i) {
        b[i] = rho[i] * scale;
        s += b[i];
    }
    const double mean = s / (double)g;
    for (size_t i = 0; i < g; ++i) b[i] -= mean;
    return b;
}

double orc_rbgs_residual(const orc_domain* d, const double* b, const double* phi) {
    const int nx = d->Nx, ny = d->Ny;
    const double dx = dom_dx(d), dy = dom_dy(d);
    const double dx2 = dx * dx, dy2 = dy * dy;
    const double denom = 2.0 * (1.0 / dx2 + 1.0 / dy2);
    const double ix2 = 1.0 / dx2, iy2 = 1.0 / dy2;
    double rr = 0.0, bb = 0.0;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int im = (i - 1 + nx) % nx, ip = (i + 1) % nx;
            const int jm = (j - 1 + ny) % ny, jp = (j + 1) % ny;
            const size_t id = (size_t)j * nx + i;
            const double we = phi[(size_t)j * nx + im] + phi[(size_t)j * nx + ip];
            const double sn = phi[(size_t)jm * nx + i] + phi[(size_t)jp * nx + i];
            const double ap = (denom * phi[id] - we * ix2) - sn * iy2;
            const double r = b[id] - ap;
            rr += r * r;
            bb += b[id] * b[id];
        }
    return bb > 0.0 ? sqrt(rr / bb) : sqrt(rr);
}

int orc_rbgs(const orc_domain* d, const double* rho, double* phi, double tol, int max_iters, int check_every,
             int* iters_out, double* resid_out) {
    const int nx = d->Nx, ny = d->Ny;
    if ((nx & 1) || (ny & 1)) return -1;
    const double dx = dom_dx(d), dy = dom_dy(d);
    const double dx2 = dx * dx, dy2 = dy * dy;
    const double ix2 = 1.0 / dx2, iy2 = 1.0 / dy2;
    const double denom = 2.0 * (1.0 / dx2 + 1.0 / dy2);
    const double inv_denom = 1.0 / denom;
    double* b = rbgs_rhs(d, rho);
    if (!b) return -2;
    if (check_every < 1) check_every = 1;
    double res = orc_rbgs_residual(d, b, phi);
    int it = 0;
    while (it < max_iters && !(res <= tol)) {
        /* multiplications by 1/dx^2, 1/dy^2, 1/denom, in the GPU kernel's order */
        for (int color = 0; color < 2; ++color)
            for (int j = 0; j < ny; ++j)
                for (int i = (j + color) & 1; i < nx; i += 2) {
                    const int im = (i - 1 + nx) % nx, ip = (i + 1) % nx;
                    const int jm = (j - 1 + ny) % ny, jp = (j + 1) % ny;
                    const size_t id = (size_t)j * nx + i;
                    const double we = phi[(size_t)j * nx + im] + phi[(size_t)j * nx + ip];
                    const double sn = phi[(size_t)jm * nx + i] + phi[(size_t)jp * nx + i];
                    phi[id] = ((we * ix2 + sn * iy2) + b[id]) * inv_denom;
                }
        ++it;
        if (it % check_every == 0 || it == max_iters) res = orc_rbgs_residual(d, b, phi);
    }
    const size_t g = (size_t)nx * ny;
    double s = 0.0;
    for (size_t i = 0; i < g; ++i) s += phi[i];
    const double mean = s / (double)g;
    for (size_t i = 0; i < g; ++i) phi[i] -= mean;
    if (iters_out) *iters_out = it;
    if (resid_out) *resid_out = res;
    free(b);
    return 0;
}

/* ======================================================================= */
/* FP64 sums                                                                */
/* ======================================================================= */

/* FieldGrid::integratedRho, src/pic/field_grid.cpp:24-30 */
double orc_integrated_rho(const orc_domain* d, const double* rho) {
    const size_t g = (size_t)d->Nx * d->Ny;
    double s = 0.0;
    for (size_t i = 0; i < g; ++i) s += rho[i];
    return s * (dom_dx(d) * dom_dy(d));
}

/* FieldGrid::fieldEnergy, src/pic/field_grid.cpp:32-38 */
double orc_field_energy(const orc_domain* d, const double* Ex, const double* Ey) {
    const size_t g = (size_t)d->Nx * d->Ny;
    double s = 0.0;
    for (size_t i = 0; i < g; ++i) s += Ex[i] * Ex[i] + Ey[i] * Ey[i];
    return 0.5 * s * (dom_dx(d) * dom_dy(d));
}

/* ParticlesSoA::kineticEnergy, src/pic/particles_aos.cpp:190-196 */
double orc_kinetic_energy(size_t n, const double* vx, const double* vy, const double* m) {
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s += 0.5 * (m ? m[i] : 1.0) * (vx[i] * vx[i] + vy[i] * vy[i]);
    return s;
}

/* chargeConservationError, src/pic/diagnostics.cpp:26-29 */
double orc_charge_error(double integrated_rho, double total_charge, double abs_charge_sum) {
    const double den = abs_charge_sum > 1e-12 ? abs_charge_sum : 1e-12;
    return fabs(integrated_rho - total_charge) / den;
}

/* ======================================================================= */
/* Restatement of the GPU data layout and fixed-point deposit.              */
/*                                                                          */
/* Layout: per particle the cell key iy*Nx+ix (from the FP64 cellCoords    */
/* above, so keys equal the reference's) and the in-cell offsets           */
/* xr = (float)wx, yr = (float)wy in [0,1]. An offset just below 0.5 that  */
/* would round up to 0.5f is stored as the float just below 0.5, so the    */
/* NGP nearest-node choice (wx >= 0.5, ngp.cpp:116-117) is kept exactly.   */
/*                                                                          */
/* Fixed point. maxq = max |(float)q|, qn = (float)q / maxq (FP32 division), */
/* so |qn| <= 1 and a uniform |q| gives qn = +-1 exactly. a = qn * 2^24 and  */
/* A = rint(a) is the particle's charge in units. Every frame node gets      */
/* v = rint((a * Y[j]) * X[i]) (FP32 products, round to nearest even), then   */
/* one node gets A - (sum of the others), so a particle deposits exactly A    */
/* units and the grid's total charge is exact: for TSC the node of the        */
/* particle's own cell (frame offset 0, weight >= 1/64), otherwise the node   */
/* of largest weight (first maximum of X and of Y). Sums are int64.           */
/* unit = ((double)maxq * inv_vol) * 2^-24; rho = acc * unit + background.   */
/* TSC with one charge for every particle uses exact integer weights        */
/* instead (tsc_int_frame below; unit 2^-30 of the particle's charge).      */
/* ======================================================================= */
void orc_to_device(const orc_domain* d, size_t n, const double* x, const double* y, uint32_t* cell, float* xr,
                   float* yr) {
    for (size_t i = 0; i < n; ++i) {
        int ix, iy;
        double wx, wy;
        orc_cell_coords(d, x[i], y[i], &ix, &iy, &wx, &wy);
        float fx = (float)wx, fy = (float)wy;
        if (wx < 0.5 && fx >= 0.5f) fx = 0.49999997f;
        if (wy < 0.5 && fy >= 0.5f) fy = 0.49999997f;
        cell[i] = (uint32_t)(iy * d->Nx + ix);
        xr[i] = fx;
        yr[i] = fy;
    }
}

void orc_normalize_charge(size_t n, const double* q, float* qn, float* maxq_out) {
    float mq = 0.0f;
    for (size_t i = 0; i < n; ++i) {
        const float a = fabsf((float)q[i]);
        if (a > mq) mq = a;
    }
    for (size_t i = 0; i < n; ++i) qn[i] = mq > 0.0f ? (float)q[i] / mq : 0.0f;
    if (maxq_out) *maxq_out = mq;
}

static inline int32_t fixed_rn(float v) { return (int32_t)lrintf(v); }

/* Frames of stencil weights relative to the particle's cell: X[i] belongs
 * to node ix + i + x_lo. Returns the frame length. */
static int frame_ngp(float r, float* X, int* lo) {
    *lo = 0;
    X[0] = r >= 0.5f ? 0.0f : 1.0f;
    X[1] = r >= 0.5f ? 1.0f : 0.0f;
    return 2;
}

static int frame_cic(float r, float* X, int* lo) {
    *lo = 0;
    X[0] = 1.0f - r;
    X[1] = r;
    return 2;
}

static int frame_tsc(float r, float* X, int* lo) {
    *lo = -1;
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
    return 4;
}

/* Trajectory-averaged weights (the reference's "Esirkepov" rho,
 * ngp.cpp:36-84) in cell-relative FP32: path r -> r + dc (dc = v*dt/dx),
 * split at integer boundaries, each piece weighted by its length over the
 * total path. `dphys` = v*dt decides the static case (|dphys| < 1e-15 gives
 * CIC weights). The fast frame covers |dc| < 1 (lo = -1, 3 nodes); larger
 * moves return -1 and are deposited by the general loop. */
static int frame_esk(float r, float dc, float dphys, float* X, int* lo) {
    *lo = -1;
    if (fabsf(dphys) < 1e-15f) {
        X[0] = 0.0f;
        X[1] = 1.0f - r;
        X[2] = r;
        return 3;
    }
    if (!(fabsf(dc) < 1.0f)) return -1;
    const float e = r + dc;
    if (dc > 0.0f) {
        if (e > 1.0f) {
            const float wb = (e - 1.0f) / (e - r);
            X[0] = 0.0f;
            X[1] = 1.0f - wb;
            X[2] = wb;
        } else {
            X[0] = 0.0f;
            X[1] = 1.0f;
            X[2] = 0.0f;
        }
    } else {
        if (e < 0.0f) {
            const float wl = (0.0f - e) / (r - e);
            X[0] = wl;
            X[1] = 1.0f - wl;
            X[2] = 0.0f;
        } else {
            X[0] = 0.0f;
            X[1] = 1.0f;
            X[2] = 0.0f;
        }
    }
    return 3;
}

/* General trajectory split for |dc| >= 1: writes (cell offset, weight)
 * pairs, weights = piece length / total path length. */
static int esk_general(float r, float dc, int* off, float* w, int cap) {
    const float e = r + dc;
    int cnt = 0;
    if (dc > 0.0f) {
        const float tot = e - r;
        float s = r;
        int c = 0;
        while (s < e && cnt < cap) {
            const float b = (float)(c + 1);
            const float nx = e < b ? e : b;
            off[cnt] = c;
            w[cnt] = (nx - s) / tot;
            ++cnt;
            s = nx;
            ++c;
        }
    } else {
        const float tot = r - e;
        float s = r;
        int c = 0;
        while (s > e && cnt < cap) {
            const float b = (float)c;
            const float nx = e > b ? e : b;
            off[cnt] = c;
            w[cnt] = (s - nx) / tot;
            ++cnt;
            s = nx;
            --c;
        }
    }
    return cnt;
}

#define ESK_GEN_CAP 256

static int first_max(const float* X, int n) {
    int m = 0;
    for (int i = 1; i < n; ++i)
        if (X[i] > X[m]) m = i;
    return m;
}

/* ----------------------------------------------------------------------- */
/* One charge for every particle (every stored qn bitwise equal, nonzero and */
/* finite: the device's upload test), TSC: exact integer weights. Per axis,  */
/* with t = r (r < 0.5) or r - 1 (r >= 0.5) as in tscWeights (ngp.cpp:28-34) */
/* written relative to the cell,                                            */
/*   WL = rint(2^14 (0.5 - t)^2) = rint(2^15 * 0.5 (0.5 - t)^2)             */
/*   WR = rint(2^14 (0.5 + t)^2)                                            */
/* each one FP32 fma (dl * (dl * 2^14) + 1.5*2^23: the product is exact and */
/* the sum rounds once, to the nearest even integer), WC = 2^15 - WL - WR.  */
/* The frame value of node (i, j) is WX[i] * WY[j], an exact integer; a     */
/* particle deposits exactly 2^30 units and the charge sign sits in the     */
/* unit: unit = ((double)maxq * inv_vol) * (qn * 2^-30).                    */
/* ----------------------------------------------------------------------- */
#define TSCI_ONE 32768
static void tsc_int_frame(float r, int64_t W[4]) {
    const int s = r >= 0.5f;
    const float t = s ? r - 1.0f : r;
    const float dl = 0.5f - t, dr = 0.5f + t;
    const float fl = fmaf(dl, dl * 16384.0f, 12582912.0f);
    const float fr = fmaf(dr, dr * 16384.0f, 12582912.0f);
    const int64_t wl = (int64_t)(fl - 12582912.0f), wr = (int64_t)(fr - 12582912.0f);
    const int64_t wc = TSCI_ONE - wl - wr;
    W[0] = s ? 0 : wl;
    W[1] = s ? wl : wc;
    W[2] = s ? wc : wr;
    W[3] = s ? wr : 0;
}

/* Nonzero when every qn equals the first, which is nonzero and finite. */
int orc_charge_uniform(size_t n, const float* qn) {
    if (n == 0 || !(qn[0] != 0.0f) || !isfinite(qn[0])) return 0;
    for (size_t p = 1; p < n; ++p)
        if (!(qn[p] == qn[0])) return 0;
    return 1;
}

int orc_deposit_fixed(const orc_domain* d, int scheme, size_t n, const uint32_t* cell, const float* xr,
                      const float* yr, const float* vx, const float* vy, const float* qn, float maxq, double dt,
                      int64_t* acc, double* unit_out) {
    const int Nx = d->Nx, Ny = d->Ny;
    const size_t g = (size_t)Nx * Ny;
    memset(acc, 0, g * sizeof(int64_t));
    const double inv_vol = 1.0 / (dom_dx(d) * dom_dy(d));
    if (scheme == ORC_TSC && orc_charge_uniform(n, qn)) {
        if (unit_out) *unit_out = ((double)maxq * inv_vol) * ((double)qn[0] * 0x1p-30);
        for (size_t p = 0; p < n; ++p) {
            const int ix = (int)(cell[p] % (uint32_t)Nx);
            const int iy = (int)(cell[p] / (uint32_t)Nx);
            int64_t X[4], Y[4];
            tsc_int_frame(xr[p], X);
            tsc_int_frame(yr[p], Y);
            for (int j = 0; j < 4; ++j) {
                const size_t row = (size_t)wrap_index(iy - 1 + j, Ny) * Nx;
                for (int i = 0; i < 4; ++i) acc[row + wrap_index(ix - 1 + i, Nx)] += X[i] * Y[j];
            }
        }
        return 0;
    }
    if (unit_out) *unit_out = ((double)maxq * inv_vol) * 5.9604644775390625e-08;
    const float dtf = (float)dt;
    const float dtdx = (float)(dt / dom_dx(d));
    const float dtdy = (float)(dt / dom_dy(d));
    for (size_t p = 0; p < n; ++p) {
        const int ix = (int)(cell[p] % (uint32_t)Nx);
        const int iy = (int)(cell[p] / (uint32_t)Nx);
        const float a = qn[p] * 16777216.0f;
        const int64_t A = fixed_rn(a);
        float X[4], Y[4];
        int xlo = 0, ylo = 0, nxf = 0, nyf = 0;
        if (scheme == ORC_NGP) {
            nxf = frame_ngp(xr[p], X, &xlo);
            nyf = frame_ngp(yr[p], Y, &ylo);
        } else if (scheme == ORC_CIC) {
            nxf = frame_cic(xr[p], X, &xlo);
            nyf = frame_cic(yr[p], Y, &ylo);
        } else if (scheme == ORC_TSC) {
            nxf = frame_tsc(xr[p], X, &xlo);
            nyf = frame_tsc(yr[p], Y, &ylo);
        } else if (scheme == ORC_ESIRKEPOV) {
            nxf = frame_esk(xr[p], vx[p] * dtdx, vx[p] * dtf, X, &xlo);
            nyf = frame_esk(yr[p], vy[p] * dtdy, vy[p] * dtf, Y, &ylo);
            if (nxf < 0 || nyf < 0) {
                /* general path: per-axis lists (static axis = CIC pair) */
                int ox[ESK_GEN_CAP], oy[ESK_GEN_CAP];
                float wx[ESK_GEN_CAP], wy[ESK_GEN_CAP];
                int cx, cy;
                if (fabsf(vx[p] * dtf) < 1e-15f) {
                    ox[0] = 0; wx[0] = 1.0f - xr[p]; ox[1] = 1; wx[1] = xr[p]; cx = 2;
                } else {
                    cx = esk_general(xr[p], vx[p] * dtdx, ox, wx, ESK_GEN_CAP);
                }
                if (fabsf(vy[p] * dtf) < 1e-15f) {
                    oy[0] = 0; wy[0] = 1.0f - yr[p]; oy[1] = 1; wy[1] = yr[p]; cy = 2;
                } else {
                    cy = esk_general(yr[p], vy[p] * dtdy, oy, wy, ESK_GEN_CAP);
                }
                const int mx = first_max(wx, cx), my = first_max(wy, cy);
                int64_t others = 0;
                for (int j = 0; j < cy; ++j) {
                    const float ay = a * wy[j];
                    for (int i = 0; i < cx; ++i)
                        if (i != mx || j != my) others += fixed_rn(ay * wx[i]);
                }
                for (int j = 0; j < cy; ++j) {
                    const float ay = a * wy[j];
                    const int gy = wrap_index(iy + oy[j], Ny);
                    for (int i = 0; i < cx; ++i) {
                        const int gx = wrap_index(ix + ox[i], Nx);
                        const int64_t v = (i == mx && j == my) ? A - others : (int64_t)fixed_rn(ay * wx[i]);
                        acc[(size_t)gy * Nx + gx] += v;
                    }
                }
                continue;
            }
        } else {
            return -1;
        }
        /* TSC: the particle's own cell node (frame offset 0) */
        const int mx = scheme == ORC_TSC ? -xlo : first_max(X, nxf);
        const int my = scheme == ORC_TSC ? -ylo : first_max(Y, nyf);
        int64_t others = 0;
        for (int j = 0; j < nyf; ++j) {
            const float ay = a * Y[j];
            for (int i = 0; i < nxf; ++i)
                if (i != mx || j != my) others += fixed_rn(ay * X[i]);
        }
        for (int j = 0; j < nyf; ++j) {
            const float ay = a * Y[j];
            const int gy = wrap_index(iy + ylo + j, Ny);
            for (int i = 0; i < nxf; ++i) {
                const int gx = wrap_index(ix + xlo + i, Nx);
                const int64_t v = (i == mx && j == my) ? A - others : (int64_t)fixed_rn(ay * X[i]);
                acc[(size_t)gy * Nx + gx] += v;
            }
        }
    }
    return 0;
}

void orc_fixed_to_rho(size_t g, const int64_t* acc, double unit, double background, double* rho) {
    for (size_t i = 0; i < g; ++i) rho[i] = (double)acc[i] * unit + background;
}

/* ======================================================================= */
/* Restatement of the GPU's cell-relative FP32 gather / push               */
/* (gatherFieldsSoA / pushParticlesSoA, deposition.cpp:335-374, in the      */
/* device layout): E is read as FP32 copies of the FP64 fields,            */
/*   e = ((E00*(1-wx))*(1-wy) + (E10*wx)*(1-wy)) + (E01*(1-wx))*wy + (E11*wx)*wy */
/*   v = v + ((-q/m)*e)*dt,   r' = r + v*dt/dx, cell moves by floor(r').    */
/* ======================================================================= */
void orc_move_f32(const orc_domain* d, size_t n, uint32_t* cell, float* xr, float* yr, float* vx, float* vy,
                  const float* qn, float maxq, const float* m, const double* Ex, const double* Ey, double dt,
                  int gather, int push) {
    const int Nx = d->Nx, Ny = d->Ny;
    const float dtf = (float)dt;
    const float dtdx = (float)(dt / dom_dx(d));
    const float dtdy = (float)(dt / dom_dy(d));
    for (size_t p = 0; p < n; ++p) {
        int iy = (int)(cell[p] / (uint32_t)Nx);
        int ix = (int)(cell[p] - (uint32_t)iy * (uint32_t)Nx);
        float rx = xr[p], ry = yr[p];
        float vxx = vx[p], vyy = vy[p];
        if (gather) {
            const int ixp = (ix + 1) % Nx, iyp = (iy + 1) % Ny;
            const size_t i00 = (size_t)iy * Nx + ix, i10 = (size_t)iy * Nx + ixp;
            const size_t i01 = (size_t)iyp * Nx + ix, i11 = (size_t)iyp * Nx + ixp;
            const float omx = 1.0f - rx, omy = 1.0f - ry;
            const float ex = ((((float)Ex[i00] * omx) * omy + ((float)Ex[i10] * rx) * omy) +
                              ((float)Ex[i01] * omx) * ry) + ((float)Ex[i11] * rx) * ry;
            const float ey = ((((float)Ey[i00] * omx) * omy + ((float)Ey[i10] * rx) * omy) +
                              ((float)Ey[i01] * omx) * ry) + ((float)Ey[i11] * rx) * ry;
            const float qf = qn[p] * maxq;
            const float coef = m ? (-qf) / m[p] : -qf;
            vxx = vxx + (coef * ex) * dtf;
            vyy = vyy + (coef * ey) * dtf;
            vx[p] = vxx;
            vy[p] = vyy;
        }
        if (push) {
            float x = rx + vxx * dtdx;
            float s = floorf(x);
            rx = x - s;
            ix = wrap_index(ix + (int)s, Nx);
            x = ry + vyy * dtdy;
            s = floorf(x);
            ry = x - s;
            iy = wrap_index(iy + (int)s, Ny);
            xr[p] = rx;
            yr[p] = ry;
            cell[p] = (uint32_t)iy * (uint32_t)Nx + (uint32_t)ix;
        }
    }
}

/* ======================================================================= */
/* Esirkepov current (new; no reference implementation).                   */
/* First-order (CIC-shape) charge-conserving current of Esirkepov, Comput. */
/* Phys. Commun. 135 (2001) 144, in 2D: with S0, S1 the CIC weights of the */
/* old and new positions and DS = S1 - S0 on a 4-node frame (cell offsets  */
/* -1..2 around the old cell),                                             */
/*   W1[j][i] = DSx[i] (S0y[j] + DSy[j]/2),  W2[j][i] = DSy[j] (S0x[i] + DSx[i]/2) */
/*   Jx(i+1/2, j) = -q/dV dx/dt sum_{i'<=i} W1[j][i'],  Jy likewise in j.  */
/* (a) FP64 restatement: orc_esirkepov_j_ref.                              */
/* (b) restatement of the GPU fixed point: orc_esirkepov_j_fixed. Per       */
/*     particle, R0/R1 are the integer CIC charges of the old/new position  */
/*     (same rounding and remainder rule as the charge deposit), W1 is      */
/*     rounded with row sums forced to 0 and column sums forced to those of */
/*     R1-R0, W2 = (R1-R0) - W1, so (R1-R0) + div J = 0 holds exactly in    */
/*     integers. J unit = max|q| inv_vol 2^-24 dx/dt (x) or dy/dt (y).      */
/* Both require |v dt| < cell size on each axis.                           */
/* ======================================================================= */

/* S0 and DS = S1 - S0 on the 4-node frame from the in-cell offset r and the
 * displacement d (|d| < 1), each DS entry formed from quantities of its own
 * size (no cancellation of S1 - S0): no crossing DS = (0,-d,d,0); crossing
 * up (fr = r+d-1) DS = (0, r-1, (1-r)-fr, fr); crossing down (e = r+d < 0)
 * DS = (-e, r+e, -r, 0). */
static void esk_ds(float r, float d, float* s0, float* ds) {
    const float e = r + d;
    const float f = floorf(e);
    const float fr = e - f;
    s0[0] = 0.0f; s0[1] = 1.0f - r; s0[2] = r; s0[3] = 0.0f;
    if (f == 0.0f) {
        ds[0] = 0.0f; ds[1] = -d; ds[2] = d; ds[3] = 0.0f;
    } else if (f > 0.0f) {
        ds[0] = 0.0f; ds[1] = r - 1.0f; ds[2] = (1.0f - r) - fr; ds[3] = fr;
    } else {
        ds[0] = -e; ds[1] = r + e; ds[2] = -r; ds[3] = 0.0f;
    }
}

int orc_esirkepov_j_ref(const orc_domain* d, size_t n, const double* x, const double* y, const double* vx,
                        const double* vy, const double* q, double dt, double* jx, double* jy) {
    const int Nx = d->Nx, Ny = d->Ny;
    const double dx = dom_dx(d), dy = dom_dy(d);
    const double inv_vol = 1.0 / (dx * dy);
    const size_t g = (size_t)Nx * Ny;
    memset(jx, 0, g * sizeof(double));
    memset(jy, 0, g * sizeof(double));
    for (size_t p = 0; p < n; ++p) {
        int ix, iy;
        double rx, ry;
        orc_cell_coords(d, x[p], y[p], &ix, &iy, &rx, &ry);
        const double ddx = vx[p] * dt / dx, ddy = vy[p] * dt / dy;
        if (!(fabs(ddx) < 1.0 && fabs(ddy) < 1.0)) return -1;
        double S0x[4] = {0, 1 - rx, rx, 0}, S0y[4] = {0, 1 - ry, ry, 0};
        double S1x[4] = {0, 0, 0, 0}, S1y[4] = {0, 0, 0, 0};
        const double ex = rx + ddx, ey = ry + ddy;
        const int kx = (int)floor(ex) + 1, ky = (int)floor(ey) + 1;
        S1x[kx] = 1 - (ex - floor(ex));
        S1x[kx + 1] = ex - floor(ex);
        S1y[ky] = 1 - (ey - floor(ey));
        S1y[ky + 1] = ey - floor(ey);
        double DSx[4], DSy[4];
        for (int i = 0; i < 4; ++i) {
            DSx[i] = S1x[i] - S0x[i];
            DSy[i] = S1y[i] - S0y[i];
        }
        const double cx = q[p] * inv_vol * dx / dt, cy = q[p] * inv_vol * dy / dt;
        for (int j = 0; j < 4; ++j) {
            double cum = 0.0;
            for (int i = 0; i < 3; ++i) {
                cum += DSx[i] * (S0y[j] + 0.5 * DSy[j]);
                jx[(size_t)wrap_index(iy - 1 + j, Ny) * Nx + wrap_index(ix - 1 + i, Nx)] += -cx * cum;
            }
        }
        for (int i = 0; i < 4; ++i) {
            double cum = 0.0;
            for (int j = 0; j < 3; ++j) {
                cum += DSy[j] * (S0x[i] + 0.5 * DSx[i]);
                jy[(size_t)wrap_index(iy - 1 + j, Ny) * Nx + wrap_index(ix - 1 + i, Nx)] += -cy * cum;
            }
        }
    }
    return 0;
}

/* integer CIC charges of a particle on the 4x4 frame; node (k, k+1) per axis */
static void cic_frame_int(float a, int A, float rx, float ry, int kx, int ky, int64_t R[4][4]) {
    const float X[2] = {1.0f - rx, rx}, Y[2] = {1.0f - ry, ry};
    int v[2][2], sum = 0;
    for (int j = 0; j < 2; ++j) {
        const float ay = a * Y[j];
        for (int i = 0; i < 2; ++i) {
            v[j][i] = fixed_rn(ay * X[i]);
            sum += v[j][i];
        }
    }
    const int mx = X[1] > X[0] ? 1 : 0, my = Y[1] > Y[0] ? 1 : 0;
    v[my][mx] += A - sum;
    for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 4; ++i) R[j][i] = 0;
    for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) R[ky + j][kx + i] = v[j][i];
}

int orc_esirkepov_j_fixed(const orc_domain* d, size_t n, const uint32_t* cell, const float* xr, const float* yr,
                          const float* vx, const float* vy, const float* qn, float maxq, double dt, int64_t* jx,
                          int64_t* jy, double* unit_x, double* unit_y) {
    const int Nx = d->Nx, Ny = d->Ny;
    const size_t g = (size_t)Nx * Ny;
    memset(jx, 0, g * sizeof(int64_t));
    memset(jy, 0, g * sizeof(int64_t));
    const double dx = dom_dx(d), dy = dom_dy(d);
    const double inv_vol = 1.0 / (dx * dy);
    const double unit = ((double)maxq * inv_vol) * 5.9604644775390625e-08;
    if (unit_x) *unit_x = unit * (dx / dt);
    if (unit_y) *unit_y = unit * (dy / dt);
    const float dtdx = (float)(dt / dx), dtdy = (float)(dt / dy);
    for (size_t p = 0; p < n; ++p) {
        const int ix = (int)(cell[p] % (uint32_t)Nx), iy = (int)(cell[p] / (uint32_t)Nx);
        const float ddx = vx[p] * dtdx, ddy = vy[p] * dtdy;
        if (!(fabsf(ddx) < 1.0f && fabsf(ddy) < 1.0f)) return -1;
        float s0x[4], dsx[4], s0y[4], dsy[4];
        esk_ds(xr[p], ddx, s0x, dsx);
        esk_ds(yr[p], ddy, s0y, dsy);
        const float a = qn[p] * 16777216.0f;
        const int A = fixed_rn(a);
        /* old / new integer charges */
        int64_t R0[4][4], R1[4][4];
        cic_frame_int(a, A, xr[p], yr[p], 1, 1, R0);
        const float ex = xr[p] + ddx, ey = yr[p] + ddy;
        const float fx = floorf(ex), fy = floorf(ey);
        cic_frame_int(a, A, ex - fx, ey - fy, (int)fx + 1, (int)fy + 1, R1);
        int64_t dR[4][4], W1[4][4], colR[4] = {0, 0, 0, 0};
        for (int j = 0; j < 4; ++j)
            for (int i = 0; i < 4; ++i) {
                dR[j][i] = R1[j][i] - R0[j][i];
                colR[i] += dR[j][i];
            }
        for (int j = 0; j < 3; ++j) {
            const float ay = a * (s0y[j] + 0.5f * dsy[j]);
            int64_t row = 0;
            for (int i = 0; i < 3; ++i) {
                W1[j][i] = fixed_rn(ay * dsx[i]);
                row += W1[j][i];
            }
            W1[j][3] = -row;
        }
        for (int i = 0; i < 4; ++i) {
            int64_t col = 0;
            for (int j = 0; j < 3; ++j) col += W1[j][i];
            W1[3][i] = colR[i] - col;
        }
        for (int j = 0; j < 4; ++j) {
            int64_t cum = 0;
            for (int i = 0; i < 3; ++i) {
                cum += W1[j][i];
                jx[(size_t)wrap_index(iy - 1 + j, Ny) * Nx + wrap_index(ix - 1 + i, Nx)] -= cum;
            }
        }
        for (int i = 0; i < 4; ++i) {
            int64_t cum = 0;
            for (int j = 0; j < 3; ++j) {
                cum += dR[j][i] - W1[j][i];
                jy[(size_t)wrap_index(iy - 1 + j, Ny) * Nx + wrap_index(ix - 1 + i, Nx)] -= cum;
            }
        }
    }
    return 0;
}
