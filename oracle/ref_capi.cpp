// C entry points over the reference's own C++ API (ehocine/pic-deposition).
//
// Test infrastructure only. oracle/Makefile compiles this file together with
// the reference's unmodified sources (src/deposition, src/sorting, src/pic)
// into oracle/_ref/libpicref.so; nothing here re-implements an algorithm, it
// only marshals flat arrays into pic::ParticlesSoA / pic::FieldGrid and calls
// the reference functions:
//   pic::depositChargeSoA / depositChargeTimedSoA  src/deposition/deposition.cpp:181-200, 257-310
//   pic::sortParticlesByCell / particleCellIndex   src/sorting/cell_sort.cpp:8-46
//   pic::gatherFieldsSoA / pushParticlesSoA        src/deposition/deposition.cpp:335-374
//   pic::PoissonSolverGS / PoissonSolverFFT        src/pic/poisson_gs.cpp:11-61, src/pic/poisson_fft.cpp:45-94
//   pic::spectralNoiseLevel                        src/pic/diagnostics.cpp:53-102
//   pic::ParticlesSoA initialisers                 src/pic/particles_aos.cpp:67-180
//   pic::Simulation::run                           src/pic/simulation.cpp:69-145
//   pic::runLangmuirValidation                     src/pic/validation.cpp:200-261
#include "deposition/deposition.hpp"
#include "pic/diagnostics.hpp"
#include "pic/poisson_fft.hpp"
#include "pic/simulation.hpp"
#include "pic/validation.hpp"
#include "sorting/cell_sort.hpp"

#include <cstring>
#include <exception>

namespace {

pic::Domain makeDomain(int nx, int ny, double lx, double ly) {
    pic::Domain d;
    d.Nx = nx;
    d.Ny = ny;
    d.Lx = lx;
    d.Ly = ly;
    d.updateDerived();
    return d;
}

void loadParticles(pic::ParticlesSoA& p, std::size_t n, const double* x, const double* y, const double* vx,
                   const double* vy, const double* q, const double* m) {
    p.resize(n);
    for (std::size_t i = 0; i < n; ++i) {
        p.x()[i] = x[i];
        p.y()[i] = y[i];
        p.vx()[i] = vx ? vx[i] : 0.0;
        p.vy()[i] = vy ? vy[i] : 0.0;
        p.q()[i] = q[i];
        p.m()[i] = m ? m[i] : 1.0;
    }
}

void storeParticles(const pic::ParticlesSoA& p, double* x, double* y, double* vx, double* vy, double* q, double* m) {
    const std::size_t n = p.size();
    if (x) std::memcpy(x, p.x().data(), n * sizeof(double));
    if (y) std::memcpy(y, p.y().data(), n * sizeof(double));
    if (vx) std::memcpy(vx, p.vx().data(), n * sizeof(double));
    if (vy) std::memcpy(vy, p.vy().data(), n * sizeof(double));
    if (q) std::memcpy(q, p.q().data(), n * sizeof(double));
    if (m) std::memcpy(m, p.m().data(), n * sizeof(double));
}

pic::DepositionScheme schemeOf(int s) {
    switch (s) {
        case 0:
            return pic::DepositionScheme::NGP;
        case 1:
            return pic::DepositionScheme::CIC;
        case 2:
            return pic::DepositionScheme::TSC;
        default:
            return pic::DepositionScheme::Esirkepov;
    }
}

}  // namespace

extern "C" {

// kind: 0 uniform Maxwellian (p0 = T), 1 cold Langmuir (p0 = amplitude, mode),
//       2 warm Langmuir (p0 = amplitude, mode, p1 = temperature),
//       3 two-stream (p0 = beam velocity, p1 = perturbation),
//       4 quasi-1D two-stream (p0, p1 as 3).
int ref_init_particles(int kind, int nx, int ny, double lx, double ly, std::size_t n, double p0, double p1, int mode,
                       unsigned seed, double* x, double* y, double* vx, double* vy, double* q, double* m) {
    try {
        const pic::Domain d = makeDomain(nx, ny, lx, ly);
        pic::ParticlesSoA p(n);
        switch (kind) {
            case 0:
                p.initializeUniformMaxwellian(d, p0, seed);
                break;
            case 1:
                p.initializeLangmuirWave(d, p0, mode, seed);
                break;
            case 2:
                p.initializeWarmLangmuirWave(d, p0, mode, p1, seed);
                break;
            case 3:
                p.initializeTwoStream(d, p0, p1, seed);
                break;
            case 4:
                p.initializeTwoStreamQuasi1D(d, p0, p1, seed);
                break;
            default:
                return -1;
        }
        storeParticles(p, x, y, vx, vy, q, m);
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

int ref_cell_index(int nx, int ny, double lx, double ly, double x, double y) {
    return pic::particleCellIndex(x, y, makeDomain(nx, ny, lx, ly));
}

int ref_deposit(int nx, int ny, double lx, double ly, int scheme, int sorted, int threads, double esirkepov_dt,
                std::size_t n, const double* x, const double* y, const double* vx, const double* vy, const double* q,
                const double* m, double* rho_out) {
    try {
        const pic::Domain d = makeDomain(nx, ny, lx, ly);
        pic::ParticlesSoA p;
        loadParticles(p, n, x, y, vx, vy, q, m);
        pic::FieldGrid grid(d);
        pic::DepositionConfig cfg;
        cfg.scheme = schemeOf(scheme);
        cfg.layout = pic::ParticleLayout::SoA;
        cfg.backend = pic::DepositionBackend::CPU;
        cfg.sorted = sorted != 0;
        cfg.num_threads = threads;
        cfg.esirkepov_dt = esirkepov_dt;
        pic::depositChargeSoA(p, grid, cfg);
        std::memcpy(rho_out, grid.rho().data(), grid.rho().size() * sizeof(double));
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

// stats_out[0..5] = sort_ms, deposit_ms, deposit_std_ms, throughput, bandwidth_gbs, charge_error
int ref_deposit_timed(int nx, int ny, double lx, double ly, int scheme, int sorted, int threads, double esirkepov_dt,
                      int repeats, std::size_t n, const double* x, const double* y, const double* vx,
                      const double* vy, const double* q, const double* m, double* stats_out) {
    try {
        const pic::Domain d = makeDomain(nx, ny, lx, ly);
        pic::ParticlesSoA p;
        loadParticles(p, n, x, y, vx, vy, q, m);
        pic::FieldGrid grid(d);
        pic::DepositionConfig cfg;
        cfg.scheme = schemeOf(scheme);
        cfg.layout = pic::ParticleLayout::SoA;
        cfg.sorted = sorted != 0;
        cfg.num_threads = threads;
        cfg.esirkepov_dt = esirkepov_dt;
        const pic::DepositionStats s = pic::depositChargeTimedSoA(p, grid, cfg, repeats);
        stats_out[0] = s.sort_ms;
        stats_out[1] = s.deposit_ms;
        stats_out[2] = s.deposit_std_ms;
        stats_out[3] = s.throughput_particles_per_s;
        stats_out[4] = s.effective_bandwidth_gbs;
        stats_out[5] = s.charge_error;
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

// Sorts the six arrays in place with the reference's (unstable) std::sort.
int ref_sort(int nx, int ny, double lx, double ly, std::size_t n, double* x, double* y, double* vx, double* vy,
             double* q, double* m) {
    try {
        const pic::Domain d = makeDomain(nx, ny, lx, ly);
        pic::ParticlesSoA p;
        loadParticles(p, n, x, y, vx, vy, q, m);
        pic::sortParticlesByCell(p, d);
        storeParticles(p, x, y, vx, vy, q, m);
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

int ref_gather(int nx, int ny, double lx, double ly, std::size_t n, const double* x, const double* y, double* vx,
               double* vy, const double* q, const double* m, const double* ex, const double* ey, double dt) {
    const pic::Domain d = makeDomain(nx, ny, lx, ly);
    pic::ParticlesSoA p;
    loadParticles(p, n, x, y, vx, vy, q, m);
    pic::FieldGrid grid(d);
    std::memcpy(grid.Ex().data(), ex, grid.Ex().size() * sizeof(double));
    std::memcpy(grid.Ey().data(), ey, grid.Ey().size() * sizeof(double));
    pic::gatherFieldsSoA(p, grid, dt);
    storeParticles(p, nullptr, nullptr, vx, vy, nullptr, nullptr);
    return 0;
}

int ref_push(int nx, int ny, double lx, double ly, std::size_t n, double* x, double* y, const double* vx,
             const double* vy, double dt) {
    const pic::Domain d = makeDomain(nx, ny, lx, ly);
    pic::ParticlesSoA p;
    loadParticles(p, n, x, y, vx, vy, vx, nullptr);
    pic::FieldGrid grid(d);
    pic::pushParticlesSoA(p, grid, dt);
    storeParticles(p, x, y, nullptr, nullptr, nullptr, nullptr);
    return 0;
}

int ref_poisson_gs(int nx, int ny, double lx, double ly, const double* rho, int max_iters, double tol, double* phi,
                   double* ex, double* ey) {
    const pic::Domain d = makeDomain(nx, ny, lx, ly);
    pic::FieldGrid grid(d);
    std::memcpy(grid.rho().data(), rho, grid.rho().size() * sizeof(double));
    pic::PoissonSolverGS solver(d, max_iters, tol);
    solver.solve(grid);
    std::memcpy(phi, grid.phi().data(), grid.phi().size() * sizeof(double));
    std::memcpy(ex, grid.Ex().data(), grid.Ex().size() * sizeof(double));
    std::memcpy(ey, grid.Ey().data(), grid.Ey().size() * sizeof(double));
    return 0;
}

int ref_poisson_fft(int nx, int ny, double lx, double ly, const double* rho, double* phi, double* ex, double* ey) {
    const pic::Domain d = makeDomain(nx, ny, lx, ly);
    pic::FieldGrid grid(d);
    std::memcpy(grid.rho().data(), rho, grid.rho().size() * sizeof(double));
    pic::PoissonSolverFFT solver(d);
    solver.solve(grid);
    std::memcpy(phi, grid.phi().data(), grid.phi().size() * sizeof(double));
    std::memcpy(ex, grid.Ex().data(), grid.Ex().size() * sizeof(double));
    std::memcpy(ey, grid.Ey().data(), grid.Ey().size() * sizeof(double));
    return 0;
}

double ref_spectral_noise(int nx, int ny, double lx, double ly, const double* rho) {
    const pic::Domain d = makeDomain(nx, ny, lx, ly);
    pic::FieldGrid grid(d);
    std::memcpy(grid.rho().data(), rho, grid.rho().size() * sizeof(double));
    return pic::spectralNoiseLevel(grid);
}

// Runs pic::Simulation::run for an SoA configuration and returns the energy
// and charge-error histories (each `steps` long) plus the final drift.
// mode: 0 uniform Maxwellian, 1 Langmuir, 2 Landau (warm Langmuir), 3 two-stream.
int ref_simulation_run(int nx, int ny, double lx, double ly, double dt, int steps, int scheme, int poisson_gs,
                       std::size_t n, unsigned seed, int mode, double temperature, double amplitude, int mode_number,
                       double landau_temperature, double beam_velocity, double perturbation, int sorted,
                       double* total_energy, double* kinetic_energy, double* field_energy, double* charge_error,
                       double* drift_out) {
    try {
        pic::SimulationConfig cfg;
        cfg.domain = makeDomain(nx, ny, lx, ly);
        cfg.domain.dt = dt;
        cfg.domain.steps = steps;
        cfg.layout = pic::ParticleLayout::SoA;
        cfg.scheme = schemeOf(scheme);
        cfg.poisson = poisson_gs ? pic::PoissonSolverType::GaussSeidel : pic::PoissonSolverType::FFT;
        cfg.num_particles = n;
        cfg.seed = seed;
        cfg.temperature = temperature;
        cfg.sorted = sorted != 0;
        cfg.langmuir_mode = mode == 1;
        cfg.landau_mode = mode == 2;
        cfg.two_stream_mode = mode == 3;
        cfg.langmuir_amplitude = amplitude;
        cfg.langmuir_mode_number = mode_number;
        cfg.landau_temperature = landau_temperature;
        cfg.two_stream_beam_velocity = beam_velocity;
        cfg.two_stream_perturbation = perturbation;
        pic::Simulation sim(cfg);
        const pic::SimulationResult r = sim.run();
        for (int s = 0; s < steps && s < static_cast<int>(r.energy_history.size()); ++s) {
            if (total_energy) total_energy[s] = r.energy_history[static_cast<std::size_t>(s)];
            if (kinetic_energy) kinetic_energy[s] = r.kinetic_energy_history[static_cast<std::size_t>(s)];
            if (field_energy) field_energy[s] = r.field_energy_history[static_cast<std::size_t>(s)];
            if (charge_error) charge_error[s] = r.charge_error_history[static_cast<std::size_t>(s)];
        }
        if (drift_out) *drift_out = r.energy_drift;
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

// out[0..4] = omega_theory, omega_measured, relative_error, omega_ratio, amplitude_decay
int ref_langmuir_validation(int nx, int ny, double lx, double ly, double dt, int steps, int scheme, std::size_t n,
                            double amplitude, int mode_number, double* out) {
    try {
        pic::SimulationConfig cfg;
        cfg.domain = makeDomain(nx, ny, lx, ly);
        cfg.domain.dt = dt;
        cfg.domain.steps = steps;
        cfg.scheme = schemeOf(scheme);
        cfg.num_particles = n;
        cfg.langmuir_amplitude = amplitude;
        cfg.langmuir_mode_number = mode_number;
        const pic::LangmuirValidationResult r = pic::runLangmuirValidation(cfg);
        out[0] = r.omega_theory;
        out[1] = r.omega_measured;
        out[2] = r.relative_error;
        out[3] = r.omega_ratio;
        out[4] = r.amplitude_decay;
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

}  // extern "C"
