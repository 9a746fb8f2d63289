// C++ host interface over the C ABI (see pic_gb300_host.hpp).
#include "pic_gb300_host.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <random>
#include <stdexcept>
#include <tuple>

#include "pic_gb300.h"

namespace pic {

namespace {

void check(int rc) {
    if (rc != PIC_OK) throw std::runtime_error(std::string("pic_gb300: ") + pic_gpu_last_error());
}

// One resident context per grid shape, grown on demand (the reference's CUDA
// backend keeps a static device pool too, deposition_cuda.cu:243-273).
struct ContextCache {
    std::mutex mu;
    std::map<std::tuple<int, int, double, double>, std::pair<pic_ctx*, std::size_t>> ctx;
    ~ContextCache() {
        for (auto& kv : ctx) pic_gpu_destroy(kv.second.first);
    }
};

ContextCache& cache() {
    static ContextCache c;
    return c;
}

pic_ctx* context_for(const Domain& d, std::size_t n) {
    auto& c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    const auto key = std::make_tuple(d.Nx, d.Ny, d.Lx, d.Ly);
    auto it = c.ctx.find(key);
    if (it != c.ctx.end() && it->second.second >= std::max<std::size_t>(n, 1)) return it->second.first;
    if (it != c.ctx.end()) {
        pic_gpu_destroy(it->second.first);
        c.ctx.erase(it);
    }
    pic_domain pd{d.Lx, d.Ly, d.Nx, d.Ny};
    pic_ctx* h = nullptr;
    const std::size_t cap = std::max<std::size_t>(n, 1);
    check(pic_gpu_create(&pd, cap, 0, &h));
    c.ctx[key] = {h, cap};
    return h;
}

// The C ABI reads the particle count through every particle pointer and Nx*Ny
// values through every grid pointer; the vectors behind them are resizable, so
// their sizes are checked here (std::runtime_error, the reference's convention).
void check_particles(const ParticlesSoA& p) {
    const std::size_t n = p.size();
    if (p.y().size() != n || p.vx().size() != n || p.vy().size() != n || p.q().size() != n || p.m().size() != n)
        throw std::runtime_error("ParticlesSoA: x, y, vx, vy, q and m differ in length");
}

void check_grid(const FieldGrid& g, const Domain& d) {
    const std::size_t cells = static_cast<std::size_t>(d.Nx) * static_cast<std::size_t>(d.Ny);
    if (g.rho().size() != cells || g.phi().size() != cells || g.Ex().size() != cells || g.Ey().size() != cells)
        throw std::runtime_error("FieldGrid: rho, phi, Ex and Ey must hold Nx*Ny values of the domain");
}

void upload(pic_ctx* h, const ParticlesSoA& p) {
    check_particles(p);
    check(pic_gpu_upload_particles(h, p.x().data(), p.y().data(), p.vx().data(), p.vy().data(), p.q().data(),
                                   p.m().data(), p.size()));
}

int scheme_code(DepositionScheme s) {
    switch (s) {
        case DepositionScheme::NGP:
            return PIC_SCHEME_NGP;
        case DepositionScheme::CIC:
            return PIC_SCHEME_CIC;
        case DepositionScheme::TSC:
            return PIC_SCHEME_TSC;
        default:
            return PIC_SCHEME_ESIRKEPOV;
    }
}

void require_gb300(const DepositionConfig& config) {
    if (config.backend != DepositionBackend::GB300)
        throw std::runtime_error("backend " + backendName(config.backend) + " is not part of the GB300 build");
}

double sample_normal(std::mt19937& rng, double stddev) {
    std::normal_distribution<double> dist(0.0, stddev);
    return dist(rng);
}

}  // namespace

// ---- particles (initialisers as the reference defines them, particles_aos.cpp:67-180) ----
void ParticlesSoA::resize(std::size_t count) {
    x_.resize(count);
    y_.resize(count);
    vx_.resize(count);
    vy_.resize(count);
    q_.resize(count);
    m_.resize(count, 1.0);
}

void ParticlesSoA::initializeUniformMaxwellian(const Domain& domain, double T, unsigned seed) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> ux(0.0, domain.Lx), uy(0.0, domain.Ly);
    const double s = std::sqrt(T);
    for (std::size_t i = 0; i < size(); ++i) {
        x_[i] = ux(rng);
        y_[i] = uy(rng);
        vx_[i] = sample_normal(rng, s);
        vy_[i] = sample_normal(rng, s);
        m_[i] = 1.0;
        q_[i] = (i % 2 == 0) ? 1.0 : -1.0;
    }
}

void ParticlesSoA::initializeLangmuirWave(const Domain& domain, double amplitude, int mode, unsigned) {
    const std::size_t n = size();
    const double k = 2.0 * M_PI * static_cast<double>(mode) / domain.Lx;
    for (std::size_t i = 0; i < n; ++i) {
        x_[i] = domain.Lx * static_cast<double>(i) / static_cast<double>(n);
        y_[i] = 0.5 * domain.Ly;
        vx_[i] = amplitude * std::sin(k * x_[i]);
        vy_[i] = 0.0;
        m_[i] = 1.0;
        q_[i] = -1.0 / static_cast<double>(n);
    }
}

void ParticlesSoA::initializeWarmLangmuirWave(const Domain& domain, double amplitude, int mode, double temperature,
                                              unsigned seed) {
    std::mt19937 rng(seed);
    const std::size_t n = size();
    const double k = 2.0 * M_PI * static_cast<double>(mode) / domain.Lx;
    const double s = std::sqrt(temperature);
    for (std::size_t i = 0; i < n; ++i) {
        x_[i] = domain.Lx * static_cast<double>(i) / static_cast<double>(n);
        y_[i] = 0.5 * domain.Ly;
        vx_[i] = amplitude * std::sin(k * x_[i]) + sample_normal(rng, s);
        vy_[i] = sample_normal(rng, s);
        m_[i] = 1.0;
        q_[i] = -1.0 / static_cast<double>(n);
    }
}

static void two_stream(ParticlesSoA& p, const Domain& domain, double v0, double pert, unsigned seed, bool quasi1d) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> ux(0.0, domain.Lx), uy(0.0, domain.Ly);
    const std::size_t n = p.size();
    const double k = 2.0 * M_PI / domain.Lx;
    for (std::size_t i = 0; i < n; ++i) {
        p.x()[i] = ux(rng);
        p.y()[i] = quasi1d ? 0.5 * domain.Ly : uy(rng);
        const double sign = (i < n / 2) ? 1.0 : -1.0;
        p.vx()[i] = sign * v0 + pert * std::sin(k * p.x()[i]);
        p.vy()[i] = 0.0;
        p.m()[i] = 1.0;
        p.q()[i] = -1.0 / static_cast<double>(n);
    }
}

void ParticlesSoA::initializeTwoStream(const Domain& domain, double beam_velocity, double perturbation, unsigned seed) {
    two_stream(*this, domain, beam_velocity, perturbation, seed, false);
}

void ParticlesSoA::initializeTwoStreamQuasi1D(const Domain& domain, double beam_velocity, double perturbation,
                                              unsigned seed) {
    two_stream(*this, domain, beam_velocity, perturbation, seed, true);
}

double ParticlesSoA::totalCharge() const {
    double s = 0.0;
    for (double v : q_) s += v;
    return s;
}

double ParticlesSoA::kineticEnergy() const {
    double s = 0.0;
    for (std::size_t i = 0; i < size(); ++i) s += 0.5 * m_[i] * (vx_[i] * vx_[i] + vy_[i] * vy_[i]);
    return s;
}

// ---- grid ----
FieldGrid::FieldGrid(const Domain& domain) : domain_(domain) {
    const std::size_t n = static_cast<std::size_t>(domain_.Nx) * domain_.Ny;
    rho_.assign(n, 0.0);
    phi_.assign(n, 0.0);
    Ex_.assign(n, 0.0);
    Ey_.assign(n, 0.0);
}

void FieldGrid::clearFields() {
    std::fill(rho_.begin(), rho_.end(), 0.0);
    std::fill(phi_.begin(), phi_.end(), 0.0);
    std::fill(Ex_.begin(), Ex_.end(), 0.0);
    std::fill(Ey_.begin(), Ey_.end(), 0.0);
}

void FieldGrid::clearRho() { std::fill(rho_.begin(), rho_.end(), 0.0); }

double FieldGrid::integratedRho() const {
    double s = 0.0;
    for (double v : rho_) s += v;
    return s * domain_.cellVolume();
}

double FieldGrid::fieldEnergy() const {
    double s = 0.0;
    for (std::size_t i = 0; i < Ex_.size(); ++i) s += Ex_[i] * Ex_[i] + Ey_[i] * Ey_[i];
    return 0.5 * s * domain_.cellVolume();
}

// ---- deposition ----
DepositionStats estimateBytes(const DepositionConfig& config, std::size_t num_particles, int nx, int ny) {
    // the reference's byte model (deposition.cpp:136-158), kept so reported bandwidths compare
    DepositionStats s;
    s.bytes_read = num_particles * (config.layout == ParticleLayout::AoS ? 48 : 40);
    std::size_t writes = 1;
    if (config.scheme == DepositionScheme::CIC || config.scheme == DepositionScheme::Esirkepov) writes = 4;
    if (config.scheme == DepositionScheme::TSC) writes = 9;
    s.bytes_written = num_particles * writes * sizeof(double) + static_cast<std::size_t>(nx * ny) * sizeof(double);
    return s;
}

void depositChargeSoA(const ParticlesSoA& particles, FieldGrid& grid, const DepositionConfig& config) {
    require_gb300(config);
    check_particles(particles);
    check_grid(grid, grid.domain());
    grid.clearRho();
    pic_ctx* h = context_for(grid.domain(), particles.size());
    upload(h, particles);
    if (config.sorted) check(pic_gpu_sort(h, nullptr, nullptr, nullptr));
    check(pic_gpu_deposit(h, scheme_code(config.scheme), config.esirkepov_dt, 0.0, grid.rho().data()));
}

DepositionStats depositChargeTimedSoA(const ParticlesSoA& particles, FieldGrid& grid, const DepositionConfig& config,
                                      int repeats) {
    require_gb300(config);
    check_particles(particles);
    check_grid(grid, grid.domain());
    using Clock = std::chrono::steady_clock;
    pic_ctx* h = context_for(grid.domain(), particles.size());
    upload(h, particles);
    const int s = scheme_code(config.scheme);
    for (int i = 0; i < 3; ++i) {  // warm-ups, as deposition.cpp:263-268
        if (config.sorted) check(pic_gpu_sort(h, nullptr, nullptr, nullptr));
        check(pic_gpu_deposit(h, s, config.esirkepov_dt, 0.0, nullptr));
    }
    check(pic_gpu_synchronize(h));
    double sort_s = 0.0;
    if (config.sorted) {
        const auto t0 = Clock::now();
        check(pic_gpu_sort(h, nullptr, nullptr, nullptr));
        check(pic_gpu_synchronize(h));
        sort_s = std::chrono::duration<double>(Clock::now() - t0).count();
    }
    std::vector<double> ms;
    for (int i = 0; i < repeats; ++i) {
        const auto t0 = Clock::now();
        check(pic_gpu_deposit(h, s, config.esirkepov_dt, 0.0, nullptr));
        check(pic_gpu_synchronize(h));
        ms.push_back(std::chrono::duration<double, std::milli>(Clock::now() - t0).count());
    }
    check(pic_gpu_get_rho(h, grid.rho().data()));
    DepositionStats st = estimateBytes(config, particles.size(), grid.domain().Nx, grid.domain().Ny);
    double mean = 0.0, var = 0.0;
    for (double v : ms) mean += v;
    mean = ms.empty() ? 0.0 : mean / ms.size();
    for (double v : ms) var += (v - mean) * (v - mean);
    st.sort_ms = sort_s * 1e3;
    st.deposit_ms = mean;
    st.deposit_std_ms = ms.size() > 1 ? std::sqrt(var / (ms.size() - 1)) : 0.0;
    st.time_ms = st.sort_ms + st.deposit_ms;
    const double dep_s = std::max(mean / 1e3, 1e-12);
    st.throughput_particles_per_s = particles.size() / dep_s;
    st.effective_bandwidth_gbs = (static_cast<double>(st.bytes_read + st.bytes_written) / 1e9) / dep_s;
    st.charge_error = chargeConservationError(grid.integratedRho(), particles.totalCharge(), totalAbsChargeSoA(particles));
    return st;
}

void gatherFieldsSoA(ParticlesSoA& particles, FieldGrid& grid, double dt) {
    check_particles(particles);
    check_grid(grid, grid.domain());
    pic_ctx* h = context_for(grid.domain(), particles.size());
    upload(h, particles);
    check(pic_gpu_set_fields(h, nullptr, grid.Ex().data(), grid.Ey().data()));
    check(pic_gpu_gather(h, dt));
    check(pic_gpu_download_particles(h, nullptr, nullptr, particles.vx().data(), particles.vy().data(), nullptr,
                                     nullptr));
}

void pushParticlesSoA(ParticlesSoA& particles, const FieldGrid& grid, double dt) {
    check_particles(particles);
    pic_ctx* h = context_for(grid.domain(), particles.size());
    upload(h, particles);
    check(pic_gpu_push(h, dt));
    check(pic_gpu_download_particles(h, particles.x().data(), particles.y().data(), nullptr, nullptr, nullptr,
                                     nullptr));
}

void sortParticlesByCell(ParticlesSoA& particles, const Domain& domain) {
    check_particles(particles);
    const std::size_t n = particles.size();
    pic_ctx* h = context_for(domain, n);
    upload(h, particles);
    std::vector<uint32_t> perm(n);
    check(pic_gpu_sort(h, nullptr, perm.data(), nullptr));
    ParticlesSoA out(n);
    for (std::size_t i = 0; i < n; ++i) {
        const std::size_t s = perm[i];
        out.x()[i] = particles.x()[s];
        out.y()[i] = particles.y()[s];
        out.vx()[i] = particles.vx()[s];
        out.vy()[i] = particles.vy()[s];
        out.q()[i] = particles.q()[s];
        out.m()[i] = particles.m()[s];
    }
    particles = std::move(out);
}

int particleCellIndex(double x, double y, const Domain& domain) {
    pic_ctx* h = context_for(domain, 1);
    const double q = 1.0;
    check(pic_gpu_upload_particles(h, &x, &y, nullptr, nullptr, &q, nullptr, 1));
    uint32_t key = 0;
    check(pic_gpu_download_device_layout(h, &key, nullptr, nullptr, nullptr, nullptr, nullptr));
    return static_cast<int>(key);
}

std::string schemeName(DepositionScheme s) {
    switch (s) {
        case DepositionScheme::NGP:
            return "NGP";
        case DepositionScheme::CIC:
            return "CIC";
        case DepositionScheme::TSC:
            return "TSC";
        case DepositionScheme::Esirkepov:
            return "Esirkepov";
    }
    return "Unknown";
}

std::string backendName(DepositionBackend b) {
    switch (b) {
        case DepositionBackend::CPU:
            return "CPU";
        case DepositionBackend::GPUAtomics:
            return "GPU_Atomics";
        case DepositionBackend::GPUPrivatized:
            return "GPU_Priv";
        case DepositionBackend::GB300:
            return "GB300";
    }
    return "Unknown";
}

DepositionScheme schemeFromString(const std::string& name) {
    if (name == "NGP") return DepositionScheme::NGP;
    if (name == "CIC") return DepositionScheme::CIC;
    if (name == "TSC") return DepositionScheme::TSC;
    if (name == "Esirkepov") return DepositionScheme::Esirkepov;
    throw std::runtime_error("Unknown deposition scheme: " + name);
}

DepositionBackend backendFromString(const std::string& name) {
    if (name == "CPU") return DepositionBackend::CPU;
    if (name == "GPU_Atomics") return DepositionBackend::GPUAtomics;
    if (name == "GPU_Priv") return DepositionBackend::GPUPrivatized;
    if (name == "GB300") return DepositionBackend::GB300;
    throw std::runtime_error("Unknown backend: " + name);
}

// ---- Poisson ----
void PoissonSolverFFT::solve(FieldGrid& grid) {
    check_grid(grid, domain_);
    pic_ctx* h = context_for(domain_, 1);
    check(pic_gpu_set_rho(h, grid.rho().data()));
    check(pic_gpu_poisson_fft(h));
    check(pic_gpu_get_fields(h, grid.phi().data(), grid.Ex().data(), grid.Ey().data()));
}

void PoissonSolverGS::solve(FieldGrid& grid) {
    check_grid(grid, domain_);
    pic_ctx* h = context_for(domain_, 1);
    check(pic_gpu_set_rho(h, grid.rho().data()));
    check(pic_gpu_set_fields(h, grid.phi().data(), nullptr, nullptr));
    double res = 0.0;
    check(pic_gpu_poisson_rbgs(h, tol_, max_iters_, 1, 16, &last_iters_, &res));
    check(pic_gpu_get_fields(h, grid.phi().data(), grid.Ex().data(), grid.Ey().data()));
}

// ---- diagnostics (diagnostics.cpp:18-51) ----
double chargeConservationError(double integrated_rho, double total_charge, double abs_charge_sum) {
    return std::abs(integrated_rho - total_charge) / std::max(abs_charge_sum, 1e-12);
}

double totalAbsChargeSoA(const ParticlesSoA& p) {
    double s = 0.0;
    for (double v : p.q()) s += std::abs(v);
    return s;
}

Diagnostics computeDiagnostics(const FieldGrid& grid, const ParticlesSoA& particles) {
    Diagnostics d;
    d.total_charge = particles.totalCharge();
    d.integrated_rho = grid.integratedRho();
    d.charge_error = chargeConservationError(d.integrated_rho, d.total_charge, totalAbsChargeSoA(particles));
    d.kinetic_energy = particles.kineticEnergy();
    d.field_energy = grid.fieldEnergy();
    d.total_energy = d.kinetic_energy + d.field_energy;
    return d;
}

// ---- Simulation ----
Simulation::Simulation(SimulationConfig config) : config_(std::move(config)), grid_(config_.domain) {
    config_.domain.updateDerived();
    grid_ = FieldGrid(config_.domain);
    particles_.resize(config_.num_particles);
    if (config_.langmuir_mode) {
        particles_.initializeLangmuirWave(config_.domain, config_.langmuir_amplitude, config_.langmuir_mode_number,
                                          config_.seed);
    } else if (config_.landau_mode) {
        particles_.initializeWarmLangmuirWave(config_.domain, config_.langmuir_amplitude, config_.langmuir_mode_number,
                                              config_.landau_temperature, config_.seed);
    } else if (config_.two_stream_mode) {
        particles_.initializeTwoStream(config_.domain, config_.two_stream_beam_velocity,
                                       config_.two_stream_perturbation, config_.seed);
    } else {
        particles_.initializeUniformMaxwellian(config_.domain, config_.temperature, config_.seed);
    }
}

SimulationResult Simulation::run() {
    SimulationResult r;
    const Domain& d = config_.domain;
    check_particles(particles_);
    check_grid(grid_, d);
    pic_ctx* h = context_for(d, particles_.size());
    upload(h, particles_);
    pic_run_config rc{};
    rc.scheme = scheme_code(config_.scheme);
    rc.poisson = config_.poisson == PoissonSolverType::FFT ? 0 : 1;
    rc.dt = d.dt;
    // applyBackgroundIfNeeded (simulation.cpp:52-59)
    rc.background = (config_.langmuir_mode || config_.landau_mode || config_.two_stream_mode) ? 1.0 / d.domainVolume()
                                                                                              : 0.0;
    rc.sort_interval = config_.sorted ? std::max(config_.sort_interval, 1) : 0;
    rc.use_graph = config_.use_graph ? 1 : 0;
    // the reference's PoissonSolverGS defaults: 500 sweeps, tolerance 1e-6
    // (here on the relative residual, poisson_gs.cpp:11-61 stops on max|dphi|)
    rc.rbgs_tol = 1e-6;
    rc.rbgs_max_iters = 500;
    rc.rbgs_check_every = 10;
    std::vector<pic_diag> hist(static_cast<std::size_t>(std::max(d.steps, 0)));
    check(pic_gpu_run(h, &rc, d.steps, hist.empty() ? nullptr : hist.data()));
    for (const auto& s : hist) {
        r.energy_history.push_back(s.total_energy);
        r.kinetic_energy_history.push_back(s.kinetic_energy);
        r.field_energy_history.push_back(s.field_energy);
        r.charge_error_history.push_back(s.charge_error);
    }
    if (!r.energy_history.empty()) {
        r.initial_energy = r.energy_history.front();
        r.final_energy = r.energy_history.back();
        r.energy_drift = (r.final_energy - r.initial_energy) / std::max(std::abs(r.initial_energy), 1e-12);
        r.final_charge_error = r.charge_error_history.back();
    }
    check(pic_gpu_download_particles(h, particles_.x().data(), particles_.y().data(), particles_.vx().data(),
                                     particles_.vy().data(), particles_.q().data(), particles_.m().data()));
    check(pic_gpu_get_fields(h, grid_.phi().data(), grid_.Ex().data(), grid_.Ey().data()));
    check(pic_gpu_get_rho(h, grid_.rho().data()));
    return r;
}

}  // namespace pic
