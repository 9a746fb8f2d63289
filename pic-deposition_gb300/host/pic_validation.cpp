// Validation drivers on the GB300 path (see pic_validation.hpp).
#include "pic_validation.hpp"

#include <algorithm>
#include <cmath>
#include <memory>
#include <stdexcept>

#include "pic_gb300.h"

namespace pic {

namespace {

void ok(int rc) {
    if (rc != PIC_OK) throw std::runtime_error(std::string("pic_gb300: ") + pic_gpu_last_error());
}

struct Ctx {
    pic_ctx* h = nullptr;
    Ctx(const Domain& d, std::size_t n) {
        pic_domain pd{d.Lx, d.Ly, d.Nx, d.Ny};
        ok(pic_gpu_create(&pd, std::max<std::size_t>(n, 1), 0, &h));
    }
    ~Ctx() { pic_gpu_destroy(h); }
    Ctx(const Ctx&) = delete;
    Ctx& operator=(const Ctx&) = delete;
};

int code(DepositionScheme s) { return static_cast<int>(s); }

const DepositionScheme kSchemes[] = {DepositionScheme::NGP, DepositionScheme::CIC, DepositionScheme::TSC,
                                     DepositionScheme::Esirkepov};

// Least-squares slope of log(max(signal, 1e-30)) against time over the middle
// half of the record (validation.cpp:121-152).
double log_slope(const std::vector<double>& s, double dt, int record_start_step) {
    const std::size_t n = s.size();
    if (n < 8) return 0.0;
    const std::size_t a = n / 4, b = (3 * n) / 4;
    if (b <= a + 2) return 0.0;
    double st = 0.0, sl = 0.0, stt = 0.0, stl = 0.0;
    int m = 0;
    for (std::size_t i = a; i < b; ++i) {
        const double t = static_cast<double>(record_start_step + static_cast<int>(i)) * dt;
        const double l = std::log(std::max(s[i], 1e-30));
        st += t;
        sl += l;
        stt += t * t;
        stl += t * l;
        ++m;
    }
    const double den = static_cast<double>(m) * stt - st * st;
    if (std::abs(den) < 1e-30) return 0.0;
    return (static_cast<double>(m) * stl - st * sl) / den;
}

// FFTW's R2HC of one line: r_k at k <= n/2, i_k at n-k for 0 < k < (n+1)/2 (the
// imaginary part with the e^{-2 pi i k t / n} sign), by direct summation.
void r2hc(const double* in, int n, int stride, double* out, std::vector<double>& cs, std::vector<double>& sn) {
    for (int k = 0; k <= n / 2; ++k) {
        double re = 0.0, im = 0.0;
        for (int t = 0; t < n; ++t) {
            const int w = static_cast<int>((static_cast<long long>(k) * t) % n);
            re += in[t * stride] * cs[w];
            im -= in[t * stride] * sn[w];
        }
        out[k * stride] = re;
        if (k > 0 && k < (n + 1) / 2) out[(n - k) * stride] = im;
    }
}

}  // namespace

double theoreticalPlasmaFrequency(const Domain& domain, std::size_t num_particles) {
    // |q_p| = 1/N_p, n_0 = N_p/V, m = 1 (validation.cpp:66-71)
    const double n0 = static_cast<double>(num_particles) / domain.domainVolume();
    const double q = 1.0 / static_cast<double>(num_particles);
    return std::sqrt(n0 * q * q);
}

double coldTwoStreamGrowthRate(const Domain& domain, std::size_t num_particles) {
    return theoreticalPlasmaFrequency(domain, num_particles) / (2.0 * std::sqrt(2.0));
}

double resonantBeamVelocity(const Domain& domain, std::size_t num_particles, int mode) {
    const double k = 2.0 * M_PI * static_cast<double>(mode) / domain.Lx;
    return k < 1e-30 ? 0.0 : theoreticalPlasmaFrequency(domain, num_particles) / k;
}

double landauDampingTheory(const Domain& domain, std::size_t num_particles, int mode, double temperature) {
    const double wp = theoreticalPlasmaFrequency(domain, num_particles);
    const double k = 2.0 * M_PI * static_cast<double>(mode) / domain.Lx;
    const double kld = k * std::sqrt(temperature) / std::max(wp, 1e-30);
    if (kld < 1e-6) return 0.0;
    const double k2 = kld * kld;
    return wp * std::sqrt(M_PI / 8.0) * k2 * std::exp(-1.0 / (2.0 * k2));
}

double extractFourierModeAmplitude(const FieldGrid& grid, int mode_x) {
    // |<Ex e^{i k x}>| with x at cell centres (validation.cpp:99-119)
    const Domain& d = grid.domain();
    const double k = 2.0 * M_PI * static_cast<double>(mode_x) / d.Lx;
    double re = 0.0, im = 0.0;
    for (int j = 0; j < d.Ny; ++j)
        for (int i = 0; i < d.Nx; ++i) {
            const double ph = k * ((static_cast<double>(i) + 0.5) * d.dx);
            const double e = grid.Ex()[static_cast<std::size_t>(j * d.Nx + i)];
            re += e * std::cos(ph);
            im += e * std::sin(ph);
        }
    const double n = static_cast<double>(d.Nx * d.Ny);
    re /= n;
    im /= n;
    return std::sqrt(re * re + im * im);
}

double estimateInstabilityGrowthRate(const std::vector<double>& signal, double dt, int record_start_step) {
    return log_slope(signal, dt, record_start_step);
}

double estimateDominantFrequency(const std::vector<double>& signal, double dt) {
    // bin of the largest DFT power of the centred signal, in cycles per unit time
    // (validation.cpp:19-54)
    if (signal.size() < 8) return 0.0;
    double mean = 0.0;
    for (double v : signal) mean += v;
    mean /= static_cast<double>(signal.size());
    const int n = static_cast<int>(signal.size());
    double best = 0.0;
    int bk = 1;
    for (int k = 1; k < n / 2; ++k) {
        double re = 0.0, im = 0.0;
        for (int t = 0; t < n; ++t) {
            const double ph = 2.0 * M_PI * static_cast<double>(k * t) / static_cast<double>(n);
            const double c = signal[static_cast<std::size_t>(t)] - mean;
            re += c * std::cos(ph);
            im -= c * std::sin(ph);
        }
        const double p = re * re + im * im;
        if (p > best) {
            best = p;
            bk = k;
        }
    }
    return static_cast<double>(bk) / (static_cast<double>(n) * dt);
}

double spectralNoiseLevel(const FieldGrid& grid) {
    // diagnostics.cpp:53-102: R2HC along x then y, power above N/3 in either index
    const Domain& d = grid.domain();
    const int nx = d.Nx, ny = d.Ny;
    std::vector<double> a(grid.rho().begin(), grid.rho().end()), b(a.size());
    std::vector<double> cs, sn;
    auto tables = [&](int n) {
        cs.resize(n);
        sn.resize(n);
        for (int w = 0; w < n; ++w) {
            cs[w] = std::cos(2.0 * M_PI * w / n);
            sn[w] = std::sin(2.0 * M_PI * w / n);
        }
    };
    tables(nx);
    for (int j = 0; j < ny; ++j) r2hc(a.data() + j * nx, nx, 1, b.data() + j * nx, cs, sn);
    tables(ny);
    for (int i = 0; i < nx; ++i) r2hc(b.data() + i, ny, nx, a.data() + i, cs, sn);
    const int kcx = std::max(1, nx / 3), kcy = std::max(1, ny / 3);
    double total = 0.0, high = 0.0;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double p = a[static_cast<std::size_t>(j * nx + i)] * a[static_cast<std::size_t>(j * nx + i)];
            total += p;
            const int kx = i <= nx / 2 ? i : nx - i, ky = j <= ny / 2 ? j : ny - j;
            if (kx >= kcx || ky >= kcy) high += p;
        }
    return total <= 1e-30 ? 0.0 : high / total;
}

LangmuirValidationResult runLangmuirValidation(const SimulationConfig& config) {
    // validation.cpp:200-261: cold Langmuir wave, push/deposit/background/FFT/gather
    // per step (pic_gpu_run, the same order), dominant frequency of the field energy
    // over the last three quarters of the run
    SimulationConfig cfg = config;
    Domain d = cfg.domain;
    d.updateDerived();
    ParticlesSoA p(cfg.num_particles);
    p.initializeLangmuirWave(d, cfg.langmuir_amplitude, cfg.langmuir_mode_number, cfg.seed);
    Ctx c(d, p.size());
    ok(pic_gpu_upload_particles(c.h, p.x().data(), p.y().data(), p.vx().data(), p.vy().data(), p.q().data(),
                                p.m().data(), p.size()));
    pic_run_config rc{};
    rc.scheme = code(cfg.scheme);
    rc.poisson = 0;
    rc.dt = d.dt;
    rc.background = 1.0 / d.domainVolume();
    rc.use_graph = 1;
    std::vector<pic_diag> h(static_cast<std::size_t>(std::max(d.steps, 0)));
    if (!h.empty()) ok(pic_gpu_run(c.h, &rc, d.steps, h.data()));
    std::vector<double> fe;
    for (int s = d.steps / 4; s < d.steps; ++s) fe.push_back(h[static_cast<std::size_t>(s)].field_energy);
    LangmuirValidationResult r;
    r.omega_theory = theoreticalPlasmaFrequency(d, cfg.num_particles);
    r.omega_measured = estimateDominantFrequency(fe, d.dt);
    if (r.omega_theory > 0.0) {
        r.relative_error = std::abs(r.omega_measured - r.omega_theory) / r.omega_theory;
        r.omega_ratio = r.omega_measured / r.omega_theory;
    }
    if (fe.size() >= 2) r.amplitude_decay = (fe.front() - fe.back()) / std::max(std::abs(fe.front()), 1e-12);
    return r;
}

std::vector<ValidationSummary> runValidationSuite(const SimulationConfig& base_config) {
    // validation.cpp:263-309
    std::vector<ValidationSummary> out;
    for (DepositionScheme s : kSchemes) {
        SimulationConfig cfg = base_config;
        cfg.scheme = s;
        cfg.deposition.scheme = s;
        Domain d = cfg.domain;
        d.updateDerived();
        FieldGrid grid(d);
        ParticlesSoA p(cfg.num_particles);
        p.initializeUniformMaxwellian(d, cfg.temperature, cfg.seed);
        DepositionConfig dep = cfg.deposition;
        dep.scheme = s;
        dep.sorted = false;
        depositChargeSoA(p, grid, dep);
        ValidationSummary v;
        v.scheme = s;
        v.spectral_noise = spectralNoiseLevel(grid);
        v.charge_error = chargeConservationError(grid.integratedRho(), p.totalCharge(), totalAbsChargeSoA(p));
        v.langmuir = runLangmuirValidation(cfg);
        out.push_back(v);
    }
    double ref = 0.0;
    for (const auto& v : out) ref += v.langmuir.omega_measured;
    ref /= static_cast<double>(out.size());
    if (ref > 0.0)
        for (auto& v : out) v.langmuir.passed = std::abs(v.langmuir.omega_measured - ref) / ref <= 0.05;
    return out;
}

std::vector<ConservationStudyResult> runConservationStudy(const SimulationConfig& base_config) {
    // validation.cpp:311-337
    std::vector<ConservationStudyResult> out;
    for (DepositionScheme s : kSchemes) {
        SimulationConfig cfg = base_config;
        cfg.scheme = s;
        cfg.deposition.scheme = s;
        cfg.sorted = true;
        Simulation sim(cfg);
        const SimulationResult r = sim.run();
        ConservationStudyResult row;
        row.scheme = s;
        row.steps = cfg.domain.steps;
        row.max_charge_error = r.charge_error_history.empty()
                                   ? r.final_charge_error
                                   : *std::max_element(r.charge_error_history.begin(), r.charge_error_history.end());
        row.final_energy_drift = r.energy_drift;
        out.push_back(row);
    }
    return out;
}

TwoStreamValidationResult runTwoStreamValidation(const SimulationConfig& config) {
    // validation.cpp:339-405: the Esirkepov variant deposits before it pushes;
    // the mode-1 amplitude of Ex is recorded over the last three quarters
    SimulationConfig cfg = config;
    Domain d = cfg.domain;
    d.updateDerived();
    const double v0 = cfg.two_stream_resonant_beams ? resonantBeamVelocity(d, cfg.num_particles, 1)
                                                    : cfg.two_stream_beam_velocity;
    ParticlesSoA p(cfg.num_particles);
    if (cfg.two_stream_quasi_1d)
        p.initializeTwoStreamQuasi1D(d, v0, cfg.two_stream_perturbation, cfg.seed);
    else
        p.initializeTwoStream(d, v0, cfg.two_stream_perturbation, cfg.seed);
    Ctx c(d, p.size());
    ok(pic_gpu_upload_particles(c.h, p.x().data(), p.y().data(), p.vx().data(), p.vy().data(), p.q().data(),
                                p.m().data(), p.size()));
    const bool esk = cfg.scheme == DepositionScheme::Esirkepov;
    const double bg = 1.0 / d.domainVolume();
    const int record = d.steps / 4;
    FieldGrid grid(d);
    std::vector<double> amp;
    for (int step = 0; step < d.steps; ++step) {
        if (esk) {
            ok(pic_gpu_deposit(c.h, code(cfg.scheme), d.dt, bg, nullptr));
            ok(pic_gpu_push(c.h, d.dt));
        } else {
            ok(pic_gpu_push(c.h, d.dt));
            ok(pic_gpu_deposit(c.h, code(cfg.scheme), 0.0, bg, nullptr));
        }
        ok(pic_gpu_poisson_fft(c.h));
        ok(pic_gpu_gather(c.h, d.dt));
        if (step >= record) {
            ok(pic_gpu_get_fields(c.h, nullptr, grid.Ex().data(), nullptr));
            amp.push_back(extractFourierModeAmplitude(grid, 1));
        }
    }
    TwoStreamValidationResult r;
    r.scheme = cfg.scheme;
    const double wp = theoreticalPlasmaFrequency(d, cfg.num_particles);
    r.omega_p_macro = wp;
    r.growth_rate_theory = coldTwoStreamGrowthRate(d, cfg.num_particles);
    // the slope of the mode amplitude is gamma/omega_p; times omega_p it is gamma
    r.growth_rate_measured = estimateInstabilityGrowthRate(amp, d.dt, record) * wp;
    if (r.growth_rate_theory > 0.0) r.growth_rate_ratio = r.growth_rate_measured / r.growth_rate_theory;
    if (wp > 0.0) r.growth_rate_over_omega_p = r.growth_rate_measured / wp;
    return r;
}

std::vector<TwoStreamValidationResult> runTwoStreamValidationSuite(const SimulationConfig& base_config) {
    // validation.cpp:407-443: agreement within 10 % of the NGP/CIC/TSC mean
    std::vector<TwoStreamValidationResult> out;
    for (DepositionScheme s : kSchemes) {
        SimulationConfig cfg = base_config;
        cfg.scheme = s;
        cfg.deposition.scheme = s;
        out.push_back(runTwoStreamValidation(cfg));
    }
    double ref = 0.0;
    int m = 0;
    for (const auto& r : out)
        if (r.scheme != DepositionScheme::Esirkepov && r.growth_rate_measured > 0.0) {
            ref += r.growth_rate_measured;
            ++m;
        }
    if (m > 0) {
        ref /= static_cast<double>(m);
        for (auto& r : out)
            r.passed = r.growth_rate_measured > 0.0 && std::abs(r.growth_rate_measured - ref) / ref <= 0.10;
    }
    return out;
}

std::vector<NoiseGridResult> runNoiseVsGridStudy(std::size_t num_particles) {
    // validation.cpp:445-472
    std::vector<NoiseGridResult> out;
    for (int g : {64, 128, 256}) {
        Domain d;
        d.Nx = g;
        d.Ny = g;
        d.updateDerived();
        for (DepositionScheme s : kSchemes) {
            FieldGrid grid(d);
            ParticlesSoA p(num_particles);
            p.initializeUniformMaxwellian(d, 1.0, 42);
            DepositionConfig dep;
            dep.scheme = s;
            dep.sorted = true;
            depositChargeSoA(p, grid, dep);
            NoiseGridResult row;
            row.grid_n = g;
            row.scheme = s;
            row.spectral_noise = spectralNoiseLevel(grid);
            out.push_back(row);
        }
    }
    return out;
}

}  // namespace pic
