// C++ host interface of the GB300 deposition path.
//
// Mirrors the hot-path interface of ehocine/pic-deposition -- the same type and
// function names, argument meaning and error behaviour (std::runtime_error) --
// so code written against the reference's
//   src/pic/domain.hpp, src/pic/particles.hpp, src/pic/field_grid.hpp,
//   src/deposition/deposition.hpp, src/sorting/cell_sort.hpp,
//   src/pic/poisson_fft.hpp, src/pic/diagnostics.hpp, src/pic/simulation.hpp
// compiles against this header. Every computation goes through the C ABI in
// include/pic_gb300.h (CUDA kernels on one GPU); nothing here computes on the
// CPU except the particle initialisers and the FP64 host sums the reference's
// own classes provide (FieldGrid::integratedRho, ParticlesSoA::totalCharge, ...).
//
// Differences from the reference, by design:
//  * DepositionBackend has one more value, GB300, and it is the only backend
//    implemented here; the others throw.
//  * sortParticlesByCell is a stable sort (the reference's std::sort is not).
//  * PoissonSolverGS is red-black Gauss-Seidel, warm-started from grid.phi(),
//    stopped on the relative residual ||b - A phi|| / ||b|| <= tol.
//  * Only the SoA layout exists (the device layout is SoA; the reference's AoS
//    overloads copy into SoA anyway).
//  * Simulation::run with sorted=true keeps the resident particles in cell order
//    (the reference sorts a copy each step), so particles() comes back permuted.
#pragma once

#include <cstddef>
#include <string>
#include <utility>
#include <vector>

namespace pic {

struct Domain {
    double Lx = 1.0;
    double Ly = 1.0;
    int Nx = 64;
    int Ny = 64;
    double dx = Lx / Nx;
    double dy = Ly / Ny;
    double dt = 0.01;
    int steps = 100;

    void updateDerived() {
        dx = Lx / Nx;
        dy = Ly / Ny;
    }
    double cellVolume() const { return dx * dy; }
    double domainVolume() const { return Lx * Ly; }
    int cellIndex(int ix, int iy) const { return iy * Nx + ix; }
};

enum class ParticleLayout { AoS, SoA };

class ParticlesSoA {
public:
    explicit ParticlesSoA(std::size_t count = 0) { resize(count); }
    std::size_t size() const { return x_.size(); }
    void resize(std::size_t count);
    void initializeUniformMaxwellian(const Domain& domain, double T, unsigned seed);
    void initializeLangmuirWave(const Domain& domain, double amplitude, int mode, unsigned seed);
    void initializeWarmLangmuirWave(const Domain& domain, double amplitude, int mode, double temperature,
                                    unsigned seed);
    void initializeTwoStream(const Domain& domain, double beam_velocity, double perturbation, unsigned seed);
    void initializeTwoStreamQuasi1D(const Domain& domain, double beam_velocity, double perturbation, unsigned seed);
    double totalCharge() const;
    double kineticEnergy() const;

    std::vector<double>& x() { return x_; }
    std::vector<double>& y() { return y_; }
    std::vector<double>& vx() { return vx_; }
    std::vector<double>& vy() { return vy_; }
    std::vector<double>& q() { return q_; }
    std::vector<double>& m() { return m_; }
    const std::vector<double>& x() const { return x_; }
    const std::vector<double>& y() const { return y_; }
    const std::vector<double>& vx() const { return vx_; }
    const std::vector<double>& vy() const { return vy_; }
    const std::vector<double>& q() const { return q_; }
    const std::vector<double>& m() const { return m_; }

private:
    std::vector<double> x_, y_, vx_, vy_, q_, m_;
};

class FieldGrid {
public:
    explicit FieldGrid(const Domain& domain);
    void clearFields();
    void clearRho();
    const Domain& domain() const { return domain_; }
    std::vector<double>& rho() { return rho_; }
    const std::vector<double>& rho() const { return rho_; }
    std::vector<double>& phi() { return phi_; }
    const std::vector<double>& phi() const { return phi_; }
    std::vector<double>& Ex() { return Ex_; }
    const std::vector<double>& Ex() const { return Ex_; }
    std::vector<double>& Ey() { return Ey_; }
    const std::vector<double>& Ey() const { return Ey_; }
    double integratedRho() const;
    double fieldEnergy() const;

private:
    Domain domain_;
    std::vector<double> rho_, phi_, Ex_, Ey_;
};

enum class DepositionScheme { NGP, CIC, TSC, Esirkepov };
enum class DepositionBackend { CPU, GPUAtomics, GPUPrivatized, GB300 };

struct DepositionConfig {
    DepositionScheme scheme = DepositionScheme::CIC;
    ParticleLayout layout = ParticleLayout::SoA;
    DepositionBackend backend = DepositionBackend::GB300;
    bool sorted = false;
    int num_threads = 1;
    double dx_esirkepov = 0.0;
    double dy_esirkepov = 0.0;
    double esirkepov_dt = 0.0;
};

struct DepositionStats {
    double sort_ms = 0.0;
    double deposit_ms = 0.0;
    double deposit_std_ms = 0.0;
    double time_ms = 0.0;
    double throughput_particles_per_s = 0.0;
    double effective_bandwidth_gbs = 0.0;
    double charge_error = 0.0;
    std::size_t bytes_read = 0;
    std::size_t bytes_written = 0;
};

DepositionStats estimateBytes(const DepositionConfig& config, std::size_t num_particles, int nx, int ny);
void depositChargeSoA(const ParticlesSoA& particles, FieldGrid& grid, const DepositionConfig& config);
DepositionStats depositChargeTimedSoA(const ParticlesSoA& particles, FieldGrid& grid, const DepositionConfig& config,
                                      int repeats = 1);
void gatherFieldsSoA(ParticlesSoA& particles, FieldGrid& grid, double dt);
void pushParticlesSoA(ParticlesSoA& particles, const FieldGrid& grid, double dt);
void sortParticlesByCell(ParticlesSoA& particles, const Domain& domain);
int particleCellIndex(double x, double y, const Domain& domain);

std::string schemeName(DepositionScheme scheme);
std::string backendName(DepositionBackend backend);
DepositionScheme schemeFromString(const std::string& name);
DepositionBackend backendFromString(const std::string& name);

class PoissonSolverFFT {
public:
    explicit PoissonSolverFFT(const Domain& domain) : domain_(domain) {}
    void solve(FieldGrid& grid);

private:
    Domain domain_;
};

class PoissonSolverGS {
public:
    explicit PoissonSolverGS(const Domain& domain, int max_iters = 500, double tol = 1e-6)
        : domain_(domain), max_iters_(max_iters), tol_(tol) {}
    void solve(FieldGrid& grid);
    int lastIterations() const { return last_iters_; }

private:
    Domain domain_;
    int max_iters_;
    double tol_;
    int last_iters_ = 0;
};

struct Diagnostics {
    double charge_error = 0.0;
    double total_charge = 0.0;
    double integrated_rho = 0.0;
    double kinetic_energy = 0.0;
    double field_energy = 0.0;
    double total_energy = 0.0;
};

double chargeConservationError(double integrated_rho, double total_charge, double abs_charge_sum);
double totalAbsChargeSoA(const ParticlesSoA& particles);
Diagnostics computeDiagnostics(const FieldGrid& grid, const ParticlesSoA& particles);

enum class PoissonSolverType { FFT, GaussSeidel };

struct SimulationConfig {
    Domain domain;
    ParticleLayout layout = ParticleLayout::SoA;
    DepositionScheme scheme = DepositionScheme::CIC;
    DepositionConfig deposition;
    PoissonSolverType poisson = PoissonSolverType::FFT;
    std::size_t num_particles = 10000;
    unsigned seed = 42;
    double temperature = 1.0;
    bool sorted = false;
    int sort_interval = 1;
    bool langmuir_mode = false;
    double langmuir_amplitude = 0.01;
    int langmuir_mode_number = 1;
    bool landau_mode = false;
    double landau_temperature = 0.1;
    bool two_stream_mode = false;
    bool two_stream_resonant_beams = true;  // read by the reference's validation drivers only
    bool two_stream_quasi_1d = false;       // read by the reference's validation drivers only
    double two_stream_beam_velocity = 0.3;
    double two_stream_perturbation = 0.01;
    bool use_graph = true;  // new: replay the step as a CUDA graph (FFT Poisson)
};

struct SimulationResult {
    std::vector<double> energy_history;
    std::vector<double> kinetic_energy_history;
    std::vector<double> field_energy_history;
    std::vector<double> charge_error_history;
    double initial_energy = 0.0;
    double final_energy = 0.0;
    double energy_drift = 0.0;
    double final_charge_error = 0.0;
    double spectral_noise = 0.0;  // not computed here (an FFTW diagnostic, off the deposition path)
};

// Simulation::run (src/pic/simulation.cpp:69-145) with every step on the GPU.
class Simulation {
public:
    explicit Simulation(SimulationConfig config);
    SimulationResult run();
    const ParticlesSoA& particles() const { return particles_; }
    const FieldGrid& grid() const { return grid_; }

private:
    SimulationConfig config_;
    FieldGrid grid_;
    ParticlesSoA particles_;
};

}  // namespace pic
