// Physics validation drivers of the reference (src/pic/validation.hpp,
// src/pic/validation.cpp:19-472, src/pic/diagnostics.cpp:53-102) on the GB300
// path: the same structs, functions and set-ups, with every deposit, solve,
// gather and push done by the GPU through the C ABI. The estimators
// (dominant-frequency DFT, log-slope fit, Fourier mode amplitude, spectral
// noise ratio) are the reference's, evaluated on the host.
#pragma once

#include <cstddef>
#include <string>
#include <vector>

#include "pic_gb300_host.hpp"

namespace pic {

struct LangmuirValidationResult {
    double omega_theory = 0.0;
    double omega_measured = 0.0;
    double relative_error = 0.0;
    double omega_ratio = 0.0;
    double amplitude_decay = 0.0;
    bool passed = false;
};

struct ValidationSummary {
    DepositionScheme scheme = DepositionScheme::CIC;
    LangmuirValidationResult langmuir;
    double spectral_noise = 0.0;
    double charge_error = 0.0;
};

struct ConservationStudyResult {
    DepositionScheme scheme = DepositionScheme::CIC;
    int steps = 0;
    double max_charge_error = 0.0;
    double final_energy_drift = 0.0;
};

struct TwoStreamValidationResult {
    DepositionScheme scheme = DepositionScheme::CIC;
    double growth_rate_measured = 0.0;
    double growth_rate_theory = 0.0;
    double growth_rate_ratio = 0.0;
    double omega_p_macro = 0.0;
    double growth_rate_over_omega_p = 0.0;
    bool passed = false;
};

struct NoiseGridResult {
    int grid_n = 64;
    DepositionScheme scheme = DepositionScheme::CIC;
    double spectral_noise = 0.0;
};

LangmuirValidationResult runLangmuirValidation(const SimulationConfig& config);
std::vector<ValidationSummary> runValidationSuite(const SimulationConfig& base_config);
std::vector<ConservationStudyResult> runConservationStudy(const SimulationConfig& base_config);
TwoStreamValidationResult runTwoStreamValidation(const SimulationConfig& config);
std::vector<TwoStreamValidationResult> runTwoStreamValidationSuite(const SimulationConfig& base_config);
std::vector<NoiseGridResult> runNoiseVsGridStudy(std::size_t num_particles);

double theoreticalPlasmaFrequency(const Domain& domain, std::size_t num_particles);
double coldTwoStreamGrowthRate(const Domain& domain, std::size_t num_particles);
double resonantBeamVelocity(const Domain& domain, std::size_t num_particles, int mode = 1);
double landauDampingTheory(const Domain& domain, std::size_t num_particles, int mode, double temperature);
double extractFourierModeAmplitude(const FieldGrid& grid, int mode_x);
double estimateInstabilityGrowthRate(const std::vector<double>& signal, double dt, int record_start_step);
double estimateDominantFrequency(const std::vector<double>& signal, double dt);
// High-k share of the power of rho's separable real (R2HC x R2HC) transform, k >= N/3.
double spectralNoiseLevel(const FieldGrid& grid);

}  // namespace pic
