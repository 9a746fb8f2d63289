// The reference's validation driver (src/main_validation.cpp) run on the GB300
// path through the ported drivers (pic_validation.hpp), printing the rows the
// reference writes to its CSVs (validation.cpp:474-505):
//   noise,<grid>,<scheme>,<spectral_noise>
//   validation,<scheme>,<spectral_noise>,<charge_error>,<omega_theory>,<omega_measured>,<passed>
//   conservation,<scheme>,<steps>,<max_charge_error>,<final_energy_drift>
//   two_stream,<scheme>,<gamma_measured>,<gamma_theory>,<ratio>,<omega_p>,<gamma/omega_p>,<passed>
#include <cstdio>

#include "pic_validation.hpp"

int main() {
    for (const auto& r : pic::runNoiseVsGridStudy(100000))
        std::printf("noise,%dx%d,%s,%.10g\n", r.grid_n, r.grid_n, pic::schemeName(r.scheme).c_str(), r.spectral_noise);

    pic::SimulationConfig cfg;  // main_validation.cpp:6-18
    cfg.domain.Nx = 64;
    cfg.domain.Ny = 64;
    cfg.domain.Lx = 1.0;
    cfg.domain.Ly = 1.0;
    cfg.domain.dt = 0.002;
    cfg.domain.steps = 16384;
    cfg.domain.updateDerived();
    cfg.num_particles = 200;
    cfg.langmuir_amplitude = 0.05;
    cfg.langmuir_mode_number = 1;
    for (const auto& s : pic::runValidationSuite(cfg))
        std::printf("validation,%s,%.10g,%.10g,%.10g,%.10g,%d\n", pic::schemeName(s.scheme).c_str(), s.spectral_noise,
                    s.charge_error, s.langmuir.omega_theory, s.langmuir.omega_measured, s.langmuir.passed ? 1 : 0);

    pic::SimulationConfig cons;  // main_validation.cpp:29-40
    cons.domain.Nx = 64;
    cons.domain.Ny = 64;
    cons.domain.Lx = 1.0;
    cons.domain.Ly = 1.0;
    cons.domain.dt = 0.005;
    cons.domain.steps = 2000;
    cons.domain.updateDerived();
    cons.num_particles = 10000;
    cons.sorted = true;
    for (const auto& c : pic::runConservationStudy(cons))
        std::printf("conservation,%s,%d,%.10g,%.10g\n", pic::schemeName(c.scheme).c_str(), c.steps, c.max_charge_error,
                    c.final_energy_drift);

    pic::SimulationConfig ts;  // main_validation.cpp:48-60
    ts.domain.Nx = 64;
    ts.domain.Ny = 64;
    ts.domain.Lx = 1.0;
    ts.domain.Ly = 1.0;
    ts.domain.dt = 0.002;
    ts.domain.steps = 2000;
    ts.domain.updateDerived();
    ts.num_particles = 5000;
    ts.two_stream_beam_velocity = 0.3;
    ts.two_stream_perturbation = 0.01;
    for (const auto& t : pic::runTwoStreamValidationSuite(ts))
        std::printf("two_stream,%s,%.10g,%.10g,%.10g,%.10g,%.10g,%d\n", pic::schemeName(t.scheme).c_str(),
                    t.growth_rate_measured, t.growth_rate_theory, t.growth_rate_ratio, t.omega_p_macro,
                    t.growth_rate_over_omega_p, t.passed ? 1 : 0);
    return 0;
}
