// Drives the C++ drop-in (include/stzg_shear_sim.hh) the way the reference
// drivers drive shear_sim (esim/sb/main/shear_test.cc:30-72): construct with
// the reference's arguments and an STZ law object, step, read fields.
// Writes chi0, then p, q, s, tau, chi, X, Y, u, v, eps_pl as raw doubles.
// Usage: dropin <out> <tol> [direct]; "direct" runs shear_sim::solve (the
// explicit step, two frames of 0.05) instead of quasi-static steps.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "stzg_shear_sim.hh"

// Public members of the reference's stz_dynamics (stz_model.hh:12-27).
struct stz_law {
    double TZ, c0, tau0, kappa, Delta, Omegaeps0, chi_inf, thetainv, rho;
};

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    const int N = 32, steps = 80;
    const double TZ = 21000, kB = 1.3806503e-23;
    stz_law stz{TZ, 0.4, 1e-13, 4.2, 8000 / TZ, 300 * 1e-30 * 1.0 * 1.1e9 / (TZ * kB), 900 / TZ, TZ / 400, 0};
    stzg_options o;
    stzg_default_options(&o);
    o.tol = std::atof(argv[2]);
    stzg::shear_sim sim(N, N, -1, 1, -1, 1, 1.0, 2.5, 0.0, 0.0, 0.0, 1.0, 0.5, 0.002, 4.0, &stz, "", 2, -1, &o);
    std::vector<double> chi((size_t)N * N);
    stzg_random_chi(N, N, 4, 600, 30, TZ, 11, chi.data());
    sim.set_chi(chi.data());
    if (argc > 3 && std::string(argv[3]) == "direct") {
        int frames = 0;
        sim.solve(0.1, 2, [&](int) { frames++; });
        if (frames != 2) return 3;
    } else {
        for (int k = 0; k < steps; k++) sim.step_forward_quasistatic(0.01);
    }
    std::FILE *f = std::fopen(argv[1], "wb");
    std::fwrite(chi.data(), sizeof(double), chi.size(), f);
    const int ids[] = {STZG_P, STZG_Q, STZG_S, STZG_TAU, STZG_CHI, STZG_X, STZG_Y, STZG_U, STZG_V, STZG_EPS_PL};
    for (int id : ids) {
        std::vector<double> v = sim.field(id);
        std::fwrite(v.data(), sizeof(double), v.size(), f);
    }
    std::fclose(f);
    std::printf("time %.17g avg_iters %.3f\n", sim.time(), sim.avg_iters());
    return 0;
}
