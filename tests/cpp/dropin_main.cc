// Drives the C++ drop-in (include/dropin/shear_sim.hh over
// include/stzg_shear_sim.hh) the way the reference drivers drive shear_sim
// (esim/sb/main/shear_test.cc:30-72, shear_random.cc:82-121): construct with
// the reference's arguments and an STZ law object, set chi, assign time,
// step or solve with frame files, read tractions and the fields.
// Writes chi0, then p, q, s, tau, chi, X, Y, u, v, eps_pl as raw doubles.
// Usage: dropin <out> <tol> <dir> [direct|frames]: quasi-static steps by
// default; "direct" runs shear_sim::solve (explicit steps, two frames of
// 0.05, files in <dir>); "frames" runs shear_sim::solve_quasistatic (two
// frames of 40 steps, files in <dir>).
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "shear_sim.hh"

int main(int argc, char **argv) {
    if (argc < 4) return 2;
    const int N = 32, steps = 80;
    const double TZ = 21000, kB = 1.3806503e-23;
    const double Omegaeps0 = 300 * 1e-30 * 1.0 * 1.1e9 / (TZ * kB);
    stz_dynamics_linear_athermal stz(TZ, 0.4, 1e-13, 4.2, 8000 / TZ, Omegaeps0, 900 / TZ, 400 / TZ, 0);
    stzg_options o;
    stzg_default_options(&o);
    o.tol = std::atof(argv[2]);
    shear_sim sim(N, N, -1, 1, -1, 1, 1.0, 2.5, 0.0, 0.0, 0.0, 1.0, 0.5, 0.002, 4.0, &stz, argv[3], &o);
    std::vector<double> chi((size_t)N * N);
    stzg_random_chi(N, N, 4, 600, 30, TZ, 11, chi.data());
    sim.set_chi(chi.data());
    sim.time = 0;
    double &t = sim.time;
    const std::string mode = argc > 4 ? argv[4] : "";
    if (mode == "direct") {
        sim.solve(0.1, 2);
    } else if (mode == "frames") {
        sim.solve_quasistatic(0.8, 2, 40);
    } else {
        for (int k = 0; k < steps; k++) sim.step_forward_quasistatic(0.01);
    }
    double bx, by, tx, ty, Q, max_qs;
    sim.tractions(bx, by, tx, ty);
    sim.qs_measure(Q, max_qs);
    std::FILE *f = std::fopen(argv[1], "wb");
    std::fwrite(chi.data(), sizeof(double), chi.size(), f);
    const int ids[] = {STZG_P, STZG_Q, STZG_S, STZG_TAU, STZG_CHI, STZG_X, STZG_Y, STZG_U, STZG_V, STZG_EPS_PL};
    for (int id : ids) {
        std::vector<double> v = sim.field(id);
        std::fwrite(v.data(), sizeof(double), v.size(), f);
    }
    std::fclose(f);
    // the host mirror holds the same state after a fetch
    sim.fetch_fields();
    const std::vector<double> p = sim.field(STZG_P);
    for (int c = 0; c < N * N; c++)
        if (sim.fm[c].p != p[(size_t)N + c]) return 4;
    std::printf("time %.17g bdry_pos %.17g avg_iters %.3f tractions %.17g %.17g %.17g %.17g\n", t, sim.bdry_pos(),
                sim.avg_iters(), bx, by, tx, ty);
    return 0;
}
