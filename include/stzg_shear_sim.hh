// stzg_shear_sim.hh - C++ drop-in for the reference's shear_sim and tgmg
// classes (esim/sb/main/shear_sim.hh:20-151, esim/tgmg/tgmg.hh:286-495) on
// top of the C ABI in stzg.h.  Header-only; link with libstzg.so.
//
// The constructor takes the reference's arguments in the reference's order
// (shear_sim.hh:95-99).  The STZ law object is read through its public
// members (TZ, c0, tau0, kappa, Delta, Omegaeps0, chi_inf, thetainv, rho,
// stz_model.hh:12-27), so a reference stz_dynamics_* object can be passed
// directly; the law is named by `model` (0 linear, 1 nonlinear, 2 linear
// athermal, 3 nonlinear athermal) and `t_model`.
//
// Error behaviour follows the reference: a failed multigrid solve prints a
// message and exits with status 1, as qs_multi::solve does
// (qs_multi.hh:51-53); other failures do the same with the library message.
#ifndef STZG_SHEAR_SIM_HH
#define STZG_SHEAR_SIM_HH

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "stzg.h"

namespace stzg {

inline void check_or_exit(int st) {
    if (st != STZG_OK) {
        std::fprintf(stderr, "stzg: %s: %s\n", stzg_strerror(st), stzg_last_message());
        std::exit(1);
    }
}

class shear_sim {
  public:
    const int m, n;
    const double ax, bx, ay, by, dx, dy, mu, K, viscosity, chi_diff, chi_len, t_scale, tmult, adapt_fac, u_bdry;

    template <class STZ>
    shear_sim(int m_, int n_, double ax_, double bx_, double ay_, double by_, double mu_, double K_, double visc_,
              double chi_diff_, double chi_len_, double t_scale_, double tmult_, double adapt_fac_,
              double u_bdry_, const STZ *stz, const char * /*filename*/, int model = 2, int t_model = -1,
              const stzg_options *opt = nullptr)
        : m(m_), n(n_), ax(ax_), bx(bx_), ay(ay_), by(by_), dx((bx_ - ax_) / m_), dy((by_ - ay_) / n_), mu(mu_),
          K(K_), viscosity(visc_), chi_diff(chi_diff_), chi_len(chi_len_), t_scale(t_scale_), tmult(tmult_),
          adapt_fac(adapt_fac_), u_bdry(u_bdry_), h(nullptr) {
        stz_params p;
        p.m = m_;
        p.n = n_;
        p.stz_model = model;
        p.t_model = t_model;
        p.ax = ax_; p.bx = bx_; p.ay = ay_; p.by = by_;
        p.mu = mu_; p.K = K_; p.viscosity = visc_; p.chi_diff = chi_diff_; p.chi_len = chi_len_;
        p.t_scale = t_scale_; p.adapt_fac = adapt_fac_; p.u_bdry = u_bdry_;
        p.TZ = stz->TZ; p.c0 = stz->c0; p.tau0 = stz->tau0; p.kappa = stz->kappa; p.Delta = stz->Delta;
        p.Omegaeps0 = stz->Omegaeps0; p.chi_inf = stz->chi_inf; p.theta = 1 / stz->thetainv; p.rho = stz->rho;
        p.s_y = 1;
        params = p;
        check_or_exit(stzg_create(&params, opt, &h));
    }
    ~shear_sim() { stzg_destroy(h); }
    shear_sim(const shear_sim &) = delete;
    shear_sim &operator=(const shear_sim &) = delete;

    // shear_sim::initialize_random (shear_sim.cc:932), seeded generator.
    void initialize_random(double l, double tem_avg, double tem_stdev, unsigned long long seed = 1) {
        std::vector<double> chi((size_t)m * n);
        check_or_exit(stzg_random_chi(m, n, l, tem_avg, tem_stdev, params.TZ, seed, chi.data()));
        check_or_exit(stzg_set_state(h, chi.data()));
    }
    void set_chi(const double *chi) { check_or_exit(stzg_set_state(h, chi)); }

    void step_forward_quasistatic(double dt) { check_or_exit(stzg_step_qs(h, dt, 1, nullptr)); }
    // shear_sim::step_forward (shear_sim.cc:185-276), the explicit step.
    void step_forward(double dt) { check_or_exit(stzg_step_direct(h, dt, 1, nullptr)); }
    // shear_sim::solve (shear_sim.cc:120-140) without file output: steps of
    // dx*dx*tmult landing exactly on every frame time; frame(k) after each.
    template <class F> void solve(double duration, int frames, F frame) {
        const double dt = dx * dx * tmult, t_start = time();
        for (int k = 1; k <= frames; k++) {
            check_or_exit(stzg_advance_direct(h, dt, t_start + duration / frames * k, nullptr));
            frame(k);
        }
    }
    void solve(double duration, int frames) {
        solve(duration, frames, [](int) {});
    }
    void advection_step(double dt) { check_or_exit(stzg_advection_step(h, dt)); }
    void projection_step(double dt) { check_or_exit(stzg_projection_step(h, dt, nullptr)); }
    // shear_sim::solve_quasistatic (shear_sim.cc:159-181) without file output;
    // frame(k) is called after every frame.
    template <class F> void solve_quasistatic(double duration, int frames, int steps, F frame) {
        const double dt = duration / frames / steps;
        for (int k = 1; k <= frames; k++) {
            check_or_exit(stzg_step_qs(h, dt, steps, nullptr));
            frame(k);
        }
    }
    void solve_quasistatic(double duration, int frames, int steps) {
        solve_quasistatic(duration, frames, steps, [](int) {});
    }
    double avg_iters() {
        double a = 0;
        check_or_exit(stzg_avg_iters(h, &a));
        return a;
    }
    double time() const {
        double t = 0;
        check_or_exit(stzg_get_time(h, &t));
        return t;
    }
    // Field access with the field ids of stzg.h.
    std::vector<double> field(int id) const {
        size_t cnt = (id == STZG_U || id == STZG_V || id == STZG_X || id == STZG_Y) ? (size_t)m * (n + 1)
                     : id == STZG_EPS_PL                                            ? (size_t)m * n
                                                                                    : (size_t)m * (n + 2);
        std::vector<double> v(cnt);
        check_or_exit(stzg_get_field(h, id, v.data()));
        return v;
    }
    // shear_sim::l2_comparison (shear_sim.cc:460-502).
    void l2_comparison(shear_sim &other, double *l2) { check_or_exit(stzg_l2_comparison(h, other.h, l2)); }

    stzg_sim *handle() { return h; }

  private:
    stz_params params;
    stzg_sim *h;
};

// tgmg<qs_multi,vec,mat> over a shear_sim's operator for one time step:
// setup() (tgmg.hh:331), solve_v_cycle() with the adaptive predictor
// (tgmg.hh:439, tgmg.in.cc:266), v_cycle() (tgmg.in.cc:313), l2_error()
// (tgmg.hh:146).  src and vel are m*(n+1) (x,y) pairs.
class tgmg_qs {
  public:
    tgmg_qs(shear_sim &s, double dt) : sim(s), dt(dt) {}
    int setup() {
        int nl = 0;
        check_or_exit(stzg_mg_levels(sim.handle(), dt, &nl, nullptr));
        return nl;
    }
    bool solve_v_cycle(const double *src, double *vel, int *ncycles = nullptr) {
        int st = stzg_mg_solve(sim.handle(), dt, src, vel, ncycles);
        if (st == STZG_ENOTCONV || st == STZG_ENAN) return false;
        check_or_exit(st);
        return true;
    }
    void v_cycle(const double *src, double *vel) { check_or_exit(stzg_mg_vcycle(sim.handle(), dt, src, vel)); }
    double l2_error(const double *src, const double *vel) {
        double e = 0;
        check_or_exit(stzg_mg_l2_error(sim.handle(), dt, src, vel, &e));
        return e;
    }

  private:
    shear_sim &sim;
    double dt;
};

}  // namespace stzg

#endif
