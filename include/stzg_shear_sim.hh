// stzg_shear_sim.hh - C++ drop-in for the reference's shear_sim class and
// its STZ law classes (esim/sb/main/shear_sim.hh:20-151,
// esim/sb/main/stz_model.hh:9-207), plus the tgmg solve it runs
// (esim/tgmg/tgmg.hh:286-495), on top of the C ABI in stzg.h.  Header-only;
// link with libstzg.so.
//
// The classes keep the reference's names, constructor arguments, public
// members and methods, so a reference driver compiles against them
// unchanged when include/dropin/shear_sim.hh stands in for the reference's
// shear_sim.hh (it brings these names into the global namespace).
//
// What differs, because the state lives on the GPU:
//   * fm, vel and src are host mirrors.  fetch_fields() copies the GPU state
//     into them, store_fields() copies fm's fields (u, v, p, q, s, tau, chi,
//     X, Y, ddev) back; the simulation methods never touch them.  compute_strain
//     writes its result into fm[].cu as the reference does (after a fetch).
//   * time is a plain public member as in the reference; every method sends
//     it to the GPU before it runs and reads it back afterwards, so drivers
//     can assign it (sim.time = 0) or hold a reference to it.
//   * chi_diffusion(dt) has no separate effect: the GPU advection step adds
//     the chi diffusion itself (the reference calls chi_diffusion from
//     advection_step, shear_sim.cc:352, and its only other effect is on the
//     change slot fm[].cchi).
//   * initialize_random draws from a counter-based generator seeded by
//     random_seed (default 1) instead of libc rand().
//   * Dplastic of the law classes is evaluated on the GPU only; the classes
//     here carry the parameters and name the law.
//
// Error behaviour follows the reference: a failed multigrid solve prints a
// message and exits with status 1, as qs_multi::solve does
// (qs_multi.hh:51-53); other failures do the same with the library message.
#ifndef STZG_SHEAR_SIM_HH
#define STZG_SHEAR_SIM_HH

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "stzg.h"

namespace stzg {

inline void check_or_exit(int st) {
    if (st != STZG_OK) {
        std::fprintf(stderr, "stzg: %s: %s\n", stzg_strerror(st), stzg_last_message());
        std::exit(1);
    }
}

// ---- STZ laws (stz_model.hh:9-207) ---------------------------------------
// Same constructors and public parameters as the reference's classes; law()
// and truncation() name the law for stz_params (stz_model, t_model).
class stz_dynamics {
  public:
    const double rt3, TZ, c0, tau0, kappa, Delta, Omegaeps0, chi_inf, thetainv, rho, s0;
    stz_dynamics(double TZ_, double c0_, double tau0_, double kappa_, double Delta_, double Omegaeps0_,
                 double chi_inf_, double theta, double rho_)
        : rt3(std::sqrt(3.0)), TZ(TZ_), c0(c0_), tau0(tau0_), kappa(kappa_), Delta(Delta_), Omegaeps0(Omegaeps0_),
          chi_inf(chi_inf_), thetainv(1 / theta), rho(rho_), s0(1) {}
    virtual ~stz_dynamics() {}
    virtual int law() const = 0;
    virtual int truncation() const { return -1; }
};

// stz_model.hh:50-68, thermal linear law.
class stz_dynamics_linear : public stz_dynamics {
  public:
    int t_model;
    stz_dynamics_linear(double TZ_, double c0_, double tau0_, double kappa_, double Delta_, double Omegaeps0_,
                        double chi_inf_, double theta, double rho_, int t_model_ = -1)
        : stz_dynamics(TZ_, c0_, tau0_, kappa_, Delta_, Omegaeps0_, chi_inf_, theta, rho_), t_model(t_model_) {}
    int law() const override { return 0; }
};

// stz_model.hh:70-88, thermal nonlinear law.
class stz_dynamics_nonlinear : public stz_dynamics {
  public:
    stz_dynamics_nonlinear(double TZ_, double c0_, double tau0_, double kappa_, double Delta_, double Omegaeps0_,
                           double chi_inf_, double theta, double rho_)
        : stz_dynamics(TZ_, c0_, tau0_, kappa_, Delta_, Omegaeps0_, chi_inf_, theta, rho_) {}
    int law() const override { return 1; }
};

// stz_model.hh:90-170, athermal linear law with its truncation models.
class stz_dynamics_linear_athermal : public stz_dynamics {
  public:
    int t_model;
    double t_icpt, t_grad;
    stz_dynamics_linear_athermal(double TZ_, double c0_, double tau0_, double kappa_, double Delta_,
                                 double Omegaeps0_, double chi_inf_, double theta, double rho_, int t_model_ = -1)
        : stz_dynamics(TZ_, c0_, tau0_, kappa_, Delta_, Omegaeps0_, chi_inf_, theta, rho_), t_model(t_model_),
          t_icpt(0), t_grad(0.5 * Omegaeps0_ / Delta_) {}
    int law() const override { return 2; }
    int truncation() const override { return t_model; }
};

// stz_model.hh:172-207, athermal nonlinear law.
class stz_dynamics_nonlinear_athermal : public stz_dynamics {
  public:
    stz_dynamics_nonlinear_athermal(double TZ_, double c0_, double tau0_, double kappa_, double Delta_,
                                    double Omegaeps0_, double chi_inf_, double theta, double rho_)
        : stz_dynamics(TZ_, c0_, tau0_, kappa_, Delta_, Omegaeps0_, chi_inf_, theta, rho_) {}
    int law() const override { return 3; }
};

// ---- fields (fields.hh:7-114, vec.hh) -----------------------------------
// The reference's per-point record, member for member (152 bytes).
struct c_field {
    double u, v, p, q, s, tau, chi, X, Y, ddev;
    double cu, cv, cp, cs, cq, ctau, cchi, cX, cY;
    inline double devsq() { return 3 * q * q + s * s + tau * tau; }
    inline double dev() { return std::sqrt(devsq()); }
    inline double sxx() { return -p + s - q; }
    inline double syy() { return -p - s - q; }
    inline double fval(int i) {
        const double f[9] = {u, v, p, q, s, tau, chi, X, Y};
        return i >= 0 && i < 9 ? f[i] : dev();
    }
};

struct vec {
    double x, y;
};

// ---- the simulation (shear_sim.hh:20-151) -------------------------------
class shear_sim {
  public:
    const int m, n, mn;
    const double ax, ay, bx, by, lx, ly, dx, dy, xsp, ysp, mu, mu_inv, K, viscosity, chi_diff, chi_len, t_scale,
        tmult, adapt_fac, u_bdry, bcs;
    stz_dynamics *stz;
    const char *filename;
    // host mirrors (see the file comment): fm has rows -1..n like the reference
    c_field *const fm;
    vec *const vel;
    vec *const src;
    double time;
    double TZ;
    double chi_inf;
    int f_num;
    // seed of initialize_random's counter-based generator
    unsigned long long random_seed = 1;

    shear_sim(const int m_, const int n_, const double ax_, const double bx_, const double ay_, const double by_,
              const double mu_, const double K_, const double visc_, const double chi_diff_, const double chi_len_,
              const double t_scale_, const double tmult_, const double adapt_fac_, const double u_bdry_,
              stz_dynamics *stz_, const char *filename_, const stzg_options *opt = nullptr)
        : m(m_), n(n_), mn(m_ * n_), ax(ax_), ay(ay_), bx(bx_), by(by_), lx(bx_ - ax_), ly(by_ - ay_),
          dx(lx / m_), dy(ly / n_), xsp(1. / dx), ysp(1. / dy), mu(mu_), mu_inv(1 / mu_), K(K_), viscosity(visc_),
          chi_diff(chi_diff_), chi_len(chi_len_), t_scale(t_scale_), tmult(tmult_), adapt_fac(adapt_fac_),
          u_bdry(u_bdry_), bcs(4), stz(stz_), filename(filename_), fm(new c_field[(size_t)m_ * (n_ + 2)] + m_),
          vel(new vec[(size_t)m_ * (n_ + 1)]), src(new vec[(size_t)m_ * (n_ + 1)]), time(0), TZ(stz_->TZ),
          chi_inf(stz_->chi_inf), f_num(0), h(nullptr) {
        stz_params p;
        p.m = m_;
        p.n = n_;
        p.stz_model = stz_->law();
        p.t_model = stz_->truncation();
        p.ax = ax_; p.bx = bx_; p.ay = ay_; p.by = by_;
        p.mu = mu_; p.K = K_; p.viscosity = visc_; p.chi_diff = chi_diff_; p.chi_len = chi_len_;
        p.t_scale = t_scale_; p.adapt_fac = adapt_fac_; p.u_bdry = u_bdry_;
        p.TZ = stz_->TZ; p.c0 = stz_->c0; p.tau0 = stz_->tau0; p.kappa = stz_->kappa; p.Delta = stz_->Delta;
        p.Omegaeps0 = stz_->Omegaeps0; p.chi_inf = stz_->chi_inf; p.theta = 1 / stz_->thetainv; p.rho = stz_->rho;
        p.s_y = stz_->s0;
        params = p;
        check_or_exit(stzg_create(&params, opt, &h));
    }
    ~shear_sim() {
        stzg_destroy(h);
        delete[] src;
        delete[] vel;
        delete[] (fm - m);
    }
    shear_sim(const shear_sim &) = delete;
    shear_sim &operator=(const shear_sim &) = delete;

    // -- set-up (shear_sim.cc:60-114, 832-909, 932-984) --
    void init_fields(int chi_case, double tem_base = 600, double tem_delta = 200) {
        check_or_exit(stzg_init_fields(h, chi_case, tem_base, tem_delta));
        pull_time();
    }
    void initialize_chi_bicubic(int mm, int nn, double *arr, double lo = 0, double sca = 1) {
        check_or_exit(stzg_chi_bicubic(h, mm, nn, arr, lo, sca));
        pull_time();
    }
    void initialize_random(double l, double tem_avg, double tem_stdev) {
        std::vector<double> chi((size_t)m * n);
        check_or_exit(stzg_random_chi(m, n, l, tem_avg, tem_stdev, TZ, random_seed, chi.data()));
        check_or_exit(stzg_set_state(h, chi.data()));
        pull_time();
    }
    // chi of every cell (m*n, row 0 at y=ay), the other fields at rest
    void set_chi(const double *chi) {
        check_or_exit(stzg_set_state(h, chi));
        pull_time();
    }

    // -- time stepping (shear_sim.cc:120-386) --
    void step_forward_quasistatic(double dt) {
        push_time();
        check_or_exit(stzg_step_qs(h, dt, 1, nullptr));
        pull_time();
    }
    void step_forward(double dt) {
        push_time();
        check_or_exit(stzg_step_direct(h, dt, 1, nullptr));
        pull_time();
    }
    void advection_step(double dt) {
        push_time();
        check_or_exit(stzg_advection_step(h, dt));
    }
    void chi_diffusion(double) {}
    void projection_step(double dt) {
        push_time();
        check_or_exit(stzg_projection_step(h, dt, nullptr));
    }
    // shear_sim::solve (shear_sim.cc:120-157): explicit steps of dx^2 tmult
    // landing on every frame time, files written after every frame.
    void solve(double duration, int frames) {
        const double dt = dx * dx * tmult, t_start = time;
        if (f_num == 0) {
            write_files(0);
            std::puts("# Output frame 0");
        }
        double t0 = wtime();
        for (int k = 1; k <= frames; k++) {
            push_time();
            long l = 0;
            check_or_exit(stzg_advance_direct(h, dt, t_start + duration / frames * k, &l));
            pull_time();
            const double t1 = wtime();
            write_files(k + f_num);
            const double t2 = wtime();
            std::printf("# Output frame %d [%ld, %.8g s, %.8g s]\n", k + f_num, l, t1 - t0, t2 - t1);
            t0 = t2;
        }
        f_num += frames;
    }
    // shear_sim::solve_quasistatic (shear_sim.cc:159-181).
    void solve_quasistatic(double duration, int frames, int steps) {
        const double dt = duration / frames * (1.0 / steps);
        if (f_num == 0) {
            write_files(0);
            std::puts("# Output frame 0");
        }
        double t0 = wtime();
        for (int k = 1; k <= frames; k++) {
            push_time();
            check_or_exit(stzg_step_qs(h, dt, steps, nullptr));
            pull_time();
            const double t1 = wtime();
            write_files(k + f_num);
            const double t2 = wtime();
            std::printf("# Output frame %d [%d, %.8g s, %.8g s] {%.2f}\n", k + f_num, steps, t1 - t0, t2 - t1,
                        avg_iters());
            t0 = t2;
        }
        f_num += frames;
    }

    // -- output and diagnostics (shear_sim.cc:460-502, 659-824, 1003-1028) --
    // Fields 4|128|256|512|1024 (p, tem, dev, X, Y) into the directory
    // `filename`, as <field>.<k>.
    void write_files(int k) {
        push_time();
        check_or_exit(stzg_write_frame(h, filename, k, 4 | 128 | 256 | 512 | 1024, nullptr));
    }
    void compute_strain() {
        std::vector<double> e((size_t)m * n);
        check_or_exit(stzg_compute_strain(h, e.data()));
        for (size_t c = 0; c < e.size(); c++) fm[c].cu = e[c];
    }
    void qs_measure(double &Q, double &max_qs, bool staggered = false) {
        check_or_exit(stzg_qs_measure(h, staggered ? 1 : 0, &Q, &max_qs));
    }
    void tractions(double &bx_, double &by_, double &tx, double &ty) {
        double t[4];
        check_or_exit(stzg_tractions(h, t));
        bx_ = t[0];
        by_ = t[1];
        tx = t[2];
        ty = t[3];
    }
    void l2_comparison(shear_sim &ss, double *l2) { check_or_exit(stzg_l2_comparison(h, ss.h, l2)); }
    double avg_iters() {
        double a = 0;
        check_or_exit(stzg_avg_iters(h, &a));
        return a;
    }
    inline double bdry_vel() { return time < 1 ? time * u_bdry : u_bdry; }
    inline double bdry_pos() { return time < 1 ? u_bdry * time * time * 0.5 : u_bdry * (time - 0.5); }

    // -- host mirrors --
    // GPU state -> fm (rows -1..n; node fields on rows 0..n), vel, src.
    void fetch_fields() {
        pull_time();
        const size_t cells = (size_t)m * (n + 2), nodes = (size_t)m * (n + 1);
        std::vector<double> a(cells);
        const int cell_ids[6] = {STZG_P, STZG_Q, STZG_S, STZG_TAU, STZG_CHI, STZG_DDEV};
        double c_field::*cell_mem[6] = {&c_field::p, &c_field::q, &c_field::s, &c_field::tau, &c_field::chi,
                                        &c_field::ddev};
        c_field *f0 = fm - m;
        for (int k = 0; k < 6; k++) {
            check_or_exit(stzg_get_field(h, cell_ids[k], a.data()));
            for (size_t c = 0; c < cells; c++) f0[c].*cell_mem[k] = a[c];
        }
        const int node_ids[4] = {STZG_U, STZG_V, STZG_X, STZG_Y};
        double c_field::*node_mem[4] = {&c_field::u, &c_field::v, &c_field::X, &c_field::Y};
        for (int k = 0; k < 4; k++) {
            check_or_exit(stzg_get_field(h, node_ids[k], a.data()));
            for (size_t c = 0; c < nodes; c++) fm[c].*node_mem[k] = a[c];
        }
        for (size_t c = 0; c < nodes; c++) {
            vel[c].x = fm[c].u;
            vel[c].y = fm[c].v;
        }
    }
    // fm -> GPU state (the same fields; time from the member).
    void store_fields() {
        push_time();
        const size_t cells = (size_t)m * (n + 2), nodes = (size_t)m * (n + 1);
        std::vector<double> a(cells);
        const int cell_ids[6] = {STZG_P, STZG_Q, STZG_S, STZG_TAU, STZG_CHI, STZG_DDEV};
        double c_field::*cell_mem[6] = {&c_field::p, &c_field::q, &c_field::s, &c_field::tau, &c_field::chi,
                                        &c_field::ddev};
        const c_field *f0 = fm - m;
        for (int k = 0; k < 6; k++) {
            for (size_t c = 0; c < cells; c++) a[c] = f0[c].*cell_mem[k];
            check_or_exit(stzg_set_field(h, cell_ids[k], a.data()));
        }
        const int node_ids[4] = {STZG_U, STZG_V, STZG_X, STZG_Y};
        double c_field::*node_mem[4] = {&c_field::u, &c_field::v, &c_field::X, &c_field::Y};
        for (int k = 0; k < 4; k++) {
            for (size_t c = 0; c < nodes; c++) a[c] = fm[c].*node_mem[k];
            check_or_exit(stzg_set_field(h, node_ids[k], a.data()));
        }
    }
    // One field with the ids of stzg.h (layouts as stzg_get_field).
    std::vector<double> field(int id) {
        size_t cnt = (id == STZG_U || id == STZG_V || id == STZG_X || id == STZG_Y) ? (size_t)m * (n + 1)
                     : id == STZG_EPS_PL                                            ? (size_t)m * n
                                                                                    : (size_t)m * (n + 2);
        std::vector<double> v(cnt);
        check_or_exit(stzg_get_field(h, id, v.data()));
        return v;
    }

    stzg_sim *handle() { return h; }

  private:
    stz_params params;
    stzg_sim *h;
    void push_time() { check_or_exit(stzg_set_time(h, time)); }
    void pull_time() { check_or_exit(stzg_get_time(h, &time)); }
    static double wtime() {
#ifdef _OPENMP
        return omp_get_wtime();
#else
        return 0;
#endif
    }
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
