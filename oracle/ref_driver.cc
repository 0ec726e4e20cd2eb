// Test-only C-ABI driver around the reference implementation itself.
//
// This file is compiled by oracle/build_ref.sh together with the reference
// sources (esim/sb/main/shear_sim.cc, qs_multi.cc, common.cc and the tgmg.cc
// that esim/tgmg/tgmg_compile.pl generates) into oracle/_ref/libstzref.so.
// Only the tests and the golden-fixture script load it, to pin the oracle
// restatement (oracle/stz_oracle.c) and the GPU path against the reference's
// own shear_sim::step_forward_quasistatic (esim/sb/main/shear_sim.cc:280).
//
// The reference keeps its multigrid problem class private inside shear_sim
// (shear_sim.hh:128) and exposes no way to tighten the solver tolerance
// (qs_multi.cc:14 hard-codes the 1e4 multiplier).  To run it as a parity
// oracle with a tighter tolerance, and to read its coarse-grid stencils, this
// translation unit opens the private members.  It never changes the
// reference's arithmetic.
#include <vector>

#define private public
#include "shear_sim.hh"
#undef private

#include <cstring>
#include <cfloat>
#include <sys/time.h>

// Layout of the parameter block shared with the oracle and the product
// (stz_params in include/stzg.h; same member order).
struct ref_params {
    int m, n, stz_model, t_model;
    double ax, bx, ay, by;
    double mu, K, viscosity, chi_diff, chi_len, t_scale, adapt_fac, u_bdry;
    double TZ, c0, tau0, kappa, Delta, Omegaeps0, chi_inf, theta, rho, s_y;
};

struct ref_handle {
    stz_dynamics *stz;
    shear_sim *sim;
};

static double wall_seconds() {
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

extern "C" {

void *stzref_create(const ref_params *p) {
    ref_handle *h = new ref_handle;
    switch (p->stz_model) {
        case 0: h->stz = new stz_dynamics_linear(p->TZ, p->c0, p->tau0, p->kappa, p->Delta,
                                                 p->Omegaeps0, p->chi_inf, p->theta, p->rho); break;
        case 1: h->stz = new stz_dynamics_nonlinear(p->TZ, p->c0, p->tau0, p->kappa, p->Delta,
                                                    p->Omegaeps0, p->chi_inf, p->theta, p->rho); break;
        case 3: h->stz = new stz_dynamics_nonlinear_athermal(p->TZ, p->c0, p->tau0, p->kappa, p->Delta,
                                                             p->Omegaeps0, p->chi_inf, p->theta, p->rho); break;
        default: h->stz = new stz_dynamics_linear_athermal(p->TZ, p->c0, p->tau0, p->kappa, p->Delta,
                                                           p->Omegaeps0, p->chi_inf, p->theta, p->rho,
                                                           p->t_model); break;
    }
    h->sim = new shear_sim(p->m, p->n, p->ax, p->bx, p->ay, p->by, p->mu, p->K, p->viscosity,
                           p->chi_diff, p->chi_len, p->t_scale, 0.5, p->adapt_fac, p->u_bdry,
                           h->stz, "");
    h->sim->qsm.mg.verbose = 0;
    // Give every slot (ghost rows included) a defined value first.
    h->sim->init_fields(0, 600, 200);
    return h;
}

void stzref_destroy(void *vh) {
    ref_handle *h = (ref_handle *)vh;
    delete h->sim;
    delete h->stz;
    delete h;
}

// Initial state used by every fixture: zero velocity and stress, identity
// reference map, chi given per cell (m*n, row-major, row 0 at y=ay), ghost
// rows filled by the same linear extrapolation set_boundaries applies
// (shear_sim.cc:552-581) at time 0.
void stzref_set_state(void *vh, const double *chi) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    int m = s.m, n = s.n;
    for (int j = -1; j <= n; j++)
        for (int i = 0; i < m; i++) {
            c_field &f = s.fm[i + m * j];
            f.u = f.v = f.ddev = 0;
            f.p = f.q = f.s = f.tau = 0;
            f.X = s.ax + i * s.dx;
            f.Y = s.ay + j * s.dy;
            if (j >= 0 && j < n) f.chi = chi[i + m * j];
        }
    for (int i = 0; i < m; i++) {
        s.fm[i - m].chi = 2 * s.fm[i].chi - s.fm[i + m].chi;
        s.fm[i + m * n].chi = 2 * s.fm[i + m * (n - 1)].chi - s.fm[i + m * (n - 2)].chi;
    }
    for (int k = 0; k < m * (n + 1); k++) s.vel[k].x = s.vel[k].y = 0;
    s.time = 0;
}

// shear_sim::init_fields (shear_sim.cc:60-114) with the solver's velocity
// array cleared (the reference leaves it unset; set_state clears it too).
void stzref_init_fields(void *vh, int chi_case, double tem_base, double tem_delta) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    s.init_fields(chi_case, tem_base, tem_delta);
    for (int k = 0; k < s.m * (s.n + 1); k++) s.vel[k].x = s.vel[k].y = 0;
    s.time = 0;
}

// shear_sim::initialize_chi_bicubic (shear_sim.cc:832-909): chi of rows
// 0..n-1 from the bicubic interpolant of arr (mm x nn); the other fields as
// init_fields sets them.  Ghost rows of chi keep their previous values in the
// reference; here they get the linear extrapolation of set_boundaries, so
// that the state is defined.
void stzref_chi_bicubic(void *vh, int mm, int nn, const double *arr, double lo, double sca) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    std::vector<double> a(arr, arr + (size_t)mm * nn);
    s.initialize_chi_bicubic(mm, nn, a.data(), lo, sca);
    int m = s.m, n = s.n;
    for (int i = 0; i < m; i++) {
        s.fm[i - m].chi = 2 * s.fm[i].chi - s.fm[i + m].chi;
        s.fm[i + m * n].chi = 2 * s.fm[i + m * (n - 1)].chi - s.fm[i + m * (n - 2)].chi;
    }
    for (int k = 0; k < m * (n + 1); k++) s.vel[k].x = s.vel[k].y = 0;
    s.time = 0;
}

// shear_sim::l2_comparison (shear_sim.cc:460-502) of two reference runs.
void stzref_l2_comparison(void *va, void *vb, double *l2) {
    ((ref_handle *)va)->sim->l2_comparison(*((ref_handle *)vb)->sim, l2);
}

// Replaces the tolerance multiplier of qs_multi.cc:14 (default 1e4).
void stzref_set_acc_mult(void *vh, double mult) {
    qs_multi &q = ((ref_handle *)vh)->sim->qsm;
    const_cast<double &>(q.acc) = tgmg_accuracy(2 * (q.tmufac1 + q.tmufac2), mult);
}

double stzref_get_acc(void *vh) { return ((ref_handle *)vh)->sim->qsm.acc; }

// Runs nsteps quasi-static steps.  When eps_pl is non-NULL it accumulates the
// plastic strain increment ddev/(2 mu) of every cell after each step (the
// reference keeps only the per-step ddev, fields.hh:27).  Returns the total
// number of V-cycles (excluding the extra cycle per solve) and the wall time.
long stzref_steps(void *vh, double dt, int nsteps, double *eps_pl, double *seconds) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    long cycles = 0;
    double t0 = wall_seconds(), acc = 0;
    for (int k = 0; k < nsteps; k++) {
        double a = wall_seconds();
        s.step_forward_quasistatic(dt);
        acc += wall_seconds() - a;
        cycles += s.qsm.tp.vcount;
        s.qsm.tp.vcount = 0;
        s.qsm.tp.solves = 0;
        if (eps_pl)
            for (int c = 0; c < s.m * s.n; c++) eps_pl[c] += s.fm[c].ddev / (2 * s.mu);
    }
    (void)t0;
    if (seconds) *seconds = acc;
    return cycles;
}

// Runs nsteps explicit steps (shear_sim::step_forward, shear_sim.cc:185-276).
// The reference stores ddev times the old |s| there (shear_sim.cc:265); when
// eps_pl is non-NULL it accumulates the raw stress drop / (2 mu), recovered
// with the |s| of each cell before the step.
void stzref_steps_direct(void *vh, double dt, int nsteps, double *eps_pl) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    std::vector<double> dev(eps_pl ? (size_t)s.m * s.n : 0);
    for (int k = 0; k < nsteps; k++) {
        if (eps_pl)
            for (int c = 0; c < s.m * s.n; c++) dev[c] = s.fm[c].dev();
        s.step_forward(dt);
        if (eps_pl)
            for (int c = 0; c < s.m * s.n; c++)
                if (dev[c] > 0) eps_pl[c] += s.fm[c].ddev / dev[c] / (2 * s.mu);
    }
}

// The frame loop of shear_sim::solve (shear_sim.cc:120-140) up to target.
long stzref_advance_direct(void *vh, double dt, double target, double *eps_pl) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    long k = 0;
    while (s.time + dt * (1 + 1e-8) < target) {
        stzref_steps_direct(vh, dt, 1, eps_pl);
        k++;
    }
    stzref_steps_direct(vh, target - s.time, 1, eps_pl);
    return k + 1;
}

// shear_sim::output (shear_sim.cc:684-720): writes <dir>/<prefix>.<sn>.
void stzref_output(void *vh, const char *dir, const char *prefix, int mode, int sn) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    const char *old = s.filename;
    s.filename = dir;
    s.output(prefix, mode, sn);
    s.filename = old;
}

// shear_sim::qs_measure (shear_sim.cc:733-775); the integrand stays in cu.
void stzref_qs_measure(void *vh, int staggered, double *Q, double *max_qs) {
    ((ref_handle *)vh)->sim->qs_measure(*Q, *max_qs, staggered != 0);
}

// shear_sim::tractions (shear_sim.cc:1003-1028): out = bx, by, tx, ty.
void stzref_tractions(void *vh, double *out) {
    ((ref_handle *)vh)->sim->tractions(out[0], out[1], out[2], out[3]);
}

// shear_sim::compute_strain (shear_sim.cc:778-824): out = cu of rows 0..n-1.
void stzref_compute_strain(void *vh, double *out) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    s.compute_strain();
    for (int c = 0; c < s.m * s.n; c++) out[c] = s.fm[c].cu;
}

// Zeroes the cu slots (rows -1..n) so that the rows qs_measure leaves alone
// read 0 in an output of mode 11.
void stzref_clear_cu(void *vh) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    for (int c = -s.m; c < s.m * (s.n + 1); c++) s.fm[c].cu = 0;
}

double stzref_time(void *vh) { return ((ref_handle *)vh)->sim->time; }

// Field ids: 0 u, 1 v, 7 X, 8 Y are node fields with rows 0..n (m*(n+1));
// 2 p, 3 q, 4 s, 5 tau, 6 chi, 9 ddev are cell fields with rows -1..n
// (m*(n+2), ghost rows included).
void stzref_get(void *vh, int field, double *out) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    int m = s.m, n = s.n;
    bool node = field == 0 || field == 1 || field == 7 || field == 8;
    int j0 = node ? 0 : -1, j1 = node ? n : n;
    double *o = out;
    for (int j = j0; j <= j1; j++)
        for (int i = 0; i < m; i++) {
            c_field &f = s.fm[i + m * j];
            double v;
            switch (field) {
                case 0: v = f.u; break;
                case 1: v = f.v; break;
                case 2: v = f.p; break;
                case 3: v = f.q; break;
                case 4: v = f.s; break;
                case 5: v = f.tau; break;
                case 6: v = f.chi; break;
                case 7: v = f.X; break;
                case 8: v = f.Y; break;
                default: v = f.ddev; break;
            }
            *o++ = v;
        }
}

// Velocity solution array of the last projection (m*(n+1) vec, x then y).
void stzref_get_vel(void *vh, double *out) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    for (int k = 0; k < s.m * (s.n + 1); k++) {
        out[2 * k] = s.vel[k].x;
        out[2 * k + 1] = s.vel[k].y;
    }
}

// Multigrid hierarchy after setup: returns the number of coarse levels and
// fills dims with (m,n) per level.
int stzref_mg_levels(void *vh, double dt, int *dims) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    s.qsm.init(s.viscosity / dt);
    tgmg<qs_multi, vec, mat> &g = s.qsm.mg;
    for (int l = 0; l < g.ml; l++) {
        dims[2 * l] = g.mg[l]->m;
        dims[2 * l + 1] = g.mg[l]->n;
    }
    return g.ml;
}

// Coarse-level stencil storage of level l: 10 mats per point (dl,dc,dr,cl,
// cc,cr,ul,uc,ur, inverse of cc), each (a,b,c,d), tgmg.hh:244-265.
void stzref_mg_stencil(void *vh, int l, double *out) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    tgmg_level<vec, mat> *lv = s.qsm.mg.mg[l];
    for (int k = 0; k < 10 * lv->mn; k++) {
        out[4 * k] = lv->s[k].a;
        out[4 * k + 1] = lv->s[k].b;
        out[4 * k + 2] = lv->s[k].c;
        out[4 * k + 3] = lv->s[k].d;
    }
}

// Runs the reference multigrid solve (tgmg::solve_v_cycle with the adaptive
// predictor, tgmg.in.cc:266) on a caller-supplied right-hand side and initial
// guess, both m*(n+1) vec.  Returns 1 on success and the V-cycle count.
int stzref_mg_solve(void *vh, double dt, const double *src, double *vel, int *ncycles) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    s.qsm.init(s.viscosity / dt);
    int mn = s.m * (s.n + 1);
    for (int k = 0; k < mn; k++) {
        s.src[k].x = src[2 * k]; s.src[k].y = src[2 * k + 1];
        s.vel[k].x = vel[2 * k]; s.vel[k].y = vel[2 * k + 1];
    }
    s.qsm.tp.vcount = 0;
    bool ok = s.qsm.mg.solve_v_cycle(s.qsm.tp);
    if (ncycles) *ncycles = s.qsm.tp.vcount;
    for (int k = 0; k < mn; k++) {
        vel[2 * k] = s.vel[k].x; vel[2 * k + 1] = s.vel[k].y;
    }
    return ok ? 1 : 0;
}

// One plain V-cycle (tgmg.in.cc:313) on caller-supplied arrays.
void stzref_mg_vcycle(void *vh, double dt, const double *src, double *vel) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    s.qsm.init(s.viscosity / dt);
    int mn = s.m * (s.n + 1);
    for (int k = 0; k < mn; k++) {
        s.src[k].x = src[2 * k]; s.src[k].y = src[2 * k + 1];
        s.vel[k].x = vel[2 * k]; s.vel[k].y = vel[2 * k + 1];
    }
    s.qsm.mg.v_cycle();
    for (int k = 0; k < mn; k++) {
        vel[2 * k] = s.vel[k].x; vel[2 * k + 1] = s.vel[k].y;
    }
}

// Mean squared residual of the current src/vel, evaluated with the problem
// class's own inline operator (qs_multi.hh:41-50) as tgmg_base::mds does
// (tgmg.in.cc:55-64); mds itself is not exported by the reference objects.
double stzref_mg_l2_error(void *vh) {
    shear_sim &s = *((ref_handle *)vh)->sim;
    qs_multi &q = s.qsm;
    double c = 0;
    for (int j = 0; j < q.mn; j += q.m)
        for (int i = 0, ij = j; i < q.m; i++, ij++) {
            vec r = s.src[ij] - q.mul_a(i, ij) - q.a_cc(i, ij) * s.vel[ij];
            c += mod_sq(r);
        }
    return c / q.mn;
}

}  // extern "C"
