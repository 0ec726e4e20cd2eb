/* CPU oracle for the quasi-static STZ time step: TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithm (SURGroup/STZ,
 * esim/sb/main/shear_sim.cc, qs_multi.{hh,cc}, stz_model.hh and the tgmg
 * multigrid library esim/tgmg/tgmg.{hh,in.cc}).  Only the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it; the product never
 * links it.
 *
 * Parity of this restatement is pinned against the reference itself, built
 * from its sources into oracle/_ref/libstzref.so by oracle/build_ref.sh, and
 * against golden vectors the reference produced (tests/golden/).
 */
#ifndef STZ_ORACLE_H
#define STZ_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Same member order as stz_params in include/stzg.h. */
typedef struct {
    int m, n;          /* cells in x (periodic) and y (walls) */
    int stz_model;     /* 0 linear, 1 nonlinear, 2 linear athermal, 3 nonlinear athermal */
    int t_model;       /* truncation model of the linear athermal law (-1..4) */
    double ax, bx, ay, by;
    double mu, K, viscosity, chi_diff, chi_len, t_scale, adapt_fac, u_bdry;
    double TZ, c0, tau0, kappa, Delta, Omegaeps0, chi_inf, theta, rho, s_y;
} stzo_params;

typedef struct stzo_sim stzo_sim;

stzo_sim *stzo_create(const stzo_params *p);
void stzo_destroy(stzo_sim *s);
/* chi: m*n cells, row-major, row 0 at y=ay.  Zero velocity and stress,
 * identity reference map, extrapolated ghost rows. */
void stzo_set_state(stzo_sim *s, const double *chi);
/* Solver stopping rule.  mode 0: reference rule, mean squared residual below
 * (DBL_EPSILON*mult*2(tmufac1+tmufac2))^2 (qs_multi.cc:14).  mode 1:
 * ||r||_2 <= tol*||b||_2. */
void stzo_set_tolerance(stzo_sim *s, int mode, double value);
long stzo_steps(stzo_sim *s, double dt, int nsteps, double *eps_pl, double *seconds);
/* Explicit steps (shear_sim::step_forward) and the frame loop of
 * shear_sim::solve up to a target time. */
void stzo_steps_direct(stzo_sim *s, double dt, int nsteps, double *eps_pl);
long stzo_advance_direct(stzo_sim *s, double dt, double target, double *eps_pl);
double stzo_time(stzo_sim *s);
/* Field ids as oracle/ref_driver.cc: 0 u,1 v,7 X,8 Y node (m*(n+1));
 * 2 p,3 q,4 s,5 tau,6 chi,9 ddev cell with ghost rows (m*(n+2)). */
void stzo_get(stzo_sim *s, int field, double *out);
void stzo_set(stzo_sim *s, int field, const double *in);
/* shear_sim::init_fields (chi cases 0-2) and initialize_chi_bicubic: the
 * other fields at rest, solver array cleared, time 0. */
void stzo_init_fields(stzo_sim *s, int chi_case, double tem_base, double tem_delta);
void stzo_chi_bicubic(stzo_sim *s, int mm, int nn, const double *arr, double lo, double sca);
/* shear_sim::l2_comparison: l2[4] = (velocity, stress, chi, reference map). */
void stzo_l2_comparison(stzo_sim *a, stzo_sim *b, double *l2);
void stzo_get_vel(stzo_sim *s, double *out);
int stzo_mg_levels(stzo_sim *s, double dt, int *dims);
void stzo_mg_stencil(stzo_sim *s, int level, double *out);
int stzo_mg_solve(stzo_sim *s, double dt, const double *src, double *vel, int *ncycles);
void stzo_mg_vcycle(stzo_sim *s, double dt, const double *src, double *vel);
double stzo_mg_l2_error(stzo_sim *s);
void stzo_mg_residual_sqnorms(stzo_sim *s, double dt, const double *src, const double *vel, double *out);
/* Seeded Gaussian random chi field (initialize_random semantics,
 * shear_sim.cc:915-998) into out[m*n]. */
void stzo_random_chi(int m, int n, double l, double tem_avg, double tem_std, double TZ,
                     unsigned long long seed, double *out);
int stzo_threads(void);
void stzo_set_threads(int k);

#ifdef __cplusplus
}
#endif
#endif
