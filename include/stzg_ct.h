/* stzg_ct.h - C ABI of the quasi-static STZ step in sheared coordinates on one GPU.
 *
 * Stands in for the coord_transforms variant of the simulation
 * (esim/coord_transforms/simple_shear/shear_sim.{hh,cc}): the grid follows a
 * simple shear of rate lamb (lt = lamb * time enters the stress equations,
 * the deviatoric norm and the elasticity operator), x is periodic and y is
 * periodic (y_prd) or bounded by walls moving at +-u_bdry.  One handle owns
 * the fields in device memory with the reference's two ghost layers, the
 * 2x2-block multigrid of stzg_tgmg.h for the projection (its operator rebuilt
 * every step, as qs_multi::init does) and a CUDA stream.  Statuses and
 * messages are those of stzg.h.
 */
#ifndef STZG_CT_H
#define STZG_CT_H

#ifdef __cplusplus
extern "C" {
#endif

/* shear_sim constructor arguments (shear_sim.hh:157-161) and the STZ law
 * (stz_model.hh: stz_model 0 linear, 1 nonlinear, 2 linear athermal,
 * 3 nonlinear athermal; s0 = 1 in this variant). */
typedef struct {
    int m, n, y_prd, stz_model, t_model;
    double ax, bx, ay, by;
    double mu, K, viscosity, chi_len, t_scale, adapt_fac, u_bdry, lamb;
    double TZ, c0, tau0, kappa, Delta, Omegaeps0, chi_inf, theta, rho;
} stzg_ct_params;

typedef struct stzg_ct stzg_ct;

/* Field ids for stzg_ct_set_field / stzg_ct_get_field: the c_field members
 * (fields.hh:15-35).  Arrays hold rows 0..n (n+1 rows of m): nodes (u, v, X,
 * Y) at the grid corners, cells (p, q, s, tau, chi, ddev) at the centres; a
 * cell row n is the first ghost row. */
enum { STZG_CT_U = 0, STZG_CT_V, STZG_CT_P, STZG_CT_Q, STZG_CT_S, STZG_CT_TAU, STZG_CT_CHI, STZG_CT_X, STZG_CT_Y,
       STZG_CT_DDEV, STZG_CT_FIELDS };

int stzg_ct_create(const stzg_ct_params *p, int device, stzg_ct **out);
int stzg_ct_destroy(stzg_ct *s);
/* shear_sim::init_fields(chi_case, tem_base, tem_delta) (shear_sim.cc:59-131). */
int stzg_ct_init_fields(stzg_ct *s, int chi_case, double tem_base, double tem_delta);
/* shear_sim::initialize_chi_bicubic(mm, nn, arr, lo, sca) (shear_sim.cc:
 * 1067-1134): chi of the cells = lo + sca * the bicubic interpolant of arr
 * (mm x nn samples over the domain, row-major, periodic in x and, when y_prd,
 * in y; nn >= 2), then set_boundaries; the other fields are unchanged. */
int stzg_ct_chi_bicubic(stzg_ct *s, int mm, int nn, const double *arr, double lo, double sca);
/* Copies one field in or out (rows 0..n).  set_field re-applies the
 * boundary conditions (set_boundaries, shear_sim.cc:778-811). */
int stzg_ct_set_field(stzg_ct *s, int field, const double *host);
int stzg_ct_get_field(stzg_ct *s, int field, double *host);
int stzg_ct_set_time(stzg_ct *s, double time);
/* The projection's solve: STZG_FP64 (0, the default) or STZG_MIXED (1) of
 * stzg.h, FP32 V-cycles inside FP64 refinement (stzg_tgmg_set_precision),
 * converged to the same threshold on the FP64 residual. */
int stzg_ct_set_precision(stzg_ct *s, int precision);
/* How many V-cycles the projection's solve runs: 0 (the default) the
 * reference's tgmg_predict counts (qs_multi::solve, tgmg.in.cc:266-301),
 * which over-solve while the prediction settles; 1 V-cycles until the
 * residual meets the same threshold, tested after each
 * (stzg_tgmg_solve_checked), then the extra one. */
int stzg_ct_set_solve_policy(stzg_ct *s, int policy);
int stzg_ct_get_time(stzg_ct *s, double *time);
/* nsteps of shear_sim::step_forward_quasistatic(dt) (shear_sim.cc:352-360):
 * advection_step (ENO2 advection, STZ plasticity, chi diffusion, updates,
 * time, boundaries), projection_step (operator for the new lt, source,
 * multigrid solve, stress correction, velocities, boundaries).  vcycles
 * (optional) receives the V-cycles counted by the solver's tgmg_predict;
 * seconds (optional) the device time. */
int stzg_ct_step_qs(stzg_ct *s, double dt, int nsteps, long *vcycles, double *seconds);

/* No counterpart in the reference, whose calibration harness (pfn.py through
 * UQpy's RunModel) runs one simulation per parameter sample, one after the
 * other.  Advances `count` independent handles (any sizes and parameters, all
 * on one device) by nsteps quasi-static steps of dt each, driven from
 * `threads` host threads (0: min(count, 16)); every handle keeps its own
 * stream, so their kernels, host-side operator updates and solver checks
 * overlap.  Each handle's result equals stzg_ct_step_qs on it alone.
 * vcycles (optional, count entries) receives each handle's V-cycles;
 * seconds (optional) the wall time of the whole batch.  On failure no further
 * handle is started, the threads finish the handles they hold, and the
 * status and message of the lowest-numbered failing handle are returned;
 * its state is as stzg_ct_step_qs leaves it. */
int stzg_ct_batch_step_qs(stzg_ct *const *handles, int count, double dt, int nsteps, int threads, long *vcycles,
                          double *seconds);

/* nsteps of shear_sim::step_forward(dt) (shear_sim.cc:218-349), the explicit
 * step: upwinded ENO2 advection of velocity, reference map, stresses and chi,
 * net force and viscous terms in sheared coordinates, the full elastic stress
 * update with STZ plasticity, chi diffusion, then time and boundaries (row 0's
 * nodes keep their values, as update_staggered leaves them).  seconds
 * (optional) receives the device time. */
int stzg_ct_step_direct(stzg_ct *s, double dt, int nsteps, double *seconds);

/* Lagrangian tracers.  stzg_ct_tracers_init: shear_sim::initialize_tracers(mm,
 * nn) (shear_sim.cc:1247-1283): mm x nn tracers at the cell centres of an
 * mm x nn grid of the domain, their reference points equal to their
 * positions, created at the current time.  stzg_ct_tracers_update:
 * shear_sim::update_tracers (shear_sim.cc:1286-1316) with correct_tracer
 * (:1322-1355): each tracer's position is predicted from its velocity
 * estimate and corrected by Newton iterations on the bicubic interpolant of
 * the reference map (bi_interp.cc), and the velocity estimate is (new - old
 * position) / (time since creation); tracers whose Newton iteration fails are
 * dropped in the reference's order and counted in *lost (optional).  A
 * tracer whose interpolation leaves the grid (the reference stops the
 * program) gives STZG_EINVAL.  stzg_ct_tracers_get: *count tracers, the first
 * min(cap, count) copied to out as (x_ref, y_ref, x, y, v_x, v_y). */
int stzg_ct_tracers_init(stzg_ct *s, int mm, int nn);
int stzg_ct_tracers_update(stzg_ct *s, int *lost);
int stzg_ct_tracers_get(stzg_ct *s, double *out, int cap, int *count);

/* Frames and diagnostics.  stzg_ct_compute_strain: shear_sim::compute_strain
 * (shear_sim.cc:1008-1059) with set_strain_boundaries (:814-850): per cell the
 * Green-Lagrange strain of the physical deformation (the sheared grid's
 * (1 lt; 0 1) applied to the inverse reference-map gradient): out holds six
 * arrays of rows 0..n (m each): E_xx, E_xy, E_yy, the trace, the second
 * invariant and the deviatoric norm.  stzg_ct_output_field: shear_sim::output
 * (shear_sim.cc:937-1004) of one mode (0 u, 1 v, 2 p, 3 q, 4 s, 5 tau, 6 chi,
 * 7 chi*TZ, 8 the untransformed deviatoric norm, 9 X, 10 Y, 11-16 the six
 * strain values) as the Gnuplot binary matrix the reference writes (header
 * row, then rows led by their y); *count receives the number of floats, out
 * may be NULL to query it.  stzg_ct_write_frame: shear_sim::write_files
 * (shear_sim.cc:892-931) into dir with the reference's flags (bit k: mode k
 * for k <= 10, dev always; 2048 Exx, Exy, Eyy; 4096 E_I, E_II, Edev; 8192
 * the tracers: update them when frame > 0, then tra.<frame> (text: position,
 * reference point, p, chi, chi*TZ and the six strain values by bicubic
 * interpolation) and teml.<frame> (chi*TZ on the tracer grid)); files are
 * <dir>/<name>.<frame>, byte for byte the reference's for the same state.
 * stzg_ct_solve_quasistatic / stzg_ct_solve: the frame loops of
 * shear_sim::solve_quasistatic (shear_sim.cc:175-202) and shear_sim::solve
 * (:133-172): frame 0 (quasi-static: only on the handle's first loop), then
 * per frame the steps and the frame's files; verbose prints the reference's
 * frame lines. */
int stzg_ct_compute_strain(stzg_ct *s, double *out);
int stzg_ct_output_field(stzg_ct *s, int mode, float *out, long *count);
int stzg_ct_write_frame(stzg_ct *s, const char *dir, int frame, unsigned fflags);
int stzg_ct_solve_quasistatic(stzg_ct *s, double duration, int frames, int steps, const char *dir,
                              unsigned fflags, int verbose);
int stzg_ct_solve(stzg_ct *s, double duration, int frames, const char *dir, unsigned fflags, int verbose);
/* shear_sim::l2_comparison_transform (shear_sim.cc:619-711): s in the
 * sheared frame against phys in the physical frame (lamb = 0, same grid):
 * phys's u, v, p, q, s, tau, chi interpolated bilinearly (bilin_interp,
 * :713-736) at the sheared node positions; l2[4] = velocity, stress, chi,
 * reference map, with the reference's weights, times dx dy.  A shift past
 * the ghost columns (where the reference reads outside its arrays) gives
 * STZG_EINVAL. */
int stzg_ct_l2_comparison_transform(stzg_ct *s, stzg_ct *phys, double *l2);

#ifdef __cplusplus
}
#endif

#endif /* STZG_CT_H */
