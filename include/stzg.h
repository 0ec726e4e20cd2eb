/* stzg.h - C ABI of the GB300-native quasi-static STZ time step.
 *
 * One handle (stzg_sim) owns one simulation on one GPU: its fields in HBM,
 * its multigrid hierarchy, its CUDA stream and captured graphs.  Host arrays
 * passed in are copied; the caller keeps ownership.  Every entry point returns
 * an int status (STZG_OK on success) and never exits the process.
 *
 * Each entry point names the reference interface it stands in for
 * (paths inside the SURGroup/STZ tree).
 */
#ifndef STZG_H
#define STZG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------
 * The reference exits the process on a failed solve (qs_multi.hh:51-53,
 * tgmg.in.cc:285-287) and on file errors (common.cc:12-29). */
enum {
    STZG_OK = 0,
    STZG_EINVAL = 1,        /* bad argument or unsupported configuration */
    STZG_ENOMEM = 2,        /* device allocation failed */
    STZG_ECUDA = 3,         /* CUDA runtime error */
    STZG_ENOTCONV = 4,      /* multigrid did not reach the tolerance (tgmg.in.cc:285) */
    STZG_ENAN = 5,          /* NaN residual (tgmg.in.cc:300) */
    STZG_ESUBSTEP = 6,      /* plastic sub-stepping hit its iteration cap */
    STZG_ENODEV = 7         /* no usable sm_103 device */
};

/* ---- parameters ---------------------------------------------------------
 * shear_sim constructor arguments (shear_sim.hh:95-99) and the STZ law
 * (stz_model.hh:9-207).  s_y is the yield stress, hard-wired to 1 in the
 * reference (stz_model.hh:26, :111). */
typedef struct {
    int m, n;          /* cells in x (periodic) and y (walls at ay, by) */
    int stz_model;     /* 0 linear, 1 nonlinear, 2 linear athermal, 3 nonlinear athermal */
    int t_model;       /* truncation model of the linear athermal law (-1..4) */
    double ax, bx, ay, by;
    double mu, K, viscosity, chi_diff, chi_len, t_scale, adapt_fac, u_bdry;
    double TZ, c0, tau0, kappa, Delta, Omegaeps0, chi_inf, theta, rho, s_y;
} stz_params;

enum { STZG_FP64 = 0, STZG_MIXED = 1 };
enum { STZG_TOL_REFERENCE = 0, STZG_TOL_RELATIVE = 1 };

typedef struct {
    int precision;     /* STZG_FP64: FP64 V-cycles; STZG_MIXED: FP32 V-cycles inside
                          FP64 iterative refinement */
    int tol_mode;      /* STZG_TOL_REFERENCE: mean squared residual below
                          (DBL_EPSILON*tol*2(tmufac1+tmufac2))^2, qs_multi.cc:14 with
                          tol the multiplier (1e4 there);  STZG_TOL_RELATIVE:
                          ||b-Az||_2 <= tol*||b||_2 */
    double tol;
    int track_plastic; /* accumulate eps_pl = sum ddev/(2 mu) per cell */
    int device;        /* CUDA device ordinal */
    int inner_cycles;  /* mixed precision: FP32 V-cycles per refinement pass (0: auto, 3) */
    int use_graphs;    /* capture the V-cycle in a CUDA graph (1 default) */
    int extrapolate;   /* initial guess of each solve instead of the previous solution
                          v(n) (tgmg keeps z between solves): 1 = linear, 2v(n) - v(n-1);
                          2 = quadratic, 3v(n) - 3v(n-1) + v(n-2) */
    int substep_cap;   /* iteration cap of the plastic sub-stepping per cell and step
                          (0: 4194304); reaching it returns STZG_ESUBSTEP */
    int advection;     /* Mixed-precision handles: STZG_ADV_AUTO (0) or STZG_ADV_SPLIT run the
                          advection, the projection source and the stress correction in
                          float-float arithmetic (pairs of floats, ~2^-44 relative) on the
                          FP64 state, each field updated by one FP64 addition, with the ENO
                          choices of the FP64 path wherever the two candidates differ by
                          more than 1e-10 of the field's scale; STZG_ADV_FP64 keeps them
                          FP64.  FP64
                          handles always run them in FP64, bit-exact with the per-point
                          ENO2. */
    int reserved[5];
} stzg_options;

enum { STZG_ADV_AUTO = 0, STZG_ADV_FP64 = 1, STZG_ADV_SPLIT = 2 };

typedef struct {
    long vcycles;      /* V-cycles counted like tgmg_predict::add_iters (tgmg_predict.hh:24) */
    long extra_vcycles;/* the extra cycle run after convergence (tgmg_config.hh:45) */
    long solves;
    long refinements;  /* FP64 outer passes (mixed precision) */
    long checks;       /* residual evaluations */
    double last_error; /* last convergence measure */
    double seconds;    /* device time of the stepped region (CUDA events) */
    long substeps_max; /* largest plastic sub-step count seen (reported when tracked) */
    long kernel_launches; /* kernels this library launched (graph nodes included) */
} stzg_stats;

/* Field ids, shared with the oracle: node fields (m x (n+1), rows 0..n):
 * 0 u, 1 v, 7 X, 8 Y.  Cell fields (m x (n+2), rows -1..n with the ghost
 * rows): 2 p, 3 q, 4 s, 5 tau, 6 chi, 9 ddev.  10 eps_pl (m x n). */
enum { STZG_U = 0, STZG_V = 1, STZG_P = 2, STZG_Q = 3, STZG_S = 4, STZG_TAU = 5,
       STZG_CHI = 6, STZG_X = 7, STZG_Y = 8, STZG_DDEV = 9, STZG_EPS_PL = 10 };

typedef struct stzg_sim stzg_sim;

void stzg_default_options(stzg_options *opt);
const char *stzg_strerror(int status);
/* Last CUDA or validation message of this thread. */
const char *stzg_last_message(void);

/* Replaces: shear_sim::shear_sim (shear_sim.cc:26-44) together with
 * qs_multi::qs_multi (qs_multi.cc:9-15) and tgmg::tgmg (tgmg.in.cc:11-30). */
int stzg_create(const stz_params *p, const stzg_options *opt, stzg_sim **out);
/* Replaces: shear_sim::~shear_sim (shear_sim.cc:47-52). */
int stzg_destroy(stzg_sim *s);

/* Initial state used by the reference drivers after initialize_random
 * (shear_sim.cc:932-984): zero velocity and stress, identity reference map,
 * chi per cell (m*n, row 0 at y=ay), ghost rows extrapolated as
 * set_boundaries (shear_sim.cc:552-581); time reset to 0. */
int stzg_set_state(stzg_sim *s, const double *chi);
/* Field access: write/read the public c_field members (fields.hh:7-114)
 * and shear_sim::time (shear_sim.hh:87).  Layouts as the field ids above. */
int stzg_set_field(stzg_sim *s, int field, const double *host);
int stzg_get_field(stzg_sim *s, int field, double *host);
/* Replaces: shear_sim::init_fields (shear_sim.cc:60-114): zero velocity
 * and stress, identity reference map, time 0, and chi from one of the
 * reference's set-ups (0 a Gaussian blip at the origin, 1 a line at 30
 * degrees, any other value sixteen blips along a sine wave) of height
 * tem_delta over tem_base (Kelvin), ghost rows included. */
int stzg_init_fields(stzg_sim *s, int chi_case, double tem_base, double tem_delta);
/* Replaces: shear_sim::initialize_chi_bicubic (shear_sim.cc:832-909): chi
 * of the cells = lo + sca * the bicubic interpolant of arr (mm x nn,
 * row-major, periodic in x, nn >= 2) stretched over the domain; the other
 * fields as stzg_init_fields.  The reference leaves chi's ghost rows as they
 * were; here they get set_boundaries' linear extrapolation. */
int stzg_chi_bicubic(stzg_sim *s, int mm, int nn, const double *arr, double lo, double sca);
int stzg_set_time(stzg_sim *s, double time);
int stzg_get_time(stzg_sim *s, double *time);

/* Bulk state transfer for callers that keep the fields in host memory, as
 * the reference does (shear_sim::fm, vel, shear_sim.hh:79-82).  up[8]:
 * p, q, s, tau, chi (m*(n+2) with ghost rows), X, Y (m*(n+1)), vel
 * (m*(n+1) x,y pairs, the solver array).  down[9]: the same plus eps_pl
 * (m*n).  Entries may be NULL to skip a field.  Time and wall speed are
 * kept.  An uploaded vel that is bit-identical to the device's keeps the
 * solver's history for extrapolated initial guesses; any other vel restarts
 * it.  Pinned host memory gives full copy bandwidth. */
int stzg_upload(stzg_sim *s, const double *const *up);
int stzg_download(stzg_sim *s, double *const *down);
/* Replaces: shear_sim::step_forward_quasistatic (shear_sim.cc:280-291) on
 * host-owned fields, as the reference holds them: stzg_upload(up), one step,
 * stzg_download(down) in one call.  The parts of the new state that the
 * projection leaves alone (chi rows, interior rows of X and Y, eps_pl) are
 * copied back while the multigrid solve runs. */
int stzg_step_qs_host(stzg_sim *s, double dt, const double *const *up, double *const *down, stzg_stats *stats);
/* No counterpart in the reference, which holds its state only as an array of
 * c_field records (fields.hh:7-114: 19 doubles, u, v, p, q, s, tau, chi, X,
 * Y, ddev first; shear_sim::fm - m, rows -1..n of m records, node values on
 * rows 0..n).  Host-side conversions (multithreaded) between that array
 * (fm_rows, m*(n+2) records) and the first 8 buffers of stzg_upload's `up` /
 * stzg_download's `down` layout: p, q, s, tau, chi (all rows), X, Y, vel
 * (x, y pairs from u, v).  NULL entries are skipped; the other record members
 * are left as they are.  A caller that keeps the reference's layout calls
 * pack, stzg_step_qs_host, unpack. */
int stzg_c_field_pack(const void *fm_rows, int m, int n, double *const *soa);
int stzg_c_field_unpack(const double *const *soa, int m, int n, void *fm_rows);

/* Replaces: shear_sim::step_forward_quasistatic (shear_sim.cc:280-291),
 * called nsteps times; stats may be NULL.  With the relative stopping rule
 * and graphs (and, for mixed precision, the extra V-cycle), the steps of one
 * call run without a host round trip between them: a failure (NaN residual,
 * pass cap, plastic sub-step cap) is reported once the call's last step has
 * run, and the state is then undefined, as after any failed step. */
int stzg_step_qs(stzg_sim *s, double dt, int nsteps, stzg_stats *stats);
/* Replaces: shear_sim::step_forward (shear_sim.cc:185-276), the explicit
 * (direct) step: velocity and reference map advected with ENO2 and driven by
 * the net force of the stress and a viscous term, stresses advected and
 * loaded elastically by the velocity gradient, STZ plasticity, chi diffusion,
 * set_boundaries; nsteps steps of dt; stats may be NULL. */
int stzg_step_direct(stzg_sim *s, double dt, int nsteps, stzg_stats *stats);
/* Replaces: the frame loop of shear_sim::solve (shear_sim.cc:120-140)
 * without file output: explicit steps of dt while time + dt(1+1e-8) stays
 * below target, then one step of the remaining time; *nsteps (may be NULL)
 * receives the number of steps.  The reference uses dt = dx^2 * tmult. */
int stzg_advance_direct(stzg_sim *s, double dt, double target, long *nsteps);
/* Replaces: shear_sim::advection_step + chi_diffusion (shear_sim.cc:296-386),
 * one call, time not advanced. */
int stzg_advection_step(stzg_sim *s, double dt);
/* Replaces: shear_sim::projection_step (shear_sim.cc:391-438). */
int stzg_projection_step(stzg_sim *s, double dt, stzg_stats *stats);
/* Replaces: shear_sim::avg_iters (shear_sim.hh:116) / tgmg_predict::avg_iters
 * (tgmg_predict.hh:28-32): mean V-cycles per solve since the last call. */
int stzg_avg_iters(stzg_sim *s, double *avg);

/* tgmg drop-in.  Replaces: tgmg<qs_multi,vec,mat>::solve_v_cycle(tgmg_predict&)
 * (tgmg.hh:439-441, tgmg.in.cc:266-301) on this handle's operator for time
 * step dt (qs_multi::init(visc/dt), qs_multi.cc:31-55).  src and vel are
 * m*(n+1) (x,y) pairs; vel holds the initial guess and receives the solution. */
int stzg_mg_solve(stzg_sim *s, double dt, const double *src, double *vel, int *ncycles);
/* Replaces: tgmg::v_cycle (tgmg.in.cc:313-328), one cycle. */
int stzg_mg_vcycle(stzg_sim *s, double dt, const double *src, double *vel);
/* Replaces: tgmg_base::l2_error (tgmg.hh:146) = mds()/mn for src/vel. */
int stzg_mg_l2_error(stzg_sim *s, double dt, const double *src, const double *vel, double *err);
/* Replaces: the hierarchy of tgmg::tgmg (tgmg.in.cc:17-29): number of
 * coarse levels; dims receives (m,n) per coarse level (up to 16). */
int stzg_mg_levels(stzg_sim *s, double dt, int *nlevels, int *dims);
/* Replaces: the stored coarse stencils tgmg_level::s (tgmg.hh:235, 256-265):
 * 10 2x2 blocks (dl,dc,dr,cl,cc,cr,ul,uc,ur,inverse of cc) per point,
 * (a,b,c,d) each, of coarse level l, expanded to m*n*40 doubles. */
int stzg_mg_stencil(stzg_sim *s, double dt, int level, double *out);

/* Instrumentation (no counterpart in the reference, whose timing is
 * omp_get_wtime per frame, shear_sim.cc:165-179): average device time in ms
 * of `reps` back-to-back launches of one kernel group on the handle's stream,
 * measured with CUDA events.  kernel: 0 advection (writes the spare buffer,
 * state unchanged), 1 FP64 top-level sweep (changes the velocity iterate),
 * 2 FP32 top-level sweep (scratch), 3 FP64 V-cycle, 4 FP32 V-cycle
 * (scratch), 5 outer residual of the mixed solve (float-float) + FP32 copy +
 * norms, 6 / 7 the streaming FP32 top-level kernel down (sweep, residual,
 * restriction) / up (prolongation, sweep) alone (scratch; STZG_EINVAL where
 * the top level does not use them), 8 projection source (net force from the
 * stresses; writes the solve's right-hand side only), 9 stress correction
 * from the current velocities and the wall rows (changes the stresses: the
 * handle's state is no longer a step of the reference after it). */
int stzg_time_kernel(stzg_sim *s, double dt, int kernel, int reps, double *ms);

/* No counterpart in the reference (a schedule choice of the GPU multigrid,
 * same arithmetic either way, results bitwise equal).  on = 1: a
 * mixed-precision handle runs the FP32 V-cycle's levels of at most 512
 * columns and its single-block tail in one persistent cooperative kernel
 * with grid barriers between the level phases, where the device allows.
 * Off by default: on GB300 at 2048^2 the FP32 V-cycle takes 0.178 ms with
 * it against 0.145 ms with one launch per level chained by programmatic
 * dependent launch (0.166 ms with the persistent kernel from 128 columns
 * down); on = 0 restores the per-level launches.  on = 2 is a test of the kernel's
 * bounded grid barrier: as 1, and the barrier's arrival count is set so that
 * the next launch's first barrier never completes; each block gives up after
 * about a second, the step reports STZG_ECUDA and the handle must be
 * recreated.  STZG_EINVAL for an FP64 handle or on != 0 where the device does
 * not take the kernel.  get reports whether a V-cycle of the handle uses it
 * (0 also where no level qualifies); before the first step has built the
 * coarse operators, whether it is enabled. */
int stzg_set_mg_persistent(stzg_sim *s, int on);
int stzg_get_mg_persistent(stzg_sim *s, int *on);

/* No counterpart in the reference.  Squared residual norms of the
 * quasi-static system for time step dt on caller-owned device arrays,
 * without allocating any device memory: out_dev[0] = sum |b - A z|^2,
 * out_dev[1] = sum |b|^2 (z_dev, b_dev: m*(n+1) (x,y) pairs in the solver
 * layout of stzg_mg_solve; out_dev: 2 doubles; all on the current device).
 * For callers that cannot let a library call cudaMalloc: applications whose
 * caching allocator owns the device memory, services with a fixed memory
 * budget, and threads that must not stall the GPU (cudaMalloc/cudaFree can
 * synchronize the device).  The reduction's scratch is a fixed 128 KiB array
 * in the library's static device memory, held on every GPU that loads the
 * library until exit; grids above 8,388,608 nodes are rejected with
 * STZG_EINVAL.  The first call on a device looks up that array's device
 * address (make it before capturing work on that device into a graph) and
 * keeps it until exit, so a device must not be reset with cudaDeviceReset
 * while it is used through this call.  Calls share the array: calls that
 * overlap on the GPU race.  Work is
 * enqueued on `stream` (a cudaStream_t, NULL for the default stream) and
 * the call returns without synchronizing. */
int stzg_residual_norms_noalloc(const stz_params *p, double dt, const double *z_dev, const double *b_dev,
                                double *out_dev, void *stream);

/* ---- batches -----------------------------------------------------------
 * No single counterpart in the reference, whose drivers run one shear_sim
 * per process (the UQ harness, esim/coord_transforms/simple_shear/pfn.py,
 * launches one process per sample).  A batch owns `count` independent
 * simulations (params[k] each; grids may differ) and runs them together in
 * one CUDA graph: per instance a device-side loop over time steps, each step
 * with a device-side multigrid loop (same stopping rule as stzg_step_qs,
 * bounded at 400 passes).  stzg_batch_sim exposes instance k as an ordinary
 * handle (set_state, get_field, ...; do not destroy it). */
typedef struct stzg_batch stzg_batch;
typedef struct {
    long instances, steps, cell_steps;
    long vcycles, passes, failed;
    double seconds;          /* device time of the graph launch (CUDA events) */
    long graph_kernels;      /* kernel nodes in the graph */
    long kernel_launches;    /* kernels executed (loop bodies counted per iteration) */
} stzg_batch_stats;

int stzg_batch_create(int count, const stz_params *params, const stzg_options *opt, stzg_batch **out);
int stzg_batch_destroy(stzg_batch *b);
int stzg_batch_size(stzg_batch *b, int *count);
int stzg_batch_sim(stzg_batch *b, int k, stzg_sim **s);
/* Schedule knobs for instances of grid m x n (cells): FP32 V-cycles per
 * refinement pass, largest level (points) solved by the single-block tail
 * (<0: default), fused single-precision tile kernels on/off. */
int stzg_batch_set_tuning(stzg_batch *b, int m, int n, int inner, long tail_limit, int fuse);
/* Times the candidate knobs on the GPU for every grid size of the batch
 * (`steps` steps each, on scratch instances) and installs the fastest. */
int stzg_batch_autotune(stzg_batch *b, double dt, int steps);
int stzg_batch_get_tuning(stzg_batch *b, int m, int n, int *inner, long *tail_limit, int *fuse);
/* Replaces: shear_sim::step_forward_quasistatic (shear_sim.cc:280-291)
 * nsteps times on every instance, in one graph launch. */
int stzg_batch_run(stzg_batch *b, double dt, int nsteps, stzg_batch_stats *stats);

/* ---- adjoint -----------------------------------------------------------
 * No counterpart in the reference, which has no gradients.  A forward/
 * backward pair shaped like torch.autograd.Function around `nsteps`
 * quasi-static steps (shear_sim::step_forward_quasistatic, shear_sim.cc:
 * 280-291) from the handle's current state, with the loss
 *     L = dx dy sum_cells (eps_pl - target)^2
 * on the plastic strain after the last step (target: m*n doubles on the
 * host).  The forward pass steps the handle, stores a checkpoint every
 * `checkpoint_every` steps and writes L.  The backward pass recomputes each
 * segment from its checkpoint, runs the hand-written adjoint of every step
 * in reverse and writes dloss * dL/dp for p = (c0, Omega*eps0, chi_inf,
 * s_y) into grad_params[4] and dloss * dL/d chi(t=0) (m*n) into grad_chi0
 * (either may be NULL); the handle is left at the forward run's end state.
 * Requires track_plastic and no chi diffusion (chi_diff = chi_len = 0);
 * branch decisions (ENO stencils, upwind sides, yield, sub-step counts) are
 * those of the forward run. */
int stzg_adjoint_forward(stzg_sim *s, double dt, int nsteps, int checkpoint_every, const double *target,
                         double *loss);
int stzg_adjoint_backward(stzg_sim *s, double dloss, double *grad_params, double *grad_chi0);

/* ---- frame export and diagnostics ---------------------------------------
 * Replaces: shear_sim::output (shear_sim.cc:684-720): the Gnuplot binary
 * matrix (float32) of one field, the bytes the reference writes to
 * <dir>/<prefix>.<frame>.  mode: 0 u, 1 v, 2 p, 3 q, 4 s, 5 tau, 6 chi,
 * 7 chi*TZ ("tem"), 8 |s| ("dev"), 9 X, 10 Y, 11 the last qs_measure
 * integrand ("proj").  Cell fields (2-8): (n+1) rows of m+1 floats; node
 * fields: (n+2) rows of m+2.  *count (may be NULL) receives the number of
 * floats; out == NULL only queries it. */
int stzg_output_field(stzg_sim *s, int mode, float *out, long *count);
/* Replaces: shear_sim::write_files (shear_sim.cc:659-676) with the field
 * selection as flags (bit k = mode k, the reference writes 4|128|256|512|1024;
 * bit 11 first runs qs_measure and returns Q, max in qs[2], may be NULL). */
int stzg_write_frame(stzg_sim *s, const char *dir, int frame, unsigned flags, double *qs);
/* Replaces: shear_sim::qs_measure (shear_sim.cc:733-775): Q over the
 * interior rows and its maximum integrand; the integrand per node is kept
 * for output mode 11. */
int stzg_qs_measure(stzg_sim *s, int staggered, double *Q, double *max_qs);
/* Replaces: shear_sim::tractions (shear_sim.cc:1003-1028): out[4] = bottom
 * (x, y), top (x, y). */
int stzg_tractions(stzg_sim *s, double *out);
/* Replaces: shear_sim::compute_strain (shear_sim.cc:778-824): the Hencky
 * strain magnitude per cell, out[m*n] (rows 0..n-1), restating the
 * reference's y differences as they are (interior rows give 0). */
int stzg_compute_strain(stzg_sim *s, double *out);

/* Replaces: shear_sim::l2_comparison (shear_sim.cc:460-502) between two
 * handles of the same grid: l2[4] = velocity, stress, chi, reference map. */
int stzg_l2_comparison(stzg_sim *a, stzg_sim *b, double *l2);

/* Replaces: shear_sim::initialize_random (shear_sim.cc:932-984) with a
 * counter-based seed in place of libc rand(): writes chi (m*n) on the host. */
int stzg_random_chi(int m, int n, double l, double tem_avg, double tem_std, double TZ,
                    unsigned long long seed, double *chi);

#ifdef __cplusplus
}
#endif
#endif
