/* stzg_tgmg.h - C ABI of the general scalar geometric multigrid on one GPU.
 *
 * Stands in for the reference's tgmg<S,double,double> template
 * (esim/tgmg/tgmg.hh:42-495, tgmg.in.cc:11-856) over a problem class S
 * (the concept of esim/tgmg/poisson_fd.hh:7-61: grid m x n, periodicity
 * x_prd/y_prd, nine stencil functions a_dl..a_ur, a_cc, inv_cc, mul_a and the
 * squared-L2 threshold acc).  The operator is passed as a table of distinct
 * 9-point stencils (scalar or 2x2 blocks) plus the stencil index of every
 * grid point; coarse levels
 * are Galerkin products with the reference's restriction and interpolation
 * (tgmg.in.cc:552-736).  One handle owns the hierarchy in device memory, a
 * CUDA stream and the captured cycle graphs.  Statuses and the last message
 * are those of stzg.h (stzg_strerror, stzg_last_message).
 */
#ifndef STZG_TGMG_H
#define STZG_TGMG_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct stzg_tgmg stzg_tgmg;

/* tgmg_predict (esim/tgmg/tgmg_predict.hh:6-33) with its defaults
 * (tgmg_config.hh:26-45): lim = mult*8, mult 16, decay 32,
 * max_thresh = mult*2048, extra_iters 1. */
typedef struct {
    int mult, decay, max_thresh, extra_iters;
    int lim;
    int solves, vcount;
} stzg_tgmg_predict;

void stzg_tgmg_predict_init(stzg_tgmg_predict *tp);

/* Solver types of tgmg::solve (tgmg.hh:399-411): 0 Jacobi, 1 Gauss-Seidel,
 * 2 SOR, 3 full multigrid (fmg_pre followed by a V-cycle), 4 V-cycle,
 * 5 symmetric V-cycle. */
enum { STZG_TGMG_JACOBI = 0, STZG_TGMG_GS = 1, STZG_TGMG_SOR = 2, STZG_TGMG_FMG = 3,
       STZG_TGMG_VCYCLE = 4, STZG_TGMG_SYM_VCYCLE = 5 };

/* tgmg(S&, V* b, V* z) + setup() (tgmg.in.cc:11-33, tgmg.hh:331-335).
 * table: ntable stencils of 9 doubles in the order dl dc dr cl cc cr ul uc ur
 * (tgmg.hh:256-264); cls: m*n stencil indices, row-major (index j*m+i).
 * Entries that point outside a non-periodic grid are ignored.  acc is the
 * problem's threshold on the mean squared residual (l2_error, tgmg.hh:146).
 * device: CUDA ordinal.  A periodic direction needs at least 3 points. */
int stzg_tgmg_create(int m, int n, int x_prd, int y_prd, const double *table, int ntable, const int *cls,
                     double acc, int device, stzg_tgmg **out);
/* tgmg<S,vec,mat> (2-vector values, 2x2 blocks, as the reference's qs_multi
 * classes, esim/sb/main/qs_multi.hh:11-57): block = 2, the table holds 9
 * row-major 2x2 blocks per stencil (36 doubles) and b, z hold (x, y) per
 * point; block = 1 is stzg_tgmg_create. */
int stzg_tgmg_create_block(int m, int n, int x_prd, int y_prd, int block, const double *table, int ntable,
                           const int *cls, double acc, int device, stzg_tgmg **out);
/* New operator values on the same grid: the problem class's stencil
 * changed, e.g. qs_multi::init before each solve (coord_transforms
 * qs_multi.cc:31-46).  Rebuilds the Galerkin hierarchy (tgmg::setup).
 * cls NULL keeps the class map of the last operator (ntable must then be
 * the same); with the same class map, given or kept, only the stencil
 * values are recomputed and uploaded. */
int stzg_tgmg_set_operator(stzg_tgmg *g, const double *table, int ntable, const int *cls);
int stzg_tgmg_destroy(stzg_tgmg *g);
/* precision 1 (STZG_MIXED of stzg.h): V-cycle solves and iterations
 * (STZG_TGMG_VCYCLE, STZG_TGMG_SYM_VCYCLE) run as refinement passes, each an
 * FP32 V-cycle on the FP32 rounding of the FP64 residual b - A z, its
 * correction added to z in FP64; the predictor, l2_error and acc count and
 * test passes and FP64 residuals as they do V-cycles.  Residuals must stay
 * inside FP32's range (1e-38..3e38).  The other solver types, and precision 0
 * (STZG_FP64, the default), run in FP64. */
int stzg_tgmg_set_precision(stzg_tgmg *g, int precision);

/* The source b and solution z (block*m*n doubles, row-major), copied in and out. */
int stzg_tgmg_set_b(stzg_tgmg *g, const double *b);
int stzg_tgmg_get_b(stzg_tgmg *g, double *b);
int stzg_tgmg_set_z(stzg_tgmg *g, const double *z);
int stzg_tgmg_get_z(stzg_tgmg *g, double *z);
/* Device addresses of the top level's b and z (block*m*n doubles each, on
 * the handle's device), for callers that keep the solve's data on the GPU;
 * valid until stzg_tgmg_destroy.  Work on them must be ordered before the
 * next call on the handle (the handle's calls synchronize its stream). */
int stzg_tgmg_device_arrays(stzg_tgmg *g, double **b, double **z);
/* tgmg_base::clear_z (tgmg.in.cc:792). */
int stzg_tgmg_clear_z(stzg_tgmg *g);

/* tgmg::solve(type, tgmg_predict&, omega, cyc_down, cyc_up, hcyc_bottom)
 * (tgmg.in.cc:266-301): tp's predicted count of iterations, then more in
 * triangular steps until l2_error < acc, then tp->extra_iters more.
 * iters (optional) receives the count added to tp; l2 (optional) the last
 * l2_error.  STZG_ENOTCONV when lim exceeds max_thresh (the reference returns
 * false), STZG_ENAN on a NaN residual. */
int stzg_tgmg_solve(stzg_tgmg *g, int type, stzg_tgmg_predict *tp, double omega, int cyc_down, int cyc_up,
                    int hcyc_bottom, int *iters, double *l2);
/* tgmg::solve(type, per_loop, max_loops, ...) (tgmg.in.cc:182-197): batches
 * of per_loop iterations (solve_v_cycle(): 4 per batch, 1000 batches) until
 * l2_error <= acc. */
int stzg_tgmg_solve_fixed(stzg_tgmg *g, int type, int per_loop, int max_loops, double omega, int cyc_down,
                          int cyc_up, int hcyc_bottom, int *iters, double *l2);
/* Not in the reference: iterations of one type until l2_error < acc, the
 * residual tested before the first (a warm start may meet it already) and
 * after each, at most max_iters, then extra_iters more; iters receives the
 * count before the extra ones.  STZG_ENOTCONV past max_iters, STZG_ENAN on a
 * NaN residual.  The predictor of stzg_tgmg_solve runs the counts it
 * predicts whatever the need (tgmg.in.cc:266-301); this runs only what the
 * residual asks for, at one residual check per iteration. */
int stzg_tgmg_solve_checked(stzg_tgmg *g, int type, int max_iters, int extra_iters, double omega, int cyc_down,
                            int cyc_up, int hcyc_bottom, int *iters, double *l2);
/* count iterations of one type without convergence checks (tgmg::iters,
 * tgmg.hh:457-466): v_cycle / fmg_pre+v_cycle / jacobi / gauss_seidel / sor. */
int stzg_tgmg_iterate(stzg_tgmg *g, int type, int count, double omega, int cyc_down, int cyc_up, int hcyc_bottom);
/* tgmg_base::l2_error = mds()/mn (tgmg.hh:146, tgmg.in.cc:55-65). */
int stzg_tgmg_l2_error(stzg_tgmg *g, double *err);

/* Hierarchy: nlevels including the top; dims gets (m, n) per level. */
int stzg_tgmg_levels(stzg_tgmg *g, int *nlevels, int *dims);
/* Galerkin stencils of coarse level `level` (1 = first child) in the layout
 * of tgmg_level::s (tgmg.hh:235): 10 blocks per point (9 entries and the
 * inverse of the centre), block*block doubles each, m*n points of that level. */
int stzg_tgmg_stencil(stzg_tgmg *g, int level, double *out);
/* Device time (ms, CUDA events) of the last solve/iterate call and the
 * kernels it launched. */
int stzg_tgmg_last_timing(stzg_tgmg *g, double *ms, long *kernels);

/* The poisson_fd problem class (poisson_fd.{hh,cc}): m x n grid points on
 * [ax,bx] x [ay,by], dx = (bx-ax)/(m-1), 5-point Laplacian with Dirichlet
 * edges (edge points carry only the centre entry), acc =
 * tgmg_accuracy(hcc, 1e4).  Writes the two-stencil table (interior, edge),
 * the m*n indices and acc for stzg_tgmg_create. */
int stzg_poisson_fd(int m, int n, double ax, double bx, double ay, double by, double *table, int *cls,
                    double *acc);

#ifdef __cplusplus
}
#endif

#endif /* STZG_TGMG_H */
