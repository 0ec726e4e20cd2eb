// Time-step kernels of the quasi-static STZ simulation.
#pragma once

#include <cuda.h>

#include "common.cuh"

namespace stzg {

// Field storage: every per-point array holds rows -1..n of m entries
// (ghost rows of the cell fields; node fields use rows 0..n), index
// (j+1)*m + i.  The state is double-buffered: the advection kernel reads
// buffer `cur` and writes buffer `cur^1`.
enum { F_P = 0, F_Q, F_S, F_TAU, F_CHI, F_X, F_Y, F_COUNT };
// Slots of fields_dev::flags.
enum {
    FL_SUBSTEP_CAP = 0,
    FL_SUBSTEP_MAX,
    FL_VEL_CHANGED,
    FL_TMA,
    FL_PASSES,
    FL_LOOP_ERR,
    FL_MG_BAR_ERR,  // a grid-barrier wait of the persistent coarse multigrid kernel ran out
    FL_MG_BAR = 8,  // two words (8, 9): that barrier's arrivals and generation
    FL_PASSES_SUM = 10,  // passes of the device-loop solves since the host last cleared it
    FL_ERR_FIRST,   // the first device-loop error since then (1 pass cap, 2 NaN)
    FL_COUNT = 12
};

struct fields_dev {
    double *f[2][F_COUNT];
    double *ddev;    // per-step stress drop osbar-sbar (fields.hh:27)
    double *eps_pl;  // accumulated plastic strain (cells, m*n)
    double2 *vel;    // node velocity, rows 0..n, index j*m+i (solver array)
    double2 *src;    // projection right-hand side, same layout
    int *flags;      // FL_COUNT ints: [0] plastic sub-step cap reached, [1] max sub-steps,
                     // [2] scratch of the velocity upload, [3] an advection tile copy wait
                     // ran out, [4] passes of the last device-loop solve, [5] its error
                     // (1 pass cap reached, 2 NaN residual), [6] a coarse-kernel barrier
                     // wait ran out, [8..9] that barrier's words
    // Per-cell combinations of the advected stress that the nodal net force
    // (shear_sim::net_force, shear_sim.cc:447-453) sums with +-1 weights:
    // U = xf A + yf tau, W = xf A - yf tau, Y1 = xf tau - yf B,
    // Y2 = xf tau + yf B, A = p+q-s, B = p+q+s (xf, yf of projection_step).
    double *pre[4];
    // Float-float advection: cells that the pair yield test cannot certify as
    // elastic (their index, then their count), for the FP64 plastic pass.
    unsigned *plist;
    unsigned *pcount;
};

struct step_consts {
    int m, n;
    double ax, ay, by, dx, dy, lx, xsp, ysp;
    double mu, K;
    // STZ law
    int stz_model, t_model;
    double t_scale, adapt_fac, chi_inf, s_y, theta, Delta, Omegaeps0, tau0, c0, kappa, rho;
    double chi_diff, chi_len;
    int track_plastic;
    int substep_cap;
    double yield_cut2;  // s_y^2 (1 - 1e-12): athermal cells below it skip the plastic loop
    float yield_cut2f;  // the same lowered by 1e-6, for the float-float path's test
    // Device clock of a graph-driven run (nullptr: wall quantities come as
    // kernel arguments from the host).  Layout: CLK_* below.
    const double *clock;
    double xbc;  // bcs*cxx of the projection operator (wall source = -+xbc*bv)
    // advection, projection source and stress correction in float-float on
    // the FP64 state (mixed-precision handles); 0: all FP64, bit-exact
    int sp_increments;
};

// Device clock slots: time, wall speed of the stored state, wall speed and
// wall position at `time` (shear_sim.hh:120-124).
// CLK_CUR holds the state buffer index at the start of the step.
enum { CLK_TIME = 0, CLK_BV_STATE = 1, CLK_BV = 2, CLK_BP = 3, CLK_CUR = 4, CLK_COUNT = 5 };

step_consts make_step_consts(const stz_params &p);
// x as a float pair hi + lo (host).
void split_host(double x, float *hi, float *lo);

// |a| > |b| for finite doubles, compared as the magnitudes of their IEEE bit
// patterns on the integer pipe (same result as fabs(a) > fabs(b)).
__device__ __forceinline__ bool mag_gt(double a, double b) {
    const unsigned long long ma = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
    const unsigned long long mb = (unsigned long long)__double_as_longlong(b) & 0x7fffffffffffffffull;
    return ma > mb;
}

// ENO2 choice and value (shear_sim::eno2, shear_sim.cc:653-655): with the
// second differences d1 = p0 - 2p1 + p2 and d2 = p1 - 2p2 + p3, |d1| > |d2|
// selects 3p1 - 4p2 + p3 = d2 + 2(p1 - p2), otherwise p0 - p2 = d1 + 2(p1 - p2).
// Written through first differences: six FP64 operations and an integer
// compare.  The adjoint takes its branch decisions from eno2_pick, so both
// see the same choice.
__device__ __forceinline__ bool eno2_pick(double p0, double p1, double p2, double p3) {
    const double e = p1 - p2;
    return mag_gt((p0 - p1) - e, e - (p2 - p3));
}
__device__ __forceinline__ double eno2(double p0, double p1, double p2, double p3) {
    const double e = p1 - p2, d1 = (p0 - p1) - e, d2 = e - (p2 - p3);
    return fma(2.0, e, mag_gt(d1, d2) ? d2 : d1);
}

// shear_sim::advection_step + chi_diffusion + the field update
// (shear_sim.cc:296-386, fields.hh:61-80).  bv is the wall speed of the
// current state (u = -bv on row 0 and +bv on row n, set_boundaries).
// TMA descriptors of the seven advected fields in both state buffers: 2D
// FP64 tensors of m x (n+2) (rows -1..n), box of the advection tile (36
// columns x 12 rows).  Built once per simulation; the pointers of F must not
// change afterwards.
struct field_maps {
    CUtensorMap f[2][F_COUNT];
};
int make_field_maps(const step_consts &c, const fields_dev &F, field_maps *out);
// F.flags[FL_TMA] is set when a tile's copy wait runs out (status, no fault); that
// tile of the next state is then left unwritten.
void advection(const step_consts &c, const field_maps &maps, fields_dev &F, int cur, double dt, double bv,
               cudaStream_t st);
// Opts the advection kernel into the shared memory its tile needs (once per
// process, outside any stream capture).
cudaError_t prepare_step_kernels();
// shear_sim::step_forward (shear_sim.cc:185-276) up to set_boundaries:
// explicit update of buffer cur into cur^1, new interior node velocities in
// F.src (rows 1..n-1), chi diffusion.  bv is the wall speed of the state.
void direct_step(const step_consts &c, double viscosity, fields_dev &F, int cur, double dt, double bv,
                 cudaStream_t st);
// The per-cell combinations above from the current stress (used when the
// projection runs without the advection kernel in front of it).
void precombine(const step_consts &c, fields_dev &F, int cur, double dt, cudaStream_t st);
// projection_step source term (shear_sim.cc:399-409, net_force :447-453).
void projection_source(const step_consts &c, fields_dev &F, int cur, double dt, double xbc_bv, cudaStream_t st);
// stress correction and velocity copy (shear_sim.cc:418-434) followed by
// set_boundaries (shear_sim.cc:552-581) at the wall speed/position bv, bp.
void projection_apply(const step_consts &c, fields_dev &F, int cur, double dt, double bv, double bp,
                      cudaStream_t st);
// set_boundaries alone (ghost rows and wall nodes of buffer cur).
void set_boundaries(const step_consts &c, fields_dev &F, int cur, double bp, cudaStream_t st);

}  // namespace stzg
