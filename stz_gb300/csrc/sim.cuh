// The simulation handle behind the C ABI and the internal operations that
// the single-simulation path (api.cu) and the batched graph (batch.cu) share.
#pragma once

#include <vector>

#include "mg.cuh"
#include "step.cuh"

struct stzg_adjoint;

struct stzg_sim {
    stz_params P;
    stzg_options O;
    int m, n;
    double time = 0;
    double bv_state = 0;  // wall speed of the stored state (u=-bv on row 0, +bv on row n)
    cudaStream_t st = nullptr;
    stzg::step_consts sc;
    stzg::fields_dev F;
    stzg::field_maps *maps = nullptr;  // TMA descriptors of F's advected fields
    int cur = 0;
    std::vector<void *> owned;
    // multigrid
    stzg::qs_constants q;
    double viscdt = -1;
    std::vector<stzg::level_ops> ops;
    stzg::hierarchy<double> h64;
    stzg::hierarchy<float> h32;
    double *partials = nullptr;  // device, 2 per block
    double *dnorm = nullptr;     // device: [r2, b2]
    double *hnorm = nullptr;     // pinned host copy
    int npart = 0;
    // tgmg_predict state (tgmg_predict.hh:6-33, tgmg_config.hh:26-45)
    int lim = 16 * 8, mult = 16, decay = 32, max_thresh = 16 * 2048, extra_iters = 1;
    long avg_vcount = 0, avg_solves = 0;
    stzg_stats acc{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // captured graphs: one FP64 V-cycle; mixed: initial residual, one pass
    cudaGraphExec_t g_vc64 = nullptr, g_res32 = nullptr, g_pass32 = nullptr;
    long n_vc64 = 0, n_res32 = 0, n_pass32 = 0;  // kernel nodes per graph
    int g_inner = 0;
    // relative-tolerance solve with its convergence loop on the device: one
    // graph (set-up, WHILE node over passes, finish); kernel nodes outside
    // and inside the loop body
    cudaGraphExec_t g_loop = nullptr;
    cudaGraphExec_t g_loop_x = nullptr;  // the same with the guess's extrapolation fused into its split
    int g_loop_x_inner = 0;
    // multi-step calls: solves launched without reading their pass counts
    bool defer_checks = false;
    long defer_solves = 0;
    int defer_inner = 1;
    long n_loop_outer = 0, n_loop_body = 0, n_loop_merge = 0;
    int g_loop_inner = 0;
    int *hflags = nullptr;  // pinned host copy of F.flags (FL_COUNT ints)
    double2 *vel_prev = nullptr;  // previous solution (extrapolated guesses)
    double2 *vel_prev2 = nullptr; // the one before (quadratic extrapolation)
    bool have_prev2 = false;
    // mixed precision: float-float copies (hi + lo) of the iterate and of the
    // right-hand side for the duration of a solve
    float2 *zhi = nullptr, *zlo = nullptr, *bhi = nullptr, *blo = nullptr;
    bool have_prev = false;
    stzg_adjoint *adj = nullptr;  // adjoint workspace (adjoint.cu), created on first use
    double *proj = nullptr;       // qs_measure integrand per node (output.cu), created on first use
    // bulk host transfers: copies spread over several streams (copy engines)
    static constexpr int kCopyStreams = 4;
    cudaStream_t cst[kCopyStreams] = {};
    cudaEvent_t cev_ready = nullptr, cev[kCopyStreams] = {};
};


namespace stzg {

int dev_alloc(stzg_sim *s, void **p, size_t bytes);
double bdry_vel(const stzg_sim *s, double t);
double bdry_pos(const stzg_sim *s, double t);
int validate(const stz_params *p);
void drop_graphs(stzg_sim *s);
int ensure_ops(stzg_sim *s, double dt);
void launch_norms(stzg_sim *s, bool mixed);
// Mixed solve: vel, src -> float-float iterate and right-hand side, and back.
void mixed_begin(stzg_sim *s);
void mixed_end(stzg_sim *s);
int read_check(stzg_sim *s, double *err, bool *ok);
int check_flags(stzg_sim *s);
size_t cell_count(const stzg_sim *s);
void adjoint_release(stzg_sim *s);

}  // namespace stzg
