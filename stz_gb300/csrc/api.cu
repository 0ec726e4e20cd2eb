// C ABI (include/stzg.h): handle management, the time-step driver and the
// multigrid solve policy.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <algorithm>
#include <vector>

#include "mg.cuh"
#include "step.cuh"

#include <atomic>

namespace stzg {

static thread_local std::string g_msg;
// Kernels launched by this thread (every count the library reports is a
// difference taken within one call, so host threads driving separate handles
// do not see each other's launches).
struct launch_counter {
    long n = 0;
    void fetch_add(long k) { n += k; }
    void fetch_sub(long k) { n -= k; }
};
static thread_local launch_counter g_launches;

void note_launch() { g_launches.fetch_add(1); }
long launch_count() { return g_launches.n; }
void discount_launches(long k) { g_launches.fetch_sub(k); }

int fail(int status, const std::string &msg) {
    g_msg = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char *what) {
    g_msg = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return STZG_ENOMEM;
    return STZG_ECUDA;
}

}  // namespace stzg

using namespace stzg;

#include "sim.cuh"

namespace stzg {
// Host set-ups of chi (chi_init.cpp).
void init_fields_chi(const stz_params &p, int chi_case, double tem_base, double tem_delta, double *chi);
void bicubic_chi(const stz_params &p, int mm, int nn, const double *arr, double lo, double sca, double *chi);
}  // namespace stzg

namespace stzg {

int dev_alloc(stzg_sim *s, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    s->owned.push_back(*p);
    STZG_CUDA(cudaMemsetAsync(*p, 0, bytes, s->st));
    return STZG_OK;
}

double bdry_vel(const stzg_sim *s, double t) { return t < 1 ? t * s->P.u_bdry : s->P.u_bdry; }
double bdry_pos(const stzg_sim *s, double t) {
    return t < 1 ? s->P.u_bdry * t * t * 0.5 : s->P.u_bdry * (t - 0.5);
}

int validate(const stz_params *p) {
    if (!p) return fail(STZG_EINVAL, "null parameters");
    if (p->m < 4 || p->n < 4) return fail(STZG_EINVAL, "grid needs m,n >= 4");
    if (p->m & 1) return fail(STZG_EINVAL, "m must be even (two-colour top-level smoother on a periodic line)");
    if (!(p->bx > p->ax) || !(p->by > p->ay)) return fail(STZG_EINVAL, "empty domain");
    if (p->stz_model < 0 || p->stz_model > 3) return fail(STZG_EINVAL, "unknown STZ law");
    if (!(p->mu > 0)) return fail(STZG_EINVAL, "shear modulus must be positive");
    long pts = (long)p->m * (p->n + 2);
    if (pts > (1L << 31) / 2) return fail(STZG_EINVAL, "grid too large for 32-bit row indexing");
    return STZG_OK;
}

void drop_graphs(stzg_sim *s) {
    cudaGraphExec_t *g[5] = {&s->g_vc64, &s->g_res32, &s->g_pass32, &s->g_loop, &s->g_loop_x};
    for (int k = 0; k < 5; k++)
        if (*g[k]) {
            cudaGraphExecDestroy(*g[k]);
            *g[k] = nullptr;
        }
}

// Captures the work `body` enqueues on the handle's stream into *out;
// *nodes receives the number of kernels it holds.
template <class F> int capture(stzg_sim *s, cudaGraphExec_t *out, long *nodes, F &&body) {
    if (*out) return STZG_OK;
    STZG_CUDA(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    const long c0 = launch_count();
    body();
    *nodes = launch_count() - c0;
    g_launches.fetch_sub(*nodes);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s->st, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *out = nullptr;
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    return STZG_OK;
}

// Sets up the operator hierarchy for viscosity/dt (qs_multi::init,
// qs_multi.cc:31-55 -> tgmg::setup, tgmg.hh:331-351).
int ensure_ops(stzg_sim *s, double dt) {
    double viscdt = s->P.viscosity / dt;
    if (viscdt == s->viscdt && !s->ops.empty()) return STZG_OK;
    drop_graphs(s);
    s->q.init(s->P, viscdt);
    s->ops = build_coarse_ops(s->q, s->m, s->n + 1);
    top_op<double> o = s->q.op<double>();
    STZG_CHECK(s->h64.upload_ops(s->ops, o));
    if (s->O.precision == STZG_MIXED) STZG_CHECK(s->h32.upload_ops(s->ops, o));
    s->viscdt = viscdt;
    return STZG_OK;
}

// Residual norms of the current vel/src (FP64) into dnorm = [r.r, b.b];
// the mixed variant also leaves r in FP32 as the right-hand side of the
// next FP32 V-cycles.
void launch_norms(stzg_sim *s, bool mixed) {
    const int M = s->m, N = s->n + 1;
    if (mixed)
        ff_residual(s->q.op<double>(), s->zhi, s->zlo, s->bhi, s->blo, M, N, s->h32.lv[0].b, s->partials, s->npart,
                    s->dnorm, s->dnorm + 1, s->st);
    else
        top_residual_sqnorm(s->h64, s->partials, s->npart, s->dnorm, s->dnorm + 1, s->st);
}

void mixed_begin(stzg_sim *s) {
    ff_split(s->F.vel, s->zhi, s->zlo, s->F.src, s->bhi, s->blo, (long)s->m * (s->n + 1), s->st);
}

void mixed_end(stzg_sim *s) { ff_merge(s->zhi, s->zlo, s->F.vel, (long)s->m * (s->n + 1), s->st); }

// Reads dnorm and evaluates the stopping rule.
int read_check(stzg_sim *s, double *err, bool *ok) {
    const int M = s->m, N = s->n + 1;
    STZG_CUDA(cudaMemcpyAsync(s->hnorm, s->dnorm, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    s->acc.checks++;
    double r2 = s->hnorm[0], b2 = s->hnorm[1];
    if (std::isnan(r2)) return fail(STZG_ENAN, "NaN residual");
    if (s->O.tol_mode == STZG_TOL_REFERENCE) {
        *err = r2 / ((double)M * N);  // l2_error() = mds()/mn, tgmg.hh:146
        *ok = *err < s->q.reference_acc(s->O.tol);
    } else {
        *err = b2 > 0 ? std::sqrt(r2 / b2) : std::sqrt(r2);
        *ok = b2 > 0 ? r2 <= s->O.tol * s->O.tol * b2 : r2 == 0;
    }
    s->acc.last_error = *err;
    return STZG_OK;
}

int check(stzg_sim *s, bool mixed, double *err, bool *ok) {
    launch_norms(s, mixed);
    return read_check(s, err, ok);
}

int run_vcycles(stzg_sim *s, int k) {
    if (k <= 0) return STZG_OK;
    if (s->O.use_graphs) {
        STZG_CHECK(capture(s, &s->g_vc64, &s->n_vc64, [&] { vcycle<double>(s->h64, s->st, 10, 1); }));
        for (int c = 0; c < k; c++) {
            STZG_CUDA(cudaGraphLaunch(s->g_vc64, s->st));
            g_launches.fetch_add(s->n_vc64);
        }
    } else {
        for (int c = 0; c < k; c++) vcycle<double>(s->h64, s->st, 10, 1);
    }
    return STZG_OK;
}

// tgmg::solve(4, tgmg_predict&) (tgmg.in.cc:266-301) in FP64.
int solve_fp64(stzg_sim *s, int *ncyc) {
    int nc = s->lim / s->mult;
    STZG_CHECK(run_vcycles(s, nc));
    double err;
    bool ok;
    STZG_CHECK(check(s, false, &err, &ok));
    if (ok) {
        if (s->lim > 0) s->lim -= 1 + s->lim / s->decay;
    } else {
        int k = 0;
        do {
            s->lim += ++k * s->mult;
            if (s->lim > s->max_thresh) return fail(STZG_ENOTCONV, "multigrid did not converge");
            nc += k;
            STZG_CHECK(run_vcycles(s, k));
            STZG_CHECK(check(s, false, &err, &ok));
        } while (!ok);
    }
    STZG_CHECK(run_vcycles(s, s->extra_iters));
    s->acc.vcycles += nc;
    s->acc.extra_vcycles += s->extra_iters;
    s->acc.solves++;
    s->avg_vcount += nc;
    s->avg_solves++;
    if (ncyc) *ncyc = nc;
    return STZG_OK;
}

// FP32 V-cycles inside iterative refinement.  One pass: e = 0, `inner` FP32
// V-cycles on A e = r (coarsest level solved in FP64), z += e on the
// float-float iterate, then the float-float residual r = b - A z (kept in
// FP32 for the next pass) and its norm.  The number of passes between host checks follows the
// tgmg_predict policy (tgmg.in.cc:266-301) applied to passes.
int run_passes(stzg_sim *s, int k) {
    const long count = (long)s->m * (s->n + 1);
    const int inner = s->g_inner;
    auto pass = [&] {
        for (int c = 0; c < inner; c++) vcycle<float>(s->h32, s->st, 10, 1, c == 0);
        ff_correct(s->zhi, s->zlo, s->h32.lv[0].z, count, s->st);
        launch_norms(s, true);
    };
    if (k <= 0) return STZG_OK;
    if (s->O.use_graphs) {
        STZG_CHECK(capture(s, &s->g_pass32, &s->n_pass32, pass));
        for (int c = 0; c < k; c++) {
            STZG_CUDA(cudaGraphLaunch(s->g_pass32, s->st));
            g_launches.fetch_add(s->n_pass32);
        }
    } else {
        for (int c = 0; c < k; c++) pass();
    }
    s->acc.refinements += k;
    return STZG_OK;
}

int solve_mixed(stzg_sim *s, int *ncyc) {
    const int inner = s->O.inner_cycles > 0 ? s->O.inner_cycles : 3;
    if (inner != s->g_inner && s->g_pass32) {
        cudaGraphExecDestroy(s->g_pass32);
        s->g_pass32 = nullptr;
    }
    s->g_inner = inner;
    mixed_begin(s);
    launch_norms(s, true);  // initial residual of the warm start
    int np = s->lim / s->mult;
    STZG_CHECK(run_passes(s, np));
    double err;
    bool ok;
    STZG_CHECK(read_check(s, &err, &ok));
    if (ok) {
        if (s->lim > 0) s->lim -= 1 + s->lim / s->decay;
    } else {
        int k = 0;
        do {
            s->lim += ++k * s->mult;
            if (s->lim > s->max_thresh) return fail(STZG_ENOTCONV, "iterative refinement did not converge");
            np += k;
            STZG_CHECK(run_passes(s, k));
            STZG_CHECK(read_check(s, &err, &ok));
        } while (!ok);
    }
    mixed_end(s);
    const int cycles = np * inner;
    s->acc.vcycles += cycles;
    s->acc.solves++;
    s->avg_vcount += cycles;
    s->avg_solves++;
    if (ncyc) *ncyc = cycles;
    return STZG_OK;
}

// Relative-tolerance solves keep their convergence loop on the device: a
// WHILE graph node runs one pass (mixed: `inner` FP32 V-cycles, the
// float-float correction and residual; FP64: one V-cycle and the residual
// norm) per iteration until ||r|| <= tol ||b||, so the host neither predicts
// a cycle count nor waits for a check between passes.  The initial residual
// is tested first: a warm start that already meets the tolerance runs no
// pass.  A pass cap (the tgmg_predict threshold, tgmg_config.hh:26-45, in
// V-cycles) ends a solve that does not converge, with an error flag.
// h_ran: the IF node after the loop (the float-float merge of the mixed
// solve), taken only when a pass ran: otherwise the FP64 velocity is still
// the solution and stays as it is.
__global__ void k_loop_start(const double *dnorm, int *flags, double tol2, cudaGraphConditionalHandle h,
                             cudaGraphConditionalHandle h_ran, int has_ran) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double r2 = dnorm[0], b2 = dnorm[1];
        const bool conv = b2 > 0 ? r2 <= tol2 * b2 : r2 == 0;
        const bool nan = isnan(r2);
        flags[FL_PASSES] = 0;
        flags[FL_LOOP_ERR] = nan ? 2 : 0;
        if (nan && !flags[FL_ERR_FIRST]) flags[FL_ERR_FIRST] = 2;
        cudaGraphSetConditional(h, (!conv && !nan) ? 1u : 0u);
        if (has_ran) cudaGraphSetConditional(h_ran, (!conv && !nan) ? 1u : 0u);
    }
}

__global__ void k_loop_check(const double *dnorm, int *flags, double tol2, int cap, cudaGraphConditionalHandle h) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double r2 = dnorm[0], b2 = dnorm[1];
        const bool conv = b2 > 0 ? r2 <= tol2 * b2 : r2 == 0;
        const bool nan = isnan(r2);
        const int it = ++flags[FL_PASSES];
        ++flags[FL_PASSES_SUM];
        if (nan) flags[FL_LOOP_ERR] = 2;
        else if (!conv && it >= cap) flags[FL_LOOP_ERR] = 1;
        if (flags[FL_LOOP_ERR] && !flags[FL_ERR_FIRST]) flags[FL_ERR_FIRST] = flags[FL_LOOP_ERR];
        cudaGraphSetConditional(h, (!conv && !nan && it < cap) ? 1u : 0u);
    }
}

static int loop_cap(const stzg_sim *s, int per_pass) {
    return std::max(1, s->max_thresh / s->mult / per_pass);
}

// Ends a capture that failed half-way, so the stream is usable again.
static int abandon_capture(stzg_sim *s, int status) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(s->st, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return status;
}

static int build_loop_graph(stzg_sim *s, bool mixed, int inner, bool fused_extrap) {
    cudaGraphExec_t &slot = fused_extrap ? s->g_loop_x : s->g_loop;
    int &slot_inner = fused_extrap ? s->g_loop_x_inner : s->g_loop_inner;
    if (slot && slot_inner == inner) return STZG_OK;
    if (slot) {
        cudaGraphExecDestroy(slot);
        slot = nullptr;
    }
    const long count = (long)s->m * (s->n + 1);
    const double tol2 = s->O.tol * s->O.tol;
    const int per_pass = mixed ? inner : 1;
    cudaGraph_t root = nullptr;
    STZG_CUDA(cudaGraphCreate(&root, 0));
    cudaGraphConditionalHandle h, h_ran = 0;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, root, 0, 0);
    // the reference's extra V-cycle after convergence (tgmg_config.hh:45), in
    // FP32 on the last residual for mixed handles: it keeps the solution well
    // inside the tolerance, so the next step's extrapolated guess usually
    // meets it without a pass (2048^2 over 300 steps: 1.13 against 1.29
    // ms/step, stresses 1e-11 from the FP64 path's instead of 6e-11 to 7e-9)
    const int mixed_extra = mixed ? s->extra_iters : 0;
    if (e == cudaSuccess && mixed && mixed_extra == 0) e = cudaGraphConditionalHandleCreate(&h_ran, root, 0, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(root);
        return cuda_fail(e, "cudaGraphConditionalHandleCreate");
    }
    cudaGraphNodeParams wp = {};
    int st = STZG_OK;
    const long c0 = launch_count();
    e = cudaStreamBeginCaptureToGraph(s->st, root, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(root);
        return cuda_fail(e, "cudaStreamBeginCaptureToGraph");
    }
    // set-up: initial residual of the warm start, then the loop and the finish
    if (mixed && fused_extrap)
        extrap_split(s->F.vel, s->vel_prev, s->F.src, s->zhi, s->zlo, s->bhi, s->blo, count, s->st);
    else if (mixed)
        mixed_begin(s);
    launch_norms(s, mixed);
    k_loop_start<<<1, 32, 0, s->st>>>(s->dnorm, s->F.flags, tol2, h, h_ran, mixed && mixed_extra == 0 ? 1 : 0);
    note_launch();
    {
        cudaStreamCaptureStatus cs;
        cudaGraph_t cg;
        const cudaGraphNode_t *deps = nullptr;
        size_t ndeps = 0;
        e = cudaStreamGetCaptureInfo(s->st, &cs, nullptr, &cg, &deps, nullptr, &ndeps);
        cudaGraphNode_t wnode;
        if (e == cudaSuccess) {
            wp.type = cudaGraphNodeTypeConditional;
            wp.conditional.handle = h;
            wp.conditional.type = cudaGraphCondTypeWhile;
            wp.conditional.size = 1;
            e = cudaGraphAddNode(&wnode, cg, deps, nullptr, ndeps, &wp);
        }
        if (e == cudaSuccess)
            e = cudaStreamUpdateCaptureDependencies(s->st, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e != cudaSuccess) st = cuda_fail(e, "conditional node");
    }
    if (st != STZG_OK) {
        cudaGraphDestroy(root);
        return abandon_capture(s, st);
    }
    cudaGraphNodeParams ip = {};  // mixed: IF a pass ran { merge }
    if (mixed_extra > 0) {
        // after convergence: the extra FP32 V-cycles on the last residual, then
        // the correction and the merge in one pass
        const long count = (long)s->m * (s->n + 1);
        for (int c = 0; c < mixed_extra; c++) vcycle<float>(s->h32, s->st, 10, 1, c == 0);
        ff_correct_merge(s->zhi, s->zlo, s->h32.lv[0].z, s->F.vel, count, s->st);
    } else if (mixed) {
        cudaStreamCaptureStatus cs;
        cudaGraph_t cg;
        const cudaGraphNode_t *deps = nullptr;
        size_t ndeps = 0;
        e = cudaStreamGetCaptureInfo(s->st, &cs, nullptr, &cg, &deps, nullptr, &ndeps);
        cudaGraphNode_t inode;
        if (e == cudaSuccess) {
            ip.type = cudaGraphNodeTypeConditional;
            ip.conditional.handle = h_ran;
            ip.conditional.type = cudaGraphCondTypeIf;
            ip.conditional.size = 1;
            e = cudaGraphAddNode(&inode, cg, deps, nullptr, ndeps, &ip);
        }
        if (e == cudaSuccess)
            e = cudaStreamUpdateCaptureDependencies(s->st, &inode, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e != cudaSuccess) {
            cudaGraphDestroy(root);
            return abandon_capture(s, cuda_fail(e, "conditional node"));
        }
    } else {
        for (int c = 0; c < s->extra_iters; c++) vcycle<double>(s->h64, s->st, 10, 1);
    }
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(s->st, &got);
    if (e != cudaSuccess) {
        cudaGraphDestroy(root);
        return cuda_fail(e, "cudaStreamEndCapture");
    }
    const long cm0 = launch_count();
    if (mixed && mixed_extra == 0) {
        e = cudaStreamBeginCaptureToGraph(s->st, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaGraphDestroy(root);
            return cuda_fail(e, "cudaStreamBeginCaptureToGraph(merge)");
        }
        mixed_end(s);
        e = cudaStreamEndCapture(s->st, &got);
        if (e != cudaSuccess) {
            cudaGraphDestroy(root);
            return cuda_fail(e, "cudaStreamEndCapture(merge)");
        }
    }
    const long c1 = launch_count();
    // loop body: one pass and the convergence test
    e = cudaStreamBeginCaptureToGraph(s->st, wp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(root);
        return cuda_fail(e, "cudaStreamBeginCaptureToGraph(body)");
    }
    if (mixed) {
        for (int c = 0; c < inner; c++) vcycle<float>(s->h32, s->st, 10, 1, c == 0);
        ff_correct(s->zhi, s->zlo, s->h32.lv[0].z, count, s->st);
    } else {
        vcycle<double>(s->h64, s->st, 10, 1);
    }
    launch_norms(s, mixed);
    k_loop_check<<<1, 32, 0, s->st>>>(s->dnorm, s->F.flags, tol2, loop_cap(s, per_pass), h);
    note_launch();
    e = cudaStreamEndCapture(s->st, &got);
    if (e != cudaSuccess) {
        cudaGraphDestroy(root);
        return cuda_fail(e, "cudaStreamEndCapture(body)");
    }
    const long c2 = launch_count();
    discount_launches(c2 - c0);  // graph nodes, counted when they execute
    s->n_loop_merge = c1 - cm0;
    s->n_loop_outer = cm0 - c0;
    s->n_loop_body = c2 - c1;
    e = cudaGraphInstantiate(&slot, root, 0);
    cudaGraphDestroy(root);
    if (e != cudaSuccess) {
        slot = nullptr;
        return cuda_fail(e, "cudaGraphInstantiate(solve loop)");
    }
    slot_inner = inner;
    return STZG_OK;
}

static int solve_device_loop(stzg_sim *s, int *ncyc, bool fused_extrap) {
    const bool mixed = s->O.precision == STZG_MIXED;
    // three FP32 V-cycles per pass by default: with the extra V-cycle after
    // the loop, one, two and three per pass run equally fast at 2048^2, and
    // three leave the smallest error against the FP64 path
    const int inner = mixed ? (s->O.inner_cycles > 0 ? s->O.inner_cycles : 3) : 1;
    STZG_CHECK(build_loop_graph(s, mixed, inner, fused_extrap));
    STZG_CUDA(cudaGraphLaunch(fused_extrap ? s->g_loop_x : s->g_loop, s->st));
    if (s->defer_checks) {
        // a multi-step call reads the pass counts and errors once, at its end
        g_launches.fetch_add(s->n_loop_outer);
        s->defer_solves++;
        s->defer_inner = inner;
        if (ncyc) *ncyc = 0;
        return STZG_OK;
    }
    STZG_CUDA(cudaMemcpyAsync(s->hflags, s->F.flags, FL_COUNT * sizeof(int), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaMemcpyAsync(s->hnorm, s->dnorm, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    const int passes = s->hflags[FL_PASSES], err = s->hflags[FL_LOOP_ERR];
    g_launches.fetch_add(s->n_loop_outer + (passes > 0 ? s->n_loop_merge : 0) + passes * s->n_loop_body);
    const double r2 = s->hnorm[0], b2 = s->hnorm[1];
    s->acc.checks += passes + 1;
    s->acc.last_error = b2 > 0 ? std::sqrt(r2 / b2) : std::sqrt(r2);
    if (s->hflags[FL_MG_BAR_ERR]) return check_flags(s);  // reports and clears the barrier error
    if (err == 2) return fail(STZG_ENAN, "NaN residual");
    if (err == 1) return fail(STZG_ENOTCONV, mixed ? "iterative refinement did not converge"
                                                   : "multigrid did not converge");
    const int cycles = passes * inner;
    s->acc.vcycles += cycles;
    if (mixed) s->acc.refinements += passes;
    s->acc.extra_vcycles += s->extra_iters;
    s->acc.solves++;
    s->avg_vcount += cycles;
    s->avg_solves++;
    if (ncyc) *ncyc = cycles;
    return STZG_OK;
}

int solve(stzg_sim *s, int *ncyc) {
    if (s->O.tol_mode == STZG_TOL_RELATIVE && s->O.use_graphs) return solve_device_loop(s, ncyc, false);
    return s->O.precision == STZG_MIXED ? solve_mixed(s, ncyc) : solve_fp64(s, ncyc);
}

// Whether the next solve takes its linear extrapolation inside the solve
// graph (fused with the float-float split): mixed precision in the
// device-side loop with the extra V-cycle, whose merge rewrites the velocity.
static bool fused_extrapolation(const stzg_sim *s) {
    return s->O.precision == STZG_MIXED && s->O.tol_mode == STZG_TOL_RELATIVE && s->O.use_graphs &&
           s->O.extrapolate == 1 && s->have_prev && s->extra_iters > 0;
}

int do_projection(stzg_sim *s, double dt, bool fresh_combinations) {
    STZG_CHECK(ensure_ops(s, dt));
    if (!fresh_combinations) precombine(s->sc, s->F, s->cur, dt, s->st);
    const double bv = bdry_vel(s, s->time), bp = bdry_pos(s, s->time);
    projection_source(s->sc, s->F, s->cur, dt, s->q.bcs * s->q.cxx * bv, s->st);
    if (fused_extrapolation(s)) {
        STZG_CHECK(solve_device_loop(s, nullptr, true));
        projection_apply(s->sc, s->F, s->cur, dt, bv, bp, s->st);
        s->bv_state = bv;
        return STZG_OK;
    }
    if (s->O.extrapolate) {
        const long cnt = (long)s->m * (s->n + 1);
        if (s->have_prev && s->O.extrapolate >= 2 && s->have_prev2) {
            extrapolate_guess2(s->F.vel, s->vel_prev, s->vel_prev2, cnt, s->st);
        } else if (s->have_prev) {
            if (s->O.extrapolate >= 2) {
                STZG_CUDA(cudaMemcpyAsync(s->vel_prev2, s->vel_prev, cnt * sizeof(double2), cudaMemcpyDeviceToDevice,
                                          s->st));
                s->have_prev2 = true;
            }
            extrapolate_guess(s->F.vel, s->vel_prev, cnt, s->st);
        } else {
            STZG_CUDA(cudaMemcpyAsync(s->vel_prev, s->F.vel, cnt * sizeof(double2), cudaMemcpyDeviceToDevice, s->st));
            s->have_prev = true;
        }
    }
    STZG_CHECK(solve(s, nullptr));
    projection_apply(s->sc, s->F, s->cur, dt, bv, bp, s->st);
    s->bv_state = bv;
    return STZG_OK;
}

int do_advection(stzg_sim *s, double dt) {
    advection(s->sc, *s->maps, s->F, s->cur, dt, s->bv_state, s->st);
    s->cur ^= 1;
    return STZG_OK;
}

int check_flags(stzg_sim *s) {
    int *h = s->hflags;
    STZG_CUDA(cudaMemcpyAsync(h, s->F.flags, FL_COUNT * sizeof(int), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    if (h[FL_SUBSTEP_MAX] > s->acc.substeps_max) s->acc.substeps_max = h[FL_SUBSTEP_MAX];
    if (h[FL_TMA])
        return fail(STZG_ECUDA, "an advection tile copy did not complete in time; tiles of the step were "
                                "left unwritten, so the handle's state is undefined: recreate the handle");
    if (h[FL_SUBSTEP_CAP]) return fail(STZG_ESUBSTEP, "plastic sub-stepping reached its iteration cap");
    if (h[FL_MG_BAR_ERR]) {
        // the barrier's words are left mid-count: clear them for the next launch
        STZG_CUDA(cudaMemsetAsync(s->F.flags + FL_MG_BAR_ERR, 0, (FL_MG_BAR + 2 - FL_MG_BAR_ERR) * sizeof(int), s->st));
        STZG_CUDA(cudaStreamSynchronize(s->st));
        return fail(STZG_ECUDA, "a grid barrier of the persistent coarse multigrid kernel timed out; the "
                                "velocity of the step is invalid: recreate the handle");
    }
    return STZG_OK;
}

size_t cell_count(const stzg_sim *s) { return (size_t)s->m * (s->n + 2); }

}  // namespace stzg

extern "C" {

void stzg_default_options(stzg_options *o) {
    std::memset(o, 0, sizeof(*o));
    o->precision = STZG_FP64;
    o->tol_mode = STZG_TOL_REFERENCE;
    o->tol = 1e4;
    o->track_plastic = 1;
    o->device = 0;
    o->inner_cycles = 0;
    o->use_graphs = 1;
    o->extrapolate = 0;
}

const char *stzg_strerror(int st) {
    switch (st) {
        case STZG_OK: return "ok";
        case STZG_EINVAL: return "invalid argument";
        case STZG_ENOMEM: return "out of device memory";
        case STZG_ECUDA: return "CUDA error";
        case STZG_ENOTCONV: return "multigrid did not converge";
        case STZG_ENAN: return "NaN residual";
        case STZG_ESUBSTEP: return "plastic sub-step cap reached";
        case STZG_ENODEV: return "no usable GPU";
    }
    return "unknown status";
}

const char *stzg_last_message(void) { return g_msg.c_str(); }

int stzg_create(const stz_params *p, const stzg_options *opt, stzg_sim **out) {
    if (!out) return fail(STZG_EINVAL, "null output handle");
    *out = nullptr;
    STZG_CHECK(validate(p));
    stzg_options o;
    if (opt) o = *opt;
    else stzg_default_options(&o);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(STZG_ENODEV, "no CUDA device");
    if (o.device < 0 || o.device >= ndev) return fail(STZG_EINVAL, "device ordinal out of range");
    STZG_CUDA(cudaSetDevice(o.device));
    STZG_CUDA(prepare_step_kernels());
    stzg_sim *s = new stzg_sim;
    s->P = *p;
    s->O = o;
    s->m = p->m;
    s->n = p->n;
    s->sc = make_step_consts(*p);
    s->sc.track_plastic = o.track_plastic;
    s->sc.sp_increments = o.precision == STZG_MIXED && o.advection != STZG_ADV_FP64;
    if (o.substep_cap > 0) s->sc.substep_cap = o.substep_cap;
    int st = STZG_OK;
    auto bail = [&](int code) {
        stzg_destroy(s);
        return code;
    };
    if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(STZG_ECUDA, "stream creation failed"));
    const size_t nc = cell_count(s), nn = (size_t)s->m * (s->n + 1);
    std::memset(&s->F, 0, sizeof(s->F));
    for (int b = 0; b < 2; b++)
        for (int k = 0; k < F_COUNT; k++)
            if ((st = dev_alloc(s, (void **)&s->F.f[b][k], nc * sizeof(double))) != STZG_OK) return bail(st);
    if ((st = dev_alloc(s, (void **)&s->F.ddev, nc * sizeof(double))) != STZG_OK) return bail(st);
    if ((st = dev_alloc(s, (void **)&s->F.eps_pl, (size_t)s->m * s->n * sizeof(double))) != STZG_OK) return bail(st);
    if ((st = dev_alloc(s, (void **)&s->F.vel, nn * sizeof(double2))) != STZG_OK) return bail(st);
    if ((st = dev_alloc(s, (void **)&s->F.src, nn * sizeof(double2))) != STZG_OK) return bail(st);
    if ((st = dev_alloc(s, (void **)&s->F.flags, FL_COUNT * sizeof(int))) != STZG_OK) return bail(st);
    for (int k = 0; k < 4; k++)
        if ((st = dev_alloc(s, (void **)&s->F.pre[k], nc * sizeof(double))) != STZG_OK) return bail(st);
    // cells the float-float advection hands to the FP64 plastic pass (at most all of them)
    if ((st = dev_alloc(s, (void **)&s->F.plist, (size_t)s->m * s->n * sizeof(unsigned))) != STZG_OK) return bail(st);
    if ((st = dev_alloc(s, (void **)&s->F.pcount, sizeof(unsigned))) != STZG_OK) return bail(st);
    s->maps = new field_maps;
    if ((st = make_field_maps(s->sc, s->F, s->maps)) != STZG_OK) return bail(st);
    if (o.extrapolate)
        if ((st = dev_alloc(s, (void **)&s->vel_prev, nn * sizeof(double2))) != STZG_OK) return bail(st);
    if (o.extrapolate >= 2)
        if ((st = dev_alloc(s, (void **)&s->vel_prev2, nn * sizeof(double2))) != STZG_OK) return bail(st);
    s->npart = reduction_blocks();
    if ((st = dev_alloc(s, (void **)&s->partials, 2 * s->npart * sizeof(double))) != STZG_OK) return bail(st);
    if ((st = dev_alloc(s, (void **)&s->dnorm, 2 * sizeof(double))) != STZG_OK) return bail(st);
    if (cudaMallocHost(&s->hnorm, 2 * sizeof(double)) != cudaSuccess) return bail(fail(STZG_ENOMEM, "pinned alloc"));
    if (cudaMallocHost(&s->hflags, FL_COUNT * sizeof(int)) != cudaSuccess)
        return bail(fail(STZG_ENOMEM, "pinned alloc"));
    // FP64 hierarchy over vel/src; FP32 hierarchy with its own top arrays
    if ((st = s->h64.allocate(s->m, s->n + 1, s->F.vel, s->F.src)) != STZG_OK) return bail(st);
    if (o.precision == STZG_MIXED) {
        if ((st = s->h32.allocate(s->m, s->n + 1, nullptr, nullptr)) != STZG_OK) return bail(st);
        // the grid barrier of the persistent coarse kernel lives in the handle's
        // flag words; the kernel is off by default (stzg_set_mg_persistent)
        s->h32.bar = reinterpret_cast<unsigned *>(s->F.flags + FL_MG_BAR);
        s->h32.bar_err = s->F.flags + FL_MG_BAR_ERR;
        s->h32.persist = 0;
        float2 **ffa[4] = {&s->zhi, &s->zlo, &s->bhi, &s->blo};
        for (int k = 0; k < 4; k++)
            if ((st = dev_alloc(s, (void **)ffa[k], nn * sizeof(float2))) != STZG_OK) return bail(st);
    }
    cudaEventCreate(&s->ev0);
    cudaEventCreate(&s->ev1);
    if (cudaStreamSynchronize(s->st) != cudaSuccess) return bail(fail(STZG_ECUDA, "set-up failed"));
    *out = s;
    return STZG_OK;
}

int stzg_destroy(stzg_sim *s) {
    if (!s) return STZG_OK;
    if (s->st) cudaStreamSynchronize(s->st);
    drop_graphs(s);
    adjoint_release(s);
    for (int k = 0; k < stzg_sim::kCopyStreams; k++) {
        if (s->cst[k]) cudaStreamDestroy(s->cst[k]);
        if (s->cev[k]) cudaEventDestroy(s->cev[k]);
    }
    if (s->cev_ready) cudaEventDestroy(s->cev_ready);
    for (void *p : s->owned) cudaFree(p);
    delete s->maps;
    s->h64.release();
    s->h32.release();
    if (s->hnorm) cudaFreeHost(s->hnorm);
    if (s->hflags) cudaFreeHost(s->hflags);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
    return STZG_OK;
}

int stzg_set_state(stzg_sim *s, const double *chi) {
    if (!s || !chi) return fail(STZG_EINVAL, "null argument");
    const int m = s->m, n = s->n;
    const size_t nc = cell_count(s);
    std::vector<double> zero(nc, 0.0), X(nc, 0.0), Y(nc, 0.0), C(nc, 0.0);
    const double dx = (s->P.bx - s->P.ax) / m, dy = (s->P.by - s->P.ay) / n;
    for (int j = -1; j <= n; j++)
        for (int i = 0; i < m; i++) {
            size_t k = (size_t)(j + 1) * m + i;
            X[k] = s->P.ax + i * dx;
            Y[k] = s->P.ay + j * dy;
            if (j >= 0 && j < n) C[k] = chi[(size_t)j * m + i];
        }
    for (int i = 0; i < m; i++) {
        C[i] = 2 * C[(size_t)m + i] - C[(size_t)2 * m + i];
        C[(size_t)(n + 1) * m + i] = 2 * C[(size_t)n * m + i] - C[(size_t)(n - 1) * m + i];
    }
    for (int b = 0; b < 2; b++) {
        for (int k = 0; k < F_CHI; k++)
            STZG_CUDA(cudaMemcpyAsync(s->F.f[b][k], zero.data(), nc * 8, cudaMemcpyHostToDevice, s->st));
        STZG_CUDA(cudaMemcpyAsync(s->F.f[b][F_CHI], C.data(), nc * 8, cudaMemcpyHostToDevice, s->st));
        STZG_CUDA(cudaMemcpyAsync(s->F.f[b][F_X], X.data(), nc * 8, cudaMemcpyHostToDevice, s->st));
        STZG_CUDA(cudaMemcpyAsync(s->F.f[b][F_Y], Y.data(), nc * 8, cudaMemcpyHostToDevice, s->st));
    }
    STZG_CUDA(cudaMemsetAsync(s->F.ddev, 0, nc * 8, s->st));
    STZG_CUDA(cudaMemsetAsync(s->F.eps_pl, 0, (size_t)m * n * 8, s->st));
    STZG_CUDA(cudaMemsetAsync(s->F.vel, 0, (size_t)m * (n + 1) * sizeof(double2), s->st));
    STZG_CUDA(cudaMemsetAsync(s->F.flags, 0, FL_COUNT * sizeof(int), s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    s->time = 0;
    s->bv_state = 0;
    s->cur = 0;
    s->have_prev = s->have_prev2 = false;
    return STZG_OK;
}

static int field_slot(int field) {
    switch (field) {
        case STZG_P: return F_P;
        case STZG_Q: return F_Q;
        case STZG_S: return F_S;
        case STZG_TAU: return F_TAU;
        case STZG_CHI: return F_CHI;
        case STZG_X: return F_X;
        case STZG_Y: return F_Y;
    }
    return -1;
}

int stzg_get_field(stzg_sim *s, int field, double *host) {
    if (!s || !host) return fail(STZG_EINVAL, "null argument");
    const int m = s->m, n = s->n;
    const size_t nn = (size_t)m * (n + 1), nc = cell_count(s);
    if (field == STZG_U || field == STZG_V) {
        std::vector<double2> v(nn);
        STZG_CUDA(cudaMemcpyAsync(v.data(), s->F.vel, nn * sizeof(double2), cudaMemcpyDeviceToHost, s->st));
        STZG_CUDA(cudaStreamSynchronize(s->st));
        const double bv = s->bv_state;
        for (int j = 0; j <= n; j++)
            for (int i = 0; i < m; i++) {
                size_t k = (size_t)j * m + i;
                double val = field == STZG_U ? v[k].x : v[k].y;
                if (j == 0) val = field == STZG_U ? -bv : 0.0;
                if (j == n) val = field == STZG_U ? bv : 0.0;
                host[k] = val;
            }
        return STZG_OK;
    }
    if (field == STZG_EPS_PL) {
        STZG_CUDA(cudaMemcpyAsync(host, s->F.eps_pl, (size_t)m * n * 8, cudaMemcpyDeviceToHost, s->st));
        STZG_CUDA(cudaStreamSynchronize(s->st));
        return STZG_OK;
    }
    if (field == STZG_DDEV) {
        STZG_CUDA(cudaMemcpyAsync(host, s->F.ddev, nc * 8, cudaMemcpyDeviceToHost, s->st));
        STZG_CUDA(cudaStreamSynchronize(s->st));
        return STZG_OK;
    }
    int slot = field_slot(field);
    if (slot < 0) return fail(STZG_EINVAL, "unknown field id");
    const double *src = s->F.f[s->cur][slot];
    if (slot == F_X || slot == F_Y) src += m;  // node rows 0..n
    size_t cnt = (slot == F_X || slot == F_Y) ? nn : nc;
    STZG_CUDA(cudaMemcpyAsync(host, src, cnt * 8, cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

int stzg_set_field(stzg_sim *s, int field, const double *host) {
    if (!s || !host) return fail(STZG_EINVAL, "null argument");
    const int m = s->m, n = s->n;
    const size_t nn = (size_t)m * (n + 1), nc = cell_count(s);
    if (field == STZG_U || field == STZG_V) {
        std::vector<double2> v(nn);
        STZG_CUDA(cudaMemcpy(v.data(), s->F.vel, nn * sizeof(double2), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < nn; k++) (field == STZG_U ? v[k].x : v[k].y) = host[k];
        STZG_CUDA(cudaMemcpy(s->F.vel, v.data(), nn * sizeof(double2), cudaMemcpyHostToDevice));
        s->have_prev = s->have_prev2 = false;
        // walls carry +-bv on u and 0 on v (set_boundaries, shear_sim.cc:557-572)
        if (field == STZG_U) s->bv_state = host[(size_t)n * m];
        return STZG_OK;
    }
    if (field == STZG_EPS_PL) {
        STZG_CUDA(cudaMemcpy(s->F.eps_pl, host, (size_t)m * n * 8, cudaMemcpyHostToDevice));
        return STZG_OK;
    }
    if (field == STZG_DDEV) {
        STZG_CUDA(cudaMemcpy(s->F.ddev, host, nc * 8, cudaMemcpyHostToDevice));
        return STZG_OK;
    }
    int slot = field_slot(field);
    if (slot < 0) return fail(STZG_EINVAL, "unknown field id");
    for (int b = 0; b < 2; b++) {
        double *dst = s->F.f[b][slot];
        if (slot == F_X || slot == F_Y) dst += m;
        size_t cnt = (slot == F_X || slot == F_Y) ? nn : nc;
        STZG_CUDA(cudaMemcpy(dst, host, cnt * 8, cudaMemcpyHostToDevice));
    }
    return STZG_OK;
}

int stzg_init_fields(stzg_sim *s, int chi_case, double tem_base, double tem_delta) {
    if (!s) return fail(STZG_EINVAL, "null handle");
    const int m = s->m, n = s->n;
    std::vector<double> full((size_t)m * (n + 2));
    init_fields_chi(s->P, chi_case, tem_base, tem_delta, full.data());
    STZG_CHECK(stzg_set_state(s, full.data() + m));
    return stzg_set_field(s, STZG_CHI, full.data());  // the formula's own ghost rows
}

int stzg_chi_bicubic(stzg_sim *s, int mm, int nn, const double *arr, double lo, double sca) {
    if (!s || !arr) return fail(STZG_EINVAL, "null argument");
    if (mm < 1 || nn < 2) return fail(STZG_EINVAL, "the sample grid needs mm >= 1 and nn >= 2");
    std::vector<double> chi((size_t)s->m * s->n);
    bicubic_chi(s->P, mm, nn, arr, lo, sca, chi.data());
    return stzg_set_state(s, chi.data());
}

int stzg_set_time(stzg_sim *s, double t) {
    if (!s) return fail(STZG_EINVAL, "null handle");
    s->time = t;
    return STZG_OK;
}

int stzg_get_time(stzg_sim *s, double *t) {
    if (!s || !t) return fail(STZG_EINVAL, "null argument");
    *t = s->time;
    return STZG_OK;
}

// The end of a multi-step call with deferred checks: the accumulated pass
// count and the first error of its solves.
static int finish_deferred(stzg_sim *s) {
    s->defer_checks = false;
    STZG_CUDA(cudaMemcpyAsync(s->hflags, s->F.flags, FL_COUNT * sizeof(int), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaMemcpyAsync(s->hnorm, s->dnorm, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    const bool mixed = s->O.precision == STZG_MIXED;
    const long passes = s->hflags[FL_PASSES_SUM], solves = s->defer_solves;
    const int err = s->hflags[FL_ERR_FIRST];
    g_launches.fetch_add(passes * s->n_loop_body);
    const double r2 = s->hnorm[0], b2 = s->hnorm[1];
    s->acc.checks += passes + solves;
    s->acc.last_error = b2 > 0 ? std::sqrt(r2 / b2) : std::sqrt(r2);
    // the step kernels' own failures (sub-step cap, tile copies, coarse
    // barrier) come first: a solver error after them is their consequence
    STZG_CHECK(check_flags(s));
    if (err == 2) return fail(STZG_ENAN, "NaN residual");
    if (err == 1) return fail(STZG_ENOTCONV, mixed ? "iterative refinement did not converge"
                                                   : "multigrid did not converge");
    const long cycles = passes * s->defer_inner;
    s->acc.vcycles += cycles;
    if (mixed) s->acc.refinements += passes;
    s->acc.extra_vcycles += solves * s->extra_iters;
    s->acc.solves += solves;
    s->avg_vcount += cycles;
    s->avg_solves += solves;
    return STZG_OK;
}

int stzg_step_qs(stzg_sim *s, double dt, int nsteps, stzg_stats *stats) {
    if (!s || nsteps < 0 || !(dt > 0)) return fail(STZG_EINVAL, "bad step arguments");
    stzg_stats before = s->acc;
    const long l0 = launch_count();
    STZG_CHECK(ensure_ops(s, dt));
    // Several steps in one call run without a host round trip between them:
    // the device-side solve loops accumulate their pass counts and their
    // first error in the flag words, read once after the last step.  A
    // failure is then reported after that step (the state is undefined after
    // a failed step either way).  Needs the device loop and no pass-dependent
    // merge (the extra V-cycle merges every solve).
    const bool defer = nsteps > 1 && s->O.tol_mode == STZG_TOL_RELATIVE && s->O.use_graphs &&
                       (s->O.precision != STZG_MIXED || s->extra_iters > 0);
    if (defer) {
        STZG_CUDA(cudaMemsetAsync(s->F.flags + FL_PASSES_SUM, 0, 2 * sizeof(int), s->st));
        s->defer_checks = true;
        s->defer_solves = 0;
    }
    STZG_CUDA(cudaEventRecord(s->ev0, s->st));
    for (int k = 0; k < nsteps; k++) {
        s->time += dt;  // shear_sim.cc:283
        int st = do_advection(s, dt);
        if (st == STZG_OK) st = do_projection(s, dt, true);
        if (st == STZG_OK && !defer) st = check_flags(s);
        if (st != STZG_OK) {
            s->defer_checks = false;
            return st;
        }
    }
    STZG_CUDA(cudaEventRecord(s->ev1, s->st));
    STZG_CUDA(cudaEventSynchronize(s->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->acc.seconds += ms * 1e-3;
    if (defer) STZG_CHECK(finish_deferred(s));
    STZG_CHECK(check_flags(s));
    if (stats) {
        *stats = s->acc;
        stats->vcycles -= before.vcycles;
        stats->extra_vcycles -= before.extra_vcycles;
        stats->solves -= before.solves;
        stats->refinements -= before.refinements;
        stats->checks -= before.checks;
        stats->seconds -= before.seconds;
        stats->kernel_launches = launch_count() - l0;
    }
    return STZG_OK;
}

// Bulk transfers: the field copies are spread over kCopyStreams streams so
// that several copy engines move data at once; they start after the work
// already queued on the handle's stream and the call returns when all are
// done.
static int copy_streams(stzg_sim *s) {
    if (s->cev_ready) return STZG_OK;
    for (int k = 0; k < stzg_sim::kCopyStreams; k++) {
        STZG_CUDA(cudaStreamCreateWithFlags(&s->cst[k], cudaStreamNonBlocking));
        STZG_CUDA(cudaEventCreateWithFlags(&s->cev[k], cudaEventDisableTiming));
    }
    STZG_CUDA(cudaEventCreateWithFlags(&s->cev_ready, cudaEventDisableTiming));
    return STZG_OK;
}

struct copy_job {
    void *dst;
    const void *src;
    size_t bytes;
};

// Enqueues the copies on the copy streams after the work queued so far on
// the handle's stream; returns without waiting.
static int enqueue_copies(stzg_sim *s, const std::vector<copy_job> &jobs, cudaMemcpyKind kind) {
    STZG_CHECK(copy_streams(s));
    STZG_CUDA(cudaEventRecord(s->cev_ready, s->st));
    const int ns = stzg_sim::kCopyStreams;
    for (int k = 0; k < ns; k++) STZG_CUDA(cudaStreamWaitEvent(s->cst[k], s->cev_ready, 0));
    // every copy in ns pieces of whole 8-byte words, one per stream
    for (const copy_job &j : jobs) {
        const size_t words = j.bytes / 8, per = (words + ns - 1) / ns;
        for (int k = 0; k < ns; k++) {
            const size_t w0 = (size_t)k * per, w1 = std::min(words, w0 + per);
            if (w1 <= w0) continue;
            STZG_CUDA(cudaMemcpyAsync((char *)j.dst + 8 * w0, (const char *)j.src + 8 * w0, 8 * (w1 - w0), kind,
                                      s->cst[k]));
        }
    }
    return STZG_OK;
}

// Makes the handle's stream wait for every copy enqueued so far.
static int join_copies(stzg_sim *s) {
    for (int k = 0; k < stzg_sim::kCopyStreams; k++) {
        STZG_CUDA(cudaEventRecord(s->cev[k], s->cst[k]));
        STZG_CUDA(cudaStreamWaitEvent(s->st, s->cev[k], 0));
    }
    return STZG_OK;
}

static int run_copies(stzg_sim *s, const std::vector<copy_job> &jobs, cudaMemcpyKind kind) {
    STZG_CHECK(enqueue_copies(s, jobs, kind));
    STZG_CHECK(join_copies(s));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

// Installs an uploaded velocity (staged in src, which every step rewrites)
// and flags whether it differs bitwise from the velocity it replaces.
__global__ void k_accept_vel(const double2 *__restrict__ staged, double2 *__restrict__ vel, long count,
                             int *changed) {
    int diff = 0;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
        const double2 a = staged[k], b = vel[k];
        diff |= (__double_as_longlong(a.x) != __double_as_longlong(b.x)) |
                (__double_as_longlong(a.y) != __double_as_longlong(b.y));
        vel[k] = a;
    }
    if (__syncthreads_or(diff) && threadIdx.x == 0) atomicExch(changed, 1);
}

int stzg_upload(stzg_sim *s, const double *const *up) {
    if (!s || !up) return fail(STZG_EINVAL, "null argument");
    const int m = s->m;
    const size_t nn = (size_t)m * (s->n + 1), nc = cell_count(s);
    std::vector<copy_job> jobs;
    for (int k = 0; k < 7; k++) {
        if (!up[k]) continue;
        double *dst = s->F.f[s->cur][k];
        size_t cnt = nc;
        if (k == F_X || k == F_Y) {
            dst += m;
            cnt = nn;
        }
        jobs.push_back({dst, up[k], cnt * 8});
    }
    // The velocity goes through a staging copy: when it is bit-identical to
    // the one on the device (a caller that downloads and uploads the state
    // around every step), the solver keeps its history for the extrapolated
    // initial guess; any other velocity restarts that history.
    if (up[7]) jobs.push_back({s->F.src, up[7], nn * sizeof(double2)});
    STZG_CHECK(run_copies(s, jobs, cudaMemcpyHostToDevice));
    if (up[7]) {
        STZG_CUDA(cudaMemsetAsync(s->F.flags + 2, 0, sizeof(int), s->st));
        k_accept_vel<<<4 * 152, 256, 0, s->st>>>(s->F.src, s->F.vel, (long)nn, s->F.flags + 2);
        note_launch();
        int changed = 0;
        STZG_CUDA(cudaMemcpyAsync(&changed, s->F.flags + 2, sizeof(int), cudaMemcpyDeviceToHost, s->st));
        STZG_CUDA(cudaStreamSynchronize(s->st));
        if (changed) s->have_prev = s->have_prev2 = false;
    }
    return STZG_OK;
}

// One quasi-static step on host-owned fields: upload, step, download.  The
// parts of the new state that the projection does not change (the rows of
// chi, the interior rows of X and Y, eps_pl) are copied back while the
// multigrid solve runs; the rest follows the projection.
int stzg_step_qs_host(stzg_sim *s, double dt, const double *const *up, double *const *down, stzg_stats *stats) {
    if (!s || !up || !down || !(dt > 0)) return fail(STZG_EINVAL, "bad step arguments");
    STZG_CHECK(stzg_upload(s, up));
    stzg_stats before = s->acc;
    const long l0 = launch_count();
    STZG_CHECK(ensure_ops(s, dt));
    STZG_CUDA(cudaEventRecord(s->ev0, s->st));
    s->time += dt;  // shear_sim.cc:283
    STZG_CHECK(do_advection(s, dt));
    const int m = s->m, n = s->n;
    const size_t nn = (size_t)m * (n + 1), nc = cell_count(s), row = (size_t)m * 8;
    double *const *f = s->F.f[s->cur];
    std::vector<copy_job> early, late;
    if (down[F_CHI]) {
        early.push_back({down[F_CHI] + m, f[F_CHI] + m, n * row});
        late.push_back({down[F_CHI], f[F_CHI], row});
        late.push_back({down[F_CHI] + (size_t)(n + 1) * m, f[F_CHI] + (size_t)(n + 1) * m, row});
    }
    for (int k : {F_X, F_Y}) {
        if (!down[k]) continue;
        // node rows 0..n live at offset m of the cell-layout array
        early.push_back({down[k] + m, f[k] + 2 * (size_t)m, (n - 1) * row});
        late.push_back({down[k], f[k] + m, row});
        late.push_back({down[k] + (size_t)n * m, f[k] + (size_t)(n + 1) * m, row});
    }
    if (down[8]) early.push_back({down[8], s->F.eps_pl, (size_t)m * n * 8});
    STZG_CHECK(enqueue_copies(s, early, cudaMemcpyDeviceToHost));
    {
        // on failure, the copies already queued into the caller's buffers
        // finish before the call returns
        const int st = do_projection(s, dt, true);
        if (st != STZG_OK) {
            join_copies(s);
            cudaStreamSynchronize(s->st);
            return st;
        }
    }
    for (int k = 0; k < F_CHI; k++)
        if (down[k]) late.push_back({down[k], f[k], nc * 8});
    if (down[7]) late.push_back({down[7], s->F.vel, nn * sizeof(double2)});
    STZG_CUDA(cudaEventRecord(s->ev1, s->st));
    STZG_CHECK(enqueue_copies(s, late, cudaMemcpyDeviceToHost));
    STZG_CHECK(join_copies(s));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->acc.seconds += ms * 1e-3;
    STZG_CHECK(check_flags(s));
    if (stats) {
        *stats = s->acc;
        stats->vcycles -= before.vcycles;
        stats->extra_vcycles -= before.extra_vcycles;
        stats->solves -= before.solves;
        stats->refinements -= before.refinements;
        stats->checks -= before.checks;
        stats->seconds -= before.seconds;
        stats->kernel_launches = launch_count() - l0;
    }
    return STZG_OK;
}

int stzg_download(stzg_sim *s, double *const *down) {
    if (!s || !down) return fail(STZG_EINVAL, "null argument");
    const int m = s->m;
    const size_t nn = (size_t)m * (s->n + 1), nc = cell_count(s);
    std::vector<copy_job> jobs;
    for (int k = 0; k < 7; k++) {
        if (!down[k]) continue;
        const double *src = s->F.f[s->cur][k];
        size_t cnt = nc;
        if (k == F_X || k == F_Y) {
            src += m;
            cnt = nn;
        }
        jobs.push_back({down[k], src, cnt * 8});
    }
    if (down[7]) jobs.push_back({down[7], s->F.vel, nn * sizeof(double2)});
    if (down[8]) jobs.push_back({down[8], s->F.eps_pl, (size_t)m * s->n * 8});
    return run_copies(s, jobs, cudaMemcpyDeviceToHost);
}

int stzg_set_mg_persistent(stzg_sim *s, int on) {
    if (!s || s->O.precision != STZG_MIXED) return fail(STZG_EINVAL, "needs a mixed-precision handle");
    STZG_CUDA(cudaSetDevice(s->O.device));
    if (on && !coarse_persist_supported())
        return fail(STZG_EINVAL, "the device does not take the persistent coarse kernel");
    if ((on != 0) != (s->h32.persist != 0)) {
        STZG_CUDA(cudaStreamSynchronize(s->st));
        drop_graphs(s);  // captured V-cycles used the other schedule
        s->h32.persist = on ? 1 : 0;
    }
    if (on == 2) {
        // test of the barrier's time limit: an arrival count that no block
        // completes, so the next persistent launch's first barrier runs out
        STZG_CUDA(cudaMemsetAsync(s->F.flags + FL_MG_BAR, 0x40, sizeof(int), s->st));
        STZG_CUDA(cudaStreamSynchronize(s->st));
    }
    return STZG_OK;
}

int stzg_get_mg_persistent(stzg_sim *s, int *on) {
    if (!s || !on) return fail(STZG_EINVAL, "null argument");
    if (s->O.precision != STZG_MIXED) *on = 0;
    else if (!s->h32.bottom_inv) *on = s->h32.persist;  // operators not built yet (first step)
    else *on = coarse_persist_active(s->h32) ? 1 : 0;
    return STZG_OK;
}

int stzg_time_kernel(stzg_sim *s, double dt, int kernel, int reps, double *ms) {
    if (!s || !ms || reps < 1 || !(dt > 0)) return fail(STZG_EINVAL, "bad arguments");
    STZG_CHECK(ensure_ops(s, dt));
    if ((kernel == 2 || (kernel >= 4 && kernel <= 7)) && s->O.precision != STZG_MIXED)
        return fail(STZG_EINVAL, "FP32 kernels need a mixed-precision handle");
    auto one = [&]() -> int {
        switch (kernel) {
            case 0: advection(s->sc, *s->maps, s->F, s->cur, dt, s->bv_state, s->st); break;
            case 1: top_sweep<double>(s->h64, s->st); break;
            case 2: top_sweep<float>(s->h32, s->st); break;
            case 3: vcycle<double>(s->h64, s->st, 10, 1); break;
            case 4: vcycle<float>(s->h32, s->st, 10, 1); break;
            case 5: launch_norms(s, true); break;
            case 6:
            case 7:
                if (!top_level_kernel(s->h32, kernel - 6, s->st))
                    return fail(STZG_EINVAL, "the top level does not use the streaming kernels");
                break;
            case 8:
                precombine(s->sc, s->F, s->cur, dt, s->st);
                projection_source(s->sc, s->F, s->cur, dt, s->q.bcs * s->q.cxx * s->bv_state, s->st);
                break;
            case 9:
                projection_apply(s->sc, s->F, s->cur, dt, s->bv_state, bdry_pos(s, s->time), s->st);
                break;
            default: return fail(STZG_EINVAL, "unknown kernel id");
        }
        return STZG_OK;
    };
    STZG_CHECK(one());  // warm-up
    STZG_CUDA(cudaEventRecord(s->ev0, s->st));
    for (int r = 0; r < reps; r++) STZG_CHECK(one());
    STZG_CUDA(cudaEventRecord(s->ev1, s->st));
    STZG_CUDA(cudaEventSynchronize(s->ev1));
    float t = 0;
    cudaEventElapsedTime(&t, s->ev0, s->ev1);
    *ms = t / reps;
    return STZG_OK;
}

// One explicit step (shear_sim::step_forward, shear_sim.cc:185-276): time
// first, the fused update, the new interior velocities from the staging
// array, then set_boundaries at the new time.
static int do_direct(stzg_sim *s, double dt) {
    s->time += dt;
    direct_step(s->sc, s->P.viscosity, s->F, s->cur, dt, s->bv_state, s->st);
    const size_t m = s->m;
    if (s->n > 1)
        STZG_CUDA(cudaMemcpyAsync(s->F.vel + m, s->F.src + m, (size_t)(s->n - 1) * m * sizeof(double2),
                                  cudaMemcpyDeviceToDevice, s->st));
    s->cur ^= 1;
    const double bv = bdry_vel(s, s->time), bp = bdry_pos(s, s->time);
    set_boundaries(s->sc, s->F, s->cur, bp, s->st);
    s->bv_state = bv;
    // the velocity no longer comes from a solve: restart the guess history
    s->have_prev = s->have_prev2 = false;
    return STZG_OK;
}

int stzg_step_direct(stzg_sim *s, double dt, int nsteps, stzg_stats *stats) {
    if (!s || nsteps < 0 || !(dt > 0)) return fail(STZG_EINVAL, "bad step arguments");
    const long l0 = launch_count();
    STZG_CUDA(cudaEventRecord(s->ev0, s->st));
    for (int k = 0; k < nsteps; k++) STZG_CHECK(do_direct(s, dt));
    STZG_CUDA(cudaEventRecord(s->ev1, s->st));
    STZG_CUDA(cudaEventSynchronize(s->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->acc.seconds += ms * 1e-3;
    STZG_CHECK(check_flags(s));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->seconds = ms * 1e-3;
        stats->substeps_max = s->acc.substeps_max;
        stats->kernel_launches = launch_count() - l0;
    }
    return STZG_OK;
}

int stzg_advance_direct(stzg_sim *s, double dt, double target, long *nsteps) {
    if (!s || !(dt > 0)) return fail(STZG_EINVAL, "bad step arguments");
    if (!(target > s->time)) return fail(STZG_EINVAL, "target time not after the current time");
    long k = 0;
    while (s->time + dt * (1 + 1e-8) < target) {
        STZG_CHECK(do_direct(s, dt));
        if (++k % 64 == 0) STZG_CHECK(check_flags(s));
    }
    STZG_CHECK(do_direct(s, target - s->time));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    STZG_CHECK(check_flags(s));
    if (nsteps) *nsteps = k + 1;
    return STZG_OK;
}

int stzg_advection_step(stzg_sim *s, double dt) {
    if (!s || !(dt > 0)) return fail(STZG_EINVAL, "bad arguments");
    STZG_CHECK(do_advection(s, dt));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return check_flags(s);
}

int stzg_projection_step(stzg_sim *s, double dt, stzg_stats *stats) {
    if (!s || !(dt > 0)) return fail(STZG_EINVAL, "bad arguments");
    STZG_CHECK(do_projection(s, dt, false));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    if (stats) *stats = s->acc;
    return STZG_OK;
}

int stzg_avg_iters(stzg_sim *s, double *avg) {
    if (!s || !avg) return fail(STZG_EINVAL, "null argument");
    *avg = s->avg_solves ? (double)s->avg_vcount / s->avg_solves : 0.0;
    s->avg_vcount = s->avg_solves = 0;
    return STZG_OK;
}

int stzg_mg_solve(stzg_sim *s, double dt, const double *src, double *vel, int *ncycles) {
    if (!s || !src || !vel || !(dt > 0)) return fail(STZG_EINVAL, "bad arguments");
    STZG_CHECK(ensure_ops(s, dt));
    const size_t nn = (size_t)s->m * (s->n + 1);
    STZG_CUDA(cudaMemcpyAsync(s->F.src, src, nn * sizeof(double2), cudaMemcpyHostToDevice, s->st));
    STZG_CUDA(cudaMemcpyAsync(s->F.vel, vel, nn * sizeof(double2), cudaMemcpyHostToDevice, s->st));
    int st = solve(s, ncycles);
    STZG_CUDA(cudaMemcpyAsync(vel, s->F.vel, nn * sizeof(double2), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return st;
}

int stzg_mg_vcycle(stzg_sim *s, double dt, const double *src, double *vel) {
    if (!s || !src || !vel || !(dt > 0)) return fail(STZG_EINVAL, "bad arguments");
    STZG_CHECK(ensure_ops(s, dt));
    const size_t nn = (size_t)s->m * (s->n + 1);
    STZG_CUDA(cudaMemcpyAsync(s->F.src, src, nn * sizeof(double2), cudaMemcpyHostToDevice, s->st));
    STZG_CUDA(cudaMemcpyAsync(s->F.vel, vel, nn * sizeof(double2), cudaMemcpyHostToDevice, s->st));
    STZG_CHECK(run_vcycles(s, 1));
    STZG_CUDA(cudaMemcpyAsync(vel, s->F.vel, nn * sizeof(double2), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

int stzg_mg_l2_error(stzg_sim *s, double dt, const double *src, const double *vel, double *err) {
    if (!s || !src || !vel || !err || !(dt > 0)) return fail(STZG_EINVAL, "bad arguments");
    STZG_CHECK(ensure_ops(s, dt));
    const size_t nn = (size_t)s->m * (s->n + 1);
    STZG_CUDA(cudaMemcpyAsync(s->F.src, src, nn * sizeof(double2), cudaMemcpyHostToDevice, s->st));
    STZG_CUDA(cudaMemcpyAsync(s->F.vel, vel, nn * sizeof(double2), cudaMemcpyHostToDevice, s->st));
    top_residual_sqnorm(s->h64, s->partials, s->npart, s->dnorm, s->dnorm + 1, s->st);
    STZG_CUDA(cudaMemcpyAsync(s->hnorm, s->dnorm, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    *err = s->hnorm[0] / (double)nn;
    return STZG_OK;
}

int stzg_mg_levels(stzg_sim *s, double dt, int *nlevels, int *dims) {
    if (!s || !nlevels || !(dt > 0)) return fail(STZG_EINVAL, "bad arguments");
    STZG_CHECK(ensure_ops(s, dt));
    *nlevels = (int)s->ops.size();
    if (dims)
        for (size_t l = 0; l < s->ops.size(); l++) {
            dims[2 * l] = s->ops[l].m;
            dims[2 * l + 1] = s->ops[l].n;
        }
    return STZG_OK;
}

int stzg_mg_stencil(stzg_sim *s, double dt, int level, double *out) {
    if (!s || !out || !(dt > 0)) return fail(STZG_EINVAL, "bad arguments");
    STZG_CHECK(ensure_ops(s, dt));
    if (level < 0 || level >= (int)s->ops.size()) return fail(STZG_EINVAL, "level out of range");
    const level_ops &L = s->ops[level];
    for (int j = 0; j < L.n; j++)
        for (int i = 0; i < L.m; i++) {
            int c = L.homog ? L.cls[j] : L.cls[(size_t)j * L.m + i];
            const stencil9<double> &t = L.table[c];
            double *o = out + 40 * ((size_t)j * L.m + i);
            for (int e = 0; e < 10; e++) {
                o[4 * e] = t.e[e].a;
                o[4 * e + 1] = t.e[e].b;
                o[4 * e + 2] = t.e[e].c;
                o[4 * e + 3] = t.e[e].d;
            }
        }
    return STZG_OK;
}

int stzg_l2_comparison(stzg_sim *a, stzg_sim *b, double *l2) {
    if (!a || !b || !l2) return fail(STZG_EINVAL, "null argument");
    if (a->m != b->m || a->n != b->n) return fail(STZG_EINVAL, "grids differ");
    const int m = a->m, n = a->n;
    const size_t nn = (size_t)m * (n + 1), nc = cell_count(a);
    std::vector<double> fa(nc), fb(nc);
    // shear_sim::l2_comparison, shear_sim.cc:460-502
    double c[4] = {0, 0, 0, 0};
    std::vector<double> ua(nn), ub(nn), va(nn), vb(nn), Xa(nn), Xb(nn), Ya(nn), Yb(nn);
    STZG_CHECK(stzg_get_field(a, STZG_U, ua.data()));
    STZG_CHECK(stzg_get_field(b, STZG_U, ub.data()));
    STZG_CHECK(stzg_get_field(a, STZG_V, va.data()));
    STZG_CHECK(stzg_get_field(b, STZG_V, vb.data()));
    STZG_CHECK(stzg_get_field(a, STZG_X, Xa.data()));
    STZG_CHECK(stzg_get_field(b, STZG_X, Xb.data()));
    STZG_CHECK(stzg_get_field(a, STZG_Y, Ya.data()));
    STZG_CHECK(stzg_get_field(b, STZG_Y, Yb.data()));
    std::vector<std::vector<double>> SA(5, std::vector<double>(nc)), SB(5, std::vector<double>(nc));
    const int ids[5] = {STZG_P, STZG_Q, STZG_S, STZG_TAU, STZG_CHI};
    for (int k = 0; k < 5; k++) {
        STZG_CHECK(stzg_get_field(a, ids[k], SA[k].data()));
        STZG_CHECK(stzg_get_field(b, ids[k], SB[k].data()));
    }
    for (int j = 0; j <= n; j++) {
        double c0 = 0, c3 = 0;
        for (int i = 0; i < m; i++) {
            size_t k = (size_t)j * m + i;
            double du = ua[k] - ub[k], dv = va[k] - vb[k], dX = Xa[k] - Xb[k], dY = Ya[k] - Yb[k];
            c0 += du * du + dv * dv;
            c3 += dX * dX + dY * dY;
        }
        double w = (j == 0 || j == n) ? 0.5 : 1.0;
        c[0] += w * c0;
        c[3] += w * c3;
    }
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            size_t k = (size_t)(j + 1) * m + i;
            double dp = SA[0][k] - SB[0][k], dq = SA[1][k] - SB[1][k], ds = SA[2][k] - SB[2][k],
                   dt = SA[3][k] - SB[3][k], dc = SA[4][k] - SB[4][k];
            c[1] += 2 * (dt * dt + ds * ds) + 3 * dp * dp + 6 * dq * dq;
            c[2] += dc * dc;
        }
    const double fac = ((a->P.bx - a->P.ax) / m) * ((a->P.by - a->P.ay) / n);
    for (int k = 0; k < 4; k++) l2[k] = c[k] * fac;
    return STZG_OK;
}

}  // extern "C"
