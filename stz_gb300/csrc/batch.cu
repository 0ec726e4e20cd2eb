// Many independent simulations in one CUDA graph.
//
// Every instance keeps its own handle (fields, multigrid hierarchies) and the
// batch builds one root graph holding, per instance, a WHILE node over time
// steps.  A step body is the single-simulation step with the time-dependent
// quantities (time, wall speed and position, state buffer index) read from a
// device clock, and a nested WHILE node over multigrid passes: FP64, one
// V-cycle then the residual norm; mixed, one refinement pass (FP32 V-cycles,
// FP64 correction and residual).  A one-thread check kernel decides, with the
// same stopping rule as the host path, whether the solve loop goes on (and
// stops it at an iteration cap with an error flag, so no loop is unbounded);
// another decides whether the step loop goes on.  The instances are
// independent branches of the root graph, so the small ones run concurrently.
//
// The schedule knobs of each instance (FP32 V-cycles per refinement pass,
// tail size, fused tile kernels) come from a table keyed by grid size that
// stzg_batch_autotune fills by timing the candidates on the GPU.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "sim.cuh"

namespace stzg {
namespace {

enum { CTR_STEP = 0, CTR_ITERS, CTR_CYCLES, CTR_ERR, CTR_PASSES, CTR_COUNT };

struct tuning {
    int inner;        // FP32 V-cycles per refinement pass
    long tail_limit;  // largest level in the single-block tail
    int fuse;         // fused tile kernels on wide FP32 levels
};

__global__ void k_step_begin(double *clk, double dt, double u_bdry) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double t = clk[CLK_TIME] + dt;  // shear_sim.cc:283
        clk[CLK_TIME] = t;
        clk[CLK_BV] = t < 1 ? t * u_bdry : u_bdry;                               // bdry_vel
        clk[CLK_BP] = t < 1 ? u_bdry * t * t * 0.5 : u_bdry * (t - 0.5);         // bdry_pos
    }
}

__global__ void k_solve_reset(int *ctr, cudaGraphConditionalHandle h) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        ctr[CTR_ITERS] = 0;
        cudaGraphSetConditional(h, 1u);
    }
}

// Stopping rule of the solve loop: reference rule (mean squared residual
// below acc) or relative 2-norm; the loop also stops at `cap` passes.
__global__ void k_solve_check(const double *dnorm, int *ctr, int cycles_per_pass, int relative, double tol2,
                              double acc, double inv_nodes, int cap, cudaGraphConditionalHandle h) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double r2 = dnorm[0], b2 = dnorm[1];
        const int it = ++ctr[CTR_ITERS];
        ctr[CTR_CYCLES] += cycles_per_pass;
        ctr[CTR_PASSES] += 1;
        const bool conv = relative ? (r2 <= tol2 * b2) : (r2 * inv_nodes < acc);
        const bool bad = isnan(r2) || (!conv && it >= cap);
        if (bad) ctr[CTR_ERR] = 1;
        cudaGraphSetConditional(h, (!conv && !bad) ? 1u : 0u);
    }
}

__global__ void k_step_end(double *clk, int *ctr, int nsteps, cudaGraphConditionalHandle h) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        clk[CLK_BV_STATE] = clk[CLK_BV];
        clk[CLK_CUR] = (double)((int)clk[CLK_CUR] ^ 1);
        const int s = ++ctr[CTR_STEP];
        cudaGraphSetConditional(h, (s < nsteps && !ctr[CTR_ERR]) ? 1u : 0u);
    }
}

}  // namespace
}  // namespace stzg

using namespace stzg;

struct stzg_batch {
    std::vector<stzg_sim *> sims;
    stzg_options O;
    cudaStream_t st = nullptr;
    double *dclock = nullptr;  // CLK_COUNT per instance
    int *dctr = nullptr;       // CTR_COUNT per instance
    cudaGraphExec_t exec = nullptr;
    double g_dt = -1;
    int g_nsteps = -1;
    long nodes = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::map<std::pair<int, int>, tuning> table;  // (m, n) -> knobs
    int cap = 400;
    std::vector<long> step_kernels, pass_kernels;  // kernels per step body / per solve pass
};

namespace {

tuning default_tuning(const stzg_batch *b) {
    tuning t;
    t.inner = b->O.inner_cycles > 0 ? b->O.inner_cycles : 3;
    t.tail_limit = -1;
    t.fuse = 1;
    return t;
}

tuning tuning_for(const stzg_batch *b, const stzg_sim *s) {
    auto it = b->table.find(std::make_pair(s->m, s->n));
    return it == b->table.end() ? default_tuning(b) : it->second;
}

void drop_batch_graph(stzg_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->g_dt = -1;
    b->g_nsteps = -1;
}

// Appends instance k's step loop to the root graph.
int add_instance(stzg_batch *b, cudaGraph_t root, int k, double dt, int nsteps, long *kernels) {
    stzg_sim *s = b->sims[k];
    STZG_CHECK(ensure_ops(s, dt));
    const tuning tn = tuning_for(b, s);
    const bool mixed = s->O.precision == STZG_MIXED;
    if (s->h64.tail_limit != tn.tail_limit || s->h64.fuse != tn.fuse || s->h32.tail_limit != tn.tail_limit ||
        s->h32.fuse != tn.fuse || s->h32.persist)
        drop_graphs(s);  // the handle's own captured cycles used other knobs
    // the instances' V-cycles run side by side: no cooperative whole-GPU kernel
    s->h32.persist = 0;
    s->h64.tail_limit = tn.tail_limit;
    s->h64.fuse = tn.fuse;
    s->h32.tail_limit = tn.tail_limit;
    s->h32.fuse = tn.fuse;
    double *clk = b->dclock + (size_t)k * CLK_COUNT;
    int *ctr = b->dctr + (size_t)k * CTR_COUNT;
    // the captured step kernels read time, wall data and buffer index from the clock
    step_consts sc = s->sc;
    sc.clock = clk;
    sc.xbc = s->q.bcs * s->q.cxx;
    const long count = (long)s->m * (s->n + 1);

    cudaGraphConditionalHandle hstep;
    STZG_CUDA(cudaGraphConditionalHandleCreate(&hstep, root, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hstep;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    STZG_CUDA(cudaGraphAddNode(&wnode, root, nullptr, nullptr, 0, &wp));
    cudaGraph_t body = wp.conditional.phGraph_out[0];

    cudaGraphConditionalHandle hsolve;
    STZG_CUDA(cudaGraphConditionalHandleCreate(&hsolve, body, 1, 0));

    // step body: clock, advection, source, guess, initial residual | solve loop | projection, end
    const long c0 = launch_count();
    STZG_CUDA(cudaStreamBeginCaptureToGraph(s->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    k_step_begin<<<1, 32, 0, s->st>>>(clk, dt, s->P.u_bdry);
    note_launch();
    advection(sc, *s->maps, s->F, 0, dt, 0.0, s->st);
    projection_source(sc, s->F, 0, dt, 0.0, s->st);
    if (s->O.extrapolate) extrapolate_guess(s->F.vel, s->vel_prev, count, s->st);
    if (mixed) {
        mixed_begin(s);
        launch_norms(s, true);
    }
    k_solve_reset<<<1, 32, 0, s->st>>>(ctr, hsolve);
    note_launch();
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    STZG_CUDA(cudaStreamGetCaptureInfo(s->st, &cs, nullptr, &cg, &deps, nullptr, &ndeps));
    cudaGraphNodeParams sp = {};
    sp.type = cudaGraphNodeTypeConditional;
    sp.conditional.handle = hsolve;
    sp.conditional.type = cudaGraphCondTypeWhile;
    sp.conditional.size = 1;
    cudaGraphNode_t snode;
    STZG_CUDA(cudaGraphAddNode(&snode, cg, deps, nullptr, ndeps, &sp));
    STZG_CUDA(cudaStreamUpdateCaptureDependencies(s->st, &snode, nullptr, 1, cudaStreamSetCaptureDependencies));
    if (mixed) mixed_end(s);
    projection_apply(sc, s->F, 0, dt, 0.0, 0.0, s->st);
    k_step_end<<<1, 32, 0, s->st>>>(clk, ctr, nsteps, hstep);
    note_launch();
    cudaGraph_t got = nullptr;
    STZG_CUDA(cudaStreamEndCapture(s->st, &got));
    const long c1 = launch_count();

    // solve-loop body
    cudaGraph_t sbody = sp.conditional.phGraph_out[0];
    STZG_CUDA(cudaStreamBeginCaptureToGraph(s->st, sbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int per_pass = 1;
    if (mixed) {
        per_pass = tn.inner;
        for (int c = 0; c < tn.inner; c++) vcycle<float>(s->h32, s->st, 10, 1, c == 0);
        ff_correct(s->zhi, s->zlo, s->h32.lv[0].z, count, s->st);
        launch_norms(s, true);
    } else {
        vcycle<double>(s->h64, s->st, 10, 1);
        launch_norms(s, false);
    }
    const int relative = s->O.tol_mode == STZG_TOL_RELATIVE;
    k_solve_check<<<1, 32, 0, s->st>>>(s->dnorm, ctr, per_pass, relative, s->O.tol * s->O.tol,
                                        s->q.reference_acc(s->O.tol), 1.0 / (double)count, b->cap, hsolve);
    note_launch();
    STZG_CUDA(cudaStreamEndCapture(s->st, &got));
    const long c2 = launch_count();
    b->step_kernels[k] = c1 - c0;
    b->pass_kernels[k] = c2 - c1;
    discount_launches(c2 - c0);  // graph nodes, counted when they execute
    *kernels += c2 - c0;
    return STZG_OK;
}

int build_graph(stzg_batch *b, double dt, int nsteps) {
    if (b->exec && b->g_dt == dt && b->g_nsteps == nsteps) return STZG_OK;
    drop_batch_graph(b);
    cudaGraph_t root;
    STZG_CUDA(cudaGraphCreate(&root, 0));
    long kernels = 0;
    int st = STZG_OK;
    b->step_kernels.assign(b->sims.size(), 0);
    b->pass_kernels.assign(b->sims.size(), 0);
    for (size_t k = 0; k < b->sims.size() && st == STZG_OK; k++) st = add_instance(b, root, (int)k, dt, nsteps, &kernels);
    if (st == STZG_OK) {
        cudaError_t e = cudaGraphInstantiate(&b->exec, root, 0);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaGraphInstantiate(batch)");
    }
    cudaGraphDestroy(root);
    if (st != STZG_OK) {
        b->exec = nullptr;
        return st;
    }
    b->g_dt = dt;
    b->g_nsteps = nsteps;
    b->nodes = kernels;
    return STZG_OK;
}

}  // namespace

extern "C" {

int stzg_batch_create(int count, const stz_params *params, const stzg_options *opt, stzg_batch **out) {
    if (!out || count < 1 || !params) return fail(STZG_EINVAL, "bad batch arguments");
    *out = nullptr;
    stzg_batch *b = new stzg_batch;
    if (opt) b->O = *opt;
    else stzg_default_options(&b->O);
    b->O.use_graphs = 1;
    int st = STZG_OK;
    for (int k = 0; k < count && st == STZG_OK; k++) {
        stzg_sim *s = nullptr;
        stzg_options o = b->O;
        st = stzg_create(&params[k], &o, &s);
        if (st == STZG_OK) b->sims.push_back(s);
    }
    if (st == STZG_OK && cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess)
        st = fail(STZG_ECUDA, "stream creation failed");
    if (st == STZG_OK && cudaMalloc(&b->dclock, sizeof(double) * CLK_COUNT * count) != cudaSuccess)
        st = fail(STZG_ENOMEM, "batch clock allocation failed");
    if (st == STZG_OK && cudaMalloc(&b->dctr, sizeof(int) * CTR_COUNT * count) != cudaSuccess)
        st = fail(STZG_ENOMEM, "batch counter allocation failed");
    if (st == STZG_OK) {
        cudaEventCreate(&b->e0);
        cudaEventCreate(&b->e1);
    }
    if (st != STZG_OK) {
        stzg_batch_destroy(b);
        return st;
    }
    *out = b;
    return STZG_OK;
}

int stzg_batch_destroy(stzg_batch *b) {
    if (!b) return STZG_OK;
    if (b->st) cudaStreamSynchronize(b->st);
    drop_batch_graph(b);
    for (stzg_sim *s : b->sims) stzg_destroy(s);
    if (b->dclock) cudaFree(b->dclock);
    if (b->dctr) cudaFree(b->dctr);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return STZG_OK;
}

int stzg_batch_size(stzg_batch *b, int *count) {
    if (!b || !count) return fail(STZG_EINVAL, "null argument");
    *count = (int)b->sims.size();
    return STZG_OK;
}

int stzg_batch_sim(stzg_batch *b, int k, stzg_sim **s) {
    if (!b || !s || k < 0 || k >= (int)b->sims.size()) return fail(STZG_EINVAL, "instance index out of range");
    *s = b->sims[k];
    return STZG_OK;
}

int stzg_batch_set_tuning(stzg_batch *b, int m, int n, int inner, long tail_limit, int fuse) {
    if (!b || inner < 1) return fail(STZG_EINVAL, "bad tuning");
    tuning t{inner, tail_limit, fuse};
    b->table[std::make_pair(m, n)] = t;
    drop_batch_graph(b);
    return STZG_OK;
}

int stzg_batch_autotune(stzg_batch *b, double dt, int steps) {
    if (!b || !(dt > 0) || steps < 1) return fail(STZG_EINVAL, "bad autotune arguments");
    std::map<std::pair<int, int>, int> first;
    for (size_t k = 0; k < b->sims.size(); k++) first.emplace(std::make_pair(b->sims[k]->m, b->sims[k]->n), (int)k);
    const bool mixed = b->O.precision == STZG_MIXED;
    std::vector<int> inners = mixed ? std::vector<int>{2, 3, 4} : std::vector<int>{1};
    std::vector<long> tails = mixed ? std::vector<long>{-1, 1100, 300} : std::vector<long>{-1, 72, 1100};
    std::vector<int> fuses = mixed ? std::vector<int>{1, 0} : std::vector<int>{1};
    for (auto &kv : first) {
        const stz_params P = b->sims[kv.second]->P;
        std::vector<double> chi((size_t)P.m * P.n, 600.0 / P.TZ);
        double best = 1e300;
        tuning pick = default_tuning(b);
        for (int in : inners)
            for (long tl : tails)
                for (int fu : fuses) {
                    stzg_batch *t = nullptr;
                    if (stzg_batch_create(1, &P, &b->O, &t) != STZG_OK) continue;
                    stzg_batch_stats st;
                    int ok = stzg_set_state(t->sims[0], chi.data()) == STZG_OK &&
                             stzg_batch_set_tuning(t, P.m, P.n, in, tl, fu) == STZG_OK &&
                             stzg_batch_run(t, dt, steps, &st) == STZG_OK;
                    stzg_batch_destroy(t);
                    if (ok && st.seconds < best) {
                        best = st.seconds;
                        pick = tuning{in, tl, fu};
                    }
                }
        b->table[kv.first] = pick;
    }
    drop_batch_graph(b);
    return STZG_OK;
}

int stzg_batch_get_tuning(stzg_batch *b, int m, int n, int *inner, long *tail_limit, int *fuse) {
    if (!b || !inner || !tail_limit || !fuse) return fail(STZG_EINVAL, "null argument");
    auto it = b->table.find(std::make_pair(m, n));
    tuning t = it == b->table.end() ? default_tuning(b) : it->second;
    *inner = t.inner;
    *tail_limit = t.tail_limit;
    *fuse = t.fuse;
    return STZG_OK;
}

int stzg_batch_run(stzg_batch *b, double dt, int nsteps, stzg_batch_stats *stats) {
    if (!b || !(dt > 0) || nsteps < 0) return fail(STZG_EINVAL, "bad batch run arguments");
    if (nsteps == 0) return STZG_OK;
    const int count = (int)b->sims.size();
    // initial clock and counters from the handles
    std::vector<double> clk((size_t)CLK_COUNT * count, 0.0);
    for (int k = 0; k < count; k++) {
        stzg_sim *s = b->sims[k];
        clk[(size_t)k * CLK_COUNT + CLK_TIME] = s->time;
        clk[(size_t)k * CLK_COUNT + CLK_BV_STATE] = s->bv_state;
        clk[(size_t)k * CLK_COUNT + CLK_CUR] = s->cur;
        if (s->O.extrapolate && !s->have_prev) {
            STZG_CUDA(cudaMemcpyAsync(s->vel_prev, s->F.vel, sizeof(double2) * (size_t)s->m * (s->n + 1),
                                      cudaMemcpyDeviceToDevice, s->st));
            s->have_prev = true;
        }
        STZG_CUDA(cudaStreamSynchronize(s->st));
    }
    STZG_CHECK(build_graph(b, dt, nsteps));
    STZG_CUDA(cudaMemcpyAsync(b->dclock, clk.data(), sizeof(double) * clk.size(), cudaMemcpyHostToDevice, b->st));
    STZG_CUDA(cudaMemsetAsync(b->dctr, 0, sizeof(int) * CTR_COUNT * count, b->st));
    STZG_CUDA(cudaEventRecord(b->e0, b->st));
    STZG_CUDA(cudaGraphLaunch(b->exec, b->st));
    STZG_CUDA(cudaEventRecord(b->e1, b->st));
    STZG_CUDA(cudaEventSynchronize(b->e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, b->e0, b->e1);
    std::vector<int> ctr((size_t)CTR_COUNT * count);
    STZG_CUDA(cudaMemcpy(ctr.data(), b->dctr, sizeof(int) * ctr.size(), cudaMemcpyDeviceToHost));
    STZG_CUDA(cudaMemcpy(clk.data(), b->dclock, sizeof(double) * clk.size(), cudaMemcpyDeviceToHost));
    long cycles = 0, passes = 0, failed = 0, steps_done = 0, cells = 0, executed = 0;
    for (int k = 0; k < count; k++) {
        stzg_sim *s = b->sims[k];
        const int *c = &ctr[(size_t)k * CTR_COUNT];
        executed += b->step_kernels[k] * c[CTR_STEP] + b->pass_kernels[k] * c[CTR_PASSES];
        s->time = clk[(size_t)k * CLK_COUNT + CLK_TIME];
        s->bv_state = clk[(size_t)k * CLK_COUNT + CLK_BV_STATE];
        s->cur = (int)clk[(size_t)k * CLK_COUNT + CLK_CUR];
        cycles += c[CTR_CYCLES];
        passes += c[CTR_PASSES];
        steps_done += c[CTR_STEP];
        cells += (long)s->m * s->n * c[CTR_STEP];
        if (c[CTR_ERR]) failed++;
        s->acc.vcycles += c[CTR_CYCLES];
        s->acc.solves += c[CTR_STEP];
    }
    long flag_err = 0;
    for (int k = 0; k < count; k++)
        if (check_flags(b->sims[k]) != STZG_OK) flag_err++;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->instances = count;
        stats->steps = steps_done;
        stats->cell_steps = cells;
        stats->vcycles = cycles;
        stats->passes = passes;
        stats->failed = failed;
        stats->seconds = ms * 1e-3;
        stats->graph_kernels = b->nodes;
        stats->kernel_launches = executed;
    }
    for (long e = 0; e < executed; e++) note_launch();
    if (failed) return fail(STZG_ENOTCONV, "a batch instance did not converge within the pass cap");
    if (flag_err) return fail(STZG_ESUBSTEP, "a batch instance reached the plastic sub-step cap");
    return STZG_OK;
}

}  // extern "C"
