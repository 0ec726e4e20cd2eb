// Test-only C-ABI driver around the reference's general multigrid itself.
//
// Compiled by oracle/build_ref.sh together with the reference's
// esim/tgmg/poisson_fd.cc (which includes the tgmg.cc that
// esim/tgmg/tgmg_compile.pl generates and instantiates
// tgmg<poisson_fd,double,double>) into oracle/_ref/libtgmgref.so.  Only the
// tests and the golden-fixture script load it, to pin the CPU restatement
// (oracle/tgmg_oracle.py) and the GPU path (stz_gb300/csrc/tgmg.cu) against
// the reference's own hierarchy, Galerkin stencils and solves.  It never
// changes the reference's arithmetic.
#include <cstring>
#include <sys/time.h>

#include "poisson_fd.hh"
#include "tgmg.hh"
// The template definitions, so that the members this driver calls directly
// (l2_error -> mds) are instantiated here as well.
#include "tgmg.cc"

struct tg_handle {
    poisson_fd *q;
    tgmg<poisson_fd, double, double> *mg;
    tgmg_predict *tp;
};

static double wall_seconds() {
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

extern "C" {

void *tgref_create(int m, int n, double ax, double bx, double ay, double by) {
    tg_handle *h = new tg_handle;
    h->q = new poisson_fd(m, n, ax, bx, ay, by);
    h->mg = new tgmg<poisson_fd, double, double>(*h->q, h->q->b, h->q->z);
    h->mg->verbose = 0;
    h->mg->setup();
    h->mg->clear_z();
    for (int k = 0; k < m * n; k++) h->q->b[k] = 0;
    h->tp = new tgmg_predict;
    return h;
}

void tgref_destroy(void *p) {
    tg_handle *h = (tg_handle *)p;
    delete h->tp;
    delete h->mg;
    delete h->q;
    delete h;
}

double tgref_acc(void *p) { return ((tg_handle *)p)->q->acc; }

void tgref_set_b(void *p, const double *b) {
    tg_handle *h = (tg_handle *)p;
    std::memcpy(h->q->b, b, sizeof(double) * h->q->mn);
}
void tgref_get_b(void *p, double *b) {
    tg_handle *h = (tg_handle *)p;
    std::memcpy(b, h->q->b, sizeof(double) * h->q->mn);
}
void tgref_set_z(void *p, const double *z) {
    tg_handle *h = (tg_handle *)p;
    std::memcpy(h->q->z, z, sizeof(double) * h->q->mn);
}
void tgref_get_z(void *p, double *z) {
    tg_handle *h = (tg_handle *)p;
    std::memcpy(z, h->q->z, sizeof(double) * h->q->mn);
}

void tgref_gaussian(void *p, double gx, double gy, double r, double amp) {
    ((tg_handle *)p)->q->gaussian_source_term(gx, gy, r, amp);
}

// type 3 = full multigrid, 4 = V-cycle, 5 = symmetric V-cycle, with the
// handle's tgmg_predict; returns 1 on convergence and the cycles counted.
int tgref_solve(void *p, int type, int *iters, int *lim) {
    tg_handle *h = (tg_handle *)p;
    const int v0 = h->tp->vcount;
    bool ok = type == 3 ? h->mg->solve_full_multigrid(*h->tp)
                        : type == 5 ? h->mg->solve_sym_v_cycle(*h->tp) : h->mg->solve_v_cycle(*h->tp);
    if (iters) *iters = h->tp->vcount - v0;
    if (lim) *lim = h->tp->lim;
    return ok ? 1 : 0;
}

// solve_v_cycle() without a predictor (batches of 4 V-cycles).
int tgref_solve_fixed(void *p) { return ((tg_handle *)p)->mg->solve_v_cycle() ? 1 : 0; }

void tgref_vcycles(void *p, int count) {
    tg_handle *h = (tg_handle *)p;
    for (int k = 0; k < count; k++) h->mg->v_cycle();
}

double tgref_l2(void *p) { return ((tg_handle *)p)->mg->l2_error(); }

// Levels including the top; dims gets (m, n) per level.
int tgref_levels(void *p, int *dims) {
    tg_handle *h = (tg_handle *)p;
    dims[0] = h->q->m;
    dims[1] = h->q->n;
    for (int l = 0; l < h->mg->ml; l++) {
        dims[2 * l + 2] = h->mg->mg[l]->m;
        dims[2 * l + 3] = h->mg->mg[l]->n;
    }
    return h->mg->ml + 1;
}

// tgmg_level::s of coarse level `level` (1 = first child): 10 per point.
void tgref_stencil(void *p, int level, double *out) {
    tg_handle *h = (tg_handle *)p;
    tgmg_level<double, double> *L = h->mg->mg[level - 1];
    std::memcpy(out, L->s, sizeof(double) * 10 * L->mn);
}

// The pfd_time.cc loop (esim/tgmg/pfd_time.cc:30-60): trials solves of a
// Gaussian source rotated through one turn, each by solve_v_cycle with the
// handle's predictor; returns the wall seconds of the solves only and the
// V-cycle count.
double tgref_time_rotating(void *p, int trials, int *vcycles) {
    tg_handle *h = (tg_handle *)p;
    const double step = 2. * M_PI / trials;
    double t = 0;
    const int v0 = h->tp->vcount;
    for (int k = 0; k < trials; k++) {
        h->q->gaussian_source_term(6 * cos(step * k), 6 * sin(step * k), 1, 1);
        const double t0 = wall_seconds();
        h->mg->solve_v_cycle(*h->tp);
        t += wall_seconds() - t0;
    }
    if (vcycles) *vcycles = h->tp->vcount - v0;
    return t;
}

}  // extern "C"
