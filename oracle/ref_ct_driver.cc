// Test-only C-ABI driver around the reference's coord_transforms variant of
// the simulation (esim/coord_transforms/simple_shear/shear_sim.{hh,cc}).
//
// Compiled by oracle/build_ref.sh together with that directory's
// shear_sim.cc, qs_multi.cc (which includes the generated tgmg.cc),
// common.cc, extra.cc, bi_interp.cc and esim/shared/mat.cc into
// oracle/_ref/libctref.so.  Only the tests and the golden-fixture script
// load it, to pin the GPU path (stz_gb300/csrc/ct.cu) against the
// reference's own step_forward_quasistatic (shear_sim.cc:352-360).  Fields
// are read and written in place (fm is public); set_boundaries is private,
// so this translation unit opens the private members.  It never changes the
// reference's arithmetic.
#include <cstring>
#include <vector>

#define private public
#include "shear_sim.hh"
#undef private

// Same member order as stzg_ct_params (include/stzg_ct.h).
struct ct_params {
    int m, n, y_prd, stz_model, t_model;
    double ax, bx, ay, by;
    double mu, K, viscosity, chi_len, t_scale, adapt_fac, u_bdry, lamb;
    double TZ, c0, tau0, kappa, Delta, Omegaeps0, chi_inf, theta, rho;
};

struct ct_handle {
    stz_dynamics *stz;
    shear_sim *sim;
};

static double *member(c_field &f, int id) {
    switch (id) {
        case 0: return &f.u;
        case 1: return &f.v;
        case 2: return &f.p;
        case 3: return &f.q;
        case 4: return &f.s;
        case 5: return &f.tau;
        case 6: return &f.chi;
        case 7: return &f.X;
        case 8: return &f.Y;
        default: return &f.ddev;
    }
}

extern "C" {

void *ctref_create(const ct_params *p) {
    ct_handle *h = new ct_handle;
    switch (p->stz_model) {
        case 0: h->stz = new stz_dynamics_linear(p->TZ, p->c0, p->tau0, p->kappa, p->Delta, p->Omegaeps0,
                                                 p->chi_inf, p->theta, p->rho); break;
        case 1: h->stz = new stz_dynamics_nonlinear(p->TZ, p->c0, p->tau0, p->kappa, p->Delta, p->Omegaeps0,
                                                    p->chi_inf, p->theta, p->rho); break;
        case 3: h->stz = new stz_dynamics_nonlinear_athermal(p->TZ, p->c0, p->tau0, p->kappa, p->Delta,
                                                             p->Omegaeps0, p->chi_inf, p->theta, p->rho); break;
        default: h->stz = new stz_dynamics_linear_athermal(p->TZ, p->c0, p->tau0, p->kappa, p->Delta,
                                                           p->Omegaeps0, p->chi_inf, p->theta, p->rho,
                                                           p->t_model); break;
    }
    h->sim = new shear_sim(p->m, p->n, p->ax, p->bx, p->ay, p->by, p->mu, p->K, p->viscosity, p->chi_len,
                           p->t_scale, p->adapt_fac, p->u_bdry, p->lamb, h->stz, p->y_prd != 0, 0, "");
    h->sim->qsm.mg.verbose = 0;
    return h;
}

void ctref_destroy(void *vh) {
    ct_handle *h = (ct_handle *)vh;
    delete h->sim;
    delete h->stz;
    delete h;
}

void ctref_init_fields(void *vh, int chi_case, double base, double delta) {
    ((ct_handle *)vh)->sim->init_fields(chi_case, base, delta);
}

// Rows 0..n of one field (m per row).
// shear_sim::initialize_chi_bicubic (shear_sim.cc:1067-1134), as it is.
void ctref_chi_bicubic(void *vh, int mm, int nn, const double *arr, double lo, double sca) {
    std::vector<double> a(arr, arr + (size_t)mm * nn);
    ((ct_handle *)vh)->sim->initialize_chi_bicubic(mm, nn, a.data(), lo, sca);
}

// shear_sim::write_files(k) (shear_sim.cc:892-931) into dir with the given
// output flags (both are constructor settings in the reference).
void ctref_write_files(void *vh, const char *dir, int k, unsigned fflags) {
    shear_sim &s = *((ct_handle *)vh)->sim;
    const_cast<unsigned int &>(s.fflags) = fflags;
    s.filename = dir;
    s.write_files(k);
}

// shear_sim::l2_comparison_transform (shear_sim.cc:619-711) of two reference runs.
void ctref_l2_comparison_transform(void *vt, void *vp, double *l2) {
    ((ct_handle *)vt)->sim->l2_comparison_transform(*((ct_handle *)vp)->sim, l2);
}

void ctref_get_field(void *vh, int id, double *out) {
    shear_sim &s = *((ct_handle *)vh)->sim;
    for (int j = 0; j <= s.n; j++)
        for (int i = 0; i < s.m; i++) out[j * s.m + i] = *member(s.fm[j * s.gm + i], id);
}

void ctref_set_field(void *vh, int id, const double *in) {
    shear_sim &s = *((ct_handle *)vh)->sim;
    for (int j = 0; j <= s.n; j++)
        for (int i = 0; i < s.m; i++) *member(s.fm[j * s.gm + i], id) = in[j * s.m + i];
    s.set_boundaries();
}

void ctref_steps(void *vh, double dt, int k) {
    shear_sim &s = *((ct_handle *)vh)->sim;
    for (int q = 0; q < k; q++) s.step_forward_quasistatic(dt);
}

void ctref_steps_direct(void *vh, double dt, int k) {
    shear_sim &s = *((ct_handle *)vh)->sim;
    for (int q = 0; q < k; q++) s.step_forward(dt);
}

double ctref_time(void *vh) { return ((ct_handle *)vh)->sim->time; }

void ctref_set_time(void *vh, double t) { ((ct_handle *)vh)->sim->time = t; }

int ctref_vcount(void *vh) { return ((ct_handle *)vh)->sim->qsm.tp.vcount; }

// Lagrangian tracers (shear_sim.cc:1247-1316).
void ctref_init_tracers(void *vh, int mm, int nn) { ((ct_handle *)vh)->sim->initialize_tracers(mm, nn); }

void ctref_update_tracers(void *vh) { ((ct_handle *)vh)->sim->update_tracers(); }

// Copies min(cap, ntrace) tracers (6 doubles each); returns ntrace.
int ctref_get_tracers(void *vh, double *out, int cap) {
    shear_sim &s = *((ct_handle *)vh)->sim;
    const int k = cap < s.ntrace ? cap : s.ntrace;
    if (out && k > 0) std::memcpy(out, s.tr, sizeof(double) * 6 * (size_t)k);
    return s.ntrace;
}

}  // extern "C"
