// stzg_tgmg.hh - C++ drop-in for the reference's general multigrid template
// tgmg<S,double,double> (esim/tgmg/tgmg.hh:286-495) and tgmg_predict
// (esim/tgmg/tgmg_predict.hh:6-33) on top of the C ABI in stzg_tgmg.h.
// Header-only; link with libstzg.so.
//
// S is a problem class with the reference's concept (poisson_fd.hh:7-61):
// members m, n, x_prd, y_prd, acc and the stencil functions a_dl, a_dc,
// a_dr, a_cl, a_cc, a_cr, a_ul, a_uc, a_ur taking (i, ij).  The constructor
// evaluates them at every grid point, keeps each distinct stencil once and
// builds the GPU hierarchy, so a reference problem class can be passed
// directly.  Like the reference, the solver works on the caller's b and z
// arrays: each solve copies them to the GPU and z back.  A solve that exceeds
// the predictor's threshold returns false as in the reference
// (tgmg.in.cc:282-287); other failures print the library message and exit
// with status 1, as tgmg_fatal_error does (tgmg.hh:29-32).
#ifndef STZG_TGMG_HH
#define STZG_TGMG_HH

#include <array>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <vector>

#include "stzg.h"
#include "stzg_tgmg.h"

namespace stzg {

inline void tgmg_check_or_exit(int st) {
    if (st != STZG_OK) {
        std::fprintf(stderr, "tgmg: %s: %s\n", stzg_strerror(st), stzg_last_message());
        std::exit(1);
    }
}

struct tgmg_predict : stzg_tgmg_predict {
    tgmg_predict() { stzg_tgmg_predict_init(this); }
    inline void add_iters(int k) {
        solves++;
        vcount += k;
    }
    inline float avg_iters() {
        float ans = static_cast<float>(vcount) / static_cast<float>(solves);
        solves = vcount = 0;
        return ans;
    }
};

template <class S> class tgmg {
  public:
    const int m, n, mn;
    int ml = 0;        // number of coarse levels
    int verbose = 1;   // accepted for source compatibility; the GPU solver prints nothing
    tgmg(S &q, double *b, double *z) : m(q.m), n(q.n), mn(q.m * q.n), q_(q), b_(b), z_(z) {
        std::map<std::array<double, 9>, int> index;
        std::vector<double> table;
        std::vector<int> cls(mn);
        for (int j = 0, ij = 0; j < n; j++)
            for (int i = 0; i < m; i++, ij++) {
                std::array<double, 9> s = {q.a_dl(i, ij), q.a_dc(i, ij), q.a_dr(i, ij), q.a_cl(i, ij), q.a_cc(i, ij),
                                           q.a_cr(i, ij), q.a_ul(i, ij), q.a_uc(i, ij), q.a_ur(i, ij)};
                auto it = index.find(s);
                if (it == index.end()) {
                    it = index.emplace(s, (int)index.size()).first;
                    table.insert(table.end(), s.begin(), s.end());
                }
                cls[ij] = it->second;
            }
        tgmg_check_or_exit(stzg_tgmg_create(m, n, q.x_prd ? 1 : 0, q.y_prd ? 1 : 0, table.data(),
                                            (int)index.size(), cls.data(), q.acc, 0, &h_));
        int nl = 0;
        tgmg_check_or_exit(stzg_tgmg_levels(h_, &nl, nullptr));
        ml = nl - 1;
    }
    ~tgmg() { stzg_tgmg_destroy(h_); }
    tgmg(const tgmg &) = delete;
    tgmg &operator=(const tgmg &) = delete;

    // tgmg::setup (tgmg.hh:331-335): the hierarchy is built by the constructor.
    void setup() {}
    // Not in the reference: V-cycle solves as FP32 V-cycles inside FP64
    // refinement (stzg_tgmg_set_precision), to the same acc.
    void set_mixed_precision(bool on) { tgmg_check_or_exit(stzg_tgmg_set_precision(h_, on ? 1 : 0)); }
    void clear_z() {
        for (int k = 0; k < mn; k++) z_[k] = 0;
    }

    bool solve_v_cycle(tgmg_predict &tp, int cyc_down = 1, int cyc_up = 1, int hcyc_bottom = 10) {
        return solve(STZG_TGMG_VCYCLE, &tp, 1, cyc_down, cyc_up, hcyc_bottom);
    }
    bool solve_v_cycle(int cyc_down = 1, int cyc_up = 1, int hcyc_bottom = 10) {
        return solve_fixed(STZG_TGMG_VCYCLE, 4, 1000, 1, cyc_down, cyc_up, hcyc_bottom);
    }
    bool solve_sym_v_cycle(tgmg_predict &tp, int cyc_down = 1, int cyc_up = 1, int hcyc_bottom = 10) {
        return solve(STZG_TGMG_SYM_VCYCLE, &tp, 1, cyc_down, cyc_up, hcyc_bottom);
    }
    bool solve_full_multigrid(tgmg_predict &tp, int cyc_down = 1, int cyc_up = 1, int hcyc_bottom = 10) {
        return solve(STZG_TGMG_FMG, &tp, 1, cyc_down, cyc_up, hcyc_bottom);
    }
    bool solve_full_multigrid(int cyc_down = 1, int cyc_up = 1, int hcyc_bottom = 10) {
        return solve_fixed(STZG_TGMG_FMG, 2, 1000, 1, cyc_down, cyc_up, hcyc_bottom);
    }
    bool solve_jacobi() { return solve_fixed(STZG_TGMG_JACOBI, 100, 400, 1, 1, 1, 10); }
    bool solve_jacobi(tgmg_predict &tp) { return solve(STZG_TGMG_JACOBI, &tp, 1, 1, 1, 10); }
    bool solve_gauss_seidel() { return solve_fixed(STZG_TGMG_GS, 20, 2000, 1, 1, 1, 10); }
    bool solve_gauss_seidel(tgmg_predict &tp) { return solve(STZG_TGMG_GS, &tp, 1, 1, 1, 10); }
    bool solve_sor(double omega) { return solve_fixed(STZG_TGMG_SOR, 20, 1000, omega, 1, 1, 10); }
    bool solve_sor(tgmg_predict &tp, double omega) { return solve(STZG_TGMG_SOR, &tp, omega, 1, 1, 10); }

    // Not in the reference: V-cycles until l2_error < acc, tested before the
    // first and after each (stzg_tgmg_solve_checked), then extra_iters more.
    bool solve_v_cycle_checked(int max_iters = 2048, int extra_iters = 1, int cyc_down = 1, int cyc_up = 1,
                               int hcyc_bottom = 10) {
        push();
        return finish(stzg_tgmg_solve_checked(h_, STZG_TGMG_VCYCLE, max_iters, extra_iters, 1, cyc_down, cyc_up,
                                              hcyc_bottom, nullptr, nullptr));
    }

    void v_cycle(int cyc_down = 1, int cyc_up = 1, int hcyc_bottom = 10, bool symmetric = false) {
        iterate(symmetric ? STZG_TGMG_SYM_VCYCLE : STZG_TGMG_VCYCLE, 1, 1, cyc_down, cyc_up, hcyc_bottom);
    }
    void jacobi() { iterate(STZG_TGMG_JACOBI, 1, 1, 1, 1, 10); }
    void gauss_seidel() { iterate(STZG_TGMG_GS, 1, 1, 1, 1, 10); }
    void sor(double omega) { iterate(STZG_TGMG_SOR, 1, omega, 1, 1, 10); }

    // l2_error = mds()/mn (tgmg.hh:146)
    double l2_error() {
        push();
        double e = 0;
        tgmg_check_or_exit(stzg_tgmg_l2_error(h_, &e));
        return e;
    }

  private:
    S &q_;
    double *b_, *z_;
    stzg_tgmg *h_ = nullptr;

    void push() {
        tgmg_check_or_exit(stzg_tgmg_set_b(h_, b_));
        tgmg_check_or_exit(stzg_tgmg_set_z(h_, z_));
    }
    void pull() { tgmg_check_or_exit(stzg_tgmg_get_z(h_, z_)); }
    bool finish(int st) {
        pull();
        if (st == STZG_ENOTCONV) return false;
        tgmg_check_or_exit(st);
        return true;
    }
    bool solve(int type, tgmg_predict *tp, double omega, int cd, int cu, int hb) {
        push();
        return finish(stzg_tgmg_solve(h_, type, tp, omega, cd, cu, hb, nullptr, nullptr));
    }
    bool solve_fixed(int type, int per_loop, int max_loops, double omega, int cd, int cu, int hb) {
        push();
        return finish(stzg_tgmg_solve_fixed(h_, type, per_loop, max_loops, omega, cd, cu, hb, nullptr, nullptr));
    }
    void iterate(int type, int count, double omega, int cd, int cu, int hb) {
        push();
        tgmg_check_or_exit(stzg_tgmg_iterate(h_, type, count, omega, cd, cu, hb));
        pull();
    }
};

}  // namespace stzg

#endif  // STZG_TGMG_HH
