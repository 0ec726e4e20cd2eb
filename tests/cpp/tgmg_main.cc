// Drives the C++ multigrid drop-in (include/stzg_tgmg.hh) the way the
// reference's test programs drive tgmg<poisson_fd,double,double>
// (esim/tgmg/pfd_test.cc:6-20): a problem class with the reference's concept,
// tgmg(q, q.b, q.z), setup(), solve_v_cycle(tgmg_predict&).
// Usage: tgmg_main <m> <n> <ax> <bx> <ay> <by> <b.bin> <z.bin>
// Reads b (m*n doubles), writes z, prints the V-cycle count and l2_error.
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "stzg_tgmg.hh"

// A 5-point Laplacian with Dirichlet edges, the stencil concept of
// poisson_fd.hh:7-61 written out for this test.
struct dirichlet_laplacian {
    const int m, n, mn;
    static const bool x_prd = false, y_prd = false;
    const double dx, dy, hcc, hxx, hyy, acc;
    std::vector<double> bv, zv;
    double *b, *z;
    dirichlet_laplacian(int m_, int n_, double ax, double bx, double ay, double by)
        : m(m_), n(n_), mn(m_ * n_), dx((bx - ax) / (m_ - 1)), dy((by - ay) / (n_ - 1)),
          hcc(-2 / (dx * dx) - 2 / (dy * dy)), hxx(1. / (dx * dx)), hyy(1. / (dy * dy)),
          acc((DBL_EPSILON * 1e4 * hcc) * (DBL_EPSILON * 1e4 * hcc)), bv(mn, 0.0), zv(mn, 0.0),
          b(bv.data()), z(zv.data()) {}
    bool edge(int i, int ij) const { return i == 0 || i == m - 1 || ij < m || ij >= mn - m; }
    double a_dl(int, int) const { return 0; }
    double a_dr(int, int) const { return 0; }
    double a_ul(int, int) const { return 0; }
    double a_ur(int, int) const { return 0; }
    double a_dc(int i, int ij) const { return edge(i, ij) ? 0 : hyy; }
    double a_uc(int i, int ij) const { return edge(i, ij) ? 0 : hyy; }
    double a_cl(int i, int ij) const { return edge(i, ij) ? 0 : hxx; }
    double a_cr(int i, int ij) const { return edge(i, ij) ? 0 : hxx; }
    double a_cc(int, int) const { return hcc; }
};

int main(int argc, char **argv) {
    if (argc < 9) return 2;
    const int m = std::atoi(argv[1]), n = std::atoi(argv[2]);
    dirichlet_laplacian q(m, n, std::atof(argv[3]), std::atof(argv[4]), std::atof(argv[5]), std::atof(argv[6]));
    std::FILE *f = std::fopen(argv[7], "rb");
    if (!f || std::fread(q.b, sizeof(double), q.mn, f) != (size_t)q.mn) return 3;
    std::fclose(f);
    stzg::tgmg<dirichlet_laplacian> mg(q, q.b, q.z);
    mg.verbose = 0;
    mg.setup();
    mg.clear_z();
    stzg::tgmg_predict tp;
    if (!mg.solve_v_cycle(tp)) return 4;
    f = std::fopen(argv[8], "wb");
    std::fwrite(q.z, sizeof(double), q.mn, f);
    std::fclose(f);
    std::printf("levels %d vcycles %d l2 %.3e acc %.3e\n", mg.ml + 1, tp.vcount, mg.l2_error(), q.acc);
    return 0;
}
