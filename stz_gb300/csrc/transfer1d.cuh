// One-dimensional transfer operators of the tgmg hierarchy, shared by the
// quasi-static multigrid (mg.cu) and the general scalar multigrid (tgmg.cu).
#pragma once

namespace stzg {

// 1D prolongation: coarse points (and weights) that feed fine index f of a
// line of um points (apply_t / t_line, tgmg.in.cc:552-621).
__host__ __device__ inline int p1d(int f, int um, int prd, int *c, double *w) {
    int sm = (um + (prd ? 1 : 2)) >> 1;
    if (!(f & 1)) { c[0] = f >> 1; w[0] = 1; return 1; }
    if (!prd && !(um & 1) && f == um - 1) { c[0] = sm - 1; w[0] = 1; return 1; }
    c[0] = f >> 1; w[0] = 0.5;
    c[1] = (prd && f == um - 1) ? 0 : (f >> 1) + 1; w[1] = 0.5;
    return 2;
}
// Weight of coarse index c at fine index f (0 when c does not feed f).
__host__ __device__ inline double pw(int f, int um, int prd, int c) {
    int cc[2]; double ww[2];
    int k = p1d(f, um, prd, cc, ww);
    double w = 0;
    for (int a = 0; a < k; a++) if (cc[a] == c) w += ww[a];
    return w;
}

// Integer form used by the kernels: halves (1 or 2) instead of weights, so
// that single-precision transfer kernels do no double-precision arithmetic.
__host__ __device__ inline int p1d_halves(int f, int um, int prd, int *c, int *h) {
    int sm = (um + (prd ? 1 : 2)) >> 1;
    if (!(f & 1)) { c[0] = f >> 1; h[0] = 2; return 1; }
    if (!prd && !(um & 1) && f == um - 1) { c[0] = sm - 1; h[0] = 2; return 1; }
    c[0] = f >> 1; h[0] = 1;
    c[1] = (prd && f == um - 1) ? 0 : (f >> 1) + 1; h[1] = 1;
    return 2;
}
__host__ __device__ inline int halves_of(int f, int um, int prd, int c) {
    int cc[2], hh[2];
    int k = p1d_halves(f, um, prd, cc, hh), w = 0;
    for (int a = 0; a < k; a++) if (cc[a] == c) w += hh[a];
    return w;
}

}  // namespace stzg
