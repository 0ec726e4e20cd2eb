// Quasi-static STZ step in sheared coordinates (include/stzg_ct.h): the
// coord_transforms variant of the simulation
// (esim/coord_transforms/simple_shear/shear_sim.cc:352-546, fields.hh,
// qs_multi.{hh,cc}) on one GPU.
//
// Layout: each field of the reference's c_field (u, v, p, q, s, tau, chi, X,
// Y) is an FP64 array of (m+4) x (n+4) points with the reference's two ghost
// layers, index (j+2)*(m+4) + (i+2), in two buffers: the advection kernel
// reads buffer cur and writes buffer cur^1.  ddev is one array of the same
// shape whose ghost points stay zero (the reference never writes them).  The
// projection solves with the 2x2-block multigrid of tgmg.cu on m x lsn nodes
// (lsn = n rows when y is periodic, n+1 with walls), its operator rebuilt
// every step for the new shear lt = lamb*time as qs_multi::init does
// (qs_multi.cc:31-46); source and velocities stay on the GPU.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "step.cuh"
#include "stz_law.cuh"
#include "stzg_ct.h"
#include "stzg_tgmg.h"

namespace stzg {
namespace {

enum { CU = 0, CV, CP, CQ, CS, CTAU, CCHI, CX, CY, CF };

struct ct_consts {
    int m, n, gm, yp, lsn;
    double ax, ay, bx, by, lx, ly, dx, dy, xsp, ysp;
    double mu, mu_inv, K, chi_len, lamb, u_bdry;
    stz_law_params<double> law;
};

struct ct_fields {
    double *f[2][CF];
    double *ddev;
};

__device__ __forceinline__ size_t gidx(const ct_consts &c, int i, int j) { return (size_t)(j + 2) * c.gm + (i + 2); }

// shear_sim::eno2 (shear_sim.cc:886-888)
__device__ __forceinline__ double eno2_ct(double p0, double p1, double p2, double p3) {
    return fabs(p0 - 2 * p1 + p2) > fabs(p1 - 2 * p2 + p3) ? 3 * p1 - 4 * p2 + p3 : p0 - p2;
}

// hs * eno2 along step d from point k (rm_eno2 / st_eno2, shear_sim.cc:864-884)
__device__ __forceinline__ double eno_d(const double *f, size_t k, long d, double hs) {
    return hs * eno2_ct(f[k - d], f[k], f[k + d], f[k + 2 * d]);
}

// Advection and plasticity per cell (i,j) and its lower-left node
// (shear_sim::advection_step, shear_sim.cc:365-417); the new values go to
// buffer cur^1 (chi without its diffusion).
__global__ void k_ct_advect(ct_consts c, ct_fields F, int cur, double dt, double time) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= c.m || j >= c.n) return;
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt;
    const double third = 1. / 3., lt = c.lamb * time, ltsq = lt * lt;
    const double *const *A = F.f[cur];
    double *const *B = F.f[cur ^ 1];
    const size_t k = gidx(c, i, j);
    const long gm = c.gm;
    const double *U = A[CU], *V = A[CV];
    B[CU][k] = U[k];
    B[CV][k] = V[k];
    // reference map at the node
    if (j > 0 || c.yp) {
        const double uc = U[k], vc = V[k];
        double Xx, Yx, Xy, Yy;
        if (uc > 0) {
            Xx = eno_d(A[CX], k, -1, hx);
            Yx = eno_d(A[CY], k, -1, hx);
        } else {
            Xx = eno_d(A[CX], k, 1, -hx);
            Yx = eno_d(A[CY], k, 1, -hx);
        }
        if (vc > 0) {
            Xy = eno_d(A[CX], k, -gm, hy);
            Yy = eno_d(A[CY], k, -gm, hy);
        } else {
            Xy = eno_d(A[CX], k, gm, -hy);
            Yy = eno_d(A[CY], k, gm, -hy);
        }
        const double cX = -uc * Xx - vc * Xy, cY = -uc * Yx - vc * Yy;
        B[CX][k] = A[CX][k] + cX;
        B[CY][k] = A[CY][k] + cY;
    } else {
        B[CX][k] = A[CX][k];
        B[CY][k] = A[CY][k];
    }
    // deformation rate, staggered velocity and spin
    const double u0 = U[k], ur = U[k + 1], uu = U[k + gm], uru = U[k + gm + 1];
    const double v0 = V[k], vr = V[k + 1], vu = V[k + gm], vru = V[k + gm + 1];
    const double uc = 0.25 * (u0 + ur + uu + uru), vc = 0.25 * (v0 + vr + vu + vru);
    const double ux = hx * (-u0 + ur - uu + uru), uy = hy * (-u0 - ur + uu + uru);
    const double vx = hx * (-v0 + vr - vu + vru), vy = hy * (-v0 - vr + vu + vru);
    const double p = A[CP][k], q = A[CQ][k], s = A[CS][k], tau = A[CTAU][k], chi = A[CCHI][k];
    // calc_p (shear_sim.hh:182-184)
    const double old_p = p + (1. / 3) * c.lamb * time * (-2 * tau + c.lamb * time * (p + q + s));
    const long dx1 = uc > 0 ? -1 : 1, dy1 = vc > 0 ? -gm : gm;
    const double hsx = uc > 0 ? hx : -hx, hsy = vc > 0 ? hy : -hy;
    double f1[5], f2[5];
#pragma unroll
    for (int f = 0; f < 5; f++) {
        f1[f] = eno_d(A[CP + f], k, dx1, hsx);
        f2[f] = eno_d(A[CP + f], k, dy1, hsy);
    }
    // adaptive_plastic_term (shear_sim.cc:739-776) of the deviatoric norm in
    // the untransformed frame (c_field::devsq, fields.hh:108-141)
    const double pqs = p + q + s;
    const double unt_tau = tau - lt * pqs;
    const double unt_q = q + lt * (1 / 3.) * (-tau + lt * .5 * pqs);
    const double unt_s = s + lt * (tau - lt * .5 * pqs);
    const double sbar = sqrt(3 * unt_q * unt_q + unt_s * unt_s + unt_tau * unt_tau);
    double cchi = chi, dtmp = 0;
    if (sbar >= 1e-12) {  // below it the reference returns 0 and keeps the previous ddev
        const bool athermal = c.law.stz_model >= 2;
        if (athermal && sbar < c.law.s_y) {
            F.ddev[k] = 0;  // exactly what the sub-stepping gives below yield
        } else {
            double ddev;
            int iters;
            dtmp = adaptive_plastic(c.law, sbar, cchi, ddev, dt, iters);
            F.ddev[k] = ddev;
        }
    }
    cchi -= uc * f1[4] + vc * f2[4];
    const double cp = -uc * f1[0] - vc * f2[0] - third * dtmp * (2 * lt * tau - ltsq * (p + q + s) - ltsq * old_p) -
                      2 * third * tau * (uy + vx) - third * (p - 2 * q) * (ux + vy) + 2 * third * s * (vy - ux);
    const double cq = -uc * f1[1] - vc * f2[1] - dtmp * (q - ltsq / 6 * old_p) - third * tau * (uy + vx) +
                      third * (p - 2 * q) * (ux + vy) + third * s * (vy - ux);
    const double cs = -uc * f1[2] - vc * f2[2] - dtmp * (s + ltsq / 2 * old_p) - tau * (vx - uy) + (p + q) * (vy - ux);
    const double ctau = -uc * f1[3] - vc * f2[3] - dtmp * (tau - lt * old_p) - (p + q) * (uy + vx) + s * (vx - uy);
    B[CP][k] = p + cp;
    B[CQ][k] = q + cq;
    B[CS][k] = s + cs;
    B[CTAU][k] = tau + ctau;
    B[CCHI][k] = cchi;
}

// The explicit step per cell (i,j) and its lower-left node
// (shear_sim::step_forward, shear_sim.cc:218-349): the node's velocity and
// reference map advance by upwinded ENO2 advection, the net force of the
// four surrounding cells and the viscous terms in sheared coordinates (a
// node of row 0 keeps its values: the reference applies update_staggered
// there); the cell's stresses take the full elastic update.  New values go
// to buffer cur^1 (chi without its diffusion).
__global__ void k_ct_direct(ct_consts c, ct_fields F, int cur, double dt, double time, double viscosity) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= c.m || j >= c.n) return;
    const double third = 1. / 3., L = c.K - 2 * third * c.mu, lt = c.lamb * time, ltsq = lt * lt, mu = c.mu;
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt;
    const double hxxv = 2 * c.xsp * hx * viscosity, hyyv = 2 * c.ysp * hy * viscosity, hcv = 2 * (hxxv + hyyv);
    const double *const *A = F.f[cur];
    double *const *B = F.f[cur ^ 1];
    const size_t k = gidx(c, i, j);
    const long gm = c.gm;
    const double *U = A[CU], *V = A[CV];
    // velocity and reference map at the node
    if (j > 0) {
        const double uc = U[k], vc = V[k];
        double ux, vx, Xx, Yx, uy, vy, Xy, Yy;
        const long dx = uc > 0 ? -1 : 1, dy = vc > 0 ? -gm : gm;
        const double sx = uc > 0 ? hx : -hx, sy = vc > 0 ? hy : -hy;
        ux = eno_d(U, k, dx, sx);
        vx = eno_d(V, k, dx, sx);
        Xx = eno_d(A[CX], k, dx, sx);
        Yx = eno_d(A[CY], k, dx, sx);
        uy = eno_d(U, k, dy, sy);
        vy = eno_d(V, k, dy, sy);
        Xy = eno_d(A[CX], k, dy, sy);
        Yy = eno_d(A[CY], k, dy, sy);
        // net_force(fx, fy, -hx, -hy) of cells (i-1,j-1), (i,j-1), (i-1,j), (i,j)
        const double *P = A[CP], *Q = A[CQ], *S = A[CS], *T = A[CTAU];
        const size_t k0 = k - gm - 1, k1 = k - gm, k2 = k - 1, k3 = k;
        const double xf = -hx, yf = -hy;
        const double fx = (-P[k0] + P[k1] - P[k2] + P[k3] - Q[k0] + Q[k1] - Q[k2] + Q[k3] + S[k0] - S[k1] + S[k2] -
                           S[k3]) * xf +
                          (T[k0] + T[k1] - T[k2] - T[k3]) * yf;
        const double fy = (T[k0] - T[k1] + T[k2] - T[k3]) * xf +
                          (-P[k0] - P[k1] + P[k2] + P[k3] - Q[k0] - Q[k1] + Q[k2] + Q[k3] - S[k0] - S[k1] + S[k2] +
                           S[k3]) * yf;
        // viscosity, with the extra terms of the Laplacian in untransformed coordinates
        const double uvisc = hxxv * (U[k + 1] + U[k - 1]) + hyyv * (U[k + gm] + U[k - gm]) - hcv * uc +
                             dt * ltsq * c.xsp * c.xsp * (U[k + 1] - 2 * U[k] + U[k - 1]) -
                             .5 * lt * dt * c.xsp * c.ysp * (U[k + 1 + gm] - U[k + 1 - gm] - U[k - 1 + gm] + U[k - 1 - gm]);
        const double vvisc = hxxv * (V[k + 1] + V[k - 1]) + hyyv * (V[k + gm] + V[k - gm]) - hcv * vc +
                             dt * ltsq * c.xsp * c.xsp * (V[k + 1] - 2 * V[k] + V[k - 1]) -
                             .5 * lt * dt * c.xsp * c.ysp * (V[k + 1 + gm] - V[k + 1 - gm] - V[k - 1 + gm] + V[k - 1 - gm]);
        B[CU][k] = uc + (-uc * ux - vc * uy + c.mu_inv * (fx + uvisc) - 2 * dt * c.lamb * vc);
        B[CV][k] = vc + (-uc * vx - vc * vy + c.mu_inv * (fy + vvisc));
        B[CX][k] = A[CX][k] + (-uc * Xx - vc * Xy);
        B[CY][k] = A[CY][k] + (-uc * Yx - vc * Yy);
    } else {
        B[CU][k] = U[k];
        B[CV][k] = V[k];
        B[CX][k] = A[CX][k];
        B[CY][k] = A[CY][k];
    }
    // deformation rate, staggered velocity and spin
    const double u0 = U[k], ur = U[k + 1], uu = U[k + gm], uru = U[k + gm + 1];
    const double v0 = V[k], vr = V[k + 1], vu = V[k + gm], vru = V[k + gm + 1];
    const double uc = 0.25 * (u0 + ur + uu + uru), vc = 0.25 * (v0 + vr + vu + vru);
    const double ux = hx * (-u0 + ur - uu + uru), uy = hy * (-u0 - ur + uu + uru);
    const double vx = hx * (-v0 + vr - vu + vru), vy = hy * (-v0 - vr + vu + vru);
    const double p = A[CP][k], q = A[CQ][k], s = A[CS][k], tau = A[CTAU][k], chi = A[CCHI][k];
    const double old_p = p + (1. / 3) * c.lamb * time * (-2 * tau + c.lamb * time * (p + q + s));
    const long dx1 = uc > 0 ? -1 : 1, dy1 = vc > 0 ? -gm : gm;
    const double hsx = uc > 0 ? hx : -hx, hsy = vc > 0 ? hy : -hy;
    double f1[5], f2[5];
#pragma unroll
    for (int f = 0; f < 5; f++) {
        f1[f] = eno_d(A[CP + f], k, dx1, hsx);
        f2[f] = eno_d(A[CP + f], k, dy1, hsy);
    }
    const double pqs = p + q + s;
    const double unt_tau = tau - lt * pqs;
    const double unt_q = q + lt * (1 / 3.) * (-tau + lt * .5 * pqs);
    const double unt_s = s + lt * (tau - lt * .5 * pqs);
    const double sbar = sqrt(3 * unt_q * unt_q + unt_s * unt_s + unt_tau * unt_tau);
    double cchi = chi, dtmp = 0;
    if (sbar >= 1e-12) {
        const bool athermal = c.law.stz_model >= 2;
        if (athermal && sbar < c.law.s_y) {
            F.ddev[k] = 0;
        } else {
            double ddev;
            int iters;
            dtmp = adaptive_plastic(c.law, sbar, cchi, ddev, dt, iters);
            F.ddev[k] = ddev;
        }
    }
    cchi -= uc * f1[4] + vc * f2[4];
    const double cp = -uc * f1[0] - vc * f2[0] + 2 * c.lamb * lt * third * mu * dt +
                      third * (-dtmp * (2 * lt * tau - ltsq * (p + q + s + old_p)) - 2 * (tau - lt * mu) * (uy + vx) -
                               (3 * L + 2 * mu + p - 2 * q) * (ux + vy) + 2 * s * (vy - ux) -
                               ltsq * (L * (vy + ux) + 2 * mu * ux));
    const double cq = -uc * f1[1] - vc * f2[1] - dtmp * (q - .5 * third * ltsq * old_p) +
                      third * (dt * lt * c.lamb * mu - (tau - lt * mu) * (uy + vx) +
                               (p - 2 * q - mu - .5 * ltsq * L) * (ux + vy) - ltsq * mu * ux + s * (vy - ux));
    const double cs = -uc * f1[2] - vc * f2[2] - c.lamb * lt * mu * dt - dtmp * (s + .5 * ltsq * old_p) -
                      (tau - lt * mu) * (vx - uy) + (p + q - mu) * (vy - ux) + .5 * ltsq * L * (ux + vy) + ltsq * mu * ux;
    const double ctau = -uc * f1[3] - vc * f2[3] + dt * c.lamb * mu + ltsq * mu * vx - lt * (mu + L) * (ux + vy) +
                        (vx - uy) * s + (mu - p - q) * (vx + uy) - dtmp * (tau - lt * old_p);
    B[CP][k] = p + cp;
    B[CQ][k] = q + cq;
    B[CS][k] = s + cs;
    B[CTAU][k] = tau + ctau;
    B[CCHI][k] = cchi;
}

// Dpl-mediated chi diffusion in sheared coordinates (shear_sim::chi_diffusion,
// shear_sim.cc:437-460), from the old chi of buffer `old` into the new chi.
__global__ void k_ct_chi_diffusion(ct_consts c, ct_fields F, int old, double lt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= c.m || j >= c.n) return;
    const double dfac = 0.25 * c.chi_len * c.chi_len * c.mu_inv, dfacx = dfac * c.xsp * c.xsp,
                 dfacy = dfac * c.ysp * c.ysp, lfac = c.dy * c.xsp * lt * 0.25;
    const size_t k = gidx(c, i, j);
    const long gm = c.gm;
    const double *X = F.f[old][CCHI], *D = F.ddev;
    const double Dd = D[k] + D[k - gm], Dl = D[k] + D[k - 1], Dr = D[k] + D[k + 1], Du = D[k] + D[k + gm];
    const double Td = Dd * (X[k] - X[k - gm] - lfac * (X[k + 1] + X[k + 1 - gm] - X[k - 1] - X[k - 1 - gm]));
    const double Tl = Dl * (X[k] - X[k - 1]), Tr = Dr * (X[k + 1] - X[k]);
    const double Tu = Du * (X[k + gm] - X[k] - lfac * (X[k + 1 + gm] + X[k + 1] - X[k - 1 + gm] - X[k - 1]));
    const double diffx = dfacx * (Tr - Tl), diffy = dfacy * (Tu - Td);
    F.f[old ^ 1][CCHI][k] += (1 - lt) * diffx + diffy;
}

// set_boundaries, rows (shear_sim.cc:778-802): periodic copies with Y
// shifted by -+ly, or the walls' corner values and extrapolated cells.
__global__ void k_ct_rows(ct_consts c, ct_fields F, int b, double time) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.m) return;
    double *const *G = F.f[b];
    auto at = [&](int row) { return gidx(c, i, row); };
    if (c.yp) {
        const int n = c.n;
        const int dst[4] = {-2, -1, n, n + 1}, src[4] = {n - 2, n - 1, 0, 1};
        const double dY[4] = {-c.ly, -c.ly, c.ly, c.ly};
        for (int r = 0; r < 4; r++) {
            const size_t d = at(dst[r]), s = at(src[r]);
            for (int f = CU; f <= CCHI; f++) G[f][d] = G[f][s];
            G[CX][d] = G[CX][s] + 0.0;
            G[CY][d] = G[CY][s] + dY[r];
        }
        return;
    }
    const double U = c.u_bdry;  // bdry_vel (shear_sim.hh:170-173)
    const double bp = time < 1 ? c.u_bdry * time * time * 0.5 : c.u_bdry * (time - 0.5);
    const double xl = c.ax + bp + i * c.dx, xu = c.ax - bp + i * c.dx;
    auto corner = [&](size_t k, double u, double v, double Xv, double Yv) {
        G[CU][k] = u;
        G[CV][k] = v;
        G[CX][k] = Xv;
        G[CY][k] = Yv;
    };
    auto extrap = [&](size_t k, size_t k0, size_t k1) {
        for (int f = CP; f <= CCHI; f++) G[f][k] = 2 * G[f][k0] - G[f][k1];
    };
    const int n = c.n;
    corner(at(0), -U, 0, xl, c.ay);
    extrap(at(-1), at(0), at(1));
    corner(at(-1), -U, 0, xl, c.ay - c.dy);
    extrap(at(-2), at(-1), at(0));
    corner(at(n), U, 0, xu, c.by);
    extrap(at(n), at(n - 1), at(n - 2));
    corner(at(n + 1), U, 0, xu, c.by + c.dy);
    extrap(at(n + 1), at(n), at(n - 1));
}

// set_boundaries, ghost columns of every row (shear_sim.cc:804-810).
__global__ void k_ct_cols(ct_consts c, ct_fields F, int b) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x - 2;  // rows -2..n+1
    if (r > c.n + 1) return;
    double *const *G = F.f[b];
    const int m = c.m;
    const int dst[4] = {-2, -1, m, m + 1}, src[4] = {m - 2, m - 1, 0, 1};
    const double dX[4] = {-c.lx, -c.lx, c.lx, c.lx};
    for (int q = 0; q < 4; q++) {
        const size_t d = gidx(c, dst[q], r), s = gidx(c, src[q], r);
        for (int f = CU; f <= CCHI; f++) G[f][d] = G[f][s];
        G[CX][d] = G[CX][s] + dX[q];
        G[CY][d] = G[CY][s] + 0.0;
    }
}

// Projection source at node (i,j) (shear_sim::projection_step,
// shear_sim.cc:477-507, net_force :547-559): pre * net force, or -+(U, 0) on
// the wall rows.
__global__ void k_ct_source(ct_consts c, ct_fields F, int cur, double xfac, double yfac, double pa, double pb,
                            double pc, double pd, double2 *b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= c.m || j >= c.lsn) return;
    double2 out;
    if (!c.yp && (j == 0 || j == c.n)) {
        const double U = c.u_bdry;
        out = j == 0 ? make_double2(-U, -0.) : make_double2(U, 0.);
    } else {
        const double *const *A = F.f[cur];
        const size_t k3 = gidx(c, i, j), k2 = k3 - 1, k1 = k3 - c.gm, k0 = k1 - 1;
        const double *P = A[CP], *Q = A[CQ], *S = A[CS], *T = A[CTAU];
        const double fx = (-P[k0] + P[k1] - P[k2] + P[k3] - Q[k0] + Q[k1] - Q[k2] + Q[k3] + S[k0] - S[k1] + S[k2] -
                           S[k3]) * xfac + (T[k0] + T[k1] - T[k2] - T[k3]) * yfac;
        const double fy = (T[k0] - T[k1] + T[k2] - T[k3]) * xfac +
                          (-P[k0] - P[k1] + P[k2] + P[k3] - Q[k0] - Q[k1] + Q[k2] + Q[k3] - S[k0] - S[k1] + S[k2] +
                           S[k3]) * yfac;
        out = make_double2(pa * fx + pb * fy, pc * fx + pd * fy);
    }
    b[(size_t)j * c.m + i] = out;
}

// Stress correction and velocities per cell (shear_sim.cc:509-543).
__global__ void k_ct_project(ct_consts c, ct_fields F, int cur, const double2 *vel, double dt, double lt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= c.m || j >= c.n) return;
    const double third = 1. / 3, L = c.K - 2 * third * c.mu, ltsq = lt * lt, mu = c.mu, lamb = c.lamb;
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt;
    const int m = c.m, lsn = c.lsn;
    const int d = i == m - 1 ? 1 - m : 1, e = j == lsn - 1 ? m * (1 - lsn) : m;
    const double2 *vp = vel + (i + (size_t)m * j);
    double *const *G = F.f[cur];
    const size_t k = gidx(c, i, j);
    G[CU][k] = vp->x;
    G[CV][k] = vp->y;
    const double ux = hx * (-vp->x + vp[d].x - vp[e].x + vp[d + e].x),
                 uy = hy * (-vp->x - vp[d].x + vp[e].x + vp[d + e].x),
                 vx = hx * (-vp->y + vp[d].y - vp[e].y + vp[d + e].y),
                 vy = hy * (-vp->y - vp[d].y + vp[e].y + vp[d + e].y);
    G[CP][k] += 2 * third * lt * lamb * mu * dt + 2 * third * lt * mu * uy -
                (L + third * L * ltsq + 2 * third * mu) * (vy + ux) - 2 * third * mu * ltsq * ux +
                2 * third * mu * lt * vx;
    G[CQ][k] += third * lt * lamb * mu * dt + third * lt * mu * uy - (L * ltsq / 6 + third * mu) * (vy + ux) -
                third * ltsq * mu * ux + third * lt * mu * vx;
    G[CS][k] += -lamb * lt * mu * dt + lt * mu * (vx - uy) + (L * ltsq / 2 - mu) * vy +
                (L * ltsq / 2 + mu + ltsq * mu) * ux;
    G[CTAU][k] += lamb * mu * dt + mu * uy - lt * (L + mu) * (vy + ux) + mu * (1 + ltsq) * vx;
}

// The reference's mat (mat.hh): row-major 2x2 with its product and inverse.
struct m22 {
    double a, b, c, d;
};
inline m22 mmul(const m22 &x, const m22 &e) {
    return m22{x.a * e.a + x.b * e.c, x.a * e.b + x.b * e.d, x.c * e.a + x.d * e.c, x.c * e.b + x.d * e.d};
}
inline m22 minv(const m22 &x) {
    const double idet = 1.0 / (x.a * x.d - x.b * x.c);
    return m22{idet * x.d, -idet * x.b, -idet * x.c, idet * x.a};
}

// ---- Lagrangian tracers (shear_sim::initialize_tracers, update_tracers and
// correct_tracer, shear_sim.cc:1247-1355) ----
//
// The reference map (X, Y) is interpolated with the bicubic convolution of
// bicubic_interp (bi_interp.cc): on the ghosted node grid (origin two cells
// before ax, ay), the four rows around the point are each reduced to the
// coefficients (f1, (f2 - f0)/2, f0 - 5f1/2 + 2f2 - f3/2, (3f1 - f0 - 3f2 +
// f3)/2) of the cubic through four samples, and the same combination is
// taken across the rows.  A tracer keeps its reference point fixed; an update
// predicts the position from the velocity estimate and corrects it by Newton
// iterations on X(x) = Xref (four iterations within tolerance, at most 100).

__device__ __forceinline__ void cubic_coeffs(double f0, double f1, double f2, double f3, double *a) {
    a[0] = f1;
    a[1] = -0.5 * f0 + 0.5 * f2;
    a[2] = f0 - 2.5 * f1 + 2 * f2 - 0.5 * f3;
    a[3] = -0.5 * f0 + 1.5 * f1 - 1.5 * f2 + 0.5 * f3;
}

__device__ __forceinline__ double cubic_at(const double *a, double y) { return a[0] + y * (a[1] + y * (a[2] + y * a[3])); }
__device__ __forceinline__ double cubic_slope(const double *a, double y) { return a[1] + y * (2 * a[2] + 3 * y * a[3]); }

// Value and gradient of the bicubic interpolant of node field f at (x, y);
// false outside the grid squares the reference accepts (bi_interp.cc:17-27).
__device__ bool bicubic_grad(const ct_consts &c, const double *__restrict__ f, double x, double y, double &v, double &fx,
                             double &fy) {
    const int gm = c.gm, gn = c.n + 4;
    x = (x - (c.ax - 2 * c.dx)) * c.xsp;
    y = (y - (c.ay - 2 * c.dy)) * c.ysp;
    const int i = static_cast<int>(x), j = static_cast<int>(y);
    if (i < 1 || i > gm - 2 || j < 1 || j > gn - 2) return false;
    x -= i;
    y -= j;
    const double *up = f + i + (size_t)gm * j;
    double r[4][4], a[4][4];  // r[row][k]: cubic in x of rows j-1 .. j+2
    cubic_coeffs(up[-gm - 1], up[-gm], up[-gm + 1], up[-gm + 2], r[0]);
    cubic_coeffs(up[-1], up[0], up[1], up[2], r[1]);
    cubic_coeffs(up[gm - 1], up[gm], up[gm + 1], up[gm + 2], r[2]);
    cubic_coeffs(up[2 * gm - 1], up[2 * gm], up[2 * gm + 1], up[2 * gm + 2], r[3]);
    for (int k = 0; k < 4; k++) cubic_coeffs(r[0][k], r[1][k], r[2][k], r[3][k], a[k]);  // a[k]: cubic in y
    fx = c.xsp * (cubic_at(a[1], y) + x * (2 * cubic_at(a[2], y) + 3 * x * cubic_at(a[3], y)));
    fy = c.ysp * (cubic_slope(a[0], y) + x * (cubic_slope(a[1], y) + x * (cubic_slope(a[2], y) + x * cubic_slope(a[3], y))));
    v = cubic_at(a[0], y) + x * (cubic_at(a[1], y) + x * (cubic_at(a[2], y) + x * cubic_at(a[3], y)));
    return true;
}

// ok[t]: 1 updated, 0 Newton failed (the reference drops the tracer), -1
// the interpolation left the grid (the reference stops the program).
__global__ void k_ct_tracers(ct_consts c, const double *__restrict__ X, const double *__restrict__ Y,
                             double *__restrict__ tr, int *__restrict__ ok, int ntr, double dt, double dtinv) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntr) return;
    double *p = tr + 6 * (size_t)t;
    const double xref = p[0], yref = p[1];
    double xx = p[2] + dt * p[4], yy = p[3] + dt * p[5];
    const double tol = DBL_EPSILON, tolnewt = tol * tol * 1e6;
    const double ilx = 1 / c.lx, ily = 1 / c.ly, bigstep = c.lx * c.lx + c.ly * c.ly;
    int count = 0, iter = 0, res = 1;
    while (count < 4) {
        if (iter > 100) {
            res = 0;
            break;
        }
        const double xs = floor((xx - c.ax) * ilx) * c.lx, ys = floor((yy - c.ay) * ily) * c.ly;
        double vx, vy, fxx, fxy, fyx, fyy;
        if (!bicubic_grad(c, X, xx - xs, yy - ys, vx, fxx, fxy) || !bicubic_grad(c, Y, xx - xs, yy - ys, vy, fyx, fyy)) {
            res = -1;
            break;
        }
        const double fx = vx - xref + xs, fy = vy - yref + ys;
        if (fx * fx + fy * fy < tolnewt) count++;
        const double det = fxx * fyy - fxy * fyx;
        if (det < tol && det > -tol) {
            res = 0;
            break;
        }
        const double delx = (fyy * fx - fxy * fy) / det, dely = (-fyx * fx + fxx * fy) / det;
        if (delx * delx + dely * dely > bigstep) {
            res = 0;
            break;
        }
        xx -= delx;
        yy -= dely;
        iter++;
    }
    ok[t] = res;
    if (res == 1) {
        p[4] = (xx - p[2]) * dtinv;
        p[5] = (yy - p[3]) * dtinv;
        p[2] = xx;
        p[3] = yy;
    }
}

}  // namespace
}  // namespace stzg

using namespace stzg;

struct stzg_ct {
    stzg_ct_params P;
    ct_consts c;
    ct_fields F;
    int cur = 0;
    double time = 0;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<void *> owned;
    stzg_tgmg *mg = nullptr;
    stzg_tgmg_predict tp;
    int checked = 0;  // solve policy: 0 the reference's predictor, 1 residual checks
    double2 *mg_b = nullptr, *mg_z = nullptr;
    std::vector<double> table;
    std::vector<int> cls;
    // Lagrangian tracers: 6 doubles each (reference point, position,
    // velocity estimate), their count and creation time
    double *tr = nullptr;
    int *tr_ok = nullptr;
    int ntrace = 0, tr_cap = 0;
    int tr_m = 0, tr_n = 0;  // the tracer grid of the last stzg_ct_tracers_init
    int f_num = 0;           // frames written by the frame loops (shear_sim::f_num)
    double tr_time = 0;
};

namespace {

int ct_alloc(stzg_ct *s, double **p, size_t count) {
    void *q;
    cudaError_t e = cudaMalloc(&q, count * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    s->owned.push_back(q);
    STZG_CUDA(cudaMemsetAsync(q, 0, count * sizeof(double), s->st));
    *p = (double *)q;
    return STZG_OK;
}

const dim3 kB2(32, 8);
inline dim3 g2(int m, int n) { return dim3(ceil_div(m, 32), ceil_div(n, 8)); }


void boundaries(stzg_ct *s, int b) {
    k_ct_rows<<<ceil_div(s->c.m, 128), 128, 0, s->st>>>(s->c, s->F, b, s->time);
    note_launch();
    k_ct_cols<<<ceil_div(s->c.n + 4, 128), 128, 0, s->st>>>(s->c, s->F, b);
    note_launch();
}

// qs_multi::init(viscdt, lt) (coord_transforms qs_multi.cc:31-46): the
// preconditioned blocks, as a two-stencil table (interior; wall rows that
// carry only the identity) for the block multigrid, and the source's
// preconditioner pre = regci * (1 lt; 0 1) (shear_sim.cc:476).
void operator_for(stzg_ct *s, double lt, m22 &pre) {
    const ct_consts &c = s->c;
    const double ltsq = lt * lt, L = c.K - 2. / 3. * c.mu, mu = c.mu;
    const double xsp2 = c.xsp * c.xsp, ysp2 = c.ysp * c.ysp, xsp = c.xsp, ysp = c.ysp;
    m22 regh{(L + 2 * mu + ltsq * mu) * xsp2, (lt * mu + lt * ltsq * mu) * xsp2, -lt * (L + mu) * xsp2,
             mu * (1 + ltsq) * xsp2};
    m22 regv{mu * ysp2, lt * mu * ysp2, 0, (L + 2 * mu) * ysp2};
    const m22 sum{regh.a + regv.a, regh.b + regv.b, regh.c + regv.c, regh.d + regv.d};
    const m22 regc{-2. * sum.a, -2. * sum.b, -2. * sum.c, -2. * sum.d};
    const m22 regci = minv(regc);
    m22 regd{-0.5 * xsp * ysp * lt * mu, 0.25 * xsp * ysp * (L + mu - 2 * ltsq * mu), 0.25 * xsp * ysp * (L + mu),
             -0.25 * xsp * ysp * lt * (L + 3 * mu)};
    regh = mmul(regci, regh);
    regv = mmul(regci, regv);
    regd = mmul(regci, regd);
    pre = mmul(regci, m22{1., lt, 0, 1.});
    const m22 nd{-regd.a, -regd.b, -regd.c, -regd.d};
    const m22 blocks[9] = {regd, regv, nd, regh, m22{1, 0, 0, 1}, regh, nd, regv, regd};
    s->table.assign(2 * 36, 0.0);
    for (int k = 0; k < 9; k++) {
        s->table[4 * k + 0] = blocks[k].a;
        s->table[4 * k + 1] = blocks[k].b;
        s->table[4 * k + 2] = blocks[k].c;
        s->table[4 * k + 3] = blocks[k].d;
    }
    s->table[36 + 16] = 1;  // wall stencil: identity centre (regz elsewhere, rego)
    s->table[36 + 19] = 1;
}

int advection_step(stzg_ct *s, double dt) {
    k_ct_advect<<<g2(s->c.m, s->c.n), kB2, 0, s->st>>>(s->c, s->F, s->cur, dt, s->time);
    note_launch();
    if (s->c.chi_len != 0) {
        k_ct_chi_diffusion<<<g2(s->c.m, s->c.n), kB2, 0, s->st>>>(s->c, s->F, s->cur, s->c.lamb * s->time);
        note_launch();
    }
    s->cur ^= 1;
    s->time += dt;
    boundaries(s, s->cur);
    return STZG_OK;
}

// shear_sim::step_forward (shear_sim.cc:218-349): the explicit update, chi
// diffusion, time, boundaries.
int direct_step(stzg_ct *s, double dt) {
    k_ct_direct<<<g2(s->c.m, s->c.n), kB2, 0, s->st>>>(s->c, s->F, s->cur, dt, s->time, s->P.viscosity);
    note_launch();
    if (s->c.chi_len != 0) {
        k_ct_chi_diffusion<<<g2(s->c.m, s->c.n), kB2, 0, s->st>>>(s->c, s->F, s->cur, s->c.lamb * s->time);
        note_launch();
    }
    s->cur ^= 1;
    s->time += dt;
    boundaries(s, s->cur);
    return STZG_OK;
}

int projection_step(stzg_ct *s, double dt, long *vcycles) {
    const double lt = s->c.lamb * s->time;
    m22 pre;
    operator_for(s, lt, pre);
    STZG_CUDA(cudaStreamSynchronize(s->st));
    // the class map (wall rows or not) is the one the solver was created with
    STZG_CHECK(stzg_tgmg_set_operator(s->mg, s->table.data(), 2, nullptr));
    const double xfac = 0.5 / dt * s->c.xsp, yfac = 0.5 / dt * s->c.ysp;
    k_ct_source<<<g2(s->c.m, s->c.lsn), kB2, 0, s->st>>>(s->c, s->F, s->cur, xfac, yfac, pre.a, pre.b, pre.c,
                                                        pre.d, s->mg_b);
    note_launch();
    STZG_CUDA(cudaStreamSynchronize(s->st));
    int it = 0;
    // checked: V-cycles until the residual meets acc (at most the predictor's
    // own limit, max_thresh / mult), then the extra one
    const int st = s->checked ? stzg_tgmg_solve_checked(s->mg, STZG_TGMG_VCYCLE, s->tp.max_thresh / s->tp.mult,
                                                        s->tp.extra_iters, 1.0, 1, 1, 10, &it, nullptr)
                              : stzg_tgmg_solve(s->mg, STZG_TGMG_VCYCLE, &s->tp, 1.0, 1, 1, 10, &it, nullptr);
    if (st != STZG_OK) return st;
    if (vcycles) *vcycles += it;
    k_ct_project<<<g2(s->c.m, s->c.n), kB2, 0, s->st>>>(s->c, s->F, s->cur, s->mg_z, dt, lt);
    note_launch();
    boundaries(s, s->cur);
    return STZG_OK;
}

// ---- frames, strain and tracer files (shear_sim.cc:892-1059, 1360-1420) ----
// Frames are written from a host copy of the ghosted arrays; the arithmetic
// restates the reference's expressions in its order (host code is built
// without floating-point contraction), so files written from the same state
// hold the same bytes.

// The ghosted host arrays of the current state: u, v, p, q, s, tau, chi, X,
// Y, then the six strain values (cu, cv, cp, cq, cs, ctau of the reference's
// c_field after compute_strain).
struct ct_host {
    int m, n, gm, gn;
    std::vector<double> f[CF + 6];
    size_t at(int i, int j) const { return (size_t)(j + 2) * gm + (i + 2); }  // i, j >= -2
};

int ct_fetch(stzg_ct *s, ct_host &h) {
    const ct_consts &c = s->c;
    h.m = c.m;
    h.n = c.n;
    h.gm = c.gm;
    h.gn = c.n + 4;
    const size_t pts = (size_t)h.gm * h.gn;
    for (int f = 0; f < CF; f++) {
        h.f[f].resize(pts);
        STZG_CUDA(cudaMemcpyAsync(h.f[f].data(), s->F.f[s->cur][f], pts * sizeof(double), cudaMemcpyDeviceToHost,
                                  s->st));
    }
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

// shear_sim::compute_strain (shear_sim.cc:1008-1059): the Green-Lagrange
// strain of the physical deformation gradient T * (d(X,Y)/d(x,y))^-1, T = (1
// lt; 0 1), with its components (E_xx, E_xy, E_yy), trace, second invariant
// and deviatoric norm per cell, then set_strain_boundaries
// (shear_sim.cc:814-850): ghost rows extrapolated (walls) or periodic, ghost
// columns periodic.
void ct_strain(const stzg_ct *s, ct_host &h, double lt) {
    const ct_consts &c = s->c;
    const int m = h.m, n = h.n;
    double *E6[6];
    for (int k = 0; k < 6; k++) {
        h.f[CF + k].assign((size_t)h.gm * h.gn, 0.0);
        E6[k] = h.f[CF + k].data();
    }
    const double *X = h.f[CX].data(), *Y = h.f[CY].data();
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            const size_t k = h.at(i, j);
            const double Xy = 0.5 * c.ysp * (X[k + h.gm] - X[k - h.gm]), Yy = 0.5 * c.ysp * (Y[k + h.gm] - Y[k - h.gm]);
            const double Xx = 0.5 * c.xsp * (X[k + 1] - X[k - 1]), Yx = 0.5 * c.xsp * (Y[k + 1] - Y[k - 1]);
            const double J = 1 / (Xx * Yy - Xy * Yx);
            const double ma = Yy * J, mb = -Xy * J, mc = -Yx * J, md = Xx * J;
            // T * M with T = (1 lt; 0 1), in the order of mat::operator*
            const double Fa = 1 * ma + lt * mc, Fb = 1 * mb + lt * md, Fc = 0 * ma + 1 * mc, Fd = 0 * mb + 1 * md;
            // E = (F^T F - I) / 2 (mat::ATA)
            double ea = Fa * Fa + Fc * Fc, eb = Fa * Fb + Fc * Fd, ed = Fb * Fb + Fd * Fd;
            ea -= 1.;
            ed -= 1.;
            ea *= 0.5;
            eb *= 0.5;
            ed *= 0.5;
            E6[0][k] = ea;
            E6[1][k] = eb;
            E6[2][k] = ed;
            const double tr = ea + ed;
            E6[3][k] = tr;
            E6[4][k] = ea * ed - eb * eb;
            const double tfac = 1 / 3. * tr;
            ea -= tfac;
            ed -= tfac;
            E6[5][k] = std::sqrt(ea * ea + 2 * eb * eb + ed * ed + tfac * tfac);
        }
    auto copy6 = [&](size_t to, size_t from) {
        for (int q = 0; q < 6; q++) E6[q][to] = E6[q][from];
    };
    for (int i = 0; i < m; i++) {
        if (c.yp) {
            copy6(h.at(i, -2), h.at(i, n - 2));
            copy6(h.at(i, -1), h.at(i, n - 1));
            copy6(h.at(i, n), h.at(i, 0));
            copy6(h.at(i, n + 1), h.at(i, 1));
        } else {
            for (int q = 0; q < 6; q++) {
                double *e = E6[q];
                e[h.at(i, -1)] = 2 * e[h.at(i, 0)] - e[h.at(i, 1)];
                e[h.at(i, -2)] = 2 * e[h.at(i, -1)] - e[h.at(i, 0)];
                e[h.at(i, n)] = 2 * e[h.at(i, n - 1)] - e[h.at(i, n - 2)];
                e[h.at(i, n + 1)] = 2 * e[h.at(i, n)] - e[h.at(i, n - 1)];
            }
        }
    }
    for (int j = -2; j < n + 2; j++) {
        copy6(h.at(-2, j), h.at(m - 2, j));
        copy6(h.at(-1, j), h.at(m - 1, j));
        copy6(h.at(m, j), h.at(0, j));
        copy6(h.at(m + 1, j), h.at(1, j));
    }
}

// c_field::dev(lt) (fields.hh): the deviatoric norm of the untransformed stress
double ct_dev(const ct_host &h, size_t k, double lt) {
    const double p = h.f[CP][k], q = h.f[CQ][k], s = h.f[CS][k], tau = h.f[CTAU][k];
    const double unt_tau = tau - lt * (p + q + s);
    const double unt_q = q + lt * (1 / 3.) * (-tau + lt * .5 * (p + q + s));
    const double unt_s = s + lt * (tau - lt * .5 * (p + q + s));
    return std::sqrt(3 * unt_q * unt_q + unt_s * unt_s + unt_tau * unt_tau);
}

// shear_sim::output (shear_sim.cc:937-1004) of one mode into out: staggered
// modes 2-8 on n rows of m cell centres; the others on n (y periodic) or n+1
// rows of m nodes, plus (walls) the periodic copy of the first node, shifted
// by the period for X.  Each row is led by its y coordinate, the header row
// by the row length and the x coordinates.
void ct_output(const stzg_ct *s, const ct_host &h, int mode, std::vector<float> &out) {
    const ct_consts &c = s->c;
    const int m = h.m, n = h.n;
    const bool st = mode >= 2 && mode <= 8;
    const int l = st ? m : (c.yp ? m : m + 1);
    const int rows = st ? n : (c.yp ? n : n + 1);
    const double lt = c.lamb * s->time;
    out.assign((size_t)(rows + 1) * (l + 1), 0.f);
    std::vector<float> buf(m + 2);
    buf[0] = (float)l;
    for (int i = 0; i < l; i++) buf[i + 1] = (float)(c.ax + (st ? (i + 0.5) * c.dx : i * c.dx));
    std::copy(buf.begin(), buf.begin() + l + 1, out.begin());
    for (int j = 0; j < rows; j++) {
        buf[0] = (float)(c.ay + (st ? (j + 0.5) * c.dy : j * c.dy));
        for (int i = 0; i < m; i++) {
            const size_t k = h.at(i, j);
            double v;
            switch (mode) {
                case 7: v = h.f[CCHI][k] * s->P.TZ; break;
                case 8: v = ct_dev(h, k, lt); break;
                default: v = mode <= 6 ? h.f[mode][k] : (mode <= 10 ? h.f[mode - 2][k] : h.f[CF + mode - 11][k]);
            }
            buf[i + 1] = (float)v;
        }
        if (!st) buf[m + 1] = mode == 9 ? (float)(buf[1] + c.bx - c.ax) : buf[1];
        std::copy(buf.begin(), buf.begin() + l + 1, out.begin() + (size_t)(j + 1) * (l + 1));
    }
}

int ct_write_floats(const char *dir, const char *prefix, int sn, const std::vector<float> &v) {
    char path[4096];
    std::snprintf(path, sizeof(path), "%s/%s.%d", dir, prefix, sn);
    std::FILE *fp = std::fopen(path, "wb");
    if (!fp) return fail(STZG_EINVAL, std::string("cannot open ") + path);
    const size_t w = std::fwrite(v.data(), sizeof(float), v.size(), fp);
    std::fclose(fp);
    if (w != v.size()) return fail(STZG_EINVAL, std::string("short write to ") + path);
    return STZG_OK;
}

// bicubic_interp (bi_interp.cc) of field `mode` (fval order: u, v, p, q, s,
// tau, chi, X, Y, then the six strain values) at (x, y): the cubic
// convolution through four samples in x on four rows, then across the rows,
// on the ghosted grid (origin 2 cells before (ax, ay) for the node fields u,
// v, X, Y, 1.5 cells for the others).  false where the grid square leaves
// the ghosted grid (the reference stops the program there).  The reference
// keeps the last grid square's coefficients between calls, stale when the
// field has changed since; here they are formed anew each time.
bool ct_bicubic(const stzg_ct *s, const ct_host &h, int mode, double x, double y, double *val) {
    const ct_consts &c = s->c;
    const bool cor = (1 << mode) & (3 | 384);
    const double ox = c.ax - (cor ? 2 : 1.5) * c.dx, oy = c.ay - (cor ? 2 : 1.5) * c.dy;
    x = (x - ox) * c.xsp;
    y = (y - oy) * c.ysp;
    const int i = (int)x, j = (int)y;
    if (i < 1 || i > h.gm - 2 || j < 1 || j > h.gn - 2) return false;
    const int fi = mode <= 8 ? mode : CF + mode - 9;
    const double *F = h.f[fi].data();
    auto cx = [&](int jj, double *q) {  // compute_x on ghosted row jj at column i
        const size_t r = (size_t)jj * h.gm;
        const double f0 = F[r + i - 1], f1 = F[r + i], f2 = F[r + i + 1], f3 = F[r + i + 2];
        q[0] = f1;
        q[1] = -0.5 * f0 + 0.5 * f2;
        q[2] = f0 - 2.5 * f1 + 2 * f2 - 0.5 * f3;
        q[3] = -0.5 * f0 + 1.5 * f1 - 1.5 * f2 + 0.5 * f3;
    };
    double r0[4], r1[4], r2[4], r3[4], a[16];
    cx(j, r1);
    cx(j + 1, r2);
    cx(j - 1, r0);
    cx(j + 2, r3);
    for (int q = 0; q < 4; q++) {  // fill_a over the rows for the x power q
        double *ap = a + 4 * q;
        const double c0 = r0[q], c1 = r1[q], c2 = r2[q], c3 = r3[q];
        ap[0] = c1;
        ap[1] = -0.5 * c0 + 0.5 * c2;
        ap[2] = c0 - 2.5 * c1 + 2 * c2 - 0.5 * c3;
        ap[3] = -0.5 * c0 + 1.5 * c1 - 1.5 * c2 + 0.5 * c3;
    }
    x -= i;
    y -= j;
    auto yl = [&](const double *ap) { return *ap + y * (ap[1] + y * (ap[2] + y * ap[3])); };
    *val = yl(a) + x * (yl(a + 4) + x * (yl(a + 8) + x * yl(a + 12)));
    return true;
}

// shear_sim::write_files (shear_sim.cc:892-931) into directory dir.
int ct_write_files(stzg_ct *s, const char *dir, int k, unsigned fflags) {
    static const char *names[17] = {"u", "v", "p", "q", "s", "tau", "chi", "tem", "dev", "X", "Y",
                                    "Exx", "Exy", "Eyy", "E_I", "E_II", "Edev"};
    ct_host h;
    STZG_CHECK(ct_fetch(s, h));
    std::vector<float> buf;
    for (int mode = 0; mode <= 10; mode++)
        if ((fflags & (1u << mode)) || mode == 8) {  // the reference writes dev whatever the flags
            ct_output(s, h, mode, buf);
            STZG_CHECK(ct_write_floats(dir, names[mode], k, buf));
        }
    if (fflags & 14336) ct_strain(s, h, s->c.lamb * s->time);
    for (int mode = 11; mode <= 16; mode++)
        if (fflags & (mode <= 13 ? 2048u : 4096u)) {
            ct_output(s, h, mode, buf);
            STZG_CHECK(ct_write_floats(dir, names[mode], k, buf));
        }
    if ((fflags & 8192) && s->tr) {
        if (k > 0) STZG_CHECK(stzg_ct_tracers_update(s, nullptr));  // the fields stay as fetched
        std::vector<double> tr((size_t)6 * s->ntrace);
        if (s->ntrace)
            STZG_CUDA(cudaMemcpy(tr.data(), s->tr, sizeof(double) * tr.size(), cudaMemcpyDeviceToHost));
        const ct_consts &c = s->c;
        const double ilx = 1 / c.lx, ily = 1 / c.ly;
        // output_tracers (shear_sim.cc:1360-1386)
        char path[4096];
        std::snprintf(path, sizeof(path), "%s/tra.%d", dir, k);
        std::FILE *fp = std::fopen(path, "w");
        if (!fp) return fail(STZG_EINVAL, std::string("cannot open ") + path);
        for (int t = 0; t < s->ntrace; t++) {
            const double *q = &tr[(size_t)6 * t];
            const double xx = q[2], yy = q[3];
            const double xw = xx - std::floor((xx - c.ax) * ilx) * c.lx, yw = yy - std::floor((yy - c.ay) * ily) * c.ly;
            double v[8];
            const int modes[8] = {2, 6, 9, 10, 11, 12, 13, 14};
            for (int u = 0; u < 8; u++)
                if (!ct_bicubic(s, h, modes[u], xw, yw, &v[u])) {
                    std::fclose(fp);
                    return fail(STZG_EINVAL, "a tracer left the interpolation grid");
                }
            std::fprintf(fp, "%.12g %.12g %.12g %.12g %.12g %.12g %.12g %.10g %.10g %.10g %.10g %.10g %.10g\n", xx, yy,
                         q[0], q[1], v[0], v[1], v[1] * s->P.TZ, v[2], v[3], v[4], v[5], v[6], v[7]);
        }
        std::fclose(fp);
        // output_tracers_matrix("teml", 4, k) (shear_sim.cc:1389-1420): chi*TZ at each
        // tracer of the tracer grid
        if (s->tr_m > c.m + 1) return fail(STZG_EINVAL, "tracer grid wider than the output buffer");
        if (s->ntrace != s->tr_m * s->tr_n) return fail(STZG_EINVAL, "matrix output after tracers were lost");
        const double delx = c.lx / s->tr_m, dely = (c.by - c.ay) / s->tr_n;
        std::vector<float> mat((size_t)(s->tr_n + 1) * (s->tr_m + 1));
        mat[0] = (float)s->tr_m;
        for (int i = 0; i < s->tr_m; i++) mat[i + 1] = (float)(c.ax + (i + 0.5) * delx);
        for (int j = 0; j < s->tr_n; j++) {
            float *row = &mat[(size_t)(j + 1) * (s->tr_m + 1)];
            row[0] = (float)(c.ay + (j + 0.5) * dely);
            for (int i = 0; i < s->tr_m; i++) {
                const double *q = &tr[(size_t)6 * (j * s->tr_m + i)];
                const double xx = q[2], xw = xx - std::floor((xx - c.ax) * ilx) * c.lx, yy = q[3],
                             yw = yy - std::floor((yy - c.ay) * ily) * c.ly;
                double v;
                if (!ct_bicubic(s, h, 6, xw, yw, &v)) return fail(STZG_EINVAL, "a tracer left the interpolation grid");
                row[i + 1] = (float)(v * s->P.TZ);
            }
        }
        STZG_CHECK(ct_write_floats(dir, "teml", k, mat));
    }
    return STZG_OK;
}

}  // namespace

extern "C" {

int stzg_ct_create(const stzg_ct_params *p, int device, stzg_ct **out) {
    if (!out || !p) return fail(STZG_EINVAL, "null argument");
    *out = nullptr;
    if (p->m < 4 || p->n < 4 || (p->m & 1)) return fail(STZG_EINVAL, "grid needs m >= 4 even and n >= 4");
    if (p->stz_model < 0 || p->stz_model > 3) return fail(STZG_EINVAL, "unknown STZ law");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(STZG_ENODEV, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(STZG_EINVAL, "device ordinal out of range");
    STZG_CUDA(cudaSetDevice(device));
    stzg_ct *s = new stzg_ct;
    s->P = *p;
    s->device = device;
    auto bail = [&](int st) {
        stzg_ct_destroy(s);
        return st;
    };
    ct_consts &c = s->c;
    c.m = p->m;
    c.n = p->n;
    c.gm = p->m + 4;
    c.yp = p->y_prd ? 1 : 0;
    c.lsn = c.yp ? p->n : p->n + 1;
    c.ax = p->ax;
    c.ay = p->ay;
    c.bx = p->bx;
    c.by = p->by;
    c.lx = p->bx - p->ax;
    c.ly = p->by - p->ay;
    c.dx = c.lx / p->m;
    c.dy = c.ly / p->n;
    c.xsp = 1. / c.dx;
    c.ysp = 1. / c.dy;
    c.mu = p->mu;
    c.mu_inv = 1. / p->mu;
    c.K = p->K;
    c.chi_len = p->chi_len;
    c.lamb = p->lamb;
    c.u_bdry = p->u_bdry;
    stz_law_params<double> &L = c.law;
    L.stz_model = p->stz_model;
    L.t_model = p->t_model;
    L.substep_cap = 1 << 22;
    L.t_scale = p->t_scale;
    L.adapt_fac = p->adapt_fac;
    L.theta = p->theta;
    L.Delta = p->Delta;
    L.tau0 = p->tau0;
    L.kappa = p->kappa;
    L.rho = p->rho;
    L.mu = p->mu;
    L.c0 = p->c0;
    L.Omegaeps0 = p->Omegaeps0;
    L.chi_inf = p->chi_inf;
    L.s_y = 1;  // s0 of this variant's stz_dynamics (stz_model.hh:20)
    if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess)
        return bail(fail(STZG_ECUDA, "stream/event creation failed"));
    const size_t pts = (size_t)(p->m + 4) * (p->n + 4);
    int st;
    for (int b = 0; b < 2; b++)
        for (int f = 0; f < CF; f++)
            if ((st = ct_alloc(s, &s->F.f[b][f], pts)) != STZG_OK) return bail(st);
    if ((st = ct_alloc(s, &s->F.ddev, pts)) != STZG_OK) return bail(st);
    // the block multigrid on the m x lsn nodes; wall rows carry the identity
    s->cls.assign((size_t)p->m * c.lsn, 0);
    if (!c.yp)
        for (int i = 0; i < p->m; i++) s->cls[i] = s->cls[(size_t)p->n * p->m + i] = 1;
    m22 pre;
    operator_for(s, 0.0, pre);
    const double a = DBL_EPSILON * 1e4 * 2.;  // acc = tgmg_accuracy(2., 1e4), qs_multi.cc:11
    if ((st = stzg_tgmg_create_block(p->m, c.lsn, 1, c.yp, 2, s->table.data(), 2, s->cls.data(), a * a, device,
                                     &s->mg)) != STZG_OK)
        return bail(st);
    stzg_tgmg_predict_init(&s->tp);
    double *b, *z;
    if ((st = stzg_tgmg_device_arrays(s->mg, &b, &z)) != STZG_OK) return bail(st);
    s->mg_b = (double2 *)b;
    s->mg_z = (double2 *)z;
    if (cudaStreamSynchronize(s->st) != cudaSuccess) return bail(fail(STZG_ECUDA, "setup failed"));
    *out = s;
    return STZG_OK;
}

int stzg_ct_destroy(stzg_ct *s) {
    if (!s) return STZG_OK;
    cudaSetDevice(s->device);
    if (s->st) cudaStreamSynchronize(s->st);
    if (s->mg) stzg_tgmg_destroy(s->mg);
    for (void *p : s->owned) cudaFree(p);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
    return STZG_OK;
}

int stzg_ct_init_fields(stzg_ct *s, int chi_case, double tem_base, double tem_delta) {
    if (!s || chi_case < 0 || chi_case > 2) return fail(STZG_EINVAL, "bad arguments");
    STZG_CUDA(cudaSetDevice(s->device));
    const ct_consts &c = s->c;
    const stzg_ct_params &P = s->P;
    const double chi0 = tem_base / P.TZ, chi1 = tem_delta / P.TZ;
    double sx[16], sy[16];
    if (chi_case == 2)
        for (int i = 0; i < 16; i++) {
            sx[i] = c.ax + c.lx * (i + 0.5) * 0.0625;
            sy[i] = 0.2 * sin(M_PI * 0.0625 * (2 * i + 1));
        }
    const size_t pts = (size_t)c.gm * (c.n + 4);
    std::vector<double> h[CF];
    for (int f = 0; f < CF; f++) h[f].assign(pts, 0.0);
    // shear_sim::init_fields (shear_sim.cc:59-131)
    for (int j = 0; j < (c.yp ? c.n : c.n + 1); j++) {
        const double Y = c.ay + j * c.dy, Ys = Y + 0.5 * c.dy;
        for (int i = 0; i < c.m; i++) {
            const size_t k = (size_t)(j + 2) * c.gm + (i + 2);
            const double X = c.ax + i * c.dx, Xs = X + 0.5 * c.dx;
            h[CU][k] = Y * c.u_bdry;
            h[CV][k] = 0;
            double chi;
            if (chi_case == 0) {
                chi = chi0 + chi1 * exp(-200 * (Xs * Xs + Ys * Ys));
            } else if (chi_case == 1) {
                const double csa = cos(30 * M_PI / 180.), sia = sin(30 * M_PI / 180.);
                double Xr = csa * Xs + sia * Ys, Yr = -sia * Xs + csa * Ys;
                Xr = (Xr < -1) ? Xr + 1 : ((Xr > 1) ? Xr - 1 : 0);
                chi = chi0 + chi1 * exp(-200 * (Xr * Xr + Yr * Yr));
            } else {
                double R = 1e100, Rt, Xr, Yr;
                for (int q = 0; q < 16; q++) {
                    Xr = sx[q] - Xs;
                    if (Xr < -c.lx * 0.5) Xr += c.lx;
                    if (Xr > c.lx * 0.5) Xr -= c.lx;
                    Yr = sy[q] - Ys;
                    Rt = Xr * Xr + Yr * Yr;
                    if (Rt < R) R = Rt;
                }
                chi = chi0 + chi1 * exp(-200 * R);
            }
            h[CCHI][k] = chi;
            h[CX][k] = X;
            h[CY][k] = Y;
        }
    }
    for (int f = 0; f < CF; f++)
        STZG_CUDA(cudaMemcpyAsync(s->F.f[s->cur][f], h[f].data(), pts * sizeof(double), cudaMemcpyHostToDevice,
                                  s->st));
    boundaries(s, s->cur);
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

// shear_sim::initialize_chi_bicubic of the variant
// (coord_transforms/simple_shear/shear_sim.cc:1067-1134): chi of the cells
// (rows 0..n-1) = lo + sca times the bicubic Hermite interpolant of arr
// (mm x nn, periodic in x, and in y when y is periodic), derivatives by
// centred differences; with walls the first and last sample rows use the
// row itself as the missing neighbour with the factor 1/2 of the centred
// difference, as the reference's expression gives (its factor 1 applies only
// where j == 0 and j == mm-1 together).  Then set_boundaries.  The other
// fields are left as they are.
int stzg_ct_chi_bicubic(stzg_ct *s, int mm, int nn, const double *arr, double lo, double sca) {
    if (!s || !arr || mm < 1 || nn < 2) return fail(STZG_EINVAL, "bad arguments");
    STZG_CUDA(cudaSetDevice(s->device));
    const ct_consts &c = s->c;
    const bool yp = c.yp != 0;
    const long mn = (long)mm * nn;
    std::vector<double> ax(mn), ay(mn), axy(mn);
    for (int j = 0; j < nn; j++)
        for (int i = 0; i < mm; i++) {
            const long r = (long)j * mm;
            ax[r + i] = 0.5 * (arr[r + (i == mm - 1 ? 0 : i + 1)] - arr[r + (i == 0 ? mm - 1 : i - 1)]);
        }
    for (int j = 0; j < nn; j++) {
        const long r = (long)j * mm;
        const long rd = j == 0 ? (yp ? r + (mn - mm) : r) : r - mm;
        const long ru = j == nn - 1 ? (yp ? r + (mm - mn) : r) : r + mm;
        const double fac = (!yp && j == 0 && j == mm - 1) ? 1. : 0.5;
        for (int i = 0; i < mm; i++) {
            ay[r + i] = fac * (arr[ru + i] - arr[rd + i]);
            axy[r + i] = fac * (ax[ru + i] - ax[rd + i]);
        }
    }
    const double xs = c.dx * mm / c.lx, ys = c.dy * nn / c.ly;
    std::vector<double> chi((size_t)c.m * c.n);
    for (int j = 0; j < c.n; j++) {
        double t = (j + 0.5) * ys - 0.5;
        int hi;
        if (yp) {
            if (t < 0) t += nn;
            hi = nn - 1;
        } else {
            hi = nn - 2;
        }
        int jj = (int)t;
        jj = jj < 0 ? 0 : (jj > hi ? hi : jj);
        const long up = jj == nn - 1 ? mm - mn : mm;  // offset of the next sample row
        t -= jj;
        const double u = 1. - t;
        const double w0 = t * u * u, w1 = u * u * (1 + 2 * t), w2 = t * t * (3 - 2 * t), w3 = -t * t * u;
        for (int i = 0; i < c.m; i++) {
            double x = (i + 0.5) * xs - 0.5;
            if (x < 0) x += mm;
            int ii = (int)x;
            if (ii >= mm) ii -= mm;
            const long a = ii + (long)mm * jj, b = (ii == mm - 1 ? ii - mm : ii) + 1 + (long)mm * jj;
            x -= ii;
            const double v = 1 - x;
            const double h0 = x * v * v, h1 = v * v * (1 + 2 * x), h2 = x * x * (3 - 2 * x), h3 = -x * x * v;
            const double r0 = axy[a] * h0 + ay[a] * h1 + ay[b] * h2 + axy[b] * h3;
            const double r1 = ax[a] * h0 + arr[a] * h1 + arr[b] * h2 + ax[b] * h3;
            const double r2 = ax[a + up] * h0 + arr[a + up] * h1 + arr[b + up] * h2 + ax[b + up] * h3;
            const double r3 = axy[a + up] * h0 + ay[a + up] * h1 + ay[b + up] * h2 + axy[b + up] * h3;
            chi[(size_t)j * c.m + i] = lo + sca * (w0 * r0 + w1 * r1 + w2 * r2 + w3 * r3);
        }
    }
    double *d = s->F.f[s->cur][CCHI];
    STZG_CUDA(cudaMemcpy2DAsync(d + 2 * c.gm + 2, c.gm * sizeof(double), chi.data(), c.m * sizeof(double),
                                c.m * sizeof(double), c.n, cudaMemcpyHostToDevice, s->st));
    boundaries(s, s->cur);
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

static double *ct_field_ptr(stzg_ct *s, int field) {
    return field == STZG_CT_DDEV ? s->F.ddev : s->F.f[s->cur][field];
}

int stzg_ct_set_field(stzg_ct *s, int field, const double *host) {
    if (!s || !host || field < 0 || field >= STZG_CT_FIELDS) return fail(STZG_EINVAL, "bad arguments");
    STZG_CUDA(cudaSetDevice(s->device));
    const ct_consts &c = s->c;
    double *d = ct_field_ptr(s, field);
    STZG_CUDA(cudaMemcpy2DAsync(d + 2 * c.gm + 2, c.gm * sizeof(double), host, c.m * sizeof(double),
                                c.m * sizeof(double), c.n + 1, cudaMemcpyHostToDevice, s->st));
    if (field != STZG_CT_DDEV) boundaries(s, s->cur);
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

int stzg_ct_get_field(stzg_ct *s, int field, double *host) {
    if (!s || !host || field < 0 || field >= STZG_CT_FIELDS) return fail(STZG_EINVAL, "bad arguments");
    STZG_CUDA(cudaSetDevice(s->device));
    const ct_consts &c = s->c;
    const double *d = ct_field_ptr(s, field);
    STZG_CUDA(cudaMemcpy2DAsync(host, c.m * sizeof(double), d + 2 * c.gm + 2, c.gm * sizeof(double),
                                c.m * sizeof(double), c.n + 1, cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

int stzg_ct_set_time(stzg_ct *s, double time) {
    if (!s) return fail(STZG_EINVAL, "null handle");
    s->time = time;
    return STZG_OK;
}

int stzg_ct_set_solve_policy(stzg_ct *s, int policy) {
    if (!s) return fail(STZG_EINVAL, "null handle");
    if (policy != 0 && policy != 1) return fail(STZG_EINVAL, "policy must be 0 (predictor) or 1 (checked)");
    s->checked = policy;
    return STZG_OK;
}

int stzg_ct_set_precision(stzg_ct *s, int precision) {
    if (!s) return fail(STZG_EINVAL, "null handle");
    STZG_CUDA(cudaSetDevice(s->device));
    return stzg_tgmg_set_precision(s->mg, precision);
}

int stzg_ct_get_time(stzg_ct *s, double *time) {
    if (!s || !time) return fail(STZG_EINVAL, "null argument");
    *time = s->time;
    return STZG_OK;
}

int stzg_ct_step_direct(stzg_ct *s, double dt, int nsteps, double *seconds) {
    if (!s || !(dt > 0) || nsteps < 0) return fail(STZG_EINVAL, "bad arguments");
    STZG_CUDA(cudaSetDevice(s->device));
    STZG_CUDA(cudaEventRecord(s->ev0, s->st));
    for (int k = 0; k < nsteps; k++) STZG_CHECK(direct_step(s, dt));
    STZG_CUDA(cudaEventRecord(s->ev1, s->st));
    STZG_CUDA(cudaEventSynchronize(s->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    if (seconds) *seconds = ms * 1e-3;
    STZG_CUDA(cudaGetLastError());
    return STZG_OK;
}

int stzg_ct_tracers_init(stzg_ct *s, int mm, int nn) {
    if (!s || mm < 1 || nn < 1 || (long)mm * nn > (1L << 26)) return fail(STZG_EINVAL, "bad tracer grid");
    STZG_CUDA(cudaSetDevice(s->device));
    const int cnt = mm * nn;
    if (cnt > s->tr_cap) {
        void *a, *b;
        STZG_CUDA(cudaMalloc(&a, sizeof(double) * 6 * (size_t)cnt));
        if (cudaMalloc(&b, sizeof(int) * (size_t)cnt) != cudaSuccess) {
            cudaFree(a);
            return fail(STZG_ENOMEM, "cudaMalloc(tracers)");
        }
        s->owned.push_back(a);
        s->owned.push_back(b);
        s->tr = (double *)a;
        s->tr_ok = (int *)b;
        s->tr_cap = cnt;
    }
    // a regular grid of cell-centred points, at rest (shear_sim.cc:1265-1281)
    std::vector<double> h((size_t)6 * cnt);
    const double dxx = (s->P.bx - s->P.ax) / mm, dyy = (s->P.by - s->P.ay) / nn;
    double *q = h.data();
    for (int j = 0; j < nn; j++) {
        const double yy = s->P.ay + dyy * (j + 0.5);
        for (int i = 0; i < mm; i++) {
            const double xx = s->P.ax + dxx * (i + 0.5);
            *q++ = xx;
            *q++ = yy;
            *q++ = xx;
            *q++ = yy;
            *q++ = 0;
            *q++ = 0;
        }
    }
    STZG_CUDA(cudaMemcpyAsync(s->tr, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    s->ntrace = cnt;
    s->tr_m = mm;
    s->tr_n = nn;
    s->tr_time = s->time;
    return STZG_OK;
}

int stzg_ct_tracers_update(stzg_ct *s, int *lost) {
    if (!s) return fail(STZG_EINVAL, "null handle");
    if (!s->tr) return fail(STZG_EINVAL, "no tracers: call stzg_ct_tracers_init first");
    STZG_CUDA(cudaSetDevice(s->device));
    if (lost) *lost = 0;
    if (s->ntrace == 0) return STZG_OK;
    // dt runs from the tracers' creation, as in the reference (tr_time is
    // not advanced by update_tracers)
    const double dt = s->time - s->tr_time, dtinv = 1 / dt;
    const int n = s->ntrace;
    k_ct_tracers<<<ceil_div(n, 128), 128, 0, s->st>>>(s->c, s->F.f[s->cur][CX], s->F.f[s->cur][CY], s->tr, s->tr_ok,
                                                       n, dt, dtinv);
    STZG_CUDA(cudaGetLastError());
    std::vector<int> ok(n);
    STZG_CUDA(cudaMemcpyAsync(ok.data(), s->tr_ok, sizeof(int) * n, cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    int dropped = 0;
    for (int t = 0; t < n; t++) {
        if (ok[t] < 0) return fail(STZG_EINVAL, "a tracer left the interpolation grid");
        dropped += ok[t] == 0;
    }
    if (dropped) {
        // the reference moves the last tracer into a dropped one's slot and
        // processes it there next (shear_sim.cc:1303-1313)
        std::vector<double> h((size_t)6 * n), g;
        STZG_CUDA(cudaMemcpy(h.data(), s->tr, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
        std::vector<int> perm(n);
        for (int t = 0; t < n; t++) perm[t] = t;
        int i = 0, e = n;
        while (i < e) {
            if (ok[perm[i]]) i++;
            else perm[i] = perm[--e];
        }
        g.resize((size_t)6 * e);
        for (int t = 0; t < e; t++) std::memcpy(&g[(size_t)6 * t], &h[(size_t)6 * perm[t]], 6 * sizeof(double));
        if (e) STZG_CUDA(cudaMemcpy(s->tr, g.data(), sizeof(double) * g.size(), cudaMemcpyHostToDevice));
        s->ntrace = e;
    }
    if (lost) *lost = dropped;
    return STZG_OK;
}

int stzg_ct_tracers_get(stzg_ct *s, double *out, int cap, int *count) {
    if (!s || !count) return fail(STZG_EINVAL, "null argument");
    *count = s->ntrace;
    if (!out || s->ntrace == 0) return STZG_OK;
    STZG_CUDA(cudaSetDevice(s->device));
    const int k = cap < s->ntrace ? cap : s->ntrace;
    if (k > 0) STZG_CUDA(cudaMemcpy(out, s->tr, sizeof(double) * 6 * (size_t)k, cudaMemcpyDeviceToHost));
    return STZG_OK;
}

int stzg_ct_step_qs(stzg_ct *s, double dt, int nsteps, long *vcycles, double *seconds) {
    if (!s || !(dt > 0) || nsteps < 0) return fail(STZG_EINVAL, "bad arguments");
    STZG_CUDA(cudaSetDevice(s->device));
    if (vcycles) *vcycles = 0;
    STZG_CUDA(cudaEventRecord(s->ev0, s->st));
    for (int k = 0; k < nsteps; k++) {
        STZG_CHECK(advection_step(s, dt));
        STZG_CHECK(projection_step(s, dt, vcycles));
    }
    STZG_CUDA(cudaEventRecord(s->ev1, s->st));
    STZG_CUDA(cudaEventSynchronize(s->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    if (seconds) *seconds = 1e-3 * ms;
    STZG_CUDA(cudaGetLastError());
    return STZG_OK;
}

int stzg_ct_batch_step_qs(stzg_ct *const *handles, int count, double dt, int nsteps, int threads, long *vcycles,
                          double *seconds) {
    if (!handles || count < 1 || !(dt > 0) || nsteps < 0 || threads < 0) return fail(STZG_EINVAL, "bad arguments");
    for (int k = 0; k < count; k++)
        if (!handles[k]) return fail(STZG_EINVAL, "null handle");
    const int nt = threads > 0 ? std::min(threads, count) : std::min(count, 16);
    std::atomic<int> next(0), first_bad(count);
    std::vector<int> status(count, STZG_OK);
    std::vector<std::string> msg(count);
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&]() {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= count || first_bad.load() < count) return;
            long vc = 0;
            const int st = stzg_ct_step_qs(handles[k], dt, nsteps, &vc, nullptr);
            if (vcycles) vcycles[k] = vc;
            if (st != STZG_OK) {
                status[k] = st;
                msg[k] = stzg_last_message();
                int cur = first_bad.load();
                while (k < cur && !first_bad.compare_exchange_weak(cur, k)) {
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const int bad = first_bad.load();
    if (bad < count) return fail(status[bad], "handle " + std::to_string(bad) + ": " + msg[bad]);
    return STZG_OK;
}

int stzg_ct_compute_strain(stzg_ct *s, double *out) {
    if (!s || !out) return fail(STZG_EINVAL, "null argument");
    STZG_CUDA(cudaSetDevice(s->device));
    ct_host h;
    STZG_CHECK(ct_fetch(s, h));
    ct_strain(s, h, s->c.lamb * s->time);
    const int m = h.m, n = h.n;
    for (int q = 0; q < 6; q++)
        for (int j = 0; j <= n; j++)
            for (int i = 0; i < m; i++) out[((size_t)q * (n + 1) + j) * m + i] = h.f[CF + q][h.at(i, j)];
    return STZG_OK;
}

int stzg_ct_output_field(stzg_ct *s, int mode, float *out, long *count) {
    if (!s || mode < 0 || mode > 16) return fail(STZG_EINVAL, "bad arguments");
    STZG_CUDA(cudaSetDevice(s->device));
    ct_host h;
    STZG_CHECK(ct_fetch(s, h));
    if (mode >= 11) ct_strain(s, h, s->c.lamb * s->time);
    std::vector<float> buf;
    ct_output(s, h, mode, buf);
    if (count) *count = (long)buf.size();
    if (out) std::memcpy(out, buf.data(), buf.size() * sizeof(float));
    return STZG_OK;
}

int stzg_ct_write_frame(stzg_ct *s, const char *dir, int frame, unsigned fflags) {
    if (!s || !dir) return fail(STZG_EINVAL, "null argument");
    STZG_CUDA(cudaSetDevice(s->device));
    return ct_write_files(s, dir, frame, fflags);
}

int stzg_ct_solve_quasistatic(stzg_ct *s, double duration, int frames, int steps, const char *dir,
                              unsigned fflags, int verbose) {
    if (!s || !dir || frames < 1 || steps < 1 || !(duration > 0)) return fail(STZG_EINVAL, "bad arguments");
    const double time_interval = duration / frames, isteps = 1.0 / steps;
    if (s->f_num == 0) {
        STZG_CHECK(ct_write_files(s, dir, 0, fflags));
        if (verbose) std::puts("# Output frame 0");
    }
    long vc = 0, solves = 0;
    for (int k = 1; k <= frames; k++) {
        long v = 0;
        STZG_CHECK(stzg_ct_step_qs(s, time_interval * isteps, steps, &v, nullptr));
        vc += v;
        solves += steps;
        STZG_CHECK(ct_write_files(s, dir, k, fflags));
        if (verbose) std::printf("# Output frame %d [%d] {%.2f}\n", k, steps, solves ? (double)vc / solves : 0.0);
    }
    s->f_num += frames;
    return STZG_OK;
}

int stzg_ct_solve(stzg_ct *s, double duration, int frames, const char *dir, unsigned fflags, int verbose) {
    if (!s || !dir || frames < 1 || !(duration > 0)) return fail(STZG_EINVAL, "bad arguments");
    const ct_consts &c = s->c;
    // the explicit steps: below both the elastic-wave and the viscous limit
    const double time_interval = duration / frames, cfl = 0.25 * c.dx,
                 visc_cond = 0.25 * c.dx * c.dx / s->P.viscosity, dt = cfl < visc_cond ? cfl : visc_cond;
    const int l = (int)(time_interval / dt) + 1;
    const double adt = time_interval / l;
    if (verbose) {
        std::printf("CFL: %g\n", dt / c.dx);
        std::printf("Viscosity Condition: %g\n", s->P.viscosity * dt * (1. / (c.xsp * c.xsp + c.ysp * c.ysp)));
    }
    STZG_CHECK(ct_write_files(s, dir, 0, fflags));
    if (verbose) std::puts("# Output frame 0");
    for (int k = 1; k <= frames; k++) {
        STZG_CHECK(stzg_ct_step_direct(s, adt, l, nullptr));
        STZG_CHECK(ct_write_files(s, dir, k, fflags));
        if (verbose) std::printf("# Output frame %d [%d]\n", k, l);
    }
    return STZG_OK;
}


// shear_sim::l2_comparison_transform (shear_sim.cc:619-711): s runs in the
// sheared frame, phys in the physical frame (lamb = 0) on the same grid; the
// physical run's fields are interpolated bilinearly (bilin_interp,
// shear_sim.cc:713-736) at the sheared position i + lt xsp y_j of each node,
// and the squared differences are summed with the reference's weights
// (stresses 2 tau^2 + 2 s^2 + 3 p^2 + 6 q^2 on the cell rows, velocity and
// reference map over the node rows with the trapezoidal halves on rows 0 and
// n), times dx dy.  The reference reads past its grid where the shift passes
// the ghost columns; that is an error here.  Its extra line starts at
// fm + gmn, past the whole allocation (gmn = gm*gn); row n is summed here.
int stzg_ct_l2_comparison_transform(stzg_ct *s, stzg_ct *phys, double *l2) {
    if (!s || !phys || !l2) return fail(STZG_EINVAL, "null argument");
    if (s->c.m != phys->c.m || s->c.n != phys->c.n) return fail(STZG_EINVAL, "grids differ");
    STZG_CUDA(cudaSetDevice(s->device));
    ct_host a, b;
    STZG_CHECK(ct_fetch(s, a));
    STZG_CUDA(cudaSetDevice(phys->device));
    STZG_CHECK(ct_fetch(phys, b));
    const ct_consts &c = s->c;
    const int m = c.m, n = c.n;
    const double lt = c.lamb * s->time;
    bool bad = false;
    // bilinear values of u, v, p, q, s, tau, chi of b at (ii, jj)
    auto interp = [&](double ii, double jj, double *r) {
        const int left = (int)ii, down = (int)jj, right = left + 1, up = down + 1;
        if (left < -2 || right > m + 1 || down < -2 || up > n + 1) {
            bad = true;
            for (int k = 0; k < 7; k++) r[k] = 0;
            return;
        }
        const size_t dl = b.at(left, down), dr = dl + 1, ul = dl + b.gm, ur = dr + b.gm;
        const double f = right - ii, g = ii - left;
        for (int k = 0; k < 7; k++) {
            const double *F = b.f[k].data();
            r[k] = (up - jj) * (f * F[dl] + g * F[dr]) + (jj - down) * (f * F[ul] + g * F[ur]);
        }
    };
    double t0 = 0, t1 = 0, t2 = 0, t3 = 0, iv[7];
    for (int j = 0; j < n; j++) {
        double c0 = 0, c1 = 0, c2 = 0, c3 = 0;
        for (int i = 0; i < m; i++) {
            const double i_phys = i + lt * c.xsp * (c.ay + j * c.dy);
            interp(i_phys, (double)j, iv);
            const size_t k = a.at(i, j);
            const double du = a.f[CU][k] - iv[0], dv = a.f[CV][k] - iv[1], dp = a.f[CP][k] - iv[2],
                         dq = a.f[CQ][k] - iv[3], ds = a.f[CS][k] - iv[4], dtau = a.f[CTAU][k] - iv[5],
                         dchi = a.f[CCHI][k] - iv[6], dX = a.f[CX][k] - b.f[CX][k], dY = a.f[CY][k] - b.f[CY][k];
            c0 += du * du + dv * dv;
            c1 += dtau * dtau + ds * ds + 3 * dp * dp + 6 * dq * dq;
            c2 += dchi * dchi;
            c3 += dX * dX + dY * dY;
        }
        if (j == 0) {
            c0 *= 0.5;
            c3 *= 0.5;
        }
        t0 += c0;
        t1 += c1;
        t2 += c2;
        t3 += c3;
    }
    for (int i = 0; i < m; i++) {
        const double i_phys = i + lt * c.xsp * (c.ay + n * c.dy);
        interp(i_phys, (double)n, iv);
        const size_t k = a.at(i, n);
        const double du = a.f[CU][k] - iv[0], dv = a.f[CV][k] - iv[1], dX = a.f[CX][k] - b.f[CX][k],
                     dY = a.f[CY][k] - b.f[CY][k];
        t0 += 0.5 * (du * du + dv * dv);
        t3 += 0.5 * (dX * dX + dY * dY);
    }
    if (bad) return fail(STZG_EINVAL, "the sheared position leaves the ghosted grid");
    const double fac = c.dx * c.dy;
    l2[0] = t0 * fac;
    l2[1] = t1 * fac;
    l2[2] = t2 * fac;
    l2[3] = t3 * fac;
    return STZG_OK;
}

}  // extern "C"
