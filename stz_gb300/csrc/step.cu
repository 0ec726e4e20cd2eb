// Time-step kernels: fused ENO advection + STZ plasticity, chi diffusion,
// projection source, stress correction and boundaries.
#include "step.cuh"
#include "stz_law.cuh"

namespace stzg {

step_consts make_step_consts(const stz_params &p) {
    step_consts c;
    c.m = p.m;
    c.n = p.n;
    c.ax = p.ax;
    c.ay = p.ay;
    c.by = p.by;
    c.lx = p.bx - p.ax;
    c.dx = c.lx / p.m;
    c.dy = (p.by - p.ay) / p.n;
    c.xsp = 1. / c.dx;
    c.ysp = 1. / c.dy;
    c.mu = p.mu;
    c.K = p.K;
    c.stz_model = p.stz_model;
    c.t_model = p.t_model;
    c.t_scale = p.t_scale;
    c.adapt_fac = p.adapt_fac;
    c.chi_inf = p.chi_inf;
    c.s_y = p.s_y;
    c.theta = p.theta;
    c.Delta = p.Delta;
    c.Omegaeps0 = p.Omegaeps0;
    c.tau0 = p.tau0;
    c.c0 = p.c0;
    c.kappa = p.kappa;
    c.rho = p.rho;
    c.chi_diff = p.chi_diff;
    c.chi_len = p.chi_len;
    c.track_plastic = 0;
    c.substep_cap = 1 << 22;
    c.yield_cut2 = p.s_y * p.s_y * (1 - 1e-12);
    c.clock = nullptr;
    c.xbc = 0;
    return c;
}

namespace {

struct velo {
    const double2 *vel;
    int m, n;
    double bv;
    __device__ __forceinline__ double u(int i, int j) const {
        return j == 0 ? -bv : (j == n ? bv : vel[(size_t)j * m + i].x);
    }
    __device__ __forceinline__ double v(int i, int j) const {
        return (j == 0 || j == n) ? 0.0 : vel[(size_t)j * m + i].y;
    }
};

#define IDX(i, j) ((size_t)((j) + 1) * m + (i))

// Fused advection + STZ step per cell (i,j) and its lower-left node.
__global__ void __launch_bounds__(256) k_advect(step_consts c, fields_dev F, int cur, double dt, double bv,
                                                int emit_source) {
    const int m = c.m, n = c.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j >= n) return;
    if (c.clock) cur = (int)c.clock[CLK_CUR];
    const double *__restrict__ const *A = F.f[cur];
    double *const *B = F.f[cur ^ 1];
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt, lx = c.lx;
    const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
    const int il2 = i <= 1 ? i + m - 2 : i - 2, ir2 = i >= m - 2 ? i + 2 - m : i + 2;
    const size_t ci = IDX(i, j);
    if (c.clock) bv = c.clock[CLK_BV_STATE];
    velo V{F.vel, m, n, bv};
    // Upwind ENO values without the factor hs = +-dt/(2 dx); it is folded
    // into the velocity: -u * (hs * eno) = -(u * hs) * eno.
    // reference map at node (i,j), rows 1..n-1 (shear_sim.cc:310-327)
    if (j > 0) {
        const double *X = A[F_X], *Y = A[F_Y];
        double ex_X, ex_Y, ey_X, ey_Y;
        const double un = V.u(i, j), vn = V.v(i, j);
        const double uh = un * (un > 0 ? hx : -hx), vh = vn * (vn > 0 ? hy : -hy);
        if (un > 0) {
            ex_X = eno2(X[IDX(ir, j)] + (i == m - 1 ? lx : 0), X[ci], X[IDX(il, j)] + (i == 0 ? -lx : 0),
                        X[IDX(il2, j)] + (i <= 1 ? -lx : 0));
            ex_Y = eno2(Y[IDX(ir, j)], Y[ci], Y[IDX(il, j)], Y[IDX(il2, j)]);
        } else {
            ex_X = eno2(X[IDX(il, j)] + (i == 0 ? -lx : 0), X[ci], X[IDX(ir, j)] + (i == m - 1 ? lx : 0),
                        X[IDX(ir2, j)] + (i >= m - 2 ? lx : 0));
            ex_Y = eno2(Y[IDX(il, j)], Y[ci], Y[IDX(ir, j)], Y[IDX(ir2, j)]);
        }
        if (vn > 0) {
            if (j > 1) {
                ey_X = eno2(X[IDX(i, j + 1)], X[ci], X[IDX(i, j - 1)], X[IDX(i, j - 2)]);
                ey_Y = eno2(Y[IDX(i, j + 1)], Y[ci], Y[IDX(i, j - 1)], Y[IDX(i, j - 2)]);
            } else {
                ey_X = 2 * (X[ci] - X[IDX(i, j - 1)]);
                ey_Y = 2 * (Y[ci] - Y[IDX(i, j - 1)]);
            }
        } else {
            if (j < n - 1) {
                ey_X = eno2(X[IDX(i, j - 1)], X[ci], X[IDX(i, j + 1)], X[IDX(i, j + 2)]);
                ey_Y = eno2(Y[IDX(i, j - 1)], Y[ci], Y[IDX(i, j + 1)], Y[IDX(i, j + 2)]);
            } else {
                ey_X = 2 * (X[ci] - X[IDX(i, j + 1)]);
                ey_Y = 2 * (Y[ci] - Y[IDX(i, j + 1)]);
            }
        }
        B[F_X][ci] = X[ci] + fma(-vh, ey_X, -uh * ex_X);
        B[F_Y][ci] = Y[ci] + fma(-vh, ey_Y, -uh * ex_Y);
    }
    // staggered velocity and spin (shear_sim.cc:330-333)
    const double u00 = V.u(i, j), u10 = V.u(ir, j), u01 = V.u(i, j + 1), u11 = V.u(ir, j + 1);
    const double v00 = V.v(i, j), v10 = V.v(ir, j), v01 = V.v(i, j + 1), v11 = V.v(ir, j + 1);
    const double uc = 0.25 * (u00 + u10 + u01 + u11), vc = 0.25 * (v00 + v10 + v01 + v11);
    const double two_omega = hx * (-v00 + v10 - v01 + v11) - hy * (-u00 - u10 + u01 + u11);
    const double uh = uc * (uc > 0 ? hx : -hx), vh = vc * (vc > 0 ? hy : -hy);
    // ENO derivatives of p, q, s, tau, chi (shear_sim.cc:336-338)
    double f1[5], f2[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const double *G = A[k];
        if (uc > 0) f1[k] = eno2(G[IDX(ir, j)], G[ci], G[IDX(il, j)], G[IDX(il2, j)]);
        else f1[k] = eno2(G[IDX(il, j)], G[ci], G[IDX(ir, j)], G[IDX(ir2, j)]);
        if (vc > 0) {
            if (j > 0) f2[k] = eno2(G[IDX(i, j + 1)], G[ci], G[IDX(i, j - 1)], G[IDX(i, j - 2)]);
            else f2[k] = 2 * (G[ci] - G[IDX(i, j - 1)]);
        } else {
            if (j < n - 1) f2[k] = eno2(G[IDX(i, j - 1)], G[ci], G[IDX(i, j + 1)], G[IDX(i, j + 2)]);
            else f2[k] = 2 * (G[ci] - G[IDX(i, j + 1)]);
        }
    }
    const double p = A[F_P][ci], q = A[F_Q][ci], s = A[F_S][ci], t = A[F_TAU][ci];
    double cchi = A[F_CHI][ci] + fma(-vh, f2[4], -uh * f1[4]), ddev, dtmp;
    const double devsq = 3 * q * q + s * s + t * t;
    // Cells far enough below the cut-offs return exactly ddev = 0 and leave
    // chi unchanged in the reference loop (sbar < 1e-12, or an athermal law
    // below yield); they skip the FP64 square root and the loop.  The margin
    // keeps the test exact under the rounding of sqrt.
    // devsq >= 0, so the cut-offs compare as integers on the bit patterns
    const bool athermal = c.stz_model >= 2;
    const long long dbits = __double_as_longlong(devsq);
    if (dbits < __double_as_longlong(0.999e-24) || (athermal && dbits < __double_as_longlong(c.yield_cut2))) {
        ddev = 0;
        dtmp = 0;
    } else {
        int iters;
        const stz_law_params<double> lp = law_params(c);
        dtmp = adaptive_plastic(lp, sqrt(devsq), cchi, ddev, dt, iters);
        if (iters >= c.substep_cap) atomicExch(&F.flags[0], 1);
        if (iters > 1) atomicMax(&F.flags[1], iters);
    }
    B[F_CHI][ci] = cchi;
    F.ddev[ci] = ddev;
    if (c.track_plastic && ddev != 0) F.eps_pl[(size_t)j * m + i] += ddev / (2 * c.mu);
    const double pn = p + fma(-vh, f2[0], -uh * f1[0]);
    // dtmp is exactly 0 outside plastic flow; the terms - dtmp * (q, s, t)
    // then add exact zeros and are skipped
    double qn, sn, tn;
    if (dtmp != 0) {
        qn = q + (fma(-vh, f2[1], -uh * f1[1]) - dtmp * q);
        sn = s + (fma(-vh, f2[2], -uh * f1[2]) + two_omega * t - dtmp * s);
        tn = t + (fma(-vh, f2[3], -uh * f1[3]) - two_omega * s - dtmp * t);
    } else {
        qn = q + fma(-vh, f2[1], -uh * f1[1]);
        sn = s + (fma(-vh, f2[2], -uh * f1[2]) + two_omega * t);
        tn = t + (fma(-vh, f2[3], -uh * f1[3]) - two_omega * s);
    }
    B[F_P][ci] = pn;
    B[F_Q][ci] = qn;
    B[F_S][ci] = sn;
    B[F_TAU][ci] = tn;
    if (emit_source) {
        const double xf = 0.5 / dt * c.xsp, yf = 0.5 / dt * c.ysp;
        const double pq = pn + qn, Aa = pq - sn, Bb = pq + sn;
        F.pre[0][ci] = xf * Aa + yf * tn;
        F.pre[1][ci] = xf * Aa - yf * tn;
        F.pre[2][ci] = xf * tn - yf * Bb;
        F.pre[3][ci] = xf * tn + yf * Bb;
    }
}

// Explicit step (shear_sim::step_forward, shear_sim.cc:185-276) per cell
// (i,j) and its lower-left node: the node velocity and reference map are
// advected with ENO2 and the velocity takes the net force of the old stress
// (net_force with prefactors -hx,-hy, shear_sim.cc:447-453) and a 5-point
// viscous term, divided by mu as the reference's mu_inv; the cell fields are
// advected and take the elastic rate of the old velocity gradient and the
// plastic term.  The constant chi diffusion enters cchi before the plastic
// term (and again in k_chi_diffusion, as the reference adds it twice); ddev
// is stored times the old |s| (shear_sim.cc:265).  New node velocities go to
// F.src (rows 1..n-1), the other fields to buffer cur^1.
struct direct_consts {
    double hxxv, hyyv, hcv, hxxcd, hyycd, hccd;
};

__global__ void __launch_bounds__(256) k_direct(step_consts c, direct_consts d, fields_dev F, int cur, double dt,
                                                double bv) {
    const int m = c.m, n = c.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j >= n) return;
    const double *__restrict__ const *A = F.f[cur];
    double *const *B = F.f[cur ^ 1];
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt, lx = c.lx, mu_inv = 1 / c.mu;
    const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
    const int il2 = i <= 1 ? i + m - 2 : i - 2, ir2 = i >= m - 2 ? i + 2 - m : i + 2;
    const size_t ci = IDX(i, j);
    velo V{F.vel, m, n, bv};
    const double *P = A[F_P], *Q = A[F_Q], *S = A[F_S], *T = A[F_TAU];
    if (j > 0) {
        const double *X = A[F_X], *Y = A[F_Y];
        const double un = V.u(i, j), vn = V.v(i, j);
        const double hsx = un > 0 ? hx : -hx, hsy = vn > 0 ? hy : -hy;
        double ux, vx, Xx, Yx, uy, vy, Xy, Yy;
        if (un > 0) {
            ux = eno2(V.u(ir, j), un, V.u(il, j), V.u(il2, j));
            vx = eno2(V.v(ir, j), vn, V.v(il, j), V.v(il2, j));
            Xx = eno2(X[IDX(ir, j)] + (i == m - 1 ? lx : 0), X[ci], X[IDX(il, j)] + (i == 0 ? -lx : 0),
                      X[IDX(il2, j)] + (i <= 1 ? -lx : 0));
            Yx = eno2(Y[IDX(ir, j)], Y[ci], Y[IDX(il, j)], Y[IDX(il2, j)]);
        } else {
            ux = eno2(V.u(il, j), un, V.u(ir, j), V.u(ir2, j));
            vx = eno2(V.v(il, j), vn, V.v(ir, j), V.v(ir2, j));
            Xx = eno2(X[IDX(il, j)] + (i == 0 ? -lx : 0), X[ci], X[IDX(ir, j)] + (i == m - 1 ? lx : 0),
                      X[IDX(ir2, j)] + (i >= m - 2 ? lx : 0));
            Yx = eno2(Y[IDX(il, j)], Y[ci], Y[IDX(ir, j)], Y[IDX(ir2, j)]);
        }
        const int jn = vn > 0 ? j - 1 : j + 1;  // upwind neighbour row
        if ((vn > 0 && j > 1) || (vn <= 0 && j < n - 1)) {
            const int j0 = vn > 0 ? j + 1 : j - 1, j3 = vn > 0 ? j - 2 : j + 2;
            uy = eno2(V.u(i, j0), un, V.u(i, jn), V.u(i, j3));
            vy = eno2(V.v(i, j0), vn, V.v(i, jn), V.v(i, j3));
            Xy = eno2(X[IDX(i, j0)], X[ci], X[IDX(i, jn)], X[IDX(i, j3)]);
            Yy = eno2(Y[IDX(i, j0)], Y[ci], Y[IDX(i, jn)], Y[IDX(i, j3)]);
        } else {
            uy = 2 * (un - V.u(i, jn));
            vy = 2 * (vn - V.v(i, jn));
            Xy = 2 * (X[ci] - X[IDX(i, jn)]);
            Yy = 2 * (Y[ci] - Y[IDX(i, jn)]);
        }
        ux *= hsx; vx *= hsx; Xx *= hsx; Yx *= hsx;
        uy *= hsy; vy *= hsy; Xy *= hsy; Yy *= hsy;
        // net force from the cells (i-1,j-1), (i,j-1), (i-1,j), (i,j)
        const size_t c0 = IDX(il, j - 1), c1 = IDX(i, j - 1), c2 = IDX(il, j), c3 = ci;
        const double xf = -hx, yf = -hy;
        const double fx = (-P[c0] + P[c1] - P[c2] + P[c3] - Q[c0] + Q[c1] - Q[c2] + Q[c3] + S[c0] - S[c1] + S[c2] -
                           S[c3]) * xf + (T[c0] + T[c1] - T[c2] - T[c3]) * yf;
        const double fy = (T[c0] - T[c1] + T[c2] - T[c3]) * xf +
                          (-P[c0] - P[c1] + P[c2] + P[c3] - Q[c0] - Q[c1] + Q[c2] + Q[c3] - S[c0] - S[c1] + S[c2] +
                           S[c3]) * yf;
        const double uvisc = d.hxxv * (V.u(ir, j) + V.u(il, j)) + d.hyyv * (V.u(i, j + 1) + V.u(i, j - 1)) - d.hcv * un;
        const double vvisc = d.hxxv * (V.v(ir, j) + V.v(il, j)) + d.hyyv * (V.v(i, j + 1) + V.v(i, j - 1)) - d.hcv * vn;
        F.src[(size_t)j * m + i] = make_double2(un + (-un * ux - vn * uy + mu_inv * (fx + uvisc)),
                                                vn + (-un * vx - vn * vy + mu_inv * (fy + vvisc)));
        B[F_X][ci] = X[ci] + (-un * Xx - vn * Xy);
        B[F_Y][ci] = Y[ci] + (-un * Yx - vn * Yy);
    }
    // deformation rate, staggered velocity and spin
    const double u00 = V.u(i, j), u10 = V.u(ir, j), u01 = V.u(i, j + 1), u11 = V.u(ir, j + 1);
    const double v00 = V.v(i, j), v10 = V.v(ir, j), v01 = V.v(i, j + 1), v11 = V.v(ir, j + 1);
    const double uc = 0.25 * (u00 + u10 + u01 + u11), vc = 0.25 * (v00 + v10 + v01 + v11);
    const double ux = hx * (-u00 + u10 - u01 + u11), uy = hy * (-u00 - u10 + u01 + u11);
    const double vx = hx * (-v00 + v10 - v01 + v11), vy = hy * (-v00 - v10 + v01 + v11);
    const double two_omega = vx - uy;
    const double uh = uc * (uc > 0 ? hx : -hx), vh = vc * (vc > 0 ? hy : -hy);
    double f1[5], f2[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const double *G = A[k];
        if (uc > 0) f1[k] = eno2(G[IDX(ir, j)], G[ci], G[IDX(il, j)], G[IDX(il2, j)]);
        else f1[k] = eno2(G[IDX(il, j)], G[ci], G[IDX(ir, j)], G[IDX(ir2, j)]);
        if (vc > 0) {
            if (j > 0) f2[k] = eno2(G[IDX(i, j + 1)], G[ci], G[IDX(i, j - 1)], G[IDX(i, j - 2)]);
            else f2[k] = 2 * (G[ci] - G[IDX(i, j - 1)]);
        } else {
            if (j < n - 1) f2[k] = eno2(G[IDX(i, j - 1)], G[ci], G[IDX(i, j + 1)], G[IDX(i, j + 2)]);
            else f2[k] = 2 * (G[ci] - G[IDX(i, j + 1)]);
        }
    }
    const double *CH = A[F_CHI];
    const double p = P[ci], q = Q[ci], s = S[ci], t = T[ci];
    double cchi = CH[ci] + fma(-vh, f2[4], -uh * f1[4]) + d.hxxcd * (CH[IDX(ir, j)] + CH[IDX(il, j)]) +
                  d.hyycd * (CH[IDX(i, j + 1)] + CH[IDX(i, j - 1)]) - d.hccd * CH[ci];
    const double devsq = 3 * q * q + s * s + t * t;
    double ddev = 0, dtmp = 0, sbar = 0;
    const bool athermal = c.stz_model >= 2;
    if (!(devsq < 0.999e-24 || (athermal && devsq < c.yield_cut2))) {
        int iters;
        const stz_law_params<double> lp = law_params(c);
        sbar = sqrt(devsq);
        dtmp = adaptive_plastic(lp, sbar, cchi, ddev, dt, iters);
        if (iters >= c.substep_cap) atomicExch(&F.flags[0], 1);
        if (iters > 1) atomicMax(&F.flags[1], iters);
    }
    B[F_CHI][ci] = cchi;
    F.ddev[ci] = ddev * sbar;
    if (c.track_plastic && ddev != 0) F.eps_pl[(size_t)j * m + i] += ddev / (2 * c.mu);
    const double third = 1 / 3.0;
    B[F_P][ci] = p + (fma(-vh, f2[0], -uh * f1[0]) - c.K * (ux + vy));
    B[F_Q][ci] = q + (fma(-vh, f2[1], -uh * f1[1]) - c.mu * third * (ux + vy) - dtmp * q);
    B[F_S][ci] = s + (fma(-vh, f2[2], -uh * f1[2]) + two_omega * t + c.mu * (ux - vy) - dtmp * s);
    B[F_TAU][ci] = t + (fma(-vh, f2[3], -uh * f1[3]) - two_omega * s + c.mu * (vx + uy) - dtmp * t);
}

__global__ void k_precombine(step_consts c, fields_dev F, int cur, double xf, double yf) {
    const int m = c.m, n = c.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j >= n) return;
    const size_t k = IDX(i, j);
    const double pn = F.f[cur][F_P][k], qn = F.f[cur][F_Q][k], sn = F.f[cur][F_S][k], tn = F.f[cur][F_TAU][k];
    const double pq = pn + qn, Aa = pq - sn, Bb = pq + sn;
    F.pre[0][k] = xf * Aa + yf * tn;
    F.pre[1][k] = xf * Aa - yf * tn;
    F.pre[2][k] = xf * tn - yf * Bb;
    F.pre[3][k] = xf * tn + yf * Bb;
}

// chi_diffusion (shear_sim.cc:364-386): B.chi holds cchi; old chi in A.
__global__ void k_chi_diffusion(step_consts c, fields_dev F, int cur, double dt) {
    const int m = c.m, n = c.n;
    if (c.clock) cur = (int)c.clock[CLK_CUR];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j >= n) return;
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt;
    const double hxxcd = 2 * c.xsp * hx * c.chi_diff, hyycd = 2 * c.ysp * hy * c.chi_diff,
                 hccd = 2 * (hxxcd + hyycd);
    const double dfac = 0.25 * c.chi_len * c.chi_len * (1 / c.mu), dfacx = dfac * c.xsp * c.xsp,
                 dfacy = dfac * c.ysp * c.ysp;
    const double *ch = F.f[cur][F_CHI], *dd = F.ddev;
    const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
    const size_t k = IDX(i, j), kl = IDX(il, j), kr = IDX(ir, j), kd = IDX(i, j - 1), ku = IDX(i, j + 1);
    const double Dd = dd[k] + dd[kd], Dl = dd[k] + dd[kl], Dr = dd[k] + dd[kr], Du = dd[k] + dd[ku];
    F.f[cur ^ 1][F_CHI][k] += hxxcd * (ch[kr] + ch[kl]) + hyycd * (ch[ku] + ch[kd]) - hccd * ch[k] +
                              dfacx * (Dr * ch[kr] - (Dr + Dl) * ch[k] + Dl * ch[kl]) +
                              dfacy * (Du * ch[ku] - (Du + Dd) * ch[k] + Dd * ch[kd]);
}

// Source of the projection (shear_sim.cc:399-409): net force of the stress
// on interior nodes from the four surrounding cells (net_force,
// shear_sim.cc:447-453) as fx = U(i,j-1) - W(i-1,j-1) + W(i,j) - U(i-1,j),
// fy = Y1(i-1,j-1) - Y2(i,j-1) + Y2(i-1,j) - Y1(i,j); Dirichlet data on the
// walls.
__global__ void k_source(step_consts c, fields_dev F, double xbc_bv) {
    const int m = c.m, n = c.n;
    if (c.clock) xbc_bv = c.xbc * c.clock[CLK_BV];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j > n) return;
    double2 f;
    if (j == 0) {
        f.x = -xbc_bv;
        f.y = 0;
    } else if (j == n) {
        f.x = xbc_bv;
        f.y = 0;
    } else {
        const int il = i == 0 ? m - 1 : i - 1;
        const size_t k0 = IDX(il, j - 1), k1 = IDX(i, j - 1), k2 = IDX(il, j), k3 = IDX(i, j);
        const double *U = F.pre[0], *W = F.pre[1], *Y1 = F.pre[2], *Y2 = F.pre[3];
        f.x = (U[k1] - W[k0]) + (W[k3] - U[k2]);
        f.y = (Y1[k0] - Y2[k1]) + (Y2[k2] - Y1[k3]);
    }
    F.src[(size_t)j * m + i] = f;
}

// Stress correction from the solved velocity (shear_sim.cc:418-434).
__global__ void k_project(step_consts c, fields_dev F, int cur, double hx, double hy) {
    const int m = c.m, n = c.n;
    if (c.clock) cur = (int)c.clock[CLK_CUR] ^ 1;  // the state the advection wrote
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j >= n) return;
    const int ir = i == m - 1 ? 0 : i + 1;
    const double2 a = F.vel[(size_t)j * m + i], b = F.vel[(size_t)j * m + ir], cu = F.vel[(size_t)(j + 1) * m + i],
                  d = F.vel[(size_t)(j + 1) * m + ir];
    const double ux = hx * (-a.x + b.x - cu.x + d.x), uy = hy * (-a.x - b.x + cu.x + d.x),
                 vx = hx * (-a.y + b.y - cu.y + d.y), vy = hy * (-a.y - b.y + cu.y + d.y);
    const size_t k = IDX(i, j);
    double *const *S = F.f[cur];
    const double third = 1 / 3.0;
    S[F_P][k] += -c.K * (ux + vy);
    S[F_Q][k] += -c.mu * third * (ux + vy);
    S[F_S][k] += c.mu * (ux - vy);
    S[F_TAU][k] += c.mu * (uy + vx);
}

// set_boundaries (shear_sim.cc:552-581): ghost rows by linear extrapolation,
// wall nodes of the reference map.  Wall velocities are not stored: the
// advection kernel takes them as arguments.
__global__ void k_boundaries(step_consts c, fields_dev F, int cur, double bp) {
    const int m = c.m, n = c.n;
    if (c.clock) {
        bp = c.clock[CLK_BP];
        cur = (int)c.clock[CLK_CUR] ^ 1;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    double *const *S = F.f[cur];
    S[F_X][IDX(i, 0)] = c.ax + i * c.dx + bp;
    S[F_Y][IDX(i, 0)] = c.ay;
    S[F_X][IDX(i, n)] = c.ax + i * c.dx - bp;
    S[F_Y][IDX(i, n)] = c.by;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        double *G = S[k];
        G[IDX(i, -1)] = 2 * G[IDX(i, 0)] - G[IDX(i, 1)];
        G[IDX(i, n)] = 2 * G[IDX(i, n - 1)] - G[IDX(i, n - 2)];
    }
}

#undef IDX

inline dim3 g2(int m, int n, dim3 b) { return dim3(ceil_div(m, b.x), ceil_div(n, b.y)); }

}  // namespace

void advection(const step_consts &c, fields_dev &F, int cur, double dt, double bv, cudaStream_t st) {
    dim3 blk(32, 8);
    k_advect<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, F, cur, dt, bv, 1); note_launch();
    if (c.chi_diff != 0 || c.chi_len != 0) {
        k_chi_diffusion<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, F, cur, dt);
        note_launch();
    }
}

void direct_step(const step_consts &c, double viscosity, fields_dev &F, int cur, double dt, double bv,
                 cudaStream_t st) {
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt;
    direct_consts d;
    d.hxxv = 2 * c.xsp * hx * viscosity;
    d.hyyv = 2 * c.ysp * hy * viscosity;
    d.hcv = 2 * (d.hxxv + d.hyyv);
    d.hxxcd = 2 * c.xsp * hx * c.chi_diff;
    d.hyycd = 2 * c.ysp * hy * c.chi_diff;
    d.hccd = 2 * (d.hxxcd + d.hyycd);
    dim3 blk(32, 8);
    k_direct<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, d, F, cur, dt, bv);
    note_launch();
    if (c.chi_diff != 0 || c.chi_len != 0) {
        k_chi_diffusion<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, F, cur, dt);
        note_launch();
    }
}

void projection_source(const step_consts &c, fields_dev &F, int cur, double dt, double xbc_bv, cudaStream_t st) {
    dim3 blk(32, 8);
    k_source<<<g2(c.m, c.n + 1, blk), blk, 0, st>>>(c, F, xbc_bv);
    note_launch();
    (void)cur;
    (void)dt;
}

void precombine(const step_consts &c, fields_dev &F, int cur, double dt, cudaStream_t st) {
    dim3 blk(32, 8);
    k_precombine<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, F, cur, 0.5 / dt * c.xsp, 0.5 / dt * c.ysp);
    note_launch();
}

void projection_apply(const step_consts &c, fields_dev &F, int cur, double dt, double bv, double bp,
                      cudaStream_t st) {
    dim3 blk(32, 8);
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt;
    k_project<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, F, cur, hx, hy); note_launch();
    k_boundaries<<<ceil_div(c.m, 128), 128, 0, st>>>(c, F, cur, bp); note_launch();
    (void)bv;
}

void set_boundaries(const step_consts &c, fields_dev &F, int cur, double bp, cudaStream_t st) {
    k_boundaries<<<ceil_div(c.m, 128), 128, 0, st>>>(c, F, cur, bp); note_launch();
}

}  // namespace stzg
