// Hand-written adjoint of the quasi-static STZ time step with checkpointed
// recomputation (forward/backward pair, shaped like torch.autograd.Function).
//
// Loss: L = dx dy sum_cells (eps_pl(T) - target)^2 after nsteps steps from the
// handle's state.  Gradients: dL/d(c0, Omega*eps0, chi_inf, s_y) and dL/d chi
// of the initial state.
//
// One forward step (shear_sim.cc:280-438) is S -> advection -> S' ->
// net-force source D S' -> vel = A^-1 (D S') -> S'' = S' + G vel ->
// set_boundaries -> S_next, with eps_pl += ddev/(2 mu).  Its adjoint, given
// lambda(S_next) and lambda(vel) from the next step's advection:
//   1. fold the ghost-row extrapolation (2 G[0] - G[1]) back into the rows;
//   2. g = lambda(vel) + G^T lambda(S''), zero on the Dirichlet wall rows;
//   3. mu = A_II^-1 g: the interior operator of qs_multi (qs_multi.hh:41-50)
//      is symmetric and the wall unknowns are data, so the forward multigrid
//      solves the adjoint system with a zero wall right-hand side;
//   4. lambda(S') = lambda(S'') + D^T mu;
//   5. advection adjoint: the ENO stencils with the forward's branch choices
//      and upwind directions are linear, their transposes are scattered with
//      atomic adds; the STZ sub-stepping loop (shear_sim.cc:513-548) is
//      differentiated in forward mode with a dual number carrying six partials
//      (sbar, chi, c0, Omega*eps0, chi_inf, s_y) through all its iterations.
// Branch decisions (ENO, upwind, yield, sub-step count) are held fixed, so
// the gradient is that of the piecewise-smooth map the forward evaluates.
#include <cmath>
#include <cstring>
#include <vector>

#include "mg_device.cuh"
#include "sim.cuh"
#include "stz_law.cuh"

namespace stzg {

// ---------------------------------------------------------------------------
// Dual numbers: value and ND partial derivatives.

constexpr int ND = 6;  // d/d sbar, d/d chi, d/d c0, d/d Omegaeps0, d/d chi_inf, d/d s_y

struct dual {
    double v;
    double d[ND];
    __host__ __device__ dual() : v(0) {
        for (int k = 0; k < ND; k++) d[k] = 0;
    }
    __host__ __device__ dual(double x) : v(x) {
        for (int k = 0; k < ND; k++) d[k] = 0;
    }
    __host__ __device__ static dual var(double x, int k) {
        dual r(x);
        r.d[k] = 1;
        return r;
    }
    __device__ dual &operator+=(const dual &o) {
        v += o.v;
        for (int k = 0; k < ND; k++) d[k] += o.d[k];
        return *this;
    }
    __device__ dual &operator-=(const dual &o) {
        v -= o.v;
        for (int k = 0; k < ND; k++) d[k] -= o.d[k];
        return *this;
    }
    __device__ dual &operator/=(const dual &o);
};

__host__ __device__ inline double value(const dual &x) { return x.v; }

__device__ inline dual operator+(const dual &a, const dual &b) {
    dual r = a;
    r += b;
    return r;
}
__device__ inline dual operator-(const dual &a, const dual &b) {
    dual r = a;
    r -= b;
    return r;
}
__device__ inline dual operator-(const dual &a) {
    dual r;
    r.v = -a.v;
    for (int k = 0; k < ND; k++) r.d[k] = -a.d[k];
    return r;
}
__device__ inline dual operator*(const dual &a, const dual &b) {
    dual r;
    r.v = a.v * b.v;
    for (int k = 0; k < ND; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
__device__ inline dual operator/(const dual &a, const dual &b) {
    dual r;
    r.v = a.v / b.v;
    const double ib = 1 / b.v;
    for (int k = 0; k < ND; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
__device__ inline dual &dual::operator/=(const dual &o) {
    *this = *this / o;
    return *this;
}
__device__ inline dual operator+(double a, const dual &b) { return dual(a) + b; }
__device__ inline dual operator+(const dual &a, double b) { return a + dual(b); }
__device__ inline dual operator-(double a, const dual &b) { return dual(a) - b; }
__device__ inline dual operator-(const dual &a, double b) { return a - dual(b); }
__device__ inline dual operator*(double a, const dual &b) {
    dual r;
    r.v = a * b.v;
    for (int k = 0; k < ND; k++) r.d[k] = a * b.d[k];
    return r;
}
__device__ inline dual operator*(const dual &a, double b) { return b * a; }
__device__ inline dual operator/(const dual &a, double b) { return a * (1 / b); }
__device__ inline dual operator/(double a, const dual &b) { return dual(a) / b; }

__device__ inline dual chain(const dual &a, double f, double df) {
    dual r;
    r.v = f;
    for (int k = 0; k < ND; k++) r.d[k] = df * a.d[k];
    return r;
}
__device__ inline dual exp(const dual &a) {
    const double e = ::exp(a.v);
    return chain(a, e, e);
}
__device__ inline dual cosh(const dual &a) { return chain(a, ::cosh(a.v), ::sinh(a.v)); }
__device__ inline dual sinh(const dual &a) { return chain(a, ::sinh(a.v), ::cosh(a.v)); }
__device__ inline dual tanh(const dual &a) {
    const double t = ::tanh(a.v);
    return chain(a, t, 1 - t * t);
}
__device__ inline dual sqrt(const dual &a) {
    const double q = ::sqrt(a.v);
    return chain(a, q, 0.5 / q);
}
__device__ inline dual fabs(const dual &a) { return a.v < 0 ? -a : a; }

}  // namespace stzg

// The law templates were declared before the dual type; instantiate them here
// where its operators are visible.
#include "stz_law.cuh"

namespace stzg {
namespace {

#define IDX(i, j) ((size_t)((j) + 1) * m + (i))

// the forward kernel's branch decision (eno2 in step.cuh)
__device__ __forceinline__ bool eno_a(double p0, double p1, double p2, double p3) { return eno2_pick(p0, p1, p2, p3); }
__device__ __forceinline__ double eno_val(bool a, double p0, double p1, double p2, double p3) {
    return a ? 3 * p1 - 4 * p2 + p3 : p0 - p2;
}
// lambda of an ENO value hs*eno2(p0..p3) scattered to its four points
__device__ __forceinline__ void eno_scatter(double *L, size_t i0, size_t i1, size_t i2, size_t i3, bool a, double g) {
    if (g == 0) return;
    if (a) {
        atomicAdd(L + i1, 3 * g);
        atomicAdd(L + i2, -4 * g);
        atomicAdd(L + i3, g);
    } else {
        atomicAdd(L + i0, g);
        atomicAdd(L + i2, -g);
    }
}

struct adj_fields {
    const double *S[F_COUNT];   // state before the step (buffer with ghosts)
    const double2 *vel;         // velocity before the step
    const double *Lout[F_COUNT];// lambda of the advection outputs
    const double *Leps;         // dL/d eps_pl (cells, m*n), times leps_scale
    double leps_scale;          // upstream gradient of the loss
    double *Lin[F_COUNT];       // lambda of the step inputs (accumulated)
    double2 *Lvel;              // lambda of the input velocity (accumulated)
    double *Lpar;               // 4 parameter gradients (accumulated)
};

struct law_dual_in {
    int stz_model, t_model, substep_cap;
    double t_scale, adapt_fac, theta, Delta, tau0, kappa, rho, mu;
    double c0, Omegaeps0, chi_inf, s_y;
};

// Adjoint of k_advect (step.cu) for cell (i,j) and node (i,j).
__global__ void __launch_bounds__(128) k_adj_advect(step_consts c, adj_fields A, double dt, double bv) {
    const int m = c.m, n = c.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double lpar[4] = {0, 0, 0, 0};
    if (i < m && j < n) {
        const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt, lx = c.lx;
        const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
        const int il2 = i <= 1 ? i + m - 2 : i - 2, ir2 = i >= m - 2 ? i + 2 - m : i + 2;
        const size_t ci = IDX(i, j);
        auto U = [&](int ii, int jj) { return jj == 0 ? -bv : (jj == n ? bv : A.vel[(size_t)jj * m + ii].x); };
        auto Vv = [&](int ii, int jj) { return (jj == 0 || jj == n) ? 0.0 : A.vel[(size_t)jj * m + ii].y; };
        auto addu = [&](int ii, int jj, double gx, double gy) {
            if (jj <= 0 || jj >= n) return;  // wall velocities are boundary data
            double2 *p = A.Lvel + (size_t)jj * m + ii;
            if (gx != 0) atomicAdd(&p->x, gx);
            if (gy != 0) atomicAdd(&p->y, gy);
        };
        // ---- reference map at node (i,j), rows 1..n-1
        if (j > 0) {
            const double *X = A.S[F_X], *Y = A.S[F_Y];
            const double LX = A.Lout[F_X][ci], LY = A.Lout[F_Y][ci];
            atomicAdd(A.Lin[F_X] + ci, LX);
            atomicAdd(A.Lin[F_Y] + ci, LY);
            const double uc = U(i, j), vc = Vv(i, j);
            size_t xi[4], yi[4];
            double hsx, hsy;
            if (uc > 0) {
                xi[0] = IDX(ir, j); xi[1] = ci; xi[2] = IDX(il, j); xi[3] = IDX(il2, j);
                hsx = hx;
            } else {
                xi[0] = IDX(il, j); xi[1] = ci; xi[2] = IDX(ir, j); xi[3] = IDX(ir2, j);
                hsx = -hx;
            }
            const double s0 = uc > 0 ? (i == m - 1 ? lx : 0) : (i == 0 ? -lx : 0);
            const double s2 = uc > 0 ? (i == 0 ? -lx : 0) : (i == m - 1 ? lx : 0);
            const double s3 = uc > 0 ? (i <= 1 ? -lx : 0) : (i >= m - 2 ? lx : 0);
            const bool ax = eno_a(X[xi[0]] + s0, X[xi[1]], X[xi[2]] + s2, X[xi[3]] + s3);
            const bool ay = eno_a(Y[xi[0]], Y[xi[1]], Y[xi[2]], Y[xi[3]]);
            const double Xx = hsx * eno_val(ax, X[xi[0]] + s0, X[xi[1]], X[xi[2]] + s2, X[xi[3]] + s3);
            const double Yx = hsx * eno_val(ay, Y[xi[0]], Y[xi[1]], Y[xi[2]], Y[xi[3]]);
            bool one_sided;
            if (vc > 0) {
                one_sided = j <= 1;
                if (!one_sided) { yi[0] = IDX(i, j + 1); yi[1] = ci; yi[2] = IDX(i, j - 1); yi[3] = IDX(i, j - 2); }
                else { yi[0] = ci; yi[1] = IDX(i, j - 1); }
                hsy = hy;
            } else {
                one_sided = j >= n - 1;
                if (!one_sided) { yi[0] = IDX(i, j - 1); yi[1] = ci; yi[2] = IDX(i, j + 1); yi[3] = IDX(i, j + 2); }
                else { yi[0] = ci; yi[1] = IDX(i, j + 1); }
                hsy = -hy;
            }
            double Xy, Yy;
            bool bxa = false, bya = false;
            if (one_sided) {
                Xy = 2 * hsy * (X[yi[0]] - X[yi[1]]);
                Yy = 2 * hsy * (Y[yi[0]] - Y[yi[1]]);
            } else {
                bxa = eno_a(X[yi[0]], X[yi[1]], X[yi[2]], X[yi[3]]);
                bya = eno_a(Y[yi[0]], Y[yi[1]], Y[yi[2]], Y[yi[3]]);
                Xy = hsy * eno_val(bxa, X[yi[0]], X[yi[1]], X[yi[2]], X[yi[3]]);
                Yy = hsy * eno_val(bya, Y[yi[0]], Y[yi[1]], Y[yi[2]], Y[yi[3]]);
            }
            // X' = X - uc Xx - vc Xy, Y' likewise
            addu(i, j, -LX * Xx - LY * Yx, -LX * Xy - LY * Yy);
            eno_scatter(A.Lin[F_X], xi[0], xi[1], xi[2], xi[3], ax, -uc * LX * hsx);
            eno_scatter(A.Lin[F_Y], xi[0], xi[1], xi[2], xi[3], ay, -uc * LY * hsx);
            if (one_sided) {
                const double gX = -vc * LX * 2 * hsy, gY = -vc * LY * 2 * hsy;
                if (gX != 0) { atomicAdd(A.Lin[F_X] + yi[0], gX); atomicAdd(A.Lin[F_X] + yi[1], -gX); }
                if (gY != 0) { atomicAdd(A.Lin[F_Y] + yi[0], gY); atomicAdd(A.Lin[F_Y] + yi[1], -gY); }
            } else {
                eno_scatter(A.Lin[F_X], yi[0], yi[1], yi[2], yi[3], bxa, -vc * LX * hsy);
                eno_scatter(A.Lin[F_Y], yi[0], yi[1], yi[2], yi[3], bya, -vc * LY * hsy);
            }
        }
        // ---- cell (i,j)
        const double u00 = U(i, j), u10 = U(ir, j), u01 = U(i, j + 1), u11 = U(ir, j + 1);
        const double v00 = Vv(i, j), v10 = Vv(ir, j), v01 = Vv(i, j + 1), v11 = Vv(ir, j + 1);
        const double uc = 0.25 * (u00 + u10 + u01 + u11), vc = 0.25 * (v00 + v10 + v01 + v11);
        const double two_omega = hx * (-v00 + v10 - v01 + v11) - hy * (-u00 - u10 + u01 + u11);
        size_t xi[4], yi[4];
        double hsx, hsy;
        if (uc > 0) {
            xi[0] = IDX(ir, j); xi[1] = ci; xi[2] = IDX(il, j); xi[3] = IDX(il2, j);
            hsx = hx;
        } else {
            xi[0] = IDX(il, j); xi[1] = ci; xi[2] = IDX(ir, j); xi[3] = IDX(ir2, j);
            hsx = -hx;
        }
        bool one_sided;
        if (vc > 0) {
            one_sided = j == 0;
            if (!one_sided) { yi[0] = IDX(i, j + 1); yi[1] = ci; yi[2] = IDX(i, j - 1); yi[3] = IDX(i, j - 2); }
            else { yi[0] = ci; yi[1] = IDX(i, j - 1); }
            hsy = hy;
        } else {
            one_sided = j >= n - 1;
            if (!one_sided) { yi[0] = IDX(i, j - 1); yi[1] = ci; yi[2] = IDX(i, j + 1); yi[3] = IDX(i, j + 2); }
            else { yi[0] = ci; yi[1] = IDX(i, j + 1); }
            hsy = -hy;
        }
        double f1[5], f2[5];
        bool a1[5], a2[5];
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const double *G = A.S[k];
            a1[k] = eno_a(G[xi[0]], G[xi[1]], G[xi[2]], G[xi[3]]);
            f1[k] = hsx * eno_val(a1[k], G[xi[0]], G[xi[1]], G[xi[2]], G[xi[3]]);
            if (one_sided) {
                a2[k] = false;
                f2[k] = 2 * hsy * (G[yi[0]] - G[yi[1]]);
            } else {
                a2[k] = eno_a(G[yi[0]], G[yi[1]], G[yi[2]], G[yi[3]]);
                f2[k] = hsy * eno_val(a2[k], G[yi[0]], G[yi[1]], G[yi[2]], G[yi[3]]);
            }
        }
        const double q = A.S[F_Q][ci], s = A.S[F_S][ci], t = A.S[F_TAU][ci];
        const double cchi = A.S[F_CHI][ci] - uc * f1[4] - vc * f2[4];
        const double devsq = 3 * q * q + s * s + t * t;
        // plastic term and its partials (forward mode through the sub-steps)
        double ddev = 0, dtmp = 0, J_ddev[ND] = {0}, J_dtmp[ND] = {0}, J_chi[ND] = {0};
        J_chi[1] = 1;  // chi_out = cchi where there is no plastic flow
        const bool athermal = c.stz_model >= 2;
        if (!(devsq < 0.999e-24 || (athermal && devsq < c.yield_cut2))) {
            stz_law_params<dual> lp;
            lp.stz_model = c.stz_model; lp.t_model = c.t_model; lp.substep_cap = c.substep_cap;
            lp.t_scale = c.t_scale; lp.adapt_fac = c.adapt_fac; lp.theta = c.theta; lp.Delta = c.Delta;
            lp.tau0 = c.tau0; lp.kappa = c.kappa; lp.rho = c.rho; lp.mu = c.mu;
            lp.c0 = dual::var(c.c0, 2);
            lp.Omegaeps0 = dual::var(c.Omegaeps0, 3);
            lp.chi_inf = dual::var(c.chi_inf, 4);
            lp.s_y = dual::var(c.s_y, 5);
            dual sbar = dual::var(::sqrt(devsq), 0), chiv = dual::var(cchi, 1), dd;
            int iters;
            dual dt_ = adaptive_plastic(lp, sbar, chiv, dd, dt, iters);
            ddev = dd.v;
            dtmp = dt_.v;
            for (int k = 0; k < ND; k++) {
                J_ddev[k] = dd.d[k];
                J_dtmp[k] = dt_.d[k];
                J_chi[k] = chiv.d[k];
            }
        }
        const size_t cc = (size_t)j * m + i;
        const double Lp = A.Lout[F_P][ci], Lq = A.Lout[F_Q][ci], Ls = A.Lout[F_S][ci], Lt = A.Lout[F_TAU][ci];
        const double Lc = A.Lout[F_CHI][ci], Le = A.leps_scale * A.Leps[cc];
        const double Lddev = Le / (2 * c.mu);
        const double Ldtmp = -(Lq * q + Ls * s + Lt * t);
        double G[ND];
        for (int k = 0; k < ND; k++) G[k] = Lddev * J_ddev[k] + Ldtmp * J_dtmp[k] + Lc * J_chi[k];
        const double Lsbar = G[0], Lcchi = G[1];
        for (int k = 0; k < 4; k++) lpar[k] = G[2 + k];
        double lq = Lq * (1 - dtmp), ls = Ls * (1 - dtmp) - Lt * two_omega, lt = Lt * (1 - dtmp) + Ls * two_omega;
        if (Lsbar != 0) {
            const double sb = ::sqrt(devsq);
            lq += Lsbar * 3 * q / sb;
            ls += Lsbar * s / sb;
            lt += Lsbar * t / sb;
        }
        atomicAdd(A.Lin[F_P] + ci, Lp);
        atomicAdd(A.Lin[F_Q] + ci, lq);
        atomicAdd(A.Lin[F_S] + ci, ls);
        atomicAdd(A.Lin[F_TAU] + ci, lt);
        atomicAdd(A.Lin[F_CHI] + ci, Lcchi);
        const double Lk[5] = {Lp, Lq, Ls, Lt, Lcchi};
        double Luc = 0, Lvc = 0;
#pragma unroll
        for (int k = 0; k < 5; k++) {
            Luc -= Lk[k] * f1[k];
            Lvc -= Lk[k] * f2[k];
            eno_scatter(A.Lin[k], xi[0], xi[1], xi[2], xi[3], a1[k], -uc * Lk[k] * hsx);
            if (one_sided) {
                const double g = -vc * Lk[k] * 2 * hsy;
                if (g != 0) {
                    atomicAdd(A.Lin[k] + yi[0], g);
                    atomicAdd(A.Lin[k] + yi[1], -g);
                }
            } else {
                eno_scatter(A.Lin[k], yi[0], yi[1], yi[2], yi[3], a2[k], -vc * Lk[k] * hsy);
            }
        }
        const double Lw = Ls * t - Lt * s;  // lambda of two_omega
        // uc, vc = averages of the four corner nodes; two_omega as in the forward
        addu(i, j, 0.25 * Luc + hy * Lw, 0.25 * Lvc - hx * Lw);
        addu(ir, j, 0.25 * Luc + hy * Lw, 0.25 * Lvc + hx * Lw);
        addu(i, j + 1, 0.25 * Luc - hy * Lw, 0.25 * Lvc - hx * Lw);
        addu(ir, j + 1, 0.25 * Luc - hy * Lw, 0.25 * Lvc + hx * Lw);
    }
    // parameter gradients: block reduction, one atomic per block and parameter
    __shared__ double red[4][128];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int k = 0; k < 4; k++) red[k][tid] = lpar[k];
    __syncthreads();
    for (int w = 64; w > 0; w >>= 1) {
        if (tid < w)
            for (int k = 0; k < 4; k++) red[k][tid] += red[k][tid + w];
        __syncthreads();
    }
    if (tid == 0)
        for (int k = 0; k < 4; k++)
            if (red[k][0] != 0) atomicAdd(A.Lpar + k, red[k][0]);
}

// Ghost rows G[-1] = 2 G[0] - G[1], G[n] = 2 G[n-1] - G[n-2] (set_boundaries,
// shear_sim.cc:552-581) folded back into the rows; the wall rows of X, Y are
// boundary data.
__global__ void k_adj_fold_ghosts(int m, int n, double *L0, double *L1, double *L2, double *L3, double *L4, double *LX,
                                  double *LY) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    double *Ls[5] = {L0, L1, L2, L3, L4};
    for (int k = 0; k < 5; k++) {
        double *G = Ls[k];
        const double gb = G[IDX(i, -1)], gt = G[IDX(i, n)];
        G[IDX(i, 0)] += 2 * gb;
        G[IDX(i, 1)] -= gb;
        G[IDX(i, n - 1)] += 2 * gt;
        G[IDX(i, n - 2)] -= gt;
        G[IDX(i, -1)] = 0;
        G[IDX(i, n)] = 0;
    }
    LX[IDX(i, 0)] = 0;
    LX[IDX(i, n)] = 0;
    LY[IDX(i, 0)] = 0;
    LY[IDX(i, n)] = 0;
}

// g = lambda(vel_next) + G^T lambda(stress): the stress correction of
// shear_sim.cc:418-434 transposed, gathered per node from its four cells;
// zero on the wall rows.
__global__ void k_adj_project(int m, int n, double hx, double hy, double K, double mu, const double *Lp,
                              const double *Lq, const double *Ls, const double *Lt, const double2 *Lvel_next,
                              double2 *g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j > n) return;
    const size_t k = (size_t)j * m + i;
    if (j == 0 || j == n) {
        g[k] = make_double2(0, 0);
        return;
    }
    const double third = 1 / 3.0;
    double gx = Lvel_next ? Lvel_next[k].x : 0, gy = Lvel_next ? Lvel_next[k].y : 0;
    const int il = i == 0 ? m - 1 : i - 1;
    // cell (ci, cj) and the role (a,b,c,d) of node (i,j) in it
    const int cis[4] = {i, il, i, il}, cjs[4] = {j, j, j - 1, j - 1};
    const double sx[4] = {-1, 1, -1, 1}, sy[4] = {-1, -1, 1, 1};
    for (int r = 0; r < 4; r++) {
        const int cj = cjs[r];
        if (cj < 0 || cj >= n) continue;
        const size_t cc = IDX(cis[r], cj);
        const double lp = Lp[cc], lq = Lq[cc], ls = Ls[cc], lt = Lt[cc];
        const double Lux = -K * lp - mu * third * lq + mu * ls, Lvy = -K * lp - mu * third * lq - mu * ls;
        const double Luy = mu * lt, Lvx = mu * lt;
        gx += sx[r] * hx * Lux + sy[r] * hy * Luy;
        gy += sx[r] * hx * Lvx + sy[r] * hy * Lvy;
    }
    g[k] = make_double2(gx, gy);
}

// lambda(stress) += D^T mu: the net force of shear_sim.cc:447-453 transposed,
// gathered per cell from its four corner nodes (interior node rows only).
__global__ void k_adj_source(int m, int n, double xf, double yf, const double2 *mu_, double *Lp, double *Lq,
                             double *Ls, double *Lt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j >= n) return;
    const int ir = i == m - 1 ? 0 : i + 1;
    auto M = [&](int ii, int jj) {
        return (jj <= 0 || jj >= n) ? make_double2(0, 0) : mu_[(size_t)jj * m + ii];
    };
    // this cell is f3 of node (i,j), f2 of (i+1,j), f1 of (i,j+1), f0 of (i+1,j+1)
    const double2 n3 = M(i, j), n2 = M(ir, j), n1 = M(i, j + 1), n0 = M(ir, j + 1);
    const double LA = xf * (n3.x - n2.x + n1.x - n0.x);
    const double Ltau = yf * (-n3.x - n2.x + n1.x + n0.x) + xf * (-n3.y + n2.y - n1.y + n0.y);
    const double LB = yf * (n3.y + n2.y - n1.y - n0.y);
    const size_t c = IDX(i, j);
    Lp[c] += LA + LB;
    Lq[c] += LA + LB;
    Ls[c] += -LA + LB;
    Lt[c] += Ltau;
}

__global__ void k_loss(int m, int n, double w, const double *eps, const double *target, double *Leps,
                       double *partials) {
    __shared__ double sh[32];
    double a = 0;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < (long)m * n; k += (long)gridDim.x * blockDim.x) {
        const double d = eps[k] - target[k];
        a += w * d * d;
        Leps[k] = 2 * w * d;
    }
    a = block_sum(a, sh);
    if (threadIdx.x == 0) partials[2 * blockIdx.x] = a;
    if (threadIdx.x == 0) partials[2 * blockIdx.x + 1] = 0;
}

#undef IDX

}  // namespace
}  // namespace stzg

using namespace stzg;


namespace stzg {
// Host-side part of a saved state.
struct host_state {
    double time = 0, bv = 0;
    int lim = 0;
    bool have_prev = false, have_prev2 = false;
};
}  // namespace stzg

// Adjoint workspace of a handle: checkpoints, the states of one recomputed
// segment, the adjoint fields and an FP64 multigrid hierarchy with its own
// top-level arrays.  Sized per (nsteps, checkpoint interval); freed with the
// handle.
struct stzg_adjoint {
    int nsteps = 0, every = 0;
    double dt = 0;
    std::vector<void *> mem;
    std::vector<double *> ckpt;  // state at steps 0, every, 2 every, ...
    std::vector<stzg::host_state> ck;
    double *seg = nullptr;          // input state of every step of a segment
    double *final_state = nullptr;  // state after the last step
    stzg::host_state final_meta;
    double *lam[2][F_COUNT] = {};
    double *leps = nullptr, *target = nullptr, *lpar = nullptr;
    double2 *lvel = nullptr, *lvel_in = nullptr;
    stzg::hierarchy<double> h;
    bool h_ready = false;
    cudaGraphExec_t g_vc = nullptr;  // two V-cycles of h, captured per backward call
    long n_vc = 0;
    void drop_graph() {
        if (g_vc) cudaGraphExecDestroy(g_vc);
        g_vc = nullptr;
    }
    void free_mem() {
        for (void *p : mem) cudaFree(p);
        mem.clear();
        ckpt.clear();
        nsteps = every = 0;
    }
    ~stzg_adjoint() {
        drop_graph();
        free_mem();
    }
};

namespace stzg {
namespace {

int adj_alloc(stzg_sim *s, stzg_adjoint *a, void *p, size_t bytes) {
    void **pp = (void **)p;
    cudaError_t e = cudaMalloc(pp, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(adjoint)");
    a->mem.push_back(*pp);
    STZG_CUDA(cudaMemsetAsync(*pp, 0, bytes, s->st));
    return STZG_OK;
}

// One state: the seven fields (rows -1..n), the velocity, eps_pl and, when
// initial guesses are extrapolated, the previous velocity.  Together with
// the host scalars (time, wall speed, the multigrid predictor's lim) this is
// everything a step reads, so a segment recomputed from its checkpoint
// repeats the forward run bit for bit.
size_t slab_doubles(const stzg_sim *s) {
    const size_t nc = cell_count(s), nn = (size_t)s->m * (s->n + 1);
    return 7 * nc + 2 * nn + (size_t)s->m * s->n + (s->vel_prev ? 2 * nn : 0) + (s->vel_prev2 ? 2 * nn : 0);
}

host_state save_state(stzg_sim *s, double *slab, int *status) {
    const size_t nc = cell_count(s), nn = (size_t)s->m * (s->n + 1), mn = (size_t)s->m * s->n;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < F_COUNT && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(slab + k * nc, s->F.f[s->cur][k], nc * 8, cudaMemcpyDeviceToDevice, s->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(slab + 7 * nc, s->F.vel, nn * 16, cudaMemcpyDeviceToDevice, s->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slab + 7 * nc + 2 * nn, s->F.eps_pl, mn * 8, cudaMemcpyDeviceToDevice, s->st);
    if (e == cudaSuccess && s->vel_prev)
        e = cudaMemcpyAsync(slab + 7 * nc + 2 * nn + mn, s->vel_prev, nn * 16, cudaMemcpyDeviceToDevice, s->st);
    if (e == cudaSuccess && s->vel_prev2)
        e = cudaMemcpyAsync(slab + 7 * nc + 4 * nn + mn, s->vel_prev2, nn * 16, cudaMemcpyDeviceToDevice, s->st);
    *status = e == cudaSuccess ? STZG_OK : cuda_fail(e, "cudaMemcpyAsync(checkpoint)");
    host_state h;
    h.time = s->time;
    h.bv = s->bv_state;
    h.lim = s->lim;
    h.have_prev = s->have_prev;
    h.have_prev2 = s->have_prev2;
    return h;
}

// Restores a saved state into buffer 0 of the handle.
int load_state(stzg_sim *s, const double *slab, const host_state &h) {
    const size_t nc = cell_count(s), nn = (size_t)s->m * (s->n + 1), mn = (size_t)s->m * s->n;
    for (int k = 0; k < F_COUNT; k++)
        STZG_CUDA(cudaMemcpyAsync(s->F.f[0][k], slab + k * nc, nc * 8, cudaMemcpyDeviceToDevice, s->st));
    STZG_CUDA(cudaMemcpyAsync(s->F.vel, slab + 7 * nc, nn * 16, cudaMemcpyDeviceToDevice, s->st));
    STZG_CUDA(cudaMemcpyAsync(s->F.eps_pl, slab + 7 * nc + 2 * nn, mn * 8, cudaMemcpyDeviceToDevice, s->st));
    if (s->vel_prev)
        STZG_CUDA(cudaMemcpyAsync(s->vel_prev, slab + 7 * nc + 2 * nn + mn, nn * 16, cudaMemcpyDeviceToDevice, s->st));
    if (s->vel_prev2)
        STZG_CUDA(cudaMemcpyAsync(s->vel_prev2, slab + 7 * nc + 4 * nn + mn, nn * 16, cudaMemcpyDeviceToDevice, s->st));
    s->cur = 0;
    s->time = h.time;
    s->bv_state = h.bv;
    s->lim = h.lim;
    s->have_prev = h.have_prev;
    s->have_prev2 = h.have_prev2;
    return STZG_OK;
}

// mu = A_II^-1 g on the interior rows (g and mu zero on the wall rows), to a
// relative residual of 1e-13, warm-started from the previous step's mu.
int adjoint_solve(stzg_sim *s, stzg_adjoint *a) {
    hierarchy<double> &h = a->h;
    const size_t nn = (size_t)s->m * (s->n + 1);
    for (int it = 0; it < 200; it++) {
        top_residual_sqnorm(h, s->partials, s->npart, s->dnorm, s->dnorm + 1, s->st);
        STZG_CUDA(cudaMemcpyAsync(s->hnorm, s->dnorm, 16, cudaMemcpyDeviceToHost, s->st));
        STZG_CUDA(cudaStreamSynchronize(s->st));
        const double r2 = s->hnorm[0], b2 = s->hnorm[1];
        if (std::isnan(r2) || std::isnan(b2)) return fail(STZG_ENAN, "NaN in the adjoint solve");
        if (b2 == 0) {
            STZG_CUDA(cudaMemsetAsync(h.lv[0].z, 0, nn * 16, s->st));
            return STZG_OK;
        }
        if (r2 <= 1e-26 * b2) return STZG_OK;
        STZG_CUDA(cudaGraphLaunch(a->g_vc, s->st));
        for (long k = 0; k < a->n_vc; k++) note_launch();
    }
    return fail(STZG_ENOTCONV, "adjoint multigrid did not converge");
}

}  // namespace

void adjoint_release(stzg_sim *s) {
    delete s->adj;
    s->adj = nullptr;
}

}  // namespace stzg

extern "C" {

int stzg_adjoint_forward(stzg_sim *s, double dt, int nsteps, int every, const double *target, double *loss) {
    if (!s || !target || !loss || !(dt > 0) || nsteps < 1 || every < 1)
        return fail(STZG_EINVAL, "bad adjoint forward arguments");
    if (s->P.chi_diff != 0 || s->P.chi_len != 0)
        return fail(STZG_EINVAL, "the adjoint does not cover chi diffusion (chi_diff = chi_len = 0 required)");
    if (!s->sc.track_plastic) return fail(STZG_EINVAL, "the loss reads eps_pl: create the handle with track_plastic");
    if (!s->adj) s->adj = new stzg_adjoint;
    stzg_adjoint *a = s->adj;
    const size_t nc = cell_count(s), nn = (size_t)s->m * (s->n + 1), mn = (size_t)s->m * s->n;
    const size_t slab = slab_doubles(s);
    const int nck = (nsteps + every - 1) / every;
    if (a->nsteps != nsteps || a->every != every) {
        STZG_CUDA(cudaStreamSynchronize(s->st));
        a->free_mem();
        a->ckpt.assign(nck, nullptr);
        for (int k = 0; k < nck; k++) STZG_CHECK(adj_alloc(s, a, &a->ckpt[k], slab * 8));
        STZG_CHECK(adj_alloc(s, a, &a->seg, slab * 8 * std::min(every, nsteps)));
        STZG_CHECK(adj_alloc(s, a, &a->final_state, slab * 8));
        for (int b = 0; b < 2; b++)
            for (int k = 0; k < F_COUNT; k++) STZG_CHECK(adj_alloc(s, a, &a->lam[b][k], nc * 8));
        STZG_CHECK(adj_alloc(s, a, &a->leps, mn * 8));
        STZG_CHECK(adj_alloc(s, a, &a->target, mn * 8));
        STZG_CHECK(adj_alloc(s, a, &a->lpar, 4 * 8));
        STZG_CHECK(adj_alloc(s, a, &a->lvel, nn * 16));
        STZG_CHECK(adj_alloc(s, a, &a->lvel_in, nn * 16));
        a->nsteps = nsteps;
        a->every = every;
    }
    if (!a->h_ready) {
        STZG_CHECK(a->h.allocate(s->m, s->n + 1, nullptr, nullptr));
        a->h_ready = true;
    }
    STZG_CHECK(ensure_ops(s, dt));
    STZG_CHECK(a->h.upload_ops(s->ops, s->q.op<double>()));
    a->dt = dt;
    a->ck.assign(nck, host_state());
    int st = STZG_OK;
    STZG_CUDA(cudaMemcpyAsync(a->target, target, mn * 8, cudaMemcpyHostToDevice, s->st));
    for (int k = 0; k < nsteps; k++) {
        if (k % every == 0) {
            a->ck[k / every] = save_state(s, a->ckpt[k / every], &st);
            STZG_CHECK(st);
        }
        STZG_CHECK(stzg_step_qs(s, dt, 1, nullptr));
    }
    a->final_meta = save_state(s, a->final_state, &st);
    STZG_CHECK(st);
    const double w = ((s->P.bx - s->P.ax) / s->m) * ((s->P.by - s->P.ay) / s->n);
    k_loss<<<s->npart, 256, 0, s->st>>>(s->m, s->n, w, s->F.eps_pl, a->target, a->leps, s->partials);
    note_launch();
    std::vector<double> part(2 * (size_t)s->npart);
    STZG_CUDA(cudaMemcpyAsync(part.data(), s->partials, part.size() * 8, cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    double L = 0;
    for (int k = 0; k < s->npart; k++) L += part[2 * k];
    *loss = L;
    return STZG_OK;
}

int stzg_adjoint_backward(stzg_sim *s, double dloss, double *grad_params, double *grad_chi0) {
    if (!s || !s->adj || s->adj->nsteps == 0) return fail(STZG_EINVAL, "no adjoint forward run on this handle");
    stzg_adjoint *a = s->adj;
    const int m = s->m, n = s->n;
    const size_t nc = cell_count(s), nn = (size_t)m * (n + 1), mn = (size_t)m * n;
    const size_t slab = slab_doubles(s);
    const double dt = a->dt;
    STZG_CHECK(ensure_ops(s, dt));
    STZG_CHECK(a->h.upload_ops(s->ops, s->q.op<double>()));
    // the adjoint solve relaunches one graph of two V-cycles
    a->drop_graph();
    {
        STZG_CUDA(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
        const long c0 = launch_count();
        vcycle<double>(a->h, s->st, 10, 1);
        vcycle<double>(a->h, s->st, 10, 1);
        a->n_vc = launch_count() - c0;
        discount_launches(a->n_vc);
        cudaGraph_t g = nullptr;
        STZG_CUDA(cudaStreamEndCapture(s->st, &g));
        const cudaError_t e = cudaGraphInstantiate(&a->g_vc, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            a->g_vc = nullptr;
            return cuda_fail(e, "cudaGraphInstantiate(adjoint V-cycles)");
        }
    }
    step_consts sc = s->sc;
    sc.clock = nullptr;
    const double hx = 0.5 * sc.xsp * dt, hy = 0.5 * sc.ysp * dt;
    const double xf = 0.5 / dt * sc.xsp, yf = 0.5 / dt * sc.ysp;
    const dim3 blk(32, 4), blk8(32, 8);
    const dim3 gc(ceil_div(m, 32), ceil_div(n, 4)), gn(ceil_div(m, 32), ceil_div(n + 1, 8)),
        gs(ceil_div(m, 32), ceil_div(n, 8));
    int cur = 0;  // lam[cur]: lambda of the state after the step being reversed
    for (int b = 0; b < 2; b++)
        for (int k = 0; k < F_COUNT; k++) STZG_CUDA(cudaMemsetAsync(a->lam[b][k], 0, nc * 8, s->st));
    STZG_CUDA(cudaMemsetAsync(a->lvel, 0, nn * 16, s->st));
    STZG_CUDA(cudaMemsetAsync(a->lpar, 0, 32, s->st));
    STZG_CUDA(cudaMemsetAsync(a->h.lv[0].z, 0, nn * 16, s->st));
    const int nck = (int)a->ckpt.size();
    std::vector<double> seg_bv(a->every);
    int st = STZG_OK;
    for (int c = nck - 1; c >= 0; c--) {
        const int k0 = c * a->every, k1 = std::min(a->nsteps, k0 + a->every);
        // recompute the segment from its checkpoint, keeping each step's input
        STZG_CHECK(load_state(s, a->ckpt[c], a->ck[c]));
        for (int k = k0; k < k1; k++) {
            seg_bv[k - k0] = save_state(s, a->seg + (size_t)(k - k0) * slab, &st).bv;
            STZG_CHECK(st);
            STZG_CHECK(stzg_step_qs(s, dt, 1, nullptr));
        }
        for (int k = k1 - 1; k >= k0; k--) {
            const double *st_in = a->seg + (size_t)(k - k0) * slab;
            double *const *L = a->lam[cur];
            double *const *Lin = a->lam[cur ^ 1];
            // 1. ghost rows and wall nodes of set_boundaries
            k_adj_fold_ghosts<<<ceil_div(m, 128), 128, 0, s->st>>>(m, n, L[0], L[1], L[2], L[3], L[4], L[5], L[6]);
            note_launch();
            // 2. g = lambda(vel) + G^T lambda(stress)
            k_adj_project<<<gn, blk8, 0, s->st>>>(m, n, hx, hy, sc.K, sc.mu, L[F_P], L[F_Q], L[F_S], L[F_TAU],
                                                  a->lvel, a->h.lv[0].b);
            note_launch();
            // 3. mu = A^-1 g
            STZG_CHECK(adjoint_solve(s, a));
            // 4. lambda(stress after advection) += D^T mu
            k_adj_source<<<gs, blk8, 0, s->st>>>(m, n, xf, yf, a->h.lv[0].z, L[F_P], L[F_Q], L[F_S], L[F_TAU]);
            note_launch();
            // 5. advection + plasticity, into lambda of the step's input state
            for (int f = 0; f < F_COUNT; f++) STZG_CUDA(cudaMemsetAsync(Lin[f], 0, nc * 8, s->st));
            STZG_CUDA(cudaMemsetAsync(a->lvel_in, 0, nn * 16, s->st));
            adj_fields A;
            for (int f = 0; f < F_COUNT; f++) {
                A.S[f] = st_in + f * nc;
                A.Lout[f] = L[f];
                A.Lin[f] = Lin[f];
            }
            A.vel = (const double2 *)(st_in + 7 * nc);
            A.Leps = a->leps;
            A.leps_scale = dloss;
            A.Lvel = a->lvel_in;
            A.Lpar = a->lpar;
            k_adj_advect<<<gc, blk, 0, s->st>>>(sc, A, dt, seg_bv[k - k0]);
            note_launch();
            std::swap(a->lvel, a->lvel_in);
            cur ^= 1;
        }
    }
    // the initial state's ghost rows were extrapolated from its rows
    double *const *L = a->lam[cur];
    k_adj_fold_ghosts<<<ceil_div(m, 128), 128, 0, s->st>>>(m, n, L[0], L[1], L[2], L[3], L[4], L[5], L[6]);
    note_launch();
    STZG_CUDA(cudaGetLastError());
    if (grad_chi0) STZG_CUDA(cudaMemcpyAsync(grad_chi0, L[F_CHI] + m, mn * 8, cudaMemcpyDeviceToHost, s->st));
    if (grad_params) STZG_CUDA(cudaMemcpyAsync(grad_params, a->lpar, 32, cudaMemcpyDeviceToHost, s->st));
    // leave the handle at the end of the forward run
    STZG_CHECK(load_state(s, a->final_state, a->final_meta));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

}  // extern "C"
