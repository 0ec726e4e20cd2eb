// Time-step kernels: fused ENO advection + STZ plasticity, chi diffusion,
// projection source, stress correction and boundaries.
#include "ff.cuh"
#include "step.cuh"
#include "stz_law.cuh"

namespace stzg {

// x = hi + lo as floats on the host (hi the nearest float, lo the nearest
// float of the remainder): the float-float form of a launch constant.
void split_host(double x, float *hi, float *lo) {
    *hi = (float)x;
    *lo = (float)(x - (double)*hi);
}

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
    c.yield_cut2f = (float)(c.yield_cut2 * (1 - 1e-6));
    c.clock = nullptr;
    c.xbc = 0;
    c.sp_increments = 0;
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

// Fused advection + STZ step over a tile of ATX x ATY cells (i,j) and their
// lower-left nodes.
//
// ENO2 through shared differences: on a line f, the first differences
// D(c+1/2) = f(c+1) - f(c) and second differences S(c) = D(c+1/2) - D(c-1/2)
// are computed once per tile (with a halo) into shared memory, and each
// point's ENO2 value is one FMA on them:
//   upwind from the left:  eno2 = 2 D(i-1/2) + (|S(i)| > |S(i-1)| ? S(i-1) : S(i))
//   upwind from the right: eno2 = -2 D(i+1/2) + (|S(i)| > |S(i+1)| ? S(i+1) : S(i))
// These are the values of eno2(p0..p3) in step.cuh operation for operation
// (p0 - p1, p1 - p2 and p2 - p3 are the D's up to exact negations, and
// (-a) - (-b) rounds as b - a), so the result is the same double.  A point
// costs three FP64 operations per direction plus its share of the tile's
// halo instead of six.  The reference map X is unwrapped across the periodic
// seam by the column's offset (+-lx) before differencing, as the per-point
// form adds it to each shifted value.
constexpr int ATX = 32, ATY = 8;
constexpr int ADXW = ATX + 3;  // D(c+1/2), tile columns c = -2..ATX
constexpr int ASXW = ATX + 2;  // S(c), c = -1..ATX
constexpr int ADYH = ATY + 3;  // D(r+1/2), tile rows r = -2..ATY
constexpr int ASYH = ATY + 2;  // S(r), r = -1..ATY
constexpr int ACOLS = ATX + 4; // tile columns -2..ATX+1

__device__ __forceinline__ double eno_left(const double *d, const double *s, int k) {
    // d[k] = D(i-1/2), s[k] = S(i), s[k-1] = S(i-1)
    const double s0 = s[k], s1 = s[k - 1];
    return fma(2.0, d[k], mag_gt(s0, s1) ? s1 : s0);
}
__device__ __forceinline__ double eno_right(const double *d, const double *s, int k) {
    // d[k+1] = D(i+1/2), s[k] = S(i), s[k+1] = S(i+1)
    const double s0 = s[k], s1 = s[k + 1];
    return fma(-2.0, d[k + 1], mag_gt(s0, s1) ? s1 : s0);
}

template <int NF> struct eno_tile {
    double dx[NF][ATY][ADXW];
    double dy[NF][ADYH][ATX];
    double sx[NF][ATY][ASXW];
    double sy[NF][ASYH][ATX];
    double xo[ACOLS];  // X offset of the unwrapped column
    int col[ACOLS];    // storage column of tile column c-2
};
typedef eno_tile<F_COUNT> adv_tile;

// Storage column and X offset of every tile column (unwrapped column
// i0 + t - 2 for t = 0..ACOLS-1); threads 0..ACOLS-1 write them.
template <int NF> __device__ __forceinline__ void tile_columns(eno_tile<NF> &T, int i0, int m, double lx) {
    const int tid = threadIdx.y * ATX + threadIdx.x;
    if (tid < ACOLS) {
        const int u = i0 + tid - 2;  // unwrapped column
        int w = u % m;
        if (w < 0) w += m;
        T.col[tid] = w;
        T.xo[tid] = u < 0 ? -lx : (u >= m ? lx : 0.0);
    }
}

// Fills the tile's first and second differences of NF fields over cell rows
// j0..j0+ATY-1 (x) and rows j0-2..j0+ATY+1 (y), after tile_columns and a
// barrier.  get(f, row, t) reads field f at row -1..n and tile column t;
// rows below low(f) (-1 for the stored fields, 0 for the node velocity) and
// above n hold no value, and the differences that would need them are never
// used.  Field xf (the reference map X) is unwrapped across the periodic
// seam.  Ends with __syncthreads.
template <int NF, typename Get, typename Low>
__device__ __forceinline__ void tile_differences(eno_tile<NF> &T, int i0, int j0, int m, int n, int xf, Get get,
                                                 Low low) {
    const int tid = threadIdx.y * ATX + threadIdx.x;
    for (int k = tid; k < NF * ATY * ADXW; k += ATX * ATY) {
        const int f = k / (ATY * ADXW), rem = k - f * (ATY * ADXW), r = rem / ADXW, cc = rem - r * ADXW;
        const int jj = j0 + r;
        double d = 0;
        if (jj < n) {
            double hi = get(f, jj, cc + 1), lo = get(f, jj, cc);
            if (f == xf) {
                if (T.xo[cc + 1] != 0) hi += T.xo[cc + 1];
                if (T.xo[cc] != 0) lo += T.xo[cc];
            }
            d = hi - lo;
        }
        T.dx[f][r][cc] = d;
    }
    for (int k = tid; k < NF * ADYH * ATX; k += ATX * ATY) {
        const int f = k / (ADYH * ATX), rem = k - f * (ADYH * ATX), r = rem / ATX, cc = rem - r * ATX;
        const int jj = j0 + r - 2, ii = i0 + cc;
        double d = 0;
        if (jj >= low(f) && jj + 1 <= n && ii < m) d = get(f, jj + 1, cc + 2) - get(f, jj, cc + 2);
        T.dy[f][r][cc] = d;
    }
    __syncthreads();
    for (int k = tid; k < NF * ATY * ASXW; k += ATX * ATY) {
        const int f = k / (ATY * ASXW), rem = k - f * (ATY * ASXW), r = rem / ASXW, cc = rem - r * ASXW;
        T.sx[f][r][cc] = T.dx[f][r][cc + 1] - T.dx[f][r][cc];
    }
    for (int k = tid; k < NF * ASYH * ATX; k += ATX * ATY) {
        const int f = k / (ASYH * ATX), rem = k - f * (ASYH * ATX), r = rem / ATX, cc = rem - r * ATX;
        T.sy[f][r][cc] = T.dy[f][r + 1][cc] - T.dy[f][r][cc];
    }
    __syncthreads();
}

// ENO2 values of a point at tile column tx / row ty from the tile (the
// factor hs is applied by the caller).
template <int NF>
__device__ __forceinline__ double tile_eno_x(const eno_tile<NF> &T, int f, int ty, int tx, bool from_left) {
    const double *d = T.dx[f][ty], *s = T.sx[f][ty];
    const int k = tx + 1;
    return from_left ? eno_left(d, s, k) : eno_right(d, s, k);
}
// y direction with the one-sided wall rows: `inner` is false on the last row
// before the wall on the upwind side.
template <int NF>
__device__ __forceinline__ double tile_eno_y(const eno_tile<NF> &T, int f, int ty, int tx, bool from_below,
                                             bool inner) {
    const int ky = ty + 1;
    const double s0 = T.sy[f][ky][tx];
    if (from_below) {
        const double d = T.dy[f][ky][tx];
        if (!inner) return 2 * d;
        const double s1 = T.sy[f][ky - 1][tx];
        return fma(2.0, d, mag_gt(s0, s1) ? s1 : s0);
    }
    const double d = T.dy[f][ky + 1][tx];
    if (!inner) return -2 * d;
    const double s1 = T.sy[f][ky + 1][tx];
    return fma(-2.0, d, mag_gt(s0, s1) ? s1 : s0);
}

// ---- TMA staging of the field tiles -----------------------------------------
// Rows of the staged tile: cell rows j0-2..j0+ATY+1 (storage rows j0-1..).
constexpr int AROWS = ATY + 4;
constexpr unsigned kTileBytes = F_COUNT * AROWS * ACOLS * sizeof(double);
// Iterations of the bounded wait on the tile copies (each try_wait itself
// suspends for a while); past it the block flags F.flags[FL_TMA].
constexpr int kTmaWaitIters = 1 << 20;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// 2D tiled TMA load of box (x, y) of `map` into dst, completing on bar.
// x (the column) must be even for FP64 (16-byte rule); it and y may lie
// outside the tensor, whose missing elements arrive as zeros.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_addr(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// Bounded wait for phase 0 of bar; false when it ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar) {
    for (int it = 0; it < kTmaWaitIters; it++)
        if (mbar_try_wait(bar, 0)) return true;
    return false;
}

// Per-launch constants of the step that depend on dt (computed on the host
// with the same operations the per-thread code used).
struct advect_consts {
    double hx, hy;  // dt/(2 dx), dt/(2 dy)
    double xf, yf;  // 1/(2 dt dx), 1/(2 dt dy) of projection_step
};

struct adv_smem {
    double tile[F_COUNT][AROWS][ACOLS];  // staged fields, first: 128-byte aligned
    adv_tile T;
    uint64_t bar;
};

__global__ void __launch_bounds__(ATX * ATY) k_advect(step_consts c, advect_consts a, const __grid_constant__ field_maps maps,
                                                      fields_dev F, int cur, double dt, double bv, int emit_source) {
    extern __shared__ __align__(128) unsigned char adv_raw[];
    adv_smem &Sm = *reinterpret_cast<adv_smem *>(adv_raw + ((128 - (smem_addr(adv_raw) & 127)) & 127));
    adv_tile &T = Sm.T;
    const int m = c.m, n = c.n;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * ATX + tx;
    const int i0 = blockIdx.x * ATX, j0 = blockIdx.y * ATY;
    const int i = i0 + tx, j = j0 + ty;
    if (c.clock) cur = (int)c.clock[CLK_CUR];
    const double *__restrict__ const *A = F.f[cur];
    double *const *B = F.f[cur ^ 1];
    // One thread copies the seven field tiles (columns i0-2.., storage rows
    // j0-1..) by TMA while the block sets up the column tables.
    if (tid == 0) mbar_init(&Sm.bar, 1);
    tile_columns(T, i0, m, c.lx);
    __syncthreads();
    if (tid == 0) {
        mbar_expect_tx(&Sm.bar, kTileBytes);
        for (int f = 0; f < F_COUNT; f++) tma_load_2d(&Sm.tile[f][0][0], &maps.f[cur][f], i0 - 2, j0 - 1, &Sm.bar);
    }
    if (__syncthreads_or(!mbar_wait_bounded(&Sm.bar))) {
        // a copy did not arrive in time: flag it, wait once more for the
        // copies in flight, and leave this tile of the next state unwritten
        if (tid == 0) atomicExch(&F.flags[FL_TMA], 1);
        mbar_wait_bounded(&Sm.bar);
        return;
    }
    // Columns across the periodic seam arrive as zeros: blocks at either end
    // fetch them from their wrapped columns.
    if (i0 == 0 || i0 + ACOLS - 2 > m) {
        for (int k = tid; k < F_COUNT * AROWS * ACOLS; k += ATX * ATY) {
            const int f = k / (AROWS * ACOLS), rem = k - f * (AROWS * ACOLS), r = rem / ACOLS, t = rem - r * ACOLS;
            const int u = i0 + t - 2, sr = j0 - 1 + r;
            if ((u < 0 || u >= m) && sr >= 0 && sr <= n + 1) Sm.tile[f][r][t] = A[f][(size_t)sr * m + T.col[t]];
        }
        __syncthreads();
    }
    tile_differences<F_COUNT>(
        T, i0, j0, m, n, F_X, [&](int f, int row, int t) { return Sm.tile[f][row - j0 + 2][t]; },
        [](int) { return -1; });
    if (i >= m || j >= n) return;
    const double hx = a.hx, hy = a.hy;
    const size_t ci = (size_t)(j + 1) * m + i;
    const int ir = T.col[tx + 3];
    if (c.clock) bv = c.clock[CLK_BV_STATE];
    velo V{F.vel, m, n, bv};
    // Upwind ENO values without the factor hs = +-dt/(2 dx); it is folded
    // into the velocity: -u * (hs * eno) = -(u * hs) * eno.
    // reference map at node (i,j), rows 1..n-1 (shear_sim.cc:310-327)
    if (j > 0) {
        const double Xc = Sm.tile[F_X][ty + 2][tx + 2], Yc = Sm.tile[F_Y][ty + 2][tx + 2];
        double ex_X, ex_Y, ey_X, ey_Y;
        const double un = V.u(i, j), vn = V.v(i, j);
        const double uh = un * (un > 0 ? hx : -hx), vh = vn * (vn > 0 ? hy : -hy);
        ex_X = tile_eno_x(T, F_X, ty, tx, un > 0);
        ex_Y = tile_eno_x(T, F_Y, ty, tx, un > 0);
        const bool inner = vn > 0 ? j > 1 : j < n - 1;
        ey_X = tile_eno_y(T, F_X, ty, tx, vn > 0, inner);
        ey_Y = tile_eno_y(T, F_Y, ty, tx, vn > 0, inner);
        B[F_X][ci] = Xc + fma(-vh, ey_X, -uh * ex_X);
        B[F_Y][ci] = Yc + fma(-vh, ey_Y, -uh * ex_Y);
    }
    // staggered velocity and spin (shear_sim.cc:330-333)
    const double u00 = V.u(i, j), u10 = V.u(ir, j), u01 = V.u(i, j + 1), u11 = V.u(ir, j + 1);
    const double v00 = V.v(i, j), v10 = V.v(ir, j), v01 = V.v(i, j + 1), v11 = V.v(ir, j + 1);
    const double uc = 0.25 * (u00 + u10 + u01 + u11), vc = 0.25 * (v00 + v10 + v01 + v11);
    const double two_omega = hx * (-v00 + v10 - v01 + v11) - hy * (-u00 - u10 + u01 + u11);
    const double uh = uc * (uc > 0 ? hx : -hx), vh = vc * (vc > 0 ? hy : -hy);
    // ENO derivatives of p, q, s, tau, chi (shear_sim.cc:336-338)
    double f1[5], f2[5];
    const bool inner = vc > 0 ? j > 0 : j < n - 1;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        f1[k] = tile_eno_x(T, k, ty, tx, uc > 0);
        f2[k] = tile_eno_y(T, k, ty, tx, vc > 0, inner);
    }
    const double p = Sm.tile[F_P][ty + 2][tx + 2], q = Sm.tile[F_Q][ty + 2][tx + 2];
    const double s = Sm.tile[F_S][ty + 2][tx + 2], t = Sm.tile[F_TAU][ty + 2][tx + 2];
    double cchi = Sm.tile[F_CHI][ty + 2][tx + 2] + fma(-vh, f2[4], -uh * f1[4]), ddev, dtmp;
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
        const double pq = pn + qn, Aa = pq - sn, Bb = pq + sn;
        F.pre[0][ci] = a.xf * Aa + a.yf * tn;
        F.pre[1][ci] = a.xf * Aa - a.yf * tn;
        F.pre[2][ci] = a.xf * tn - a.yf * Bb;
        F.pre[3][ci] = a.xf * tn + a.yf * Bb;
    }
}

// ---- float-float advection (mixed-precision handles) ------------------------
// The same step with the ENO differences, the upwind products and the
// increments in float-float (double-word) arithmetic on the FP32 pipe while
// the state stays FP64.  Every staged value is split on the integer pipe
// into a float pair hi + lo (ff_split_d, 48 of its 53 significant bits); each
// first difference f(c+1) - f(c) is formed from the pairs by TwoSum and kept
// as a pair (relative error ~2^-44 of the difference, plus ~2^-47 of the
// values); the ENO value is the chosen second difference plus twice the
// centre difference, the increment u hs eno in both directions with the
// product errors (FMA) and the sums by TwoSum, and the spin from pair
// differences of the node velocities.  Each field takes its increment with
// two FP64 additions (hi, then lo), so the state carries the rounding of the
// FP64 path plus ~2^-44 of the increment per step.  The ENO choice
// |S(i)| > |S(i-1)| is taken on the pair second differences where the two
// magnitudes differ by more than their error bound; near ties between
// different values it is recomputed in FP64 from the staged tile with
// k_advect's operations, so the choice is always the FP64 path's (a
// different choice changes the value by the difference of two second
// differences, which near an inflection is not small).  The yield test runs on a float-float stress norm; cells near or
// above a cut-off take the FP64 norm and the FP64 plastic law as k_advect
// does.  The net force is formed by k_source_ff from the stresses, so no
// per-cell combinations are written.  GB300 issues FP64 at 1/57 of the FP32
// rate; an elastic cell here needs two FP64 additions per field.
// Shared memory of k_advect_ff: the split values, then the FP64 tile (the
// TMA destination, needed only until it is split) overlaid by the first
// differences, so that three blocks fit on an SM.
struct adv_smem_ff {
    float2 t2[F_COUNT][AROWS][ACOLS];  // staged values as (hi, lo) pairs: one 64-bit access each
    union {
        double tile[F_COUNT][AROWS][ACOLS];  // staged fields (128-byte aligned: 24192 B precede it)
        struct {
            float2 dx[F_COUNT][ATY][ADXW];  // first differences in x (pairs): tile columns cc, cc+1
            float2 dy[F_COUNT][ADYH][ATX];  // first differences in y (pairs): tile rows r, r+1
        } d;
    } u;
    ff nu[ATY + 1][ATX + 1];  // node velocities (i0+c, j0+r) as pairs, walls substituted
    ff nv[ATY + 1][ATX + 1];
    int xs[ACOLS];   // period shift of the unwrapped column: -1, 0, +1
    int col[ACOLS];  // storage column of tile column c-2
    uint64_t bar;
};
static_assert(sizeof(float) * 2 * F_COUNT * AROWS * ACOLS % 128 == 0, "the TMA tile must stay 128-byte aligned");

__device__ __forceinline__ ff split_ff(double d) {
    ff r;
    ff_split_d(d, r.hi, r.lo);
    return r;
}

// a - b for pairs a = (ah, al), b = (bh, bl): TwoSum of the high parts, the
// low parts added to its error, renormalised.
__device__ __forceinline__ ff ff_pair_diff(float ah, float al, float bh, float bl) {
    const float s = ah - bh, bb = s - ah;
    float e = (ah - (s - bb)) + (-bh - bb);
    e += al - bl;
    return ff_fast2sum(s, e);
}
__device__ __forceinline__ ff ff_x2(ff a) { return ff{2.f * a.hi, 2.f * a.lo}; }
__device__ __forceinline__ float ffabs_hi(ff a) { return fabsf(a.hi); }

// FP64 choice of k_advect in x (tile_differences with the X column
// offsets, then eno_left / eno_right's magnitude test) from the state in
// global memory (row: storage row, cols: the tile's storage columns, xs: the
// tile's period shifts): true where it takes the outer second difference.
__device__ __noinline__ bool pick_x64(const double *__restrict__ f, size_t row, const int *cols, const int *xs,
                                      bool is_x, double lx, int tx, bool from_left) {
    const int c0 = from_left ? tx : tx + 1;  // tile columns c0 .. c0+3
    double g[4];
    for (int q = 0; q < 4; q++) {
        g[q] = f[row + cols[c0 + q]];
        if (is_x && xs[c0 + q] != 0) g[q] += xs[c0 + q] < 0 ? -lx : lx;
    }
    const double da = g[1] - g[0], db = g[2] - g[1], dc = g[3] - g[2];
    // from the left: s0 = S(i) = dc - db, s1 = S(i-1) = db - da;
    // from the right: s0 = S(i) = db - da, s1 = S(i+1) = dc - db
    return from_left ? mag_gt(dc - db, db - da) : mag_gt(db - da, dc - db);
}
// FP64 choice in y (difference r between cell rows j0+r-2 and j0+r-1, zero
// where k_advect's tile_differences leaves it zero) at storage column i.
__device__ __noinline__ bool pick_y64(const double *__restrict__ f, int m, int i, int ty, bool from_below, int j0,
                                      int n) {
    const int r0 = from_below ? ty : ty + 1;  // differences r0 .. r0+2
    double d[3];
    for (int q = 0; q < 3; q++) {
        const int r = r0 + q, jj = j0 + r - 2;  // cell rows jj, jj+1 = storage rows jj+1, jj+2
        d[q] = (jj >= -1 && jj + 1 <= n) ? f[(size_t)(jj + 2) * m + i] - f[(size_t)(jj + 1) * m + i] : 0.0;
    }
    return from_below ? mag_gt(d[2] - d[1], d[1] - d[0]) : mag_gt(d[1] - d[0], d[2] - d[1]);
}

// ENO2 value from three consecutive first differences Da, Db, Dc around the
// point (Db is the upwind centre difference): from the left (outer = Db - Da)
// 2 Db + (|Dc - Db| > |Db - Da| ? Db - Da : Dc - Db); from the right
// (outer = Dc - Db) -2 Db + (|Db - Da| > |Dc - Db| ? Dc - Db : Db - Da).
// The second differences are pairs; their magnitudes are compared in pairs
// too, decided where they differ by more than the pairs' error bound (the
// differences' ~2^-44 plus the split's ~2^-47 of the values, with room).
// Within the margin, candidates of the same sign (equal up to the margin)
// give values within the float-float path's own error either way; a near tie
// of opposite signs (the candidates differ by twice their size) takes the
// inner candidate below kEnoTieRel of the field's scale and `exact`, the
// FP64 path's own choice, above it.
__device__ __forceinline__ ff ff_abs(ff a) { return a.hi < 0.f ? ff_neg(a) : a; }
constexpr float kEnoTieRel = 1e-10f;
template <typename Exact>
__device__ __forceinline__ ff eno_ff(ff Da, ff Db, ff Dc, bool from_left, float vmag, Exact exact) {
    // second differences from the high parts: within |lo| parts and one
    // float rounding of the pairs' values, themselves within ~2^-44 of the
    // differences and ~2^-47 of the values of the exact ones
    const float fab = Db.hi - Da.hi, fbc = Dc.hi - Db.hi;
    const float fin = from_left ? fbc : fab, fout = from_left ? fab : fbc;
    const float gap0 = fabsf(fin) - fabsf(fout);
    const float big = fabsf(Da.hi) + 2.f * fabsf(Db.hi) + fabsf(Dc.hi);
    // bounds the low parts (<= 2^-24 big), one float rounding of each second
    // difference (<= 2.4e-7 (|fin| + |fout|) <= 2.4e-7 big) and the pairs'
    // own error (1e-12 big + 4e-13 vmag)
    const float m0 = 3.1e-7f * big + 4e-13f * vmag;
    bool take_outer;
    if (fabsf(gap0) > m0) {
        take_outer = gap0 > 0.f;
    } else {
        const ff sab = ff_sub(Db, Da), sbc = ff_sub(Dc, Db);
        const ff inner = from_left ? sbc : sab, outer = from_left ? sab : sbc;
        const ff g = ff_sub(ff_abs(inner), ff_abs(outer));
        const float gap = g.hi + g.lo;
        const float margin = 1e-12f * big + 4e-13f * vmag, small = kEnoTieRel * (vmag + big);
        if (fabsf(gap) > margin) take_outer = gap > 0.f;
        // Within the margin the two candidates differ by at most |gap| plus
        // its error where they have the same sign (or one is zero): either
        // choice then moves the value by less than ~2e-12 (|value| +
        // |differences|) times the upwind factor.  Of opposite signs they
        // differ by twice their size: below kEnoTieRel (|value| +
        // |differences|) that is grid-scale noise of the field at the level
        // of the solver's tolerance, and the inner candidate is taken; above
        // it the FP64 path's own choice.
        else if (inner.hi * outer.hi >= 0.f || (fabsf(inner.hi) <= small && fabsf(outer.hi) <= small))
            take_outer = false;
        else take_outer = exact();
    }
    // outer: from the left Db - Da, from the right Dc - Db
    const bool lower = from_left == take_outer;
    const ff s = ff_sub(lower ? Db : Dc, lower ? Da : Db);
    return ff_add(from_left ? ff_x2(Db) : ff_neg(ff_x2(Db)), s);
}

__device__ __forceinline__ ff dx_pair(const adv_smem_ff &Sm, int f, int ty, int c) {
    const float2 v = Sm.u.d.dx[f][ty][c];
    return ff{v.x, v.y};
}
__device__ __forceinline__ ff dy_pair(const adv_smem_ff &Sm, int f, int r, int tx) {
    const float2 v = Sm.u.d.dy[f][r][tx];
    return ff{v.x, v.y};
}

// Where the FP64 choice is needed, the state buffer read (A), the point's
// storage row and the tile geometry.
struct eno_ctx {
    const double *__restrict__ const *A;
    int m, n, j0, j;
    double lx;
};

__device__ __forceinline__ ff eno_x_ff(const adv_smem_ff &Sm, const eno_ctx &e, int f, int ty, int tx,
                                       bool from_left) {
    const int c = from_left ? tx : tx + 1;  // differences c .. c+2 (tile columns c .. c+3)
    const float vmag = fabsf(Sm.t2[f][ty + 2][tx + 2].x);
    return eno_ff(dx_pair(Sm, f, ty, c), dx_pair(Sm, f, ty, c + 1), dx_pair(Sm, f, ty, c + 2), from_left, vmag, [&] {
        return pick_x64(e.A[f], (size_t)(e.j + 1) * e.m, Sm.col, Sm.xs, f == F_X, e.lx, tx, from_left);
    });
}
// y with the one-sided wall rows: `inner` is false on the last row before
// the wall on the upwind side (value +-2 Db there).
__device__ __forceinline__ ff eno_y_ff(const adv_smem_ff &Sm, const eno_ctx &e, int f, int ty, int tx,
                                       bool from_below, bool inner) {
    const int r = from_below ? ty : ty + 1;  // differences r .. r+2
    const ff Db = dy_pair(Sm, f, r + 1, tx);
    if (!inner) return from_below ? ff_x2(Db) : ff_neg(ff_x2(Db));
    const float vmag = fabsf(Sm.t2[f][ty + 2][tx + 2].x);
    return eno_ff(dy_pair(Sm, f, r, tx), Db, dy_pair(Sm, f, r + 2, tx), from_below, vmag, [&] {
        return pick_y64(e.A[f], e.m, Sm.col[tx + 2], ty, from_below, e.j0, e.n);
    });
}

// -(uh eno_x + vh eno_y)
__device__ __forceinline__ ff upwind_inc(ff uh, ff ex, ff vh, ff ey) {
    return ff_neg(ff_add(ff_mul(uh, ex), ff_mul(vh, ey)));
}
// a + inc for the FP64 state value a with one FP64 addition (the pair formed
// as a double on the integer pipe)
__device__ __forceinline__ double add_ff(double a, ff inc) { return a + ff_to_d(inc.hi, inc.lo); }
// u > 0 for a finite double, on the integer pipe
__device__ __forceinline__ bool dpos(double u) { return __double_as_longlong(u) > 0; }

// Float-float pairs of the per-launch constants hx, hy and of the period lx.
struct advect_ff_consts {
    float hxh, hxl, hyh, hyl, lxh, lxl;
};

// Node velocity as float pairs, the walls' +-bv substituted (no FP64 work).
struct velo_ff {
    const double2 *vel;
    int m, n;
    ff bv;
    __device__ __forceinline__ ff u(int i, int j) const {
        return j == 0 ? ff_neg(bv) : (j == n ? bv : split_ff(vel[(size_t)j * m + i].x));
    }
    __device__ __forceinline__ ff v(int i, int j) const {
        return (j == 0 || j == n) ? ff{0.f, 0.f} : split_ff(vel[(size_t)j * m + i].y);
    }
};

__global__ void __launch_bounds__(ATX * ATY, 3)
    k_advect_ff(step_consts c, advect_ff_consts h, const __grid_constant__ field_maps maps, fields_dev F, int cur,
                double dt, double bv) {
    extern __shared__ __align__(128) unsigned char adv_raw_ff[];
    adv_smem_ff &Sm = *reinterpret_cast<adv_smem_ff *>(adv_raw_ff + ((128 - (smem_addr(adv_raw_ff) & 127)) & 127));
    const int m = c.m, n = c.n;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * ATX + tx;
    const int i0 = blockIdx.x * ATX, j0 = blockIdx.y * ATY;
    const int i = i0 + tx, j = j0 + ty;
    if (c.clock) cur = (int)c.clock[CLK_CUR];
    const double *__restrict__ const *A = F.f[cur];
    double *const *B = F.f[cur ^ 1];
    if (tid == 0) mbar_init(&Sm.bar, 1);
    if (tid < ACOLS) {
        const int u = i0 + tid - 2;
        int w = u % m;
        if (w < 0) w += m;
        Sm.col[tid] = w;
        Sm.xs[tid] = u < 0 ? -1 : (u >= m ? 1 : 0);
    }
    __syncthreads();
    if (tid == 0) {
        mbar_expect_tx(&Sm.bar, kTileBytes);
        for (int f = 0; f < F_COUNT; f++) tma_load_2d(&Sm.u.tile[f][0][0], &maps.f[cur][f], i0 - 2, j0 - 1, &Sm.bar);
    }
    // node velocities of the block as pairs while the tile arrives
    if (c.clock) bv = c.clock[CLK_BV_STATE];
    {
        const velo_ff V{F.vel, m, n, split_ff(bv)};
        for (int p = tid; p < (ATY + 1) * (ATX + 1); p += ATX * ATY) {
            const int r = p / (ATX + 1), cc = p - r * (ATX + 1), nj = j0 + r;
            if (nj > n) continue;
            const int ni = Sm.col[cc + 2];
            Sm.nu[r][cc] = V.u(ni, nj);
            Sm.nv[r][cc] = V.v(ni, nj);
        }
    }
    if (__syncthreads_or(!mbar_wait_bounded(&Sm.bar))) {
        if (tid == 0) atomicExch(&F.flags[FL_TMA], 1);
        mbar_wait_bounded(&Sm.bar);
        return;
    }
    constexpr int kTileVals = F_COUNT * AROWS * ACOLS;
    // columns across the periodic seam arrive as zeros: edge blocks fetch them
    if (i0 == 0 || i0 + ACOLS - 2 > m) {
        for (int k = tid; k < kTileVals; k += ATX * ATY) {
            const int f = k / (AROWS * ACOLS), rem = k - f * (AROWS * ACOLS), r = rem / ACOLS, t = rem - r * ACOLS;
            const int u = i0 + t - 2, sr = j0 - 1 + r;
            if ((u < 0 || u >= m) && sr >= 0 && sr <= n + 1) Sm.u.tile[f][r][t] = A[f][(size_t)sr * m + Sm.col[t]];
        }
        __syncthreads();
    }
    // split every staged value into a float pair (one position per thread and
    // pass, all fields: the position's index arithmetic is done once)
    for (int p = tid; p < AROWS * ACOLS; p += ATX * ATY) {
        const int r = p / ACOLS, t = p - r * ACOLS;
#pragma unroll
        for (int f = 0; f < F_COUNT; f++) {
            float hh, ll;
            ff_split_d(Sm.u.tile[f][r][t], hh, ll);
            Sm.t2[f][r][t] = make_float2(hh, ll);
        }
    }
    __syncthreads();
    // first differences: x on cell rows j0..j0+ATY-1, y on rows j0-2..j0+ATY+1;
    // X across the periodic seam gets the period (the unwrapped difference)
    const ff lx{h.lxh, h.lxl};
    for (int p = tid; p < ATY * ADXW; p += ATX * ATY) {
        const int r = p / ADXW, cc = p - r * ADXW;
        const bool live = j0 + r < n;
        const int sh = Sm.xs[cc + 1] - Sm.xs[cc];
#pragma unroll
        for (int f = 0; f < F_COUNT; f++) {
            ff d{0.f, 0.f};
            if (live) {
                const float2 a = Sm.t2[f][r + 2][cc + 1], b = Sm.t2[f][r + 2][cc];
                d = ff_pair_diff(a.x, a.y, b.x, b.y);
                if (f == F_X && sh != 0) d = ff_add(d, sh > 0 ? lx : ff_neg(lx));
            }
            Sm.u.d.dx[f][r][cc] = make_float2(d.hi, d.lo);
        }
    }
    for (int p = tid; p < ADYH * ATX; p += ATX * ATY) {
        const int r = p / ATX, cc = p - r * ATX;
        const int jj = j0 + r - 2;
        const bool live = jj >= -1 && jj + 1 <= n && i0 + cc < m;
#pragma unroll
        for (int f = 0; f < F_COUNT; f++) {
            ff d{0.f, 0.f};
            if (live) {
                const float2 a = Sm.t2[f][r + 1][cc + 2], b = Sm.t2[f][r][cc + 2];
                d = ff_pair_diff(a.x, a.y, b.x, b.y);
            }
            Sm.u.d.dy[f][r][cc] = make_float2(d.hi, d.lo);
        }
    }
    __syncthreads();
    if (i >= m || j >= n) return;
    const ff hx{h.hxh, h.hxl}, hy{h.hyh, h.hyl};
    const size_t ci = (size_t)(j + 1) * m + i;
    const eno_ctx e{A, m, n, j0, j, c.lx};
    // reference map at node (i,j), rows 1..n-1 (shear_sim.cc:310-327)
    if (j > 0) {
        const ff un = Sm.nu[ty][tx], vn = Sm.nv[ty][tx];
        const bool ru = un.hi > 0.f, rv = vn.hi > 0.f;
        const ff uh = ff_mul(un, ru ? hx : ff_neg(hx)), vh = ff_mul(vn, rv ? hy : ff_neg(hy));
        const bool inner = rv ? j > 1 : j < n - 1;
#pragma unroll
        for (int f = F_X; f <= F_Y; f++) {
            const ff ex = eno_x_ff(Sm, e, f, ty, tx, ru), ey = eno_y_ff(Sm, e, f, ty, tx, rv, inner);
            B[f][ci] = add_ff(A[f][ci], upwind_inc(uh, ex, vh, ey));
        }
    }
    // staggered velocity and spin (shear_sim.cc:330-333) in pairs
    const ff u00 = Sm.nu[ty][tx], u10 = Sm.nu[ty][tx + 1], u01 = Sm.nu[ty + 1][tx], u11 = Sm.nu[ty + 1][tx + 1];
    const ff v00 = Sm.nv[ty][tx], v10 = Sm.nv[ty][tx + 1], v01 = Sm.nv[ty + 1][tx], v11 = Sm.nv[ty + 1][tx + 1];
    ff uc = ff_add(ff_add(u00, u10), ff_add(u01, u11)), vc = ff_add(ff_add(v00, v10), ff_add(v01, v11));
    uc = ff{0.25f * uc.hi, 0.25f * uc.lo};
    vc = ff{0.25f * vc.hi, 0.25f * vc.lo};
    const ff two_omega = ff_sub(ff_mul(hx, ff_add(ff_sub(v10, v00), ff_sub(v11, v01))),
                                ff_mul(hy, ff_add(ff_sub(u01, u00), ff_sub(u11, u10))));
    const bool ru = uc.hi > 0.f, rv = vc.hi > 0.f;
    const ff uh = ff_mul(uc, ru ? hx : ff_neg(hx)), vh = ff_mul(vc, rv ? hy : ff_neg(hy));
    const bool inner = rv ? j > 0 : j < n - 1;
    auto inc_of = [&](int f) {
        return upwind_inc(uh, eno_x_ff(Sm, e, f, ty, tx, ru), vh, eno_y_ff(Sm, e, f, ty, tx, rv, inner));
    };
    const float2 q2 = Sm.t2[F_Q][ty + 2][tx + 2], s2 = Sm.t2[F_S][ty + 2][tx + 2], t2 = Sm.t2[F_TAU][ty + 2][tx + 2];
    const ff qf{q2.x, q2.y}, sf{s2.x, s2.y}, tf{t2.x, t2.y};
    const double ddev = 0;
    // chi first, then p, q, s, tau
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int f = k == 0 ? F_CHI : k - 1;
        ff inc = inc_of(f);
        if (f == F_S) inc = ff_add(inc, ff_mul(two_omega, tf));
        else if (f == F_TAU) inc = ff_sub(inc, ff_mul(two_omega, sf));
        const double a0 = A[f][ci];
        double v = add_ff(a0, inc);
        if (f == F_CHI) {
            // Yield test: 3q^2 + s^2 + tau^2 in pairs (relative error ~2^-44);
            // a cell clearly below the cut-offs of k_advect (1e-24, or an
            // athermal law below yield) is elastic there too; any other cell
            // takes k_advect's FP64 path.
            const ff dsq = ff_add(ff_mul(ff{3.f, 0.f}, ff_mul(qf, qf)), ff_add(ff_mul(sf, sf), ff_mul(tf, tf)));
            const float dv = dsq.hi + dsq.lo;
            const bool athermal = c.stz_model >= 2;
            const bool clearly_elastic = dv < 0.999e-24f * (1.f - 1e-6f) || (athermal && dv < c.yield_cut2f);
            // the FP64 test and the plastic law run in k_plastic_ff, on the
            // listed cells after this kernel (kept out of this one, whose
            // registers they would otherwise set)
            if (!clearly_elastic) F.plist[atomicAdd(F.pcount, 1u)] = (unsigned)ci;
            F.ddev[ci] = ddev;
        }
        B[f][ci] = v;
    }
}

// The plastic part of the float-float step for the cells k_advect_ff listed:
// k_advect's FP64 yield test and, above the cut-offs, the FP64 plastic law
// (adaptive_plastic_term, shear_sim.cc:513-548) on the advected chi, then
// q, s, tau -= dtmp times their old values, ddev and the plastic strain.  The
// same operations in the same order as k_advect, so the cell ends where the
// one-pass form would take it.
__global__ void k_plastic_ff(step_consts c, fields_dev F, int cur, double dt) {
    if (c.clock) cur = (int)c.clock[CLK_CUR];
    const unsigned cnt = *F.pcount;
    const double *__restrict__ const *A = F.f[cur];
    double *const *B = F.f[cur ^ 1];
    const bool athermal = c.stz_model >= 2;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
        const size_t ci = F.plist[k];
        const double q = A[F_Q][ci], s = A[F_S][ci], t = A[F_TAU][ci];
        const double devsq = 3 * q * q + s * s + t * t;
        const long long dbits = __double_as_longlong(devsq);
        if (dbits < __double_as_longlong(0.999e-24) || (athermal && dbits < __double_as_longlong(c.yield_cut2)))
            continue;
        int iters;
        double chi = B[F_CHI][ci], ddev = 0;
        const stz_law_params<double> lp = law_params(c);
        const double dtmp = adaptive_plastic(lp, sqrt(devsq), chi, ddev, dt, iters);
        if (iters >= c.substep_cap) atomicExch(&F.flags[FL_SUBSTEP_CAP], 1);
        if (iters > 1) atomicMax(&F.flags[FL_SUBSTEP_MAX], iters);
        B[F_CHI][ci] = chi;
        F.ddev[ci] = ddev;
        if (c.track_plastic && ddev != 0) {
            const int m = c.m, j = (int)(ci / (size_t)m) - 1, i = (int)(ci - (size_t)(j + 1) * m);
            F.eps_pl[(size_t)j * m + i] += ddev / (2 * c.mu);
        }
        if (dtmp != 0) {
            B[F_Q][ci] -= dtmp * q;
            B[F_S][ci] -= dtmp * s;
            B[F_TAU][ci] -= dtmp * t;
        }
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
    double hx, hy, mu_inv;
};

// Tile fields of the explicit step: the seven stored fields, then the node
// velocity components u and v (rows 0..n, walls substituted).
enum { DF_U = F_COUNT, DF_V, DF_COUNT };
typedef eno_tile<DF_COUNT> direct_tile;

__global__ void __launch_bounds__(ATX * ATY) k_direct(step_consts c, direct_consts d, fields_dev F, int cur,
                                                      double dt, double bv) {
    extern __shared__ __align__(16) unsigned char dir_smem[];
    direct_tile &TT = *reinterpret_cast<direct_tile *>(dir_smem);
    const int m = c.m, n = c.n;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * ATX, j0 = blockIdx.y * ATY;
    const int i = i0 + tx, j = j0 + ty;
    const double *__restrict__ const *A = F.f[cur];
    double *const *B = F.f[cur ^ 1];
    velo V{F.vel, m, n, bv};
    tile_columns(TT, i0, m, c.lx);
    __syncthreads();
    tile_differences<DF_COUNT>(
        TT, i0, j0, m, n, F_X,
        [&](int f, int row, int t) {
            const int col = TT.col[t];
            return f == DF_U ? V.u(col, row) : (f == DF_V ? V.v(col, row) : A[f][(size_t)(row + 1) * m + col]);
        },
        [](int f) { return f >= DF_U ? 0 : -1; });
    if (i >= m || j >= n) return;
    const double hx = d.hx, hy = d.hy, mu_inv = d.mu_inv;
    const int il = TT.col[tx + 1], ir = TT.col[tx + 3];
    const size_t ci = IDX(i, j);
    const double *P = A[F_P], *Q = A[F_Q], *S = A[F_S], *T = A[F_TAU];
    if (j > 0) {
        const double *X = A[F_X], *Y = A[F_Y];
        const double un = V.u(i, j), vn = V.v(i, j);
        const double hsx = un > 0 ? hx : -hx, hsy = vn > 0 ? hy : -hy;
        double ux = tile_eno_x(TT, DF_U, ty, tx, un > 0), vx = tile_eno_x(TT, DF_V, ty, tx, un > 0);
        double Xx = tile_eno_x(TT, F_X, ty, tx, un > 0), Yx = tile_eno_x(TT, F_Y, ty, tx, un > 0);
        const bool inner = vn > 0 ? j > 1 : j < n - 1;
        double uy = tile_eno_y(TT, DF_U, ty, tx, vn > 0, inner), vy = tile_eno_y(TT, DF_V, ty, tx, vn > 0, inner);
        double Xy = tile_eno_y(TT, F_X, ty, tx, vn > 0, inner), Yy = tile_eno_y(TT, F_Y, ty, tx, vn > 0, inner);
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
    const bool inner = vc > 0 ? j > 0 : j < n - 1;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        f1[k] = tile_eno_x(TT, k, ty, tx, uc > 0);
        f2[k] = tile_eno_y(TT, k, ty, tx, vc > 0, inner);
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

// The projection source of the float-float path (k_advect_ff writes no
// per-cell combinations): net_force (shear_sim.cc:447-453) at the interior
// nodes from the stresses of the four surrounding cells.  A block of 32 x 32
// nodes (four rows per thread) first forms, for each of the 33 x 33 cells
// around it, the pairs
// A = p + q - s, B = p + q + s and tau from the split stresses (float-float
// sums, error ~2^-47 of the values) in shared memory; each node then takes
// the cell-to-cell differences of those pairs, whose high parts cancel
// exactly where the cells agree, so the force keeps ~2^-44 of its own size
// plus ~2^-47 of the stresses, and scales them by xf, yf in pairs.  The wall
// rows as k_source.
struct source_ff_consts {
    float xfh, xfl, yfh, yfl;
};

constexpr int SFX = 32, SFY = 8;  // threads of a block
constexpr int SFR = 4;            // node (cell) rows per thread: a block covers 32 x 32

__global__ void __launch_bounds__(SFX * SFY) k_source_ff(step_consts c, fields_dev F, int cur, source_ff_consts h,
                                                         double xbc_bv) {
    constexpr int TY = SFY * SFR;  // node rows of the block
    __shared__ ff cA[TY + 1][SFX + 1], cB[TY + 1][SFX + 1], cT[TY + 1][SFX + 1];
    const int m = c.m, n = c.n;
    if (c.clock) {
        xbc_bv = c.xbc * c.clock[CLK_BV];
        cur = (int)c.clock[CLK_CUR] ^ 1;  // the state the advection wrote
    }
    const int i0 = blockIdx.x * SFX, j0 = blockIdx.y * TY;
    const int tid = threadIdx.y * SFX + threadIdx.x;
    const double *P = F.f[cur][F_P], *Q = F.f[cur][F_Q], *S = F.f[cur][F_S], *T = F.f[cur][F_TAU];
    // cells (i0 - 1 + cc, j0 - 1 + r); storage rows -1 .. n exist.  The
    // passes go in two halves, each issuing all its loads before it splits
    // anything, so that more loads are in flight per thread.
    constexpr int kCells = (TY + 1) * (SFX + 1), kPasses = (kCells + SFX * SFY - 1) / (SFX * SFY);
    constexpr int kHalf = (kPasses + 1) / 2;
#pragma unroll
    for (int h0 = 0; h0 < kPasses; h0 += kHalf) {
        double vp[kHalf], vq[kHalf], vs[kHalf], vt[kHalf];
        int rr[kHalf], cw[kHalf];
#pragma unroll
        for (int it = 0; it < kHalf; it++) {
            const int k = tid + (h0 + it) * SFX * SFY;
            const int r = k / (SFX + 1), cc = k - r * (SFX + 1);
            const int cj = j0 - 1 + r;
            int ci = i0 - 1 + cc;
            ci = ci < 0 ? ci + m : (ci >= m ? ci % m : ci);
            const bool live = h0 + it < kPasses && k < kCells && cj <= n;
            rr[it] = live ? r : -1;
            cw[it] = cc;
            const size_t q = live ? IDX(ci, cj) : 0;
            vp[it] = live ? P[q] : 0.0;
            vq[it] = live ? Q[q] : 0.0;
            vs[it] = live ? S[q] : 0.0;
            vt[it] = live ? T[q] : 0.0;
        }
#pragma unroll
        for (int it = 0; it < kHalf; it++) {
            if (rr[it] < 0) continue;
            const ff pp = split_ff(vp[it]), qq = split_ff(vq[it]), ss = split_ff(vs[it]);
            const ff pq = ff_add(pp, qq);
            cA[rr[it]][cw[it]] = ff_sub(pq, ss);
            cB[rr[it]][cw[it]] = ff_add(pq, ss);
            cT[rr[it]][cw[it]] = split_ff(vt[it]);
        }
    }
    __syncthreads();
    const int tx = threadIdx.x, i = i0 + tx;
    if (i >= m) return;
    const ff xf{h.xfh, h.xfl}, yf{h.yfh, h.yfl};
#pragma unroll
    for (int q = 0; q < SFR; q++) {
        const int ty = threadIdx.y + q * SFY, j = j0 + ty;
        if (j > n) break;
        double2 out;
        if (j == 0 || j == n) {
            out.x = j == 0 ? -xbc_bv : xbc_bv;
            out.y = 0;
        } else {
            // cells k0 = (i-1, j-1), k1 = (i, j-1), k2 = (i-1, j), k3 = (i, j)
            const ff dAx = ff_add(ff_sub(cA[ty][tx + 1], cA[ty][tx]), ff_sub(cA[ty + 1][tx + 1], cA[ty + 1][tx]));
            const ff dBy = ff_add(ff_sub(cB[ty + 1][tx], cB[ty][tx]), ff_sub(cB[ty + 1][tx + 1], cB[ty][tx + 1]));
            const ff dTy = ff_add(ff_sub(cT[ty][tx], cT[ty + 1][tx]), ff_sub(cT[ty][tx + 1], cT[ty + 1][tx + 1]));
            const ff dTx = ff_add(ff_sub(cT[ty][tx], cT[ty][tx + 1]), ff_sub(cT[ty + 1][tx], cT[ty + 1][tx + 1]));
            const ff fx = ff_add(ff_mul(xf, dAx), ff_mul(yf, dTy)), fy = ff_add(ff_mul(xf, dTx), ff_mul(yf, dBy));
            out.x = ff_to_d(fx.hi, fx.lo);
            out.y = ff_to_d(fy.hi, fy.lo);
        }
        F.src[(size_t)j * m + i] = out;
    }
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

// The stress correction of the float-float path: each node's velocity is
// split into float pairs once (a block of 32 x 32 cells, four rows per
// thread, stages its 33 x 33 nodes in shared memory), the velocity differences of k_project are taken
// from the pairs, the products with hx, hy, K, mu/3 and mu in pairs, and each
// stress component takes its correction with two FP64 additions.
struct project_ff_consts {
    float hxh, hxl, hyh, hyl, Kh, Kl, m3h, m3l, muh, mul;
};

__global__ void __launch_bounds__(SFX * SFY) k_project_ff(step_consts c, fields_dev F, int cur, project_ff_consts h) {
    constexpr int TY = SFY * SFR;  // cell rows of the block
    // velocities of the block's 33 x 33 nodes as pairs, split once each
    __shared__ ff nU[TY + 1][SFX + 1], nV[TY + 1][SFX + 1];
    const int m = c.m, n = c.n;
    if (c.clock) cur = (int)c.clock[CLK_CUR] ^ 1;  // the state the advection wrote
    const int i0 = blockIdx.x * SFX, j0 = blockIdx.y * TY;
    const int tid = threadIdx.y * SFX + threadIdx.x;
#pragma unroll
    for (int k = tid; k < (TY + 1) * (SFX + 1); k += SFX * SFY) {
        const int r = k / (SFX + 1), cc = k - r * (SFX + 1);
        const int nj = j0 + r;
        int ni = i0 + cc;
        ni = ni >= m ? ni % m : ni;
        if (nj > n) continue;
        const double2 v = F.vel[(size_t)nj * m + ni];
        nU[r][cc] = split_ff(v.x);
        nV[r][cc] = split_ff(v.y);
    }
    __syncthreads();
    const int tx = threadIdx.x, i = i0 + tx;
    if (i >= m) return;
    const ff hx{h.hxh, h.hxl}, hy{h.hyh, h.hyl};
    double *const *S = F.f[cur];
#pragma unroll
    for (int q = 0; q < SFR; q++) {
        const int ty = threadIdx.y + q * SFY, j = j0 + ty;
        if (j >= n) break;
        // nodes a = (i, j), b = (i+1, j), c = (i, j+1), d = (i+1, j+1)
        const ff ax = nU[ty][tx], bx = nU[ty][tx + 1], cx = nU[ty + 1][tx], dx = nU[ty + 1][tx + 1];
        const ff ay = nV[ty][tx], by = nV[ty][tx + 1], cy = nV[ty + 1][tx], dy = nV[ty + 1][tx + 1];
        const ff ux = ff_mul(hx, ff_add(ff_sub(bx, ax), ff_sub(dx, cx)));
        const ff uy = ff_mul(hy, ff_add(ff_sub(cx, ax), ff_sub(dx, bx)));
        const ff vx = ff_mul(hx, ff_add(ff_sub(by, ay), ff_sub(dy, cy)));
        const ff vy = ff_mul(hy, ff_add(ff_sub(cy, ay), ff_sub(dy, by)));
        const ff div = ff_add(ux, vy);
        const size_t k = IDX(i, j);
        S[F_P][k] = add_ff(S[F_P][k], ff_neg(ff_mul(ff{h.Kh, h.Kl}, div)));
        S[F_Q][k] = add_ff(S[F_Q][k], ff_neg(ff_mul(ff{h.m3h, h.m3l}, div)));
        S[F_S][k] = add_ff(S[F_S][k], ff_mul(ff{h.muh, h.mul}, ff_sub(ux, vy)));
        S[F_TAU][k] = add_ff(S[F_TAU][k], ff_mul(ff{h.muh, h.mul}, ff_add(uy, vx)));
    }
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

cudaError_t prepare_step_kernels() {
    static unsigned long long done = 0;  // per device ordinal
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 64 && (done >> dev & 1)) return cudaSuccess;
    e = cudaFuncSetAttribute(k_advect, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(adv_smem) + 128));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_advect_ff, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(adv_smem_ff) + 128));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_direct, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(direct_tile));
    if (e == cudaSuccess && dev < 64) done |= 1ull << dev;
    return e;
}

int make_field_maps(const step_consts &c, const fields_dev &F, field_maps *out) {
    typedef CUresult (*encode_fn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static encode_fn encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return fail(STZG_ECUDA, "cuTensorMapEncodeTiled is not available");
        encode = (encode_fn)fn;
    }
    // 16-byte rules: row stride m*8 and the box's inner extent ACOLS*8
    if ((c.m * sizeof(double)) % 16 != 0) return fail(STZG_EINVAL, "tile copies need an even m");
    const cuuint64_t dims[2] = {(cuuint64_t)c.m, (cuuint64_t)c.n + 2};
    const cuuint64_t strides[1] = {(cuuint64_t)c.m * sizeof(double)};
    const cuuint32_t box[2] = {ACOLS, AROWS};
    const cuuint32_t estr[2] = {1, 1};
    for (int b = 0; b < 2; b++)
        for (int f = 0; f < F_COUNT; f++) {
            if (((uintptr_t)F.f[b][f]) % 16 != 0) return fail(STZG_EINVAL, "field not 16-byte aligned");
            const CUresult r = encode(&out->f[b][f], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void *)F.f[b][f], dims,
                                      strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return fail(STZG_ECUDA, "cuTensorMapEncodeTiled failed");
        }
    return STZG_OK;
}

void advection(const step_consts &c, const field_maps &maps, fields_dev &F, int cur, double dt, double bv,
               cudaStream_t st) {
    dim3 blk(32, 8);
    advect_consts a;
    a.hx = 0.5 * c.xsp * dt;
    a.hy = 0.5 * c.ysp * dt;
    a.xf = 0.5 / dt * c.xsp;
    a.yf = 0.5 / dt * c.ysp;
    const dim3 grid(ceil_div(c.m, ATX), ceil_div(c.n, ATY));
    if (c.sp_increments) {
        advect_ff_consts h;
        split_host(a.hx, &h.hxh, &h.hxl);
        split_host(a.hy, &h.hyh, &h.hyl);
        split_host(c.lx, &h.lxh, &h.lxl);
        cudaMemsetAsync(F.pcount, 0, sizeof(unsigned), st);
        k_advect_ff<<<grid, dim3(ATX, ATY), sizeof(adv_smem_ff) + 128, st>>>(c, h, maps, F, cur, dt, bv);
        note_launch();
        k_plastic_ff<<<2 * 152, 256, 0, st>>>(c, F, cur, dt);
    } else {
        k_advect<<<grid, dim3(ATX, ATY), sizeof(adv_smem) + 128, st>>>(c, a, maps, F, cur, dt, bv, 1);
    }
    note_launch();
    if (c.chi_diff != 0 || c.chi_len != 0) {
        k_chi_diffusion<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, F, cur, dt);
        note_launch();
    }
}

void direct_step(const step_consts &c, double viscosity, fields_dev &F, int cur, double dt, double bv,
                 cudaStream_t st) {
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt;
    direct_consts d;
    d.hx = hx;
    d.hy = hy;
    d.mu_inv = 1 / c.mu;
    d.hxxv = 2 * c.xsp * hx * viscosity;
    d.hyyv = 2 * c.ysp * hy * viscosity;
    d.hcv = 2 * (d.hxxv + d.hyyv);
    d.hxxcd = 2 * c.xsp * hx * c.chi_diff;
    d.hyycd = 2 * c.ysp * hy * c.chi_diff;
    d.hccd = 2 * (d.hxxcd + d.hyycd);
    dim3 blk(ATX, ATY);
    k_direct<<<g2(c.m, c.n, blk), blk, sizeof(direct_tile), st>>>(c, d, F, cur, dt, bv);
    note_launch();
    if (c.chi_diff != 0 || c.chi_len != 0) {
        k_chi_diffusion<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, F, cur, dt);
        note_launch();
    }
}

void projection_source(const step_consts &c, fields_dev &F, int cur, double dt, double xbc_bv, cudaStream_t st) {
    dim3 blk(32, 8);
    if (c.sp_increments) {
        source_ff_consts h;
        split_host(0.5 / dt * c.xsp, &h.xfh, &h.xfl);
        split_host(0.5 / dt * c.ysp, &h.yfh, &h.yfl);
        const dim3 sb(SFX, SFY);
        k_source_ff<<<g2(c.m, c.n + 1, dim3(SFX, SFY * SFR)), sb, 0, st>>>(c, F, cur, h, xbc_bv);
    } else {
        k_source<<<g2(c.m, c.n + 1, blk), blk, 0, st>>>(c, F, xbc_bv);
    }
    note_launch();
}

void precombine(const step_consts &c, fields_dev &F, int cur, double dt, cudaStream_t st) {
    if (c.sp_increments) return;  // k_source_ff reads the stresses themselves
    dim3 blk(32, 8);
    k_precombine<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, F, cur, 0.5 / dt * c.xsp, 0.5 / dt * c.ysp);
    note_launch();
}

void projection_apply(const step_consts &c, fields_dev &F, int cur, double dt, double bv, double bp,
                      cudaStream_t st) {
    dim3 blk(32, 8);
    const double hx = 0.5 * c.xsp * dt, hy = 0.5 * c.ysp * dt;
    if (c.sp_increments) {
        project_ff_consts h;
        split_host(hx, &h.hxh, &h.hxl);
        split_host(hy, &h.hyh, &h.hyl);
        split_host(c.K, &h.Kh, &h.Kl);
        split_host(c.mu * (1 / 3.0), &h.m3h, &h.m3l);
        split_host(c.mu, &h.muh, &h.mul);
        const dim3 sb(SFX, SFY);
        k_project_ff<<<g2(c.m, c.n, dim3(SFX, SFY * SFR)), sb, 0, st>>>(c, F, cur, h);
    } else {
        k_project<<<g2(c.m, c.n, blk), blk, 0, st>>>(c, F, cur, hx, hy);
    }
    note_launch();
    k_boundaries<<<ceil_div(c.m, 128), 128, 0, st>>>(c, F, cur, bp); note_launch();
    (void)bv;
}

void set_boundaries(const step_consts &c, fields_dev &F, int cur, double bp, cudaStream_t st) {
    k_boundaries<<<ceil_div(c.m, 128), 128, 0, st>>>(c, F, cur, bp); note_launch();
}

}  // namespace stzg
