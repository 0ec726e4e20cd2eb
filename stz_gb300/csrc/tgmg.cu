// General geometric multigrid on one GPU (include/stzg_tgmg.h): the
// tgmg<S,V,M> template of esim/tgmg (tgmg.hh:42-495, tgmg.in.cc:11-856) for
// problem classes with scalar values (V = M = double, e.g. poisson_fd,
// esim/tgmg/poisson_fd.hh:7-61) or 2-vectors with 2x2 blocks (V = vec,
// M = mat, e.g. the qs_multi classes of esim/sb and esim/coord_transforms).
//
// Layout: every level keeps z, b and a residual buffer r (FP64, row-major,
// index j*m+i, B components per point) and its operator as a table of
// distinct 9-point block stencils plus the inverse centre block, with a
// stencil index per point; the top level uses the problem's own table.
// Coarse operators are the Galerkin products P^T A P of tgmg_base::rat
// (tgmg.in.cc:667-736) with the reference's one-dimensional interpolation in
// each direction (apply_t / t_line, tgmg.in.cc:552-621; restriction is its
// transpose, apply_r :626-647), applied to every block component.
// Gauss-Seidel runs in four colours ((i&1),(j&1)), a true Gauss-Seidel
// ordering for 9-point stencils, with a third colour for the last line of an
// odd periodic direction; the reference sweeps zebra-lexicographically
// (tgmg.in.cc:128-208), so iterates differ and converged solutions agree.
// The coarsest level (more than 10 points, the next coarsening would have
// at most 10, tgmg_config.hh:23) is solved exactly with a dense inverse
// where it has at most 1024 unknowns and is not singular, else smoothed like
// the reference.  A mixed-precision solver (stzg_tgmg_set_precision) runs its
// V-cycle solves as FP32 V-cycles on FP32 copies of the levels, inside FP64
// refinement on the top level.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "stzg_tgmg.h"
#include "transfer1d.cuh"

namespace stzg {
namespace {

// Value of a point (B components) and a block (B x B, row-major: the
// reference's vec and mat, vec.hh / mat.hh).
template <int B, typename T = double> struct bv {
    T c[B];
};
template <int B, typename T = double> struct bm {
    T c[B * B];
};

template <int B, typename T> __host__ __device__ __forceinline__ bv<B, T> vzero() {
    bv<B, T> r;
#pragma unroll
    for (int k = 0; k < B; k++) r.c[k] = 0;
    return r;
}
__device__ __forceinline__ double tfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float tfma(float a, float b, float c) { return fmaf(a, b, c); }

// a += M x
template <int B, typename T> __device__ __forceinline__ void madd(bv<B, T> &a, const bm<B, T> &M, const bv<B, T> &x) {
#pragma unroll
    for (int r = 0; r < B; r++)
#pragma unroll
        for (int c = 0; c < B; c++) a.c[r] = tfma(M.c[r * B + c], x.c[c], a.c[r]);
}
template <int B, typename T> __device__ __forceinline__ bv<B, T> mul(const bm<B, T> &M, const bv<B, T> &x) {
    bv<B, T> r;
#pragma unroll
    for (int i = 0; i < B; i++) {
        T a = M.c[i * B] * x.c[0];
#pragma unroll
        for (int c = 1; c < B; c++) a = tfma(M.c[i * B + c], x.c[c], a);
        r.c[i] = a;
    }
    return r;
}
template <int B, typename T> __device__ __forceinline__ bv<B, T> vsub(const bv<B, T> &a, const bv<B, T> &b) {
    bv<B, T> r;
#pragma unroll
    for (int k = 0; k < B; k++) r.c[k] = a.c[k] - b.c[k];
    return r;
}

template <int B, typename T = double> struct gst {
    bm<B, T> e[10];  // dl dc dr cl cc cr ul uc ur, inverse of cc (tgmg_level::s, tgmg.hh:256-265)
    int nz;       // bit k set where off-diagonal block k is nonzero
    int pad;
};

template <int B, typename T = double> struct glevel {
    int m, n, xp, yp;
    int cx_n, cy_n;  // colours per direction: 2, or 3 on an odd periodic line
    const int *cls;
    const gst<B, T> *st;
    bv<B, T> *z, *b, *r;
};

constexpr int kMaxLevels = 17;
constexpr int kGridMin = 10;        // tgmg_grid_min, tgmg_config.hh:23
constexpr int kBottomDirect = 1024; // most unknowns of a coarsest level solved by a dense inverse
constexpr int kRedBlocks = 4 * 152;
constexpr int kRedThreads = 256;
constexpr size_t kTailSmem = 200 * 1024; // shared memory of the single-block tail
// Largest level the tail takes: one SM's FP64 pipe is slow (a 65 x 65
// level alone kept the tail at ~120 us a cycle), so the tail starts at 33 x 33;
// in FP32 one SM sweeps a 64 x 32 level of 2x2 blocks in well under the time
// of the 11 launches the level otherwise costs.
constexpr long kTailPoints = 1200;
constexpr long kTailPointsF = 2048;

// First level of the single-block tail for values of vbytes bytes per point:
// the small levels that fit in its shared memory together (z, b, r), if
// they are at least two (the coarsest alone is the bottom); 1 << 30 if none.
inline int tail_start_for(const int *m, const int *n, int nl, size_t vbytes, long max_points) {
    size_t bytes = 0;
    int t = nl;
    for (int l = nl - 1; l >= 1; l--) {
        const long pts = (long)m[l] * n[l];
        const size_t b = 3 * vbytes * (size_t)pts;
        if (pts > max_points || bytes + b > kTailSmem) break;
        bytes += b;
        t = l;
    }
    return t <= nl - 2 ? t : 1 << 30;
}

// Neighbour index on a line of m points, or -1 outside a non-periodic line.
__host__ __device__ inline int nbr(int i, int d, int m, int prd) {
    const int k = i + d;
    if (k < 0) return prd ? k + m : -1;
    if (k >= m) return prd ? k - m : -1;
    return k;
}

// Off-diagonal product sum_k A_k z_k at (i, j) (tgmg_level::mul_a,
// tgmg.in.cc:536-547); neighbours outside a non-periodic grid are skipped, and
// so are zero blocks (an integer test on the stencil's mask: the FP64 pipe,
// GB300's scarce one, only sees the nonzero products).
template <int B, typename T>
__device__ __forceinline__ bv<B, T> offdiag(const glevel<B, T> &L, const gst<B, T> &s, int i, int j) {
    const int il = nbr(i, -1, L.m, L.xp), ir = nbr(i, 1, L.m, L.xp);
    const int jd = nbr(j, -1, L.n, L.yp), ju = nbr(j, 1, L.n, L.yp);
    const int nz = s.nz;
    bv<B, T> a = vzero<B, T>();
    if (jd >= 0) {
        const bv<B, T> *zr = L.z + (size_t)jd * L.m;
        if ((nz & 1) && il >= 0) madd(a, s.e[0], zr[il]);
        if (nz & 2) madd(a, s.e[1], zr[i]);
        if ((nz & 4) && ir >= 0) madd(a, s.e[2], zr[ir]);
    }
    {
        const bv<B, T> *zr = L.z + (size_t)j * L.m;
        if ((nz & 8) && il >= 0) madd(a, s.e[3], zr[il]);
        if ((nz & 32) && ir >= 0) madd(a, s.e[5], zr[ir]);
    }
    if (ju >= 0) {
        const bv<B, T> *zr = L.z + (size_t)ju * L.m;
        if ((nz & 64) && il >= 0) madd(a, s.e[6], zr[il]);
        if (nz & 128) madd(a, s.e[7], zr[i]);
        if ((nz & 256) && ir >= 0) madd(a, s.e[8], zr[ir]);
    }
    return a;
}

// r = b - A z at (i, j)
template <int B, typename T>
__device__ __forceinline__ bv<B, T> residual_at(const glevel<B, T> &L, const gst<B, T> &s, size_t ij, int i, int j) {
    bv<B, T> a = offdiag(L, s, i, j);
    madd(a, s.e[4], L.z[ij]);
    return vsub(L.b[ij], a);
}

// k-th line of colour c on a line of m points with cn colours: colour 0 the
// even lines, 1 the odd ones, 2 the last line of an odd periodic direction
// (a neighbour of line 0); -1 when there is none.
__device__ __forceinline__ int color_line(int k, int c, int m, int cn) {
    if (c == 2) return k == 0 ? m - 1 : -1;
    const int i = c + 2 * k;
    if (i >= m || (cn == 3 && i == m - 1)) return -1;
    return i;
}

// One colour of Gauss-Seidel or SOR: z += omega (D^-1 (b - A'z) - z)
// (gauss_seidel, sor: tgmg.in.cc:128-230).
template <int B, typename T, bool Relax>
__global__ void k_tg_color(glevel<B, T> L, int cx, int cy, double omega) {
    const int i = color_line(blockIdx.x * blockDim.x + threadIdx.x, cx, L.m, L.cx_n);
    const int j = color_line(blockIdx.y * blockDim.y + threadIdx.y, cy, L.n, L.cy_n);
    if (i < 0 || j < 0) return;
    const size_t ij = (size_t)j * L.m + i;
    const gst<B, T> &s = L.st[L.cls[ij]];
    const bv<B, T> t = mul(s.e[9], vsub(L.b[ij], offdiag(L, s, i, j)));
    if (Relax) {
        bv<B, T> z = L.z[ij];
#pragma unroll
        for (int k = 0; k < B; k++) z.c[k] += T(omega) * (t.c[k] - z.c[k]);
        L.z[ij] = z;
    } else {
        L.z[ij] = t;
    }
}

// Jacobi update into r (jacobi, tgmg.in.cc:69-85); the caller copies r to z.
template <int B> __global__ void k_tg_jacobi(glevel<B> L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= L.m || j >= L.n) return;
    const size_t ij = (size_t)j * L.m + i;
    const gst<B> &s = L.st[L.cls[ij]];
    L.r[ij] = mul(s.e[9], vsub(L.b[ij], offdiag(L, s, i, j)));
}

// r = b - A z (tgmg_base::res, tgmg.hh:197-199).
template <int B, typename T> __global__ void k_tg_residual(glevel<B, T> L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= L.m || j >= L.n) return;
    const size_t ij = (size_t)j * L.m + i;
    L.r[ij] = residual_at(L, L.st[L.cls[ij]], ij, i, j);
}

// Fine line index 2I+d, wrapped on a periodic line; -1 outside.
__device__ __forceinline__ int fine_at(int I, int d, int m, int prd) {
    int f = 2 * I + d;
    if (f < 0 || f >= m) {
        if (!prd) return -1;
        f = f < 0 ? f + m : f - m;
    }
    return f;
}

// Child b = P^T r at (I, J) (apply_r, tgmg.in.cc:626-647): weights 1, 1/2,
// 1/4 from the interpolation's halves in each direction, summed as
// (sum over rows of hy * (sum over columns of hx * r)) / 4 with the factors 2
// applied as additions.
template <int B, typename T>
__device__ __forceinline__ bv<B, T> restrict_at(const glevel<B, T> &F, const bv<B, T> *r, int I, int J) {
    bv<B, T> acc = vzero<B, T>();
#pragma unroll
    for (int dy = -1; dy <= 1; dy++) {
        const int fy = fine_at(J, dy, F.n, F.yp);
        if (fy < 0) continue;
        const int hy = halves_of(fy, F.n, F.yp, J);
        if (!hy) continue;
        const bv<B, T> *rr = r + (size_t)fy * F.m;
        bv<B, T> row = vzero<B, T>();
#pragma unroll
        for (int dx = -1; dx <= 1; dx++) {
            const int fx = fine_at(I, dx, F.m, F.xp);
            if (fx < 0) continue;
            const int hx = halves_of(fx, F.m, F.xp, I);
            if (!hx) continue;
#pragma unroll
            for (int k = 0; k < B; k++) row.c[k] += hx == 2 ? rr[fx].c[k] + rr[fx].c[k] : rr[fx].c[k];
        }
#pragma unroll
        for (int k = 0; k < B; k++) acc.c[k] += hy == 2 ? row.c[k] + row.c[k] : row.c[k];
    }
#pragma unroll
    for (int k = 0; k < B; k++) acc.c[k] *= T(0.25);
    return acc;
}

template <int B, typename T> __global__ void k_tg_restrict(glevel<B, T> F, glevel<B, T> C) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y * blockDim.y + threadIdx.y;
    if (I >= C.m || J >= C.n) return;
    C.b[(size_t)J * C.m + I] = restrict_at(F, F.r, I, J);
}

// Interpolated child value at a parent point from the coarse indices of
// p1d_halves: injection, the mean of two, or the mean of four (exact weights
// 1, 1/2, 1/4 applied as one multiplication).
template <int B, typename T>
__device__ __forceinline__ bv<B, T> interp_at(const glevel<B, T> &C, int ny, const int *cy, int nx, const int *cx) {
    const bv<B, T> *r0 = C.z + (size_t)cy[0] * C.m, *r1 = C.z + (size_t)cy[ny - 1] * C.m;
    bv<B, T> o;
#pragma unroll
    for (int k = 0; k < B; k++) {
        if (ny == 1) o.c[k] = nx == 1 ? r0[cx[0]].c[k] : T(0.5) * (r0[cx[0]].c[k] + r0[cx[1]].c[k]);
        else if (nx == 1) o.c[k] = T(0.5) * (r0[cx[0]].c[k] + r1[cx[0]].c[k]);
        else o.c[k] = T(0.25) * ((r0[cx[0]].c[k] + r0[cx[1]].c[k]) + (r1[cx[0]].c[k] + r1[cx[1]].c[k]));
    }
    return o;
}

// Parent z += P z_child (apply_t, tgmg.in.cc:552-606).
template <int B, typename T> __global__ void k_tg_prolong(glevel<B, T> C, glevel<B, T> F) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= F.m || j >= F.n) return;
    int cy[2], hy[2], cx[2], hx[2];
    const int ny = p1d_halves(j, F.n, F.yp, cy, hy), nx = p1d_halves(i, F.m, F.xp, cx, hx);
    const bv<B, T> a = interp_at(C, ny, cy, nx, cx);
    bv<B, T> &z = F.z[(size_t)j * F.m + i];
#pragma unroll
    for (int k = 0; k < B; k++) z.c[k] += a.c[k];
}

// Coarsest level: z = A^-1 b with the dense inverse over its N unknowns (FP64;
// its FP32 rounding in the correction cycles of a mixed-precision solver).
template <int B, typename T> __global__ void k_tg_bottom(glevel<B, T> L, const T *__restrict__ inv, int N) {
    __shared__ T bb[kBottomDirect];
    const T *b = (const T *)L.b;
    T *z = (T *)L.z;
    for (int k = threadIdx.x; k < N; k += blockDim.x) bb[k] = b[k];
    __syncthreads();
    for (int r = threadIdx.x; r < N; r += blockDim.x) {
        const T *row = inv + (size_t)r * N;
        T a = 0;
        for (int k = 0; k < N; k++) a += row[k] * bb[k];
        z[r] = a;
    }
}

// Deterministic sum of squared residuals (mds, tgmg.in.cc:55-65): per-block
// partial sums in a fixed order, then one block adds the partials in order.
__device__ __forceinline__ double block_reduce(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;
}

template <int B> __global__ void k_tg_sqnorm(glevel<B> L, double *partials) {
    __shared__ double sh[32];
    const int mn = L.m * L.n;  // at most 2^30 points (checked at creation): 32-bit indices
    double acc = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < mn; k += gridDim.x * blockDim.x) {
        const int j = k / L.m, i = k - j * L.m;
        const bv<B> r = residual_at(L, L.st[L.cls[k]], (size_t)k, i, j);
#pragma unroll
        for (int c = 0; c < B; c++) acc += r.c[c] * r.c[c];
    }
    const double t = block_reduce(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

__global__ void k_tg_sum(const double *partials, int np, double *out) {
    __shared__ double sh[32];
    double a = 0;
    for (int k = threadIdx.x; k < np; k += blockDim.x) a += partials[k];
    const double t = block_reduce(a, sh);
    if (threadIdx.x == 0) *out = t;
}

// Mixed precision, once per refinement pass on the top level: r = b - A z in
// FP64, its FP32 rounding as the correction cycle's b, the correction's z
// cleared, and per-block partial sums of |r|^2 in the order of k_tg_sqnorm
// (the l2_error of a z is the same number either way).
template <int B> __global__ void k_tg_resid_split(glevel<B> L, glevel<B, float> F, double *partials) {
    __shared__ double sh[32];
    const int mn = L.m * L.n;  // at most 2^30 points (checked at creation): 32-bit indices
    double acc = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < mn; k += gridDim.x * blockDim.x) {
        const int j = k / L.m, i = k - j * L.m;
        const bv<B> r = residual_at(L, L.st[L.cls[k]], (size_t)k, i, j);
        bv<B, float> rf, zf;
#pragma unroll
        for (int c = 0; c < B; c++) {
            acc += r.c[c] * r.c[c];
            rf.c[c] = (float)r.c[c];
            zf.c[c] = 0.f;
        }
        F.b[k] = rf;
        F.z[k] = zf;
    }
    const double t = block_reduce(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// z += e: a correction cycle's FP32 result added to the FP64 solution.
template <int B> __global__ void k_tg_correct(glevel<B> L, const bv<B, float> *__restrict__ e) {
    const int mn = L.m * L.n;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < mn; k += gridDim.x * blockDim.x) {
        const bv<B, float> d = e[k];
        bv<B> z = L.z[k];
#pragma unroll
        for (int c = 0; c < B; c++) z.c[c] += (double)d.c[c];
        L.z[k] = z;
    }
}

// ---------------------------------------------------------------------------
// Tail of the cycle on the small levels, one block of 32 x 32 threads: the
// recursive V-cycle below level t (down sweeps from zero, residual and
// restriction level by level, the coarsest solve, prolongation and up sweeps)
// with z, b and r of levels t..L in shared memory; b of level t comes from
// and z of level t goes to global memory.  Phases are separated by
// __syncthreads.

template <int B, typename T> struct tail_args {
    int t, L, cd, cu, hb, sym;
    const T *inv;
    int inv_n;
    glevel<B, T> lv[kMaxLevels];
};

template <int B, typename T> __device__ void tail_sweep(const glevel<B, T> &L, bool reverse) {
    const int nc = L.cx_n * L.cy_n;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    const int kx = (L.m + 1) / 2, ky = (L.n + 1) / 2;
    for (int q = 0; q < nc; q++) {
        const int c = reverse ? nc - 1 - q : q;
        const int cy = c / L.cx_n, cx = c % L.cx_n;
        for (int k = tid; k < kx * ky; k += nth) {
            const int i = color_line(k % kx, cx, L.m, L.cx_n), j = color_line(k / kx, cy, L.n, L.cy_n);
            if (i < 0 || j < 0) continue;
            const size_t ij = (size_t)j * L.m + i;
            const gst<B, T> &s = L.st[L.cls[ij]];
            L.z[ij] = mul(s.e[9], vsub(L.b[ij], offdiag(L, s, i, j)));
        }
        __syncthreads();
    }
}

template <int B, typename T> __device__ void tail_clear(const glevel<B, T> &L) {
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    for (int k = tid; k < L.m * L.n; k += nth) L.z[k] = vzero<B, T>();
    __syncthreads();
}

template <int B, typename T> __global__ void __launch_bounds__(1024) k_tg_tail(tail_args<B, T> a) {
    extern __shared__ __align__(16) double tsm[];
    __shared__ glevel<B, T> S[kMaxLevels];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    if (tid == 0) {
        size_t off = 0;
        bv<B, T> *base = (bv<B, T> *)tsm;
        for (int l = a.t; l <= a.L; l++) {
            S[l] = a.lv[l];
            const size_t mn = (size_t)S[l].m * S[l].n;
            S[l].z = base + off;
            S[l].b = base + off + mn;
            S[l].r = base + off + 2 * mn;
            off += 3 * mn;
        }
    }
    __syncthreads();
    {
        const glevel<B, T> &Lt = S[a.t];
        for (int k = tid; k < Lt.m * Lt.n; k += nth) Lt.b[k] = a.lv[a.t].b[k];
        __syncthreads();
    }
    // down: levels t..L-1 (down_gs_iterations, then residual and restriction)
    for (int i = a.t; i < a.L; i++) {
        const glevel<B, T> &L = S[i], &C = S[i + 1];
        tail_clear(L);
        for (int c = 0; c < a.cd; c++) tail_sweep(L, false);
        for (int k = tid; k < L.m * L.n; k += nth) {
            const int j = k / L.m, ii = k - j * L.m;
            L.r[k] = residual_at(L, L.st[L.cls[k]], (size_t)k, ii, j);
        }
        __syncthreads();
        for (int k = tid; k < C.m * C.n; k += nth) {
            const int J = k / C.m, I = k - J * C.m;
            C.b[k] = restrict_at(L, L.r, I, J);
        }
        __syncthreads();
    }
    // coarsest level
    {
        const glevel<B, T> &Bt = S[a.L];
        if (a.inv) {
            const T *b = (const T *)Bt.b;
            T *z = (T *)Bt.z;
            for (int r = tid; r < a.inv_n; r += nth) {
                const T *row = a.inv + (size_t)r * a.inv_n;
                T acc = 0;
                for (int k = 0; k < a.inv_n; k++) acc += row[k] * b[k];
                z[r] = acc;
            }
            __syncthreads();
        } else {
            tail_clear(Bt);
            for (int c = 0; c < 2 * a.hb; c++) tail_sweep(Bt, a.sym && c >= a.hb);
        }
    }
    // up: prolongation and up_gs_iterations on levels L-1..t
    for (int i = a.L; i > a.t; i--) {
        const glevel<B, T> &C = S[i], &F = S[i - 1];
        for (int k = tid; k < F.m * F.n; k += nth) {
            const int j = k / F.m, ii = k - j * F.m;
            int cy[2], hy[2], cx[2], hx[2];
            const int ny = p1d_halves(j, F.n, F.yp, cy, hy), nx = p1d_halves(ii, F.m, F.xp, cx, hx);
            const bv<B, T> v = interp_at(C, ny, cy, nx, cx);
#pragma unroll
            for (int q = 0; q < B; q++) F.z[k].c[q] += v.c[q];
        }
        __syncthreads();
        for (int c = 0; c < a.cu; c++) tail_sweep(F, a.sym != 0);
    }
    {
        const glevel<B, T> &Lt = S[a.t];
        for (int k = tid; k < Lt.m * Lt.n; k += nth) a.lv[a.t].z[k] = Lt.z[k];
    }
}

// ---------------------------------------------------------------------------
// Host side: hierarchy sizes, Galerkin products, dense coarsest inverse.

template <int B> struct host_level {
    int m, n;
    bool rows;  // the stencil depends on the row only
    std::vector<int> cls;
    std::vector<int> row_ids;  // rows: the stencil index of each row
    bool cls_kept = false;     // cls equals the device copy already uploaded
    std::vector<gst<B>> table;
};

// Child sizes (tgmg_base constructor, tgmg.hh:108-110) while the child has
// more than tgmg_grid_min points (tgmg.in.cc:17-31).  A periodic line
// shorter than 3 would alias its own neighbours; coarsening stops there
// (the reference collapses such lines, tgmg.in.cc:738-781).
std::vector<std::pair<int, int>> level_sizes(int m, int n, int xp, int yp) {
    std::vector<std::pair<int, int>> out;
    out.push_back(std::make_pair(m, n));
    int am = (m + (xp ? 1 : 2)) >> 1, an = (n + (yp ? 1 : 2)) >> 1;
    while ((long)am * an > kGridMin && (int)out.size() < kMaxLevels && (!xp || am >= 3) && (!yp || an >= 3)) {
        out.push_back(std::make_pair(am, an));
        const int nm = (am + (xp ? 1 : 2)) >> 1, nn = (an + (yp ? 1 : 2)) >> 1;
        am = nm;
        an = nn;
    }
    return out;
}

inline int wrap_line(int f, int m, int prd) {
    if (f >= 0 && f < m) return f;
    if (!prd) return -1;
    return f < 0 ? f + m : f - m;
}

// Coarse offset -1..1 of coarse index c relative to C on a line of cm points.
inline int coarse_offset(int c, int C, int cm, int prd) {
    int o = c - C;
    if (prd) {
        if (o > 1) o -= cm;
        if (o < -1) o += cm;
    }
    return o;
}

template <int B> bool block_zero(const bm<B> &a) {
    for (int q = 0; q < B * B; q++)
        if (a.c[q] != 0) return false;
    return true;
}

template <int B> int nonzero_mask(const gst<B> &s) {
    int nz = 0;
    for (int k = 0; k < 9; k++)
        if (k != 4 && !block_zero(s.e[k])) nz |= 1 << k;
    return nz;
}

// Inverse of a block (the reference's operator/(double,mat), mat.hh).
template <int B> bm<B> block_inverse(const bm<B> &a);
template <> bm<1> block_inverse<1>(const bm<1> &a) {
    bm<1> r;
    r.c[0] = 1. / a.c[0];
    return r;
}
template <> bm<2> block_inverse<2>(const bm<2> &f) {
    const double idet = 1. / (f.c[0] * f.c[3] - f.c[1] * f.c[2]);
    bm<2> r;
    r.c[0] = f.c[3] * idet;
    r.c[1] = -f.c[1] * idet;
    r.c[2] = -f.c[2] * idet;
    r.c[3] = f.c[0] * idet;
    return r;
}

// Galerkin stencil at coarse point (I, J): sum over fine points k near
// (2I, 2J) and their neighbours l of P(k, (I,J)) A(k, l) P(l, neighbour).
template <int B>
gst<B> rap_point(const host_level<B> &F, int xp, int yp, int cm, int cn, int I, int J) {
    bm<B> acc[9];
    for (int k = 0; k < 9; k++)
        for (int q = 0; q < B * B; q++) acc[k].c[q] = 0;
    for (int dy = -1; dy <= 1; dy++) {
        const int fy = wrap_line(2 * J + dy, F.n, yp);
        if (fy < 0) continue;
        const double wy = pw(fy, F.n, yp, J);
        if (wy == 0) continue;
        for (int dx = -1; dx <= 1; dx++) {
            const int fx = wrap_line(2 * I + dx, F.m, xp);
            if (fx < 0) continue;
            const double wx = pw(fx, F.m, xp, I);
            if (wx == 0) continue;
            const gst<B> &s = F.table[F.cls[(size_t)fy * F.m + fx]];
            for (int sy = -1; sy <= 1; sy++) {
                const int ly = wrap_line(fy + sy, F.n, yp);
                if (ly < 0) continue;
                for (int sx = -1; sx <= 1; sx++) {
                    const int lx = wrap_line(fx + sx, F.m, xp);
                    if (lx < 0) continue;
                    const bm<B> &a = s.e[(sy + 1) * 3 + sx + 1];
                    if (block_zero(a)) continue;
                    int cy[2], cx[2];
                    double wyl[2], wxl[2];
                    const int ny = p1d(ly, F.n, yp, cy, wyl), nx = p1d(lx, F.m, xp, cx, wxl);
                    for (int q = 0; q < ny; q++)
                        for (int p = 0; p < nx; p++) {
                            const int oy = coarse_offset(cy[q], J, cn, yp), ox = coarse_offset(cx[p], I, cm, xp);
                            bm<B> &t = acc[(oy + 1) * 3 + ox + 1];
                            for (int e = 0; e < B * B; e++) t.c[e] += wx * wy * a.c[e] * wxl[p] * wyl[q];
                        }
                }
            }
        }
    }
    gst<B> out;
    std::memset(&out, 0, sizeof(out));
    for (int k = 0; k < 9; k++) out.e[k] = acc[k];
    out.e[9] = block_inverse<B>(acc[4]);
    out.nz = nonzero_mask(out);
    return out;
}

template <int B> struct gst_hash {
    size_t operator()(const gst<B> &s) const {
        uint64_t h = 1469598103934665603ull;
        const unsigned char *p = (const unsigned char *)&s;
        for (size_t k = 0; k < sizeof(gst<B>); k++) h = (h ^ p[k]) * 1099511628211ull;
        return (size_t)h;
    }
};
template <int B> struct gst_eq {
    bool operator()(const gst<B> &a, const gst<B> &b) const { return std::memcmp(&a, &b, sizeof(gst<B>)) == 0; }
};

// Child level.  A fine level whose stencil depends on the row only, on an
// even periodic x line, coarsens uniformly: its child depends on the row
// only too and one Galerkin product per row suffices.  With the previous
// child `old` of the same shape whose rows map to the same stencil indices,
// its class map is taken over (only the stencil values are new).
template <int B>
host_level<B> coarsen(const host_level<B> &F, int xp, int yp, int cm, int cn, host_level<B> *old = nullptr) {
    host_level<B> C;
    C.m = cm;
    C.n = cn;
    C.rows = F.rows && xp && (F.m % 2 == 0);
    std::vector<gst<B>> all;
    if (C.rows) {
        all.resize(cn);
#pragma omp parallel for schedule(static)
        for (int J = 0; J < cn; J++) all[J] = rap_point(F, xp, yp, cm, cn, 0, J);
    } else {
        all.resize((size_t)cm * cn);
#pragma omp parallel for schedule(static)
        for (int J = 0; J < cn; J++)
            for (int I = 0; I < cm; I++) all[(size_t)J * cm + I] = rap_point(F, xp, yp, cm, cn, I, J);
    }
    std::unordered_map<gst<B>, int, gst_hash<B>, gst_eq<B>> index;
    std::vector<int> ids(all.size());
    for (size_t k = 0; k < all.size(); k++) {
        auto it = index.find(all[k]);
        if (it == index.end()) {
            it = index.emplace(all[k], (int)C.table.size()).first;
            C.table.push_back(all[k]);
        }
        ids[k] = it->second;
    }
    if (C.rows) {
        if (old && old->rows && old->m == cm && old->n == cn && old->row_ids == ids) {
            C.cls.swap(old->cls);
            C.cls_kept = true;
        } else {
            C.cls.resize((size_t)cm * cn);
            for (int J = 0; J < cn; J++)
                for (int I = 0; I < cm; I++) C.cls[(size_t)J * cm + I] = ids[J];
        }
        C.row_ids.swap(ids);
    } else {
        C.cls.swap(ids);
        if (old && old->m == cm && old->n == cn && old->cls == C.cls) C.cls_kept = true;
    }
    return C;
}

// Dense inverse by Gauss-Jordan elimination with partial pivoting; empty if
// singular.  Unknown B*(j*m+i)+c.
template <int B> std::vector<double> dense_inverse(const host_level<B> &L, int xp, int yp) {
    const int N = B * L.m * L.n;
    std::vector<double> A((size_t)N * N, 0.0), X((size_t)N * N, 0.0);
    for (int j = 0; j < L.n; j++)
        for (int i = 0; i < L.m; i++) {
            const int p = j * L.m + i;
            const gst<B> &s = L.table[L.cls[p]];
            for (int sy = -1; sy <= 1; sy++) {
                const int ly = wrap_line(j + sy, L.n, yp);
                if (ly < 0) continue;
                for (int sx = -1; sx <= 1; sx++) {
                    const int lx = wrap_line(i + sx, L.m, xp);
                    if (lx < 0) continue;
                    const bm<B> &a = s.e[(sy + 1) * 3 + sx + 1];
                    const int q = ly * L.m + lx;
                    for (int r = 0; r < B; r++)
                        for (int c = 0; c < B; c++) A[(size_t)(B * p + r) * N + B * q + c] += a.c[r * B + c];
                }
            }
        }
    for (int r = 0; r < N; r++) X[(size_t)r * N + r] = 1;
    // a pivot at rounding level means a singular level (a periodic operator
    // that annihilates constants): no inverse, the bottom is smoothed.  After
    // six to eight Galerkin products the rounding pivots of such a level
    // reach 4e-10 of its largest entry (the next pivot is ~0.3 of it), so the
    // test sits well above them; an inverse built on them would carry
    // entries ~1e10 times the operator's inverse scale.
    double amax = 0;
    for (double v : A) amax = std::max(amax, std::fabs(v));
    const double tiny = 1e-8 * amax;
    for (int c = 0; c < N; c++) {
        int p = c;
        for (int r = c + 1; r < N; r++)
            if (std::fabs(A[(size_t)r * N + c]) > std::fabs(A[(size_t)p * N + c])) p = r;
        if (!(std::fabs(A[(size_t)p * N + c]) > tiny)) return std::vector<double>();
        if (p != c)
            for (int k = 0; k < N; k++) {
                std::swap(A[(size_t)p * N + k], A[(size_t)c * N + k]);
                std::swap(X[(size_t)p * N + k], X[(size_t)c * N + k]);
            }
        const double d = 1. / A[(size_t)c * N + c];
        for (int k = 0; k < N; k++) {
            A[(size_t)c * N + k] *= d;
            X[(size_t)c * N + k] *= d;
        }
        for (int r = 0; r < N; r++) {
            if (r == c) continue;
            const double f = A[(size_t)r * N + c];
            if (f == 0) continue;
            for (int k = 0; k < N; k++) {
                A[(size_t)r * N + k] -= f * A[(size_t)c * N + k];
                X[(size_t)r * N + k] -= f * X[(size_t)c * N + k];
            }
        }
    }
    return X;
}

inline dim3 grid_of(int m, int n, dim3 b) { return dim3(ceil_div(m, b.x), ceil_div(n, b.y)); }

// ---------------------------------------------------------------------------
// The solver state of one handle, for B components per point.

// The levels one cycle runs on, with the coarsest level's dense inverse (null
// where the bottom is smoothed): the solver's FP64 levels, or the FP32 levels
// of a mixed-precision solver's correction cycles.
template <int B, typename T> struct hview {
    const glevel<B, T> *lv;
    const T *inv;
    int inv_n;
    int tail_start;  // first level handled by k_tg_tail (none if > nl-1)
};

template <int B> struct tg {
    int device = 0;
    int xp = 0, yp = 0;
    double acc = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int nl = 0;
    glevel<B> lv[kMaxLevels];
    std::vector<host_level<B>> host;
    std::vector<void *> owned;
    size_t st_cap[kMaxLevels] = {0};
    double *inv = nullptr, *inv_buf = nullptr;
    int inv_n = 0;
    size_t inv_cap = 0;
    int tail_start = 1 << 30;  // first level handled by k_tg_tail (none if > nl-1)
    double *partials = nullptr, *dsum = nullptr, *hsum = nullptr;
    std::vector<double> inv_host;  // the coarsest inverse, for its FP32 copy
    std::vector<std::vector<gst<B, float>>> host32;  // FP32 tables as uploaded
    std::vector<float> inv_host32;
    // Mixed precision (V-cycle solves as refinement passes: FP32 V-cycles on
    // the FP64 residual, corrections added in FP64): FP32 levels sharing the
    // class maps of lv, their tables and the FP32 coarsest inverse.
    bool mixed = false, have32 = false;
    glevel<B, float> lf[kMaxLevels];
    size_t stf_cap[kMaxLevels] = {0};
    float *inv_f = nullptr;
    size_t inv_f_cap = 0;
    int tail_start_f = 1 << 30;  // the FP32 levels' tail start
    hview<B, double> v64() const { return hview<B, double>{lv, inv, inv_n, tail_start}; }
    hview<B, float> v32() const { return hview<B, float>{lf, inv ? inv_f : nullptr, inv_n, tail_start_f}; }
    // graph of one iteration of the last (type, omega, cycles) used
    cudaGraphExec_t gexec = nullptr;
    int gkey[5] = {-1, 0, 0, 0, 0};
    double gomega = 0;
    long gnodes = 0;
    double last_ms = 0;
    long last_kernels = 0;
    long kernels = 0;
};

template <int B> int g_alloc(tg<B> *g, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    g->owned.push_back(*p);
    STZG_CUDA(cudaMemsetAsync(*p, 0, bytes, g->st));
    return STZG_OK;
}

template <int B> void launch_note(tg<B> *g) {
    g->kernels++;
    note_launch();
}

const dim3 kBlk(32, 8);

template <int B, typename T> void sweep(tg<B> *g, const glevel<B, T> &L, bool reverse, double omega) {
    const int nc = L.cx_n * L.cy_n;
    for (int q = 0; q < nc; q++) {
        const int c = reverse ? nc - 1 - q : q;
        const int cy = c / L.cx_n, cx = c % L.cx_n;
        const dim3 gr = grid_of((L.m + 1) / 2, (L.n + 1) / 2, kBlk);
        if (omega == 1.0) k_tg_color<B, T, false><<<gr, kBlk, 0, g->st>>>(L, cx, cy, omega);
        else k_tg_color<B, T, true><<<gr, kBlk, 0, g->st>>>(L, cx, cy, omega);
        launch_note(g);
    }
}

template <int B, typename T> void clear_z(tg<B> *g, const glevel<B, T> &L) {
    cudaMemsetAsync(L.z, 0, sizeof(bv<B, T>) * (size_t)L.m * L.n, g->st);
}

// down_gs_iterations (tgmg.hh:273-279): clear z, then cyc sweeps (the first
// from zero).
template <int B, typename T> void down_gs(tg<B> *g, const glevel<B, T> &L, int cyc) {
    clear_z(g, L);
    for (int c = 0; c < cyc; c++) sweep(g, L, false, 1.0);
}

// up_gs_iterations (tgmg.hh:183-187): cyc sweeps, reversed when symmetric.
template <int B, typename T> void up_gs(tg<B> *g, const glevel<B, T> &L, int cyc, bool sym) {
    for (int c = 0; c < cyc; c++) sweep(g, L, sym, 1.0);
}

template <int B, typename T> void restrict_to(tg<B> *g, const glevel<B, T> &F, const glevel<B, T> &C) {
    k_tg_residual<B, T><<<grid_of(F.m, F.n, kBlk), kBlk, 0, g->st>>>(F);
    launch_note(g);
    k_tg_restrict<B, T><<<grid_of(C.m, C.n, kBlk), kBlk, 0, g->st>>>(F, C);
    launch_note(g);
}

template <int B, typename T> void prolong(tg<B> *g, const glevel<B, T> &C, const glevel<B, T> &F) {
    k_tg_prolong<B, T><<<grid_of(F.m, F.n, kBlk), kBlk, 0, g->st>>>(C, F);
    launch_note(g);
}

// Coarsest level: the reference's hcyc_bottom sweeps down and up
// (tgmg.in.cc:350-352), replaced by the exact solve where it is available.
template <int B, typename T> void bottom(tg<B> *g, const hview<B, T> &h, int hcyc, bool sym) {
    const glevel<B, T> &Bt = h.lv[g->nl - 1];
    if (h.inv) {
        k_tg_bottom<B, T><<<1, 256, 0, g->st>>>(Bt, h.inv, h.inv_n);
        launch_note(g);
    } else {
        down_gs(g, Bt, hcyc);
        up_gs(g, Bt, hcyc, sym);
    }
}

template <int B, typename T> size_t tail_bytes(const tg<B> *g, const hview<B, T> &h, int i) {
    size_t smem = 0;
    for (int l = i; l < g->nl; l++) smem += 3 * sizeof(bv<B, T>) * (size_t)h.lv[l].m * h.lv[l].n;
    return smem;
}

template <int B, typename T> void tail(tg<B> *g, const hview<B, T> &h, int i, int cd, int cu, int hb, bool sym) {
    tail_args<B, T> a;
    a.t = i;
    a.L = g->nl - 1;
    a.cd = cd;
    a.cu = cu;
    a.hb = hb;
    a.sym = sym ? 1 : 0;
    a.inv = h.inv;
    a.inv_n = h.inv_n;
    for (int l = 0; l < g->nl; l++) a.lv[l] = h.lv[l];
    k_tg_tail<B, T><<<1, dim3(32, 32), tail_bytes(g, h, i), g->st>>>(a);
    launch_note(g);
}

// The V-cycle from level i (>= 1) on its b: down_gs, restriction, the cycle
// below, prolongation, up_gs; the coarsest level is the bottom solve.  This
// is v_cycle_internal (tgmg.in.cc:341-359) written recursively; levels from
// tail_start down run in one k_tg_tail launch.
template <int B, typename T> void vc(tg<B> *g, const hview<B, T> &h, int i, int cd, int cu, int hb, bool sym) {
    const int L = g->nl - 1;
    if (i == L) {
        bottom(g, h, hb, sym);
        return;
    }
    if (i >= h.tail_start) {
        tail(g, h, i, cd, cu, hb, sym);
        return;
    }
    down_gs(g, h.lv[i], cd);
    restrict_to(g, h.lv[i], h.lv[i + 1]);
    vc(g, h, i + 1, cd, cu, hb, sym);
    prolong(g, h.lv[i + 1], h.lv[i]);
    up_gs(g, h.lv[i], cu, sym);
}

// v_cycle_internal from a level whose z has had its down sweeps: restrict,
// cycle below, prolong, up sweeps.
template <int B, typename T>
void internal(tg<B> *g, const hview<B, T> &h, int level, int cd, int cu, int hb, bool sym) {
    restrict_to(g, h.lv[level], h.lv[level + 1]);
    vc(g, h, level + 1, cd, cu, hb, sym);
    prolong(g, h.lv[level + 1], h.lv[level]);
    up_gs(g, h.lv[level], cu, sym);
}

// tgmg::v_cycle (tgmg.in.cc:313-328).
template <int B, typename T> void v_cycle(tg<B> *g, const hview<B, T> &h, int cd, int cu, int hb, bool sym) {
    for (int c = 0; c < cd; c++) sweep(g, h.lv[0], false, 1.0);
    if (g->nl > 1) {
        restrict_to(g, h.lv[0], h.lv[1]);
        vc(g, h, 1, cd, cu, hb, sym);
        prolong(g, h.lv[1], h.lv[0]);
    }
    up_gs(g, h.lv[0], cu, sym);
}

// tgmg::fmg_pre (tgmg.in.cc:369-402).
template <int B> void fmg_pre(tg<B> *g, int cd, int cu, int hb, bool sym) {
    const hview<B, double> h = g->v64();
    const int L = g->nl - 1;
    for (int c = 0; c < cd; c++) sweep(g, h.lv[0], false, 1.0);
    if (L > 0) {
        restrict_to(g, h.lv[0], h.lv[1]);
        for (int i = 1; i < L; i++) {
            down_gs(g, h.lv[i], cd);
            restrict_to(g, h.lv[i], h.lv[i + 1]);
        }
        bottom(g, h, hb, sym);
        for (int i = L; i > 1; i--) {
            prolong(g, h.lv[i], h.lv[i - 1]);
            up_gs(g, h.lv[i - 1], cu, sym);
            for (int c = 0; c < cd; c++) sweep(g, h.lv[i - 1], false, 1.0);
            internal(g, h, i - 1, cd, cu, hb, sym);
        }
        prolong(g, h.lv[1], h.lv[0]);
    }
    up_gs(g, h.lv[0], cu, sym);
}

template <int B> bool uses_mixed(const tg<B> *g, int type) {
    return g->mixed && (type == STZG_TGMG_VCYCLE || type == STZG_TGMG_SYM_VCYCLE);
}

// Mixed precision: the top level's FP64 residual of the current z into the
// FP32 correction cycle's b, with its squared-norm partials.
template <int B> void resid_split(tg<B> *g) {
    k_tg_resid_split<B><<<kRedBlocks, kRedThreads, 0, g->st>>>(g->lv[0], g->lf[0], g->partials);
    launch_note(g);
}

// One refinement pass of a mixed-precision V-cycle solve, after resid_split:
// an FP32 V-cycle on the residual from a zero correction, the correction
// added to the FP64 solution, and the new residual with its norm partials.
// With a V-cycle's contraction per pass (the FP32 rounding of the correction
// costs ~1e-7 of it), passes converge like FP64 V-cycles.
template <int B> void mixed_pass(tg<B> *g, int cd, int cu, int hb, bool sym) {
    v_cycle(g, g->v32(), cd, cu, hb, sym);
    k_tg_correct<B><<<kRedBlocks, kRedThreads, 0, g->st>>>(g->lv[0], g->lf[0].z);
    launch_note(g);
    resid_split(g);
}

// One iteration of a solver type (tgmg::iters, tgmg.hh:457-466); a V-cycle of
// a mixed-precision solver is one refinement pass.
template <int B> void one_iteration(tg<B> *g, int type, double omega, int cd, int cu, int hb) {
    const glevel<B> &T = g->lv[0];
    if (uses_mixed(g, type)) {
        mixed_pass(g, cd, cu, hb, type == STZG_TGMG_SYM_VCYCLE);
        return;
    }
    switch (type) {
        case STZG_TGMG_JACOBI:
            k_tg_jacobi<B><<<grid_of(T.m, T.n, kBlk), kBlk, 0, g->st>>>(T);
            launch_note(g);
            cudaMemcpyAsync(T.z, T.r, sizeof(bv<B>) * (size_t)T.m * T.n, cudaMemcpyDeviceToDevice, g->st);
            break;
        case STZG_TGMG_GS: sweep(g, T, false, 1.0); break;
        case STZG_TGMG_SOR: sweep(g, T, false, omega); break;
        case STZG_TGMG_FMG:
            fmg_pre(g, cd, cu, hb, false);
            v_cycle(g, g->v64(), cd, cu, hb, false);
            break;
        case STZG_TGMG_VCYCLE: v_cycle(g, g->v64(), cd, cu, hb, false); break;
        default: v_cycle(g, g->v64(), cd, cu, hb, true); break;
    }
}

template <int B> void drop_graph(tg<B> *g) {
    if (g->gexec) cudaGraphExecDestroy(g->gexec);
    g->gexec = nullptr;
    g->gkey[0] = -1;
}

template <int B> int run_iterations(tg<B> *g, int type, int count, double omega, int cd, int cu, int hb) {
    if (count <= 0) return STZG_OK;
    const int key[5] = {type, cd, cu, hb, uses_mixed(g, type) ? 2 : 1};
    if (!g->gexec || std::memcmp(key, g->gkey, sizeof(key)) != 0 || g->gomega != omega) {
        drop_graph(g);
        const long k0 = g->kernels;
        const long n0 = launch_count();
        cudaGraph_t graph;
        STZG_CUDA(cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal));
        one_iteration(g, type, omega, cd, cu, hb);
        STZG_CUDA(cudaStreamEndCapture(g->st, &graph));
        discount_launches(launch_count() - n0);
        g->gnodes = g->kernels - k0;
        g->kernels = k0;
        cudaError_t e = cudaGraphInstantiate(&g->gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        std::memcpy(g->gkey, key, sizeof(key));
        g->gomega = omega;
    }
    for (int c = 0; c < count; c++) {
        STZG_CUDA(cudaGraphLaunch(g->gexec, g->st));
        g->kernels += g->gnodes;
        for (long k = 0; k < g->gnodes; k++) note_launch();
    }
    return STZG_OK;
}

// l2_error = mds / mn (tgmg.hh:146).
template <int B> int l2_error(tg<B> *g, double *err) {
    const glevel<B> &T = g->lv[0];
    k_tg_sqnorm<B><<<kRedBlocks, kRedThreads, 0, g->st>>>(T, g->partials);
    launch_note(g);
    k_tg_sum<<<1, 256, 0, g->st>>>(g->partials, kRedBlocks, g->dsum);
    launch_note(g);
    STZG_CUDA(cudaMemcpyAsync(g->hsum, g->dsum, sizeof(double), cudaMemcpyDeviceToHost, g->st));
    STZG_CUDA(cudaStreamSynchronize(g->st));
    *err = g->hsum[0] / ((double)T.m * T.n);
    return STZG_OK;
}

// l2_error of the z the last resid_split saw, from its partials.
template <int B> int l2_partials(tg<B> *g, double *err) {
    const glevel<B> &T = g->lv[0];
    k_tg_sum<<<1, 256, 0, g->st>>>(g->partials, kRedBlocks, g->dsum);
    launch_note(g);
    STZG_CUDA(cudaMemcpyAsync(g->hsum, g->dsum, sizeof(double), cudaMemcpyDeviceToHost, g->st));
    STZG_CUDA(cudaStreamSynchronize(g->st));
    *err = g->hsum[0] / ((double)T.m * T.n);
    return STZG_OK;
}

template <int B> int check_l2(tg<B> *g, int type, double *err) {
    return uses_mixed(g, type) ? l2_partials(g, err) : l2_error(g, err);
}

bool valid_type(int t) { return t >= STZG_TGMG_JACOBI && t <= STZG_TGMG_SYM_VCYCLE; }

template <int B> struct timed {
    tg<B> *g;
    long k0;
    explicit timed(tg<B> *g_) : g(g_), k0(g_->kernels) { cudaEventRecord(g->ev0, g->st); }
    void done() {
        cudaEventRecord(g->ev1, g->st);
        cudaEventSynchronize(g->ev1);
        float t = 0;
        cudaEventElapsedTime(&t, g->ev0, g->ev1);
        g->last_ms = t;
        g->last_kernels = g->kernels - k0;
    }
};

// The top level's stencils from the problem's table (9 blocks per stencil,
// B*B doubles each).
template <int B> int fill_top_table(const double *table, int ntable, host_level<B> &top) {
    top.table.resize(ntable);
    std::memset(top.table.data(), 0, sizeof(gst<B>) * ntable);
    for (int c = 0; c < ntable; c++) {
        for (int k = 0; k < 9; k++)
            for (int q = 0; q < B * B; q++) top.table[c].e[k].c[q] = table[((size_t)c * 9 + k) * B * B + q];
        if (block_zero(top.table[c].e[4])) return fail(STZG_EINVAL, "zero diagonal block");
        top.table[c].e[9] = block_inverse<B>(top.table[c].e[4]);
        top.table[c].nz = nonzero_mask(top.table[c]);
    }
    return STZG_OK;
}

// Top level from the problem's table and class map.
template <int B> int top_level(int m, int n, const double *table, int ntable, const int *cls, host_level<B> &top) {
    const size_t mn = (size_t)m * n;
    for (size_t k = 0; k < mn; k++)
        if (cls[k] < 0 || cls[k] >= ntable) return fail(STZG_EINVAL, "stencil index out of range");
    top.m = m;
    top.n = n;
    top.cls.assign(cls, cls + mn);
    STZG_CHECK(fill_top_table<B>(table, ntable, top));
    top.rows = true;
    for (int j = 0; j < n && top.rows; j++)
        for (int i = 1; i < m; i++)
            if (cls[(size_t)j * m + i] != cls[(size_t)j * m]) {
                top.rows = false;
                break;
            }
    return STZG_OK;
}

// Galerkin hierarchy below the top and its upload (tables grow as needed;
// sizes and z/b/r stay).  Also the dense coarsest inverse.
// FP32 copies of every level's stencil table and of the coarsest inverse, for
// the correction cycles of a mixed-precision solver (the FP32 levels share
// the FP64 levels' class maps).  *moved is set where a buffer was
// reallocated.  The host copies stay in the handle.
template <int B> int upload_f32(tg<B> *g, bool *moved) {
    g->host32.resize(g->nl);
    for (int l = 0; l < g->nl; l++) {
        const host_level<B> &H = g->host[l];
        std::vector<gst<B, float>> &t = g->host32[l];
        t.assign(H.table.size(), gst<B, float>{});
        for (size_t c = 0; c < t.size(); c++) {
            for (int k = 0; k < 10; k++)
                for (int q = 0; q < B * B; q++) t[c].e[k].c[q] = (float)H.table[c].e[k].c[q];
            t[c].nz = H.table[c].nz;
        }
        glevel<B, float> &F = g->lf[l];
        if (t.size() > g->stf_cap[l]) {
            void *p;
            STZG_CHECK(g_alloc(g, &p, t.size() * sizeof(gst<B, float>)));
            F.st = (const gst<B, float> *)p;
            g->stf_cap[l] = t.size();
            *moved = true;
        }
        STZG_CUDA(cudaMemcpyAsync((void *)F.st, t.data(), t.size() * sizeof(gst<B, float>), cudaMemcpyHostToDevice,
                                  g->st));
    }
    if (!g->inv_host.empty()) {
        std::vector<float> &f = g->inv_host32;
        f.assign(g->inv_host.begin(), g->inv_host.end());
        if (f.size() > g->inv_f_cap) {
            void *p;
            STZG_CHECK(g_alloc(g, &p, f.size() * sizeof(float)));
            g->inv_f = (float *)p;
            g->inv_f_cap = f.size();
            *moved = true;
        }
        STZG_CUDA(cudaMemcpyAsync(g->inv_f, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice, g->st));
    }
    return STZG_OK;
}

// Galerkin hierarchy below the top and its upload.  A level's class map goes
// up only when it changed (the top's when the caller says so), so a new
// operator on the same stencil pattern (the sheared-coordinates step: the
// strain rate changes the values every step, not which point uses which
// stencil) moves only the tables, a few hundred stencils.  The captured
// iteration graph holds the levels' table pointers and the coarsest inverse
// by value; it is dropped only when one of them moved or the bottom changed
// between the dense inverse and smoothing.
template <int B> int build_hierarchy(tg<B> *g, bool top_cls_kept = false) {
    const std::vector<std::pair<int, int>> sizes = level_sizes(g->host[0].m, g->host[0].n, g->xp, g->yp);
    std::vector<host_level<B>> prev;
    for (size_t l = 1; l < g->host.size(); l++) prev.push_back(std::move(g->host[l]));
    g->host.resize(1);
    g->host[0].cls_kept = top_cls_kept;
    for (size_t l = 1; l < sizes.size(); l++)
        g->host.push_back(coarsen(g->host[l - 1], g->xp, g->yp, sizes[l].first, sizes[l].second,
                                  l - 1 < prev.size() ? &prev[l - 1] : nullptr));
    bool moved = false;
    for (int l = 0; l < g->nl; l++) {
        const host_level<B> &H = g->host[l];
        glevel<B> &L = g->lv[l];
        const size_t pts = (size_t)H.m * H.n;
        if (!H.cls_kept)
            STZG_CUDA(cudaMemcpyAsync((void *)L.cls, H.cls.data(), pts * sizeof(int), cudaMemcpyHostToDevice, g->st));
        if (H.table.size() > g->st_cap[l]) {
            void *p;
            STZG_CHECK(g_alloc(g, &p, H.table.size() * sizeof(gst<B>)));
            L.st = (const gst<B> *)p;
            g->st_cap[l] = H.table.size();
            moved = true;
        }
        STZG_CUDA(cudaMemcpyAsync((void *)L.st, H.table.data(), H.table.size() * sizeof(gst<B>),
                                  cudaMemcpyHostToDevice, g->st));
    }
    const host_level<B> &Bt = g->host.back();
    const double *inv_was = g->inv;
    g->inv = nullptr;
    g->inv_n = 0;
    g->inv_host.clear();
    if (g->nl > 1 && (long)B * Bt.m * Bt.n <= kBottomDirect) {
        std::vector<double> inv = dense_inverse(Bt, g->xp, g->yp);
        g->inv_host = inv;
        if (!inv.empty()) {
            if (inv.size() > g->inv_cap) {
                void *p;
                STZG_CHECK(g_alloc(g, &p, inv.size() * sizeof(double)));
                g->inv_buf = (double *)p;
                g->inv_cap = inv.size();
            }
            g->inv = g->inv_buf;
            g->inv_n = B * Bt.m * Bt.n;
            STZG_CUDA(cudaMemcpyAsync(g->inv, inv.data(), inv.size() * sizeof(double), cudaMemcpyHostToDevice,
                                      g->st));
        }
    }
    if (g->have32) STZG_CHECK(upload_f32(g, &moved));
    if (moved || g->inv != inv_was) drop_graph(g);
    STZG_CUDA(cudaStreamSynchronize(g->st));  // the host vectors are uploaded before they go
    return STZG_OK;
}

// Mixed precision on (V-cycle solves as refinement passes) or off.  The FP32
// levels are made on first use: z, b, r per level and the tables.
template <int B> int tg_set_precision(tg<B> *g, int precision) {
    if (precision == 0) {
        g->mixed = false;
        return STZG_OK;
    }
    if (!g->have32) {
        for (int l = 0; l < g->nl; l++) {
            const glevel<B> &L = g->lv[l];
            glevel<B, float> &F = g->lf[l];
            F.m = L.m;
            F.n = L.n;
            F.xp = L.xp;
            F.yp = L.yp;
            F.cx_n = L.cx_n;
            F.cy_n = L.cy_n;
            F.cls = L.cls;
            const size_t bytes = sizeof(bv<B, float>) * (size_t)L.m * L.n;
            void *p;
            STZG_CHECK(g_alloc(g, &p, bytes));
            F.z = (bv<B, float> *)p;
            STZG_CHECK(g_alloc(g, &p, bytes));
            F.b = (bv<B, float> *)p;
            STZG_CHECK(g_alloc(g, &p, bytes));
            F.r = (bv<B, float> *)p;
        }
        if (g->tail_start_f < g->nl &&
            cudaFuncSetAttribute(k_tg_tail<B, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTailSmem) !=
                cudaSuccess)
            return fail(STZG_ECUDA, "tail kernel attribute");
        bool moved = false;
        STZG_CHECK(upload_f32(g, &moved));
        STZG_CUDA(cudaStreamSynchronize(g->st));
        g->have32 = true;
    }
    g->mixed = true;
    return STZG_OK;
}

}  // namespace
}  // namespace stzg

using namespace stzg;

struct stzg_tgmg {
    int B = 1;
    tg<1> *s1 = nullptr;
    tg<2> *s2 = nullptr;
};

namespace {

template <int B> void tg_destroy(tg<B> *g) {
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->st) cudaStreamSynchronize(g->st);
    drop_graph(g);
    for (void *p : g->owned) cudaFree(p);
    if (g->hsum) cudaFreeHost(g->hsum);
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    if (g->st) cudaStreamDestroy(g->st);
    delete g;
}

template <int B>
int tg_create(int m, int n, int xp, int yp, const double *table, int ntable, const int *cls, double acc, int device,
              tg<B> **out) {
    tg<B> *g = new tg<B>;
    g->device = device;
    g->xp = xp ? 1 : 0;
    g->yp = yp ? 1 : 0;
    g->acc = acc;
    auto bail = [&](int st) {
        tg_destroy(g);
        return st;
    };
    if (cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&g->ev0) != cudaSuccess || cudaEventCreate(&g->ev1) != cudaSuccess)
        return bail(fail(STZG_ECUDA, "stream/event creation failed"));
    host_level<B> top;
    int st;
    if ((st = top_level<B>(m, n, table, ntable, cls, top)) != STZG_OK) return bail(st);
    g->host.push_back(top);
    const std::vector<std::pair<int, int>> sizes = level_sizes(m, n, g->xp, g->yp);
    g->nl = (int)sizes.size();
    for (int l = 0; l < g->nl; l++) {
        glevel<B> &L = g->lv[l];
        L.m = sizes[l].first;
        L.n = sizes[l].second;
        L.xp = g->xp;
        L.yp = g->yp;
        L.cx_n = (g->xp && (L.m & 1)) ? 3 : 2;
        L.cy_n = (g->yp && (L.n & 1)) ? 3 : 2;
        const size_t pts = (size_t)L.m * L.n;
        void *p;
        if ((st = g_alloc(g, &p, pts * sizeof(bv<B>))) != STZG_OK) return bail(st);
        L.z = (bv<B> *)p;
        if ((st = g_alloc(g, &p, pts * sizeof(bv<B>))) != STZG_OK) return bail(st);
        L.b = (bv<B> *)p;
        if ((st = g_alloc(g, &p, pts * sizeof(bv<B>))) != STZG_OK) return bail(st);
        L.r = (bv<B> *)p;
        if ((st = g_alloc(g, &p, pts * sizeof(int))) != STZG_OK) return bail(st);
        L.cls = (const int *)p;
        L.st = nullptr;
    }
    if ((st = build_hierarchy(g)) != STZG_OK) return bail(st);
    // single-block tail: the small levels that fit in its shared memory
    // together, if they are at least two (the coarsest alone is the bottom)
    {
        int ms[kMaxLevels], ns[kMaxLevels];
        for (int l = 0; l < g->nl; l++) {
            ms[l] = g->lv[l].m;
            ns[l] = g->lv[l].n;
        }
        g->tail_start = tail_start_for(ms, ns, g->nl, sizeof(bv<B>), kTailPoints);
        g->tail_start_f = tail_start_for(ms, ns, g->nl, sizeof(bv<B, float>), kTailPointsF);
        if (g->tail_start < g->nl &&
            cudaFuncSetAttribute(k_tg_tail<B, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTailSmem) !=
                cudaSuccess)
            return bail(fail(STZG_ECUDA, "tail kernel attribute"));
    }
    {
        void *p;
        if ((st = g_alloc(g, &p, kRedBlocks * sizeof(double))) != STZG_OK) return bail(st);
        g->partials = (double *)p;
        if ((st = g_alloc(g, &p, sizeof(double))) != STZG_OK) return bail(st);
        g->dsum = (double *)p;
        if (cudaMallocHost(&p, sizeof(double)) != cudaSuccess) return bail(fail(STZG_ENOMEM, "pinned allocation"));
        g->hsum = (double *)p;
    }
    if (cudaStreamSynchronize(g->st) != cudaSuccess) return bail(fail(STZG_ECUDA, "setup failed"));
    *out = g;
    return STZG_OK;
}

// cls null: the class map of the last operator stays (ntable must match).
template <int B> int tg_set_operator(tg<B> *g, const double *table, int ntable, const int *cls) {
    host_level<B> &T = g->host[0];
    const size_t mn = (size_t)T.m * T.n;
    const bool kept = !cls || std::memcmp(cls, T.cls.data(), mn * sizeof(int)) == 0;
    if (!cls && ntable != (int)T.table.size()) return fail(STZG_EINVAL, "stencil count differs from the class map's");
    host_level<B> top;
    if (kept) {
        // the same class map: new stencil values only
        for (size_t k = 0; k < mn && cls; k++)
            if (cls[k] >= ntable) return fail(STZG_EINVAL, "stencil index out of range");
        top.m = T.m;
        top.n = T.n;
        top.rows = T.rows;
        top.cls.swap(T.cls);
        const int st = fill_top_table<B>(table, ntable, top);
        if (st != STZG_OK) {
            T.cls.swap(top.cls);
            return st;
        }
    } else {
        STZG_CHECK(top_level<B>(T.m, T.n, table, ntable, cls, top));
    }
    STZG_CUDA(cudaStreamSynchronize(g->st));
    g->host[0] = std::move(top);
    return build_hierarchy(g, kept);
}

template <int B> int tg_copy(tg<B> *g, bv<B> *dev, const double *src, double *dst) {
    const size_t bytes = sizeof(bv<B>) * (size_t)g->lv[0].m * g->lv[0].n;
    if (src) STZG_CUDA(cudaMemcpyAsync(dev, src, bytes, cudaMemcpyHostToDevice, g->st));
    else STZG_CUDA(cudaMemcpyAsync(dst, dev, bytes, cudaMemcpyDeviceToHost, g->st));
    STZG_CUDA(cudaStreamSynchronize(g->st));
    return STZG_OK;
}

template <int B>
int tg_solve(tg<B> *g, int type, stzg_tgmg_predict *tp, double omega, int cd, int cu, int hb, int *iters,
             double *l2) {
    timed<B> t(g);
    // tgmg::solve(type, tgmg_predict&, ...), tgmg.in.cc:266-301
    if (uses_mixed(g, type)) resid_split(g);
    int nit = tp->lim / tp->mult;
    STZG_CHECK(run_iterations(g, type, nit, omega, cd, cu, hb));
    double acc;
    STZG_CHECK(check_l2(g, type, &acc));
    if (acc < g->acc) {
        if (tp->lim > 0) tp->lim -= 1 + tp->lim / tp->decay;
    } else {
        int k = 0;
        do {
            tp->lim += ++k * tp->mult;
            if (tp->lim > tp->max_thresh) {
                t.done();
                if (l2) *l2 = acc;
                return fail(STZG_ENOTCONV, "tgmg did not converge");
            }
            nit += k;
            STZG_CHECK(run_iterations(g, type, k, omega, cd, cu, hb));
            STZG_CHECK(check_l2(g, type, &acc));
        } while (acc >= g->acc && !std::isnan(acc));
    }
    tp->solves++;
    tp->vcount += nit;
    STZG_CHECK(run_iterations(g, type, tp->extra_iters, omega, cd, cu, hb));
    t.done();
    if (iters) *iters = nit;
    if (l2) *l2 = acc;
    if (std::isnan(acc)) return fail(STZG_ENAN, "NaN residual");
    return STZG_OK;
}

// Not in the reference: iterations until l2_error < acc, tested before the
// first (a warm start may already meet it) and after every one, at most
// max_iters, then extra more (the reference's extra_iters).  Unlike the
// predictor's counts, none beyond the need.
template <int B>
int tg_solve_checked(tg<B> *g, int type, int max_iters, int extra, double omega, int cd, int cu, int hb, int *iters,
                     double *l2) {
    timed<B> t(g);
    if (uses_mixed(g, type)) resid_split(g);
    double acc;
    int nit = 0;
    STZG_CHECK(check_l2(g, type, &acc));
    while (acc >= g->acc && !std::isnan(acc)) {
        if (nit == max_iters) {
            t.done();
            if (iters) *iters = nit;
            if (l2) *l2 = acc;
            return fail(STZG_ENOTCONV, "tgmg did not converge");
        }
        STZG_CHECK(run_iterations(g, type, 1, omega, cd, cu, hb));
        nit++;
        STZG_CHECK(check_l2(g, type, &acc));
    }
    if (!std::isnan(acc)) STZG_CHECK(run_iterations(g, type, extra, omega, cd, cu, hb));
    t.done();
    if (iters) *iters = nit;
    if (l2) *l2 = acc;
    if (std::isnan(acc)) return fail(STZG_ENAN, "NaN residual");
    return STZG_OK;
}

template <int B>
int tg_solve_fixed(tg<B> *g, int type, int per_loop, int max_loops, double omega, int cd, int cu, int hb,
                   int *iters, double *l2) {
    timed<B> t(g);
    // tgmg::solve(type, per_loop, max_loops, ...), tgmg.in.cc:182-197
    if (uses_mixed(g, type)) resid_split(g);
    double acc = 0;
    int nloop = 0;
    do {
        if (++nloop == max_loops) {
            t.done();
            if (iters) *iters = nloop * per_loop;
            if (l2) *l2 = acc;
            return fail(STZG_ENOTCONV, "tgmg did not converge");
        }
        STZG_CHECK(run_iterations(g, type, per_loop, omega, cd, cu, hb));
        STZG_CHECK(check_l2(g, type, &acc));
    } while (acc > g->acc && !std::isnan(acc));
    t.done();
    if (iters) *iters = nloop * per_loop;
    if (l2) *l2 = acc;
    if (std::isnan(acc)) return fail(STZG_ENAN, "NaN residual");
    return STZG_OK;
}

template <int B> int tg_iterate(tg<B> *g, int type, int count, double omega, int cd, int cu, int hb) {
    timed<B> t(g);
    if (uses_mixed(g, type) && count > 0) resid_split(g);
    STZG_CHECK(run_iterations(g, type, count, omega, cd, cu, hb));
    t.done();
    STZG_CUDA(cudaGetLastError());
    return STZG_OK;
}

template <int B> int tg_levels(tg<B> *g, int *nlevels, int *dims) {
    *nlevels = g->nl;
    if (dims)
        for (int l = 0; l < g->nl; l++) {
            dims[2 * l] = g->lv[l].m;
            dims[2 * l + 1] = g->lv[l].n;
        }
    return STZG_OK;
}

template <int B> int tg_stencil(tg<B> *g, int level, double *out) {
    if (level < 1 || level >= g->nl) return fail(STZG_EINVAL, "bad level");
    const host_level<B> &H = g->host[level];
    const size_t pts = (size_t)H.m * H.n, per = 10 * B * B;
    for (size_t k = 0; k < pts; k++) std::memcpy(out + per * k, H.table[H.cls[k]].e, per * sizeof(double));
    return STZG_OK;
}

// Calls f on the handle's state with its block size.
template <typename F> int dispatch(stzg_tgmg *g, F f) {
    if (!g) return fail(STZG_EINVAL, "null handle");
    if (g->B == 1) {
        STZG_CUDA(cudaSetDevice(g->s1->device));
        return f(g->s1);
    }
    STZG_CUDA(cudaSetDevice(g->s2->device));
    return f(g->s2);
}

}  // namespace

extern "C" {

void stzg_tgmg_predict_init(stzg_tgmg_predict *tp) {
    if (!tp) return;
    tp->mult = 16;
    tp->decay = 32;
    tp->max_thresh = 16 * 2048;
    tp->extra_iters = 1;
    tp->lim = 16 * 8;
    tp->solves = 0;
    tp->vcount = 0;
}

int stzg_poisson_fd(int m, int n, double ax, double bx, double ay, double by, double *table, int *cls,
                    double *acc) {
    if (m < 2 || n < 2 || !table || !cls || !acc) return fail(STZG_EINVAL, "poisson_fd needs m,n >= 2");
    // poisson_fd::poisson_fd (poisson_fd.cc:12-16)
    const double dx = (bx - ax) / (m - 1), dy = (by - ay) / (n - 1);
    const double hcc = -2 / (dx * dx) - 2 / (dy * dy), hxx = 1. / (dx * dx), hyy = 1. / (dy * dy);
    const double a = DBL_EPSILON * 1e4 * hcc;  // tgmg_accuracy(hcc, 1e4), tgmg.hh:42-45
    *acc = a * a;
    const double interior[9] = {0, hyy, 0, hxx, hcc, hxx, 0, hyy, 0};
    for (int k = 0; k < 9; k++) {
        table[k] = interior[k];
        table[9 + k] = k == 4 ? hcc : 0;
    }
    // edge() (poisson_fd.hh:38): i==0 || i==m-1 || first or last row
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) cls[(size_t)j * m + i] = (i == 0 || i == m - 1 || j == 0 || j == n - 1) ? 1 : 0;
    return STZG_OK;
}

int stzg_tgmg_create_block(int m, int n, int x_prd, int y_prd, int block, const double *table, int ntable,
                           const int *cls, double acc, int device, stzg_tgmg **out) {
    if (!out) return fail(STZG_EINVAL, "null handle pointer");
    *out = nullptr;
    if (block != 1 && block != 2) return fail(STZG_EINVAL, "block must be 1 or 2");
    if (m < 1 || n < 1 || !table || ntable < 1 || !cls) return fail(STZG_EINVAL, "bad grid or operator");
    if ((long)m * n > (1L << 30)) return fail(STZG_EINVAL, "more than 2^30 grid points");
    if ((x_prd && m < 3) || (y_prd && n < 3)) return fail(STZG_EINVAL, "a periodic direction needs >= 3 points");
    if (!(acc >= 0)) return fail(STZG_EINVAL, "acc must be >= 0");
    const size_t mn = (size_t)m * n;
    for (size_t k = 0; k < mn; k++)
        if (cls[k] < 0 || cls[k] >= ntable) return fail(STZG_EINVAL, "stencil index out of range");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(STZG_ENODEV, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(STZG_EINVAL, "device ordinal out of range");
    STZG_CUDA(cudaSetDevice(device));
    stzg_tgmg *g = new stzg_tgmg;
    g->B = block;
    const int st = block == 1 ? tg_create<1>(m, n, x_prd, y_prd, table, ntable, cls, acc, device, &g->s1)
                              : tg_create<2>(m, n, x_prd, y_prd, table, ntable, cls, acc, device, &g->s2);
    if (st != STZG_OK) {
        delete g;
        return st;
    }
    *out = g;
    return STZG_OK;
}

int stzg_tgmg_create(int m, int n, int x_prd, int y_prd, const double *table, int ntable, const int *cls,
                     double acc, int device, stzg_tgmg **out) {
    return stzg_tgmg_create_block(m, n, x_prd, y_prd, 1, table, ntable, cls, acc, device, out);
}

int stzg_tgmg_destroy(stzg_tgmg *g) {
    if (!g) return STZG_OK;
    tg_destroy(g->s1);
    tg_destroy(g->s2);
    delete g;
    return STZG_OK;
}

int stzg_tgmg_set_operator(stzg_tgmg *g, const double *table, int ntable, const int *cls) {
    if (!table || ntable < 1) return fail(STZG_EINVAL, "bad operator");
    return dispatch(g, [&](auto *s) { return tg_set_operator(s, table, ntable, cls); });
}

int stzg_tgmg_set_precision(stzg_tgmg *g, int precision) {
    if (precision != 0 && precision != 1) return fail(STZG_EINVAL, "precision must be 0 (FP64) or 1 (mixed)");
    return dispatch(g, [&](auto *s) { return tg_set_precision(s, precision); });
}

int stzg_tgmg_set_b(stzg_tgmg *g, const double *b) {
    if (!b) return fail(STZG_EINVAL, "null argument");
    return dispatch(g, [&](auto *s) { return tg_copy(s, s->lv[0].b, b, nullptr); });
}
int stzg_tgmg_get_b(stzg_tgmg *g, double *b) {
    if (!b) return fail(STZG_EINVAL, "null argument");
    return dispatch(g, [&](auto *s) { return tg_copy(s, s->lv[0].b, nullptr, b); });
}
int stzg_tgmg_set_z(stzg_tgmg *g, const double *z) {
    if (!z) return fail(STZG_EINVAL, "null argument");
    return dispatch(g, [&](auto *s) { return tg_copy(s, s->lv[0].z, z, nullptr); });
}
int stzg_tgmg_get_z(stzg_tgmg *g, double *z) {
    if (!z) return fail(STZG_EINVAL, "null argument");
    return dispatch(g, [&](auto *s) { return tg_copy(s, s->lv[0].z, nullptr, z); });
}

int stzg_tgmg_device_arrays(stzg_tgmg *g, double **b, double **z) {
    if (!g || !b || !z) return fail(STZG_EINVAL, "null argument");
    if (g->B == 1) {
        *b = (double *)g->s1->lv[0].b;
        *z = (double *)g->s1->lv[0].z;
    } else {
        *b = (double *)g->s2->lv[0].b;
        *z = (double *)g->s2->lv[0].z;
    }
    return STZG_OK;
}

int stzg_tgmg_clear_z(stzg_tgmg *g) {
    return dispatch(g, [&](auto *s) -> int {
        clear_z(s, s->lv[0]);
        STZG_CUDA(cudaStreamSynchronize(s->st));
        return STZG_OK;
    });
}

int stzg_tgmg_l2_error(stzg_tgmg *g, double *err) {
    if (!err) return fail(STZG_EINVAL, "null argument");
    return dispatch(g, [&](auto *s) { return l2_error(s, err); });
}

int stzg_tgmg_iterate(stzg_tgmg *g, int type, int count, double omega, int cyc_down, int cyc_up, int hcyc_bottom) {
    if (!valid_type(type) || count < 0 || cyc_down < 0 || cyc_up < 0 || hcyc_bottom < 0)
        return fail(STZG_EINVAL, "bad iterate arguments");
    return dispatch(g, [&](auto *s) { return tg_iterate(s, type, count, omega, cyc_down, cyc_up, hcyc_bottom); });
}

int stzg_tgmg_solve(stzg_tgmg *g, int type, stzg_tgmg_predict *tp, double omega, int cyc_down, int cyc_up,
                    int hcyc_bottom, int *iters, double *l2) {
    if (!tp || !valid_type(type) || tp->mult < 1 || cyc_down < 0 || cyc_up < 0 || hcyc_bottom < 0)
        return fail(STZG_EINVAL, "bad solve arguments");
    return dispatch(g, [&](auto *s) { return tg_solve(s, type, tp, omega, cyc_down, cyc_up, hcyc_bottom, iters, l2); });
}

int stzg_tgmg_solve_fixed(stzg_tgmg *g, int type, int per_loop, int max_loops, double omega, int cyc_down,
                          int cyc_up, int hcyc_bottom, int *iters, double *l2) {
    if (!valid_type(type) || per_loop < 1 || max_loops < 1 || cyc_down < 0 || cyc_up < 0 || hcyc_bottom < 0)
        return fail(STZG_EINVAL, "bad solve arguments");
    return dispatch(g, [&](auto *s) {
        return tg_solve_fixed(s, type, per_loop, max_loops, omega, cyc_down, cyc_up, hcyc_bottom, iters, l2);
    });
}

int stzg_tgmg_solve_checked(stzg_tgmg *g, int type, int max_iters, int extra_iters, double omega, int cyc_down,
                            int cyc_up, int hcyc_bottom, int *iters, double *l2) {
    if (!valid_type(type) || max_iters < 0 || extra_iters < 0 || cyc_down < 0 || cyc_up < 0 || hcyc_bottom < 0)
        return fail(STZG_EINVAL, "bad solve arguments");
    return dispatch(g, [&](auto *s) {
        return tg_solve_checked(s, type, max_iters, extra_iters, omega, cyc_down, cyc_up, hcyc_bottom, iters, l2);
    });
}

int stzg_tgmg_levels(stzg_tgmg *g, int *nlevels, int *dims) {
    if (!nlevels) return fail(STZG_EINVAL, "null argument");
    if (!g) return fail(STZG_EINVAL, "null handle");
    return g->B == 1 ? tg_levels(g->s1, nlevels, dims) : tg_levels(g->s2, nlevels, dims);
}

int stzg_tgmg_stencil(stzg_tgmg *g, int level, double *out) {
    if (!out || !g) return fail(STZG_EINVAL, "null argument");
    return g->B == 1 ? tg_stencil(g->s1, level, out) : tg_stencil(g->s2, level, out);
}

int stzg_tgmg_last_timing(stzg_tgmg *g, double *ms, long *kernels) {
    if (!g) return fail(STZG_EINVAL, "null handle");
    const double t = g->B == 1 ? g->s1->last_ms : g->s2->last_ms;
    const long k = g->B == 1 ? g->s1->last_kernels : g->s2->last_kernels;
    if (ms) *ms = t;
    if (kernels) *kernels = k;
    return STZG_OK;
}

}  // extern "C"
