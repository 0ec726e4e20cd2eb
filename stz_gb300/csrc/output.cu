// Frame export and diagnostics on the device: the Gnuplot binary matrices
// of shear_sim::output (shear_sim.cc:684-720) and write_files (:659-676),
// the quasi-staticity measure qs_measure (:733-775), the wall tractions
// (:1003-1028) and the Hencky strain compute_strain (:778-824).
//
// Every matrix is assembled in FP32 on the GPU (header row of x positions,
// one row per grid line with its y position first), so one device-to-host
// copy gives the file's bytes.  Coordinates and the derived values (|s|,
// chi*TZ, the periodic copy of X) are computed with the reference's
// operation order in IEEE double (no contraction) before the float
// conversion, so the bytes match the reference's files.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "sim.cuh"

namespace stzg {
namespace {

#define IDX(i, j) ((size_t)((j) + 1) * m + (i))

struct out_args {
    const double *f[F_COUNT];  // state buffer (rows -1..n)
    const double2 *vel;        // node velocity (rows 0..n), walls substituted
    const double *proj;        // qs_measure integrand per node (rows 0..n), or null
    int m, n, mode;
    double bv, ax, ay, bx, dx, dy, TZ;
};

__device__ __forceinline__ bool staggered_mode(int mode) { return mode >= 2 && mode <= 8; }

__device__ double out_value(const out_args &a, int i, int j) {
    const int m = a.m, n = a.n;
    switch (a.mode) {
        case 0: return j == 0 ? -a.bv : (j == n ? a.bv : a.vel[(size_t)j * m + i].x);
        case 1: return (j == 0 || j == n) ? 0.0 : a.vel[(size_t)j * m + i].y;
        case 2: return a.f[F_P][IDX(i, j)];
        case 3: return a.f[F_Q][IDX(i, j)];
        case 4: return a.f[F_S][IDX(i, j)];
        case 5: return a.f[F_TAU][IDX(i, j)];
        case 6: return a.f[F_CHI][IDX(i, j)];
        case 7: return __dmul_rn(a.f[F_CHI][IDX(i, j)], a.TZ);
        case 8: {  // c_field::dev(), fields.hh:85-93
            const double q = a.f[F_Q][IDX(i, j)], s = a.f[F_S][IDX(i, j)], t = a.f[F_TAU][IDX(i, j)];
            return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(3.0, q), q), __dmul_rn(s, s)), __dmul_rn(t, t)));
        }
        case 9: return a.f[F_X][IDX(i, j)];
        case 10: return a.f[F_Y][IDX(i, j)];
        default: return a.proj ? a.proj[(size_t)j * m + i] : 0.0;
    }
}

// One thread per float of the matrix ((rows + 1) x (l + 1)).
__global__ void k_gnuplot(out_args a, float *out) {
    const bool st = staggered_mode(a.mode);
    const int l = st ? a.m : a.m + 1, rows = st ? a.n : a.n + 1, w = l + 1;
    const long total = (long)(rows + 1) * w;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (long)gridDim.x * blockDim.x) {
        const int r = (int)(k / w), c = (int)(k - (long)r * w);
        float v;
        if (r == 0) {
            v = c == 0 ? (float)l
                       : (float)__dadd_rn(a.ax, st ? __dmul_rn((c - 1) + 0.5, a.dx) : __dmul_rn((double)(c - 1), a.dx));
        } else {
            const int j = r - 1;
            if (c == 0) {
                v = (float)__dadd_rn(a.ay, st ? __dmul_rn(j + 0.5, a.dy) : __dmul_rn((double)j, a.dy));
            } else if (c <= a.m) {
                v = (float)out_value(a, c - 1, j);
            } else {
                // periodic copy of the first value (X shifted by the period)
                const float first = (float)out_value(a, 0, j);
                v = a.mode == 9 ? (float)__dadd_rn(__dadd_rn((double)first, a.bx), -a.ax) : first;
            }
        }
        out[k] = v;
    }
}

// Integrand of qs_measure on rows 1..n-2 (proj rows 0, n-1, n stay zero)
// and per-block partial sum and maximum.  Staggered: the velocity gradient
// of the cell spanned by nodes (i,j)..(i+1,j+1) of the solver array;
// otherwise central differences of the node velocity.
__global__ void k_qs_measure(const double2 *__restrict__ vel, int m, int n, double bv, double xsp, double ysp,
                             double qsf1, double qsf2, int staggered, double *proj, double *partials) {
    __shared__ double ssum[256], smax[256];
    double sum = 0, mx = 0;
    const long total = (long)m * (n > 2 ? n - 2 : 0);
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (long)gridDim.x * blockDim.x) {
        const int j = 1 + (int)(k / m), i = (int)(k % m);
        double ux, uy, vx, vy;
        if (staggered) {
            const int ir = i == m - 1 ? 0 : i + 1;
            const double2 a = vel[(size_t)j * m + i], b = vel[(size_t)j * m + ir], c = vel[(size_t)(j + 1) * m + i],
                          d = vel[(size_t)(j + 1) * m + ir];
            ux = 0.5 * xsp * (-a.x + b.x - c.x + d.x);
            uy = 0.5 * ysp * (-a.x - b.x + c.x + d.x);
            vx = 0.5 * xsp * (-a.y + b.y - c.y + d.y);
            vy = 0.5 * ysp * (-a.y - b.y + c.y + d.y);
        } else {
            const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
            auto U = [&](int ii, int jj) { return jj == 0 ? -bv : (jj == n ? bv : vel[(size_t)jj * m + ii].x); };
            auto V = [&](int ii, int jj) { return (jj == 0 || jj == n) ? 0.0 : vel[(size_t)jj * m + ii].y; };
            ux = 0.5 * xsp * (U(ir, j) - U(il, j));
            vx = 0.5 * xsp * (V(ir, j) - V(il, j));
            uy = 0.5 * ysp * (U(i, j + 1) - U(i, j - 1));
            vy = 0.5 * ysp * (V(i, j + 1) - V(i, j - 1));
        }
        const double l1 = ux + vy, l2 = ux - vy, l3 = uy + vx;
        const double q = qsf1 * l1 * l1 + qsf2 * (l2 * l2 + l3 * l3);
        proj[(size_t)j * m + i] = q;
        sum += q;
        mx = fmax(mx, q);
    }
    ssum[threadIdx.x] = sum;
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            ssum[threadIdx.x] += ssum[threadIdx.x + w];
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = ssum[0];
        partials[2 * blockIdx.x + 1] = smax[0];
    }
}

// Wall tractions: sums over the bottom two and top two cell rows.
__global__ void k_tractions(const double *__restrict__ P, const double *__restrict__ Q, const double *__restrict__ S,
                            const double *__restrict__ T, int m, int n, double *out) {
    __shared__ double sh[4][256];
    double acc[4] = {0, 0, 0, 0};
    auto syy = [&](size_t c) { return -P[c] - S[c] - Q[c]; };  // c_field::syy, fields.hh:97-99
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const size_t c0 = IDX(i, 0), c1 = IDX(i, 1), a = IDX(i, n - 2), b = IDX(i, n - 1);
        acc[0] += 3 * T[c0] - T[c1];
        acc[1] += 3 * syy(c0) - syy(c1);
        acc[2] -= 3 * T[b] - T[a];
        acc[3] -= 3 * syy(b) - syy(a);
    }
    for (int k = 0; k < 4; k++) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < 4; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 4) out[threadIdx.x] = sh[threadIdx.x][0];
}

// Hencky strain |dev(0.5 log(F^T F))| per c_field (i, j), j = 0..n-1, from
// the reference map at the node (i, j) (shear_sim::compute_strain).  The
// reference's interior y difference subtracts the row above from itself
// (fd = fp + m, shear_sim.cc:799), so Xy = Yy = 0 there, the deformation
// gradient is singular and the strain is 0; rows 0 and n-1 use one-sided
// differences.  Both are restated as they are.
__global__ void k_strain(const double *__restrict__ X, const double *__restrict__ Y, int m, int n, double lx,
                         double xsp, double ysp, double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j >= n) return;
    double Xx, Yx;
    if (i == 0) {
        Xx = X[IDX(1, j)] - X[IDX(m - 1, j)] + lx;
        Yx = Y[IDX(1, j)] - Y[IDX(m - 1, j)];
    } else if (i == m - 1) {
        Xx = X[IDX(0, j)] - X[IDX(m - 2, j)] - lx;
        Yx = Y[IDX(0, j)] - Y[IDX(m - 2, j)];
    } else {
        Xx = X[IDX(i + 1, j)] - X[IDX(i - 1, j)];
        Yx = Y[IDX(i + 1, j)] - Y[IDX(i - 1, j)];
    }
    Xx *= 0.5 * xsp;
    Yx *= 0.5 * xsp;
    double yfac;
    size_t fu, fd;
    if (j == 0 || j == n - 1) {
        yfac = ysp;
        fu = IDX(i, j + 1);
        fd = IDX(i, j);
    } else {
        yfac = 0.5 * ysp;
        fu = IDX(i, j + 1);
        fd = IDX(i, j + 1);
    }
    const double Xy = yfac * (X[fu] - X[fd]), Yy = yfac * (Y[fu] - Y[fd]);
    const double Jinv = Xx * Yy - Xy * Yx, J = 1 / Jinv;
    const double Fa = Yy * J, Fb = -Xy * J, Fc = -Yx * J, Fd = Xx * J;
    // F^T F (mat::transpose, mat::operator*, mat.hh:21,57)
    const double a = Fa * Fa + Fc * Fc, b = Fa * Fb + Fc * Fd, c = Fb * Fa + Fd * Fc, d = Fb * Fb + Fd * Fd;
    // mat::sym_eigenvectors (esim/shared/mat.cc:8-26)
    double l1, l2, La, Lb, Lc, Ld;
    if (fabs(b) < 1e-12 * (fabs(a) + fabs(d))) {
        if (a > d) {
            l1 = a; l2 = d; La = 1; Lb = 0; Lc = 0; Ld = 1;
        } else {
            l1 = d; l2 = a; La = 0; Lb = 1; Lc = 1; Ld = 0;
        }
    } else {
        const double det = sqrt((a - d) * (a - d) + 4 * b * b);
        l1 = 0.5 * (a + d + det);
        l2 = 0.5 * (a + d - det);
        const double r = b, s = a - l1, nor1 = 1 / sqrt(r * r + s * s);
        La = r * nor1; Lb = -s * nor1; Lc = s * nor1; Ld = r * nor1;
    }
    (void)c;
    double res = 0;
    if (l1 > 0 || l2 > 0) {
        const double e1 = 0.5 * log(l1), e2 = 0.5 * log(l2);
        // Lam^T diag(e1, e2) Lam
        const double Ma = La * e1, Mb = Lc * e2, Mc = Lb * e1, Md = Ld * e2;  // Lam^T * diag
        const double sa = Ma * La + Mb * Lc, sb = Ma * Lb + Mb * Ld, sc = Mc * La + Md * Lc, sd = Mc * Lb + Md * Ld;
        res = sqrt(0.5 * (sa - sd) * (sa - sd) + sb * sb + sc * sc);  // mat::devmod, mat.hh:51
    }
    out[(size_t)j * m + i] = res;
}

#undef IDX

const char *mode_prefix(int mode) {
    static const char *names[12] = {"u", "v", "p", "q", "s", "tau", "chi", "tem", "dev", "X", "Y", "proj"};
    return names[mode];
}

int ensure_proj(stzg_sim *s) {
    if (s->proj) return STZG_OK;
    return dev_alloc(s, (void **)&s->proj, (size_t)s->m * (s->n + 1) * sizeof(double));
}

}  // namespace
}  // namespace stzg

using namespace stzg;

extern "C" {

int stzg_output_field(stzg_sim *s, int mode, float *out, long *count) {
    if (!s || mode < 0 || mode > 11) return fail(STZG_EINVAL, "output mode must be 0..11");
    const bool st = mode >= 2 && mode <= 8;
    const long l = st ? s->m : s->m + 1, rows = st ? s->n : s->n + 1, total = (rows + 1) * (l + 1);
    if (count) *count = total;
    if (!out) return STZG_OK;
    out_args a;
    for (int k = 0; k < F_COUNT; k++) a.f[k] = s->F.f[s->cur][k];
    a.vel = s->F.vel;
    a.proj = s->proj;
    a.m = s->m;
    a.n = s->n;
    a.mode = mode;
    a.bv = s->bv_state;
    a.ax = s->P.ax;
    a.ay = s->P.ay;
    a.bx = s->P.bx;
    a.dx = (s->P.bx - s->P.ax) / s->m;
    a.dy = (s->P.by - s->P.ay) / s->n;
    a.TZ = s->P.TZ;
    float *dev = nullptr;
    STZG_CUDA(cudaMallocAsync((void **)&dev, total * sizeof(float), s->st));
    k_gnuplot<<<ceil_div(total, 256) < 4 * 152 ? ceil_div(total, 256) : 4 * 152, 256, 0, s->st>>>(a, dev);
    note_launch();
    cudaError_t e = cudaMemcpyAsync(out, dev, total * sizeof(float), cudaMemcpyDeviceToHost, s->st);
    cudaFreeAsync(dev, s->st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(output)");
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

int stzg_qs_measure(stzg_sim *s, int staggered, double *Q, double *max_qs) {
    if (!s || !Q || !max_qs) return fail(STZG_EINVAL, "null argument");
    STZG_CHECK(ensure_proj(s));
    const double K = s->P.K, mu = s->P.mu;
    const double qsf1 = 6 * K * mu * (K + (1 / 3.0) * mu), qsf2 = 6 * K * mu * mu;
    const double dx = (s->P.bx - s->P.ax) / s->m, dy = (s->P.by - s->P.ay) / s->n;
    k_qs_measure<<<s->npart, 256, 0, s->st>>>(s->F.vel, s->m, s->n, s->bv_state, 1 / dx, 1 / dy, qsf1, qsf2,
                                              staggered, s->proj, s->partials);
    note_launch();
    std::vector<double> part(2 * (size_t)s->npart);
    STZG_CUDA(cudaMemcpyAsync(part.data(), s->partials, part.size() * 8, cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    double sum = 0, mx = 0;
    for (int k = 0; k < s->npart; k++) {
        sum += part[2 * k];
        mx = std::fmax(mx, part[2 * k + 1]);
    }
    *Q = std::sqrt(sum * dx * dy);
    *max_qs = mx;
    return STZG_OK;
}

int stzg_tractions(stzg_sim *s, double *out) {
    if (!s || !out) return fail(STZG_EINVAL, "null argument");
    if (s->n < 2) return fail(STZG_EINVAL, "tractions need two cell rows");
    double *const *f = s->F.f[s->cur];
    k_tractions<<<1, 256, 0, s->st>>>(f[F_P], f[F_Q], f[F_S], f[F_TAU], s->m, s->n, s->partials);
    note_launch();
    double h[4];
    STZG_CUDA(cudaMemcpyAsync(h, s->partials, sizeof(h), cudaMemcpyDeviceToHost, s->st));
    STZG_CUDA(cudaStreamSynchronize(s->st));
    const double dx = (s->P.bx - s->P.ax) / s->m;
    for (int k = 0; k < 4; k++) out[k] = h[k] * (0.5 * dx);
    return STZG_OK;
}

int stzg_compute_strain(stzg_sim *s, double *out) {
    if (!s || !out) return fail(STZG_EINVAL, "null argument");
    const size_t mn = (size_t)s->m * s->n;
    double *dev = nullptr;
    STZG_CUDA(cudaMallocAsync((void **)&dev, mn * sizeof(double), s->st));
    double *const *f = s->F.f[s->cur];
    const double dx = (s->P.bx - s->P.ax) / s->m, dy = (s->P.by - s->P.ay) / s->n;
    dim3 blk(32, 8), grd(ceil_div(s->m, 32), ceil_div(s->n, 8));
    k_strain<<<grd, blk, 0, s->st>>>(f[F_X], f[F_Y], s->m, s->n, s->P.bx - s->P.ax, 1 / dx, 1 / dy, dev);
    note_launch();
    cudaError_t e = cudaMemcpyAsync(out, dev, mn * sizeof(double), cudaMemcpyDeviceToHost, s->st);
    cudaFreeAsync(dev, s->st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(strain)");
    STZG_CUDA(cudaStreamSynchronize(s->st));
    return STZG_OK;
}

int stzg_write_frame(stzg_sim *s, const char *dir, int frame, unsigned flags, double *qs) {
    if (!s || !dir) return fail(STZG_EINVAL, "null argument");
    if (flags & 2048) {
        double Q, mx;
        STZG_CHECK(stzg_qs_measure(s, 0, &Q, &mx));
        if (qs) {
            qs[0] = Q;
            qs[1] = mx;
        }
    }
    std::vector<float> buf;
    for (int mode = 0; mode < 12; mode++) {
        if (!(flags & (1u << mode))) continue;
        long count = 0;
        STZG_CHECK(stzg_output_field(s, mode, nullptr, &count));
        buf.resize(count);
        STZG_CHECK(stzg_output_field(s, mode, buf.data(), &count));
        const std::string path = std::string(dir) + "/" + mode_prefix(mode) + "." + std::to_string(frame);
        FILE *fp = std::fopen(path.c_str(), "wb");
        if (!fp) return fail(STZG_EINVAL, "cannot open " + path);
        const size_t wrote = std::fwrite(buf.data(), sizeof(float), (size_t)count, fp);
        std::fclose(fp);
        if (wrote != (size_t)count) return fail(STZG_EINVAL, "short write to " + path);
    }
    return STZG_OK;
}

}  // extern "C"
