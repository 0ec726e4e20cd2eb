// Multigrid kernels and hierarchy set-up (see mg.cuh for the design).
#include "mg.cuh"
#include "mg_device.cuh"
#include "ff.cuh"
#include "transfer1d.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>

namespace stzg {

// ---------------------------------------------------------------------------
// qs_multi constants (qs_multi.cc:9-15 and qs_multi::init, qs_multi.cc:31-55)

void qs_constants::init(const stz_params &p, double viscdt) {
    const double dx = (p.bx - p.ax) / p.m, dy = (p.by - p.ay) / p.n;
    const double xsp = 1. / dx, ysp = 1. / dy;
    mu = p.mu;
    Kq = p.K + p.mu / 3.0;
    qK = .25 * Kq * xsp * ysp;
    Kmu = Kq + p.mu;
    xsp2 = xsp * xsp;
    ysp2 = ysp * ysp;
    xyfac = xsp2 + ysp2;
    tmufac1 = Kmu * xsp2 + p.mu * ysp2;
    tmufac2 = p.mu * xsp2 + Kmu * ysp2;
    bcs = 4;
    Kmx = (Kmu + viscdt) * xsp2;
    Kmy = (Kmu + viscdt) * ysp2;
    mx = (p.mu + viscdt) * xsp2;
    my = (p.mu + viscdt) * ysp2;
    cxx = -2 * (tmufac1 + viscdt * xyfac);
    cyy = -2 * (tmufac2 + viscdt * xyfac);
}

double qs_constants::reference_acc(double mult) const {
    double a = DBL_EPSILON * mult * (2 * (tmufac1 + tmufac2));
    return a * a;
}

template <typename T> top_op<T> qs_constants::op() const {
    top_op<T> o;
    o.Kmx = (T)Kmx; o.Kmy = (T)Kmy; o.mx = (T)mx; o.my = (T)my; o.qK = (T)qK;
    o.cxx = (T)cxx; o.cyy = (T)cyy;
    o.icxx = (T)(1 / cxx); o.icyy = (T)(1 / cyy);
    o.bcxx = (T)(bcs * cxx); o.bcyy = (T)(bcs * cyy);
    o.ibcxx = (T)(1 / (bcs * cxx)); o.ibcyy = (T)(1 / (bcs * cyy));
    return o;
}
template top_op<double> qs_constants::op<double>() const;
template top_op<float> qs_constants::op<float>() const;

// ---------------------------------------------------------------------------
// Hierarchy sizes: child of (m,n) is ((m+1)>>1, (n+2)>>1) for x periodic and
// y bounded (tgmg.hh:108-110); stop once m*n <= 10 (tgmg_config.hh:23).  A
// periodic line shorter than 3 would alias its own neighbours, so
// coarsening also stops there (the reference collapses such levels,
// tgmg.in.cc:738-746).

std::vector<std::pair<int, int>> coarse_sizes(int m, int n) {
    std::vector<std::pair<int, int>> out;
    int am = (m + 1) >> 1, an = (n + 2) >> 1;
    while (am * an > 10 && am >= 3 && (int)out.size() < 16) {
        out.push_back(std::make_pair(am, an));
        int nm = (am + 1) >> 1, nn = (an + 2) >> 1;
        am = nm;
        an = nn;
    }
    return out;
}

// ---------------------------------------------------------------------------
// Galerkin coarse operators (tgmg_base::rat and the generated compute_rat,
// tgmg.in.cc:667-736, tgmg_compile.pl:151-338), formed as sum_k sum_l
// P(k,I) A(k,l) P(l,J) per coarse point I and neighbour J.

namespace {

typedef mat2<double> M2;

inline M2 mz() { M2 r = {0, 0, 0, 0}; return r; }
inline M2 mk(double a, double b, double c, double d) { M2 r = {a, b, c, d}; return r; }
inline bool is_zero(const M2 &A) { return A.a == 0 && A.b == 0 && A.c == 0 && A.d == 0; }
inline M2 inverse(const M2 &f) {  // 1/M as the reference's operator/(double,mat)
    double idet = 1. / (f.a * f.d - f.b * f.c);
    return mk(f.d * idet, -f.b * idet, -f.c * idet, f.a * idet);
}

// Fine operator of a level, entry k (dl dc dr cl cc cr ul uc ur) at (i,j).
struct fine_access {
    const qs_constants *q = nullptr;  // top level when set
    const level_ops *L = nullptr;
    int m, n;
    M2 entry(int i, int j, int k) const {
        if (q) {
            bool wall = j == 0 || j == n - 1;
            if (wall) return k == 4 ? mk(q->bcs * q->cxx, 0, 0, q->bcs * q->cyy) : mz();
            switch (k) {
                case 0: case 8: return mk(0, q->qK, q->qK, 0);
                case 2: case 6: return mk(0, -q->qK, -q->qK, 0);
                // The operator applied by qs_multi::mul_a (qs_multi.hh:41-50):
                // horizontal neighbours (Kmx, mx), vertical (my, Kmy).  The
                // reference's a_cl/a_dc (qs_multi.hh:26-29) swap mx and my in
                // the second component, which only agrees for dx == dy.
                case 3: case 5: return mk(q->Kmx, 0, 0, q->mx);
                case 1: case 7: return mk(q->my, 0, 0, q->Kmy);
                default: return mk(q->cxx, 0, 0, q->cyy);
            }
        }
        int c = L->homog ? L->cls[j] : L->cls[(size_t)j * m + i];
        return L->table[c].e[k];
    }
};

void rap_point(const fine_access &A, int cm, int cn, int I, int J, stencil9<double> &out) {
    const int fm = A.m, fn = A.n;
    M2 acc[9];
    for (int k = 0; k < 9; k++) acc[k] = mz();
    for (int fy = 2 * J - 1; fy <= 2 * J + 1; fy++) {
        if (fy < 0 || fy >= fn) continue;
        double wyk = pw(fy, fn, 0, J);
        if (wyk == 0) continue;
        for (int d = -1; d <= 1; d++) {
            int fx = ((2 * I + d) % fm + fm) % fm;
            double wxk = pw(fx, fm, 1, I);
            if (wxk == 0) continue;
            double rk = wxk * wyk;
            for (int sy = -1; sy <= 1; sy++) {
                int ly = fy + sy;
                if (ly < 0 || ly >= fn) continue;
                for (int sx = -1; sx <= 1; sx++) {
                    int lx = ((fx + sx) % fm + fm) % fm;
                    M2 a = A.entry(fx, fy, (sy + 1) * 3 + sx + 1);
                    if (is_zero(a)) continue;
                    int cy[2], cx[2], ny, nx;
                    double wy[2], wx[2];
                    ny = p1d(ly, fn, 0, cy, wy);
                    nx = p1d(lx, fm, 1, cx, wx);
                    for (int b = 0; b < ny; b++)
                        for (int c = 0; c < nx; c++) {
                            int oy = cy[b] - J, ox = cx[c] - I;
                            if (ox > cm / 2) ox -= cm;
                            if (ox < -(cm / 2)) ox += cm;
                            int k = (oy + 1) * 3 + ox + 1;
                            double w = rk * wx[c] * wy[b];
                            acc[k].a += w * a.a; acc[k].b += w * a.b;
                            acc[k].c += w * a.c; acc[k].d += w * a.d;
                        }
                }
            }
        }
    }
    for (int k = 0; k < 9; k++) out.e[k] = acc[k];
    out.e[9] = inverse(acc[4]);
}

bool same(const stencil9<double> &a, const stencil9<double> &b) {
    return std::memcmp(&a, &b, sizeof(a)) == 0;
}

int class_of(std::vector<stencil9<double>> &table, const stencil9<double> &s) {
    for (size_t k = 0; k < table.size(); k++)
        if (same(table[k], s)) return (int)k;
    table.push_back(s);
    return (int)table.size() - 1;
}

}  // namespace

std::vector<level_ops> build_coarse_ops(const qs_constants &q, int m, int n) {
    std::vector<level_ops> out;
    std::vector<std::pair<int, int>> sizes = coarse_sizes(m, n);
    fine_access A;
    A.q = &q;
    A.m = m;
    A.n = n;
    bool fine_homog = true;
    for (size_t l = 0; l < sizes.size(); l++) {
        level_ops L;
        L.m = sizes[l].first;
        L.n = sizes[l].second;
        // Uniform coarsening of a homogeneous periodic line keeps the
        // operator x-homogeneous: one column per row suffices.
        L.homog = fine_homog && (A.m % 2 == 0);
        if (L.homog) {
            L.cls.resize(L.n);
            for (int J = 0; J < L.n; J++) {
                stencil9<double> s;
                rap_point(A, L.m, L.n, 0, J, s);
                L.cls[J] = class_of(L.table, s);
            }
        } else {
            L.cls.resize((size_t)L.m * L.n);
            for (int J = 0; J < L.n; J++)
                for (int I = 0; I < L.m; I++) {
                    stencil9<double> s;
                    rap_point(A, L.m, L.n, I, J, s);
                    L.cls[(size_t)J * L.m + I] = class_of(L.table, s);
                }
        }
        out.push_back(L);
        fine_homog = L.homog;
        A.q = nullptr;
        A.L = &out.back();
        A.m = L.m;
        A.n = L.n;
        // out may reallocate on the next push_back: re-point after it.
        A.L = nullptr;
        A.L = &out[l];
    }
    return out;
}

// Dense inverse of the coarsest operator by Gauss-Jordan elimination with
// partial pivoting.  The reference smooths the coarsest level with 10+10
// Gauss-Seidel sweeps (tgmg.in.cc:350-352); an exact solve is at least as
// accurate and replaces ~80 dependent colour phases by one product.
std::vector<double> coarsest_inverse(const level_ops &L) {
    const int m = L.m, n = L.n, N = 2 * m * n;
    std::vector<double> inv;
    if (N > 1024) return inv;
    std::vector<double> A((size_t)N * N, 0.0);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            const int c = L.homog ? L.cls[j] : L.cls[(size_t)j * m + i];
            const stencil9<double> &s = L.table[c];
            const int row = 2 * (j * m + i);
            for (int dy = -1; dy <= 1; dy++) {
                int y = j + dy;
                if (y < 0 || y >= n) continue;
                for (int dx = -1; dx <= 1; dx++) {
                    int x = ((i + dx) % m + m) % m;
                    const mat2<double> &b = s.e[(dy + 1) * 3 + dx + 1];
                    const int col = 2 * (y * m + x);
                    A[(size_t)row * N + col] += b.a;
                    A[(size_t)row * N + col + 1] += b.b;
                    A[(size_t)(row + 1) * N + col] += b.c;
                    A[(size_t)(row + 1) * N + col + 1] += b.d;
                }
            }
        }
    inv.assign((size_t)N * N, 0.0);
    for (int k = 0; k < N; k++) inv[(size_t)k * N + k] = 1;
    for (int c = 0; c < N; c++) {
        int piv = c;
        for (int r = c + 1; r < N; r++)
            if (std::fabs(A[(size_t)r * N + c]) > std::fabs(A[(size_t)piv * N + c])) piv = r;
        if (A[(size_t)piv * N + c] == 0) return std::vector<double>();
        if (piv != c)
            for (int k = 0; k < N; k++) {
                std::swap(A[(size_t)piv * N + k], A[(size_t)c * N + k]);
                std::swap(inv[(size_t)piv * N + k], inv[(size_t)c * N + k]);
            }
        const double d = 1.0 / A[(size_t)c * N + c];
        for (int k = 0; k < N; k++) {
            A[(size_t)c * N + k] *= d;
            inv[(size_t)c * N + k] *= d;
        }
        for (int r = 0; r < N; r++) {
            if (r == c) continue;
            const double f = A[(size_t)r * N + c];
            if (f == 0) continue;
            for (int k = 0; k < N; k++) {
                A[(size_t)r * N + k] -= f * A[(size_t)c * N + k];
                inv[(size_t)r * N + k] -= f * inv[(size_t)c * N + k];
            }
        }
    }
    return inv;
}

// ---------------------------------------------------------------------------
// Device hierarchy

template <typename T> int hierarchy<T>::allocate(int m, int n, V *top_z, V *top_b) {
    release();
    std::vector<std::pair<int, int>> sz = coarse_sizes(m, n);
    nl = 1 + (int)sz.size();
    for (int l = 0; l < nl; l++) {
        level_view<T> &L = lv[l];
        std::memset(&L, 0, sizeof(L));
        L.m = l == 0 ? m : sz[l - 1].first;
        L.n = l == 0 ? n : sz[l - 1].second;
        L.colors_x = (L.m & 1) ? 3 : 2;
        size_t cnt = (size_t)L.m * L.n;
        V *p[3] = {nullptr, nullptr, nullptr};
        for (int k = 0; k < 3; k++) {
            if (l == 0 && k == 0 && top_z) { p[k] = top_z; continue; }
            if (l == 0 && k == 1 && top_b) { p[k] = top_b; continue; }
            cudaError_t e = cudaMalloc((void **)&p[k], cnt * sizeof(V));
            if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(level)");
            cudaMemset(p[k], 0, cnt * sizeof(V));
            owned_.push_back(p[k]);
            bytes_ += cnt * sizeof(V);
        }
        L.z = p[0];
        L.b = p[1];
        L.r = p[2];
    }
    return STZG_OK;
}

template <typename T> cudaError_t prepare_tail_kernel();

template <typename T> int hierarchy<T>::upload_ops(const std::vector<level_ops> &ops, const top_op<double> &o) {
    op.Kmx = (T)o.Kmx; op.Kmy = (T)o.Kmy; op.mx = (T)o.mx; op.my = (T)o.my; op.qK = (T)o.qK;
    op.cxx = (T)o.cxx; op.cyy = (T)o.cyy; op.icxx = (T)o.icxx; op.icyy = (T)o.icyy;
    op.bcxx = (T)o.bcxx; op.bcyy = (T)o.bcyy; op.ibcxx = (T)o.ibcxx; op.ibcyy = (T)o.ibcyy;
    if ((int)ops.size() != nl - 1) return fail(STZG_EINVAL, "hierarchy/operator level mismatch");
    for (int l = 1; l < nl; l++) {
        const level_ops &L = ops[l - 1];
        level_view<T> &D = lv[l];
        D.homog = L.homog ? 1 : 0;
        std::vector<stencil9<T>> tab(L.table.size());
        for (size_t k = 0; k < L.table.size(); k++)
            for (int e = 0; e < 10; e++) {
                tab[k].e[e].a = (T)L.table[k].e[e].a; tab[k].e[e].b = (T)L.table[k].e[e].b;
                tab[k].e[e].c = (T)L.table[k].e[e].c; tab[k].e[e].d = (T)L.table[k].e[e].d;
            }
        STZG_CHECK(grow(l, tab.size(), L.cls.size()));
        D.nst = (int)tab.size();
        D.ncls = (int)L.cls.size();
        STZG_CUDA(cudaMemcpy((void *)D.st, tab.data(), sizeof(stencil9<T>) * tab.size(), cudaMemcpyHostToDevice));
        STZG_CUDA(cudaMemcpy((void *)D.cls, L.cls.data(), sizeof(int) * L.cls.size(), cudaMemcpyHostToDevice));
    }
    STZG_CUDA(prepare_tail_kernel<T>());
    bottom_inv = nullptr;
    bottom_unknowns = 0;
    if (nl > 1) {
        std::vector<double> inv = coarsest_inverse(ops.back());
        if (!inv.empty()) {
            if (inv.size() > inv_cap_) {
                void *p;
                cudaError_t e = cudaMalloc(&p, sizeof(double) * inv.size());
                if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(coarsest inverse)");
                owned_.push_back(p);
                bytes_ += sizeof(double) * inv.size();
                inv_dev_ = (double *)p;
                inv_cap_ = inv.size();
            }
            STZG_CUDA(cudaMemcpy(inv_dev_, inv.data(), sizeof(double) * inv.size(), cudaMemcpyHostToDevice));
            bottom_inv = inv_dev_;
            bottom_unknowns = 2 * ops.back().m * ops.back().n;
        }
    }
    return STZG_OK;
}

template <typename T> int hierarchy<T>::grow(int l, size_t st_need, size_t cls_need) {
    level_view<T> &D = lv[l];
    if (st_need > st_cap_[l]) {
        void *p;
        cudaError_t e = cudaMalloc(&p, sizeof(stencil9<T>) * st_need);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(stencils)");
        owned_.push_back(p);
        bytes_ += sizeof(stencil9<T>) * st_need;
        D.st = (const stencil9<T> *)p;
        st_cap_[l] = st_need;
    }
    if (cls_need > cls_cap_[l]) {
        void *p;
        cudaError_t e = cudaMalloc(&p, sizeof(int) * cls_need);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(classes)");
        owned_.push_back(p);
        bytes_ += sizeof(int) * cls_need;
        D.cls = (const int *)p;
        cls_cap_[l] = cls_need;
    }
    return STZG_OK;
}

template <typename T> void hierarchy<T>::release() {
    for (int l = 0; l < 17; l++) st_cap_[l] = cls_cap_[l] = 0;
    inv_cap_ = 0;
    inv_dev_ = nullptr;
    bottom_inv = nullptr;
    for (void *p : owned_) cudaFree(p);
    owned_.clear();
    bytes_ = 0;
    nl = 0;
}

template class hierarchy<double>;
template class hierarchy<float>;

// ---------------------------------------------------------------------------
// Kernels

namespace {

template <typename V, typename T> __device__ inline void madd(V &acc, const mat2<T> &A, const V &z) {
    acc.x += A.a * z.x + A.b * z.y;
    acc.y += A.c * z.x + A.d * z.y;
}

// One colour of the top-level Gauss-Seidel sweep.  Colour c updates the x
// component where (i+j)&1 == c and the y component elsewhere.  A thread takes
// the node pair (2p, 2p+1) of a row and performs the x update on one and the y
// update on the other, so lanes never diverge on the component.
template <typename T>
__global__ void k_top_color(top_op<T> op, typename vec2_t<T>::type *__restrict__ z,
                            const typename vec2_t<T>::type *__restrict__ b, int m, int n, int color) {
    typedef typename vec2_t<T>::type V;
    const int pr = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (2 * pr >= m || j >= n) return;
    const int ia = 2 * pr;
    const bool a_is_x = ((ia + j) & 1) == color;
    const int ix = a_is_x ? ia : ia + 1, iy = a_is_x ? ia + 1 : ia;
    const size_t row = (size_t)j * m;
    if (j == 0 || j == n - 1) {  // Dirichlet wall rows: z = regcbi*b
        z[row + ix].x = op.ibcxx * b[row + ix].x;
        z[row + iy].y = op.ibcyy * b[row + iy].y;
        return;
    }
    const V *zd = z + row - m, *zc = z + row, *zu = z + row + m;
    {
        const int il = ix == 0 ? m - 1 : ix - 1, ir = ix == m - 1 ? 0 : ix + 1;
        T a = op.Kmx * (zc[il].x + zc[ir].x) + op.my * (zd[ix].x + zu[ix].x) +
              op.qK * (zd[il].y + zu[ir].y - zd[ir].y - zu[il].y);
        z[row + ix].x = op.icxx * (b[row + ix].x - a);
    }
    {
        const int il = iy == 0 ? m - 1 : iy - 1, ir = iy == m - 1 ? 0 : iy + 1;
        T a = op.mx * (zc[il].y + zc[ir].y) + op.Kmy * (zd[iy].y + zu[iy].y) +
              op.qK * (zd[il].x + zu[ir].x - zd[ir].x - zu[il].x);
        z[row + iy].y = op.icyy * (b[row + iy].y - a);
    }
}

template <typename T>
__global__ void k_top_residual(top_op<T> op, const typename vec2_t<T>::type *__restrict__ z,
                               const typename vec2_t<T>::type *__restrict__ b,
                               typename vec2_t<T>::type *__restrict__ r, int m, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= m || j >= n) return;
    r[(size_t)j * m + i] = top_res<T>(op, z, b, m, n, i, j);
}

template <typename T>
__device__ inline const stencil9<T> &stencil_at(const level_view<T> &L, int i, int j) {
    int c = L.homog ? L.cls[j] : L.cls[(size_t)j * L.m + i];
    return L.st[c];
}

// Off-diagonal product of a coarse level (tgmg_level::mul_a, tgmg.in.cc:536-547)
template <typename T, typename V>
__device__ inline V lev_offdiag(const level_view<T> &L, const stencil9<T> &s, const V *__restrict__ z, int i, int j) {
    const int m = L.m, n = L.n;
    const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
    V acc;
    acc.x = 0;
    acc.y = 0;
    if (j > 0) {
        const V *zd = z + (size_t)(j - 1) * m;
        madd(acc, s.e[0], zd[il]); madd(acc, s.e[1], zd[i]); madd(acc, s.e[2], zd[ir]);
    }
    const V *zc = z + (size_t)j * m;
    madd(acc, s.e[3], zc[il]); madd(acc, s.e[5], zc[ir]);
    if (j < n - 1) {
        const V *zu = z + (size_t)(j + 1) * m;
        madd(acc, s.e[6], zu[il]); madd(acc, s.e[7], zu[i]); madd(acc, s.e[8], zu[ir]);
    }
    return acc;
}

template <typename T>
__device__ inline int color_of(const level_view<T> &L, int i, int j) {
    int cx = (L.colors_x == 3 && i == L.m - 1) ? 2 : (i & 1);
    return (j & 1) * L.colors_x + cx;
}

// One colour (cx, cy) of a coarse-level sweep; thread (ti, tj) owns point
// (2 ti + cx, 2 tj + cy), or the last column for the third colour of an odd
// periodic line.
template <typename T> __global__ void k_lev_color(level_view<T> L, int cx, int cy) {
    typedef typename vec2_t<T>::type V;
    const int ti = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 2 * (blockIdx.y * blockDim.y + threadIdx.y) + cy;
    if (j >= L.n) return;
    int i;
    if (cx == 2) {
        if (ti > 0) return;
        i = L.m - 1;
    } else {
        i = 2 * ti + cx;
        if (i >= L.m || (L.colors_x == 3 && i == L.m - 1)) return;
    }
    const stencil9<T> &s = stencil_at(L, i, j);
    const size_t ij = (size_t)j * L.m + i;
    V a = lev_offdiag<T, V>(L, s, L.z, i, j);
    V r, out;
    r.x = L.b[ij].x - a.x;
    r.y = L.b[ij].y - a.y;
    out.x = s.e[9].a * r.x + s.e[9].b * r.y;
    out.y = s.e[9].c * r.x + s.e[9].d * r.y;
    L.z[ij] = out;
}

template <typename T> __global__ void k_lev_residual(level_view<T> L) {
    typedef typename vec2_t<T>::type V;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= L.m || j >= L.n) return;
    const stencil9<T> &s = stencil_at(L, i, j);
    const size_t ij = (size_t)j * L.m + i;
    V a = lev_offdiag<T, V>(L, s, L.z, i, j);
    madd(a, s.e[4], L.z[ij]);
    V r;
    r.x = L.b[ij].x - a.x;
    r.y = L.b[ij].y - a.y;
    L.r[ij] = r;
}

// Full-weighting restriction b_c = P^T r_f (apply_r, tgmg.in.cc:626-647):
// every coarse point gathers its fine support (within +-1 of 2I, 2J).
template <typename T>
__global__ void k_restrict(const typename vec2_t<T>::type *__restrict__ r, int fm, int fn,
                           typename vec2_t<T>::type *__restrict__ bc, int cm, int cn) {
    typedef typename vec2_t<T>::type V;
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    if (I >= cm || J >= cn) return;
    T ax = 0, ay = 0;
    for (int dy = -1; dy <= 1; dy++) {
        int fy = 2 * J + dy;
        if (fy < 0 || fy >= fn) continue;
        int hy = halves_of(fy, fn, 0, J);
        if (hy == 0) continue;
        for (int dx = -1; dx <= 1; dx++) {
            int fx = 2 * I + dx;
            fx = fx < 0 ? fx + fm : (fx >= fm ? fx - fm : fx);
            int hx = halves_of(fx, fm, 1, I);
            if (hx == 0) continue;
            const T w = (T)(hx * hy) * (T)0.25;
            V v = r[(size_t)fy * fm + fx];
            ax += w * v.x;
            ay += w * v.y;
        }
    }
    V o;
    o.x = ax;
    o.y = ay;
    bc[(size_t)J * cm + I] = o;
}

// Bilinear prolongation added to the fine z (apply_t, tgmg.in.cc:552-621).
template <typename T>
__global__ void k_prolong_add(const typename vec2_t<T>::type *__restrict__ zc, int cm, int cn,
                              typename vec2_t<T>::type *__restrict__ zf, int fm, int fn) {
    typedef typename vec2_t<T>::type V;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= fm || j >= fn) return;
    int cy[2], cx[2], hy[2], hx[2];
    int ny = p1d_halves(j, fn, 0, cy, hy), nx = p1d_halves(i, fm, 1, cx, hx);
    T ax = 0, ay = 0;
    for (int b = 0; b < ny; b++)
        for (int a = 0; a < nx; a++) {
            const T w = (T)(hx[a] * hy[b]) * (T)0.25;
            V v = zc[(size_t)cy[b] * cm + cx[a]];
            ax += w * v.x;
            ay += w * v.y;
        }
    V &f = zf[(size_t)j * fm + i];
    f.x += ax;
    f.y += ay;
}

// Bottom level: `down` sweeps from zero then `up` sweeps (v_cycle_internal,
// tgmg.in.cc:350-352), one block, arithmetic in TC.
template <typename T, typename TC> __global__ void k_bottom(level_view<T> L, int down, int up) {
    typedef typename vec2_t<T>::type V;
    const int mn = L.m * L.n;
    const int ncol = 2 * L.colors_x;
    for (int k = threadIdx.x; k < mn; k += blockDim.x) {
        L.z[k].x = 0;
        L.z[k].y = 0;
    }
    __syncthreads();
    for (int sweep = 0; sweep < down + up; sweep++) {
        for (int c = 0; c < ncol; c++) {
            for (int k = threadIdx.x; k < mn; k += blockDim.x) {
                int i = k % L.m, j = k / L.m;
                if (color_of(L, i, j) != c) continue;
                const stencil9<T> &s = stencil_at(L, i, j);
                const int il = i == 0 ? L.m - 1 : i - 1, ir = i == L.m - 1 ? 0 : i + 1;
                TC ax = 0, ay = 0;
                const int nb[9][2] = {{il, j - 1}, {i, j - 1}, {ir, j - 1}, {il, j}, {i, j}, {ir, j},
                                      {il, j + 1}, {i, j + 1}, {ir, j + 1}};
                for (int e = 0; e < 9; e++) {
                    if (e == 4) continue;
                    int y = nb[e][1];
                    if (y < 0 || y >= L.n) continue;
                    V zz = L.z[(size_t)y * L.m + nb[e][0]];
                    ax += (TC)s.e[e].a * (TC)zz.x + (TC)s.e[e].b * (TC)zz.y;
                    ay += (TC)s.e[e].c * (TC)zz.x + (TC)s.e[e].d * (TC)zz.y;
                }
                TC rx = (TC)L.b[k].x - ax, ry = (TC)L.b[k].y - ay;
                V o;
                o.x = (T)((TC)s.e[9].a * rx + (TC)s.e[9].b * ry);
                o.y = (T)((TC)s.e[9].c * rx + (TC)s.e[9].d * ry);
                L.z[k] = o;
            }
            __syncthreads();
        }
    }
}

// Exact coarsest solve z = A^-1 b (FP64 arithmetic, any storage precision).
template <typename T> __global__ void k_bottom_direct(level_view<T> L, const double *__restrict__ inv, int N) {
    typedef typename vec2_t<T>::type V;
    extern __shared__ double bsh[];
    for (int k = threadIdx.x; k < N / 2; k += blockDim.x) {
        V b = L.b[k];
        bsh[2 * k] = (double)b.x;
        bsh[2 * k + 1] = (double)b.y;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < N; r += blockDim.x) {
        const double *row = inv + (size_t)r * N;
        double a = 0;
        for (int k = 0; k < N; k++) a += row[k] * bsh[k];
        T *zz = (T *)L.z;
        zz[r] = (T)a;
    }
}

constexpr int kRedThreads = 256;

template <typename T>
__global__ void k_top_sqnorm(top_op<T> op, const typename vec2_t<T>::type *__restrict__ z,
                             const typename vec2_t<T>::type *__restrict__ b, int m, int n, double *partials) {
    typedef typename vec2_t<T>::type V;
    __shared__ double sh[32];
    // 32-bit indices (grids are limited to 2^30 points): the division by m
    // is a short unsigned sequence instead of a 64-bit division routine
    const unsigned total = (unsigned)m * (unsigned)n;
    double sr = 0, sb = 0;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        const int j = (int)(k / (unsigned)m), i = (int)k - j * m;
        V r = top_res<T>(op, z, b, m, n, i, j);
        sr += (double)r.x * r.x + (double)r.y * r.y;
        V bb = b[k];
        sb += (double)bb.x * bb.x + (double)bb.y * bb.y;
    }
    double a = block_sum(sr, sh);
    double c = block_sum(sb, sh);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = c;
    }
}

// Sums the per-block partials with one block in a fixed order.
__global__ void k_final_sum(const double *partials, int npart, double *out, double *out_b) {
    __shared__ double sh[32];
    double a = 0, c = 0;
    for (int k = threadIdx.x; k < npart; k += blockDim.x) {
        a += partials[2 * k];
        c += partials[2 * k + 1];
    }
    a = block_sum(a, sh);
    c = block_sum(c, sh);
    if (threadIdx.x == 0) {
        *out = a;
        if (out_b) *out_b = c;
    }
}

__global__ void k_mixed_residual(top_op<double> op, const double2 *__restrict__ z, const double2 *__restrict__ b,
                                 int m, int n, float2 *__restrict__ r32, double *partials) {
    __shared__ double sh[32];
    const unsigned total = (unsigned)m * (unsigned)n;
    double sr = 0, sb = 0;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        const int j = (int)(k / (unsigned)m), i = (int)k - j * m;
        double2 r = top_res<double>(op, z, b, m, n, i, j);
        r32[k] = make_float2((float)r.x, (float)r.y);
        sr += r.x * r.x + r.y * r.y;
        double2 bb = b[k];
        sb += bb.x * bb.x + bb.y * bb.y;
    }
    double a = block_sum(sr, sh);
    double c = block_sum(sb, sh);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = c;
    }
}

__global__ void k_mixed_correct(double2 *__restrict__ z, const float2 *__restrict__ e, long count) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
        float2 d = e[k];
        double2 v = z[k];
        v.x += (double)d.x;
        v.y += (double)d.y;
        z[k] = v;
    }
}

// Quadratic extrapolation through the last three solutions:
// z <- 3 z - 3 prev + prev2, prev2 <- prev, prev <- old z.
__global__ void k_extrapolate2(double2 *__restrict__ z, double2 *__restrict__ prev, double2 *__restrict__ prev2,
                               long count) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
        const double2 a = z[k], p = prev[k], q = prev2[k];
        prev2[k] = p;
        prev[k] = a;
        z[k] = make_double2(3 * (a.x - p.x) + q.x, 3 * (a.y - p.y) + q.y);
    }
}

__global__ void k_extrapolate(double2 *__restrict__ z, double2 *__restrict__ prev, long count) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
        double2 a = z[k], p = prev[k];
        prev[k] = a;
        z[k] = make_double2(2 * a.x - p.x, 2 * a.y - p.y);
    }
}

// ---------------------------------------------------------------------------
// Float-float iterates of the mixed-precision solve.  GB300 issues FP64 at
// 1/57 of the FP32 rate, so the outer residual b - A z, computed in FP64,
// was ALU-bound.  Here z and b are kept as unevaluated sums hi + lo of two
// floats (~48 significant bits) and the residual is evaluated with
// error-free transformations in FP32: Knuth's TwoSum, Dekker's
// Fast2Sum and the FMA product error (a*b - p exactly = fmaf(a, b, -p)).
// The additions are the "sloppy" double-float sum, whose error is bounded
// by ~2^-44 (|x| + |y|): the residual's error is then ~1e-13 |b|, three
// orders below the 1e-10 stopping tolerance, while the FP32 value handed to
// the V-cycles needs only single precision.

// The linear extrapolation of the guess (k_extrapolate's arithmetic) fused
// with the split: prev takes the last solution, the guess 2 v - prev goes
// straight into pairs (hi, lo) without an FP64 store (the solve ends by
// merging its result into v), and the source b into its pairs.
__global__ void k_extrap_split(const double2 *__restrict__ v, double2 *__restrict__ prev,
                               const double2 *__restrict__ b, float2 *__restrict__ hi, float2 *__restrict__ lo,
                               float2 *__restrict__ bhi, float2 *__restrict__ blo, long count) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
        const double2 a = v[k], p = prev[k], w = b[k];
        prev[k] = a;
        const double gx = 2 * a.x - p.x, gy = 2 * a.y - p.y;
        float2 h, l;
        ff_split_d(gx, h.x, l.x);
        ff_split_d(gy, h.y, l.y);
        hi[k] = h;
        lo[k] = l;
        ff_split_d(w.x, h.x, l.x);
        ff_split_d(w.y, h.y, l.y);
        bhi[k] = h;
        blo[k] = l;
    }
}

__global__ void k_ff_split(const double2 *__restrict__ a, float2 *__restrict__ hi, float2 *__restrict__ lo,
                           const double2 *__restrict__ a2, float2 *__restrict__ hi2, float2 *__restrict__ lo2,
                           long count) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
        float2 h, l;
        const double2 v = a[k];
        ff_split_d(v.x, h.x, l.x);
        ff_split_d(v.y, h.y, l.y);
        hi[k] = h;
        lo[k] = l;
        if (a2) {
            const double2 w = a2[k];
            ff_split_d(w.x, h.x, l.x);
            ff_split_d(w.y, h.y, l.y);
            hi2[k] = h;
            lo2[k] = l;
        }
    }
}

__global__ void k_ff_merge(const float2 *__restrict__ hi, const float2 *__restrict__ lo, double2 *__restrict__ a,
                           long count) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
        const float2 h = hi[k], l = lo[k];
        a[k] = make_double2(ff_to_d(h.x, l.x), ff_to_d(h.y, l.y));
    }
}

__global__ void k_ff_correct(float2 *__restrict__ hi, float2 *__restrict__ lo, const float2 *__restrict__ e,
                             long count) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
        const float2 h = hi[k], l = lo[k], d = e[k];
        const ff x = ff_add_f(ff{h.x, l.x}, d.x), y = ff_add_f(ff{h.y, l.y}, d.y);
        hi[k] = make_float2(x.hi, y.hi);
        lo[k] = make_float2(x.lo, y.lo);
    }
}

// The last correction and the merge in one pass: a = (hi, lo) + e as a
// double, without writing the pairs back (the solve ends here).
__global__ void k_ff_correct_merge(const float2 *__restrict__ hi, const float2 *__restrict__ lo,
                                   const float2 *__restrict__ e, double2 *__restrict__ a, long count) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (long)gridDim.x * blockDim.x) {
        const float2 h = hi[k], l = lo[k], d = e[k];
        const ff x = ff_add_f(ff{h.x, l.x}, d.x), y = ff_add_f(ff{h.y, l.y}, d.y);
        a[k] = make_double2(ff_to_d(x.hi, x.lo), ff_to_d(y.hi, y.lo));
    }
}

// Constants of the top-level operator as float-float pairs.
struct ff_op {
    ff Kmx, Kmy, mx, my, qK, bcxx, bcyy;
    ff dxx, dyy;  // cxx + 2 (Kmx + my), cyy + 2 (mx + Kmy): zero up to rounding
};

// r = b - A z (qs_multi::mul_a + a_cc) in float-float; r is stored in FP32
// as the next right-hand side; sum r^2 and sum b^2 go to the partials
// (FP32 per thread, FP64 across threads).
__global__ void k_ff_residual(ff_op op, const float2 *__restrict__ zh, const float2 *__restrict__ zl,
                              const float2 *__restrict__ bh, const float2 *__restrict__ bl, int m, int n,
                              float2 *__restrict__ r32, double *partials) {
    __shared__ double sh[32];
    const unsigned total = (unsigned)m * (unsigned)n;
    float sr = 0.f, sb = 0.f;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        const int j = (int)(k / (unsigned)m), i = (int)k - j * m;
        const float2 b0h = bh[k], b0l = bl[k];
        const ff bx{b0h.x, b0l.x}, by{b0h.y, b0l.y};
        const float2 ch = zh[k], cl = zl[k];
        const ff cx{ch.x, cl.x}, cy{ch.y, cl.y};
        ff rx, ry;
        if (j == 0 || j == n - 1) {
            rx = ff_sub(bx, ff_mul(op.bcxx, cx));
            ry = ff_sub(by, ff_mul(op.bcyy, cy));
        } else {
            const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
            const unsigned rd = k - (unsigned)m, ru = k + (unsigned)m;
            auto ld = [&](unsigned q, ff &x, ff &y) {
                const float2 h = zh[q], l = zl[q];
                x = ff{h.x, l.x};
                y = ff{h.y, l.y};
            };
            ff lx, ly, rrx, rry, dx, dy, ux, uy, dlx, dly, urx, ury, drx, dry, ulx, uly;
            ld(k - i + il, lx, ly);
            ld(k - i + ir, rrx, rry);
            ld(rd, dx, dy);
            ld(ru, ux, uy);
            ld(rd - i + il, dlx, dly);
            ld(ru - i + ir, urx, ury);
            ld(rd - i + ir, drx, dry);
            ld(ru - i + il, ulx, uly);
            // cxx = -2 (Kmx + my) and cyy = -2 (mx + Kmy) up to rounding
            // (qs_multi.cc:31-55), so A z is evaluated on differences from
            // the centre value, which are small for smooth z: the float-float
            // rounding then scales with them rather than with z itself.
            const ff axx = ff_add(
                ff_add(ff_mul(op.Kmx, ff_add(ff_sub(lx, cx), ff_sub(rrx, cx))),
                       ff_mul(op.my, ff_add(ff_sub(dx, cx), ff_sub(ux, cx)))),
                ff_add(ff_mul(op.qK, ff_add(ff_sub(dly, dry), ff_sub(ury, uly))), ff_mul(op.dxx, cx)));
            const ff ayy = ff_add(
                ff_add(ff_mul(op.mx, ff_add(ff_sub(ly, cy), ff_sub(rry, cy))),
                       ff_mul(op.Kmy, ff_add(ff_sub(dy, cy), ff_sub(uy, cy)))),
                ff_add(ff_mul(op.qK, ff_add(ff_sub(dlx, drx), ff_sub(urx, ulx))), ff_mul(op.dyy, cy)));
            rx = ff_sub(bx, axx);
            ry = ff_sub(by, ayy);
        }
        const float2 r = make_float2(rx.hi + rx.lo, ry.hi + ry.lo);
        r32[k] = r;
        sr = fmaf(r.x, r.x, fmaf(r.y, r.y, sr));
        sb = fmaf(b0h.x, b0h.x, fmaf(b0h.y, b0h.y, sb));
    }
    const double a = block_sum((double)sr, sh);
    const double c = block_sum((double)sb, sh);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = c;
    }
}

// ---------------------------------------------------------------------------
// Streaming top-level kernels (single precision).  A warp owns a strip of 64
// fine columns and marches down the rows of its tile with a register
// window: lane L holds the node pair (xs + 2L, xs + 2L + 1) of each row as a
// float4 (x and y of the even node, x and y of the odd node), neighbours in
// x come from the adjacent lanes by shuffles and neighbours in y from the
// window.  Each row step takes one new row of z and b (from a shared-memory
// ring that cp.async fills several rows ahead), sweeps colour 0 one row behind it and colour 1 two rows behind
// (down: and evaluates the residual three rows behind), so that a warp
// reads every node of its strip once and writes it once.  The outer lanes
// and rows are halo: a colour update is exact one node further in than the
// values it reads, and the owned columns and rows are those the two colours
// (and the residual) still reach exactly.  The sweep reads z_in and writes
// z_out, different arrays, so the halo a warp recomputes never sees another
// warp's results.
//
// Colour c updates the x component of nodes with (i + j) & 1 == c and the y
// component of the others (qs_multi::mul_a couples x to x on edge
// neighbours and to y on corners only, qs_multi.hh:41-50, so each colour is
// a set of independent unknowns); with xs even, the even node of a pair
// updates x in colour c exactly when (j & 1) == c.

__device__ __forceinline__ int wrapx(int x, int m) { return x < 0 ? x + m : (x >= m ? x - m : x); }

// Flattened loop over a RH x RW rectangle of a tile starting at (R0, C0).
#define TILE_FOR(RH, RW, R0, C0, ty, tx)                                                   \
    for (int k_ = threadIdx.y * blockDim.x + threadIdx.x; k_ < (RH) * (RW); k_ += blockDim.x * blockDim.y) \
        if (const int ty = (R0) + k_ / (RW), tx = (C0) + k_ % (RW); true)

constexpr int kFusedThreads = 256;     // blockDim of the coarse tile kernels
constexpr int kFusedMinWidth = 80;     // narrowest even periodic line of the tile and strip kernels
constexpr int kMarchWarps = 4;         // warps (row tiles) per block of the top-level kernels
constexpr int kDownRows = 8;  // coarse rows per warp tile (down)
constexpr int kUpRows = 8;      // coarse rows per warp tile (up)
constexpr int kMarchMinWidth = 64;     // narrowest even periodic line of the streaming kernels
constexpr int kDownCols = 28;          // coarse columns per strip (down): fine [xs + 4, xs + 60)
constexpr int kUpCols = 30;            // coarse columns per strip (up):   fine [xs + 2, xs + 62)

// Off-diagonal sums of the two equations a pair updates in one colour, in
// the association of the per-node form (x - the 4 edge terms - the 4 corner
// terms).  ex: the even node's equation is the x one (and the odd node's
// the y one); d, c, u: the rows below, at and above.
struct pair_sums {
    float a0, a1;
};

template <bool EX>
__device__ __forceinline__ pair_sums march_offdiag(const top_op<float> &op, const float4 &d, const float4 &c,
                                                   const float4 &u) {
    constexpr unsigned F = 0xffffffffu;
    pair_sums s;
    if constexpr (EX) {
        const float xl = __shfl_up_sync(F, c.z, 1);    // x(a-1, j)
        const float dl = __shfl_up_sync(F, d.w, 1);    // y(a-1, j-1)
        const float ul = __shfl_up_sync(F, u.w, 1);    // y(a-1, j+1)
        const float yr = __shfl_down_sync(F, c.y, 1);  // y(b+1, j)
        const float ur = __shfl_down_sync(F, u.x, 1);  // x(b+1, j+1)
        const float dr = __shfl_down_sync(F, d.x, 1);  // x(b+1, j-1)
        s.a0 = op.Kmx * (xl + c.z) + op.my * (d.x + u.x) + op.qK * (dl + u.w - d.w - ul);
        s.a1 = op.mx * (c.y + yr) + op.Kmy * (d.w + u.w) + op.qK * (d.x + ur - dr - u.x);
    } else {
        const float yl = __shfl_up_sync(F, c.w, 1);    // y(a-1, j)
        const float dl = __shfl_up_sync(F, d.z, 1);    // x(a-1, j-1)
        const float ul = __shfl_up_sync(F, u.z, 1);    // x(a-1, j+1)
        const float xr = __shfl_down_sync(F, c.x, 1);  // x(b+1, j)
        const float ur = __shfl_down_sync(F, u.y, 1);  // y(b+1, j+1)
        const float dr = __shfl_down_sync(F, d.y, 1);  // y(b+1, j-1)
        s.a0 = op.mx * (yl + c.w) + op.Kmy * (d.y + u.y) + op.qK * (dl + u.z - d.z - ul);
        s.a1 = op.Kmx * (c.x + xr) + op.my * (d.z + u.z) + op.qK * (d.y + ur - dr - u.y);
    }
    return s;
}

// One colour on row j of the pair (the Dirichlet wall rows take z =
// regcbi*b).  EX = ((j & 1) == colour), known at compile time in the
// unrolled marches (their rows start at an even index).
template <bool EX>
__device__ __forceinline__ void march_color(const top_op<float> &op, const float4 &d, float4 &c, const float4 &u,
                                            const float4 &bb, int j, int n) {
    if (j == 0 || j == n - 1) {
        if constexpr (EX) {
            c.x = op.ibcxx * bb.x;
            c.w = op.ibcyy * bb.w;
        } else {
            c.y = op.ibcyy * bb.y;
            c.z = op.ibcxx * bb.z;
        }
        return;
    }
    const pair_sums s = march_offdiag<EX>(op, d, c, u);
    if constexpr (EX) {
        c.x = op.icxx * (bb.x - s.a0);
        c.w = op.icyy * (bb.w - s.a1);
    } else {
        c.y = op.icyy * (bb.y - s.a0);
        c.z = op.icxx * (bb.z - s.a1);
    }
}

// Residual of the colour-0 equations of the pair on row j after the sweep
// (the colour-1 ones are zero up to rounding: their unknowns were updated
// last and none of their neighbours changed since).  .x belongs to the even
// node, .y to the odd one; the x component of the even node when j is even
// (EX = j even).
template <bool EX>
__device__ __forceinline__ float2 march_residual(const top_op<float> &op, const float4 &d, const float4 &c,
                                                 const float4 &u, const float4 &bb, int j, int n) {
    float2 r = make_float2(0.f, 0.f);
    if (j <= 0 || j >= n - 1) return r;
    const pair_sums s = march_offdiag<EX>(op, d, c, u);
    if constexpr (EX) {
        r.x = bb.x - s.a0 - op.cxx * c.x;
        r.y = bb.w - s.a1 - op.cyy * c.w;
    } else {
        r.x = bb.y - s.a0 - op.cyy * c.y;
        r.y = bb.z - s.a1 - op.cxx * c.z;
    }
    return r;
}

// Loads through the read-only path, or (CG) from L2: the persistent coarse
// kernel reads data other blocks wrote earlier in the same launch.
template <bool CG, typename V> __device__ __forceinline__ V ld_lvl(const V *p) { return CG ? __ldcg(p) : __ldg(p); }

// Row j of a strip (pairs at xs + 2 lane, wrapped); zero outside the grid.
template <bool CG = false>
__device__ __forceinline__ float4 march_load(const float2 *__restrict__ a, int j, int m, int n, int gx) {
    if (j < 0 || j >= n) return make_float4(0.f, 0.f, 0.f, 0.f);
    return ld_lvl<CG>(reinterpret_cast<const float4 *>(a + (size_t)j * m + gx));
}

// halves_of(2J + q - 1, n, 0, J) for q = 0, 1, 2 on a bounded line of n
// points (p1d_halves: even fine rows inject, odd ones average, and an even
// line injects its last point into the last coarse one).
__device__ __forceinline__ int restrict_hy(int q, int J, int n) {
    const int fy = 2 * J + q - 1;
    if (fy < 0 || fy >= n) return 0;
    if (q == 1) return 2;
    if ((n & 1) || fy != n - 1) return 1;
    return q == 0 ? 2 : 0;
}

// Full weighting (1,2,1)x(1,2,1)/4 of the residual rows 2J-1, 2J, 2J+1 (r0,
// r1, r2) at the coarse point under the lane's even node, y rows through
// halves_of for the walls.
__device__ __forceinline__ float2 march_restrict(const float2 &r0, const float2 &r1, const float2 &r2, int J, int n) {
    constexpr unsigned F = 0xffffffffu;
    const float2 rr[3] = {r0, r1, r2};
    float ax = 0, ay = 0;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const float left = __shfl_up_sync(F, rr[q].y, 1);  // odd node of the lane to the left
        const int fy = 2 * J + q - 1;
        const int hy = restrict_hy(q, J, n);
        if (!hy) continue;
        const float w1 = (float)hy * 0.25f, w2 = (float)(2 * hy) * 0.25f;
        if (!(fy & 1)) {
            // even row: x residual on the even nodes, y on the odd ones
            ax += w2 * rr[q].x;
            ay += w1 * left;
            ay += w1 * rr[q].y;
        } else {
            ax += w1 * left;
            ax += w1 * rr[q].y;
            ay += w2 * rr[q].x;
        }
    }
    return make_float2(ax, ay);
}

// Coarse z of a strip staged by one warp: columns cx0 + 0..32 (wrapped) of
// rows Jlo .. Jlo + R - 1, zero outside the level.  Lane L's pair prolongs
// from columns L (even node) and L, L + 1 (odd node).
template <int R, bool CG = false>
__device__ __forceinline__ void stage_coarse(float2 (*cz)[33], const float2 *__restrict__ zc, int cm, int cn, int cx0,
                                             int Jlo, int lane) {
    for (int k = lane; k < R * 33; k += 32) {
        const int r = k / 33, c = k - r * 33, J = Jlo + r;
        float2 v = make_float2(0.f, 0.f);
        if (J >= 0 && J < cn) v = ld_lvl<CG>(zc + (size_t)J * cm + wrapx(cx0 + c, cm));
        cz[r][c] = v;
    }
    __syncwarp();
}

// Adds the child's correction to row j of the pair (apply_t / t_line,
// tgmg.in.cc:552-621): the even node takes coarse c0, the odd node the mean
// of c0 and c1 (wrapping on the even periodic line); rows through p1d_halves.
__device__ __forceinline__ void prolong_staged(float4 &z, const float2 (*cz)[33], int Jlo, int lane, int j, int n) {
    if (j < 0 || j >= n) return;
    int cy[2], hy[2];
    const int ny = p1d_halves(j, n, 0, cy, hy);
    float ax = 0, ay = 0, bx = 0, by = 0;
    for (int q = 0; q < ny; q++) {
        const float wy = (float)hy[q] * 0.25f;
        const float2 v0 = cz[cy[q] - Jlo][lane], v1 = cz[cy[q] - Jlo][lane + 1];
        ax += 2.f * wy * v0.x;
        ay += 2.f * wy * v0.y;
        bx += wy * (v0.x + v1.x);
        by += wy * (v0.y + v1.y);
    }
    z.x += ax;
    z.y += ay;
    z.z += bx;
    z.w += by;
}

// acc += A z for a 2x2 block (a b; c d) = (A.x A.y; A.z A.w), as two fused
// multiply-adds per component.
__device__ __forceinline__ void madd4(float2 &acc, const float4 &A, float zx, float zy) {
    acc.x = fmaf(A.y, zy, fmaf(A.x, zx, acc.x));
    acc.y = fmaf(A.w, zy, fmaf(A.z, zx, acc.y));
}

// Programmatic dependent launch within the FP32 V-cycle: each streaming
// kernel lets the next one be scheduled as soon as it starts
// (griddepcontrol.launch_dependents) and waits for its predecessor's results
// (griddepcontrol.wait) only after the set-up that needs none, so launch
// latency and set-up overlap the previous level's work.  Kernels launched
// with the attribute all execute the wait before touching data another
// kernel writes.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

template <typename... K, typename... A>
void launch_pdl(void (*kern)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

// Per-warp ring of rows of z and b for the top-level kernels, filled by
// cp.async kRing - 1 rows ahead of the row being consumed: row k of a march
// sits in slot (k - kb) mod kRing.  A lane copies and later reads only its
// own 16-byte pair, so its own cp.async.wait_group is the only
// synchronisation; a slot is refilled one step after it was read.  Rows
// outside the grid arrive as zeros (source size 0).
constexpr int kRing = 6;

__device__ __forceinline__ void cp_async16(float4 *dst, const float2 *src, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(src), "r"(valid ? 16 : 0) : "memory");
}

__device__ __forceinline__ void ring_issue(float4 (*ring)[2][32], int slot, const float2 *__restrict__ z,
                                           const float2 *__restrict__ b, int j, int m, int n, int gx, int lane) {
    // z == nullptr: the iterate is zero and only b is read
    const bool v = j >= 0 && j < n;
    const size_t o = v ? (size_t)j * m + gx : 0;
    cp_async16(&ring[slot][0][lane], z ? z + o : b + o, v && z);
    cp_async16(&ring[slot][1][lane], b + o, v);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void ring_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(kRing - 2) : "memory"); }

// The row windows of the top-level marches are circular arrays of kRing
// entries indexed by (row - kb) mod kRing, the same index as the row's ring
// slot; the step loop is unrolled kRing times so that every index is a
// compile-time constant and no register moves shift the window.
struct top_march {
    top_op<float> op;
    const float2 *zin, *b;
    float2 *zout, *bc;
    int m, n, cm, cn, y0, kb, ke, gx, lane, I;
    bool own;
    float4 (*rg)[2][32];
};

// One row step of the down march: row k arrives, colour 0 on row k-1,
// colour 1 on row k-2 (stored when owned), the residual on row k-3, and the
// restriction to coarse row (k-4)/2 when k-3 is odd.
template <int U>
__device__ __forceinline__ void top_down_step(const top_march &t, int k, float4 (&Z)[kRing], float4 (&B)[kRing],
                                              float2 (&R)[kRing]) {
    constexpr int P1 = (U + 5) % 6, P2 = (U + 4) % 6, P3 = (U + 3) % 6, P4 = (U + 2) % 6, P5 = (U + 1) % 6;
    static_assert(kRing == 6, "window indices assume six slots");
    ring_wait();
    Z[U] = t.rg[U][0][t.lane];
    B[U] = t.rg[U][1][t.lane];
    const int jn = k + kRing - 1;
    ring_issue(t.rg, P1, t.zin, t.b, jn <= t.ke ? jn : -1, t.m, t.n, t.gx, t.lane);
    const int j0 = k - 1, j1 = k - 2, j2 = k - 3, n = t.n;
    // k has the parity of U (kb is even): row k-1 is odd when U is even
    constexpr bool E0 = (U & 1) == 1, E1 = (U & 1) == 1, ER = (U & 1) == 1;
    if (j0 >= t.y0 - 3 && j0 >= 0 && j0 < n) march_color<E0>(t.op, Z[P2], Z[P1], Z[U], B[P1], j0, n);
    if (j1 >= t.y0 - 2 && j1 >= 0 && j1 < n) {
        march_color<E1>(t.op, Z[P3], Z[P2], Z[P1], B[P2], j1, n);
        if (j1 >= t.y0 && j1 < t.y0 + 2 * kDownRows && t.own)
            *reinterpret_cast<float4 *>(t.zout + (size_t)j1 * t.m + t.gx) = Z[P2];
    }
    if (j2 >= t.y0 - 1) {
        R[P3] = march_residual<ER>(t.op, Z[P4], Z[P3], Z[P2], B[P3], j2, n);
        if ((j2 & 1) && j2 >= t.y0 + 1) {
            const int J = (j2 - 1) >> 1;
            const float2 w = march_restrict(R[P5], R[P4], R[P3], J, n);
            if (t.own && J < t.cn) t.bc[(size_t)J * t.cm + t.I] = w;
        }
    }
}

// Pre-smooth + residual + restriction of the top level (apply_r after one
// gauss_seidel, tgmg.in.cc:313-320): z_out = one sweep of z_in, bc = R(b - A z_out).
__global__ void __launch_bounds__(32 * kMarchWarps) k_top_down(top_op<float> op, const float2 *__restrict__ zin,
                                                               const float2 *__restrict__ b, int m, int n,
                                                               float2 *__restrict__ zout, float2 *__restrict__ bc,
                                                               int cm, int cn) {
    __shared__ __align__(16) float4 ring[kMarchWarps][kRing][2][32];
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const int J0 = (blockIdx.y * kMarchWarps + (threadIdx.x >> 5)) * kDownRows;
    if (J0 >= cn) return;
    const int I0 = blockIdx.x * kDownCols;
    top_march t;
    t.op = op;
    t.zin = zin;
    t.b = b;
    t.zout = zout;
    t.bc = bc;
    t.m = m;
    t.n = n;
    t.cm = cm;
    t.cn = cn;
    t.y0 = 2 * J0;
    t.kb = t.y0 - 4;
    t.ke = t.y0 + 2 * kDownRows + 2;
    const int xs = 2 * I0 - 4;
    t.gx = wrapx(xs + 2 * lane, m);
    t.lane = lane;
    t.I = I0 + lane - 2;
    t.own = lane >= 2 && lane < 2 + kDownCols && t.I < cm;  // columns [xs + 4, xs + 60)
    t.rg = ring[threadIdx.x >> 5];
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 Z[kRing], B[kRing];
    float2 R[kRing];
#pragma unroll
    for (int i = 0; i < kRing; i++) {
        Z[i] = zero;
        B[i] = zero;
        R[i] = make_float2(0.f, 0.f);
    }
    pdl_wait();
    for (int d = 0; d < kRing - 1; d++) ring_issue(t.rg, d, zin, b, t.kb + d, m, n, t.gx, lane);
    for (int k = t.kb; k <= t.ke; k += kRing) {
        top_down_step<0>(t, k, Z, B, R);
        if (k + 1 > t.ke) break;
        top_down_step<1>(t, k + 1, Z, B, R);
        if (k + 2 > t.ke) break;
        top_down_step<2>(t, k + 2, Z, B, R);
        if (k + 3 > t.ke) break;
        top_down_step<3>(t, k + 3, Z, B, R);
        if (k + 4 > t.ke) break;
        top_down_step<4>(t, k + 4, Z, B, R);
        if (k + 5 > t.ke) break;
        top_down_step<5>(t, k + 5, Z, B, R);
    }
}

// One row step of the up march: row k arrives with the child's correction,
// colour 0 on row k-1, colour 1 on row k-2 (stored when owned).
template <int U>
__device__ __forceinline__ void top_up_step(const top_march &t, const float2 (*czs)[33], int J0, int k,
                                            float4 (&Z)[kRing], float4 (&B)[kRing]) {
    constexpr int P1 = (U + 5) % 6, P2 = (U + 4) % 6, P3 = (U + 3) % 6;
    ring_wait();
    float4 zn = t.rg[U][0][t.lane];
    B[U] = t.rg[U][1][t.lane];
    const int jn = k + kRing - 1;
    ring_issue(t.rg, P1, t.zin, t.b, jn <= t.ke ? jn : -1, t.m, t.n, t.gx, t.lane);
    prolong_staged(zn, czs, J0 - 1, t.lane, k, t.n);
    Z[U] = zn;
    const int j0 = k - 1, j1 = k - 2, n = t.n;
    constexpr bool E0 = (U & 1) == 1, E1 = (U & 1) == 1;  // as in top_down_step
    if (j0 >= t.y0 - 1 && j0 >= 0 && j0 < n) march_color<E0>(t.op, Z[P2], Z[P1], Z[U], B[P1], j0, n);
    if (j1 >= t.y0 && j1 < n) {
        march_color<E1>(t.op, Z[P3], Z[P2], Z[P1], B[P2], j1, n);
        if (t.own) *reinterpret_cast<float4 *>(t.zout + (size_t)j1 * t.m + t.gx) = Z[P2];
    }
}

// Prolongation + post-smooth of the top level (apply_t of level 0, then
// up_gs_iterations, tgmg.in.cc:323-327): z_out = one sweep of z_in + P zc.
// Fine node i takes coarse i/2 (even) or the mean of (i-1)/2 and (i+1)/2
// (odd, wrapping on the even periodic line); rows through p1d_halves.
__global__ void __launch_bounds__(32 * kMarchWarps) k_top_up(top_op<float> op, const float2 *__restrict__ zin,
                                                             const float2 *__restrict__ b, int m, int n,
                                                             const float2 *__restrict__ zc, int cm, int cn,
                                                             float2 *__restrict__ zout) {
    __shared__ __align__(16) float4 ring[kMarchWarps][kRing][2][32];
    __shared__ float2 czs[kMarchWarps][kUpRows + 3][33];
    pdl_trigger();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int J0 = (blockIdx.y * kMarchWarps + w) * kUpRows;
    if (J0 >= cn) return;
    const int I0 = blockIdx.x * kUpCols;
    const int xs = 2 * I0 - 2;
    top_march t;
    t.op = op;
    t.zin = zin;
    t.b = b;
    t.zout = zout;
    t.bc = nullptr;
    t.m = m;
    t.n = n;
    t.cm = cm;
    t.cn = cn;
    t.y0 = 2 * J0;
    t.kb = t.y0 - 2;
    t.ke = t.y0 + 2 * kUpRows + 1;
    t.gx = wrapx(xs + 2 * lane, m);
    t.lane = lane;
    t.I = 0;
    t.own = lane >= 1 && lane < 1 + kUpCols && xs + 2 * lane < m;  // columns [xs + 2, xs + 62)
    t.rg = ring[w];
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 Z[kRing], B[kRing];
#pragma unroll
    for (int i = 0; i < kRing; i++) {
        Z[i] = zero;
        B[i] = zero;
    }
    pdl_wait();
    for (int d = 0; d < kRing - 1; d++) ring_issue(t.rg, d, zin, b, t.kb + d, m, n, t.gx, lane);
    stage_coarse<kUpRows + 3>(czs[w], zc, cm, cn, xs / 2, J0 - 1, lane);
    for (int k = t.kb; k <= t.ke; k += kRing) {
        top_up_step<0>(t, czs[w], J0, k, Z, B);
        if (k + 1 > t.ke) break;
        top_up_step<1>(t, czs[w], J0, k + 1, Z, B);
        if (k + 2 > t.ke) break;
        top_up_step<2>(t, czs[w], J0, k + 2, Z, B);
        if (k + 3 > t.ke) break;
        top_up_step<3>(t, czs[w], J0, k + 3, Z, B);
        if (k + 4 > t.ke) break;
        top_up_step<4>(t, czs[w], J0, k + 4, Z, B);
        if (k + 5 > t.ke) break;
        top_up_step<5>(t, czs[w], J0, k + 5, Z, B);
    }
}

// Full weighting of the residual held in rs at coarse point (I, J); the fine
// point 2I+dx sits at tile column cx0 + dx.  Periodic x with an even line
// always has the weights (1, 2, 1)/2.
template <typename T, typename Tile>
__device__ __forceinline__ typename vec2_t<T>::type restrict_at(Tile &rs, int I, int J, int n, int cx0, int cy0) {
    typedef typename vec2_t<T>::type V;
    T ax = 0, ay = 0;
#pragma unroll
    for (int dy = -1; dy <= 1; dy++) {
        const int fy = 2 * J + dy;
        if (fy < 0 || fy >= n) continue;
        const int hy = halves_of(fy, n, 0, J);
        if (!hy) continue;
#pragma unroll
        for (int dx = -1; dx <= 1; dx++) {
            const T wgt = (T)((dx == 0 ? 2 : 1) * hy) * (T)0.25;
            const V r = rs(cy0 + dy, cx0 + dx);
            ax += wgt * r.x;
            ay += wgt * r.y;
        }
    }
    V o;
    o.x = ax;
    o.y = ay;
    (void)I;
    return o;
}

// ---------------------------------------------------------------------------
// Fused coarse-level kernels (single precision, even periodic lines): the
// same tiling as the top level, with the four-colour block Gauss-Seidel of
// the stored Galerkin stencils.  Down: the sweep starts from z = 0
// (down_gs_iterations, tgmg.hh:273-279), so only b is read; the residual is
// restricted to the child.  Up: prolongation of the child plus one sweep.

// Coarse tiles of TX x TY points; smaller levels take smaller tiles (more
// blocks, shorter phases), see lev_tile below.

// A W x H shared-memory tile of (x, y) pairs with each row stored
// parity-major: the even tile columns first, then the odd ones.  A colour of
// the four-colour sweep takes every other column; in this layout the points
// of one colour, and their neighbours at tx - 1 and tx + 1, lie at
// consecutive addresses, so a warp's 8-byte loads need two shared-memory
// wavefronts instead of the four of the natural layout (stride 16 bytes).
template <typename V, int W, int H> struct ptile {
    static constexpr int HALF = (W + 1) / 2;
    V d[H][2 * HALF];
    __device__ __forceinline__ V &operator()(int ty, int tx) { return d[ty][(tx & 1) * HALF + (tx >> 1)]; }
};

template <typename T, typename Tile>
__device__ __forceinline__ typename vec2_t<T>::type lev_offdiag_tile(const stencil9<T> &s, Tile &zs, int ty, int tx,
                                                                     bool has_d, bool has_u) {
    typedef typename vec2_t<T>::type V;
    V a;
    a.x = a.y = 0;
    if (has_d) {
        madd(a, s.e[0], zs(ty - 1, tx - 1));
        madd(a, s.e[1], zs(ty - 1, tx));
        madd(a, s.e[2], zs(ty - 1, tx + 1));
    }
    madd(a, s.e[3], zs(ty, tx - 1));
    madd(a, s.e[5], zs(ty, tx + 1));
    if (has_u) {
        madd(a, s.e[6], zs(ty + 1, tx - 1));
        madd(a, s.e[7], zs(ty + 1, tx));
        madd(a, s.e[8], zs(ty + 1, tx + 1));
    }
    return a;
}

// Stencils of the tile's rows: on an x-homogeneous level the stencil depends
// on the row only, and the tile's H rows are copied to shared memory once;
// otherwise each point reads its own class from global memory.
template <typename T, int H>
__device__ inline void stage_row_stencils(const level_view<T> &L, stencil9<T> *rows, int y0) {
    if (!L.homog) return;
    constexpr int NE = (int)(sizeof(stencil9<T>) / sizeof(T));
    T *dst = (T *)rows;
    for (int k = threadIdx.y * blockDim.x + threadIdx.x; k < H * NE; k += blockDim.x * blockDim.y) {
        const int ty = k / NE, e = k % NE, gy = y0 + ty;
        if (gy >= 0 && gy < L.n) dst[k] = ((const T *)&L.st[L.cls[gy]])[e];
    }
}

template <typename T>
__device__ __forceinline__ const stencil9<T> &tile_stencil(const level_view<T> &L, const stencil9<T> *rows, int ty,
                                                          int gx, int gy) {
    return L.homog ? rows[ty] : stencil_at(L, gx, gy);
}

// Colour (cx, cy) on tile rows/columns [LO, H-1-LO] x [LO, W-1-LO]; the
// colour's rows and columns are enumerated with compile-time strides.
template <typename T, int W, int H, int LO>
__device__ inline void tile_lev_color(const level_view<T> &L, const stencil9<T> *rows,
                                      ptile<typename vec2_t<T>::type, W, H> &zs,
                                      ptile<typename vec2_t<T>::type, W, H> &bs, int x0, int y0, int cx, int cy) {
    typedef typename vec2_t<T>::type V;
    constexpr int NC = (W - 2 * LO + 1) / 2, NRW = (H - 2 * LO + 1) / 2;
    const int ty0 = LO + ((cy - (y0 + LO)) & 1), tx0 = LO + ((cx - (x0 + LO)) & 1);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    for (int k = tid; k < NRW * NC; k += nth) {
        const int ty = ty0 + 2 * (k / NC), tx = tx0 + 2 * (k % NC);
        if (ty > H - 1 - LO || tx > W - 1 - LO) continue;
        const int gy = y0 + ty;
        if (gy < 0 || gy >= L.n) continue;
        const stencil9<T> &s = tile_stencil(L, rows, ty, wrapx(x0 + tx, L.m), gy);
        const V a = lev_offdiag_tile<T>(s, zs, ty, tx, gy > 0, gy < L.n - 1);
        const V bb = bs(ty, tx);
        const T rx = bb.x - a.x, ry = bb.y - a.y;
        V o;
        o.x = s.e[9].a * rx + s.e[9].b * ry;
        o.y = s.e[9].c * rx + s.e[9].d * ry;
        zs(ty, tx) = o;
    }
}

template <typename T, int TX, int TY>
__global__ void __launch_bounds__(kFusedThreads) k_lev_down(level_view<T> L, level_view<T> C) {
    typedef typename vec2_t<T>::type V;
    constexpr int LDW = 2 * TX + 11, LDH = 2 * TY + 11;  // fine x in [2I0-6, 2I1+4]
    __shared__ ptile<V, LDW, LDH> zs, bs;
    __shared__ stencil9<T> rows[LDH];
    const int I0 = blockIdx.x * TX, J0 = blockIdx.y * TY;
    const int x0 = 2 * I0 - 6, y0 = 2 * J0 - 6;
    stage_row_stencils<T, LDH>(L, rows, y0);
    TILE_FOR(LDH, LDW, 0, 0, ty, tx) {
        const int gy = y0 + ty;
        V bb, zz;
        bb.x = bb.y = zz.x = zz.y = 0;
        if (gy >= 0 && gy < L.n) bb = L.b[(size_t)gy * L.m + wrapx(x0 + tx, L.m)];
        zs(ty, tx) = zz;
        bs(ty, tx) = bb;
    }
    __syncthreads();
    tile_lev_color<T, LDW, LDH, 1>(L, rows, zs, bs, x0, y0, 0, 0);
    __syncthreads();
    tile_lev_color<T, LDW, LDH, 2>(L, rows, zs, bs, x0, y0, 1, 0);
    __syncthreads();
    tile_lev_color<T, LDW, LDH, 3>(L, rows, zs, bs, x0, y0, 0, 1);
    __syncthreads();
    tile_lev_color<T, LDW, LDH, 4>(L, rows, zs, bs, x0, y0, 1, 1);
    __syncthreads();
    TILE_FOR(LDH - 10, LDW - 10, 5, 5, ty, tx) {
        const int gy = y0 + ty;
        if (gy < 0 || gy >= L.n) continue;
        const stencil9<T> &s = tile_stencil(L, rows, ty, wrapx(x0 + tx, L.m), gy);
        V a = lev_offdiag_tile<T>(s, zs, ty, tx, gy > 0, gy < L.n - 1);
        madd(a, s.e[4], zs(ty, tx));
        V r;
        r.x = bs(ty, tx).x - a.x;
        r.y = bs(ty, tx).y - a.y;
        bs(ty, tx) = r;
    }
    __syncthreads();
    TILE_FOR(TY, TX, 0, 0, cJ, cI) {
        const int I = I0 + cI, J = J0 + cJ;
        if (I < C.m && J < C.n) C.b[(size_t)J * C.m + I] = restrict_at<T>(bs, I, J, L.n, 2 * cI + 6, 2 * cJ + 6);
    }
    TILE_FOR(2 * TY, 2 * TX, 6, 6, ty, tx) {
        const int gy = y0 + ty, gx = x0 + tx;
        if (gy < L.n && gx < L.m) L.z[(size_t)gy * L.m + gx] = zs(ty, tx);
    }
}

template <typename T, int TX, int TY>
__global__ void __launch_bounds__(kFusedThreads) k_lev_up(level_view<T> L, level_view<T> C) {
    typedef typename vec2_t<T>::type V;
    constexpr int LUW = 2 * TX + 8, LUH = 2 * TY + 8;    // fine x in [2I0-4, 2I1+3]
    __shared__ ptile<V, LUW, LUH> zs, bs;
    __shared__ V cs[TY + 5][TX + 5];
    __shared__ stencil9<T> rows[LUH];
    const int I0 = blockIdx.x * TX, J0 = blockIdx.y * TY;
    const int x0 = 2 * I0 - 4, y0 = 2 * J0 - 4;
    stage_row_stencils<T, LUH>(L, rows, y0);
    TILE_FOR(LUH, LUW, 0, 0, ty, tx) {
        const int gy = y0 + ty;
        V zz, bb;
        zz.x = zz.y = bb.x = bb.y = 0;
        if (gy >= 0 && gy < L.n) {
            const size_t g = (size_t)gy * L.m + wrapx(x0 + tx, L.m);
            zz = L.z[g];
            bb = L.b[g];
        }
        zs(ty, tx) = zz;
        bs(ty, tx) = bb;
    }
    TILE_FOR(TY + 5, TX + 5, 0, 0, ly, lx) {
        const int J = J0 - 2 + ly;
        V v;
        v.x = v.y = 0;
        if (J >= 0 && J < C.n) v = C.z[(size_t)J * C.m + wrapx(I0 - 2 + lx, C.m)];
        cs[ly][lx] = v;
    }
    __syncthreads();
    TILE_FOR(LUH, LUW, 0, 0, ty, tx) {
        const int gy = y0 + ty;
        if (gy < 0 || gy >= L.n) continue;
        int cy[2], hy[2];
        const int ny = p1d_halves(gy, L.n, 0, cy, hy);
        {
            const int gx = wrapx(x0 + tx, L.m);
            const int c0 = gx >> 1, c1 = (gx == L.m - 1) ? 0 : c0 + 1;
            const bool odd = gx & 1;
            int l0 = c0 - (I0 - 2), l1 = c1 - (I0 - 2);
            l0 += l0 < 0 ? C.m : (l0 >= C.m ? -C.m : 0);
            l1 += l1 < 0 ? C.m : (l1 >= C.m ? -C.m : 0);
            T ax = 0, ay = 0;
            bool inside = true;
            for (int q = 0; q < ny; q++) {
                const int ly = cy[q] - (J0 - 2);
                if (ly < 0 || ly >= TY + 5 || l0 < 0 || l0 >= TX + 5 || (odd && (l1 < 0 || l1 >= TX + 5))) {
                    inside = false;
                    continue;
                }
                const T wy = (T)hy[q] * (T)0.25;
                if (odd) {
                    const V v0 = cs[ly][l0], v1 = cs[ly][l1];
                    ax += wy * (v0.x + v1.x);
                    ay += wy * (v0.y + v1.y);
                } else {
                    const V v0 = cs[ly][l0];
                    ax += (T)2 * wy * v0.x;
                    ay += (T)2 * wy * v0.y;
                }
            }
            if (!inside) ax = ay = 0;
            zs(ty, tx).x += ax;
            zs(ty, tx).y += ay;
        }
    }
    __syncthreads();
    tile_lev_color<T, LUW, LUH, 1>(L, rows, zs, bs, x0, y0, 0, 0);
    __syncthreads();
    tile_lev_color<T, LUW, LUH, 2>(L, rows, zs, bs, x0, y0, 1, 0);
    __syncthreads();
    tile_lev_color<T, LUW, LUH, 3>(L, rows, zs, bs, x0, y0, 0, 1);
    __syncthreads();
    tile_lev_color<T, LUW, LUH, 4>(L, rows, zs, bs, x0, y0, 1, 1);
    __syncthreads();
    TILE_FOR(2 * TY, 2 * TX, 4, 4, ty, tx) {
        const int gy = y0 + ty, gx = x0 + tx;
        if (gy < L.n && gx < L.m) L.z[(size_t)gy * L.m + gx] = zs(ty, tx);
    }
}

// ---------------------------------------------------------------------------
// Streaming coarse-level kernels (single precision, levels with one stencil
// class per row and an even periodic line).  The strip-and-window scheme of
// the top level with the four-colour block Gauss-Seidel of the stored
// Galerkin stencils: an even row takes colours (0,0) and (1,0) while both of
// its odd neighbour rows still hold their values from before the sweep, and
// the odd row below it then takes (0,1) and (1,1) between two finished even
// rows, so a warp advances two rows per iteration.  Within a row the even
// node of a pair is updated first (it reads the odd node of the lane to the
// left), then the odd node (it reads the new even node of the lane to the
// right).  Down: the sweep starts from z = 0 (down_gs_iterations,
// tgmg.hh:273-279), so only b is read; the swept z goes to the level's r
// array and the restricted residual to the child's b.  Up: z is taken from
// r, the child's correction added, and the sweep written back to z.  The
// outer four columns and the last two of a strip are halo, as are the rows
// before y0 and after the owned block.

constexpr int kLevDownCols = 27;  // coarse columns per strip (down): lanes 3..29
constexpr int kLevUpCols = 29;    // coarse columns per strip (up): lanes 2..30
constexpr int kMarchStencils = 16; // stencil classes a streaming level may have (staged in shared memory)

__device__ __forceinline__ float4 st_e(const stencil9<float> *s, int e) {
    return *reinterpret_cast<const float4 *>(s->e + e);
}

// The level's stencil table, copied to shared memory by the whole block.
__device__ __forceinline__ void stage_stencils(stencil9<float> *tab, const level_view<float> &L) {
    const float4 *src = reinterpret_cast<const float4 *>(L.st);
    float4 *dst = reinterpret_cast<float4 *>(tab);
    for (int k = threadIdx.x; k < L.nst * 10; k += blockDim.x) dst[k] = __ldg(src + k);
    __syncthreads();
}

// Stencil class of row j (0 outside the level; such rows are never swept).
__device__ __forceinline__ int row_class(const level_view<float> &L, int j) {
    return j >= 0 && j < L.n ? __ldg(L.cls + j) : 0;
}

// Off-diagonal products at the even node of the pair (tgmg_level::mul_a,
// tgmg.in.cc:536-547, in the order of lev_offdiag).
__device__ __forceinline__ float2 offdiag_even(const stencil9<float> *s, const float4 &d, const float4 &c,
                                               const float4 &u, bool has_d, bool has_u, int lsrc) {
    constexpr unsigned F = 0xffffffffu;
    const float dlx = __shfl_sync(F, d.z, lsrc), dly = __shfl_sync(F, d.w, lsrc);
    const float clx = __shfl_sync(F, c.z, lsrc), cly = __shfl_sync(F, c.w, lsrc);
    const float ulx = __shfl_sync(F, u.z, lsrc), uly = __shfl_sync(F, u.w, lsrc);
    float2 a = make_float2(0.f, 0.f);
    if (has_d) {
        madd4(a, st_e(s, 0), dlx, dly);
        madd4(a, st_e(s, 1), d.x, d.y);
        madd4(a, st_e(s, 2), d.z, d.w);
    }
    madd4(a, st_e(s, 3), clx, cly);
    madd4(a, st_e(s, 5), c.z, c.w);
    if (has_u) {
        madd4(a, st_e(s, 6), ulx, uly);
        madd4(a, st_e(s, 7), u.x, u.y);
        madd4(a, st_e(s, 8), u.z, u.w);
    }
    return a;
}

// The same at the odd node of the pair.
__device__ __forceinline__ float2 offdiag_odd(const stencil9<float> *s, const float4 &d, const float4 &c,
                                              const float4 &u, bool has_d, bool has_u, int rsrc) {
    constexpr unsigned F = 0xffffffffu;
    const float drx = __shfl_sync(F, d.x, rsrc), dry = __shfl_sync(F, d.y, rsrc);
    const float crx = __shfl_sync(F, c.x, rsrc), cry = __shfl_sync(F, c.y, rsrc);
    const float urx = __shfl_sync(F, u.x, rsrc), ury = __shfl_sync(F, u.y, rsrc);
    float2 a = make_float2(0.f, 0.f);
    if (has_d) {
        madd4(a, st_e(s, 0), d.x, d.y);
        madd4(a, st_e(s, 1), d.z, d.w);
        madd4(a, st_e(s, 2), drx, dry);
    }
    madd4(a, st_e(s, 3), c.x, c.y);
    madd4(a, st_e(s, 5), crx, cry);
    if (has_u) {
        madd4(a, st_e(s, 6), u.x, u.y);
        madd4(a, st_e(s, 7), u.z, u.w);
        madd4(a, st_e(s, 8), urx, ury);
    }
    return a;
}

// Both colours of row j (stencil s) that touch the pair: even node, then odd
// node; lsrc / rsrc: the lanes holding the pairs to the left and right.
__device__ __forceinline__ void lev_row_sweep(const stencil9<float> *s, int j, int n, const float4 &d, float4 &c,
                                              const float4 &u, const float4 &bb, int lsrc, int rsrc) {
    const bool hd = j > 0, hu = j < n - 1;
    const float4 iv = st_e(s, 9);
    float2 a = offdiag_even(s, d, c, u, hd, hu, lsrc);
    float rx = bb.x - a.x, ry = bb.y - a.y;
    c.x = iv.x * rx + iv.y * ry;
    c.y = iv.z * rx + iv.w * ry;
    a = offdiag_odd(s, d, c, u, hd, hu, rsrc);
    rx = bb.z - a.x;
    ry = bb.w - a.y;
    c.z = iv.x * rx + iv.y * ry;
    c.w = iv.z * rx + iv.w * ry;
}

// Residual b - A z of the pair on row j (even node .x .y, odd node .z .w).
__device__ __forceinline__ float4 lev_pair_residual(const stencil9<float> *s, int j, int n, const float4 &d,
                                                    const float4 &c, const float4 &u, const float4 &bb, int lsrc,
                                                    int rsrc) {
    const bool hd = j > 0, hu = j < n - 1;
    const float4 cc = st_e(s, 4);
    float2 a = offdiag_even(s, d, c, u, hd, hu, lsrc);
    madd4(a, cc, c.x, c.y);
    // the odd node of an odd row took the last colour, (1,1), and none of its
    // neighbours changed after: its residual is zero up to rounding
    if (j & 1) return make_float4(bb.x - a.x, bb.y - a.y, 0.f, 0.f);
    float2 e = offdiag_odd(s, d, c, u, hd, hu, rsrc);
    madd4(e, cc, c.z, c.w);
    return make_float4(bb.x - a.x, bb.y - a.y, bb.z - e.x, bb.w - e.y);
}

// Full weighting of the residual rows 2J-1, 2J, 2J+1 at the coarse point
// under the lane's even node (restrict_at).
__device__ __forceinline__ float2 lev_restrict(const float4 &r0, const float4 &r1, const float4 &r2, int J, int n,
                                               int lsrc) {
    constexpr unsigned F = 0xffffffffu;
    const float4 rr[3] = {r0, r1, r2};
    float ax = 0, ay = 0;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const float lx = __shfl_sync(F, rr[q].z, lsrc), ly = __shfl_sync(F, rr[q].w, lsrc);
        const int hy = restrict_hy(q, J, n);
        if (!hy) continue;
        const float w1 = (float)hy * 0.25f, w2 = (float)(2 * hy) * 0.25f;
        ax += w1 * lx;
        ay += w1 * ly;
        ax += w2 * rr[q].x;
        ay += w2 * rr[q].y;
        ax += w1 * rr[q].z;
        ay += w1 * rr[q].w;
    }
    return make_float2(ax, ay);
}

// One warp's march down a strip (coarse columns I0 .., coarse rows J0 ..
// J0+TCH-1): the level's sweep, its residual and the restriction into the
// child's b.  tab: the level's stencil table in shared memory.
template <int TCH, bool CG>
__device__ __forceinline__ void lev_down_march(const level_view<float> &L, const level_view<float> &C,
                                               const stencil9<float> *tab, int I0, int J0, int lane) {
    const int lsrc = (lane + 31) & 31, rsrc = (lane + 1) & 31;
    const int m = L.m, n = L.n;
    const int xs = 2 * I0 - 6, y0 = 2 * J0;
    const int gx = wrapx(xs + 2 * lane, m);
    const int I = I0 + lane - 3;
    const bool own = lane >= 3 && lane < 3 + kLevDownCols && I < C.m;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 W0 = zero, W1 = zero, W2 = zero, W3 = zero, W4 = zero;  // z rows k-4 .. k
    float4 B0 = zero, B1 = zero, B2 = zero, B3 = zero;             // b rows k-3 .. k
    int S0 = 0, S1 = 0, S2 = 0, S3 = 0;                            // stencil classes of rows k-3 .. k
    float4 Rp = zero;                                              // residual row k-4
    const int kb = y0 - 4, ke = y0 + 2 * TCH + 1;
    float4 nb0 = march_load<CG>(L.b, kb, m, n, gx), nb1 = march_load<CG>(L.b, kb + 1, m, n, gx);
    int ns0 = row_class(L, kb), ns1 = row_class(L, kb + 1);
    for (int k = kb + 1; k <= ke; k += 2) {
        W0 = W2; W1 = W3; W2 = W4; W3 = zero; W4 = zero;
        B0 = B2; B1 = B3; B2 = nb0; B3 = nb1;
        S0 = S2; S1 = S3; S2 = ns0; S3 = ns1;
        if (k + 2 <= ke) {
            nb0 = march_load<CG>(L.b, k + 1, m, n, gx);
            nb1 = march_load<CG>(L.b, k + 2, m, n, gx);
            ns0 = row_class(L, k + 1);
            ns1 = row_class(L, k + 2);
        }
        const int je = k - 1, jo = k - 2;
        if (je >= 0 && je < n) lev_row_sweep(tab + S2, je, n, W2, W3, W4, B2, lsrc, rsrc);
        if (jo >= kb + 1 && jo >= 0 && jo < n) lev_row_sweep(tab + S1, jo, n, W1, W2, W3, B1, lsrc, rsrc);
        if (own) {
            if (je >= y0 && je < y0 + 2 * TCH && je < n) *reinterpret_cast<float4 *>(L.r + (size_t)je * m + gx) = W3;
            if (jo >= y0 && jo < y0 + 2 * TCH && jo < n) *reinterpret_cast<float4 *>(L.r + (size_t)jo * m + gx) = W2;
        }
        const int j3 = k - 3, j2 = k - 2;
        float4 R3 = zero, R2 = zero;
        if (j3 >= y0 - 1 && j3 >= 0 && j3 < n) R3 = lev_pair_residual(tab + S0, j3, n, W0, W1, W2, B0, lsrc, rsrc);
        if (j2 >= y0 - 1 && j2 >= 0 && j2 < n) R2 = lev_pair_residual(tab + S1, j2, n, W1, W2, W3, B1, lsrc, rsrc);
        const int J = j3 >> 1;  // rows 2J-1, 2J, 2J+1 = k-4, k-3, k-2
        if (j3 >= y0) {
            const float2 w = lev_restrict(Rp, R3, R2, J, n, lsrc);
            if (own && J < C.n) C.b[(size_t)J * C.m + I] = w;
        }
        Rp = R2;
    }
}

template <int TCH>
__global__ void __launch_bounds__(32 * kMarchWarps) k_lev_down_m(level_view<float> L, level_view<float> C) {
    __shared__ stencil9<float> tab[kMarchStencils];
    pdl_trigger();
    stage_stencils(tab, L);
    const int J0 = (blockIdx.y * kMarchWarps + (threadIdx.x >> 5)) * TCH;
    if (J0 >= C.n) return;
    pdl_wait();
    lev_down_march<TCH, false>(L, C, tab, blockIdx.x * kLevDownCols, J0, threadIdx.x & 31);
}

// One warp's march up a strip: the child's correction added to the swept z
// the down march left in r (czs: the warp's shared staging of the child's
// strip, TCH + 3 rows), the level's sweep, the result written to z.
template <int TCH, bool CG>
__device__ __forceinline__ void lev_up_march(const level_view<float> &L, const level_view<float> &C,
                                             const stencil9<float> *tab, float2 (*czs)[33], int I0, int J0, int lane) {
    const int lsrc = (lane + 31) & 31, rsrc = (lane + 1) & 31;
    const int m = L.m, n = L.n;
    const int xs = 2 * I0 - 4, y0 = 2 * J0;
    const int gx = wrapx(xs + 2 * lane, m);
    const bool own = lane >= 2 && lane < 2 + kLevUpCols && xs + 2 * lane < m;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 W0 = zero, W1 = zero, W2 = zero, W3 = zero;  // z rows k-3 .. k
    float4 B0 = zero, B1 = zero, B2 = zero;             // b rows k-2 .. k
    int S0 = 0, S1 = 0, S2 = 0;                         // stencil classes of rows k-2 .. k
    const int kb = y0 - 2, ke = y0 + 2 * TCH + 1;
    float4 nz0 = march_load<CG>(L.r, kb, m, n, gx), nz1 = march_load<CG>(L.r, kb + 1, m, n, gx);
    float4 nb0 = march_load<CG>(L.b, kb, m, n, gx), nb1 = march_load<CG>(L.b, kb + 1, m, n, gx);
    int ns0 = row_class(L, kb), ns1 = row_class(L, kb + 1);
    stage_coarse<TCH + 3, CG>(czs, C.z, C.m, C.n, xs / 2, J0 - 1, lane);
    for (int k = kb + 1; k <= ke; k += 2) {
        float4 z0 = nz0, z1 = nz1;
        B0 = B2; B1 = nb0; B2 = nb1;
        S0 = S2; S1 = ns0; S2 = ns1;
        if (k + 2 <= ke) {
            nz0 = march_load<CG>(L.r, k + 1, m, n, gx);
            nz1 = march_load<CG>(L.r, k + 2, m, n, gx);
            nb0 = march_load<CG>(L.b, k + 1, m, n, gx);
            nb1 = march_load<CG>(L.b, k + 2, m, n, gx);
            ns0 = row_class(L, k + 1);
            ns1 = row_class(L, k + 2);
        }
        prolong_staged(z0, czs, J0 - 1, lane, k - 1, n);
        prolong_staged(z1, czs, J0 - 1, lane, k, n);
        W0 = W2; W1 = W3; W2 = z0; W3 = z1;
        const int je = k - 1, jo = k - 2;
        if (je >= 0 && je < n) lev_row_sweep(tab + S1, je, n, W1, W2, W3, B1, lsrc, rsrc);
        if (jo >= kb + 1 && jo >= 0 && jo < n) lev_row_sweep(tab + S0, jo, n, W0, W1, W2, B0, lsrc, rsrc);
        if (own) {
            if (je >= y0 && je < y0 + 2 * TCH && je < n) *reinterpret_cast<float4 *>(L.z + (size_t)je * m + gx) = W2;
            if (jo >= y0 && jo < y0 + 2 * TCH && jo < n) *reinterpret_cast<float4 *>(L.z + (size_t)jo * m + gx) = W1;
        }
    }
}

template <int TCH>
__global__ void __launch_bounds__(32 * kMarchWarps) k_lev_up_m(level_view<float> L, level_view<float> C) {
    __shared__ stencil9<float> tab[kMarchStencils];
    __shared__ float2 czs[kMarchWarps][TCH + 3][33];
    pdl_trigger();
    stage_stencils(tab, L);
    const int w = threadIdx.x >> 5;
    const int J0 = (blockIdx.y * kMarchWarps + w) * TCH;
    if (J0 >= C.n) return;
    pdl_wait();
    lev_up_march<TCH, false>(L, C, tab, czs[w], blockIdx.x * kLevUpCols, J0, threadIdx.x & 31);
}

// ---------------------------------------------------------------------------
// Tail of the V-cycle on small levels, one block of 32 x 32 threads: levels
// t..ml-1 go down (clear, sweep, residual, restriction), the coarsest level
// is solved, and the levels come back up to t (prolongation, sweep).  All
// levels live in shared memory; level t exchanges b and z with its global
// arrays.  Phases are separated by __syncthreads.

struct tail_levels {
    int t, ml;
    const double *inv;
    int inv_n;
    int inv_off;  // byte offset of a shared-memory copy of inv (pair tail), -1: none
};

template <typename T>
__device__ void tail_sweep(const level_view<T> &L) {
    typedef typename vec2_t<T>::type V;
    for (int cy = 0; cy < 2; cy++)
        for (int cx = 0; cx < L.colors_x; cx++) {
            for (int j = cy + 2 * threadIdx.y; j < L.n; j += 2 * blockDim.y) {
                const int ist = cx == 2 ? L.m - 1 + 2 * threadIdx.x : cx + 2 * threadIdx.x;
                for (int i = ist; i < L.m; i += 2 * blockDim.x) {
                    if (cx < 2 && L.colors_x == 3 && i == L.m - 1) continue;
                    const stencil9<T> &s = stencil_at(L, i, j);
                    const size_t ij = (size_t)j * L.m + i;
                    V a = lev_offdiag<T, V>(L, s, L.z, i, j);
                    V r, o;
                    r.x = L.b[ij].x - a.x;
                    r.y = L.b[ij].y - a.y;
                    o.x = s.e[9].a * r.x + s.e[9].b * r.y;
                    o.y = s.e[9].c * r.x + s.e[9].d * r.y;
                    L.z[ij] = o;
                }
            }
            __syncthreads();
        }
}

// Stencil tables and class arrays of the tail levels are copied into shared
// memory when they are small (x-homogeneous levels: a few stencils and one
// class per row), so that the sweeps' stencil reads do not wait on L2.
constexpr size_t kTailStageMax = 16 * 1024;

template <typename T> __host__ __device__ inline size_t tail_stage_bytes(int nst, int ncls) {
    return sizeof(stencil9<T>) * (size_t)nst + sizeof(int) * (size_t)ncls;
}

// Prologue of the tail kernels: places every tail level (z, b, r) and the
// small stencil tables in shared memory, copies the first level's b in and
// clears its z (the down sweeps start from z = 0, gauss_seidel_from_zero;
// coarser levels get their zero z with their b in the restriction).
template <typename T>
__device__ void tail_prologue(const tail_levels &tl, const hierarchy_view<T> &H, level_view<T> *S,
                              unsigned char *tail_raw, int tid, int nth) {
    typedef typename vec2_t<T>::type V;
    if (tid == 0) {
        size_t off = (sizeof(double) * tl.inv_n + 15) & ~(size_t)15;
        for (int l = tl.t; l <= tl.ml; l++) {
            S[l] = H.lv[l];
            const size_t mn = (size_t)S[l].m * S[l].n;
            S[l].z = (V *)(tail_raw + off);
            S[l].b = S[l].z + mn;
            S[l].r = S[l].b + mn;
            off += 3 * sizeof(V) * mn;
        }
        for (int l = tl.t; l < tl.ml; l++) {
            if (tail_stage_bytes<T>(S[l].nst, S[l].ncls) > kTailStageMax) continue;
            off = (off + 31) & ~(size_t)31;
            S[l].st = (const stencil9<T> *)(tail_raw + off);
            off += sizeof(stencil9<T>) * (size_t)S[l].nst;
            S[l].cls = (const int *)(tail_raw + off);
            off += sizeof(int) * (size_t)S[l].ncls;
        }
    }
    __syncthreads();
    for (int l = tl.t; l < tl.ml; l++) {
        if (S[l].st == H.lv[l].st) continue;  // not staged
        T *st = (T *)S[l].st;
        const T *src = (const T *)H.lv[l].st;
        const int nt = S[l].nst * (int)(sizeof(stencil9<T>) / sizeof(T));
        for (int k = tid; k < nt; k += nth) st[k] = src[k];
        int *cl = (int *)S[l].cls;
        for (int k = tid; k < S[l].ncls; k += nth) cl[k] = H.lv[l].cls[k];
    }
    const int mn = S[tl.t].m * S[tl.t].n;
    for (int k = tid; k < mn; k += nth) {
        S[tl.t].b[k] = __ldcg(H.lv[tl.t].b + k);  // written by other blocks in the persistent kernel
        S[tl.t].z[k].x = 0;
        S[tl.t].z[k].y = 0;
    }
    __syncthreads();
}

// Coarsest level: z = A^-1 b in FP64, one warp per row of the inverse
// (coalesced reads, shuffle sum); inv in global or shared memory.
template <typename T>
__device__ void tail_bottom(const tail_levels &tl, const double *inv, const level_view<T> &B, double *tsh, int tid,
                            int nth) {
    const int N = tl.inv_n;
    for (int k = tid; k < N / 2; k += nth) {
        tsh[2 * k] = (double)B.b[k].x;
        tsh[2 * k + 1] = (double)B.b[k].y;
    }
    __syncthreads();
    T *zz = (T *)B.z;
    const int lane = tid & 31, nw = nth >> 5;
    for (int r = tid >> 5; r < N; r += nw) {
        const double *row = inv + (size_t)r * N;
        double a = 0;
        for (int k = lane; k < N; k += 32) a += row[k] * tsh[k];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) zz[r] = (T)a;
    }
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(1024) k_tail(tail_levels tl, hierarchy_view<T> H) {
    typedef typename vec2_t<T>::type V;
    extern __shared__ __align__(32) unsigned char tail_raw[];
    __shared__ level_view<T> S[17];  // the levels' views, read by every phase
    double *tsh = (double *)tail_raw;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    tail_prologue(tl, H, S, tail_raw, tid, nth);
    for (int i = tl.t; i < tl.ml; i++) {
        const level_view<T> &L = S[i];
        tail_sweep(L);
        for (int jj = threadIdx.y; jj < L.n; jj += blockDim.y)
            for (int ii = threadIdx.x; ii < L.m; ii += blockDim.x) {
                const size_t k = (size_t)jj * L.m + ii;
                const stencil9<T> &s = stencil_at(L, ii, jj);
                V a = lev_offdiag<T, V>(L, s, L.z, ii, jj);
                madd(a, s.e[4], L.z[k]);
                V r;
                r.x = L.b[k].x - a.x;
                r.y = L.b[k].y - a.y;
                L.r[k] = r;
            }
        __syncthreads();
        const level_view<T> &C = S[i + 1];
        for (int J = threadIdx.y; J < C.n; J += blockDim.y)
            for (int I = threadIdx.x; I < C.m; I += blockDim.x) {
                T ax = 0, ay = 0;
                for (int dy = -1; dy <= 1; dy++) {
                    const int fy = 2 * J + dy;
                    if (fy < 0 || fy >= L.n) continue;
                    const int hy = halves_of(fy, L.n, 0, J);
                    if (!hy) continue;
                    for (int dx = -1; dx <= 1; dx++) {
                        const int fx = wrapx(2 * I + dx, L.m);
                        const int hx = halves_of(fx, L.m, 1, I);
                        if (!hx) continue;
                        const V v = L.r[(size_t)fy * L.m + fx];
                        const T wgt = (T)(hx * hy) * (T)0.25;
                        ax += wgt * v.x;
                        ay += wgt * v.y;
                    }
                }
                V o;
                o.x = ax;
                o.y = ay;
                C.b[(size_t)J * C.m + I] = o;
                o.x = o.y = 0;
                C.z[(size_t)J * C.m + I] = o;
            }
        __syncthreads();
    }
    tail_bottom(tl, tl.inv, S[tl.ml], tsh, tid, nth);
    for (int i = tl.ml; i > tl.t; i--) {
        const level_view<T> &C = S[i], &F = S[i - 1];
        for (int jj = threadIdx.y; jj < F.n; jj += blockDim.y) {
            int cy[2], hy[2];
            const int ny = p1d_halves(jj, F.n, 0, cy, hy);
            for (int ii = threadIdx.x; ii < F.m; ii += blockDim.x) {
                int cx[2], hx[2];
                const int nx = p1d_halves(ii, F.m, 1, cx, hx);
                T ax = 0, ay = 0;
                for (int bq = 0; bq < ny; bq++)
                    for (int a = 0; a < nx; a++) {
                        const V v = C.z[(size_t)cy[bq] * C.m + cx[a]];
                        const T wgt = (T)(hx[a] * hy[bq]) * (T)0.25;
                        ax += wgt * v.x;
                        ay += wgt * v.y;
                    }
                const size_t k = (size_t)jj * F.m + ii;
                F.z[k].x += ax;
                F.z[k].y += ay;
            }
        }
        __syncthreads();
        tail_sweep(F);
    }
    {
        const int mn = S[tl.t].m * S[tl.t].n;
        for (int k = tid; k < mn; k += nth) H.lv[tl.t].z[k] = S[tl.t].z[k];
    }
}

// Tail of the V-cycle with the pair scheme of the streaming kernels (single
// precision; every level above the coarsest of even width <= 64, one stencil
// class per row, its table staged): a warp holds a whole row of a level,
// lane L the node pair (2L, 2L+1), and the periodic neighbours come by
// shuffles from lanes L-1 and L+1 modulo m/2.  A sweep is two phases (the
// even rows with colours (0,0), (1,0), then the odd rows with (0,1),
// (1,1)); residual, restriction and prolongation take one phase each.

// Shared-memory addresses of a tail level, rebuilt from byte offsets so that
// the compiler sees the shared state space (plain shared loads and stores).
struct pair_level {
    float4 *z, *r;
    const float4 *b;
    float2 *z2, *b2;
    const stencil9<float> *st;
    const int *cls;
};

__device__ __forceinline__ pair_level pair_view(unsigned char *raw, const unsigned (*offs)[5], int l) {
    pair_level v;
    v.z = reinterpret_cast<float4 *>(raw + offs[l][0]);
    v.b = reinterpret_cast<const float4 *>(raw + offs[l][1]);
    v.r = reinterpret_cast<float4 *>(raw + offs[l][2]);
    v.z2 = reinterpret_cast<float2 *>(raw + offs[l][0]);
    v.b2 = reinterpret_cast<float2 *>(raw + offs[l][1]);
    v.st = reinterpret_cast<const stencil9<float> *>(raw + offs[l][3]);
    v.cls = reinterpret_cast<const int *>(raw + offs[l][4]);
    return v;
}

__device__ __forceinline__ void tail_pair_sweep(const pair_level &V, int n, int P, int ln, int lane, int lsrc,
                                                int rsrc, int w, int nw) {
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int par = 0; par < 2; par++) {
        for (int j = 2 * w + par; j < n; j += 2 * nw) {
            const float4 d = j > 0 ? V.z[(j - 1) * P + ln] : zero;
            float4 c = V.z[j * P + ln];
            const float4 u = j < n - 1 ? V.z[(j + 1) * P + ln] : zero;
            lev_row_sweep(V.st + V.cls[j], j, n, d, c, u, V.b[j * P + ln], lsrc, rsrc);
            if (lane < P) V.z[j * P + lane] = c;
        }
        __syncthreads();
    }
}

// The coarsest inverse copied into the tail's shared memory (when it has a
// place there), asynchronously: it arrives while the down sweeps run.
__device__ __forceinline__ void tail_inv_prefetch(const tail_levels &tl, unsigned char *tail_raw, int tid, int nth) {
    if (tl.inv_off < 0) return;
    const int N = tl.inv_n;
    double *dst = reinterpret_cast<double *>(tail_raw + tl.inv_off);
    for (int k = tid; k < N * N; k += nth) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + k);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(tl.inv + k) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// The pair tail on one block of 32 x nw threads (lane, warp w): levels t ..
// ml-1 down, the coarsest solve, back up to t; level t's b is read from and
// its z written to global memory.  S, offs: the caller's shared views.
__device__ void tail_pairs_body(const tail_levels &tl, const hierarchy_view<float> &H, unsigned char *tail_raw,
                                level_view<float> *S, unsigned (*offs)[5], int lane, int w, int nw) {
    double *tsh = (double *)tail_raw;
    const int tid = w * 32 + lane, nth = 32 * nw;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    tail_prologue(tl, H, S, tail_raw, tid, nth);
    if (tid == 0)
        for (int l = tl.t; l <= tl.ml; l++) {
            offs[l][0] = (unsigned)((const unsigned char *)S[l].z - tail_raw);
            offs[l][1] = (unsigned)((const unsigned char *)S[l].b - tail_raw);
            offs[l][2] = (unsigned)((const unsigned char *)S[l].r - tail_raw);
            offs[l][3] = l < tl.ml ? (unsigned)((const unsigned char *)S[l].st - tail_raw) : 0u;
            offs[l][4] = l < tl.ml ? (unsigned)((const unsigned char *)S[l].cls - tail_raw) : 0u;
        }
    __syncthreads();
    for (int l = tl.t; l < tl.ml; l++) {
        const pair_level V = pair_view(tail_raw, offs, l), Cv = pair_view(tail_raw, offs, l + 1);
        const int P = S[l].m >> 1, n = S[l].n, cn = S[l + 1].n, ln = lane < P ? lane : P - 1;
        const int lsrc = ln == 0 ? P - 1 : ln - 1, rsrc = ln + 1 == P ? 0 : ln + 1;
        tail_pair_sweep(V, n, P, ln, lane, lsrc, rsrc, w, nw);
        for (int j = w; j < n; j += nw) {
            const float4 d = j > 0 ? V.z[(j - 1) * P + ln] : zero, c = V.z[j * P + ln];
            const float4 u = j < n - 1 ? V.z[(j + 1) * P + ln] : zero;
            const float4 r = lev_pair_residual(V.st + V.cls[j], j, n, d, c, u, V.b[j * P + ln], lsrc, rsrc);
            if (lane < P) V.r[j * P + lane] = r;
        }
        __syncthreads();
        for (int J = w; J < cn; J += nw) {
            const int f0 = 2 * J - 1;
            const float4 r0 = f0 >= 0 && f0 < n ? V.r[f0 * P + ln] : zero;
            const float4 r1 = f0 + 1 < n ? V.r[(f0 + 1) * P + ln] : zero;
            const float4 r2 = f0 + 2 < n ? V.r[(f0 + 2) * P + ln] : zero;
            const float2 v = lev_restrict(r0, r1, r2, J, n, lsrc);
            if (lane < P) {
                Cv.b2[J * P + lane] = v;
                Cv.z2[J * P + lane] = make_float2(0.f, 0.f);
            }
        }
        __syncthreads();
    }
    if (tl.inv_off >= 0) {
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        __syncthreads();
        tail_bottom(tl, reinterpret_cast<const double *>(tail_raw + tl.inv_off), S[tl.ml], tsh, tid, nth);
    } else {
        tail_bottom(tl, tl.inv, S[tl.ml], tsh, tid, nth);
    }
    for (int l = tl.ml - 1; l >= tl.t; l--) {
        const pair_level V = pair_view(tail_raw, offs, l), Cv = pair_view(tail_raw, offs, l + 1);
        const int P = S[l].m >> 1, n = S[l].n, ln = lane < P ? lane : P - 1;
        const int lsrc = ln == 0 ? P - 1 : ln - 1, rsrc = ln + 1 == P ? 0 : ln + 1;
        // the child has m/2 = P columns: the even node takes coarse ln, the
        // odd node the mean of ln and rsrc
        for (int j = w; j < n; j += nw) {
            int cy[2], hy[2];
            const int ny = p1d_halves(j, n, 0, cy, hy);
            float ax = 0, ay = 0, bx = 0, by = 0;
            for (int q = 0; q < ny; q++) {
                const float wy = (float)hy[q] * 0.25f;
                const float2 v0 = Cv.z2[cy[q] * P + ln], v1 = Cv.z2[cy[q] * P + rsrc];
                ax += 2.f * wy * v0.x;
                ay += 2.f * wy * v0.y;
                bx += wy * (v0.x + v1.x);
                by += wy * (v0.y + v1.y);
            }
            if (lane < P) {
                float4 z = V.z[j * P + lane];
                z.x += ax;
                z.y += ay;
                z.z += bx;
                z.w += by;
                V.z[j * P + lane] = z;
            }
        }
        __syncthreads();
        tail_pair_sweep(V, n, P, ln, lane, lsrc, rsrc, w, nw);
    }
    const pair_level V = pair_view(tail_raw, offs, tl.t);
    const int mn = S[tl.t].m * S[tl.t].n;
    for (int k = tid; k < mn; k += nth) H.lv[tl.t].z[k] = V.z2[k];
}

__global__ void __launch_bounds__(1024) k_tail_pairs(tail_levels tl, hierarchy_view<float> H) {
    extern __shared__ __align__(32) unsigned char tail_raw[];
    __shared__ level_view<float> S[17];
    __shared__ unsigned offs[17][5];
    const int lane = threadIdx.x, w = threadIdx.y, nw = blockDim.y;
    tail_inv_prefetch(tl, tail_raw, w * 32 + lane, 32 * nw);
    pdl_trigger();
    pdl_wait();
    tail_pairs_body(tl, H, tail_raw, S, offs, lane, w, nw);
}

// ---------------------------------------------------------------------------
// Persistent coarse kernel: the streaming levels p .. t-1 (all at most
// kPersistWidth wide), the pair tail on levels t .. ml and the way back up in
// ONE cooperative launch of one block per SM.  Each level's march down is a
// phase in which the grid's warps take the level's (strip, row block) units in
// turn; a grid barrier separates the phases.  Block 0 runs the tail while the
// others wait at the barrier after it.  Data that other blocks wrote in an
// earlier phase are read through L2 (__ldcg): L1 is not coherent across SMs.
// The barrier's waits are bounded: past kBarrierPolls polls the waiting block
// sets the error word and the whole grid leaves at its next barrier (the
// V-cycle's result is then invalid and the host reports the error).

#ifndef STZG_PERSIST_WIDTH
#define STZG_PERSIST_WIDTH 512
#endif
#ifndef STZG_BARRIER_SLEEP_NS
#define STZG_BARRIER_SLEEP_NS 32
#endif
constexpr int kPersistWidth = STZG_PERSIST_WIDTH;  // widest level the persistent kernel marches
constexpr int kPersistWarps = 16;    // warps per block (32 x 16 threads)
constexpr int kPersistRows = 2;      // coarse rows per march unit
constexpr long kBarrierPolls = 1L << 21;

struct coarse_plan {
    int p, t;        // streaming levels [p, t); the tail takes [t, ml]
    tail_levels tl;
    unsigned *bar;   // [0] arrivals, [1] generation
    int *err;        // set to 1 when a barrier wait runs out
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// All blocks of the grid meet here; false when a wait ran out (here or in
// another block), after which the caller returns.
__device__ bool grid_barrier(const coarse_plan &cp, unsigned &gen, int *s_ok) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        int ok = 1;
        __threadfence();
        if (atomicAdd(cp.bar, 1u) == gridDim.x - 1) {
            atomicExch(cp.bar, 0u);
            __threadfence();
            atomicExch(cp.bar + 1, gen + 1);
        } else {
            long polls = 0;
            while (ld_acquire(cp.bar + 1) == gen) {
                if (++polls > kBarrierPolls) {
                    atomicExch(cp.err, 1);
                    ok = 0;
                    break;
                }
                if ((polls & 1023) == 0 && *(volatile int *)cp.err) break;  // another block gave up
                if (STZG_BARRIER_SLEEP_NS > 0) __nanosleep(STZG_BARRIER_SLEEP_NS);
            }
        }
        gen++;
        if (ok && *(volatile int *)cp.err) ok = 0;
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// The level's stencil table into shared memory by the whole block.
__device__ __forceinline__ void stage_table(stencil9<float> *tab, const level_view<float> &L, int tid, int nth) {
    const float4 *src = reinterpret_cast<const float4 *>(L.st);
    float4 *dst = reinterpret_cast<float4 *>(tab);
    for (int k = tid; k < L.nst * 10; k += nth) dst[k] = __ldg(src + k);
    __syncthreads();
}

__global__ void __launch_bounds__(32 * kPersistWarps, 1)
    k_coarse_persist(coarse_plan cp, const __grid_constant__ hierarchy_view<float> H) {
    extern __shared__ __align__(32) unsigned char tail_raw[];
    __shared__ stencil9<float> tab[kMarchStencils];
    __shared__ level_view<float> S[17];
    __shared__ unsigned offs[17][5];
    __shared__ int s_ok;
    if (cp.p > cp.t) return;  // empty plan (set-up probe)
    // a barrier of an earlier launch timed out: its words are stale until the
    // host clears them, so this V-cycle is skipped (the host reports the error)
    if (*(volatile int *)cp.err) return;
    const int lane = threadIdx.x, w = threadIdx.y, tid = w * 32 + lane, nth = 32 * kPersistWarps;
    const int gw = blockIdx.x * kPersistWarps + w, nwarps = gridDim.x * kPersistWarps;
    // the generation cannot move before every block has arrived once
    unsigned gen = tid == 0 ? ld_acquire(cp.bar + 1) : 0u;
    if (blockIdx.x == 0) tail_inv_prefetch(cp.tl, tail_raw, tid, nth);
    for (int l = cp.p; l < cp.t; l++) {
        const level_view<float> &L = H.lv[l], &C = H.lv[l + 1];
        stage_table(tab, L, tid, nth);
        const int strips = (C.m + kLevDownCols - 1) / kLevDownCols;
        const int units = strips * ((C.n + kPersistRows - 1) / kPersistRows);
        for (int u = gw; u < units; u += nwarps) {
            const int sx = u % strips, ry = u / strips;
            lev_down_march<kPersistRows, true>(L, C, tab, sx * kLevDownCols, ry * kPersistRows, lane);
        }
        if (!grid_barrier(cp, gen, &s_ok)) return;
    }
    if (blockIdx.x == 0) tail_pairs_body(cp.tl, H, tail_raw, S, offs, lane, w, kPersistWarps);
    if (!grid_barrier(cp, gen, &s_ok)) return;
    // the up marches stage the child's strip per warp where the tail was
    float2 (*czs)[33] = reinterpret_cast<float2 (*)[33]>(tail_raw) + w * (kPersistRows + 3);
    for (int l = cp.t - 1; l >= cp.p; l--) {
        const level_view<float> &L = H.lv[l], &C = H.lv[l + 1];
        stage_table(tab, L, tid, nth);
        const int strips = (C.m + kLevUpCols - 1) / kLevUpCols;
        const int units = strips * ((C.n + kPersistRows - 1) / kPersistRows);
        for (int u = gw; u < units; u += nwarps) {
            const int sx = u % strips, ry = u / strips;
            lev_up_march<kPersistRows, true>(L, C, tab, czs, sx * kLevUpCols, ry * kPersistRows, lane);
            __syncwarp();  // the next unit restages czs
        }
        if (l > cp.p && !grid_barrier(cp, gen, &s_ok)) return;
    }
}

constexpr size_t kTailSmem = 200 * 1024;
#ifndef STZG_TAIL_WARPS
#define STZG_TAIL_WARPS 32
#endif

// Shared memory of the tail from level t: the same partition as k_tail.
template <typename T> size_t tail_smem_bytes(const hierarchy<T> &h, int t) {
    size_t b = ((sizeof(double) * h.bottom_unknowns + 15) & ~(size_t)15);
    for (int l = t; l < h.nl; l++) b += 3 * sizeof(typename vec2_t<T>::type) * (size_t)h.lv[l].m * h.lv[l].n;
    for (int l = t; l < h.nl - 1; l++) {
        const size_t sb = tail_stage_bytes<T>(h.lv[l].nst, h.lv[l].ncls);
        if (sb <= kTailStageMax) b = ((b + 31) & ~(size_t)31) + sb;
    }
    return b;
}

}  // namespace

// Opt the tail kernel into the shared memory it needs (set once per
// process, outside any stream capture).
template <typename T> cudaError_t prepare_tail_kernel() {
    static bool done = false;
    if (done) return cudaSuccess;
    done = true;
    cudaError_t e = cudaFuncSetAttribute(k_tail<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTailSmem + 1024);
    if (e == cudaSuccess && sizeof(T) == 4)
        e = cudaFuncSetAttribute(k_tail_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTailSmem + 1024);
    return e;
}
template cudaError_t prepare_tail_kernel<float>();
template cudaError_t prepare_tail_kernel<double>();

namespace {

inline dim3 grid2(int m, int n, dim3 blk) { return dim3(ceil_div(m, blk.x), ceil_div(n, blk.y)); }

}  // namespace

int reduction_blocks() { return 4 * 152; }

template <typename T> void top_sweep(hierarchy<T> &h, cudaStream_t st) {
    level_view<T> &L = h.lv[0];
    dim3 blk(32, 8);
    for (int c = 0; c < 2; c++) {
        k_top_color<T><<<grid2((L.m + 1) / 2, L.n, blk), blk, 0, st>>>(h.op, L.z, L.b, L.m, L.n, c);
        note_launch();
    }
}

template <typename T> static void lev_sweep(level_view<T> &L, cudaStream_t st) {
    dim3 blk(32, 8);
    dim3 g(ceil_div((L.m + 1) / 2, blk.x), ceil_div((L.n + 1) / 2, blk.y));
    for (int cy = 0; cy < 2; cy++)
        for (int cx = 0; cx < L.colors_x; cx++) {
            k_lev_color<T><<<g, blk, 0, st>>>(L, cx, cy);
            note_launch();
        }
}


// The pair tail covers levels t .. ml-1 of even width <= 64 with one
// stencil class per row and their tables staged in shared memory.
template <typename T> static bool pair_tail(const hierarchy<T> &h, int t) {
    for (int l = t; l < h.nl - 1; l++) {
        const level_view<T> &L = h.lv[l];
        if ((L.m & 1) || L.m > 64 || !L.homog || tail_stage_bytes<T>(L.nst, L.ncls) > kTailStageMax) return false;
    }
    return true;
}

// Levels wide enough for the single-precision tile kernels (an even periodic
// line that the halo cannot wrap onto itself).
template <typename T> static bool tile_level(const hierarchy<T> &h, const level_view<T> &L) {
    return h.fuse && sizeof(T) == 4 && L.colors_x == 2 && L.m >= kFusedMinWidth;
}

// Levels for the streaming coarse kernels: tile levels with one stencil
// class per row.
template <typename T> static bool march_level(const hierarchy<T> &h, const level_view<T> &L) {
    return h.fuse && sizeof(T) == 4 && L.colors_x == 2 && L.m >= kMarchMinWidth && L.homog &&
           L.nst <= kMarchStencils;
}

#ifndef STZG_TAIL_MARCH_MAX
#define STZG_TAIL_MARCH_MAX 0  // widest streaming level the tail may take instead
#endif

// First level handled by the single-block tail (levels of at most
// tail_points points, plus a direct coarsest solve); ml+1 when there is none.
template <typename T> static int tail_start(const hierarchy<T> &h) {
    const int ml = h.nl - 1;
    if (ml < 1 || !h.bottom_inv) return ml + 1;
    const long limit = h.tail_limit >= 0 ? h.tail_limit : (sizeof(T) == 4 ? 4400 : 300);
    int t = ml;
    // a level the streaming kernels take stays out of the tail (they are faster)
    while (t > 1 && (long)h.lv[t - 1].m * h.lv[t - 1].n <= limit && tail_smem_bytes(h, t - 1) <= kTailSmem &&
           (!march_level(h, h.lv[t - 1]) || h.lv[t - 1].m <= STZG_TAIL_MARCH_MAX))
        t--;
    if (tail_smem_bytes(h, t) > kTailSmem) return ml + 1;
    return t;
}

// Coarse rows per warp of a streaming coarse kernel: the largest of 16, 8
// and 4 that still gives sixteen warps per SM, else 2 (small levels are
// latency-bound: shorter marches finish sooner).
inline int march_rows(int strips, int cn) {
    const long want = 16L * 152;
    for (int t = 16; t >= 4; t >>= 1)
        if ((long)strips * ceil_div(cn, t) >= want) return t;
    return 2;
}

template <typename T> void launch_lev_down_m(level_view<T> &L, level_view<T> &C, cudaStream_t st) {
    if constexpr (sizeof(T) == 4) {
        const int strips = ceil_div(C.m, kLevDownCols);
        const int t = march_rows(strips, C.n);
        const dim3 g(strips, ceil_div(ceil_div(C.n, t), kMarchWarps)), blk(32 * kMarchWarps);
        switch (t) {
            case 16: launch_pdl(k_lev_down_m<16>, g, blk, 0, st, L, C); break;
            case 8: launch_pdl(k_lev_down_m<8>, g, blk, 0, st, L, C); break;
            case 4: launch_pdl(k_lev_down_m<4>, g, blk, 0, st, L, C); break;
            default: launch_pdl(k_lev_down_m<2>, g, blk, 0, st, L, C);
        }
        note_launch();
    }
}

template <typename T> void launch_lev_up_m(level_view<T> &F, level_view<T> &C, cudaStream_t st) {
    if constexpr (sizeof(T) == 4) {
        const int strips = ceil_div(C.m, kLevUpCols);
        const int t = march_rows(strips, C.n);
        const dim3 g(strips, ceil_div(ceil_div(C.n, t), kMarchWarps)), blk(32 * kMarchWarps);
        switch (t) {
            case 16: launch_pdl(k_lev_up_m<16>, g, blk, 0, st, F, C); break;
            case 8: launch_pdl(k_lev_up_m<8>, g, blk, 0, st, F, C); break;
            case 4: launch_pdl(k_lev_up_m<4>, g, blk, 0, st, F, C); break;
            default: launch_pdl(k_lev_up_m<2>, g, blk, 0, st, F, C);
        }
        note_launch();
    }
}

// Coarse tile of a tile-kernel level: the largest of 32x8, 16x4 and 8x4
// coarse points that still gives two blocks per SM; the coarse levels are
// latency-bound, and a smaller tile shortens every phase of a block.
inline int lev_tile(int cm, int cn) {
    const long want = 2L * 152;
    if ((long)ceil_div(cm, 32) * ceil_div(cn, 8) >= want) return 0;
    if ((long)ceil_div(cm, 16) * ceil_div(cn, 4) >= want) return 1;
    return 2;
}

template <typename T> void launch_lev_down(level_view<T> &L, level_view<T> &C, cudaStream_t st) {
    switch (lev_tile(C.m, C.n)) {
        case 0: k_lev_down<T, 32, 8><<<dim3(ceil_div(C.m, 32), ceil_div(C.n, 8)), dim3(32, 8), 0, st>>>(L, C); break;
        case 1: k_lev_down<T, 16, 4><<<dim3(ceil_div(C.m, 16), ceil_div(C.n, 4)), dim3(32, 8), 0, st>>>(L, C); break;
        default: k_lev_down<T, 8, 4><<<dim3(ceil_div(C.m, 8), ceil_div(C.n, 4)), dim3(32, 8), 0, st>>>(L, C);
    }
    note_launch();
}

template <typename T> void launch_lev_up(level_view<T> &F, level_view<T> &C, cudaStream_t st) {
    switch (lev_tile(C.m, C.n)) {
        case 0: k_lev_up<T, 32, 8><<<dim3(ceil_div(C.m, 32), ceil_div(C.n, 8)), dim3(32, 8), 0, st>>>(F, C); break;
        case 1: k_lev_up<T, 16, 4><<<dim3(ceil_div(C.m, 16), ceil_div(C.n, 4)), dim3(32, 8), 0, st>>>(F, C); break;
        default: k_lev_up<T, 8, 4><<<dim3(ceil_div(C.m, 8), ceil_div(C.n, 4)), dim3(32, 8), 0, st>>>(F, C);
    }
    note_launch();
}

// The streaming top-level kernels (single precision only): the swept z goes
// to the level's r array on the way down and back to z on the way up.
template <typename T> void launch_top_down(hierarchy<T> &h, cudaStream_t st, bool zero_start) {
    if constexpr (sizeof(T) == 4) {
        level_view<T> &T0 = h.lv[0], &C = h.lv[1];
        dim3 g(ceil_div(C.m, kDownCols), ceil_div(ceil_div(C.n, kDownRows), kMarchWarps));
        launch_pdl(k_top_down, g, dim3(32 * kMarchWarps), 0, st, h.op,
                   zero_start ? (const float2 *)nullptr : (const float2 *)T0.z, (const float2 *)T0.b,
                   T0.m, T0.n, T0.r, C.b, C.m, C.n);
        note_launch();
    }
}

template <typename T> void launch_top_up(hierarchy<T> &h, cudaStream_t st) {
    if constexpr (sizeof(T) == 4) {
        level_view<T> &T0 = h.lv[0], &C = h.lv[1];
        dim3 g(ceil_div(C.m, kUpCols), ceil_div(ceil_div(C.n, kUpRows), kMarchWarps));
        launch_pdl(k_top_up, g, dim3(32 * kMarchWarps), 0, st, h.op, (const float2 *)T0.r, (const float2 *)T0.b,
                   T0.m, T0.n, (const float2 *)C.z, C.m, C.n, T0.z);
        note_launch();
    }
}

// Shared memory of the pair tail from level t, with the coarsest inverse
// after the levels when it fits (its offset in *inv_off, else -1).
template <typename T> static size_t pair_tail_smem(const hierarchy<T> &h, int t, int *inv_off) {
    size_t smem = tail_smem_bytes(h, t);
    *inv_off = -1;
    const size_t off = (smem + 15) & ~(size_t)15;
    const size_t need = sizeof(double) * (size_t)h.bottom_unknowns * h.bottom_unknowns;
    if (off + need <= kTailSmem) {
        *inv_off = (int)off;
        smem = off + need;
    }
    return smem;
}

// First level of the persistent coarse kernel for a V-cycle whose tail
// starts at t, or 0 where it does not apply: levels p .. t-1 stream and are at
// most kPersistWidth wide, and the tail is a pair tail.
static int persist_start(const hierarchy<float> &h, int t) {
    if (!h.persist || !h.bar || !h.bar_err) return 0;
    const int ml = h.nl - 1;
    if (t > ml || t < 2 || !pair_tail(h, t)) return 0;
    int p = t;
    while (p > 1 && march_level(h, h.lv[p - 1]) && h.lv[p - 1].m <= kPersistWidth) p--;
    return p < t ? p : 0;
}

static int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n < 1) n = 1;
    }
    return n;
}

constexpr size_t kPersistStage = sizeof(float2) * kPersistWarps * (kPersistRows + 3) * 33;

static cudaError_t launch_persist(const coarse_plan &cp, const hierarchy_view<float> &hv, size_t smem,
                                  cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(sm_count());
    cfg.blockDim = dim3(32, kPersistWarps);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_coarse_persist, cp, hv);
}

static void coarse_persist(hierarchy<float> &h, int p, int t, cudaStream_t st) {
    hierarchy_view<float> hv;
    for (int l = 0; l < h.nl; l++) hv.lv[l] = h.lv[l];
    coarse_plan cp;
    cp.p = p;
    cp.t = t;
    cp.tl = tail_levels{t, h.nl - 1, h.bottom_inv, h.bottom_unknowns, -1};
    size_t smem = pair_tail_smem(h, t, &cp.tl.inv_off);
    if (smem < kPersistStage) smem = kPersistStage;
    cp.bar = h.bar;
    cp.err = h.bar_err;
    launch_persist(cp, hv, smem, st);
    note_launch();
}

__global__ void k_probe_stop(cudaGraphConditionalHandle h) { cudaGraphSetConditional(h, 0); }

bool coarse_persist_supported() {
    static signed char state[64];
    static bool init = false;
    if (!init) {
        for (auto &x : state) x = -1;
        init = true;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    if (state[dev] >= 0) return state[dev] == 1;
    state[dev] = 0;
    int coop = 0, nb = 0;
    const size_t smem = kTailSmem + 1024;
    bool ok = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess && coop &&
              cudaFuncSetAttribute(k_coarse_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
                  cudaSuccess &&
              cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_coarse_persist, 32 * kPersistWarps, smem) ==
                  cudaSuccess &&
              nb >= 1;
    // one empty launch inside a WHILE body that runs once
    cudaStream_t st = nullptr;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    if (ok) ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) ok = cudaGraphCreate(&g, 0) == cudaSuccess;
    cudaGraphConditionalHandle hc;
    if (ok) ok = cudaGraphConditionalHandleCreate(&hc, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    cudaGraphNodeParams wp = {};
    cudaGraphNode_t wnode;
    if (ok) {
        wp.type = cudaGraphNodeTypeConditional;
        wp.conditional.handle = hc;
        wp.conditional.type = cudaGraphCondTypeWhile;
        wp.conditional.size = 1;
        ok = cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp) == cudaSuccess;
    }
    if (ok) {
        ok = cudaStreamBeginCaptureToGraph(st, wp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            coarse_plan cp = {};
            cp.p = 1;
            cp.t = 0;  // empty
            cp.tl.inv_off = -1;
            hierarchy_view<float> hv = {};
            bool launched = launch_persist(cp, hv, smem, st) == cudaSuccess;
            k_probe_stop<<<1, 1, 0, st>>>(hc);
            cudaGraph_t got = nullptr;
            ok = cudaStreamEndCapture(st, &got) == cudaSuccess && launched;
        }
    }
    if (ok) ok = cudaGraphInstantiate(&ex, g, 0) == cudaSuccess;
    if (ok) ok = cudaGraphLaunch(ex, st) == cudaSuccess && cudaStreamSynchronize(st) == cudaSuccess;
    if (ex) cudaGraphExecDestroy(ex);
    if (g) cudaGraphDestroy(g);
    if (st) cudaStreamDestroy(st);
    cudaGetLastError();  // a refused form leaves a non-sticky error behind
    state[dev] = ok ? 1 : 0;
    return ok;
}

bool coarse_persist_active(const hierarchy<float> &h) { return persist_start(h, tail_start(h)) > 0; }

template <typename T> void vcycle(hierarchy<T> &h, cudaStream_t st, int bottom_sweeps, int bottom_fp64, bool zero_start) {
    typedef typename vec2_t<T>::type V;
    dim3 blk(32, 8);
    const int ml = h.nl - 1;
    level_view<T> &T0 = h.lv[0];
    const bool fused = h.fuse && sizeof(T) == 4 && ml > 0 && T0.colors_x == 2 && T0.m >= kFusedMinWidth;
    if (ml == 0) {
        top_sweep(h, st);
        top_sweep(h, st);
        return;
    }
    const int t = tail_start(h);
    if (zero_start && !fused) cudaMemsetAsync(T0.z, 0, sizeof(V) * (size_t)T0.m * T0.n, st);
    if (fused) {
        launch_top_down(h, st, zero_start);
    } else {
        top_sweep(h, st);
        k_top_residual<T><<<grid2(T0.m, T0.n, blk), blk, 0, st>>>(h.op, T0.z, T0.b, T0.r, T0.m, T0.n);
        note_launch();
        k_restrict<T><<<grid2(h.lv[1].m, h.lv[1].n, blk), blk, 0, st>>>(T0.r, T0.m, T0.n, h.lv[1].b, h.lv[1].m,
                                                                       h.lv[1].n);
        note_launch();
    }
    int p = 0;  // first level of the persistent coarse kernel (0: none)
    if constexpr (sizeof(T) == 4) p = persist_start(h, t);
    // levels [1, down_end) go down outside the tail (and the persistent kernel)
    const int down_end = p ? p : (t <= ml ? t : ml);
    for (int i = 1; i < down_end; i++) {
        level_view<T> &L = h.lv[i];
        level_view<T> &C = h.lv[i + 1];
        if (march_level(h, L)) {
            launch_lev_down_m(L, C, st);
            continue;
        }
        if (tile_level(h, L)) {
            launch_lev_down(L, C, st);
            continue;
        }
        cudaMemsetAsync(L.z, 0, sizeof(V) * (size_t)L.m * L.n, st);
        lev_sweep(L, st);
        k_lev_residual<T><<<grid2(L.m, L.n, blk), blk, 0, st>>>(L);
        note_launch();
        k_restrict<T><<<grid2(C.m, C.n, blk), blk, 0, st>>>(L.r, L.m, L.n, C.b, C.m, C.n);
        note_launch();
    }
    int up_from;
    if (p) {
        if constexpr (sizeof(T) == 4) coarse_persist(h, p, t, st);
        up_from = p;
    } else if (t <= ml) {
        hierarchy_view<T> hv;
        for (int l = 0; l < h.nl; l++) hv.lv[l] = h.lv[l];
        tail_levels tl{t, ml, h.bottom_inv, h.bottom_unknowns, -1};
        size_t smem = tail_smem_bytes(h, t);
        // room for a copy of the coarsest inverse after the levels
        if (sizeof(T) == 4 && pair_tail(h, t)) smem = pair_tail_smem(h, t, &tl.inv_off);
        if constexpr (sizeof(T) == 4) {
            if (pair_tail(h, t))
                launch_pdl(k_tail_pairs, dim3(1), dim3(32, STZG_TAIL_WARPS), smem, st, tl, hv);
            else
                k_tail<T><<<1, dim3(32, 32), smem, st>>>(tl, hv);
        } else {
            k_tail<T><<<1, dim3(32, 32), smem, st>>>(tl, hv);
        }
        note_launch();
        up_from = t;
    } else {
        level_view<T> &B = h.lv[ml];
        if (h.bottom_inv)
            k_bottom_direct<T><<<1, 256, sizeof(double) * h.bottom_unknowns, st>>>(B, h.bottom_inv,
                                                                                  h.bottom_unknowns);
        else if (bottom_fp64)
            k_bottom<T, double><<<1, 256, 0, st>>>(B, bottom_sweeps, bottom_sweeps);
        else
            k_bottom<T, T><<<1, 256, 0, st>>>(B, bottom_sweeps, bottom_sweeps);
        note_launch();
        up_from = ml;
    }
    for (int i = up_from; i >= 2; i--) {
        level_view<T> &C = h.lv[i], &F = h.lv[i - 1];
        if (march_level(h, F)) {
            launch_lev_up_m(F, C, st);
            continue;
        }
        if (tile_level(h, F)) {
            launch_lev_up(F, C, st);
            continue;
        }
        k_prolong_add<T><<<grid2(F.m, F.n, blk), blk, 0, st>>>(C.z, C.m, C.n, F.z, F.m, F.n);
        note_launch();
        lev_sweep(F, st);
    }
    if (fused) {
        launch_top_up(h, st);
    } else {
        k_prolong_add<T><<<grid2(T0.m, T0.n, blk), blk, 0, st>>>(h.lv[1].z, h.lv[1].m, h.lv[1].n, T0.z, T0.m,
                                                                 T0.n);
        note_launch();
        top_sweep(h, st);
    }
}

template <typename T>
void top_residual_sqnorm(hierarchy<T> &h, double *partials, int npart, double *out, double *out_b,
                         cudaStream_t st) {
    level_view<T> &L = h.lv[0];
    k_top_sqnorm<T><<<npart, kRedThreads, 0, st>>>(h.op, L.z, L.b, L.m, L.n, partials); note_launch();
    k_final_sum<<<1, 256, 0, st>>>(partials, npart, out, out_b); note_launch();
}

void mixed_residual(const top_op<double> &op64, const double2 *z64, const double2 *b64, int m, int n, float2 *r32,
                    double *partials, int npart, double *out, double *out_b, cudaStream_t st) {
    k_mixed_residual<<<npart, kRedThreads, 0, st>>>(op64, z64, b64, m, n, r32, partials); note_launch();
    k_final_sum<<<1, 256, 0, st>>>(partials, npart, out, out_b); note_launch();
}

static ff ff_of(double d) {
    const float hi = (float)d;
    return ff{hi, (float)(d - (double)hi)};
}

void ff_split(const double2 *a, float2 *hi, float2 *lo, const double2 *a2, float2 *hi2, float2 *lo2, long count,
              cudaStream_t st) {
    k_ff_split<<<4 * 152, 256, 0, st>>>(a, hi, lo, a2, hi2, lo2, count); note_launch();
}

void extrap_split(const double2 *v, double2 *prev, const double2 *b, float2 *hi, float2 *lo, float2 *bhi,
                  float2 *blo, long count, cudaStream_t st) {
    k_extrap_split<<<4 * 152, 256, 0, st>>>(v, prev, b, hi, lo, bhi, blo, count); note_launch();
}

void ff_merge(const float2 *hi, const float2 *lo, double2 *a, long count, cudaStream_t st) {
    k_ff_merge<<<4 * 152, 256, 0, st>>>(hi, lo, a, count); note_launch();
}

void ff_correct(float2 *hi, float2 *lo, const float2 *e32, long count, cudaStream_t st) {
    k_ff_correct<<<4 * 152, 256, 0, st>>>(hi, lo, e32, count); note_launch();
}

void ff_correct_merge(const float2 *hi, const float2 *lo, const float2 *e32, double2 *a, long count, cudaStream_t st) {
    k_ff_correct_merge<<<4 * 152, 256, 0, st>>>(hi, lo, e32, a, count); note_launch();
}

void ff_residual(const top_op<double> &o, const float2 *zhi, const float2 *zlo, const float2 *bhi, const float2 *blo,
                 int m, int n, float2 *r32, double *partials, int npart, double *out, double *out_b, cudaStream_t st) {
    ff_op f;
    f.Kmx = ff_of(o.Kmx); f.Kmy = ff_of(o.Kmy); f.mx = ff_of(o.mx); f.my = ff_of(o.my); f.qK = ff_of(o.qK);
    f.bcxx = ff_of(o.bcxx); f.bcyy = ff_of(o.bcyy);
    f.dxx = ff_of(o.cxx + 2 * (o.Kmx + o.my));
    f.dyy = ff_of(o.cyy + 2 * (o.mx + o.Kmy));
    k_ff_residual<<<npart, kRedThreads, 0, st>>>(f, zhi, zlo, bhi, blo, m, n, r32, partials); note_launch();
    k_final_sum<<<1, 256, 0, st>>>(partials, npart, out, out_b); note_launch();
}

void mixed_correct(double2 *z64, const float2 *e32, long count, cudaStream_t st) {
    k_mixed_correct<<<4 * 152, 256, 0, st>>>(z64, e32, count); note_launch();
}

void extrapolate_guess2(double2 *z, double2 *prev, double2 *prev2, long count, cudaStream_t st) {
    k_extrapolate2<<<4 * 152, 256, 0, st>>>(z, prev, prev2, count); note_launch();
}

void extrapolate_guess(double2 *z, double2 *prev, long count, cudaStream_t st) {
    k_extrapolate<<<4 * 152, 256, 0, st>>>(z, prev, count); note_launch();
}

bool top_level_kernel(hierarchy<float> &h, int which, cudaStream_t st) {
    const level_view<float> &T0 = h.lv[0];
    if (!(h.fuse && h.nl > 1 && T0.colors_x == 2 && T0.m >= kFusedMinWidth)) return false;
    if (which == 0)
        launch_top_down(h, st, false);
    else
        launch_top_up(h, st);
    return true;
}

template void vcycle<double>(hierarchy<double> &, cudaStream_t, int, int, bool);
template void vcycle<float>(hierarchy<float> &, cudaStream_t, int, int, bool);
template void top_sweep<double>(hierarchy<double> &, cudaStream_t);
template void top_sweep<float>(hierarchy<float> &, cudaStream_t);
template void top_residual_sqnorm<double>(hierarchy<double> &, double *, int, double *, double *, cudaStream_t);
template void top_residual_sqnorm<float>(hierarchy<float> &, double *, int, double *, double *, cudaStream_t);

}  // namespace stzg
