// Seeded Gaussian random chi field (host, set-up only).
//
// Semantics of shear_sim::initialize_random (esim/sb/main/shear_sim.cc:932-984):
// white noise on a grid padded by cut=int(5 l) rows above and below, periodic
// in x, smoothed by the truncated kernel exp(-r^2/(2 l^2)) over |di|,|dj|<=cut,
// scaled by tem_std / (gaussian_normal_factor * TZ) (shear_sim.cc:915-925) and
// offset by tem_avg/TZ.  The reference draws the noise from libc rand(); here
// every noise point draws from its own splitmix64 stream keyed by (seed,
// index), so the field does not depend on thread count or platform, and the
// 2D kernel is applied as two 1D passes (it is separable).
#include <cmath>
#include <cstdint>
#include <vector>

#include "stzg.h"

namespace {

inline uint64_t splitmix(uint64_t &st) {
    uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

inline double uniform01(uint64_t &st) { return (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0); }

// Polar Box-Muller as shear_sim::box_muller (shear_sim.cc:988-998).
double normal_at(uint64_t seed, uint64_t idx) {
    uint64_t st = seed * 0xD1342543DE82EF95ULL + idx * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;
    double x, y, r;
    do {
        x = 2 * uniform01(st) - 1;
        y = 2 * uniform01(st) - 1;
        r = x * x + y * y;
    } while (r == 0.0 || r > 1.0);
    return x * std::sqrt(-2.0 * std::log(r) / r);
}

}  // namespace

extern "C" int stzg_random_chi(int m, int n, double l, double tem_avg, double tem_std, double TZ,
                               unsigned long long seed, double *chi) {
    if (m < 1 || n < 1 || !(l > 0) || !chi || !(TZ > 0)) return STZG_EINVAL;
    const int cut = (int)(l * 5.), rows = n + 2 * cut;
    const double llinv = 0.5 / (l * l);
    double vfac = 1;  // gaussian_normal_factor
    for (int j = 1; j < cut; j++) {
        double q = std::exp(-j * j * llinv);
        for (int k = 0; k <= j; k++) {
            double q2 = q * std::exp(-k * k * llinv);
            vfac += (k == 0 || k == j ? 4 : 8) * q2 * q2;
        }
    }
    const double chi0 = tem_avg / TZ, chi1 = tem_std / (std::sqrt(vfac) * TZ);
    std::vector<double> g(2 * cut + 1);
    for (int d = -cut; d <= cut; d++) g[d + cut] = std::exp(-llinv * d * d);
    std::vector<double> noise((size_t)m * rows), tmp((size_t)m * rows);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < rows; r++)
        for (int i = 0; i < m; i++) noise[(size_t)r * m + i] = normal_at(seed, (uint64_t)r * m + i);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < rows; r++)
        for (int i = 0; i < m; i++) {
            double a = 0;
            for (int d = -cut; d <= cut; d++) {
                int ii = ((i + d) % m + m) % m;
                a += noise[(size_t)r * m + ii] * g[d + cut];
            }
            tmp[(size_t)r * m + i] = a;
        }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            double a = 0;
            for (int d = -cut; d <= cut; d++) a += tmp[(size_t)(j + cut + d) * m + i] * g[d + cut];
            chi[(size_t)j * m + i] = chi0 + a * chi1;
        }
    return STZG_OK;
}

namespace stzg {

// chi of shear_sim::init_fields (esim/sb/main/shear_sim.cc:60-114) at the
// cell centres of rows -1..n (m*(n+2), row j at offset (j+1)m): case 0 a
// Gaussian blip at the origin, case 1 a line rotated by 30 degrees (wrapped
// back into |x_r| <= 1), any other case sixteen blips on a sine wave (the
// nearest one, x-periodic); each of width exp(-200 r^2) over tem_base.
void init_fields_chi(const stz_params &p, int chi_case, double tem_base, double tem_delta, double *chi) {
    const double pi = 3.1415926535897932384626433832795;
    const int m = p.m, n = p.n;
    const double lx = p.bx - p.ax, dx = lx / m, dy = (p.by - p.ay) / n;
    const double c0 = tem_base / p.TZ, c1 = tem_delta / p.TZ;
    double bx_[16], by_[16];
    for (int k = 0; k < 16; k++) {
        bx_[k] = p.ax + lx * (k + 0.5) * 0.0625;
        by_[k] = -0.2 * std::sin(pi * 0.0625 * (2 * k + 1));
    }
    const double ca = std::cos(30 * pi / 180.), sa = std::sin(30 * pi / 180.);
#pragma omp parallel for schedule(static)
    for (int j = -1; j <= n; j++) {
        const double yc = (p.ay + j * dy) + 0.5 * dy;
        for (int i = 0; i < m; i++) {
            const double xc = (p.ax + i * dx) + 0.5 * dx;
            double r2;
            if (chi_case == 0) {
                r2 = xc * xc + yc * yc;
            } else if (chi_case == 1) {
                double u = ca * xc + sa * yc;
                const double w = -sa * xc + ca * yc;
                u = u < -1 ? u + 1 : (u > 1 ? u - 1 : 0);
                r2 = u * u + w * w;
            } else {
                r2 = 1e100;
                for (int k = 0; k < 16; k++) {
                    double u = bx_[k] - xc;
                    if (u < -lx * 0.5) u += lx;
                    if (u > lx * 0.5) u -= lx;
                    const double w = by_[k] - yc, t = u * u + w * w;
                    if (t < r2) r2 = t;
                }
            }
            chi[(size_t)(j + 1) * m + i] = c0 + c1 * std::exp(-200 * r2);
        }
    }
}

// chi of shear_sim::initialize_chi_bicubic (shear_sim.cc:832-909) on rows
// 0..n-1 (m*n): lo + sca times the bicubic Hermite interpolant of arr
// (mm x nn samples spanning the domain, periodic in x) whose derivatives are
// centred differences (one-sided on the first and last sample rows).
void bicubic_chi(const stz_params &p, int mm, int nn, const double *arr, double lo, double sca, double *chi) {
    const int m = p.m, n = p.n;
    const size_t cnt = (size_t)mm * nn;
    std::vector<double> dxa(cnt), dya(cnt), dxya(cnt);
    for (int j = 0; j < nn; j++)
        for (int i = 0; i < mm; i++) {
            const size_t c = (size_t)j * mm;
            dxa[c + i] = 0.5 * (arr[c + (i == mm - 1 ? 0 : i + 1)] - arr[c + (i == 0 ? mm - 1 : i - 1)]);
        }
    for (int j = 0; j < nn; j++)
        for (int i = 0; i < mm; i++) {
            const size_t c = (size_t)j * mm + i;
            if (j == 0) {
                dya[c] = arr[c + mm] - arr[c];
                dxya[c] = dxa[c + mm] - dxa[c];
            } else if (j == nn - 1) {
                dya[c] = arr[c] - arr[c - mm];
                dxya[c] = dxa[c] - dxa[c - mm];
            } else {
                dya[c] = 0.5 * (arr[c + mm] - arr[c - mm]);
                dxya[c] = 0.5 * (dxa[c + mm] - dxa[c - mm]);
            }
        }
    const double dx = (p.bx - p.ax) / m, dy = (p.by - p.ay) / n;
    const double xs = dx * mm / (p.bx - p.ax), ys = dy * nn / (p.by - p.ay);
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; j++) {
        double t = (j + 0.5) * ys - 0.5;
        int jj = (int)t;
        jj = jj < 0 ? 0 : (jj > nn - 2 ? nn - 2 : jj);
        t -= jj;
        const double u = 1 - t;
        // Hermite weights: slope at 0, value at 0, value at 1, slope at 1
        const double w0 = t * u * u, w1 = u * u * (1 + 2 * t), w2 = t * t * (3 - 2 * t), w3 = -t * t * u;
        for (int i = 0; i < m; i++) {
            double s = (i + 0.5) * xs - 0.5;
            if (s < 0) s += mm;
            int ii = (int)s;
            if (ii >= mm) ii -= mm;
            const size_t a = (size_t)jj * mm + ii, b = (size_t)jj * mm + (ii == mm - 1 ? 0 : ii + 1);
            s -= ii;
            const double v = 1 - s;
            const double h0 = s * v * v, h1 = v * v * (1 + 2 * s), h2 = s * s * (3 - 2 * s), h3 = -s * s * v;
            const double r0 = dxya[a] * h0 + dya[a] * h1 + dya[b] * h2 + dxya[b] * h3;
            const double r1 = dxa[a] * h0 + arr[a] * h1 + arr[b] * h2 + dxa[b] * h3;
            const double r2 = dxa[a + mm] * h0 + arr[a + mm] * h1 + arr[b + mm] * h2 + dxa[b + mm] * h3;
            const double r3 = dxya[a + mm] * h0 + dya[a + mm] * h1 + dya[b + mm] * h2 + dxya[b + mm] * h3;
            chi[(size_t)j * m + i] = lo + sca * (w0 * r0 + w1 * r1 + w2 * r2 + w3 * r3);
        }
    }
}

}  // namespace stzg
