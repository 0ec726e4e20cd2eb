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
