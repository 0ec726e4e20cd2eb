// Host conversions between the reference's own state layout, an array of
// c_field records (esim/sb/main/fields.hh:7-114: 19 doubles per point, u, v,
// p, q, s, tau, chi, X, Y, ddev first, then the update scratch), and the
// per-field buffers of stzg_upload / stzg_download.  The reference keeps
// cell and node values of point (i, j) in one record at index (j + 1) * m + i
// of the array that starts at shear_sim::fm - m (rows -1..n; cell fields on
// all rows, node fields on rows 0..n); the solver's velocity array vel holds
// u, v of the nodes.  Rows are converted in parallel (OpenMP).
#include <cstddef>

#include "stzg.h"

namespace {

constexpr int kRecord = 19;  // doubles per c_field
enum { R_U = 0, R_V, R_P, R_Q, R_S, R_TAU, R_CHI, R_X, R_Y, R_DDEV };

}  // namespace

extern "C" {

int stzg_c_field_pack(const void *fm_rows, int m, int n, double *const *soa) {
    if (!fm_rows || !soa || m < 1 || n < 1) return STZG_EINVAL;
    const double *rec = static_cast<const double *>(fm_rows);
    const int cell_mem[5] = {R_P, R_Q, R_S, R_TAU, R_CHI};
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n + 2; r++) {
        for (int i = 0; i < m; i++) {
            const size_t k = (size_t)r * m + i;
            const double *f = rec + k * kRecord;
            for (int q = 0; q < 5; q++)
                if (soa[q]) soa[q][k] = f[cell_mem[q]];
            if (r == 0) continue;  // row -1 holds no node values
            const size_t nd = (size_t)(r - 1) * m + i;
            if (soa[5]) soa[5][nd] = f[R_X];
            if (soa[6]) soa[6][nd] = f[R_Y];
            if (soa[7]) {
                soa[7][2 * nd] = f[R_U];
                soa[7][2 * nd + 1] = f[R_V];
            }
        }
    }
    return STZG_OK;
}

int stzg_c_field_unpack(const double *const *soa, int m, int n, void *fm_rows) {
    if (!fm_rows || !soa || m < 1 || n < 1) return STZG_EINVAL;
    double *rec = static_cast<double *>(fm_rows);
    const int cell_mem[5] = {R_P, R_Q, R_S, R_TAU, R_CHI};
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n + 2; r++) {
        for (int i = 0; i < m; i++) {
            const size_t k = (size_t)r * m + i;
            double *f = rec + k * kRecord;
            for (int q = 0; q < 5; q++)
                if (soa[q]) f[cell_mem[q]] = soa[q][k];
            if (r == 0) continue;  // node rows 0..n are storage rows 1..n+1
            const size_t nd = (size_t)(r - 1) * m + i;
            if (soa[5]) f[R_X] = soa[5][nd];
            if (soa[6]) f[R_Y] = soa[6][nd];
            if (soa[7]) {
                f[R_U] = soa[7][2 * nd];
                f[R_V] = soa[7][2 * nd + 1];
            }
        }
    }
    return STZG_OK;
}

}  // extern "C"
