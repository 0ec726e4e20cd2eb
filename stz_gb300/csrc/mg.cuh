// Geometric multigrid for the quasi-static elasticity system on one GPU.
//
// Restates the tgmg V-cycle the reference runs through qs_multi
// (esim/tgmg/tgmg.hh:42-495, tgmg.in.cc:11-856, esim/sb/main/qs_multi.{hh,cc})
// with a GB300 layout:
//   * the top level is matrix-free: the qs_multi 9-point 2x2-block operator
//     is rebuilt from eight constants (qs_multi.hh:41-50);
//   * coarse Galerkin operators (tgmg_base::rat, tgmg.in.cc:667-736) are kept
//     as a small table of distinct stencils plus a class index per row (rows
//     of an x-periodic level with uniform coarsening share one stencil), or
//     per point where the level is not x-homogeneous;
//   * Gauss-Seidel is multi-colour instead of zebra-lexicographic
//     (tgmg.in.cc:128-165): two colours on the top level, where x couples to
//     x on edge neighbours and to y on corners only, so {x at even i+j, y at
//     odd i+j} is an independent set; four colours ((i&1),(j&1)) on coarse
//     levels, six where a periodic line is odd;
//   * every level stores z, b and a residual buffer r in one precision T.
#pragma once

#include <vector>

#include "common.cuh"

namespace stzg {

// Constants of the qs_multi operator for one viscosity/dt (qs_multi::init,
// qs_multi.cc:31-55), in the precision the kernels use.
template <typename T> struct top_op {
    T Kmx, Kmy, mx, my, qK;
    T cxx, cyy;           // diagonal of interior rows (regc)
    T icxx, icyy;         // regci = (1/cxx, 1/cyy)
    T bcxx, bcyy;         // wall rows: regcb = bcs*regc
    T ibcxx, ibcyy;       // regcbi = (1/(bcs*cxx), 1/(bcs*cyy))
};

// One level as the kernels see it.
template <typename T> struct level_view {
    typedef typename vec2_t<T>::type V;
    int m, n;             // nodes: x (periodic), y
    int homog;            // 1: stencil class per row, 0: per point
    int colors_x;         // 2, or 3 where m is odd
    const int *cls;       // class index per row or per point (coarse levels)
    const stencil9<T> *st;// stencil table (coarse levels)
    V *z, *b, *r;
    int nst, ncls;        // entries of st and cls
};

// All levels by value, for kernels that walk several levels.
template <typename T> struct hierarchy_view {
    level_view<T> lv[17];
};

// Host copy of a coarse level's operator.
struct level_ops {
    int m, n;
    bool homog;
    std::vector<int> cls;
    std::vector<stencil9<double>> table;
};

// Dense inverse of the coarsest operator (2mn x 2mn, row-major, unknown
// 2*(j*m+i)+c); empty when the level is too large for a direct solve.
std::vector<double> coarsest_inverse(const level_ops &L);

// Builds the qs_multi constants for viscdt = viscosity/dt.
struct qs_constants {
    double Kq, qK, Kmu, mu, xsp2, ysp2, xyfac, tmufac1, tmufac2, bcs;
    double Kmx, Kmy, mx, my, cxx, cyy;
    void init(const stz_params &p, double viscdt);
    double reference_acc(double mult) const;  // tgmg_accuracy(2(tmufac1+tmufac2), mult)
    template <typename T> top_op<T> op() const;
};

// Coarse hierarchy sizes (tgmg.in.cc:17-29): returns (m,n) per coarse level.
std::vector<std::pair<int, int>> coarse_sizes(int m, int n);

// Galerkin products for the whole hierarchy below the top operator.
std::vector<level_ops> build_coarse_ops(const qs_constants &q, int m, int n);

// Device hierarchy in precision T.
template <typename T> class hierarchy {
  public:
    typedef typename vec2_t<T>::type V;
    int nl = 0;                         // levels including the top
    level_view<T> lv[17];
    top_op<T> op;
    // allocation: top z/b may be external (FP64 path uses vel/src directly)
    int allocate(int m, int n, V *top_z, V *top_b);
    int upload_ops(const std::vector<level_ops> &ops, const top_op<double> &op64);
    // exact coarsest solve z = A^-1 b in FP64 (nullptr: Gauss-Seidel sweeps)
    const double *bottom_inv = nullptr;
    int bottom_unknowns = 0;
    // schedule knobs (autotuned per grid size for batches): largest level
    // (points) handled by the single-block tail (<0: default by precision),
    // and whether wide single-precision levels use the fused tile kernels
    long tail_limit = -1;
    int fuse = 1;
    // single precision: the coarse levels at most 512 wide and the tail in
    // one cooperative persistent kernel (set by the owner once
    // coarse_persist_supported() holds; bar: two zeroed device words for its
    // grid barrier, bar_err: a device word it sets when a barrier wait runs
    // out).  Off for hierarchies whose V-cycles may run concurrently with
    // other kernels (batched graphs).
    int persist = 0;
    unsigned *bar = nullptr;
    int *bar_err = nullptr;
    void release();
    ~hierarchy() { release(); }
    size_t device_bytes() const { return bytes_; }
  private:
    std::vector<void *> owned_;
    size_t bytes_ = 0;
    size_t st_cap_[17] = {0}, cls_cap_[17] = {0}, inv_cap_ = 0;
    int grow(int l, size_t st_need, size_t cls_need);
    double *inv_dev_ = nullptr;
};

// Kernel-level building blocks (mg.cu).
// zero_start: the top-level z is taken as zero (the first cycle of a pass);
// the V-cycle then clears it itself or never reads it.
template <typename T>
void vcycle(hierarchy<T> &h, cudaStream_t st, int bottom_sweeps, int bottom_fp64, bool zero_start = false);
template <typename T> void top_sweep(hierarchy<T> &h, cudaStream_t st);
// One launch of the streaming top-level kernel down (0) or up (1) of the FP32
// V-cycle, for timing; false where the top level does not use them.
bool top_level_kernel(hierarchy<float> &h, int which, cudaStream_t st);
// Whether this device takes the persistent coarse kernel: cooperative
// launches, one block per SM with the tail's shared memory, and a launch
// inside a conditional (WHILE) graph body, tried once per process on a
// private stream with an empty plan.  Call outside any stream capture.
bool coarse_persist_supported();
// Whether a V-cycle of h would use the persistent coarse kernel.
bool coarse_persist_active(const hierarchy<float> &h);

// Sum of squared residuals of the top level into *out (device), optional
// sum of squared b into *out_b.  Deterministic: fixed grid, ordered final sum.
template <typename T>
void top_residual_sqnorm(hierarchy<T> &h, double *partials, int npart, double *out, double *out_b,
                         cudaStream_t st);

// Mixed precision: r32 = b64 - A64 z64 (FP64 arithmetic) stored in h32's top
// b, with squared norms of r and b accumulated like top_residual_sqnorm.
void mixed_residual(const top_op<double> &op64, const double2 *z64, const double2 *b64, int m, int n,
                    float2 *r32, double *partials, int npart, double *out, double *out_b, cudaStream_t st);
// z64 += e32
void mixed_correct(double2 *z64, const float2 *e32, long count, cudaStream_t st);
// Float-float iterates (hi + lo pairs of FP32 vectors) of the mixed solve:
// split FP64 vectors (a, and a2 unless null), merge back, add an FP32
// correction, and the residual r32 = b - A z in float-float arithmetic with
// squared norms like top_residual_sqnorm.
void ff_split(const double2 *a, float2 *hi, float2 *lo, const double2 *a2, float2 *hi2, float2 *lo2, long count,
              cudaStream_t st);
void ff_merge(const float2 *hi, const float2 *lo, double2 *a, long count, cudaStream_t st);
void ff_correct(float2 *hi, float2 *lo, const float2 *e32, long count, cudaStream_t st);
// prev = v; (hi, lo) = split(2 v - prev_old); (bhi, blo) = split(b)
void extrap_split(const double2 *v, double2 *prev, const double2 *b, float2 *hi, float2 *lo, float2 *bhi,
                  float2 *blo, long count, cudaStream_t st);
// a = (hi, lo) + e32 as doubles (the last correction and the merge in one pass)
void ff_correct_merge(const float2 *hi, const float2 *lo, const float2 *e32, double2 *a, long count, cudaStream_t st);
void ff_residual(const top_op<double> &op64, const float2 *zhi, const float2 *zlo, const float2 *bhi,
                 const float2 *blo, int m, int n, float2 *r32, double *partials, int npart, double *out,
                 double *out_b, cudaStream_t st);
// Linear extrapolation of the initial guess: z <- 2 z - prev, prev <- old z.
void extrapolate_guess(double2 *z, double2 *prev, long count, cudaStream_t st);
// Quadratic: z <- 3 z - 3 prev + prev2, prev2 <- prev, prev <- old z.
void extrapolate_guess2(double2 *z, double2 *prev, double2 *prev2, long count, cudaStream_t st);

int reduction_blocks();

}  // namespace stzg
