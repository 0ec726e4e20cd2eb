// Shared device/host helpers of the STZ step library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "stzg.h"

namespace stzg {

// Records a message for stzg_last_message() and returns the status.
int fail(int status, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define STZG_CUDA(call)                                          \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return ::stzg::cuda_fail(e_, #call); \
    } while (0)

#define STZG_CHECK(status_expr)          \
    do {                                 \
        int st_ = (status_expr);         \
        if (st_ != STZG_OK) return st_;  \
    } while (0)

// Two-component vector of the node grid (the reference's vec, vec.hh:6-49).
template <typename T> struct vec2_t;
template <> struct vec2_t<double> { typedef double2 type; };
template <> struct vec2_t<float> { typedef float2 type; };

// 2x2 block (the reference's mat, mat.hh:12-83), row-major (a b; c d).
template <typename T> struct alignas(sizeof(T) * 4) mat2 {
    T a, b, c, d;
};

// Coarse stencil of one point class: dl dc dr cl cc cr ul uc ur, inverse(cc)
// (tgmg_level::s layout, tgmg.hh:235, 256-265).
template <typename T> struct stencil9 {
    mat2<T> e[10];
};

__host__ __device__ inline int wrap_left(int i, int m) { return i == 0 ? m - 1 : i - 1; }
__host__ __device__ inline int wrap_right(int i, int m) { return i == m - 1 ? 0 : i + 1; }

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

// Kernel launches issued by this library (host counter; launches recorded
// while a stream is being captured belong to the captured graph).
void note_launch();
long launch_count();
// Removes launches that were recorded while capturing a graph.
void discount_launches(long k);

// Device-wide numbers used for grid sizing.
struct device_info {
    int sm_count;
    int cc_major, cc_minor;
};

}  // namespace stzg
