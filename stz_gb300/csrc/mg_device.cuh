// Device helpers shared by the multigrid kernels and the no-allocation
// residual-norm entry point.
#pragma once

#include "mg.cuh"

namespace stzg {

// Residual of the top level: r = b - A z (qs_multi::mul_a + a_cc).
template <typename T, typename V>
__device__ __forceinline__ V top_res(const top_op<T> &op, const V *__restrict__ z, const V *__restrict__ b, int m, int n,
                            int i, int j) {
    const size_t ij = (size_t)j * m + i;
    V r;
    if (j == 0 || j == n - 1) {
        r.x = b[ij].x - op.bcxx * z[ij].x;
        r.y = b[ij].y - op.bcyy * z[ij].y;
        return r;
    }
    const int il = i == 0 ? m - 1 : i - 1, ir = i == m - 1 ? 0 : i + 1;
    const V *zd = z + (size_t)(j - 1) * m, *zc = z + (size_t)j * m, *zu = z + (size_t)(j + 1) * m;
    T ax = op.Kmx * (zc[il].x + zc[ir].x) + op.my * (zd[i].x + zu[i].x) +
           op.qK * (zd[il].y + zu[ir].y - zd[ir].y - zu[il].y);
    T ay = op.mx * (zc[il].y + zc[ir].y) + op.Kmy * (zd[i].y + zu[i].y) +
           op.qK * (zd[il].x + zu[ir].x - zd[ir].x - zu[il].x);
    r.x = b[ij].x - ax - op.cxx * zc[i].x;
    r.y = b[ij].y - ay - op.cyy * zc[i].y;
    return r;
}

// Deterministic block reduction of a double (warp shuffles, fixed order).
__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;
}

}  // namespace stzg
