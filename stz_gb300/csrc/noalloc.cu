// Residual norms of the quasi-static system on caller-owned device arrays,
// without allocating device memory.
//
// Some callers cannot let a library call cudaMalloc: applications whose own
// caching allocator owns all device memory (a second allocator fragments it
// and can fail where theirs would not), services that run under a fixed
// device-memory budget, and host threads that must not stall the GPU (the
// first cudaMalloc on a context, and cudaFree, synchronize the device).
// stzg_residual_norms_noalloc serves them: the per-block partial sums of the
// reduction live in a fixed array in this library's static device memory, so
// a call only launches two kernels on the caller's stream.
//
// The static array is kNoallocMaxBlocks x 2 doubles (128 KiB).  Every GPU on
// which the library is loaded holds it until the process exits.  One block
// covers kNodesPerBlock nodes, so the largest grid is
// kNoallocMaxBlocks * kNodesPerBlock = 8,388,608 nodes (for example
// 2896 x 2896 cells); larger grids are rejected with STZG_EINVAL.
//
// All calls share the array: calls whose kernels overlap on the GPU (two
// streams, or two host threads without ordering) race on it.  Each call
// writes every partial it reads, so nothing has to be cleared between calls.
//
// The array's device address is looked up once per device, on the first
// call made with that device current, and kept for the life of the process;
// a cudaDeviceReset while the library is loaded invalidates it (as it does
// every handle of this library), so callers must not reset a device they
// keep using through it.
#include <mutex>

#include "mg.cuh"
#include "mg_device.cuh"

namespace stzg {

namespace {

constexpr int kNoallocMaxBlocks = 8192;
constexpr int kNodesPerBlock = 1024;
constexpr int kNoallocThreads = 256;
constexpr int kMaxDevices = 64;

// Host code must not take this symbol's address directly: here it is a
// host-side stand-in, not a device address (see device_scratch()).
static __device__ __align__(256) double g_noalloc_partials[2 * kNoallocMaxBlocks];

double *g_scratch_ptr[kMaxDevices];
std::mutex g_scratch_mutex;

// Device address of the scratch array on the current device, looked up once
// per device with that device current.
int device_scratch(double **out) {
    int dev = -1;
    STZG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(STZG_EINVAL, "device ordinal beyond the scratch table");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
        g_scratch_ptr[dev] = (double *)p;
    }
    *out = g_scratch_ptr[dev];
    return STZG_OK;
}

__global__ void __launch_bounds__(kNoallocThreads)
    k_noalloc_partials(top_op<double> op, const double2 *__restrict__ z, const double2 *__restrict__ b, int m,
                       int n, double *partials) {
    __shared__ double sh[32];
    const long total = (long)m * n;
    const long base = (long)blockIdx.x * kNodesPerBlock;
    double sr = 0, sb = 0;
    for (int k = threadIdx.x; k < kNodesPerBlock; k += blockDim.x) {
        const long g = base + k;
        if (g >= total) break;
        const int i = (int)(g % m), j = (int)(g / m);
        const double2 r = top_res<double>(op, z, b, m, n, i, j);
        sr += r.x * r.x + r.y * r.y;
        const double2 bb = b[g];
        sb += bb.x * bb.x + bb.y * bb.y;
    }
    const double a = block_sum(sr, sh);
    const double c = block_sum(sb, sh);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = c;
    }
}

__global__ void k_noalloc_sum(const double *__restrict__ partials, int nblocks, double *out) {
    __shared__ double sh[32];
    double a = 0, c = 0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) {
        a += partials[2 * k];
        c += partials[2 * k + 1];
    }
    a = block_sum(a, sh);
    c = block_sum(c, sh);
    if (threadIdx.x == 0) {
        out[0] = a;
        out[1] = c;
    }
}

}  // namespace

}  // namespace stzg

using namespace stzg;

extern "C" int stzg_residual_norms_noalloc(const stz_params *p, double dt, const double *z_dev,
                                           const double *b_dev, double *out_dev, void *stream) {
    if (!p || !z_dev || !b_dev || !out_dev || !(dt > 0)) return fail(STZG_EINVAL, "null argument or dt <= 0");
    if (p->m < 4 || p->n < 4 || (p->m & 1)) return fail(STZG_EINVAL, "grid needs even m >= 4 and n >= 4");
    const int M = p->m, N = p->n + 1;
    const long nodes = (long)M * N;
    const long blocks = (nodes + kNodesPerBlock - 1) / kNodesPerBlock;
    if (blocks > kNoallocMaxBlocks)
        return fail(STZG_EINVAL, "grid too large for the no-allocation scratch (at most 8388608 nodes, "
                                 "m*(n+1) of the cell grid)");
    double *scratch = nullptr;
    STZG_CHECK(device_scratch(&scratch));
    qs_constants q;
    q.init(*p, p->viscosity / dt);
    const top_op<double> op = q.op<double>();
    cudaStream_t st = (cudaStream_t)stream;
    k_noalloc_partials<<<(int)blocks, kNoallocThreads, 0, st>>>(op, (const double2 *)z_dev, (const double2 *)b_dev,
                                                              M, N, scratch);
    note_launch();
    k_noalloc_sum<<<1, 256, 0, st>>>(scratch, (int)blocks, out_dev);
    note_launch();
    STZG_CUDA(cudaGetLastError());
    return STZG_OK;
}
