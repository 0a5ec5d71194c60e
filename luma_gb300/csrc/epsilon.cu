// The rigid bodies' epsilon system on the device (FP64): the dense
// partial-pivot LU and transposed solve that ObjectManager::ibm_findEpsilon
// hands to LAPACK through GridUtils::solveLinearSystem
// (src/ObjectManager_ops_ibm.cpp:773-920, src/GridUtils.cpp:356-395:
// dgetrf_ on the row-major matrix read column-major, dgetrs_ with
// trans = 'T', which solves A x = b).
//
// Every matrix and solution element sees the operations of the serial
// algorithm in its order (this unit is built without FMA contraction), so
// the result equals the host LU's; what the device skips are exact no-ops.
// Markers couple only through shared support nodes, so the system is
// banded: with no entry more than b rows below or columns right of the
// diagonal, partial pivoting keeps step k's multipliers in rows k+1..k+b
// and the pivot row's entries in columns up to k+2b.  A step is two
// launches: one block searches the pivot, swaps the two rows (whole rows,
// as the dense algorithm does: earlier columns of L move with them) and
// scales the multipliers; then the rank-1 update of the b x 2b window runs
// over many blocks.  The forward solve keeps one pending row per thread and
// subtracts each term as its unknown arrives (the serial order); the
// backward solve runs its sums in one thread, nearest term first.
#include <cuda_runtime.h>

#include <vector>

#include "grid.hpp"

namespace {

constexpr int kThreads = 1024;

#define AC(r, c) A[(size_t)(c) * n + (r)]

// pivot of column k (first row of largest magnitude), row swap, multipliers
__global__ void __launch_bounds__(kThreads) k_eps_pivot(double *A, int n, int b, int k, int *ipiv, int *live) {
    __shared__ unsigned long long sbest[kThreads / 32];
    __shared__ int srow[kThreads / 32];
    __shared__ int sp;
    const int rend = k + b + 1 < n ? k + b + 1 : n;
    unsigned long long best = 0;
    int p = n;
    for (int r = k + threadIdx.x; r < rend; r += blockDim.x) {
        const unsigned long long v = (unsigned long long)__double_as_longlong(AC(r, k)) & 0x7fffffffffffffffull;
        if (p == n || v > best) { best = v; p = r; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int op = __shfl_xor_sync(0xffffffffu, p, o);
        if (op < n && (p == n || ob > best || (ob == best && op < p))) { best = ob; p = op; }
    }
    if ((threadIdx.x & 31) == 0) { sbest[threadIdx.x >> 5] = best; srow[threadIdx.x >> 5] = p; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bb = 0;
        int pp = n;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            if (srow[w] < n && (pp == n || sbest[w] > bb || (sbest[w] == bb && srow[w] < pp))) {
                bb = sbest[w];
                pp = srow[w];
            }
        sp = pp;
        ipiv[k] = pp + 1;
        *live = AC(pp, k) != 0.0;
    }
    __syncthreads();
    const int pr = sp;
    if (AC(pr, k) == 0.0) return;
    if (pr != k)
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            const double t = AC(k, c);
            AC(k, c) = AC(pr, c);
            AC(pr, c) = t;
        }
    __syncthreads();
    const double inv = 1.0 / AC(k, k);
    for (int r = k + 1 + threadIdx.x; r < rend; r += blockDim.x) AC(r, k) = AC(r, k) * inv;
}

// rank-1 update of rows k+1..k+b, columns k+1..k+2b (one column per block row)
__global__ void k_eps_update(double *A, int n, int b, int k, const int *live) {
    if (!*live) return;
    const int c = k + 1 + blockIdx.y;
    if (c >= n) return;
    const double akc = AC(k, c);
    if (akc == 0.0) return;
    const int rend = k + b + 1 < n ? k + b + 1 : n;
    for (int r = k + 1 + blockIdx.x * blockDim.x + threadIdx.x; r < rend; r += gridDim.x * blockDim.x)
        AC(r, c) = AC(r, c) - AC(r, k) * akc;
}

// Last row holding a non-zero of column r of L (row swaps can carry L
// entries below the band); r when none.
__global__ void k_eps_lower_extent(const double *A, int n, int *lim) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    int c = n - 1;
    while (c > r && AC(c, r) == 0.0) --c;
    lim[r] = c;
}

// forward U^T y = x (pending rows, one per thread, within 2b of the
// newest unknown), backward L^T z = y, then the row interchanges
__global__ void __launch_bounds__(kThreads) k_eps_solve(const double *A, int n, int b, const int *ipiv,
                                                        const int *lim, double *x) {
    __shared__ double ybuf[2];
    const int t = threadIdx.x;
    const int T = blockDim.x;
    double s = t < n ? x[t] : 0.0;
    int row = t;  // this thread's pending row: the first r >= c with r = t (mod T)
    for (int c = 0; c < n; ++c) {
        if (row == c) ybuf[c & 1] = s / AC(c, c);
        __syncthreads();
        const double y = ybuf[c & 1];
        if (row == c) {
            x[c] = y;
            row += T;
            s = row < n ? x[row] : 0.0;
        } else if (row < n && row <= c + 2 * b) {
            s = s - AC(c, row) * y;
        }
    }
    __syncthreads();
    if (t == 0) {
        for (int r = n - 1; r >= 0; --r) {
            double z = x[r];
            for (int c = r + 1; c <= lim[r]; ++c) z = z - AC(c, r) * x[c];
            x[r] = z;
        }
        for (int k = n - 1; k >= 0; --k) {
            const int p = ipiv[k] - 1;
            if (p != k) { const double tmp = x[k]; x[k] = x[p]; x[p] = tmp; }
        }
    }
}

#undef AC

}  // namespace

// Solves the n x n row-major system a (a[I*n + J]) for x (in: right-hand
// side, out: solution) on the device, with the same arithmetic as the host
// LU.  `band` bounds |I - J| over the non-zero entries.  The forward solve
// keeps one pending row per thread: bands over (kThreads - 1) / 2 are
// refused (LUMA_E_INVALID: the caller solves on the host).  Blocks until x
// is on the host.
int luma_eps_solve_device(int n, int band, const std::vector<double> &a, std::vector<double> &x,
                          cudaStream_t s) {
    if (n <= 0) return LUMA_OK;
    if (band < 0 || band > n - 1) band = n - 1;
    if (2 * band + 1 > kThreads) return LUMA_E_INVALID;
    double *dA = nullptr, *dx = nullptr;
    int *dip = nullptr, *dlim = nullptr, *dlive = nullptr;
    auto release = [&]() { cudaFree(dA); cudaFree(dx); cudaFree(dip); cudaFree(dlim); cudaFree(dlive); };
    const size_t bytes = (size_t)n * n * sizeof(double);
    if (cudaMalloc(&dA, bytes) != cudaSuccess || cudaMalloc(&dx, n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dip, n * sizeof(int)) != cudaSuccess || cudaMalloc(&dlim, n * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&dlive, sizeof(int)) != cudaSuccess) {
        release();
        cudaGetLastError();
        return luma_set_error(LUMA_E_NOMEM, "epsilon system: device allocation of %d x %d failed", n, n);
    }
    cudaError_t e = cudaMemcpyAsync(dA, a.data(), bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x.data(), n * sizeof(double), cudaMemcpyHostToDevice, s);
    for (int k = 0; k < n && e == cudaSuccess; ++k) {
        k_eps_pivot<<<1, kThreads, 0, s>>>(dA, n, band, k, dip, dlive);
        const int rows = band < n - 1 - k ? band : n - 1 - k;
        const int cols = 2 * band < n - 1 - k ? 2 * band : n - 1 - k;
        if (rows > 0 && cols > 0) {
            const dim3 grid((unsigned)((rows + 127) / 128), (unsigned)cols);
            k_eps_update<<<grid, 128, 0, s>>>(dA, n, band, k, dlive);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_eps_lower_extent<<<(n + 255) / 256, 256, 0, s>>>(dA, n, dlim);
        k_eps_solve<<<1, kThreads, 0, s>>>(dA, n, band, dip, dlim, dx);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(x.data(), dx, n * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    release();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "epsilon system solve: %s", cudaGetErrorString(e));
    return LUMA_OK;
}
