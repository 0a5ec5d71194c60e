// Layout conversion between the reference's host arrays (interleaved FP64,
// f[v + id*Q], u[d + id*dims]) and the device layout (SoA, FP64 or shifted
// FP32, plain or AA-pattern state), plus FP64 reductions over a grid.
#include <cuda_runtime.h>

#include "device.cuh"
#include "kernels.hpp"

namespace luma {

namespace {

// The interleaved host arrays are read and written one block of kTile sites
// at a time through shared memory: the block's Q*kTile (or dims*kTile)
// consecutive values move with consecutive threads on consecutive
// addresses, which matters most when the array is host memory the kernel
// reaches in place (a site-per-thread access would touch a new 32-byte
// sector per thread for each value).  The conversion of each value is the
// same expression as before.
constexpr int kTile = 128;

template <int Q, class P>
__global__ void __launch_bounds__(kTile) k_pop_in(const double *__restrict__ aos, typename P::S *__restrict__ soa,
                                                  int N, int M, int K, int layout, double rho0) {
    using L = Lattice<Q>;
    __shared__ double tile[kTile * Q];
    const size_t n = (size_t)N * M * K;
    const size_t base = (size_t)blockIdx.x * kTile;
    const int nsite = n - base < (size_t)kTile ? (int)(n - base) : kTile;
    for (int t = threadIdx.x; t < nsite * Q; t += kTile) tile[t] = aos[base * Q + t];
    __syncthreads();
    if ((int)threadIdx.x >= nsite) return;
    const size_t id = base + threadIdx.x;
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        double f = tile[threadIdx.x * Q + v];
        if (P::shifted) f -= L::w(v) * rho0;
        const int slot = layout == kPopAAE ? L::opp(v) : v;
        soa[(size_t)slot * n + id] = typename P::S(f);
    }
}

template <int Q, class P>
__global__ void __launch_bounds__(kTile) k_pop_out(const typename P::S *__restrict__ soa, double *__restrict__ aos,
                                                   int N, int M, int K, int layout, double rho0) {
    using L = Lattice<Q>;
    __shared__ double tile[kTile * Q];
    const size_t n = (size_t)N * M * K;
    const size_t base = (size_t)blockIdx.x * kTile;
    const int nsite = n - base < (size_t)kTile ? (int)(n - base) : kTile;
    if ((int)threadIdx.x < nsite) {
        const size_t id = base + threadIdx.x;
        const int k = (int)(id % K), j = (int)((id / K) % M), i = (int)(id / ((size_t)K * M));
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            size_t src;
            if (layout == kPopAAE) {
                src = (size_t)L::opp(v) * n + id;
            } else if (layout == kPopAAO) {
                int x = i + L::c(v, 0), y = j + L::c(v, 1), z = k + L::c(v, 2);
                x = (x + N) % N;
                y = (y + M) % M;
                z = (z + K) % K;
                src = (size_t)v * n + (size_t)z + (size_t)K * ((size_t)y + (size_t)M * x);
            } else {
                src = (size_t)v * n + id;
            }
            double f = double(soa[src]);
            if (P::shifted) f += L::w(v) * rho0;
            tile[threadIdx.x * Q + v] = f;
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nsite * Q; t += kTile) aos[base * Q + t] = tile[t];
}

template <class P>
__global__ void __launch_bounds__(kTile) k_vec_in(const double *__restrict__ aos, typename P::R *__restrict__ soa,
                                                  size_t n, int dims) {
    __shared__ double tile[kTile * 3];
    const size_t base = (size_t)blockIdx.x * kTile;
    const int nsite = n - base < (size_t)kTile ? (int)(n - base) : kTile;
    for (int t = threadIdx.x; t < nsite * dims; t += kTile) tile[t] = aos[base * dims + t];
    __syncthreads();
    if ((int)threadIdx.x >= nsite) return;
    const size_t id = base + threadIdx.x;
    for (int d = 0; d < dims; ++d) soa[(size_t)d * n + id] = typename P::R(tile[threadIdx.x * dims + d]);
}

template <class P>
__global__ void __launch_bounds__(kTile) k_vec_out(const typename P::R *__restrict__ soa, double *__restrict__ aos,
                                                   size_t n, int dims) {
    __shared__ double tile[kTile * 3];
    const size_t base = (size_t)blockIdx.x * kTile;
    const int nsite = n - base < (size_t)kTile ? (int)(n - base) : kTile;
    if ((int)threadIdx.x < nsite) {
        const size_t id = base + threadIdx.x;
        for (int d = 0; d < dims; ++d) tile[threadIdx.x * dims + d] = double(soa[(size_t)d * n + id]);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nsite * dims; t += kTile) aos[base * dims + t] = tile[t];
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Sums over the sites the macroscopic step updates (fluid, BFL, slip and
// transition-to-finer), accumulated in FP64: mass, momentum, kinetic energy;
// max |u| and a count of non-finite values.  Deterministic: each of the
// kReduceBlocks blocks sums a fixed set of sites (grid stride) in a fixed
// order and writes its partials to its own slot; k_reduce_fold then adds the
// slots in block order.  The same state gives the same bits on every run.
template <class P>
__global__ void __launch_bounds__(256) k_reduce(const uint8_t *__restrict__ typ, const typename P::R *__restrict__ rho,
                                                const typename P::R *__restrict__ u, size_t n, int dims,
                                                double *partials) {
    __shared__ double sh[8][8];
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
        const int t = typ[id];
        if (!(t == LUMA_SITE_FLUID || t == LUMA_SITE_BFL || t == LUMA_SITE_SLIP || t == LUMA_SITE_TL_TO_FINER))
            continue;
        const double r = double(rho[id]);
        const double ux = double(u[id]), uy = double(u[n + id]), uz = dims == 3 ? double(u[2 * n + id]) : 0.0;
        if (!isfinite(r) || !isfinite(ux) || !isfinite(uy) || !isfinite(uz)) {
            v[6] += 1.0;
            continue;
        }
        v[0] += r;
        v[1] += r * ux;
        v[2] += r * uy;
        v[3] += r * uz;
        const double q = ux * ux + uy * uy + uz * uz;
        v[4] += 0.5 * r * q;
        v[5] = fmax(v[5], sqrt(q));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const double w = k == 5 ? warp_max(v[k]) : warp_sum(v[k]);
        if (lane == 0) sh[warp][k] = w;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        const int k = threadIdx.x;
        double acc = sh[0][k];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) acc = k == 5 ? fmax(acc, sh[w][k]) : acc + sh[w][k];
        partials[(size_t)blockIdx.x * 8 + k] = acc;
    }
}

__global__ void k_reduce_fold(const double *__restrict__ partials, int nblocks, double *out) {
    const int k = threadIdx.x;
    if (k >= 8) return;
    double acc = partials[k];
    for (int b = 1; b < nblocks; ++b) {
        const double x = partials[(size_t)b * 8 + k];
        acc = k == 5 ? fmax(acc, x) : acc + x;
    }
    out[k] = acc;
}

}  // namespace

template <int Q, class P>
cudaError_t launch_pop_in(const double *aos, void *soa, int N, int M, int K, int layout, double rho0,
                          cudaStream_t s) {
    const size_t n = (size_t)N * M * K;
    k_pop_in<Q, P><<<(unsigned)((n + kTile - 1) / kTile), kTile, 0, s>>>(aos, static_cast<typename P::S *>(soa), N,
                                                                          M, K, layout, rho0);
    return cudaGetLastError();
}
template <int Q, class P>
cudaError_t launch_pop_out(const void *soa, double *aos, int N, int M, int K, int layout, double rho0,
                           cudaStream_t s) {
    const size_t n = (size_t)N * M * K;
    k_pop_out<Q, P><<<(unsigned)((n + kTile - 1) / kTile), kTile, 0, s>>>(static_cast<const typename P::S *>(soa),
                                                                           aos, N, M, K, layout, rho0);
    return cudaGetLastError();
}
template <class P>
cudaError_t launch_vec_in(const double *aos, void *soa, size_t n, int dims, cudaStream_t s) {
    k_vec_in<P><<<(unsigned)((n + kTile - 1) / kTile), kTile, 0, s>>>(aos, static_cast<typename P::R *>(soa), n, dims);
    return cudaGetLastError();
}
template <class P>
cudaError_t launch_vec_out(const void *soa, double *aos, size_t n, int dims, cudaStream_t s) {
    k_vec_out<P><<<(unsigned)((n + kTile - 1) / kTile), kTile, 0, s>>>(static_cast<const typename P::R *>(soa), aos, n,
                                                                       dims);
    return cudaGetLastError();
}
template <class P>
cudaError_t launch_reduce(const uint8_t *typ, const void *rho, const void *u, size_t n, int dims, double *acc,
                          cudaStream_t s) {
    double *partials = acc + 8;
    k_reduce<P><<<kReduceBlocks, 256, 0, s>>>(typ, static_cast<const typename P::R *>(rho),
                                               static_cast<const typename P::R *>(u), n, dims, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_reduce_fold<<<1, 32, 0, s>>>(partials, kReduceBlocks, acc);
    return cudaGetLastError();
}

#define LUMA_INST_T(Q, P)                                                                                  \
    template cudaError_t launch_pop_in<Q, P>(const double *, void *, int, int, int, int, double, cudaStream_t); \
    template cudaError_t launch_pop_out<Q, P>(const void *, double *, int, int, int, int, double, cudaStream_t);
LUMA_INST_T(9, P64)
LUMA_INST_T(19, P64)
LUMA_INST_T(27, P64)
LUMA_INST_T(9, P32)
LUMA_INST_T(19, P32)
LUMA_INST_T(27, P32)
template cudaError_t launch_vec_in<P64>(const double *, void *, size_t, int, cudaStream_t);
template cudaError_t launch_vec_in<P32>(const double *, void *, size_t, int, cudaStream_t);
template cudaError_t launch_vec_out<P64>(const void *, double *, size_t, int, cudaStream_t);
template cudaError_t launch_vec_out<P32>(const void *, double *, size_t, int, cudaStream_t);
template cudaError_t launch_reduce<P64>(const uint8_t *, const void *, const void *, size_t, int, double *,
                                        cudaStream_t);
template cudaError_t launch_reduce<P32>(const uint8_t *, const void *, const void *, size_t, int, double *,
                                        cudaStream_t);

}  // namespace luma
