// Layout conversion between the reference's host arrays (interleaved FP64,
// f[v + id*Q], u[d + id*dims]) and the device layout (SoA, FP64 or shifted
// FP32, plain or AA-pattern state), plus FP64 reductions over a grid.
#include <cuda_runtime.h>

#include "device.cuh"
#include "kernels.hpp"

namespace luma {

namespace {

template <int Q, class P>
__global__ void k_pop_in(const double *__restrict__ aos, typename P::S *__restrict__ soa, int N, int M, int K,
                         int layout, double rho0) {
    using L = Lattice<Q>;
    const size_t n = (size_t)N * M * K;
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        double f = aos[(size_t)v + id * Q];
        if (P::shifted) f -= L::w(v) * rho0;
        const int slot = layout == kPopAAE ? L::opp(v) : v;
        soa[(size_t)slot * n + id] = typename P::S(f);
    }
}

template <int Q, class P>
__global__ void k_pop_out(const typename P::S *__restrict__ soa, double *__restrict__ aos, int N, int M, int K,
                          int layout, double rho0) {
    using L = Lattice<Q>;
    const size_t n = (size_t)N * M * K;
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
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
        aos[(size_t)v + id * Q] = f;
    }
}

template <class P>
__global__ void k_vec_in(const double *__restrict__ aos, typename P::R *__restrict__ soa, size_t n, int dims) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    for (int d = 0; d < dims; ++d) soa[(size_t)d * n + id] = typename P::R(aos[(size_t)d + id * dims]);
}

template <class P>
__global__ void k_vec_out(const typename P::R *__restrict__ soa, double *__restrict__ aos, size_t n, int dims) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    for (int d = 0; d < dims; ++d) aos[(size_t)d + id * dims] = double(soa[(size_t)d * n + id]);
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
// max |u| and a count of non-finite values.
template <class P>
__global__ void k_reduce(const uint8_t *__restrict__ typ, const typename P::R *__restrict__ rho,
                         const typename P::R *__restrict__ u, size_t n, int dims, double *acc) {
    double m = 0, mx = 0, my = 0, mz = 0, ke = 0, umax = 0, bad = 0;
    for (size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
        const int t = typ[id];
        if (!(t == LUMA_SITE_FLUID || t == LUMA_SITE_BFL || t == LUMA_SITE_SLIP || t == LUMA_SITE_TL_TO_FINER))
            continue;
        const double r = double(rho[id]);
        const double ux = double(u[id]), uy = double(u[n + id]), uz = dims == 3 ? double(u[2 * n + id]) : 0.0;
        if (!isfinite(r) || !isfinite(ux) || !isfinite(uy) || !isfinite(uz)) {
            bad += 1.0;
            continue;
        }
        m += r;
        mx += r * ux;
        my += r * uy;
        mz += r * uz;
        const double q = ux * ux + uy * uy + uz * uz;
        ke += 0.5 * r * q;
        umax = fmax(umax, sqrt(q));
    }
    m = warp_sum(m);
    mx = warp_sum(mx);
    my = warp_sum(my);
    mz = warp_sum(mz);
    ke = warp_sum(ke);
    bad = warp_sum(bad);
    umax = warp_max(umax);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc + 0, m);
        atomicAdd(acc + 1, mx);
        atomicAdd(acc + 2, my);
        atomicAdd(acc + 3, mz);
        atomicAdd(acc + 4, ke);
        atomicMax(reinterpret_cast<unsigned long long *>(acc + 5), (unsigned long long)__double_as_longlong(umax));
        atomicAdd(acc + 6, bad);
    }
}

}  // namespace

template <int Q, class P>
cudaError_t launch_pop_in(const double *aos, void *soa, int N, int M, int K, int layout, double rho0,
                          cudaStream_t s) {
    const size_t n = (size_t)N * M * K;
    k_pop_in<Q, P><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(aos, static_cast<typename P::S *>(soa), N, M, K,
                                                               layout, rho0);
    return cudaGetLastError();
}
template <int Q, class P>
cudaError_t launch_pop_out(const void *soa, double *aos, int N, int M, int K, int layout, double rho0,
                           cudaStream_t s) {
    const size_t n = (size_t)N * M * K;
    k_pop_out<Q, P><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<const typename P::S *>(soa), aos, N,
                                                                M, K, layout, rho0);
    return cudaGetLastError();
}
template <class P>
cudaError_t launch_vec_in(const double *aos, void *soa, size_t n, int dims, cudaStream_t s) {
    k_vec_in<P><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(aos, static_cast<typename P::R *>(soa), n, dims);
    return cudaGetLastError();
}
template <class P>
cudaError_t launch_vec_out(const void *soa, double *aos, size_t n, int dims, cudaStream_t s) {
    k_vec_out<P><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<const typename P::R *>(soa), aos, n, dims);
    return cudaGetLastError();
}
template <class P>
cudaError_t launch_reduce(const uint8_t *typ, const void *rho, const void *u, size_t n, int dims, double *acc,
                          cudaStream_t s) {
    cudaMemsetAsync(acc, 0, 7 * sizeof(double), s);
    k_reduce<P><<<152 * 4, 256, 0, s>>>(typ, static_cast<const typename P::R *>(rho),
                                         static_cast<const typename P::R *>(u), n, dims, acc);
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
