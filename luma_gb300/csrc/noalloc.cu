// Field reductions for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc or let a library do it
// for them: hosts that hand the GPU's memory to a fixed-size pool at
// start-up and forbid any later allocation, and real-time loops where an
// allocation's latency, or its failure under memory pressure, is not
// acceptable.  luma_gpu_reduce_fields_noalloc gives them the FP64 mass /
// momentum / energy reduction of luma_gpu_reduce over device arrays they
// already own, using only the fixed scratch array below.  The call blocks
// until the result is on the host.
//
// Scratch: one file-scope __device__ array of (kBlocks + 1) * 8 doubles
// (64 KiB + 64 B).  Every GPU that loads this library holds it until the
// process exits.  Every call shares it and it keeps the last call's
// contents: the first pass overwrites every partial slot it later reads, so
// nothing needs clearing, but two calls whose kernels overlap on the GPU
// (different streams, or different host threads on one stream without
// ordering) race on it and must not be issued.
//
// In host code the array's name is only a host-side stand-in, not a device
// address: the device address is obtained once per device with
// cudaGetSymbolAddress, with that device current, and passed to the
// kernels.  The first call on each device performs that set-up.  A call on
// a stream under capture is refused before it does anything.  The address
// is cached for the life of the process: after cudaDeviceReset the cached
// address is stale and the call must not be used again in that process.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "grid.hpp"

namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 1024;                     // partial-sum slots
constexpr int kItemsPerThread = 64;
constexpr int64_t kMaxSites = (int64_t)kBlocks * kThreads * kItemsPerThread;  // 16,777,216
constexpr int kValues = 8;                        // mass, mx, my, mz, ke, max|u|, nonfinite, spare

static __device__ __align__(256) double g_reduce_scratch[(kBlocks + 1) * kValues];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_ptr[kMaxDevices] = {nullptr};

__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double wmax(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Pass 1: block b reduces sites [b*chunk, (b+1)*chunk) into slot b.
__global__ void __launch_bounds__(kThreads) k_partials(const uint8_t *__restrict__ typ, const double *__restrict__ rho,
                                                       const double *__restrict__ u, int64_t n, int dims,
                                                       int64_t chunk, double *scratch) {
    __shared__ double sh[kThreads / 32][kValues];
    double v[kValues] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int64_t lo = (int64_t)blockIdx.x * chunk;
    const int64_t hi = lo + chunk < n ? lo + chunk : n;
    for (int64_t id = lo + threadIdx.x; id < hi; id += blockDim.x) {
        const int t = typ[id];
        if (!(t == LUMA_SITE_FLUID || t == LUMA_SITE_BFL || t == LUMA_SITE_SLIP || t == LUMA_SITE_TL_TO_FINER))
            continue;
        const double r = rho[id];
        const double ux = u[id], uy = u[n + id], uz = dims == 3 ? u[2 * n + id] : 0.0;
        if (!isfinite(r) || !isfinite(ux) || !isfinite(uy) || !isfinite(uz)) {
            v[6] += 1.0;
            continue;
        }
        const double q = ux * ux + uy * uy + uz * uz;
        v[0] += r;
        v[1] += r * ux;
        v[2] += r * uy;
        v[3] += r * uz;
        v[4] += 0.5 * r * q;
        v[5] = fmax(v[5], sqrt(q));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < kValues; ++k) {
        const double w = k == 5 ? wmax(v[k]) : wsum(v[k]);
        if (lane == 0) sh[warp][k] = w;
    }
    __syncthreads();
    if (threadIdx.x < kValues) {
        const int k = threadIdx.x;
        double acc = sh[0][k];
        for (int w = 1; w < kThreads / 32; ++w) acc = k == 5 ? fmax(acc, sh[w][k]) : acc + sh[w][k];
        scratch[blockIdx.x * kValues + k] = acc;
    }
}

// Pass 2: one block folds the partial slots in a fixed order into the
// result slot (deterministic for a given size).
__global__ void k_fold(int nblocks, double *scratch) {
    const int k = threadIdx.x;
    if (k >= kValues) return;
    double acc = scratch[k];
    for (int b = 1; b < nblocks; ++b) {
        const double x = scratch[b * kValues + k];
        acc = k == 5 ? fmax(acc, x) : acc + x;
    }
    scratch[kBlocks * kValues + k] = acc;
}

// Device address of the scratch array on the current device (set up once
// per device, with that device current).
int scratch_address(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return luma_set_error(LUMA_E_INVALID, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        double *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, g_reduce_scratch);
        if (e != cudaSuccess)
            return luma_set_error(LUMA_E_CUDA, "cudaGetSymbolAddress(reduce scratch): %s", cudaGetErrorString(e));
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return LUMA_OK;
}

}  // namespace

extern "C" int luma_gpu_reduce_fields_noalloc(const uint8_t *typ, const double *rho, const double *u, int64_t n,
                                              int dims, void *cuda_stream, luma_reduction *out) {
    if (!typ || !rho || !u || !out) return luma_set_error(LUMA_E_INVALID, "null argument");
    if (dims != 2 && dims != 3) return luma_set_error(LUMA_E_INVALID, "dims must be 2 or 3, got %d", dims);
    if (n <= 0) return luma_set_error(LUMA_E_INVALID, "site count must be positive, got %lld", (long long)n);
    if (n > kMaxSites)
        return luma_set_error(LUMA_E_INVALID,
                              "luma_gpu_reduce_fields_noalloc handles at most %lld sites (its fixed scratch holds "
                              "%d partial sums of %d sites); got %lld — use luma_gpu_reduce",
                              (long long)kMaxSites, kBlocks, kThreads * kItemsPerThread, (long long)n);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    // the call ends with a copy to the host and a wait on the stream, and a
    // capturing stream takes neither: refuse before anything is recorded
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess) cudaGetLastError();  // this query's own error, reported below
    if (e != cudaSuccess || cap != cudaStreamCaptureStatusNone)
        return luma_set_error(LUMA_E_INVALID,
                              "luma_gpu_reduce_fields_noalloc cannot run on a stream under capture (it blocks until "
                              "the sums are on the host)%s%s",
                              e != cudaSuccess ? ": " : "", e != cudaSuccess ? cudaGetErrorString(e) : "");
    double *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    // an error left pending by an earlier, unrelated call belongs to that
    // call's owner: report it without clearing it and launch nothing
    e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return luma_set_error(LUMA_E_CUDA, "a CUDA error was pending before the reduction: %s", cudaGetErrorString(e));
    const int64_t chunk = (int64_t)kThreads * kItemsPerThread;
    const int nblocks = (int)((n + chunk - 1) / chunk);
    k_partials<<<nblocks, kThreads, 0, s>>>(typ, rho, u, n, dims, chunk, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "k_partials launch: %s", cudaGetErrorString(e));
    k_fold<<<1, 32, 0, s>>>(nblocks, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "k_fold launch: %s", cudaGetErrorString(e));
    double h[kValues];
    e = cudaMemcpyAsync(h, scratch + kBlocks * kValues, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "reduction result: %s", cudaGetErrorString(e));
    out->mass = h[0];
    out->momentum[0] = h[1];
    out->momentum[1] = h[2];
    out->momentum[2] = h[3];
    out->kinetic_energy = h[4];
    out->max_speed = h[5];
    out->nonfinite = (int64_t)h[6];
    return LUMA_OK;
}
