// Momentum-exchange force of the bounce-back (solid) sites of a grid:
// ObjectManager::computeLiftDrag for bounce-back bodies (LUMA
// src/ObjectManager.cpp:93-165), which the reference accumulates inside
// GridObj::LBM_multi_opt under L_LD_OUT (src/GridObj_ops_lbm_optimised.cpp:
// 63-88).  Every solid site adds, for each direction n whose neighbour
// x_dest = x - c_opp(n) is a fluid site on the grid (no periodic wrap),
// 2 c_opp(n) f_opp(n)(x_dest) from the populations the next step streams.
// Like the reference, every solid site counts (walls included).
//
// FP64 sums in a fixed order: each thread sums its sites (grid-stride) over
// n in order, blocks reduce in shared memory, one block folds the block
// partials in order; the result does not depend on the run.
#include <cuda_runtime.h>

#include "device.cuh"
#include "dispatch.hpp"
#include "grid.hpp"

using namespace luma;

namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 608;  // 4 per SM

template <int Q, class P>
__global__ void __launch_bounds__(kThreads) k_momex(const void *f, const uint8_t *typ, int N, int M, int K,
                                                    double rho0, double *partial) {
    using L = Lattice<Q>;
    const size_t n = (size_t)N * M * K;
    double s[3] = {0.0, 0.0, 0.0};
    for (size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
        if (typ[id] != LUMA_SITE_SOLID) continue;
        const int k = (int)(id % K), j = (int)((id / K) % M), i = (int)(id / ((size_t)K * M));
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            const int o = L::opp(v);
            const int xd = i - L::c(o, 0), yd = j - L::c(o, 1), zd = k - L::c(o, 2);
            double cx = 0.0, cy = 0.0, cz = 0.0;
            if (xd >= 0 && xd < N && yd >= 0 && yd < M && zd >= 0 && zd < K) {
                const size_t did = (size_t)zd + (size_t)yd * K + (size_t)xd * K * M;
                if (typ[did] == LUMA_SITE_FLUID) {
                    double fv = double(static_cast<const typename P::S *>(f)[(size_t)o * n + did]);
                    if (P::shifted) fv += L::w(o) * rho0;
                    cx = 2.0 * L::c(o, 0) * fv;
                    cy = 2.0 * L::c(o, 1) * fv;
                    cz = 2.0 * L::c(o, 2) * fv;
                }
            }
            s[0] += cx;
            s[1] += cy;
            s[2] += cz;
        }
    }
    __shared__ double sh[3][kThreads];
    for (int d = 0; d < 3; ++d) sh[d][threadIdx.x] = s[d];
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int d = 0; d < 3; ++d) sh[d][threadIdx.x] += sh[d][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 3) partial[3 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_momex_fold(const double *partial, int nb, double *out) {
    const int d = threadIdx.x;
    if (d >= 3) return;
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += partial[3 * b + d];
    out[d] = s;
}

}  // namespace

extern "C" int luma_gpu_momex_force(luma_gpu_grid *g, double force[3]) {
    if (!g || !force) return luma_set_error(LUMA_E_INVALID, "luma_gpu_momex_force: null argument");
    force[0] = force[1] = force[2] = 0.0;
    if (g->bulk) return LUMA_OK;  // the in-place path only runs all-fluid grids: no solid site
    double *buf = nullptr;
    cudaStream_t s = g->stream;
    if (cudaMallocAsync((void **)&buf, (3 * kBlocks + 3) * sizeof(double), s) != cudaSuccess)
        return luma_set_error(LUMA_E_NOMEM, "momentum exchange: scratch allocation failed");
    const luma_grid_desc &d = g->d;
    cudaError_t e = dispatch(d.Q, d.precision, [&](auto q, auto p) {
        k_momex<decltype(q)::value, decltype(p)><<<kBlocks, kThreads, 0, s>>>(g->f[g->cur], g->typ, d.N, d.M, d.K,
                                                                             d.rho_in, buf);
        return cudaGetLastError();
    });
    if (e == cudaSuccess) {
        k_momex_fold<<<1, 32, 0, s>>>(buf, kBlocks, buf + 3 * kBlocks);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(force, buf + 3 * kBlocks, 3 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(buf, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "momentum exchange: %s", cudaGetErrorString(e));
    return LUMA_OK;
}
