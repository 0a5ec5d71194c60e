// BFL (Bouzidi-Firdaouss-Lallemand) bodies on the device stream.
//
// The reference decides per pulled link inside its stream
// (GridObj::_LBM_applyBFL_opt, LUMA src/GridObj_ops_lbm_optimised.cpp:
// 1010-1113, called from _LBM_stream_opt :224-229) by looking the marker of
// the site and of the source site up by position and reading BFLBody::Q.
// That decision depends only on the labels, the per-site marker lookup and
// Q, all fixed once the body is set up, so luma_gpu_bfl_set makes it once on
// the host: every (site, direction) that carries the condition becomes a
// link record (its kind, q, direction and marker), in (site, direction)
// order.  A site with links has a record index, a bit mask of its linked
// directions and the index of its first link, so the stream finds the link
// of direction v with one population count.
//
// Link kinds:
//   0  the site is eBFL and its own Q for the reversed link is valid, the
//      stencil site (i + c_v) is on the grid: the reference interpolates
//      with a stencil index built from (i, j, k) itself (:1070-1071), which
//      leaves f_opp(v) at the site;
//   1  as 0 with the stencil off the grid: fNew is left as it was;
//   2  the source site's marker has a valid Q for v: the interpolation from
//      the site's own post-collision populations (:1093-1097).
// Kinds 0 and 2 add c_opp(v) (f_opp(v) + fNew_v) to their marker's
// momentum-exchange force (ObjectManager::computeLiftDrag(v, id, g,
// markerID), src/ObjectManager.cpp:176-189); the stream records the sum per
// link and luma_gpu_bfl_forces adds each marker's links in (site,
// direction) order, the reference's loop order.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "device.cuh"
#include "dispatch.hpp"
#include "grid.hpp"
#include "lattice.cuh"

using namespace luma;

namespace luma {
struct BflState {
    int nm = 0, nlink = 0, nrec = 0;
    int *rec = nullptr;          // per site: record index or -1
    uint32_t *mask = nullptr;    // per record: linked directions
    int *first = nullptr;        // per record: first link
    double *q = nullptr;         // per link
    uint8_t *kind = nullptr;     // per link
    uint8_t *dir = nullptr;      // per link: v
    double *val = nullptr;       // per link: f_opp + fNew_v of the latest step
    int *moff = nullptr;         // per marker: range of its force links in mlink
    int *mlink = nullptr;
    double *force = nullptr;     // nm x 3 scratch
};
}  // namespace luma

namespace {

template <int Q>
__global__ void k_bfl_forces(const double *val, const uint8_t *dir, const int *moff, const int *mlink, int nm,
                             double *force) {
    using L = Lattice<Q>;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nm) return;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int r = moff[m]; r < moff[m + 1]; ++r) {
        const int l = mlink[r];
        const int vo = L::opp(dir[l]);
        const double s = val[l];
        fx += double(L::c(vo, 0)) * s;
        fy += double(L::c(vo, 1)) * s;
        fz += double(L::c(vo, 2)) * s;
    }
    force[3 * m + 0] = fx;
    force[3 * m + 1] = fy;
    force[3 * m + 2] = fz;
}

template <class T>
int upload(T **dst, const std::vector<T> &src) {
    if (cudaMalloc((void **)dst, std::max<size_t>(1, src.size()) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        *dst = nullptr;
        return luma_set_error(LUMA_E_NOMEM, "BFL tables: device allocation failed");
    }
    if (!src.empty() && cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return luma_set_error(LUMA_E_CUDA, "BFL tables: upload failed");
    return LUMA_OK;
}

}  // namespace

void luma_bfl_free(luma_gpu_grid *g) {
    BflState *b = g->bfl;
    if (!b) return;
    cudaFree(b->rec); cudaFree(b->mask); cudaFree(b->first); cudaFree(b->q); cudaFree(b->kind);
    cudaFree(b->dir); cudaFree(b->val); cudaFree(b->moff); cudaFree(b->mlink); cudaFree(b->force);
    delete b;
    g->bfl = nullptr;
}

// The table pointers a captured step bakes in (a new body allocates new
// tables, whatever address its state object gets).
void luma_bfl_signature(const luma_gpu_grid *g, std::vector<uintptr_t> &sig) {
    const BflState *b = g->bfl;
    if (!b) return;
    for (const void *p : {(const void *)b->rec, (const void *)b->mask, (const void *)b->first, (const void *)b->q,
                          (const void *)b->kind, (const void *)b->val})
        sig.push_back((uintptr_t)p);
}

void luma_bfl_args(const luma_gpu_grid *g, StepArgs &a) {
    const BflState *b = g->bfl;
    if (!b) return;
    a.bfl_rec = b->rec;
    a.bfl_mask = b->mask;
    a.bfl_first = b->first;
    a.bfl_q = b->q;
    a.bfl_kind = b->kind;
    a.bfl_val = b->val;
}

extern "C" {

int luma_gpu_bfl_set(luma_gpu_grid *g, const int32_t *site_marker, int nmarkers, const double *q) {
    if (!g || !site_marker || nmarkers < 0 || (nmarkers > 0 && !q))
        return luma_set_error(LUMA_E_INVALID, "luma_gpu_bfl_set: null pointer or negative marker count");
    const luma_grid_desc &d = g->d;
    const int N = d.N, M = d.M, K = d.K, Q = d.Q;
    const bool reg = (d.flags & LUMA_FLAG_REGULARISED) != 0;
    for (size_t id = 0; id < g->n; ++id)
        if (site_marker[id] < -1 || site_marker[id] >= nmarkers)
            return luma_set_error(LUMA_E_INVALID, "BFL: site %zu has marker %d (of %d)", id, site_marker[id], nmarkers);
    std::vector<int> cs(3 * Q), opp(Q);
    for (int v = 0; v < Q; ++v) {
        for (int e = 0; e < 3; ++e)
            cs[3 * v + e] = Q == 9 ? Lattice<9>::c(v, e) : (Q == 19 ? Lattice<19>::c(v, e) : Lattice<27>::c(v, e));
        opp[v] = Q == 9 ? Lattice<9>::opp(v) : (Q == 19 ? Lattice<19>::opp(v) : Lattice<27>::opp(v));
    }
    const uint8_t *t = g->htyp.data();
    std::vector<int> rec(g->n, -1), first;
    std::vector<uint32_t> mask;
    std::vector<double> lq;
    std::vector<uint8_t> kind, dir;
    std::vector<int> lmarker;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < M; ++j)
            for (int k = 0; k < K; ++k) {
                const int id = k + j * K + i * K * M;
                const int ty = t[id];
                if (ty == LUMA_SITE_REFINED || ty == LUMA_SITE_SOLID || (!reg && ty == LUMA_SITE_VELOCITY))
                    continue;  // sites the stream skips
                uint32_t mk = 0;
                const int start = (int)lq.size();
                for (int v = 0; v < Q; ++v) {
                    const int x = (i - cs[3 * v] + N) % N, y = (j - cs[3 * v + 1] + M) % M;
                    const int z = (k - cs[3 * v + 2] + K) % K;
                    const int sid = z + y * K + x * K * M;
                    if (ty != LUMA_SITE_BFL && t[sid] != LUMA_SITE_BFL) continue;
                    double qv = -1.0;
                    bool current = true;
                    int marker = -1;
                    if (ty == LUMA_SITE_BFL) {
                        marker = site_marker[id];
                        if (marker < 0)
                            return luma_set_error(LUMA_E_INVALID, "BFL: eBFL site %d has no marker", id);
                        qv = q[opp[v] + (size_t)Q * marker];
                    }
                    if (qv == -1.0 && site_marker[sid] >= 0) {
                        current = false;
                        marker = site_marker[sid];
                        qv = q[v + (size_t)Q * marker];
                    }
                    if (qv == -1.0) continue;
                    int kd = 2;
                    if (current) {
                        const int si = i + cs[3 * v], sj = j + cs[3 * v + 1], sk = k + cs[3 * v + 2];
                        kd = (si >= 0 && si < N && sj >= 0 && sj < M && sk >= 0 && sk < K) ? 0 : 1;
                    }
                    mk |= 1u << v;
                    lq.push_back(qv);
                    kind.push_back((uint8_t)kd);
                    dir.push_back((uint8_t)v);
                    lmarker.push_back(marker);
                }
                if (mk) {
                    rec[id] = (int)mask.size();
                    mask.push_back(mk);
                    first.push_back(start);
                }
            }
    // per marker, its force-carrying links in link order
    std::vector<int> moff(nmarkers + 1, 0), mlink;
    for (size_t l = 0; l < lq.size(); ++l)
        if (kind[l] != 1) moff[lmarker[l] + 1]++;
    for (int m = 0; m < nmarkers; ++m) moff[m + 1] += moff[m];
    mlink.assign(moff[nmarkers], 0);
    std::vector<int> fill(moff.begin(), moff.end() - 1);
    for (size_t l = 0; l < lq.size(); ++l)
        if (kind[l] != 1) mlink[fill[lmarker[l]]++] = (int)l;
    cudaStreamSynchronize(g->stream);
    luma_bfl_free(g);
    BflState *b = new BflState();
    g->bfl = b;
    b->nm = nmarkers;
    b->nlink = (int)lq.size();
    b->nrec = (int)mask.size();
    int rc;
    std::vector<double> zeros(std::max<size_t>(1, lq.size()), 0.0), fz(3 * std::max(1, nmarkers), 0.0);
    if ((rc = upload(&b->rec, rec)) || (rc = upload(&b->mask, mask)) || (rc = upload(&b->first, first)) ||
        (rc = upload(&b->q, lq)) || (rc = upload(&b->kind, kind)) || (rc = upload(&b->dir, dir)) ||
        (rc = upload(&b->val, zeros)) || (rc = upload(&b->moff, moff)) || (rc = upload(&b->mlink, mlink)) ||
        (rc = upload(&b->force, fz))) {
        luma_bfl_free(g);
        return rc;
    }
    return LUMA_OK;
}

int luma_gpu_bfl_forces(luma_gpu_grid *g, double *forces) {
    if (!g || !forces) return luma_set_error(LUMA_E_INVALID, "luma_gpu_bfl_forces: null argument");
    const BflState *b = g->bfl;
    if (!b) return luma_set_error(LUMA_E_STATE, "luma_gpu_bfl_forces: no BFL body (luma_gpu_bfl_set)");
    if (b->nm == 0) return LUMA_OK;
    cudaStream_t s = g->stream;
    cudaError_t e = dispatch(g->d.Q, LUMA_PREC_FP64, [&](auto q, auto) {
        k_bfl_forces<decltype(q)::value><<<(b->nm + 127) / 128, 128, 0, s>>>(b->val, b->dir, b->moff, b->mlink, b->nm,
                                                                            b->force);
        return cudaGetLastError();
    });
    if (e == cudaSuccess) e = cudaMemcpyAsync(forces, b->force, 3 * (size_t)b->nm * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "BFL forces: %s", cudaGetErrorString(e));
    return LUMA_OK;
}

}  // extern "C"
