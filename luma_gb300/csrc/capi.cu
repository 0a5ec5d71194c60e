// C ABI of the GB300 LBM time step (include/luma_gpu.h): grid handles,
// state transfer, the recursive multi-grid step and reductions.
//
// The step mirrors GridObj::LBM_multi_opt (LUMA src/GridObj_ops_lbm_optimised.cpp:36-193):
// two sub-steps of every sub-grid, then this grid's stream/macro/[IBM]/
// collide, then the buffer swap.  Grids whose sites are all fluid (periodic
// box, BGK, no forcing, no refinement) run the in-place AA kernel instead of
// the two-buffer general kernel; both give the reference's result.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "device.cuh"
#include "dispatch.hpp"
#include "grid.hpp"
#include "kernels.hpp"

using namespace luma;

static thread_local std::string g_last_error;

int luma_set_error(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return luma_set_error(LUMA_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

namespace {

size_t real_size(const luma_gpu_grid *g) { return g->d.precision == LUMA_PREC_FP64 ? 8 : 4; }

// GridUtils::isWithinDomainWall (src/GridUtils.cpp:1369-1430).
bool within_domain_wall(const luma_grid_desc &d, double x, double y, double z, int nv[3], int *nd, int *edges) {
    const double *E = d.global_edges, *T = d.wall_thickness;
    nv[0] = nv[1] = nv[2] = 0;
    *nd = -1;
    *edges = 0;
    if (x > 0.0 && x < T[0]) { *nd = 0; nv[0] = 1; ++*edges; }
    if (x < E[1] && x > E[1] - T[1]) { *nd = 0; nv[0] = -1; ++*edges; }
    if (y > 0.0 && y < T[2]) { *nd = 1; nv[1] = 1; ++*edges; }
    if (y < E[3] && y > E[3] - T[3]) { *nd = 1; nv[1] = -1; ++*edges; }
    if (d.dims == 3) {
        if (z > 0.0 && z < T[4]) { *nd = 2; nv[2] = 1; ++*edges; }
        if (z < E[5] && z > E[5] - T[5]) { *nd = 2; nv[2] = -1; ++*edges; }
    }
    return *edges > 0;
}

void host_c(int Q, int v, int c[3]) {
    for (int d = 0; d < 3; ++d)
        c[d] = Q == 9 ? Lattice<9>::c(v, d) : (Q == 19 ? Lattice<19>::c(v, d) : Lattice<27>::c(v, d));
}

// GridObj::_LBM_updateReynolds with GridUtils::getReynoldsRampCoefficient
// (src/GridObj_ops_lbm_optimised.cpp:39-42, 1313-1321; src/GridUtils.cpp:
// 1825-1833): omega of the step from Re = L_RE * (1 - cos(pi t / ramp)) at
// t = (t_grid + 1) dt while t <= ramp (the coefficient reaches 2 at the end
// of the ramp, then drops to 1), in the reference's operation order.
void update_reynolds(luma_gpu_grid *g) {
    luma_grid_desc &d = g->d;
    const double t = (g->t + 1) * d.dt;
    const double coeff = t <= d.reynolds_ramp ? 1.0 - std::cos(3.14159265358979323846 * t / d.reynolds_ramp) : 1.0;
    const double nu = ((1.0 / (d.re * coeff)) * d.dt) / (d.dh * d.dh);
    d.omega = 1.0 / ((nu / g->cs2) + 0.5);
}

double ramp(const luma_grid_desc &d, double t) {
    if (d.velocity_ramp > 0.0 && t <= d.velocity_ramp) return (1.0 - std::cos(3.14159265358979323846 * t / d.velocity_ramp)) / 2.0;
    return 1.0;
}

// Host pre-processing of the boundary sites: wall normals for slip and
// regularised sites, and the last writer of each velocity site's u under a
// velocity ramp.
int build_site_tables(luma_gpu_grid *g, const int32_t *typ, const double *xpos, const double *ypos,
                      const double *zpos) {
    const luma_grid_desc &d = g->d;
    const int N = d.N, M = d.M, K = d.K, Q = d.Q;
    const bool reg = (d.flags & LUMA_FLAG_REGULARISED) != 0;
    std::vector<int8_t> wall;
    std::vector<RegSite> regs;
    bool need_wall = false;
    for (size_t id = 0; id < g->n; ++id)
        if (typ[id] == LUMA_SITE_SLIP) need_wall = true;
    if (need_wall) wall.assign(4 * g->n, 0);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < M; ++j)
            for (int k = 0; k < K; ++k) {
                const int id = k + j * K + i * K * M;
                const int t = typ[id];
                // Pulling from an extrapolate-right site reads the population two
                // sites to its left (:246-251): such sites need i >= 2.
                if (t == LUMA_SITE_EXTRAPOLATE_RIGHT && i < 2)
                    return luma_set_error(LUMA_E_INVALID, "extrapolate-right site at i=%d < 2", i);
                if (t == LUMA_SITE_SLIP || (reg && (t == LUMA_SITE_VELOCITY || t == LUMA_SITE_PRESSURE))) {
                    if (!xpos || !ypos || !zpos)
                        return luma_set_error(LUMA_E_INVALID, "slip/regularised sites need site positions");
                    int nv[3], nd, ne;
                    if (!within_domain_wall(d, xpos[i], ypos[j], zpos[k], nv, &nd, &ne))
                        return luma_set_error(LUMA_E_INVALID,
                                              "site (%d,%d,%d): boundary site not located inside a domain wall", i, j, k);
                    if (t == LUMA_SITE_SLIP) {
                        wall[4 * (size_t)id + 0] = (int8_t)nv[0];
                        wall[4 * (size_t)id + 1] = (int8_t)nv[1];
                        wall[4 * (size_t)id + 2] = (int8_t)nv[2];
                        wall[4 * (size_t)id + 3] = (int8_t)ne;
                    } else {
                        if (ne > 1 && t == LUMA_SITE_PRESSURE)
                            return luma_set_error(LUMA_E_INVALID, "Pressure BC not supported at corner/edge site");
                        RegSite r;
                        r.id = id; r.i = i; r.j = j; r.k = k;
                        r.nvec[0] = (int8_t)nv[0]; r.nvec[1] = (int8_t)nv[1]; r.nvec[2] = (int8_t)nv[2];
                        r.ndir = (int8_t)nd;
                        r.edges = (int8_t)ne;
                        // extrapolation needs two inward neighbours on the grid
                        const int i2 = i + 2 * nv[0], j2 = j + 2 * nv[1], k2 = k + 2 * nv[2];
                        if (i2 < 0 || i2 >= N || j2 < 0 || j2 >= M || k2 < 0 || k2 >= K)
                            return luma_set_error(LUMA_E_INVALID, "Extrapolation does not have enough available cells.");
                        regs.push_back(r);
                    }
                }
            }
    // Velocity sites under a ramp without regularisation: row of the last
    // (i,j,k,v)-ordered site that streams from them (:255-265).
    std::vector<int2> velu;
    if (d.velocity_ramp > 0.0 && !reg) {
        for (int si = 0; si < N; ++si)
            for (int sj = 0; sj < M; ++sj)
                for (int sk = 0; sk < K; ++sk) {
                    const int sid = sk + sj * K + si * K * M;
                    if (typ[sid] != LUMA_SITE_VELOCITY) continue;
                    long best = -1;
                    int best_row = -1;
                    for (int v = 0; v < Q; ++v) {
                        int c[3];
                        host_c(Q, v, c);
                        const int x = (si + c[0] + N) % N, y = (sj + c[1] + M) % M, z = (sk + c[2] + K) % K;
                        const int xid = z + y * K + x * K * M;
                        const int xt = typ[xid];
                        if (xt == LUMA_SITE_SOLID || xt == LUMA_SITE_REFINED || xt == LUMA_SITE_VELOCITY) continue;
                        if (xt == LUMA_SITE_SLIP) continue;  // reflected links never reach the velocity branch
                        const long key = (long)xid * Q + v;
                        if (key > best) { best = key; best_row = y; }
                    }
                    if (best_row >= 0) velu.push_back(make_int2(sid, best_row));
                }
    }
    if (need_wall) {
        CK(cudaMalloc(&g->wall, wall.size()));
        CK(cudaMemcpy(g->wall, wall.data(), wall.size(), cudaMemcpyHostToDevice));
    }
    g->nreg = (int)regs.size();
    if (g->nreg) {
        CK(cudaMalloc(&g->reg, regs.size() * sizeof(RegSite)));
        CK(cudaMemcpy(g->reg, regs.data(), regs.size() * sizeof(RegSite), cudaMemcpyHostToDevice));
    }
    g->nvelu = (int)velu.size();
    if (g->nvelu) {
        CK(cudaMalloc(&g->velu, velu.size() * sizeof(int2)));
        CK(cudaMemcpy(g->velu, velu.data(), velu.size() * sizeof(int2), cudaMemcpyHostToDevice));
    }
    return LUMA_OK;
}

}  // namespace

// Sites of an IBM grid whose collision waits for the IBM pass: the distinct
// support sites of rigid bodies, and the sites phase A does not stream
// (solid, refined, velocity; the regularised boundary sites phase B
// streams), which the reference's second loop collides as well.  Every
// other site carries the zero force of the reset through the step, so
// phase A collides it at once with the same arithmetic (the Guo term adds
// exact zeros), saving a pass over the populations.  Not used under
// gravity (non-zero force everywhere) or with flexible bodies (supports
// move within the step).
int luma_update_defer(luma_gpu_grid *g) {
    cudaFree(g->defer);
    cudaFree(g->defer_ids);
    g->defer = nullptr;
    g->defer_ids = nullptr;
    g->ndefer = 0;
    g->fuse = false;
    const luma_grid_desc &d = g->d;
    if (!(d.flags & LUMA_FLAG_IBM) || (d.flags & LUMA_FLAG_GRAVITY) || g->bulk) return LUMA_OK;
    if (g->ibm && g->ibm->has_flexible) return LUMA_OK;
    const bool reg = (d.flags & LUMA_FLAG_REGULARISED) != 0;
    std::vector<uint8_t> mask(g->n, 0);
    for (size_t id = 0; id < g->n; ++id) {
        const int t = g->htyp[id];
        if (t == LUMA_SITE_SOLID || t == LUMA_SITE_REFINED || t == LUMA_SITE_VELOCITY ||
            (reg && t == LUMA_SITE_PRESSURE))
            mask[id] = 1;
    }
    if (g->ibm && g->ibm->has_bodies && g->ibm->dev.nu > 0) {
        std::vector<int> us(g->ibm->dev.nu);
        CK(cudaMemcpy(us.data(), g->ibm->dev.usite, us.size() * sizeof(int), cudaMemcpyDeviceToHost));
        for (int id : us) mask[id] = 1;
    }
    std::vector<int> ids;
    for (size_t id = 0; id < g->n; ++id)
        if (mask[id]) ids.push_back((int)id);
    CK(cudaMalloc(&g->defer, g->n));
    CK(cudaMemcpy(g->defer, mask.data(), g->n, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&g->defer_ids, std::max<size_t>(1, ids.size()) * sizeof(int)));
    if (!ids.empty()) CK(cudaMemcpy(g->defer_ids, ids.data(), ids.size() * sizeof(int), cudaMemcpyHostToDevice));
    g->ndefer = (int)ids.size();
    g->fuse = true;
    return LUMA_OK;
}

// Sites of a general-path grid split between the interior kernel (fluid
// sites whose every pull source, wrapped periodically, is a fluid site) and
// the full site logic (the rest, less the sites the stream skips).  Grids
// below kInteriorMinSites keep the single full-logic launch: there the step
// is bound by launch latency.  Above it the full-logic kernel, latency bound
// per site (a label branch per pulled direction, 110 registers), is slower
// than the interior kernel plus a list of the other sites (a 110,592-site
// level: 33 us per launch at 121 GB/s in one kernel).
constexpr size_t kInteriorMinSites = 1u << 14;

int luma_build_interior(luma_gpu_grid *g) {
    cudaFree(g->fast);
    cudaFree(g->gen_ids);
    g->fast = nullptr;
    g->gen_ids = nullptr;
    g->ngen = 0;
    g->ngen_early = 0;
    if (g->bulk || (g->n < kInteriorMinSites && !(g->d.flags & LUMA_FLAG_SPLIT_INTERIOR))) return LUMA_OK;
    const luma_grid_desc &d = g->d;
    const int N = d.N, M = d.M, K = d.K, Q = d.Q;
    const bool reg = (d.flags & LUMA_FLAG_REGULARISED) != 0;
    std::vector<int> cs(3 * Q);
    for (int v = 0; v < Q; ++v) host_c(Q, v, &cs[3 * v]);
    std::vector<uint8_t> fast(g->n, 0);
    std::vector<int> gen, late;
    const uint8_t *t = g->htyp.data();
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < M; ++j)
            for (int k = 0; k < K; ++k) {
                const int id = k + j * K + i * K * M;
                const int ty = t[id];
                if (ty == LUMA_SITE_REFINED || ty == LUMA_SITE_SOLID || ty == LUMA_SITE_VELOCITY ||
                    (reg && ty == LUMA_SITE_PRESSURE))
                    continue;  // the stream skips these
                bool plain = ty == LUMA_SITE_FLUID;
                for (int v = 0; plain && v < Q; ++v) {
                    const int x = (i - cs[3 * v] + N) % N, y = (j - cs[3 * v + 1] + M) % M;
                    const int z = d.dims == 3 ? (k - cs[3 * v + 2] + K) % K : 0;
                    plain = t[z + y * K + x * K * M] == LUMA_SITE_FLUID;
                }
                if (plain) fast[id] = 1;
                else if (ty == LUMA_SITE_TL_TO_FINER) late.push_back(id);
                else gen.push_back(id);
            }
    // the transition sites to finer grids last: only they read the
    // sub-grids' results (coalesce) or write their macroscopic fields, so the
    // rest of the list can run beside the sub-grids' steps
    g->ngen_early = (int)gen.size();
    gen.insert(gen.end(), late.begin(), late.end());
    CK(cudaMalloc(&g->fast, g->n));
    CK(cudaMemcpy(g->fast, fast.data(), g->n, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&g->gen_ids, std::max<size_t>(1, gen.size()) * sizeof(int)));
    if (!gen.empty()) CK(cudaMemcpy(g->gen_ids, gen.data(), gen.size() * sizeof(int), cudaMemcpyHostToDevice));
    g->ngen = (int)gen.size();
    return LUMA_OK;
}

namespace {

StepArgs make_args(luma_gpu_grid *g, int subcycle) {
    const luma_grid_desc &d = g->d;
    StepArgs a;
    memset(&a, 0, sizeof a);
    a.N = d.N; a.M = d.M; a.K = d.K; a.ncell = (int)g->n;
    a.typ = g->typ;
    a.f = g->f[g->cur];
    a.fNew = g->f[g->cur ^ 1];
    a.fOut = a.fNew;
    luma_bfl_args(g, a);
    if (g->tav) {
        a.tav_rho = g->tav;
        a.tav_u = g->tav + g->n;
        a.tav_uu = g->tav + g->n * (1 + d.dims);
        a.tav_t = g->t;
    }
    a.defer = g->fuse ? g->defer : nullptr;
    a.u = g->u; a.rho = g->rho; a.force = g->force;
    a.ux_in = g->uxin; a.uy_in = g->uyin; a.uz_in = g->uzin;
    a.omega = d.omega; a.rho0 = d.rho_in; a.cs2 = g->cs2; a.csmag = d.csmag;
    a.omegaf = (float)a.omega; a.rho0f = (float)a.rho0; a.cs2f = (float)a.cs2; a.csmag2f = (float)(a.csmag * a.csmag);
    a.pdelta = d.pressure_delta;
    a.has_ramp = d.velocity_ramp > 0.0;
    a.ramp_stream = ramp(d, g->t * d.dt);
    a.ramp_reg = ramp(d, (g->t + 1) * d.dt);
    a.flags = d.flags; a.collision = d.collision; a.subcycle = subcycle;
    a.forcing = (d.flags & (LUMA_FLAG_IBM | LUMA_FLAG_GRAVITY)) != 0;
    a.ibm_split = (d.flags & LUMA_FLAG_IBM) != 0;
    a.level = d.level;
    a.unsupported = g->unsup;
    if (g->parent) {
        a.parent_f = g->parent->f[g->parent->cur];
        a.pN = g->parent->d.N; a.pM = g->parent->d.M; a.pK = g->parent->d.K;
        for (int q = 0; q < 6; ++q) a.lims[q] = d.coarse_lims[q];
    }
    a.nchild = (int)g->kids.size();
    for (int s = 0; s < a.nchild && s < kMaxChildren; ++s) {
        luma_gpu_grid *c = g->kids[s];
        a.child[s].f = c->f[c->cur];
        a.child[s].u = c->u;
        a.child[s].rho = c->rho;
        a.child[s].N = c->d.N; a.child[s].M = c->d.M; a.child[s].K = c->d.K;
        for (int q = 0; q < 6; ++q) a.child[s].lims[q] = c->d.coarse_lims[q];
    }
    return a;
}

bool bulk_eligible(const luma_gpu_grid *g, const int32_t *typ) {
    const luma_grid_desc &d = g->d;
    if (g->parent || !g->kids.empty()) return false;
    if (d.collision != LUMA_COLL_BGK) return false;
    if (d.N > 65535 || d.M > 65535) return false;  // grid.y / grid.z launch limits
    if (d.flags & (LUMA_FLAG_IBM | LUMA_FLAG_GRAVITY | LUMA_FLAG_REGULARISED | LUMA_FLAG_TWO_BUFFER |
                   LUMA_FLAG_TIME_AVERAGES))
        return false;
    for (size_t i = 0; i < g->n; ++i)
        if (typ[i] != LUMA_SITE_FLUID) return false;
    return true;
}

void set_tree_stream(luma_gpu_grid *g, cudaStream_t s) {
    g->stream = s;
    for (luma_gpu_grid *c : g->kids) set_tree_stream(c, s);
}

// A grid with sub-grids whose interior sites run in their own kernel: those
// sites read and write nothing the sub-grids' steps touch (the sub-grids
// read this grid's pre-step populations for explode; coalesce and the
// transition sites are in the list kernel), so the interior kernel runs
// beside the sub-grids' two sub-steps, which go to a high-priority stream;
// the list kernel and everything after it wait for both.
bool overlap_kids(const luma_gpu_grid *g) {
    return !g->kids.empty() && g->fast && !g->bulk && !g->adj && g->kid_stream && g->ev_fork && g->ev_join;
}

// The interior kernel and the listed sites' kernel read the populations
// of the last step and write only their own sites (populations, u, rho,
// time averages), so the list may run on its own stream beside the
// interior: on the small grids of a refinement tree each is a short,
// latency-bound launch on the sub-grids' dependency chain.
bool split_list(const luma_gpu_grid *g) {
    return g->fast && !g->bulk && !g->adj && g->list_stream && g->ev_lfork && g->ev_ljoin;
}

int step_grid(luma_gpu_grid *g, int subcycle, bool write_macro) {
    if (g->d.reynolds_ramp > 0.0) update_reynolds(g);
    const luma_grid_desc &d = g->d;
    cudaStream_t s = g->stream;
    const bool overlap = overlap_kids(g);
    // On an IBM grid without bodies of its own, the deferred sites (solid,
    // refined, velocity) are collided from values nothing else in the step
    // writes (their streamed populations are left as they are, the force is
    // the reset's zero, no phase B or velocity update runs): that collision
    // runs beside the sub-grids instead of after them.
    const bool early_c = overlap && (d.flags & LUMA_FLAG_IBM) && g->fuse && !(g->ibm && g->ibm->has_bodies) &&
                         g->nreg == 0 && g->nvelu == 0 && !g->adj;
    if (overlap) {
        StepArgs ai = make_args(g, subcycle);
        ai.macro_out = write_macro || (d.flags & (LUMA_FLAG_GRAVITY | LUMA_FLAG_REGULARISED)) ? 1 : 0;
        if (g->ibm && g->ibm->has_bodies) {
            int rc = luma_ibm_reset_forces(g, ai);
            if (rc) return rc;
        }
        CK(cudaEventRecord(g->ev_fork, s));
        CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
            return launch_general_phaseA<decltype(q)::value, decltype(p)>(ai, g->wall, g->fast, g->gen_ids, g->ngen, s,
                                                                          kPhaseAInterior);
        }));
        // the early list and the early deferred collision beside the
        // interior: the list's phase A skips the solid, refined and velocity
        // sites, which are the deferred sites here, the collision writes only
        // those sites' new populations, and both only read u and rho at
        // velocity sites; neither touches the interior sites' outputs
        const bool side = (g->ngen_early > 0 || early_c) && split_list(g);
        cudaStream_t ls = side ? g->list_stream : s;
        if (side) CK(cudaStreamWaitEvent(g->list_stream, g->ev_fork, 0));
        if (g->ngen_early > 0)
            CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
                return launch_general_phaseA<decltype(q)::value, decltype(p)>(ai, g->wall, g->fast, g->gen_ids,
                                                                              g->ngen_early, ls, kPhaseAList);
            }));
        if (early_c)
            CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
                return launch_general_phaseC<decltype(q)::value, decltype(p)>(ai, g->defer_ids, g->ndefer, ls);
            }));
        if (side) CK(cudaEventRecord(g->ev_ljoin, g->list_stream));
        CK(cudaStreamWaitEvent(g->kid_stream, g->ev_fork, 0));
        for (luma_gpu_grid *c : g->kids) set_tree_stream(c, g->kid_stream);
        int rc = LUMA_OK;
        for (luma_gpu_grid *c : g->kids)
            for (int it = 0; it < 2 && rc == LUMA_OK; ++it) rc = step_grid(c, it, true);
        for (luma_gpu_grid *c : g->kids) set_tree_stream(c, s);
        if (rc) return rc;
        CK(cudaEventRecord(g->ev_join, g->kid_stream));
        CK(cudaStreamWaitEvent(s, g->ev_join, 0));
        if (side) CK(cudaStreamWaitEvent(s, g->ev_ljoin, 0));
    } else {
        for (luma_gpu_grid *c : g->kids)
            for (int it = 0; it < 2; ++it) {
                int rc = step_grid(c, it, true);
                if (rc) return rc;
            }
    }
    if (g->bulk) {
        CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
            return launch_aa<decltype(q)::value, decltype(p)>(g->f[0], g->u, g->rho, d.N, d.M, d.K, d.omega,
                                                              d.rho_in, g->aa_odd == 0, write_macro, s);
        }));
        g->aa_odd ^= 1;
        ++g->t;
        return LUMA_OK;
    }
    StepArgs a = make_args(g, subcycle);
    // Interior u and rho are read after the step (the caller's download or
    // reduction after its last step), by the reset of a gravity force (the
    // old rho) and by the regularised BCs' extrapolation; otherwise the
    // step that follows recomputes them before any use.
    a.macro_out = write_macro || (d.flags & (LUMA_FLAG_GRAVITY | LUMA_FLAG_REGULARISED)) ? 1 : 0;
    if (g->adj) luma_adj_redirect(g, a);
    if (g->ibm && g->ibm->has_bodies && !overlap) {
        int rc = luma_ibm_reset_forces(g, a);
        if (rc) return rc;
    }
    const int list0 = overlap ? g->ngen_early : 0;  // the rest of the list ran beside the sub-grids
    if (!overlap && g->kids.empty() && g->ngen > 0 && split_list(g)) {
        CK(cudaEventRecord(g->ev_lfork, s));
        CK(cudaStreamWaitEvent(g->list_stream, g->ev_lfork, 0));
        CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
            return launch_general_phaseA<decltype(q)::value, decltype(p)>(a, g->wall, g->fast, g->gen_ids, g->ngen,
                                                                          g->list_stream, kPhaseAList);
        }));
        CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
            return launch_general_phaseA<decltype(q)::value, decltype(p)>(a, g->wall, g->fast, g->gen_ids, g->ngen, s,
                                                                          kPhaseAInterior);
        }));
        CK(cudaEventRecord(g->ev_ljoin, g->list_stream));
        CK(cudaStreamWaitEvent(s, g->ev_ljoin, 0));
    } else {
        CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
            return launch_general_phaseA<decltype(q)::value, decltype(p)>(a, g->wall, g->fast, g->gen_ids + list0,
                                                                          g->ngen - list0, s,
                                                                          overlap ? kPhaseALate : kPhaseAAll);
        }));
    }
    if (g->nreg)
        CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
            return launch_general_phaseB<decltype(q)::value, decltype(p)>(a, g->wall, g->reg, g->nreg, s);
        }));
    if (g->nvelu) {
        if (d.precision == LUMA_PREC_FP64) CK(launch_velocity_u<P64>(a, d.dims, g->velu, g->nvelu, s));
        else CK(launch_velocity_u<P32>(a, d.dims, g->velu, g->nvelu, s));
    }
    if (a.ibm_split) {
        if (g->ibm && g->ibm->has_bodies) {
            int rc = luma_ibm_apply(g, a);
            if (rc) return rc;
        }
        if (g->adj) {
            int rc = luma_adj_step_hook(g, a);
            if (rc) return rc;
        }
        if (!early_c)
            CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
                return launch_general_phaseC<decltype(q)::value, decltype(p)>(a, g->fuse ? g->defer_ids : nullptr,
                                                                              g->ndefer, s);
            }));
    }
    g->cur ^= 1;
    ++g->t;
    return LUMA_OK;
}

}  // namespace

// ---- two steps of the tree as a CUDA graph ----------------------------------
//
// On grids of modest size a step is a handful of short kernels, and the host
// launch gaps between them cost as much as the kernels.  luma_gpu_step then
// runs pairs of steps as one CUDA graph: captured once (on a private stream,
// then launched on the caller's), replayed while everything it baked in is
// unchanged.  Two steps bring every grid's buffer and storage parity back,
// so one graph serves every pair.  The signature below lists what a capture
// bakes in (device pointers, parities, sizes, paths); any change recaptures.
// Not used when a step carries host logic between its kernels (velocity
// ramp: arguments change every step; a recorded adjoint), or while the
// caller's stream is itself being captured.  Moving bodies are captured:
// their FSI loop runs its test on the device.

namespace luma {
struct StepGraph {
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<uintptr_t> sig;
    bool broken = false;  // a capture failed: steps run one launch at a time
};
}  // namespace luma

namespace {

constexpr int kGraphMinSteps = 4;

void tree_signature(const luma_gpu_grid *g, std::vector<uintptr_t> &s) {
    auto P = [&](const void *p) { s.push_back((uintptr_t)p); };
    auto V = [&](long long v) { s.push_back((uintptr_t)v); };
    P(g); P(g->f[0]); P(g->f[1]); P(g->u); P(g->rho); P(g->force); P(g->typ); P(g->wall); P(g->reg); P(g->velu);
    P(g->uxin); P(g->defer); P(g->defer_ids); P(g->fast); P(g->gen_ids); P(g->adj); P(g->bfl);
    V(g->cur); V(g->aa_odd); V(g->bulk); V(g->fuse); V(g->ngen); V(g->ngen_early); V(g->ndefer); V(g->nreg);
    V(g->nvelu);
    V(g->d.flags);
    luma_bfl_signature(g, s);
    if (g->ibm) {
        const IbmDevice &d = g->ibm->dev;
        P(d.vel); P(d.eps); P(d.ds); P(d.area); P(d.F); P(d.irho); P(d.imom); P(d.moff); P(d.msite);
        P(d.smarker); P(d.mdelta); P(d.usite); P(d.uoff); P(d.uref);
        V(d.nm); V(d.nsup); V(d.nu); V(g->ibm->has_bodies); V(g->ibm->ready); V(g->ibm->has_flexible);
        const FemDevice &fe = g->ibm->fem;
        P(fe.U); P(fe.M); P(fe.K); P(fe.fsi_state); P(fe.flex.pos); P(fe.flex.supp); P(g->ibm->u_n);
        V(fe.nfil); V(fe.k_in_smem); V(fe.eps_in_smem);
    }
    V((long long)g->kids.size());
    for (const luma_gpu_grid *c : g->kids) tree_signature(c, s);
}

bool graph_safe(const luma_gpu_grid *g) {
    if (g->d.velocity_ramp > 0.0 || g->d.reynolds_ramp > 0.0 || g->adj || g->tav) return false;
    for (const luma_gpu_grid *c : g->kids)
        if (!graph_safe(c)) return false;
    return true;
}

void save_clocks(const luma_gpu_grid *g, std::vector<int> &v) {
    v.push_back(g->t); v.push_back(g->cur); v.push_back(g->aa_odd);
    for (const luma_gpu_grid *c : g->kids) save_clocks(c, v);
}
void restore_clocks(luma_gpu_grid *g, const std::vector<int> &v, size_t &i) {
    g->t = v[i++]; g->cur = v[i++]; g->aa_odd = v[i++];
    for (luma_gpu_grid *c : g->kids) restore_clocks(c, v, i);
}
// A replayed pair of root steps: every grid's counter advances by its own
// steps (two per parent step on a child); parities are back where they were.
void advance_t(luma_gpu_grid *g, int steps) {
    g->t += steps;
    for (luma_gpu_grid *c : g->kids) advance_t(c, 2 * steps);
}

void free_graph(luma_gpu_grid *g) {
    if (!g->graph) return;
    if (g->graph->exec) cudaGraphExecDestroy(g->graph->exec);
    if (g->graph->cap) cudaStreamDestroy(g->graph->cap);
    delete g->graph;
    g->graph = nullptr;
}

int step_grid(luma_gpu_grid *g, int subcycle, bool write_macro);

// Runs `pairs` pairs of root steps as graph launches; returns the pairs run
// (0 when the tree cannot be captured: the caller steps directly).
int run_step_pairs(luma_gpu_grid *root, int pairs, int *done) {
    *done = 0;
    if (pairs <= 0 || !graph_safe(root)) return LUMA_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(root->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return LUMA_OK;
    }
    if (!root->graph) root->graph = new StepGraph();
    StepGraph &G = *root->graph;
    if (G.broken) return LUMA_OK;
    std::vector<uintptr_t> sig;
    tree_signature(root, sig);
    if (!G.exec || sig != G.sig) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        G.exec = nullptr;
        if (!G.cap && cudaStreamCreateWithFlags(&G.cap, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            G.broken = true;
            return LUMA_OK;
        }
        std::vector<int> clocks;
        save_clocks(root, clocks);
        const cudaStream_t user = root->stream;
        set_tree_stream(root, G.cap);
        int rc = LUMA_OK;
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(G.cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            rc = step_grid(root, 0, false);
            if (rc == LUMA_OK) rc = step_grid(root, 0, false);
            if (cudaStreamEndCapture(G.cap, &graph) != cudaSuccess) rc = LUMA_E_CUDA;
        } else {
            rc = LUMA_E_CUDA;
        }
        set_tree_stream(root, user);
        // node priorities as captured: the sub-grids' chain (high-priority
        // stream) is scheduled ahead of the parent's interior blocks
        if (rc == LUMA_OK && graph &&
            cudaGraphInstantiate(&G.exec, graph, cudaGraphInstantiateFlagUseNodePriority) != cudaSuccess)
            rc = LUMA_E_CUDA;
        if (graph) cudaGraphDestroy(graph);
        if (rc != LUMA_OK) {
            // nothing ran: put the host-side clocks back and step directly
            cudaGetLastError();
            size_t i = 0;
            restore_clocks(root, clocks, i);
            G.exec = nullptr;
            G.broken = true;
            return LUMA_OK;
        }
        G.sig = sig;
        // the capture advanced the host-side clocks by one pair: run it
        CK(cudaGraphLaunch(G.exec, root->stream));
        *done = 1;
    }
    for (; *done < pairs; ++*done) {
        CK(cudaGraphLaunch(G.exec, root->stream));
        advance_t(root, 2);
    }
    return LUMA_OK;
}

void free_grid(luma_gpu_grid *g) {
    if (!g) return;
    for (luma_gpu_grid *c : g->kids) free_grid(c);
    free_graph(g);
    luma_ibm_free(g);
    luma_adj_free(g);
    luma_bfl_free(g);
    luma_io_free(g);
    cudaFree(g->typ);
    cudaFree(g->f[0]);
    cudaFree(g->f[1]);
    cudaFree(g->u);
    cudaFree(g->rho);
    cudaFree(g->force);
    cudaFree(g->uxin);
    cudaFree(g->uyin);
    cudaFree(g->uzin);
    cudaFree(g->wall);
    cudaFree(g->reg);
    cudaFree(g->velu);
    cudaFree(g->acc);
    cudaFree(g->unsup);
    cudaFree(g->tav);
    cudaFree(g->defer);
    cudaFree(g->defer_ids);
    cudaFree(g->fast);
    cudaFree(g->gen_ids);
    if (g->kid_stream) cudaStreamDestroy(g->kid_stream);
    if (g->ev_fork) cudaEventDestroy(g->ev_fork);
    if (g->ev_join) cudaEventDestroy(g->ev_join);
    if (g->list_stream) cudaStreamDestroy(g->list_stream);
    if (g->ev_lfork) cudaEventDestroy(g->ev_lfork);
    if (g->ev_ljoin) cudaEventDestroy(g->ev_ljoin);
    delete g;
}

}  // namespace

// The launch-relevant state of a grid tree (buffers, lists, counts, flags):
// a graph captured under one signature replays correctly while it holds.
void luma_tree_signature(const luma_gpu_grid *g, std::vector<uintptr_t> &sig) {
    sig.clear();
    tree_signature(g, sig);
}

extern "C" {

int luma_gpu_abi_version(void) { return LUMA_GPU_ABI_VERSION; }

const char *luma_gpu_last_error_string(void) { return g_last_error.c_str(); }

int luma_gpu_grid_create(const luma_grid_desc *desc, luma_gpu_grid *parent, luma_gpu_grid **out) {
    if (!desc || !out) return luma_set_error(LUMA_E_INVALID, "null argument");
    *out = nullptr;
    const luma_grid_desc &d = *desc;
    if (d.abi_version != LUMA_GPU_ABI_VERSION)
        return luma_set_error(LUMA_E_INVALID, "ABI version %d, library is %d", d.abi_version, LUMA_GPU_ABI_VERSION);
    if (!((d.dims == 2 && d.Q == 9) || (d.dims == 3 && (d.Q == 19 || d.Q == 27))))
        return luma_set_error(LUMA_E_INVALID, "unsupported lattice D%dQ%d", d.dims, d.Q);
    if (d.N <= 0 || d.M <= 0 || d.K <= 0 || (d.dims == 2 && d.K != 1))
        return luma_set_error(LUMA_E_INVALID, "bad grid size %dx%dx%d", d.N, d.M, d.K);
    if ((double)d.N * d.M * d.K * d.Q >= 9.0e18) return luma_set_error(LUMA_E_INVALID, "grid too large");
    if ((size_t)d.N * d.M * d.K > 0x7fffffffu)
        return luma_set_error(LUMA_E_INVALID, "grid has more than 2^31-1 sites");
    if (d.precision != LUMA_PREC_FP64 && d.precision != LUMA_PREC_FP32_SHIFTED)
        return luma_set_error(LUMA_E_INVALID, "unknown precision %d", d.precision);
    if (d.collision < LUMA_COLL_BGK || d.collision > LUMA_COLL_KBC)
        return luma_set_error(LUMA_E_INVALID, "unknown collision %d", d.collision);
    if (d.collision == LUMA_COLL_KBC && d.dims == 3 && d.Q != 27)
        return luma_set_error(LUMA_E_INVALID, "3D KBC needs D3Q27 (the reference forces L_NUM_VELS 27)");
    if (d.flags & LUMA_FLAG_REGULARISED && d.Q == 27)
        return luma_set_error(LUMA_E_INVALID, "Cannot use regularised boundaries with D3Q27");
    if (!(d.omega > 0.0) || (d.omega >= 2.0 && d.collision != LUMA_COLL_BGK_SMAG))
        return luma_set_error(LUMA_E_INVALID, "relaxation frequency omega=%g out of range", d.omega);
    if ((d.flags & LUMA_FLAG_TIME_AVERAGES) && (d.flags & LUMA_FLAG_REGULARISED))
        return luma_set_error(LUMA_E_INVALID, "time averages with regularised BCs: the reference's extrapolation "
                                              "re-runs the macroscopic step at neighbour sites (not reproduced)");
    if (d.reynolds_ramp < 0.0 || (d.reynolds_ramp > 0.0 && !(d.re > 0.0)))
        return luma_set_error(LUMA_E_INVALID, "a Reynolds ramp needs re > 0 (reynolds_ramp=%g, re=%g)",
                              d.reynolds_ramp, d.re);
    if (!d.lattyp) return luma_set_error(LUMA_E_INVALID, "lattyp is required");
    if (!d.ux_in || !d.uy_in || !d.uz_in) return luma_set_error(LUMA_E_INVALID, "inlet profile arrays are required");
    if (parent) {
        if (parent->bulk_fixed) return luma_set_error(LUMA_E_STATE, "parent grid already holds state");
        if ((int)parent->kids.size() >= kMaxChildren) return luma_set_error(LUMA_E_INVALID, "too many sub-grids");
        if (parent->d.dims != d.dims || parent->d.Q != d.Q || parent->d.precision != d.precision)
            return luma_set_error(LUMA_E_INVALID, "sub-grid lattice/precision differs from its parent");
        if (d.level != parent->d.level + 1) return luma_set_error(LUMA_E_INVALID, "sub-grid level must be parent+1");
        // Explode reads parent site (fine/2 + lim) and coalesce reads the 2^d
        // children of each covered coarse site: both stay inside the two grids
        // when the limits lie on the parent and the child spans them exactly.
        const int *L = d.coarse_lims;
        const int pdim[3] = {parent->d.N, parent->d.M, parent->d.K};
        const int cdim[3] = {d.N, d.M, d.K};
        for (int a = 0; a < d.dims; ++a)
            if (L[2 * a] < 0 || L[2 * a + 1] >= pdim[a] || L[2 * a] > L[2 * a + 1] ||
                cdim[a] != 2 * (L[2 * a + 1] - L[2 * a] + 1))
                return luma_set_error(LUMA_E_INVALID, "sub-grid coarse limits/size inconsistent on axis %d", a);
    }
    luma_gpu_grid *g = new (std::nothrow) luma_gpu_grid();
    if (!g) return luma_set_error(LUMA_E_NOMEM, "host allocation failed");
    g->d = d;
    g->n = (size_t)d.N * d.M * d.K;
    {
        const double cs = 1.0 / std::sqrt(3.0);
        g->cs2 = cs * cs;
    }
    g->parent = parent;
    g->stream = parent ? parent->stream : nullptr;
    int rc = LUMA_OK;
    auto fail = [&](int code) {
        free_grid(g);
        return code;
    };
    std::vector<uint8_t> typ8(g->n);
    for (size_t i = 0; i < g->n; ++i) {
        if (d.lattyp[i] < 0 || d.lattyp[i] > LUMA_SITE_EXTRAPOLATE_RIGHT) {
            luma_set_error(LUMA_E_INVALID, "site %zu has unknown label %d", i, d.lattyp[i]);
            return fail(LUMA_E_INVALID);
        }
        typ8[i] = (uint8_t)d.lattyp[i];
    }
    const size_t rs = real_size(g);
    const size_t popb = g->n * d.Q * rs;
#define CKF(call)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            luma_set_error(e_ == cudaErrorMemoryAllocation ? LUMA_E_NOMEM : LUMA_E_CUDA, "%s: %s", #call, \
                           cudaGetErrorString(e_));                                               \
            return fail(e_ == cudaErrorMemoryAllocation ? LUMA_E_NOMEM : LUMA_E_CUDA);          \
        }                                                                                         \
    } while (0)
    CKF(cudaMalloc(&g->typ, g->n));
    CKF(cudaMemcpy(g->typ, typ8.data(), g->n, cudaMemcpyHostToDevice));
    g->bulk = bulk_eligible(g, d.lattyp);
    CKF(cudaMalloc(&g->f[0], popb));
    if (!g->bulk) CKF(cudaMalloc(&g->f[1], popb));
    CKF(cudaMalloc(&g->u, g->n * d.dims * rs));
    CKF(cudaMalloc(&g->rho, g->n * rs));
    CKF(cudaMemset(g->u, 0, g->n * d.dims * rs));
    CKF(cudaMemset(g->rho, 0, g->n * rs));
    if (d.flags & (LUMA_FLAG_IBM | LUMA_FLAG_GRAVITY)) {
        CKF(cudaMalloc(&g->force, g->n * d.dims * rs));
        CKF(cudaMemset(g->force, 0, g->n * d.dims * rs));
    }
    CKF(cudaMalloc(&g->uxin, d.M * sizeof(double)));
    CKF(cudaMalloc(&g->uyin, d.M * sizeof(double)));
    CKF(cudaMalloc(&g->uzin, d.M * sizeof(double)));
    CKF(cudaMemcpy(g->uxin, d.ux_in, d.M * sizeof(double), cudaMemcpyHostToDevice));
    CKF(cudaMemcpy(g->uyin, d.uy_in, d.M * sizeof(double), cudaMemcpyHostToDevice));
    CKF(cudaMemcpy(g->uzin, d.uz_in, d.M * sizeof(double), cudaMemcpyHostToDevice));
    CKF(cudaMalloc(&g->acc, (size_t)(kReduceBlocks + 1) * 8 * sizeof(double)));
    CKF(cudaMalloc(&g->unsup, sizeof(int)));
    CKF(cudaMemset(g->unsup, 0, sizeof(int)));
    if (d.flags & LUMA_FLAG_TIME_AVERAGES) {
        const size_t nt = g->n * (size_t)(1 + d.dims + 3 * d.dims - 3);
        CKF(cudaMalloc(&g->tav, nt * sizeof(double)));
        CKF(cudaMemset(g->tav, 0, nt * sizeof(double)));
    }
    rc = build_site_tables(g, d.lattyp, d.xpos, d.ypos, d.zpos);
    if (rc) return fail(rc);
    g->htyp.assign(d.lattyp, d.lattyp + g->n);
    g->nbfl_sites = (size_t)std::count(g->htyp.begin(), g->htyp.end(), (uint8_t)LUMA_SITE_BFL);
    if ((rc = luma_update_defer(g))) return fail(rc);
    if ((rc = luma_build_interior(g))) return fail(rc);
    if (d.xpos) g->hx.assign(d.xpos, d.xpos + d.N);
    if (d.ypos) g->hy.assign(d.ypos, d.ypos + d.M);
    if (d.zpos) g->hz.assign(d.zpos, d.zpos + d.K);
    g->d.lattyp = nullptr;
    g->d.xpos = g->d.ypos = g->d.zpos = nullptr;
    g->d.ux_in = g->d.uy_in = g->d.uz_in = nullptr;
    {
        // the listed sites' kernel steps beside the interior kernel
        // (step_grid); without the stream both run in line
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (cudaStreamCreateWithPriority(&g->list_stream, cudaStreamNonBlocking, greatest) != cudaSuccess ||
            cudaEventCreateWithFlags(&g->ev_lfork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&g->ev_ljoin, cudaEventDisableTiming) != cudaSuccess)
            cudaGetLastError();
    }
    if (parent) {
        if (!parent->kid_stream) {
            // the parent's sub-grids step on a stream of the highest priority
            // beside its interior kernel (step_grid); without it they step in line
            int least = 0, greatest = 0;
            cudaDeviceGetStreamPriorityRange(&least, &greatest);
            if (cudaStreamCreateWithPriority(&parent->kid_stream, cudaStreamNonBlocking, greatest) != cudaSuccess ||
                cudaEventCreateWithFlags(&parent->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&parent->ev_join, cudaEventDisableTiming) != cudaSuccess)
                cudaGetLastError();
        }
        parent->kids.push_back(g);
        if (parent->bulk) {
            // A grid with sub-grids takes the general path; it holds no state yet.
            parent->bulk = false;
            if (!parent->f[1] && cudaMalloc(&parent->f[1], parent->n * parent->d.Q * real_size(parent)) != cudaSuccess) {
                parent->kids.pop_back();
                luma_set_error(LUMA_E_NOMEM, "second population buffer for parent");
                return fail(LUMA_E_NOMEM);
            }
            if ((rc = luma_build_interior(parent))) {
                parent->kids.pop_back();
                return fail(rc);
            }
        }
    }
    *out = g;
    return LUMA_OK;
#undef CKF
}

int luma_gpu_grid_destroy(luma_gpu_grid *g) {
    if (!g) return LUMA_OK;
    if (g->parent) {
        auto &k = g->parent->kids;
        for (size_t i = 0; i < k.size(); ++i)
            if (k[i] == g) { k.erase(k.begin() + i); break; }
    }
    free_grid(g);
    return LUMA_OK;
}

int luma_gpu_set_stream(luma_gpu_grid *root, void *cuda_stream) {
    if (!root) return luma_set_error(LUMA_E_INVALID, "null grid");
    set_tree_stream(root, static_cast<cudaStream_t>(cuda_stream));
    return LUMA_OK;
}

}  // extern "C"

namespace {

// The device address of a host array the GPU can reach in place (pinned,
// mapped host memory), or null: the layout conversions read and write such
// arrays directly; anything else goes through a device staging buffer.
template <class T>
T *device_view(T *h) {
    if (!h) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost && at.devicePointer ? static_cast<T *>(at.devicePointer) : nullptr;
}

// A device staging buffer for the host arrays of one transfer, allocated on
// first need on the stream and freed with it.
struct Stage {
    double *p = nullptr;
    size_t n = 0;
    cudaStream_t s;
    explicit Stage(size_t count, cudaStream_t st) : n(count), s(st) {}
    cudaError_t get(double **out) {
        if (!p) {
            cudaError_t e = cudaMallocAsync(&p, n * sizeof(double), s);
            if (e != cudaSuccess) return e;
        }
        *out = p;
        return cudaSuccess;
    }
    ~Stage() {
        if (p) cudaFreeAsync(p, s);
    }
};

}  // namespace

extern "C" {

int luma_gpu_upload_state(luma_gpu_grid *g, const double *f, const double *u, const double *rho,
                          const double *force_xyz, int t) {
    if (!g) return luma_set_error(LUMA_E_INVALID, "null grid");
    const luma_grid_desc &d = g->d;
    cudaStream_t s = g->stream;
    const size_t rs = real_size(g);
    int rc = LUMA_OK;
    {
        Stage stage(g->n * (size_t)(d.Q > d.dims ? d.Q : d.dims), s);
        // the array as the conversion reads it: in place, or copied to the stage
        auto source = [&](const double *h, size_t count, const double **out) -> int {
            if ((*out = device_view(h))) return LUMA_OK;
            double *st = nullptr;
            CK(stage.get(&st));
            CK(cudaMemcpyAsync(st, h, count * sizeof(double), cudaMemcpyHostToDevice, s));
            *out = st;
            return LUMA_OK;
        };
        auto run = [&]() -> int {
            if (f) {
                const double *src = nullptr;
                if (int r = source(f, g->n * d.Q, &src)) return r;
                const int layout = g->bulk ? kPopAAE : kPopPlain;
                CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
                    return launch_pop_in<decltype(q)::value, decltype(p)>(src, g->f[0], d.N, d.M, d.K, layout, d.rho_in, s);
                }));
                if (!g->bulk) CK(cudaMemcpyAsync(g->f[1], g->f[0], g->n * d.Q * rs, cudaMemcpyDeviceToDevice, s));
                g->cur = 0;
                g->aa_odd = 0;
            }
            auto vec_in = [&](const double *h, void *dst, int dims) -> int {
                const double *src = nullptr;
                if (int r = source(h, g->n * dims, &src)) return r;
                if (d.precision == LUMA_PREC_FP64) CK(launch_vec_in<P64>(src, dst, g->n, dims, s));
                else CK(launch_vec_in<P32>(src, dst, g->n, dims, s));
                return LUMA_OK;
            };
            if (u && (rc = vec_in(u, g->u, d.dims))) return rc;
            if (rho && (rc = vec_in(rho, g->rho, 1))) return rc;
            // force_xyz is ignored on grids without a force field (the reference
            // allocates it only under L_IBM_ON or L_GRAVITY_ON).
            if (force_xyz && g->force && (rc = vec_in(force_xyz, g->force, d.dims))) return rc;
            return LUMA_OK;
        };
        rc = run();
    }
    CK(cudaStreamSynchronize(s));
    if (rc) return rc;
    g->t = t;
    g->bulk_fixed = true;
    return LUMA_OK;
}

int luma_gpu_download_state(luma_gpu_grid *g, double *f, double *u, double *rho, double *force_xyz) {
    if (!g) return luma_set_error(LUMA_E_INVALID, "null grid");
    const luma_grid_desc &d = g->d;
    cudaStream_t s = g->stream;
    int rc = LUMA_OK;
    {
        Stage stage(g->n * (size_t)(d.Q > d.dims ? d.Q : d.dims), s);
        // the conversion writes a mapped host array in place, else the stage,
        // which is then copied out
        auto target = [&](double *h, double **out) -> int {
            if ((*out = device_view(h))) return LUMA_OK;
            CK(stage.get(out));
            return LUMA_OK;
        };
        auto finish = [&](double *h, const double *dst, size_t count) -> int {
            if (dst != device_view(h))
                CK(cudaMemcpyAsync(h, dst, count * sizeof(double), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));   // the stage is reused by the next array
            return LUMA_OK;
        };
        auto run = [&]() -> int {
            if (f) {
                double *dst = nullptr;
                if (int r = target(f, &dst)) return r;
                const int layout = g->bulk ? (g->aa_odd ? kPopAAO : kPopAAE) : kPopPlain;
                const void *src = g->bulk ? g->f[0] : g->f[g->cur];
                CK(dispatch(d.Q, d.precision, [&](auto q, auto p) {
                    return launch_pop_out<decltype(q)::value, decltype(p)>(src, dst, d.N, d.M, d.K, layout, d.rho_in, s);
                }));
                if (int r = finish(f, dst, g->n * d.Q)) return r;
            }
            auto vec_out = [&](const void *src, double *h, int dims) -> int {
                double *dst = nullptr;
                if (int r = target(h, &dst)) return r;
                if (d.precision == LUMA_PREC_FP64) CK(launch_vec_out<P64>(src, dst, g->n, dims, s));
                else CK(launch_vec_out<P32>(src, dst, g->n, dims, s));
                return finish(h, dst, g->n * dims);
            };
            if (u && (rc = vec_out(g->u, u, d.dims))) return rc;
            if (rho && (rc = vec_out(g->rho, rho, 1))) return rc;
            if (force_xyz) {
                if (!g->force) memset(force_xyz, 0, g->n * d.dims * sizeof(double));
                else if ((rc = vec_out(g->force, force_xyz, d.dims))) return rc;
            }
            return LUMA_OK;
        };
        rc = run();
    }
    CK(cudaStreamSynchronize(s));
    return rc;
}

int luma_gpu_download_time_averages(luma_gpu_grid *g, double *rho_ta, double *ui_ta, double *uiuj_ta) {
    if (!g || !rho_ta || !ui_ta || !uiuj_ta) return luma_set_error(LUMA_E_INVALID, "null argument");
    if (!g->tav) return luma_set_error(LUMA_E_STATE, "grid created without LUMA_FLAG_TIME_AVERAGES");
    const int D = g->d.dims, npq = 3 * D - 3;
    const size_t n = g->n;
    std::vector<double> h(n * (size_t)(1 + D + npq));
    CK(cudaStreamSynchronize(g->stream));
    CK(cudaMemcpy(h.data(), g->tav, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t id = 0; id < n; ++id) {
        rho_ta[id] = h[id];
        for (int p = 0; p < D; ++p) ui_ta[p + id * D] = h[(1 + p) * n + id];
        for (int q = 0; q < npq; ++q) uiuj_ta[q + id * npq] = h[(1 + D + q) * n + id];
    }
    return LUMA_OK;
}

int luma_gpu_get_time(const luma_gpu_grid *g, int *t) {
    if (!g || !t) return luma_set_error(LUMA_E_INVALID, "null argument");
    *t = g->t;
    return LUMA_OK;
}

static int check_tree(const luma_gpu_grid *g) {
    if (g->nbfl_sites && !g->bfl)
        return luma_set_error(LUMA_E_STATE, "grid L%d has %zu BFL sites and no BFL body (luma_gpu_bfl_set)",
                              g->d.level, g->nbfl_sites);
    if (g->tav && g->ibm && g->ibm->has_flexible)
        return luma_set_error(LUMA_E_INVALID, "time averages with flexible bodies: the FSI loop re-runs the "
                                              "macroscopic step per sub-iteration (not reproduced)");
    for (const luma_gpu_grid *c : g->kids)
        if (int rc = check_tree(c)) return rc;
    return LUMA_OK;
}

int luma_gpu_step(luma_gpu_grid *root, int nsteps) {
    if (!root) return luma_set_error(LUMA_E_INVALID, "null grid");
    if (root->parent) return luma_set_error(LUMA_E_INVALID, "luma_gpu_step takes the level-0 grid");
    if (nsteps < 0) return luma_set_error(LUMA_E_INVALID, "negative step count");
    if (int rc = check_tree(root)) return rc;
    if (nsteps >= kGraphMinSteps) {
        // pairs as graph launches; the last step runs directly (it writes u, rho)
        int done = 0;
        const int rc = run_step_pairs(root, (nsteps - 1) / 2, &done);
        if (rc) return rc;
        nsteps -= 2 * done;
    }
    for (int s = 0; s < nsteps; ++s) {
        int rc = step_grid(root, 0, s == nsteps - 1);
        if (rc) return rc;
    }
    return LUMA_OK;
}

// Reads and clears the unsupported-site flag of every grid of a tree; the
// first grid (parent before its sub-grids) with a code set is reported.
static int take_unsupported(luma_gpu_grid *g, int *code, int *level, int *region) {
    int h = 0;
    CK(cudaMemcpyAsync(&h, g->unsup, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    if (h) {
        CK(cudaMemsetAsync(g->unsup, 0, sizeof(int), g->stream));
        if (!*code) { *code = h; *level = g->d.level; *region = g->d.region; }
    }
    if (g->ibm && g->ibm->has_flexible && g->ibm->ready)
        if (int rc = luma_fem_take_error(g)) return rc;
    for (luma_gpu_grid *c : g->kids)
        if (int rc = take_unsupported(c, code, level, region)) return rc;
    return LUMA_OK;
}

static int check_planes(const luma_gpu_grid *g, int i0, int nplanes, const void *buf) {
    if (!g || !buf) return luma_set_error(LUMA_E_INVALID, "null argument");
    if (g->bulk || !g->f[1]) return luma_set_error(LUMA_E_INVALID, "halo planes need a two-buffer grid (LUMA_FLAG_TWO_BUFFER)");
    if (nplanes <= 0 || i0 < 0 || i0 + nplanes > g->d.N)
        return luma_set_error(LUMA_E_INVALID, "planes %d..%d off the grid's %d x-planes", i0, i0 + nplanes - 1, g->d.N);
    return LUMA_OK;
}

int luma_gpu_planes_bytes(const luma_gpu_grid *g, int nplanes, size_t *bytes) {
    if (!g || !bytes || nplanes < 0) return luma_set_error(LUMA_E_INVALID, "bad argument");
    *bytes = (size_t)nplanes * g->d.M * g->d.K * g->d.Q * real_size(g);
    return LUMA_OK;
}

// Direction v's planes i0..i0+np-1 are one contiguous run of the SoA
// buffer (sites are x-major), so a transfer is one strided 2D copy of Q rows.
int luma_gpu_planes_export(luma_gpu_grid *g, int i0, int nplanes, void *buf) {
    if (int rc = check_planes(g, i0, nplanes, buf)) return rc;
    const size_t rs = real_size(g), plane = (size_t)g->d.M * g->d.K;
    const char *src = static_cast<const char *>(g->f[g->cur]) + i0 * plane * rs;
    CK(cudaMemcpy2DAsync(buf, nplanes * plane * rs, src, g->n * rs, nplanes * plane * rs, g->d.Q, cudaMemcpyDefault,
                         g->stream));
    return LUMA_OK;
}

int luma_gpu_planes_import(luma_gpu_grid *g, int i0, int nplanes, const void *buf) {
    if (int rc = check_planes(g, i0, nplanes, buf)) return rc;
    const size_t rs = real_size(g), plane = (size_t)g->d.M * g->d.K;
    char *dst = static_cast<char *>(g->f[g->cur]) + i0 * plane * rs;
    CK(cudaMemcpy2DAsync(dst, g->n * rs, buf, nplanes * plane * rs, nplanes * plane * rs, g->d.Q, cudaMemcpyDefault,
                         g->stream));
    return LUMA_OK;
}

int luma_gpu_synchronize(luma_gpu_grid *root) {
    if (!root) return luma_set_error(LUMA_E_INVALID, "null grid");
    CK(cudaStreamSynchronize(root->stream));
    int code = 0, level = 0, region = 0;
    if (int rc = take_unsupported(root, &code, &level, &region)) return rc;
    if (code)
        return luma_set_error(LUMA_E_INVALID, "grid L%d R%d: a site needed an operation outside the GPU path (code %d)",
                              level, region, code);
    return LUMA_OK;
}

int luma_gpu_reduce(luma_gpu_grid *g, luma_reduction *out) {
    if (!g || !out) return luma_set_error(LUMA_E_INVALID, "null argument");
    const luma_grid_desc &d = g->d;
    if (d.precision == LUMA_PREC_FP64) CK(launch_reduce<P64>(g->typ, g->rho, g->u, g->n, d.dims, g->acc, g->stream));
    else CK(launch_reduce<P32>(g->typ, g->rho, g->u, g->n, d.dims, g->acc, g->stream));
    double h[7];
    CK(cudaMemcpyAsync(h, g->acc, sizeof h, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    out->mass = h[0];
    out->momentum[0] = h[1];
    out->momentum[1] = h[2];
    out->momentum[2] = h[3];
    out->kinetic_energy = h[4];
    out->max_speed = h[5];
    out->nonfinite = (int64_t)h[6];
    return LUMA_OK;
}

}  // extern "C"
