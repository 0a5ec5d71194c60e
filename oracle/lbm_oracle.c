/*
 * ORACLE — test infrastructure only.  A plain-C restatement of the reference
 * LUMA v1.7.12 lattice-Boltzmann time step (GridObj::LBM_multi_opt and its
 * callees, src/GridObj_ops_lbm_optimised.cpp) used to check the CUDA path.
 * Only tests, the smoke check and the benchmark's CPU-baseline leg use it;
 * the product never links or calls it.
 *
 * It keeps the reference's arithmetic: FP64, the reference's operation
 * order, the reference's array-of-structures layout (f[v + id*Q]), two
 * population arrays swapped after every step, and the reference's quirks:
 *  - the 3D macroscopic step adds 0.5*F_z to the x-momentum (:833) unless
 *    LUMA_FLAG_FIX_MACRO3D is set;
 *  - KBC relaxes the pre-stream f (:1147,1296) unless LUMA_FLAG_FIX_KBC;
 *  - the forced-equilibrium velocity BC writes the current row's inlet
 *    velocity into the source site's u (:255-269);
 *  - transition-to-coarser sites are not collided (:144).
 * Parity of this restatement with the reference itself is pinned by the
 * golden fixtures in tests/golden (produced by the reference's own build).
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared [-fopenmp].
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/luma_gpu.h"

/* ---------------- lattice tables (src/stdafx.cpp:29-153) ---------------- */

static const int C9[9][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {1, 1, 0},
                             {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {0, 0, 0}};
static const double W9[9] = {1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 36.0,
                             1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 4.0 / 9.0};
static const int C19[19][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1},
                               {0, 0, -1}, {1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0},
                               {0, 1, 1}, {0, -1, -1}, {0, 1, -1}, {0, -1, 1}, {1, 0, 1},
                               {-1, 0, -1}, {-1, 0, 1}, {1, 0, -1}, {0, 0, 0}};
static const double W19[19] = {1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                               1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                               1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                               1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 3.0};
static const int C27[27][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1},
                               {0, 0, -1}, {0, 1, 1}, {0, -1, -1}, {0, 1, -1}, {0, -1, 1},
                               {1, 0, 1}, {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1}, {1, 1, 0},
                               {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 1, 1}, {-1, -1, -1},
                               {-1, -1, 1}, {1, 1, -1}, {-1, 1, 1}, {1, -1, -1}, {1, -1, 1},
                               {-1, 1, -1}, {0, 0, 0}};
static const double W27[27] = {
    2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  1.0 / 54.0,
    1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,
    1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0,
    1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 8.0 / 27.0};
/* Opposites and specular reflections (src/GridUtils.cpp:31-69). */
static const int OPP9[9] = {1, 0, 3, 2, 5, 4, 7, 6, 8};
static const int OPP19[19] = {1, 0, 3, 2, 5, 4, 7, 6, 9, 8, 11, 10, 13, 12, 15, 14, 17, 16, 18};
static const int OPP27[27] = {1,  0,  3,  2,  5,  4,  7,  6,  9,  8,  11, 10, 13, 12,
                              15, 14, 17, 16, 19, 18, 21, 20, 23, 22, 25, 24, 26};
static const int REF9[3][9] = {{1, 0, 2, 3, 7, 6, 5, 4, 8}, {0, 1, 3, 2, 6, 7, 4, 5, 8}, {0}};
static const int REF19[3][19] = {
    {1, 0, 2, 3, 4, 5, 9, 8, 7, 6, 10, 11, 12, 13, 16, 17, 14, 15, 18},
    {0, 1, 3, 2, 4, 5, 8, 9, 6, 7, 13, 12, 11, 10, 14, 15, 16, 17, 18},
    {0, 1, 2, 3, 5, 4, 6, 7, 8, 9, 12, 13, 10, 11, 17, 16, 15, 14, 18}};
static const int REF27[3][27] = {
    {1, 0, 2, 3, 4, 5, 6, 7, 8, 9, 13, 12, 11, 10, 17, 16, 15, 14, 22, 23, 24, 25, 18, 19, 20, 21, 26},
    {0, 1, 3, 2, 4, 5, 9, 8, 7, 6, 10, 11, 12, 13, 16, 17, 14, 15, 24, 25, 22, 23, 20, 21, 18, 19, 26},
    {0, 1, 2, 3, 5, 4, 8, 9, 6, 7, 12, 13, 10, 11, 14, 15, 16, 17, 21, 20, 19, 18, 25, 24, 23, 22, 26}};

#define SQ(x) ((x) * (x))
#define L_PI 3.14159265358979323846
#define L_SQRT2 1.4142135623730950488016887242097

typedef struct oracle_grid oracle_grid;
struct oracle_grid {
    luma_grid_desc d;
    int ncell, Q, D;
    const int (*c)[3];
    const double *w;
    const int *opp;
    const int *refl; /* [3][Q] flattened */
    int *typ;
    double *xpos, *ypos, *zpos, *ux_in, *uy_in, *uz_in;
    double *f, *fNew, *feq, *u, *rho, *force_xyz, *force_i, *u_n;
    int t;
    oracle_grid *parent;
    oracle_grid *sub[8];
    int nsub;
    int has_ibm_bodies, has_flexible_bodies;
    void (*ibm_hook)(oracle_grid *, void *); /* IBM pass (set by the IBM oracle) */
    void *ibm_ctx;
    /* BFL body 0 (oracle_bfl_set): per site the marker of its voxel (-1),
     * per marker Q[v + Q*m] and the momentum-exchange force of the step */
    int *bfl_marker;
    double *bfl_q, *bfl_force;
    int bfl_nm;
    /* running means (LUMA_FLAG_TIME_AVERAGES), reference layout */
    double *rho_ta, *ui_ta, *uiuj_ta;
    /* KBC grids: the stabiliser gamma of each site's latest collision
     * (NaN where no collision ran yet); a record for tests, not an input */
    double *kbc_gamma;
};

static char g_err[512];
static void set_err(const char *m) { snprintf(g_err, sizeof g_err, "%s", m); }
const char *oracle_last_error(void) { return g_err; }

static double cs_(void) { return 1.0 / sqrt(3.0); }

/* ---- equilibrium: _LBM_equilibrium_opt, :674-705 ---- */
static double feq_at(const oracle_grid *g, int id, int v) {
    const double cs = cs_();
    const int *c = g->c[v];
    const double *u = g->u + (size_t)id * g->D;
    double A, B;
    if (g->D == 3) {
        A = (c[0] * u[0]) + (c[1] * u[1]) + (c[2] * u[2]);
        B = (SQ(c[0]) - SQ(cs)) * SQ(u[0]) + (SQ(c[1]) - SQ(cs)) * SQ(u[1]) +
            (SQ(c[2]) - SQ(cs)) * SQ(u[2]) + 2 * c[0] * c[1] * u[0] * u[1] +
            2 * c[0] * c[2] * u[0] * u[2] + 2 * c[1] * c[2] * u[1] * u[2];
    } else {
        A = (c[0] * u[0]) + (c[1] * u[1]);
        B = (SQ(c[0]) - SQ(cs)) * SQ(u[0]) + (SQ(c[1]) - SQ(cs)) * SQ(u[1]) +
            2 * c[0] * c[1] * u[0] * u[1];
    }
    return g->rho[id] * g->w[v] * (1.0 + (A / SQ(cs)) + (B / (2.0 * SQ(cs) * SQ(cs))));
}

/* ---- GridUtils::getVelocityRampCoefficient, src/GridUtils.cpp:1808-1816 ---- */
static double ramp_coeff(const oracle_grid *g, double t) {
    if (g->d.velocity_ramp > 0.0 && t <= g->d.velocity_ramp)
        return (1.0 - cos(L_PI * t / g->d.velocity_ramp)) / 2.0;
    return 1.0;
}

/* ---- GridUtils::isWithinDomainWall, src/GridUtils.cpp:1369-1430 ---- */
static int within_domain_wall(const oracle_grid *g, double x, double y, double z, int nvec[3],
                              int *ndir, int *edges) {
    const double *E = g->d.global_edges, *T = g->d.wall_thickness;
    nvec[0] = nvec[1] = nvec[2] = 0;
    *ndir = -1;
    *edges = 0;
    if (x > 0.0 && x < T[0]) { *ndir = 0; nvec[0] = 1; (*edges)++; }
    if (x < E[1] && x > E[1] - T[1]) { *ndir = 0; nvec[0] = -1; (*edges)++; }
    if (y > 0.0 && y < T[2]) { *ndir = 1; nvec[1] = 1; (*edges)++; }
    if (y < E[3] && y > E[3] - T[3]) { *ndir = 1; nvec[1] = -1; (*edges)++; }
    if (g->D == 3) {
        if (z > 0.0 && z < T[4]) { *ndir = 2; nvec[2] = 1; (*edges)++; }
        if (z < E[5] && z > E[5] - T[5]) { *ndir = 2; nvec[2] = -1; (*edges)++; }
    }
    return *edges > 0;
}

/* ---- sub-grid lookup: GridUtils::getSubGrid, src/GridUtils.cpp:1761-1799.
 * The reference tests L0 positions against each region's global edges; the
 * region containing the site is the one whose coarse limits contain it. ---- */
static oracle_grid *sub_grid_at(oracle_grid *g, int i, int j, int k) {
    if (g->d.level > 0) return g->nsub ? g->sub[0] : NULL;
    for (int s = 0; s < g->nsub; ++s) {
        const int *L = g->sub[s]->d.coarse_lims;
        if (i >= L[0] && i <= L[1] && j >= L[2] && j <= L[3] && (g->D == 2 || (k >= L[4] && k <= L[5])))
            return g->sub[s];
    }
    return NULL;
}

static int stream_site(oracle_grid *g, int i, int j, int k, int id, int type, int subcycle);
static void macro_site(oracle_grid *g, int i, int j, int k, int id, int type);

/* ---- _LBM_coalesce_opt, :591-636 (getFineIndices, src/GridUtils.cpp:410-425) ---- */
static int coalesce(oracle_grid *g, int i, int j, int k, int id, int v) {
    oracle_grid *cg = sub_grid_at(g, i, j, k);
    if (!cg) { set_err("coalesce: no sub-grid"); return -1; }
    const int cM = cg->d.M, cK = cg->d.K, Q = g->Q;
    const int ci = 2 * (i - cg->d.coarse_lims[0] + 1) - 2;
    const int cj = 2 * (j - cg->d.coarse_lims[2] + 1) - 2;
    const int ck = g->D == 3 ? 2 * (k - cg->d.coarse_lims[4] + 1) - 2 : 0;
    double s = 0.0;
    for (int ii = 0; ii < 2; ++ii)
        for (int jj = 0; jj < 2; ++jj)
            for (int kk = 0; kk < (g->D == 3 ? 2 : 1); ++kk)
                s += cg->f[v + (ck + kk) * Q + (cj + jj) * Q * cK + (size_t)(ci + ii) * Q * cK * cM];
    s /= (g->D == 3) ? 8.0 : 4.0;
    g->fNew[v + (size_t)id * Q] = s;
    return 0;
}

/* ---- _LBM_explode_opt, :646-663 (getCoarseIndices, src/GridUtils.cpp:440-466) ---- */
static void explode(oracle_grid *g, int id, int v, int sx, int sy, int sz) {
    oracle_grid *p = g->parent;
    if (sx % 2 != 0) sx -= 1;
    if (sy % 2 != 0) sy -= 1;
    if (sz % 2 != 0) sz -= 1;
    const int pi = sx / 2 + g->d.coarse_lims[0];
    const int pj = sy / 2 + g->d.coarse_lims[2];
    const int pk = g->D == 3 ? sz / 2 + g->d.coarse_lims[4] : 0;
    const int Q = g->Q;
    g->fNew[v + (size_t)id * Q] = p->f[v + pk * Q + pj * Q * p->d.K + (size_t)pi * Q * p->d.K * p->d.M];
}

/* ---- _LBM_applySpecReflect_opt, :527-581 ---- */
static int spec_reflect(oracle_grid *g, int i, int j, int k, int id, int v, int *applied) {
    int nv[3], nd, ne;
    const int Q = g->Q;
    const int *c = g->c[v];
    *applied = 0;
    if (!within_domain_wall(g, g->xpos[i], g->ypos[j], g->zpos[k], nv, &nd, &ne)) {
        set_err("Slip wall not located inside a domain wall region");
        return -1;
    }
    int plane = -1;
    if (nv[0] == 1 && c[0] == 1) plane = 0;
    else if (nv[0] == -1 && c[0] == -1) plane = 0;
    else if (nv[1] == 1 && c[1] == 1) plane = 1;
    else if (nv[1] == -1 && c[1] == -1) plane = 1;
    else if (nv[2] == 1 && c[2] == 1) plane = 2;
    else if (nv[2] == -1 && c[2] == -1) plane = 2;
    if (plane >= 0) {
        g->fNew[v + (size_t)id * Q] = g->f[g->refl[plane * Q + v] + (size_t)id * Q];
        *applied = 1;
    }
    return 0;
}

/* ---- GridObj::_LBM_applyBFL_opt, :1010-1113 ----
 * Returns 1 when the link carries the BFL condition (fNew written or, at a
 * grid-edge stencil, left as it was), 0 for the regular stream, -1 on a
 * BFL-labelled site without a marker.  The stencil site of the near-wall
 * branch is built from (i, j, k) itself (:1070-1071), so its interpolation
 * reduces to f_opp(v) at the site. Momentum exchange as
 * ObjectManager::computeLiftDrag(v, id, g, markerID) (src/ObjectManager.cpp:
 * 176-189). */
static int apply_bfl(oracle_grid *g, int id, int sid, int v, int i, int j, int k) {
    const int Q = g->Q, N = g->d.N, M = g->d.M, K = g->d.K;
    double q = -1.0;
    int current = 1, marker = -1;
    if (g->typ[id] == LUMA_SITE_BFL) {
        marker = g->bfl_marker ? g->bfl_marker[id] : -1;
        if (marker < 0) { set_err("BFL site without a BFL marker"); return -1; }
        q = g->bfl_q[g->opp[v] + Q * marker];
    }
    if (q == -1.0) {
        const int ms = g->bfl_marker ? g->bfl_marker[sid] : -1;
        if (ms >= 0) {
            current = 0;
            marker = ms;
            q = g->bfl_q[v + Q * ms];
        }
    }
    if (q == -1.0) return 0;
    const int vo = g->opp[v];
    double *fn = &g->fNew[v + (size_t)id * Q];
    const double fo = g->f[vo + (size_t)id * Q];
    int contributes = 0;
    if (current) {
        const int si = i + g->c[v][0], sj = j + g->c[v][1], sk = k + g->c[v][2];
        if (si >= 0 && si < N && sj >= 0 && sj < M && sk >= 0 && sk < K) {
            const size_t stencil = (size_t)k + (size_t)j * K + (size_t)i * K * M;
            *fn = (1 - 2 * q) * (g->f[vo + stencil * Q] - fo) + fo;
            contributes = 1;
        }
    } else {
        *fn = (1 - 2 * q) * ((g->f[v + (size_t)id * Q] - fo) / (2 - 2 * q)) + fo;
        contributes = 1;
    }
    if (contributes && g->bfl_force) {
        const double s = fo + *fn;
        g->bfl_force[3 * marker + 0] += g->c[vo][0] * s;
        g->bfl_force[3 * marker + 1] += g->c[vo][1] * s;
        g->bfl_force[3 * marker + 2] += g->c[vo][2] * s;
    }
    return 1;
}

/* ---- _LBM_stream_opt, :206-297 ---- */
static int stream_site(oracle_grid *g, int i, int j, int k, int id, int type, int subcycle) {
    const int N = g->d.N, M = g->d.M, K = g->d.K, Q = g->Q;
    for (int v = 0; v < Q; ++v) {
        const int sx = (i - g->c[v][0] + N) % N;
        const int sy = (j - g->c[v][1] + M) % M;
        const int sz = (k - g->c[v][2] + K) % K;
        const int sid = sz + sy * K + sx * K * M;
        const int st = g->typ[sid];
        if (type == LUMA_SITE_BFL || st == LUMA_SITE_BFL) {
            const int r = apply_bfl(g, id, sid, v, i, j, k);
            if (r < 0) return -1;
            if (r) continue;
        }
        if (type == LUMA_SITE_SLIP) {
            int applied;
            if (spec_reflect(g, i, j, k, id, v, &applied)) return -1;
            if (applied) continue;
        }
        if (st == LUMA_SITE_SOLID) {
            g->fNew[v + (size_t)id * Q] = g->f[g->opp[v] + (size_t)id * Q];
        } else if (st == LUMA_SITE_EXTRAPOLATE_RIGHT) {
            g->fNew[v + (size_t)id * Q] = g->f[v + (size_t)(sid - 2 * (K * M)) * Q];
        } else if (st == LUMA_SITE_VELOCITY && !(g->d.flags & LUMA_FLAG_REGULARISED)) {
            if (g->d.velocity_ramp > 0.0) {
                const double rc = ramp_coeff(g, g->t * g->d.dt);
                g->u[0 + (size_t)sid * g->D] = g->ux_in[j] * rc;
                g->u[1 + (size_t)sid * g->D] = g->uy_in[j] * rc;
                if (g->D == 3) g->u[2 + (size_t)sid * g->D] = g->uz_in[j] * rc;
            }
            g->fNew[v + (size_t)id * Q] = feq_at(g, sid, v);
        } else if (g->parent && st == LUMA_SITE_TL_TO_COARSER && subcycle == 0) {
            explode(g, id, v, sx, sy, sz);
        } else if (g->nsub && st == LUMA_SITE_REFINED && type == LUMA_SITE_TL_TO_FINER) {
            if (coalesce(g, i, j, k, id, v)) return -1;
        } else {
            g->fNew[v + (size_t)id * Q] = g->f[v + (size_t)sid * Q];
        }
    }
    return 0;
}

/* ---- _LBM_macro_opt, :800-919 (time averages not restated) ---- */
static void macro_site(oracle_grid *g, int i, int j, int k, int id, int type) {
    const int Q = g->Q, D = g->D;
    const int forcing = (g->d.flags & (LUMA_FLAG_IBM | LUMA_FLAG_GRAVITY)) != 0;
    if (type == LUMA_SITE_FLUID || type == LUMA_SITE_BFL || type == LUMA_SITE_TL_TO_FINER ||
        type == LUMA_SITE_SLIP) {
        double r = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
        const double *fn = g->fNew + (size_t)id * Q;
        for (int v = 0; v < Q; ++v) {
            r += fn[v];
            mx += g->c[v][0] * fn[v];
            my += g->c[v][1] * fn[v];
            if (D == 3) mz += g->c[v][2] * fn[v];
        }
        if (forcing) {
            const double *F = g->force_xyz + (size_t)id * D;
            mx += 0.5 * F[0];
            my += 0.5 * F[1];
            if (D == 3) {
                if (g->d.flags & LUMA_FLAG_FIX_MACRO3D) mz += 0.5 * F[2];
                else mx += 0.5 * F[2];
            }
        }
        g->u[0 + (size_t)id * D] = mx / r;
        g->u[1 + (size_t)id * D] = my / r;
        if (D == 3) g->u[2 + (size_t)id * D] = mz / r;
        g->rho[id] = r;
    }
    if (type == LUMA_SITE_TL_TO_FINER) {
        oracle_grid *cg = sub_grid_at(g, i, j, k);
        if (!cg) goto averages;
        const int cM = cg->d.M, cK = cg->d.K;
        const int ci = 2 * (i - cg->d.coarse_lims[0] + 1) - 2;
        const int cj = 2 * (j - cg->d.coarse_lims[2] + 1) - 2;
        const int ck = D == 3 ? 2 * (k - cg->d.coarse_lims[4] + 1) - 2 : 0;
        for (int ii = 0; ii < 2; ++ii)
            for (int jj = 0; jj < 2; ++jj)
                for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk) {
                    const size_t cid = (size_t)(ck + kk) + (size_t)(cj + jj) * cK + (size_t)(ci + ii) * cK * cM;
                    for (int dd = 0; dd < D; ++dd) cg->u[dd + cid * D] = g->u[dd + (size_t)id * D];
                    cg->rho[cid] = g->rho[id];
                }
    }
averages:
    /* time-averaged quantities, :895-917: the mean over t completed steps
     * becomes the mean over t + 1 with the current value */
    if (g->rho_ta) {
        const double t = (double)g->t, t1 = (double)(g->t + 1);
        const double *u = g->u + (size_t)id * D;
        double ta = g->rho_ta[id] * t;
        ta += g->rho[id];
        g->rho_ta[id] = ta / t1;
        const int npq = 3 * D - 3;
        int pq = 0;
        for (int p = 0; p < D; ++p) {
            ta = g->ui_ta[p + (size_t)id * D] * t;
            ta += u[p];
            g->ui_ta[p + (size_t)id * D] = ta / t1;
            for (int q = p; q < D; ++q) {
                ta = g->uiuj_ta[pq + (size_t)id * npq] * t;
                ta += (u[p] * u[q]);
                g->uiuj_ta[pq + (size_t)id * npq] = ta / t1;
                pq++;
            }
        }
    }
}

/* ---- _LBM_updateAndExtrapolate (order 1), :1353-1412, and
 *      GridUtils::extrapolate, inc/GridUtils.h:232-281 ---- */
static int update_and_extrapolate(oracle_grid *g, int subcycle, const double *q, const int dir[3],
                                  int i, int j, int k, int p, int max, double *out) {
    const int N = g->d.N, M = g->d.M, K = g->d.K;
    const int id = k + j * K + i * K * M;
    const int i1 = i + dir[0], i2 = i1 + dir[0];
    const int j1 = j + dir[1], j2 = j1 + dir[1];
    const int k1 = k + dir[2], k2 = k1 + dir[2];
    if (i1 < 0 || i1 >= N || j1 < 0 || j1 >= M || k1 < 0 || k1 >= K || i2 < 0 || i2 >= N ||
        j2 < 0 || j2 >= M || k2 < 0 || k2 >= K) {
        set_err("Extrapolation does not have enough available cells.");
        return -1;
    }
    const int id1 = k1 + j1 * K + i1 * K * M;
    const int id2 = k2 + j2 * K + i2 * K * M;
    if (id1 > id) {
        if (stream_site(g, i1, j1, k1, id1, g->typ[id1], subcycle)) return -1;
        macro_site(g, i1, j1, k1, id1, g->typ[id1]);
    }
    if (id2 > id) {
        if (stream_site(g, i2, j2, k2, id2, g->typ[id2], subcycle)) return -1;
        macro_site(g, i2, j2, k2, id2, g->typ[id2]);
    }
    *out = 2.0 * q[p + (size_t)id1 * max] - q[p + (size_t)id2 * max];
    return 0;
}

/* ---- _LBM_regularised_opt, :313-510 ---- */
static int regularised(oracle_grid *g, int i, int j, int k, int id, int type, int subcycle) {
    const int Q = g->Q, D = g->D;
    const double cs = cs_();
    double vel[3];
    double dens = g->d.rho_in;
    int nv[3], nd, ne;
    double f_plus = 0.0, f_zero = 0.0;
    double Sxx = 0, Syy = 0, Sxy = 0, Szz = 0, Sxz = 0, Syz = 0;
    const double rc = ramp_coeff(g, (g->t + 1) * g->d.dt);
    if (!within_domain_wall(g, g->xpos[i], g->ypos[j], g->zpos[k], nv, &nd, &ne)) {
        set_err("Velocity site not outside domain walls is currently not supported.");
        return -1;
    }
    vel[0] = g->ux_in[j] * rc;
    vel[1] = g->uy_in[j] * rc;
    vel[2] = g->uz_in[j] * rc;
    dens += g->d.pressure_delta;
    if (ne > 1) {
        if (type == LUMA_SITE_PRESSURE) {
            set_err("Pressure BC not supported at corner/edge site.");
            return -1;
        }
        if (update_and_extrapolate(g, subcycle, g->rho, nv, i, j, k, 0, 1, &dens)) return -1;
    } else {
        for (int v = 0; v < Q; ++v) {
            if (g->c[v][nd] == -nv[nd]) f_plus += g->fNew[v + (size_t)id * Q];
            else if (g->c[v][nd] == 0) f_zero += g->fNew[v + (size_t)id * Q];
        }
        if (type == LUMA_SITE_PRESSURE) {
            for (int dd = 0; dd < D; dd++)
                if (dd != nd)
                    if (update_and_extrapolate(g, subcycle, g->u, nv, i, j, k, dd, D, &vel[dd])) return -1;
            vel[nd] = 1.0 - ((1.0 / dens) * (2.0 * f_plus + f_zero));
            if (nv[nd] == -1) vel[nd] *= -1.0;
        } else {
            double nvel = vel[nd];
            if (nv[nd] == -1) nvel *= -1.0;
            dens = (1.0 / (1.0 - nvel)) * (2.0 * f_plus + f_zero);
        }
    }
    g->rho[id] = dens;
    g->u[0 + (size_t)id * D] = vel[0];
    g->u[1 + (size_t)id * D] = vel[1];
    if (D == 3) g->u[2 + (size_t)id * D] = vel[2];

    double *fn = g->fNew + (size_t)id * Q;
    for (int v = 0; v < Q; ++v) {
        const int *c = g->c[v];
        if (ne == 1 && c[nd] == nv[nd]) {
            fn[v] = feq_at(g, id, v) + (fn[g->opp[v]] - feq_at(g, id, g->opp[v]));
        } else if (ne > 1 && (c[0] == nv[0] || c[1] == nv[1] || (D == 3 && c[2] == nv[2]))) {
            int dp = 0;
            double mag = 0.0;
            for (int dd = 0; dd < D; dd++) {
                dp += c[dd] * nv[dd];
                mag += ((double)c[dd] * (double)c[dd]);
            }
            mag = sqrt(mag);
            if (dp == 0 && mag > 1.0) fn[v] = feq_at(g, id, v);
            else fn[v] = feq_at(g, id, v) + (fn[g->opp[v]] - feq_at(g, id, g->opp[v]));
        }
        const double fneq = fn[v] - feq_at(g, id, v);
        Sxx += c[0] * c[0] * fneq;
        Syy += c[1] * c[1] * fneq;
        Sxy += c[0] * c[1] * fneq;
        if (D == 3) {
            Szz += c[2] * c[2] * fneq;
            Sxz += c[0] * c[2] * fneq;
            Syz += c[1] * c[2] * fneq;
        }
    }
    for (int v = 0; v < Q; v++) {
        const int *c = g->c[v];
        fn[v] = feq_at(g, id, v) +
                (g->w[v] / (2.0 * SQ(cs) * SQ(cs))) *
                    (((c[0] * c[0] - SQ(cs)) * Sxx) + ((c[1] * c[1] - SQ(cs)) * Syy) +
                     ((c[2] * c[2] - SQ(cs)) * Szz) + (2.0 * c[0] * c[1] * Sxy) +
                     (2.0 * c[0] * c[2] * Sxz) + (2.0 * c[1] * c[2] * Syz));
    }
    return 0;
}

/* ---- _LBM_forceGrid_opt, :928-990 ---- */
static void force_grid(oracle_grid *g, int id) {
    const int Q = g->Q, D = g->D;
    const double cs = cs_();
    double *fi = g->force_i + (size_t)id * Q;
    const double *u = g->u + (size_t)id * D;
    const double *F = g->force_xyz + (size_t)id * D;
    memset(fi, 0, sizeof(double) * Q);
    for (int v = 0; v < Q; v++) {
        double beta = 0.0;
        const double lambda = (1 - 0.5 * g->d.omega) * (g->w[v] / (cs * cs));
        for (int dd = 0; dd < D; dd++) beta += (g->c[v][dd] * u[dd]);
        beta = beta * (1 / (cs * cs));
        for (int dd = 0; dd < D; dd++) fi[v] += F[dd] * (g->c[v][dd] * (1 + beta) - u[dd]);
        fi[v] *= lambda;
    }
}

/* ---- _LBM_smag, :717-756 ---- */
static double smag(oracle_grid *g, int id, double omega) {
    const int Q = g->Q, D = g->D;
    const double cs = cs_();
    double fneq[27], S[3][3];
    for (int v = 0; v < Q; ++v) fneq[v] = g->fNew[v + (size_t)id * Q] - feq_at(g, id, v);
    memset(S, 0, sizeof S);
    for (int a = 0; a < D; ++a)
        for (int b = a; b < D; ++b) {
            S[a][b] = 0.0;
            for (int v = 0; v < Q; ++v) S[a][b] += g->c[v][a] * g->c[v][b] * fneq[v];
        }
    for (int a = 1; a < D; ++a)
        for (int b = 0; b < a; ++b) S[a][b] = S[b][a];
    /* Matrix2D % (inc/Matrix.h:65-75): per-row sums of element-wise
     * products over the 3x3 store, then the sum of the row sums. */
    double ip = 0.0;
    for (int a = 0; a < 3; ++a) {
        double row = 0.0;
        for (int b = 0; b < 3; ++b) row += S[a][b] * S[a][b];
        ip += row;
    }
    const double Qs = sqrt(2.0 * ip);
    const double tau = 1.0 / omega;
    const double tau_t =
        0.5 * (sqrt(SQ(tau) + 2.0 * L_SQRT2 * SQ(g->d.csmag) * g->d.rho_in * SQ(cs) * SQ(cs) * Qs) - tau);
    return (1.0 / (tau + tau_t));
}

/* ---- _LBM_collide_opt, :765-790 ---- */
static void collide_bgk(oracle_grid *g, int id) {
    const int Q = g->Q;
    const int forcing = (g->d.flags & (LUMA_FLAG_IBM | LUMA_FLAG_GRAVITY)) != 0;
    const double om = g->d.collision == LUMA_COLL_BGK_SMAG ? smag(g, id, g->d.omega) : g->d.omega;
    double *fn = g->fNew + (size_t)id * Q;
    for (int v = 0; v < Q; ++v) {
        if (forcing) fn[v] += om * (feq_at(g, id, v) - fn[v]) + g->force_i[v + (size_t)id * Q];
        else fn[v] += om * (feq_at(g, id, v) - fn[v]);
    }
}

/* ---- _LBM_kbcCollide_opt, :1122-1305 ---- */
static void collide_kbc(oracle_grid *g, int id) {
    const int Q = g->Q, D = g->D;
    const int forcing = (g->d.flags & (LUMA_FLAG_IBM | LUMA_FLAG_GRAVITY)) != 0;
    const double *src = (g->d.flags & LUMA_FLAG_FIX_KBC) ? g->fNew : g->f;
    double ds[27], dh[27], fneq[27], Mneq[13];
    int C[13 * 27];
    const int nm = D == 3 ? 13 : 3;
    for (int m = 0; m < nm; ++m) Mneq[m] = 0.0;
    for (int m = 0; m < nm * Q; ++m) C[m] = 1;
    double *fe = g->feq + (size_t)id * Q;
    for (int v = 0; v < Q; v++) {
        fe[v] = feq_at(g, id, v);
        fneq[v] = src[v + (size_t)id * Q] - fe[v];
        int idx = 0;
        for (int s = 0; s < D; ++s)
            for (int a = s; a < D; ++a) {
                C[idx + v * nm] = g->c[v][s] * g->c[v][a];
                Mneq[idx] += fneq[v] * C[idx + v * nm];
                idx++;
                if (D == 3)
                    for (int b = a; b < D; ++b)
                        if (s != a || a != b || s != b) {
                            C[idx + v * nm] = g->c[v][s] * g->c[v][a] * g->c[v][b];
                            Mneq[idx] += fneq[v] * C[idx + v * nm];
                            idx++;
                        }
            }
    }
    for (int v = 0; v < Q; v++) {
        const int *c = g->c[v];
        if (D == 3) {
            if (c[0] == 0) {
                if (c[1] == 0) {
                    if (c[2] == 0) ds[v] = (-(Mneq[0] + Mneq[8] + Mneq[12]));
                    else
                        ds[v] = ((-(Mneq[0] - Mneq[12]) - (Mneq[8] - Mneq[12])) / 6.0 +
                                 (Mneq[0] + Mneq[8] + Mneq[12]) / 6.0 - c[2] * 0.5 * (Mneq[2] + Mneq[9]));
                } else {
                    if (c[2] == 0)
                        ds[v] = ((-(Mneq[0] - Mneq[12]) + 2.0 * (Mneq[8] - Mneq[12])) / 6.0 +
                                 (Mneq[0] + Mneq[8] + Mneq[12]) / 6.0 - c[1] * 0.5 * (Mneq[1] + Mneq[11]));
                    else
                        ds[v] = (C[10 + v * nm] * 0.25 * Mneq[10] +
                                 (c[2] * 0.25 * Mneq[9] + c[1] * 0.25 * Mneq[11]));
                }
            } else {
                if (c[1] == 0) {
                    if (c[2] == 0)
                        ds[v] = ((2.0 * (Mneq[0] - Mneq[12]) - (Mneq[8] - Mneq[12])) / 6.0 +
                                 (Mneq[0] + Mneq[8] + Mneq[12]) / 6.0 - c[0] * 0.5 * (Mneq[4] + Mneq[7]));
                    else
                        ds[v] = (C[6 + v * nm] * 0.25 * Mneq[6] + (c[2] * 0.25 * Mneq[2] + c[0] * 0.25 * Mneq[7]));
                } else {
                    if (c[2] == 0)
                        ds[v] = (C[3 + v * nm] * 0.25 * Mneq[3] + (c[1] * 0.25 * Mneq[1] + c[0] * 0.25 * Mneq[4]));
                    else
                        ds[v] = (C[5 + v * nm] * Mneq[5] / 8.0);
                }
            }
        } else {
            if (c[0] == 0) {
                if (c[1] == 0) ds[v] = 0.0;
                else ds[v] = -0.25 * (Mneq[0] - Mneq[2]);
            } else {
                if (c[1] == 0) ds[v] = 0.25 * (Mneq[0] - Mneq[2]);
                else ds[v] = 0.25 * C[1 + v * nm] * Mneq[1];
            }
        }
        dh[v] = fneq[v] - ds[v];
    }
    double top = 0.0, bot = 0.0;
    for (int v = 0; v < Q; v++) {
        top += ds[v] * dh[v] / fe[v];
        bot += dh[v] * dh[v] / fe[v];
    }
    const double beta_m1 = 2.0 / g->d.omega;
    double gamma;
    if (bot == 0.0) gamma = 2.0;
    else gamma = beta_m1 - (2.0 - beta_m1) * (top / bot);
    if (g->kbc_gamma) g->kbc_gamma[id] = gamma;
    double *fn = g->fNew + (size_t)id * Q;
    for (int v = 0; v < Q; v++) {
        const double base = src[v + (size_t)id * Q] - (1.0 / beta_m1) * (2.0 * ds[v] + gamma * dh[v]);
        fn[v] = forcing ? base + g->force_i[v + (size_t)id * Q] : base;
    }
}

static void collide_site(oracle_grid *g, int id) {
    if (g->d.collision == LUMA_COLL_KBC) collide_kbc(g, id);
    else collide_bgk(g, id);
}

/* ---- _LBM_resetForces, :1327-1337 ---- */
static void reset_forces(oracle_grid *g) {
    if (g->d.flags & LUMA_FLAG_GRAVITY) {
        for (int id = 0; id < g->ncell; ++id)
            g->force_xyz[g->d.gravity_dir + (size_t)id * g->D] = g->rho[id] * g->d.gravity * g->d.refinement_ratio;
    } else {
        memset(g->force_xyz, 0, sizeof(double) * (size_t)g->ncell * g->D);
    }
}

/* Sites whose update touches only their own fNew/u/rho and read f: the
 * loop can run in parallel (as the reference's optional OpenMP loop does,
 * :69-71) when no site has a non-local side effect. */
static int loop_is_local(const oracle_grid *g) {
    if (g->d.velocity_ramp > 0.0 && !(g->d.flags & LUMA_FLAG_REGULARISED)) return 0;
    if (g->d.flags & LUMA_FLAG_REGULARISED) return 0;
    if (g->nsub) return 0;
    if (g->bfl_marker) return 0;  /* marker forces accumulate in site order */
    return 1;
}

/* ---- GridObj::_LBM_updateReynolds, :1313-1321, with
 * GridUtils::getReynoldsRampCoefficient (src/GridUtils.cpp:1825-1833), as
 * LBM_multi_opt calls it first (:39-42) ---- */
static void update_reynolds(oracle_grid *g) {
    const double t = (g->t + 1) * g->d.dt;
    const double coeff = t <= g->d.reynolds_ramp ? 1.0 - cos(L_PI * t / g->d.reynolds_ramp) : 1.0;
    const double nu = ((1.0 / (g->d.re * coeff)) * g->d.dt) / (g->d.dh * g->d.dh);
    const double cs = cs_();
    g->d.omega = 1.0 / ((nu / (cs * cs)) + 0.5);
}

/* ---- GridObj::LBM_multi_opt, :36-193 ---- */
static int multi_opt(oracle_grid *g, int subcycle) {
    if (g->d.reynolds_ramp > 0.0) update_reynolds(g);
    for (int s = 0; s < g->nsub; ++s)
        for (int it = 0; it < 2; ++it)
            if (multi_opt(g->sub[s], it)) return -1;
    const int ibm = (g->d.flags & LUMA_FLAG_IBM) != 0;
    const int gravity = (g->d.flags & LUMA_FLAG_GRAVITY) != 0;
    const int N = g->d.N, M = g->d.M, K = g->d.K;
    const int reg = (g->d.flags & LUMA_FLAG_REGULARISED) != 0;
    if (ibm && g->has_ibm_bodies) reset_forces(g);
    if (g->bfl_force) memset(g->bfl_force, 0, sizeof(double) * 3 * (size_t)g->bfl_nm);
    int err = 0;
    const int par = loop_is_local(g);
#pragma omp parallel for schedule(static) if (par) reduction(| : err)
    for (int i = 0; i < N; ++i) {
        for (int j = 0; j < M; ++j) {
            for (int k = 0; k < K; ++k) {
                const int id = k + j * K + i * K * M;
                const int type = g->typ[id];
                if (type == LUMA_SITE_REFINED || type == LUMA_SITE_SOLID || (!reg && type == LUMA_SITE_VELOCITY))
                    continue;
                if (stream_site(g, i, j, k, id, type, subcycle)) { err |= 1; continue; }
                if (reg && (type == LUMA_SITE_VELOCITY || type == LUMA_SITE_PRESSURE))
                    if (regularised(g, i, j, k, id, type, subcycle)) { err |= 1; continue; }
                macro_site(g, i, j, k, id, type);
                if (!ibm) {
                    if (gravity && type != LUMA_SITE_SOLID) force_grid(g, id);
                    if (type != LUMA_SITE_TL_TO_COARSER) collide_site(g, id);
                }
            }
        }
    }
    if (err) return -1;
    if (ibm) {
        if (g->has_flexible_bodies) memcpy(g->u_n, g->u, sizeof(double) * (size_t)g->ncell * g->D);
        if (g->has_ibm_bodies && g->ibm_hook) g->ibm_hook(g, g->ibm_ctx);
#pragma omp parallel for schedule(static)
        for (int id = 0; id < g->ncell; ++id) {
            const int type = g->typ[id];
            if (type != LUMA_SITE_SOLID) force_grid(g, id);
            if (type != LUMA_SITE_TL_TO_COARSER) collide_site(g, id);
        }
    }
    double *tmp = g->f;
    g->f = g->fNew;
    g->fNew = tmp;
    ++g->t;
    return 0;
}

/* ------------------------------ public API ------------------------------ */

static double *dup_d(const double *p, size_t n) {
    double *q = (double *)malloc(sizeof(double) * (n ? n : 1));
    if (p) memcpy(q, p, sizeof(double) * n);
    else memset(q, 0, sizeof(double) * (n ? n : 1));
    return q;
}

oracle_grid *oracle_grid_create(const luma_grid_desc *d, oracle_grid *parent) {
    if (!d || d->abi_version != LUMA_GPU_ABI_VERSION) { set_err("bad descriptor"); return NULL; }
    oracle_grid *g = (oracle_grid *)calloc(1, sizeof(oracle_grid));
    g->d = *d;
    g->Q = d->Q;
    g->D = d->dims;
    if (d->Q == 9 && d->dims == 2) { g->c = C9; g->w = W9; g->opp = OPP9; g->refl = &REF9[0][0]; }
    else if (d->Q == 19 && d->dims == 3) { g->c = C19; g->w = W19; g->opp = OPP19; g->refl = &REF19[0][0]; }
    else if (d->Q == 27 && d->dims == 3) { g->c = C27; g->w = W27; g->opp = OPP27; g->refl = &REF27[0][0]; }
    else { set_err("unsupported lattice"); free(g); return NULL; }
    g->ncell = d->N * d->M * d->K;
    const size_t n = (size_t)g->ncell;
    g->typ = (int *)malloc(sizeof(int) * n);
    for (size_t i = 0; i < n; ++i) g->typ[i] = d->lattyp ? d->lattyp[i] : LUMA_SITE_FLUID;
    g->xpos = dup_d(d->xpos, d->N);
    g->ypos = dup_d(d->ypos, d->M);
    g->zpos = dup_d(d->zpos, d->K);
    g->ux_in = dup_d(d->ux_in, d->M);
    g->uy_in = dup_d(d->uy_in, d->M);
    g->uz_in = dup_d(d->uz_in, d->M);
    g->f = dup_d(NULL, n * g->Q);
    g->fNew = dup_d(NULL, n * g->Q);
    g->feq = dup_d(NULL, n * g->Q);
    g->force_i = dup_d(NULL, n * g->Q);
    g->u = dup_d(NULL, n * g->D);
    g->u_n = dup_d(NULL, n * g->D);
    g->force_xyz = dup_d(NULL, n * g->D);
    g->rho = dup_d(NULL, n);
    if (d->flags & LUMA_FLAG_TIME_AVERAGES) {
        g->rho_ta = dup_d(NULL, n);
        g->ui_ta = dup_d(NULL, n * g->D);
        g->uiuj_ta = dup_d(NULL, n * (3 * g->D - 3));
    }
    if (d->collision == LUMA_COLL_KBC) {
        g->kbc_gamma = dup_d(NULL, n);
        for (size_t i = 0; i < n; ++i) g->kbc_gamma[i] = NAN;
    }
    g->d.lattyp = NULL;
    g->d.xpos = g->d.ypos = g->d.zpos = NULL;
    g->d.ux_in = g->d.uy_in = g->d.uz_in = NULL;
    g->parent = parent;
    if (parent) {
        if (parent->nsub >= 8) { set_err("too many sub-grids"); return NULL; }
        parent->sub[parent->nsub++] = g;
    }
    return g;
}

void oracle_grid_destroy(oracle_grid *g) {
    if (!g) return;
    for (int s = 0; s < g->nsub; ++s) oracle_grid_destroy(g->sub[s]);
    free(g->typ); free(g->xpos); free(g->ypos); free(g->zpos);
    free(g->ux_in); free(g->uy_in); free(g->uz_in);
    free(g->f); free(g->fNew); free(g->feq); free(g->force_i);
    free(g->u); free(g->u_n); free(g->force_xyz); free(g->rho);
    free(g->bfl_marker); free(g->bfl_q); free(g->bfl_force);
    free(g->rho_ta); free(g->ui_ta); free(g->uiuj_ta);
    free(g->kbc_gamma);
    free(g);
}

/* Running means of rho, u_p and u_p u_q (p <= q), reference layout. */
int oracle_download_time_averages(const oracle_grid *g, double *rho_ta, double *ui_ta, double *uiuj_ta) {
    if (!g->rho_ta) { set_err("grid keeps no time averages"); return -1; }
    const size_t n = (size_t)g->ncell;
    memcpy(rho_ta, g->rho_ta, sizeof(double) * n);
    memcpy(ui_ta, g->ui_ta, sizeof(double) * n * g->D);
    memcpy(uiuj_ta, g->uiuj_ta, sizeof(double) * n * (3 * g->D - 3));
    return 0;
}

/* KBC grids: the stabiliser gamma = 2/omega - (2 - 2/omega) <ds|dh>/<dh|dh>
 * (2 where <dh|dh> = 0) of each site's latest collision, NaN where none ran
 * (_LBM_kbcCollide_opt, src/GridObj_ops_lbm_optimised.cpp:1287-1289). */
int oracle_kbc_gamma(const oracle_grid *g, double *out) {
    if (!g->kbc_gamma) { set_err("not a KBC grid"); return -1; }
    memcpy(out, g->kbc_gamma, sizeof(double) * (size_t)g->ncell);
    return 0;
}

/* GridObj::fNew between steps (after the swap: the state before the latest
 * step), reference layout. */
int oracle_download_fnew(const oracle_grid *g, double *out) {
    memcpy(out, g->fNew, sizeof(double) * (size_t)g->ncell * g->Q);
    return 0;
}

/* BFL body 0 of the grid: site_marker[ncell] (Body::getMarkerData of each
 * site's position, -1 for none) and q[Q * nm] (BFLBody::Q). */
int oracle_bfl_set(oracle_grid *g, const int *site_marker, int nm, const double *q) {
    const size_t n = (size_t)g->ncell;
    for (size_t i = 0; i < n; ++i)
        if (site_marker[i] < -1 || site_marker[i] >= nm) { set_err("BFL site marker out of range"); return -1; }
    free(g->bfl_marker); free(g->bfl_q); free(g->bfl_force);
    g->bfl_marker = (int *)malloc(sizeof(int) * n);
    memcpy(g->bfl_marker, site_marker, sizeof(int) * n);
    g->bfl_q = dup_d(q, (size_t)g->Q * nm);
    g->bfl_force = dup_d(NULL, 3 * (size_t)nm);
    g->bfl_nm = nm;
    return 0;
}

/* Per-marker momentum-exchange force of the latest step (3 per marker). */
int oracle_bfl_forces(const oracle_grid *g, double *out) {
    if (!g->bfl_force) { set_err("no BFL body"); return -1; }
    memcpy(out, g->bfl_force, sizeof(double) * 3 * (size_t)g->bfl_nm);
    return 0;
}

/* Upload sets f, fNew and feq to the given populations, as LBM_initGrid
 * does (src/GridObj_init_grids.cpp:331-332). */
int oracle_upload_state(oracle_grid *g, const double *f, const double *u, const double *rho,
                        const double *force_xyz, int t) {
    const size_t n = (size_t)g->ncell;
    if (f) {
        memcpy(g->f, f, sizeof(double) * n * g->Q);
        memcpy(g->fNew, f, sizeof(double) * n * g->Q);
        memcpy(g->feq, f, sizeof(double) * n * g->Q);
    }
    if (u) { memcpy(g->u, u, sizeof(double) * n * g->D); memcpy(g->u_n, u, sizeof(double) * n * g->D); }
    if (rho) memcpy(g->rho, rho, sizeof(double) * n);
    if (force_xyz) memcpy(g->force_xyz, force_xyz, sizeof(double) * n * g->D);
    g->t = t;
    return 0;
}

int oracle_download_state(const oracle_grid *g, double *f, double *u, double *rho, double *force_xyz) {
    const size_t n = (size_t)g->ncell;
    if (f) memcpy(f, g->f, sizeof(double) * n * g->Q);
    if (u) memcpy(u, g->u, sizeof(double) * n * g->D);
    if (rho) memcpy(rho, g->rho, sizeof(double) * n);
    if (force_xyz) memcpy(force_xyz, g->force_xyz, sizeof(double) * n * g->D);
    return 0;
}

/* Equilibrium populations for the given rho/u fields (reference layout),
 * exactly as LBM_initGrid computes f (src/GridObj_init_grids.cpp:316-333). */
int oracle_equilibrium(oracle_grid *g, const double *u, const double *rho, double *f_out) {
    const size_t n = (size_t)g->ncell;
    memcpy(g->u, u, sizeof(double) * n * g->D);
    memcpy(g->rho, rho, sizeof(double) * n);
    for (size_t id = 0; id < n; ++id)
        for (int v = 0; v < g->Q; ++v) f_out[v + id * g->Q] = feq_at(g, (int)id, v);
    return 0;
}

int oracle_step(oracle_grid *root, int nsteps) {
    for (int s = 0; s < nsteps; ++s)
        if (multi_opt(root, 0)) return -1;
    return 0;
}

int oracle_get_time(const oracle_grid *g) { return g->t; }

/* ObjectManager::computeLiftDrag for bounce-back bodies
 * (src/ObjectManager.cpp:93-165): over every solid site in (i, j, k) order
 * and every direction n, the fluid neighbour x_dest = x - c_opp(n) (no
 * periodic wrap) adds 2 c_opp(n) f_opp(n)(x_dest), from the populations the
 * next step streams (GridObj::f between steps). */
void oracle_momex_force(const oracle_grid *g, double out[3]) {
    const int N = g->d.N, M = g->d.M, K = g->d.K, Q = g->Q;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < M; ++j)
            for (int k = 0; k < K; ++k) {
                const int id = k + j * K + i * K * M;
                if (g->typ[id] != LUMA_SITE_SOLID) continue;
                for (int n = 0; n < Q; ++n) {
                    const int no = g->opp[n];
                    double cx = 0.0, cy = 0.0, cz = 0.0;
                    const int xd = i - g->c[no][0], yd = j - g->c[no][1], zd = k - g->c[no][2];
                    if (xd >= 0 && xd < N && yd >= 0 && yd < M && zd >= 0 && zd < K) {
                        const int did = zd + yd * K + xd * K * M;
                        if (g->typ[did] == LUMA_SITE_FLUID) {
                            const double fv = g->f[no + (size_t)did * Q];
                            cx = 2.0 * g->c[no][0] * fv;
                            cy = 2.0 * g->c[no][1] * fv;
                            cz = 2.0 * g->c[no][2] * fv;
                        }
                    }
                    fx += cx;
                    fy += cy;
                    fz += cz;
                }
            }
    out[0] = fx;
    out[1] = fy;
    out[2] = fz;
}

int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* Hooks for the IBM oracle (ibm_oracle.c). */
void oracle_set_ibm(oracle_grid *g, int has_ibm, int has_flexible, void (*hook)(oracle_grid *, void *), void *ctx) {
    g->has_ibm_bodies = has_ibm;
    g->has_flexible_bodies = has_flexible;
    g->ibm_hook = hook;
    g->ibm_ctx = ctx;
}

/* =========================== immersed boundary ===========================
 * Restatement of ObjectManager's IBM operator for rigid bodies
 * (src/ObjectManager_ops_ibm.cpp): Roma delta kernel (:255-272), support
 * search (:279-453) with delta values (:462-491), marker spacing ds
 * (:927-981), epsilon from the dense support-overlap system (:773-920) solved
 * with the partial-pivot LU the oracle build links in place of LAPACK, then
 * per step interpolate (:498-591), force (:598-614), spread (:621-689) and
 * macroscopic update at the supports (:696-766). */

typedef struct ibm_body {
    oracle_grid *owner;
    int nm;
    double *pos, *vel, *eps, *ds, *dil, *area, *F, *irho, *imom;
    int *off;        /* CSR offsets into the support arrays, nm + 1 */
    int *si, *sj, *sk;
    double *sx, *sy, *sz, *delta;
} ibm_body;

typedef struct ibm_ctx {
    int nb;
    ibm_body *b;
    double global_edges[6];
} ibm_ctx;

static double delta_kernel(double radius, double dilation) {
    const double mag_r = fabs(radius) / dilation;
    if (mag_r > 1.5) return 0.0;
    if (mag_r > 0.5) return (5.0 - (3.0 * mag_r) - sqrt(-3.0 * pow(1.0 - mag_r, 2) + 1.0)) / 6.0;
    return (1.0 + sqrt(1.0 - 3.0 * pow(mag_r, 2))) / 3.0;
}

/* Enclosing voxel of a position on a grid (GridUtils::getEnclosingVoxel,
 * serial form): floor((x - grid start) / dh). */
static int enclosing(double x, double start, double dh) { return (int)floor((x - start) / dh); }

static double grid_start(const oracle_grid *g, int axis) {
    /* Level 0 starts at 0; a sub-grid starts half a fine cell before its first site. */
    const double *p = axis == 0 ? g->xpos : (axis == 1 ? g->ypos : g->zpos);
    return g->d.level == 0 ? 0.0 : p[0] - g->d.dh / 2.0;
}

static int within_domain(const ibm_ctx *c, const double p[3], int D) {
    const double *E = c->global_edges;
    if (p[0] < E[0] || p[0] > E[1] || p[1] < E[2] || p[1] > E[3]) return 0;
    if (D == 3 && (p[2] < E[4] || p[2] > E[5])) return 0;
    return 1;
}

static void support_delta(const ibm_body *b, int m, const double est[3], int D, double *out) {
    const double dh = b->owner->d.dh;
    const double *x = b->pos + 3 * m;
    const double dx = (est[0] - x[0]) / dh, dy = (est[1] - x[1]) / dh;
    double v = delta_kernel(dx, b->dil[m]) * delta_kernel(dy, b->dil[m]);
    if (D == 3) v = v * delta_kernel((est[2] - x[2]) / dh, b->dil[m]);
    *out = v;
}

/* ibm_findSupport (:279-453) for one body; two passes (count, fill). */
static int find_support(ibm_ctx *c, ibm_body *b) {
    oracle_grid *g = b->owner;
    const int D = g->D;
    const double dh = g->d.dh;
    int total = 0;
    for (int pass = 0; pass < 2; ++pass) {
        int n = 0;
        for (int m = 0; m < b->nm; ++m) {
            if (pass == 1) b->off[m] = n;
            const double *x = b->pos + 3 * m;
            const int in = enclosing(x[0], grid_start(g, 0), dh);
            const int jn = enclosing(x[1], grid_start(g, 1), dh);
            const int kn = D == 3 ? enclosing(x[2], grid_start(g, 2), dh) : 0;
            if (in < 0 || jn < 0 || kn < 0 || in >= g->d.N || jn >= g->d.M || kn >= g->d.K) {
                set_err("Body is no-longer inside the domain! Simulation has likely crashed.");
                return -1;
            }
            double nearpos[3] = {g->xpos[in], g->ypos[jn], D == 3 ? g->zpos[kn] : 0.0};
            if (pass == 1) {
                b->si[n] = in; b->sj[n] = jn; b->sk[n] = kn;
                b->sx[n] = nearpos[0]; b->sy[n] = nearpos[1]; b->sz[n] = nearpos[2];
                support_delta(b, m, nearpos, D, &b->delta[n]);
            }
            ++n;
            for (int i = in - 5; i <= in + 5; i++)
                for (int j = jn - 5; j <= jn + 5; j++)
                    for (int k = (D == 3 ? kn - 5 : 0); k <= (D == 3 ? kn + 5 : 0); k++) {
                        double est[3] = {nearpos[0] + (i - in) * dh, nearpos[1] + (j - jn) * dh, nearpos[2]};
                        if (D == 3) est[2] = nearpos[2] + (k - kn) * dh;
                        if ((fabs(x[0] - est[0]) / dh < 1.5 * b->dil[m]) && (fabs(x[1] - est[1]) / dh < 1.5 * b->dil[m]) &&
                            (D == 2 || fabs(x[2] - est[2]) / dh < 1.5 * b->dil[m]) && within_domain(c, est, D)) {
                            if (i != in || j != jn || (D == 3 && k != kn)) {
                                if (pass == 1) {
                                    b->si[n] = i; b->sj[n] = j; b->sk[n] = k;
                                    b->sx[n] = est[0]; b->sy[n] = est[1]; b->sz[n] = est[2];
                                    support_delta(b, m, est, D, &b->delta[n]);
                                }
                                ++n;
                            }
                        }
                    }
        }
        if (pass == 0) {
            total = n;
            free(b->si); free(b->sj); free(b->sk); free(b->sx); free(b->sy); free(b->sz); free(b->delta);
            b->si = (int *)malloc(sizeof(int) * (total + 1));
            b->sj = (int *)malloc(sizeof(int) * (total + 1));
            b->sk = (int *)malloc(sizeof(int) * (total + 1));
            b->sx = (double *)malloc(sizeof(double) * (total + 1));
            b->sy = (double *)malloc(sizeof(double) * (total + 1));
            b->sz = (double *)malloc(sizeof(double) * (total + 1));
            b->delta = (double *)malloc(sizeof(double) * (total + 1));
        } else {
            b->off[b->nm] = n;
        }
    }
    return 0;
}

/* ibm_computeDs (:927-981). */
static void compute_ds(ibm_body *b) {
    const double dh = b->owner->d.dh;
    for (int m = 0; m < b->nm; ++m) {
        double ds = 10.0;
        for (int n = 0; n < b->nm; ++n) {
            if (n == m) continue;
            double r = 0.0;
            for (int d = 0; d < 3; ++d) r += pow(b->pos[3 * m + d] - b->pos[3 * n + d], 2);
            const double dist = sqrt(r) / dh;
            if (dist < ds) ds = dist;
        }
        b->ds[m] = ds;
    }
}

/* Partial-pivot LU (column-major, 1-based pivots) and the transposed solve:
 * the algorithm the oracle build of the reference links for dgetrf_/dgetrs_. */
static int lu_factor(int n, double *a, int lda, int *ipiv) {
#define A_(r, c) a[(size_t)(c) * lda + (r)]
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = fabs(A_(k, k));
        for (int r = k + 1; r < n; ++r) {
            double v = fabs(A_(r, k));
            if (v > best) { best = v; p = r; }
        }
        ipiv[k] = p + 1;
        if (A_(p, k) == 0.0) continue;
        if (p != k)
            for (int cc = 0; cc < n; ++cc) { double t = A_(k, cc); A_(k, cc) = A_(p, cc); A_(p, cc) = t; }
        const double inv = 1.0 / A_(k, k);
        for (int r = k + 1; r < n; ++r) A_(r, k) *= inv;
        for (int cc = k + 1; cc < n; ++cc) {
            const double akc = A_(k, cc);
            if (akc == 0.0) continue;
            for (int r = k + 1; r < n; ++r) A_(r, cc) -= A_(r, k) * akc;
        }
    }
    return 0;
}
static void lu_solve_t(int n, const double *a, int lda, const int *ipiv, double *x) {
    for (int r = 0; r < n; ++r) { double s = x[r]; for (int cc = 0; cc < r; ++cc) s -= A_(cc, r) * x[cc]; x[r] = s / A_(r, r); }
    for (int r = n - 1; r >= 0; --r) { double s = x[r]; for (int cc = r + 1; cc < n; ++cc) s -= A_(cc, r) * x[cc]; x[r] = s; }
    for (int k = n - 1; k >= 0; --k) { int p = ipiv[k] - 1; if (p != k) { double t = x[k]; x[k] = x[p]; x[p] = t; } }
#undef A_
}

/* Test entries for unit known-answer checks: the lattice tables, the
 * Roma delta kernel (ibm_deltaKernel, src/ObjectManager_ops_ibm.cpp:
 * 255-272) and the Guo forcing of one site (_LBM_forceGrid_opt, :928-990). */
int oracle_lattice(int Q, int *c, double *w, int *opp, int *refl) {
    const int (*cc)[3];
    const double *ww;
    const int *oo, *rr;
    if (Q == 9) { cc = C9; ww = W9; oo = OPP9; rr = &REF9[0][0]; }
    else if (Q == 19) { cc = C19; ww = W19; oo = OPP19; rr = &REF19[0][0]; }
    else if (Q == 27) { cc = C27; ww = W27; oo = OPP27; rr = &REF27[0][0]; }
    else { set_err("unsupported lattice"); return -1; }
    for (int v = 0; v < Q; ++v) {
        for (int d = 0; d < 3; ++d) c[3 * v + d] = cc[v][d];
        w[v] = ww[v];
        opp[v] = oo[v];
        for (int p = 0; p < 3; ++p) refl[p * Q + v] = rr[p * Q + v];
    }
    return 0;
}

double oracle_delta(double r, double dilation) { return delta_kernel(r, dilation); }

int oracle_guo(int Q, int dims, double omega, const double *u, const double *F, double *out) {
    oracle_grid g;
    memset(&g, 0, sizeof g);
    g.Q = Q;
    g.D = dims;
    if (Q == 9) { g.c = C9; g.w = W9; }
    else if (Q == 19) { g.c = C19; g.w = W19; }
    else if (Q == 27) { g.c = C27; g.w = W27; }
    else { set_err("unsupported lattice"); return -1; }
    g.d.omega = omega;
    g.force_i = out;
    g.u = (double *)u;
    g.force_xyz = (double *)F;
    force_grid(&g, 0);
    return 0;
}

/* The dense solver of the epsilon and FEM systems as a test entry: solves
 * A x = b for a row-major A (destroyed) with b in x, the way
 * GridUtils::solveLinearSystem (src/GridUtils.cpp:356-395) drives LAPACK
 * (dgetrf on the transposed view, dgetrs with trans = 'T'). */
int oracle_lu_solve_rowmajor(int n, double *A, double *x) {
    int *ipiv = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    lu_factor(n, A, n, ipiv);
    lu_solve_t(n, A, n, ipiv, x);
    free(ipiv);
    return 0;
}

/* ibm_findEpsilon (:773-920) + GridUtils::solveLinearSystem
 * (src/GridUtils.cpp:356-395) over the markers of `set` concatenated in
 * order: one body, or under L_UNIVERSAL_EPSILON_CALC every body of a level
 * (ibm_universalEpsilonGather/Scatter, :1067-1142). */
static void find_epsilon_set(ibm_body *const *set, int nset) {
    int n = 0;
    for (int b = 0; b < nset; ++b) n += set[b]->nm;
    if (n == 0) return;
    const int D = set[0]->owner->D;
    const double dh = set[0]->owner->d.dh;
    int *mb = (int *)malloc(sizeof(int) * n), *mm = (int *)malloc(sizeof(int) * n);
    for (int b = 0, I = 0; b < nset; ++b)
        for (int m = 0; m < set[b]->nm; ++m, ++I) { mb[I] = b; mm[I] = m; }
    double *A = (double *)calloc((size_t)n * n, sizeof(double));  /* row-major A[I][J] */
    for (int I = 0; I < n; ++I) {
        const ibm_body *bi = set[mb[I]];
        const int i = mm[I];
        for (int J = 0; J < n; ++J) {
            const ibm_body *bj = set[mb[J]];
            const int j = mm[J];
            double aij = 0.0;
            for (int s = bi->off[i]; s < bi->off[i + 1]; ++s) {
                const double dI = bi->delta[s];
                double dJ = delta_kernel((bj->pos[3 * j + 0] - bi->sx[s]) / dh, bj->dil[j]) *
                            delta_kernel((bj->pos[3 * j + 1] - bi->sy[s]) / dh, bj->dil[j]);
                if (D == 3) dJ = dJ * delta_kernel((bj->pos[3 * j + 2] - bi->sz[s]) / dh, bj->dil[j]);
                aij += dI * dJ * bi->area[i];
            }
            A[(size_t)I * n + J] = aij * bj->ds[j];
        }
    }
    /* The row-major copy read column-major is A^T; the transposed solve
     * then solves A x = 1. */
    int *ipiv = (int *)malloc(sizeof(int) * n);
    double *x = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) x[i] = 1.0;
    lu_factor(n, A, n, ipiv);
    lu_solve_t(n, A, n, ipiv, x);
    for (int I = 0; I < n; ++I) set[mb[I]]->eps[mm[I]] = x[I];
    free(A); free(ipiv); free(x); free(mb); free(mm);
}

static void find_epsilon(ibm_body *b) { find_epsilon_set(&b, 1); }

static int g_universal_eps = 0;

/* L_UNIVERSAL_EPSILON_CALC on (1) or off (0) for the next initialisation. */
void oracle_ibm_set_universal(int on) { g_universal_eps = on != 0; }

static void fem_move_bodies(oracle_grid *g, ibm_ctx *c);
static void fem_free_all(void);
static double fem_check_vel_diff(oracle_grid *g);
static void fem_commit_start_of_step(oracle_grid *g);
static int grid_has_flexible(oracle_grid *g);

static void ibm_apply(oracle_grid *g, ibm_ctx *c, int dosub);

static void ibm_pass(oracle_grid *g, void *vctx) { ibm_apply(g, (ibm_ctx *)vctx, 1); }

static void ibm_apply(oracle_grid *g, ibm_ctx *c, int dosub) {
    const int D = g->D;
    const int K = g->d.K, M = g->d.M;
    /* interpolate (all bodies), then force, then spread, then macro: the
     * four passes of ibm_apply each run over every body of the grid. */
    for (int ib = 0; ib < c->nb; ++ib) {
        ibm_body *b = &c->b[ib];
        if (b->owner != g) continue;
        for (int m = 0; m < b->nm; ++m) {
            double r = 0.0, mom[3] = {0.0, 0.0, 0.0};
            for (int s = b->off[m]; s < b->off[m + 1]; ++s) {
                const size_t id = (size_t)b->sk[s] + (size_t)b->sj[s] * K + (size_t)b->si[s] * K * M;
                r += g->rho[id] * b->delta[s] * b->area[m];
                for (int d = 0; d < D; d++) mom[d] += g->rho[id] * g->u[d + id * D] * b->delta[s] * b->area[m];
            }
            b->irho[m] = r;
            for (int d = 0; d < D; d++) {
                b->imom[3 * m + d] = mom[d];
            }
        }
    }
    for (int ib = 0; ib < c->nb; ++ib) {
        ibm_body *b = &c->b[ib];
        if (b->owner != g) continue;
        for (int m = 0; m < b->nm; ++m)
            for (int d = 0; d < D; d++)
                b->F[3 * m + d] = 2.0 * (b->imom[3 * m + d] - b->irho[m] * b->vel[3 * m + d]) / 1.0;
    }
    for (int ib = 0; ib < c->nb; ++ib) {
        ibm_body *b = &c->b[ib];
        if (b->owner != g) continue;
        for (int m = 0; m < b->nm; ++m)
            for (int s = b->off[m]; s < b->off[m + 1]; ++s) {
                const size_t id = (size_t)b->sk[s] + (size_t)b->sj[s] * K + (size_t)b->si[s] * K * M;
                const double volWidth = b->eps[m];
                const double volDepth = D == 3 ? b->ds[m] : 1.0;
                for (int d = 0; d < D; d++)
                    g->force_xyz[d + id * D] -= b->delta[s] * b->F[3 * m + d] * volWidth * volDepth * b->ds[m];
            }
    }
    for (int ib = 0; ib < c->nb; ++ib) {
        ibm_body *b = &c->b[ib];
        if (b->owner != g) continue;
        for (int m = 0; m < b->nm; ++m)
            for (int s = b->off[m]; s < b->off[m + 1]; ++s) {
                const int id = b->sk[s] + b->sj[s] * K + b->si[s] * K * M;
                macro_site(g, b->si[s], b->sj[s], b->sk[s], id, g->typ[id]);
            }
    }
    if (grid_has_flexible(g)) fem_move_bodies(g, c);
    if (dosub && grid_has_flexible(g)) {
        /* ObjectManager::ibm_subIterate (:111-185) */
        double res;
        int it = 0;
        do {
            memcpy(g->u, g->u_n, sizeof(double) * (size_t)g->ncell * g->D);
            reset_forces(g);
            ibm_apply(g, c, 0);
            res = fem_check_vel_diff(g);
            it++;
        } while (res > 1e-4 && it < 10);
        fem_commit_start_of_step(g);
    }
}

static ibm_ctx *g_ibm = NULL;

/* Adds a rigid body of nm markers (positions xyz[3*nm]) owned by grid g.
 * Returns the body index. */
int oracle_ibm_add_body(oracle_grid *g, int nm, const double *xyz) {
    if (!g_ibm) {
        g_ibm = (ibm_ctx *)calloc(1, sizeof(ibm_ctx));
    }
    oracle_grid *root = g;
    while (root->parent) root = root->parent;
    memcpy(g_ibm->global_edges, root->d.global_edges, sizeof(double) * 6);
    g_ibm->b = (ibm_body *)realloc(g_ibm->b, sizeof(ibm_body) * (g_ibm->nb + 1));
    ibm_body *b = &g_ibm->b[g_ibm->nb];
    memset(b, 0, sizeof *b);
    b->owner = g;
    b->nm = nm;
    b->pos = dup_d(xyz, 3 * (size_t)nm);
    b->vel = dup_d(NULL, 3 * (size_t)nm);
    b->eps = dup_d(NULL, nm);
    b->ds = dup_d(NULL, nm);
    b->dil = dup_d(NULL, nm);
    b->area = dup_d(NULL, nm);
    b->F = dup_d(NULL, 3 * (size_t)nm);
    b->irho = dup_d(NULL, nm);
    b->imom = dup_d(NULL, 3 * (size_t)nm);
    for (int m = 0; m < nm; ++m) { b->eps[m] = 0.0; b->dil[m] = 1.0; b->area[m] = 1.0; b->ds[m] = 1.0; }
    b->off = (int *)calloc(nm + 1, sizeof(int));
    g->has_ibm_bodies = 1;
    g->ibm_hook = ibm_pass;
    g->ibm_ctx = g_ibm;
    return g_ibm->nb++;
}

/* ObjectManager::ibm_initialise (:190-246): supports, then ds, then epsilon. */
int oracle_ibm_initialise(void) {
    if (!g_ibm) return 0;
    for (int ib = 0; ib < g_ibm->nb; ++ib)
        if (find_support(g_ibm, &g_ibm->b[ib])) return -1;
    for (int ib = 0; ib < g_ibm->nb; ++ib) compute_ds(&g_ibm->b[ib]);
    if (!g_universal_eps) {
        for (int ib = 0; ib < g_ibm->nb; ++ib) find_epsilon(&g_ibm->b[ib]);
        return 0;
    }
    for (int ib = 0; ib < g_ibm->nb; ++ib)
        if (grid_has_flexible(g_ibm->b[ib].owner)) {
            set_err("universal epsilon with flexible bodies is not reproduced");
            return -1;
        }
    /* one system per level over its bodies in body order */
    ibm_body **set = (ibm_body **)malloc(sizeof(ibm_body *) * (g_ibm->nb > 0 ? g_ibm->nb : 1));
    for (int lev = 0; lev < 16; ++lev) {
        int ns = 0;
        for (int ib = 0; ib < g_ibm->nb; ++ib)
            if (g_ibm->b[ib].owner->d.level == lev) set[ns++] = &g_ibm->b[ib];
        if (ns) find_epsilon_set(set, ns);
    }
    free(set);
    return 0;
}

/* Per-marker state: rows of (x y z Fx Fy Fz eps ds nsupp). */
int oracle_ibm_markers(int ib, double *out) {
    if (!g_ibm || ib >= g_ibm->nb) return -1;
    ibm_body *b = &g_ibm->b[ib];
    for (int m = 0; m < b->nm; ++m) {
        double *o = out + 9 * (size_t)m;
        o[0] = b->pos[3 * m]; o[1] = b->pos[3 * m + 1]; o[2] = b->pos[3 * m + 2];
        o[3] = b->F[3 * m]; o[4] = b->F[3 * m + 1]; o[5] = b->owner->D == 3 ? b->F[3 * m + 2] : 0.0;
        o[6] = b->eps[m]; o[7] = b->ds[m]; o[8] = (double)(b->off[m + 1] - b->off[m]);
    }
    return 0;
}

/* Support lists: rows of (marker i j k delta), total count returned. */
int oracle_ibm_supports(int ib, double *out, int cap) {
    if (!g_ibm || ib >= g_ibm->nb) return -1;
    ibm_body *b = &g_ibm->b[ib];
    const int n = b->off[b->nm];
    if (out && cap >= n)
        for (int m = 0; m < b->nm; ++m)
            for (int s = b->off[m]; s < b->off[m + 1]; ++s) {
                double *o = out + 5 * (size_t)s;
                o[0] = m; o[1] = b->si[s]; o[2] = b->sj[s]; o[3] = b->sk[s]; o[4] = b->delta[s];
            }
    return n;
}

void oracle_ibm_reset(void) {
    fem_free_all();
    if (!g_ibm) return;
    for (int ib = 0; ib < g_ibm->nb; ++ib) {
        ibm_body *b = &g_ibm->b[ib];
        free(b->pos); free(b->vel); free(b->eps); free(b->ds); free(b->dil); free(b->area); free(b->F);
        free(b->irho); free(b->imom); free(b->off); free(b->si); free(b->sj); free(b->sk); free(b->sx);
        free(b->sy); free(b->sz); free(b->delta);
    }
    free(g_ibm->b);
    free(g_ibm);
    g_ibm = NULL;
}

/* ============================ FEM filaments ==============================
 * Restatement of FEMBody / FEMElement (src/FEMBody.cpp, src/FEMElement.cpp)
 * for a planar co-rotational Euler-Bernoulli beam with 3 DOFs per node,
 * Newmark-beta (alpha 0.25, delta 0.5) and Newton-Raphson (tol 1e-10, 20
 * iterations), coupled to the IB markers of its body; and the FSI
 * sub-iteration loop of ObjectManager (:61-185, :988-1032). */

#define NB_ALPHA 0.25
#define NB_DELTA 0.5
#define FSI_RELAX 0.5

typedef struct fem_el {
    double length0, length, area, I, E, density, angles;
    double T[6][6], F[6];
    int nchild;
    int child_node[64];
    double child_z1[64], child_z2[64];
} fem_el;

typedef struct fem_body {
    int ib;              /* IB body index */
    int nel, ndof, bc;
    double *pos0, *pos, *ang0, *ang;   /* nodes: pos 3 per node */
    fem_el *el;
    double *M, *K, *R, *F, *U, *U_n, *delU, *Ud, *Ud_n, *Udd, *Udd_n;  /* dense M,K row-major */
    int *parent_el;
    double *parent_zeta;
    double *mpos0;       /* marker initial positions (3 per marker) */
    double *mvel_km1;    /* previous marker velocities */
    double fsi_vel_scale; /* L_UX0 * dt / dh */
    double dm;           /* GridObj::dm of the owning grid */
    int it;
    double res;
} fem_body;

static fem_body *g_fem = NULL;
static int g_nfem = 0;

static void mat6_mul(const double A[6][6], const double B[6][6], double C[6][6]) {
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) {
            double s = 0.0;
            for (int k = 0; k < 6; ++k) s += A[r][k] * B[k][c];
            C[r][c] = s;
        }
}
static void mat6_T(const double A[6][6], double B[6][6]) {
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) B[c][r] = A[r][c];
}
/* GridUtils::matrix_multiply(A, x) for square A (:257-279). */
static void matvec(int n, const double *A, const double *x, double *y) {
    for (int r = 0; r < n; ++r) {
        double s = 0.0;
        for (int c = 0; c < n; ++c) s += A[(size_t)r * n + c] * x[c];
        y[r] = s;
    }
}

static void set_T(fem_el *e) {
    memset(e->T, 0, sizeof e->T);
    e->T[0][0] = e->T[1][1] = e->T[3][3] = e->T[4][4] = cos(e->angles);
    e->T[0][1] = e->T[3][4] = sin(e->angles);
    e->T[1][0] = e->T[4][3] = -sin(e->angles);
    e->T[2][2] = e->T[5][5] = 1.0;
}

/* FEMBody::updateFEMValues (:297-325). */
static void fem_update_values(fem_body *f) {
    const int D = 2;
    for (int n = 0; n <= f->nel; ++n) {
        for (int d = 0; d < D; d++) f->pos[3 * n + d] = f->pos0[3 * n + d] + f->U[n * 3 + d];
        f->ang[n] = f->ang0[n] + f->U[n * 3 + D];
    }
    for (int e = 0; e < f->nel; ++e) {
        double v[3];
        for (int d = 0; d < 3; ++d) v[d] = f->pos[3 * (e + 1) + d] - f->pos[3 * e + d];
        f->el[e].angles = atan2(v[1], v[0]);
        double r = 0.0;
        for (int d = 0; d < 3; ++d) r += pow(v[d], 2);
        f->el[e].length = sqrt(r);
        set_T(&f->el[e]);
    }
}

static void assemble_vec(const fem_body *f, int e, const double *loc, double *glob) {
    for (int i = 0; i < 6; ++i) glob[e * 3 + i] += loc[i];
}
static void assemble_mat(const fem_body *f, int e, const double L[6][6], double *G) {
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) G[(size_t)(e * 3 + i) * f->ndof + (e * 3 + j)] += L[i][j];
}

/* FEMElement::loadVector (:133-173). */
static void fem_load_vector(fem_body *f, int e, const ibm_body *b, double forceScale) {
    fem_el *E = &f->el[e];
    for (int q = 0; q < E->nchild; ++q) {
        const int node = E->child_node[q];
        const double a = E->child_z1[q], bb = E->child_z2[q];
        const double Ts[2][2] = {{E->T[0][0], E->T[0][1]}, {E->T[1][0], E->T[1][1]}};
        double fv[2];
        const double sc = b->eps[node] * 1.0 * forceScale;
        const double fx[2] = {b->F[3 * node] * sc, b->F[3 * node + 1] * sc};
        for (int r = 0; r < 2; ++r) {
            double s = 0.0;
            for (int c = 0; c < 2; ++c) s += Ts[r][c] * fx[c];
            fv[r] = s;
        }
        const double L = E->length;
        double R[6];
        R[0] = fv[0] * 0.5 * L * (0.5 * bb - 0.5 * a + 0.25 * SQ(a) - 0.25 * SQ(bb));
        R[1] = fv[1] * 0.5 * L * (0.5 * bb - 0.5 * a - SQ(a) * SQ(a) / 16.0 + SQ(bb) * SQ(bb) / 16.0 + 3.0 * SQ(a) / 8.0 - 3.0 * SQ(bb) / 8.0);
        R[2] = fv[1] * 0.5 * L * (L * (-SQ(a) * SQ(a) + SQ(bb) * SQ(bb)) / 32.0 - L * (-(a * a * a) + (bb * bb * bb)) / 24.0 - L * (-SQ(a) + SQ(bb)) / 16.0 + L * (bb - a) / 8.0);
        R[3] = fv[0] * 0.5 * L * (-0.25 * SQ(a) + 0.25 * SQ(bb) + 0.5 * bb - 0.5 * a);
        R[4] = fv[1] * 0.5 * L * (0.5 * bb - 0.5 * a + SQ(a) * SQ(a) / 16.0 - SQ(bb) * SQ(bb) / 16.0 - 3.0 * SQ(a) / 8.0 + 3.0 * SQ(bb) / 8.0);
        R[5] = fv[1] * 0.5 * L * (L * (-SQ(a) * SQ(a) + SQ(bb) * SQ(bb)) / 32.0 + L * (-(a * a * a) + (bb * bb * bb)) / 24.0 - L * (-SQ(a) + SQ(bb)) / 16.0 - L * (bb - a) / 8.0);
        double Tt[6][6], RG[6];
        mat6_T(E->T, Tt);
        for (int r = 0; r < 6; ++r) {
            double s = 0.0;
            for (int c = 0; c < 6; ++c) s += Tt[r][c] * R[c];
            RG[r] = s;
        }
        assemble_vec(f, e, RG, f->R);
    }
}

/* FEMElement::massMatrix (:178-213). */
static void fem_mass(fem_body *f, int e) {
    fem_el *E = &f->el[e];
    double Ml[6][6];
    memset(Ml, 0, sizeof Ml);
    const double C1 = E->density * E->area * E->length0 / 420.0, L0 = E->length0;
    Ml[0][0] = C1 * 140.0; Ml[0][3] = C1 * 70.0; Ml[1][1] = C1 * 156.0; Ml[1][2] = C1 * 22.0 * L0;
    Ml[1][4] = C1 * 54; Ml[1][5] = C1 * (-13.0 * L0); Ml[2][2] = C1 * 4.0 * SQ(L0); Ml[2][4] = C1 * 13.0 * L0;
    Ml[2][5] = C1 * (-3.0 * SQ(L0)); Ml[3][3] = C1 * 140.0; Ml[4][4] = C1 * 156.0; Ml[4][5] = C1 * (-22.0 * L0);
    Ml[5][5] = C1 * 4.0 * SQ(L0);
    for (int i = 1; i < 6; i++)
        for (int j = 0; j < i; j++) Ml[i][j] = Ml[j][i];
    double Tt[6][6], A[6][6], G[6][6];
    mat6_T(E->T, Tt);
    mat6_mul(Tt, Ml, A);
    mat6_mul(A, E->T, G);
    assemble_mat(f, e, G, f->M);
}

/* FEMElement::stiffMatrix (:218-268). */
static void fem_stiff(fem_body *f, int e) {
    fem_el *E = &f->el[e];
    double Kl[6][6];
    memset(Kl, 0, sizeof Kl);
    const double EE = E->E, A = E->area, I = E->I, L0 = E->length0;
    Kl[0][0] = EE * A / L0; Kl[0][3] = -EE * A / L0;
    Kl[1][1] = 12.0 * EE * I / (L0 * L0 * L0); Kl[1][2] = 6.0 * EE * I / SQ(L0);
    Kl[1][4] = -12.0 * EE * I / (L0 * L0 * L0); Kl[1][5] = 6.0 * EE * I / SQ(L0);
    Kl[2][2] = 4.0 * EE * I / L0; Kl[2][4] = -6.0 * EE * I / SQ(L0); Kl[2][5] = 2.0 * EE * I / L0;
    Kl[3][3] = EE * A / L0; Kl[4][4] = 12.0 * EE * I / (L0 * L0 * L0); Kl[4][5] = -6.0 * EE * I / SQ(L0);
    Kl[5][5] = 4.0 * EE * I / L0;
    for (int i = 1; i < 6; i++)
        for (int j = 0; j < i; j++) Kl[i][j] = Kl[j][i];
    const double F0 = -E->F[0], V0 = E->F[4];
    Kl[0][1] += -V0 / L0; Kl[0][4] += V0 / L0; Kl[1][0] += -V0 / L0; Kl[1][1] += F0 / L0;
    Kl[1][3] += V0 / L0; Kl[1][4] += -F0 / L0; Kl[3][1] += V0 / L0; Kl[3][4] += -V0 / L0;
    Kl[4][0] += V0 / L0; Kl[4][1] += -F0 / L0; Kl[4][3] += -V0 / L0; Kl[4][4] += F0 / L0;
    double Tt[6][6], B[6][6], G[6][6];
    mat6_T(E->T, Tt);
    mat6_mul(Tt, Kl, B);
    mat6_mul(B, E->T, G);
    assemble_mat(f, e, G, f->K);
}

/* FEMElement::forceVector (:273-302). */
static void fem_force(fem_body *f, int e) {
    fem_el *E = &f->el[e];
    const double a1 = f->ang[e], a2 = f->ang[e + 1];
    const double L = E->length, L0 = E->length0;
    const double u = (SQ(L) - SQ(L0)) / (L + L0);
    const double t1 = atan2(cos(E->angles) * sin(a1) - sin(E->angles) * cos(a1), cos(E->angles) * cos(a1) + sin(E->angles) * sin(a1));
    const double t2 = atan2(cos(E->angles) * sin(a2) - sin(E->angles) * cos(a2), cos(E->angles) * cos(a2) + sin(E->angles) * sin(a2));
    const double F0 = (E->E * E->area / L0) * u;
    const double M1 = (2 * E->E * E->I / L0) * (2.0 * t1 + t2);
    const double M2 = (2 * E->E * E->I / L0) * (t1 + 2.0 * t2);
    E->F[0] = -F0; E->F[1] = (1.0 / L0) * (M1 + M2); E->F[2] = M1;
    E->F[3] = F0; E->F[4] = -(1.0 / L0) * (M1 + M2); E->F[5] = M2;
    double Tt[6][6], FG[6];
    mat6_T(E->T, Tt);
    for (int r = 0; r < 6; ++r) {
        double s = 0.0;
        for (int c = 0; c < 6; ++c) s += Tt[r][c] * E->F[c];
        FG[r] = s;
    }
    assemble_vec(f, e, FG, f->F);
}

/* GridUtils::solveLinearSystem (src/GridUtils.cpp:356-395) with BC offset. */
static void solve_bc(int dim, const double *Arow, const double *b, int BC, double *out) {
    const int n = dim - BC;
    double *a = (double *)malloc(sizeof(double) * (size_t)dim * dim);
    memcpy(a, Arow, sizeof(double) * (size_t)dim * dim);
    for (int i = 0; i < dim; ++i) out[i] = b[i];
    int *ipiv = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
    /* row-major a read column-major from offset BC*dim+BC with lda = dim */
    double *sub = a + (size_t)BC * dim + BC;
    lu_factor(n, sub, dim, ipiv);
    lu_solve_t(n, sub, dim, ipiv, out + BC);
    for (int i = 0; i < BC; ++i) out[i] = 0.0;
    free(a);
    free(ipiv);
}

static void fem_newmark_set(fem_body *f, double Dt) {
    const int n = f->ndof;
    const double a0 = 1.0 / (NB_ALPHA * SQ(Dt)), a2 = 1.0 / (NB_ALPHA * Dt), a3 = 1.0 / (2.0 * NB_ALPHA) - 1.0;
    double *Meff = (double *)malloc(sizeof(double) * n), *MF = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) Meff[i] = a0 * (f->U_n[i] - f->U[i]) + a2 * f->Ud[i] + a3 * f->Udd[i];
    matvec(n, f->M, Meff, MF);
    for (int i = 0; i < n; i++) {
        f->F[i] = f->R[i] - f->F[i] + MF[i];
        for (int j = 0; j < n; j++) f->K[(size_t)i * n + j] += a0 * f->M[(size_t)i * n + j];
    }
    free(Meff);
    free(MF);
}

/* FEMBody::dynamicFEM (:136-179) with newtonRaphsonIterator (:183-218),
 * checkNRConvergence (:224-231), finishNewmark (:236-255). */
static void fem_dynamic(fem_body *f, ibm_body *b) {
    oracle_grid *g = b->owner;
    const int n = f->ndof;
    const double Dt = g->d.dt;
    memcpy(f->U, f->U_n, sizeof(double) * n);
    memcpy(f->Ud, f->Ud_n, sizeof(double) * n);
    memcpy(f->Udd, f->Udd_n, sizeof(double) * n);
    fem_update_values(f);
    memset(f->R, 0, sizeof(double) * n);
    const double forceScale = f->dm / SQ(Dt);
    for (int e = 0; e < f->nel; ++e) fem_load_vector(f, e, b, forceScale);
    f->it = 0;
    do {
        memset(f->F, 0, sizeof(double) * n);
        memset(f->M, 0, sizeof(double) * (size_t)n * n);
        memset(f->K, 0, sizeof(double) * (size_t)n * n);
        for (int e = 0; e < f->nel; ++e) {
            fem_force(f, e);
            fem_mass(f, e);
            fem_stiff(f, e);
        }
        fem_newmark_set(f, Dt);
        solve_bc(n, f->K, f->F, f->bc, f->delU);
        for (int i = 0; i < n; i++) f->U[i] = f->U[i] + f->delU[i];
        fem_update_values(f);
        double dp = 0.0;
        for (int i = 0; i < n; i++) dp += f->delU[i] * f->delU[i];
        const double L = f->el[0].length0 * f->nel;
        f->res = sqrt(dp / (double)n) / L;
        f->it++;
    } while (f->res > 1e-10 && f->it < 20);
    const double a6 = 1.0 / (NB_ALPHA * SQ(Dt)), a7 = -1.0 / (NB_ALPHA * Dt), a8 = -(1.0 / (2.0 * NB_ALPHA) - 1.0);
    const double a9 = Dt * (1.0 - NB_DELTA), a10 = NB_DELTA * Dt;
    for (int i = 0; i < n; i++) {
        const double s = a6 * (f->U[i] - f->U_n[i]) + a7 * f->Ud[i] + a8 * f->Udd[i];
        f->Ud[i] = f->Ud[i] + a9 * f->Udd[i] + a10 * s;
        f->Udd[i] = s;
    }
    /* FEMBody::updateIBMarkers (:329-370) */
    for (int m = 0; m < b->nm; ++m) {
        const fem_el *E = &f->el[f->parent_el[m]];
        const double z = f->parent_zeta[m];
        double dU[6], dV[6], lU[6], lV[6];
        const int e = f->parent_el[m];
        for (int i = 0; i < 6; ++i) { dU[i] = f->U[e * 3 + i]; dV[i] = f->Ud[e * 3 + i]; }
        for (int r = 0; r < 6; ++r) {
            double s1 = 0.0, s2 = 0.0;
            for (int c = 0; c < 6; ++c) { s1 += E->T[r][c] * dU[c]; s2 += E->T[r][c] * dV[c]; }
            lU[r] = s1; lV[r] = s2;
        }
        const double zz = (z + 1.0) / 2.0, L = E->length;
        const double N0 = 1.0 - (z + 1.0) / 2.0;
        const double N1 = 1.0 - 3.0 * SQ(zz) + 2.0 * (zz * zz * zz);
        const double N2 = (zz - 2.0 * SQ(zz) + (zz * zz * zz)) * L;
        const double N3 = (z + 1.0) / 2.0;
        const double N4 = 3.0 * SQ(zz) - 2.0 * (zz * zz * zz);
        const double N5 = (-SQ(zz) + (zz * zz * zz)) * L;
        const double su[2] = {lU[0] * N0 + lU[3] * N3, lU[1] * N1 + lU[2] * N2 + lU[4] * N4 + lU[5] * N5};
        const double sv[2] = {lV[0] * N0 + lV[3] * N3, lV[1] * N1 + lV[2] * N2 + lV[4] * N4 + lV[5] * N5};
        const double Tt[2][2] = {{E->T[0][0], E->T[1][0]}, {E->T[0][1], E->T[1][1]}};
        double gu[2], gv[2];
        for (int r = 0; r < 2; ++r) {
            double s1 = 0.0, s2 = 0.0;
            for (int c = 0; c < 2; ++c) { s1 += Tt[r][c] * su[c]; s2 += Tt[r][c] * sv[c]; }
            gu[r] = s1;
            gv[r] = s2 * (g->d.dt / g->d.dh);
        }
        for (int d = 0; d < 2; d++) {
            b->pos[3 * m + d] = f->mpos0[3 * m + d] + gu[d];
            f->mvel_km1[3 * m + d] = b->vel[3 * m + d];
            b->vel[3 * m + d] = FSI_RELAX * gv[d] + (1.0 - FSI_RELAX) * f->mvel_km1[3 * m + d];
        }
    }
}

static int grid_has_flexible(oracle_grid *g) {
    for (int k = 0; k < g_nfem; ++k)
        if (g_ibm->b[g_fem[k].ib].owner == g) return 1;
    return 0;
}

/* ObjectManager::ibm_moveBodies (:61-104): FEM for every flexible body on
 * the grid, new supports for them, then ds and epsilon for all bodies of
 * the grid. */
static void fem_move_bodies(oracle_grid *g, ibm_ctx *c) {
    for (int k = 0; k < g_nfem; ++k)
        if (c->b[g_fem[k].ib].owner == g) fem_dynamic(&g_fem[k], &c->b[g_fem[k].ib]);
    for (int k = 0; k < g_nfem; ++k)
        if (c->b[g_fem[k].ib].owner == g) find_support(c, &c->b[g_fem[k].ib]);
    for (int ib = 0; ib < c->nb; ++ib)
        if (c->b[ib].owner == g) compute_ds(&c->b[ib]);
    for (int ib = 0; ib < c->nb; ++ib)
        if (c->b[ib].owner == g) find_epsilon(&c->b[ib]);
}

/* ObjectManager::ibm_checkVelDiff (:988-1032). */
static double fem_check_vel_diff(oracle_grid *g) {
    double res = 0.0;
    for (int k = 0; k < g_nfem; ++k) {
        fem_body *f = &g_fem[k];
        ibm_body *b = &g_ibm->b[f->ib];
        if (b->owner != g) continue;
        for (int m = 0; m < b->nm; ++m) {
            double r = 0.0;
            for (int d = 0; d < 3; ++d) r += pow(b->vel[3 * m + d] - f->mvel_km1[3 * m + d], 2);
            const double v = sqrt(r) / f->fsi_vel_scale;
            if (fabs(v) > res) res = fabs(v);
        }
    }
    return res;
}

static void fem_commit_start_of_step(oracle_grid *g) {
    for (int k = 0; k < g_nfem; ++k) {
        fem_body *f = &g_fem[k];
        if (g_ibm->b[f->ib].owner != g) continue;
        memcpy(f->U_n, f->U, sizeof(double) * f->ndof);
        memcpy(f->Ud_n, f->Ud, sizeof(double) * f->ndof);
        memcpy(f->Udd_n, f->Udd, sizeof(double) * f->ndof);
    }
}

/* A flexible filament: the markers of Body's filament builder
 * (inc/Body.h:143-187) and its FEMBody (src/FEMBody.cpp:48-130) with the
 * IB <-> FEM node mapping (:378-424).  angle_v in degrees.  The beam is
 * planar (x-y); on a 3D grid the load and the marker update take the x and
 * y components and markers keep their z, the one change that lets the
 * reference's planar FEM run in 3D (where it aborts on a matrix-size
 * mismatch).  Returns the IB body index. */
int oracle_ibm_add_filament(oracle_grid *g, const double start[3], double length, double height, double depth,
                            double angle_v, int nel, int clamped, double density, double E, double dm,
                            double fsi_vel_scale) {
    if (g->D == 3 && !(depth > 0)) { set_err("a filament on a 3D grid needs a positive depth"); return -1; }
    const double dh = g->d.dh;
    const int nmk = (int)floor(length / dh) + 1;
    const double spacing = length / (nmk - 1);
    const double spacing_h = spacing * cos(angle_v * L_PI / 180);
    double *xyz = (double *)malloc(sizeof(double) * 3 * nmk);
    for (int i = 0; i < nmk; i++) {
        xyz[3 * i + 0] = start[0] + i * spacing_h * cos(0.0 * L_PI / 180.0);
        xyz[3 * i + 1] = start[1] + i * spacing * sin(angle_v * L_PI / 180.0);
        xyz[3 * i + 2] = start[2] + i * spacing_h * sin(0.0 * L_PI / 180.0);
    }
    const int ib = oracle_ibm_add_body(g, nmk, xyz);
    free(xyz);
    g->has_flexible_bodies = 1;
    g_fem = (fem_body *)realloc(g_fem, sizeof(fem_body) * (g_nfem + 1));
    fem_body *f = &g_fem[g_nfem++];
    memset(f, 0, sizeof *f);
    f->ib = ib;
    f->nel = nel;
    f->ndof = (nel + 1) * 3;
    f->bc = clamped ? 3 : 2;
    f->dm = dm;
    f->fsi_vel_scale = fsi_vel_scale;
    const double fspacing = length / nel;
    const double fspacing_h = fspacing * cos(angle_v * L_PI / 180);
    f->pos0 = dup_d(NULL, 3 * (size_t)(nel + 1));
    f->pos = dup_d(NULL, 3 * (size_t)(nel + 1));
    f->ang0 = dup_d(NULL, nel + 1);
    f->ang = dup_d(NULL, nel + 1);
    for (int i = 0; i < nel + 1; i++) {
        f->pos0[3 * i + 0] = start[0] + i * fspacing_h * cos(0.0 * L_PI / 180.0);
        f->pos0[3 * i + 1] = start[1] + i * fspacing * sin(angle_v * L_PI / 180.0);
        f->pos0[3 * i + 2] = start[2] + i * fspacing_h * sin(0.0 * L_PI / 180.0);
        f->ang0[i] = angle_v * L_PI / 180.0;
        f->ang[i] = f->ang0[i];
    }
    memcpy(f->pos, f->pos0, sizeof(double) * 3 * (nel + 1));
    if (g->D == 2) depth = dh; /* 2D: unit lattice depth (src/FEMBody.cpp:103-105) */
    f->el = (fem_el *)calloc(nel, sizeof(fem_el));
    for (int e = 0; e < nel; ++e) {
        fem_el *el = &f->el[e];
        el->length0 = fspacing;
        el->length = fspacing;
        el->area = height * depth;
        el->angles = angle_v * L_PI / 180.0;
        el->I = depth * (height * height * height) / 12.0;
        el->E = E;
        el->density = density;
        set_T(el);
    }
    /* computeNodeMapping */
    const int nI = nmk, nF = nel + 1;
    f->parent_el = (int *)malloc(sizeof(int) * nI);
    f->parent_zeta = (double *)malloc(sizeof(double) * nI);
    f->parent_el[0] = 0;
    f->parent_zeta[0] = -1.0;
    for (int i = 1; i < nI; i++) {
        const double q = i * ((nF - 1.0) / (nI - 1.0));
        if (fmod(q, 1.0) == 0.0) {
            f->parent_el[i] = (int)floor(q) - 1;
            f->parent_zeta[i] = 1.0;
        } else {
            f->parent_el[i] = (int)floor(q);
            f->parent_zeta[i] = fmod(q, 1.0) * 2.0 - 1.0;
        }
    }
    for (int e = 0; e < nel; ++e)
        for (int node = 0; node < nI; ++node) {
            double n1 = -1 + 2.0 * ((node - 0.5) * ((nF - 1.0) / (nI - 1.0)) - e) / 1.0;
            double n2 = -1 + 2.0 * ((node + 0.5) * ((nF - 1.0) / (nI - 1.0)) - e) / 1.0;
            if ((n1 > -1.0 && n1 < 1.0) || (n2 > -1.0 && n2 < 1.0)) {
                if (n1 < -1.0) n1 = -1.0;
                if (n2 > 1.0) n2 = 1.0;
                fem_el *el = &f->el[e];
                if (el->nchild >= 64) { set_err("too many IB nodes per element"); return -1; }
                el->child_node[el->nchild] = node;
                el->child_z1[el->nchild] = n1;
                el->child_z2[el->nchild] = n2;
                el->nchild++;
            }
        }
    const int n = f->ndof;
    f->M = dup_d(NULL, (size_t)n * n);
    f->K = dup_d(NULL, (size_t)n * n);
    f->R = dup_d(NULL, n); f->F = dup_d(NULL, n); f->U = dup_d(NULL, n); f->U_n = dup_d(NULL, n);
    f->delU = dup_d(NULL, n); f->Ud = dup_d(NULL, n); f->Ud_n = dup_d(NULL, n);
    f->Udd = dup_d(NULL, n); f->Udd_n = dup_d(NULL, n);
    ibm_body *b = &g_ibm->b[ib];
    f->mpos0 = dup_d(b->pos, 3 * (size_t)nmk);
    f->mvel_km1 = dup_d(NULL, 3 * (size_t)nmk);
    return ib;
}

/* FEM state of filament k: U (ndof values) and node positions. */
int oracle_fem_state(int k, double *U, int *ndof, int *it, double *res) {
    if (k < 0 || k >= g_nfem) return -1;
    fem_body *f = &g_fem[k];
    if (ndof) *ndof = f->ndof;
    if (U) memcpy(U, f->U_n, sizeof(double) * f->ndof);
    if (it) *it = f->it;
    if (res) *res = f->res;
    return 0;
}

static void fem_free_all(void) {
    for (int k = 0; k < g_nfem; ++k) {
        fem_body *f = &g_fem[k];
        free(f->pos0); free(f->pos); free(f->ang0); free(f->ang); free(f->el);
        free(f->M); free(f->K); free(f->R); free(f->F); free(f->U); free(f->U_n); free(f->delU);
        free(f->Ud); free(f->Ud_n); free(f->Udd); free(f->Udd_n); free(f->parent_el); free(f->parent_zeta);
        free(f->mpos0); free(f->mvel_km1);
    }
    free(g_fem);
    g_fem = NULL;
    g_nfem = 0;
}
