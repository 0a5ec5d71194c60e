// Immersed-boundary bodies and the IBM pass of a grid
// (ObjectManager::ibm_apply, LUMA src/ObjectManager_ops_ibm.cpp:33-54).
//
// Set-up runs once on the host in FP64 for rigid bodies, with the
// reference's algorithms and order: support search around the enclosing
// voxel (ibm_findSupport, :279-453) with tensor-product Roma delta values
// (:255-272, :462-491), marker spacing (ibm_computeDs, :927-981) and the
// epsilon system (ibm_findEpsilon, :773-920) solved by partial-pivot LU.
// The per-step pass runs on the device (k_general.cu): one thread per
// marker interpolates and forms the force; one thread per distinct support
// site gathers the spread contributions in the reference's order (no
// atomics) and recomputes the macroscopic values there.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

#include "dispatch.hpp"
#include "grid.hpp"
#include "kernels.hpp"

using namespace luma;

namespace {

double delta_kernel(double radius, double dilation) {
    const double mag_r = std::fabs(radius) / dilation;
    if (mag_r > 1.5) return 0.0;
    if (mag_r > 0.5) return (5.0 - (3.0 * mag_r) - std::sqrt(-3.0 * std::pow(1.0 - mag_r, 2) + 1.0)) / 6.0;
    return (1.0 + std::sqrt(1.0 - 3.0 * std::pow(mag_r, 2))) / 3.0;
}

const luma_gpu_grid *root_of(const luma_gpu_grid *g) {
    while (g->parent) g = g->parent;
    return g;
}

// What the rigid-body set-up reads of a grid: sizes, spacing, site
// positions and the level-0 edges.  Built from a device grid or, for the
// host-only entry point, from a grid descriptor.
struct GridView {
    int dims, N, M, K, level;
    double dh;
    const double *x, *y, *z;  // site positions
    const double *E;          // level-0 global edges
};

GridView view_of(const luma_gpu_grid *g) {
    return GridView{g->d.dims, g->d.N, g->d.M, g->d.K, g->d.level, g->d.dh,
                    g->hx.data(), g->hy.data(), g->hz.data(), root_of(g)->d.global_edges};
}

double grid_start(const GridView &g, int axis) {
    const double *p = axis == 0 ? g.x : (axis == 1 ? g.y : g.z);
    return g.level == 0 ? 0.0 : p[0] - g.dh / 2.0;
}

void support_delta(const GridView &g, const IbmBody &b, int m, const double est[3], double *out) {
    const double dh = g.dh;
    const double *x = &b.pos[3 * m];
    double v = delta_kernel((est[0] - x[0]) / dh, b.dil[m]) * delta_kernel((est[1] - x[1]) / dh, b.dil[m]);
    if (g.dims == 3) v = v * delta_kernel((est[2] - x[2]) / dh, b.dil[m]);
    *out = v;
}

int find_support(const GridView &g, IbmBody &b) {
    const int D = g.dims;
    const double dh = g.dh;
    const double *E = g.E;
    b.off.assign(b.nm + 1, 0);
    b.si.clear(); b.sj.clear(); b.sk.clear();
    b.sx.clear(); b.sy.clear(); b.sz.clear(); b.delta.clear();
    auto push = [&](int i, int j, int k, const double p[3], int m) {
        b.si.push_back(i); b.sj.push_back(j); b.sk.push_back(k);
        b.sx.push_back(p[0]); b.sy.push_back(p[1]); b.sz.push_back(p[2]);
        double dv;
        support_delta(g, b, m, p, &dv);
        b.delta.push_back(dv);
    };
    for (int m = 0; m < b.nm; ++m) {
        b.off[m] = (int)b.si.size();
        const double *x = &b.pos[3 * m];
        const int in = (int)std::floor((x[0] - grid_start(g, 0)) / dh);
        const int jn = (int)std::floor((x[1] - grid_start(g, 1)) / dh);
        const int kn = D == 3 ? (int)std::floor((x[2] - grid_start(g, 2)) / dh) : 0;
        if (in < 0 || jn < 0 || kn < 0 || in >= g.N || jn >= g.M || kn >= g.K)
            return luma_set_error(LUMA_E_DOMAIN, "IB marker %d is no longer inside its grid", m);
        const double near[3] = {g.x[in], g.y[jn], D == 3 ? g.z[kn] : 0.0};
        push(in, jn, kn, near, m);
        for (int i = in - 5; i <= in + 5; i++)
            for (int j = jn - 5; j <= jn + 5; j++)
                for (int k = (D == 3 ? kn - 5 : 0); k <= (D == 3 ? kn + 5 : 0); k++) {
                    double est[3] = {near[0] + (i - in) * dh, near[1] + (j - jn) * dh, near[2]};
                    if (D == 3) est[2] = near[2] + (k - kn) * dh;
                    const bool in_cage = (std::fabs(x[0] - est[0]) / dh < 1.5 * b.dil[m]) &&
                                         (std::fabs(x[1] - est[1]) / dh < 1.5 * b.dil[m]) &&
                                         (D == 2 || std::fabs(x[2] - est[2]) / dh < 1.5 * b.dil[m]);
                    const bool in_domain = !(est[0] < E[0] || est[0] > E[1] || est[1] < E[2] || est[1] > E[3] ||
                                             (D == 3 && (est[2] < E[4] || est[2] > E[5])));
                    if (in_cage && in_domain && (i != in || j != jn || (D == 3 && k != kn))) {
                        if (i < 0 || j < 0 || k < 0 || i >= g.N || j >= g.M || k >= g.K)
                            return luma_set_error(LUMA_E_DOMAIN, "IB marker %d has supports off its grid", m);
                        push(i, j, k, est, m);
                    }
                }
    }
    b.off[b.nm] = (int)b.si.size();
    return LUMA_OK;
}

void compute_ds(const GridView &g, IbmBody &b) {
    const double dh = g.dh;
#pragma omp parallel for schedule(static) if (b.nm > 512)
    for (int m = 0; m < b.nm; ++m) {
        double ds = 10.0;
        for (int n = 0; n < b.nm; ++n) {
            if (n == m) continue;
            double r = 0.0;
            for (int d = 0; d < 3; ++d) r += std::pow(b.pos[3 * m + d] - b.pos[3 * n + d], 2);
            const double dist = std::sqrt(r) / dh;
            if (dist < ds) ds = dist;
        }
        b.ds[m] = ds;
    }
}

// Dense LU with partial pivoting, column-major, then the transposed solve
// (the reference calls dgetrf_/dgetrs_ with trans='T' on a row-major copy,
// which solves A x = b).  The column updates of one elimination step are
// independent, so they run on all host threads without changing a single
// floating-point operation.
void lu_solve_transposed(int n, std::vector<double> &a, std::vector<double> &x) {
    std::vector<int> ipiv(n);
#define A_(r, c) a[(size_t)(c) * n + (r)]
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = std::fabs(A_(k, k));
        for (int r = k + 1; r < n; ++r) {
            const double v = std::fabs(A_(r, k));
            if (v > best) { best = v; p = r; }
        }
        ipiv[k] = p + 1;
        if (A_(p, k) == 0.0) continue;
        if (p != k)
            for (int c = 0; c < n; ++c) std::swap(A_(k, c), A_(p, c));
        const double inv = 1.0 / A_(k, k);
        for (int r = k + 1; r < n; ++r) A_(r, k) *= inv;
#pragma omp parallel for schedule(static) if (n - k > 256)
        for (int c = k + 1; c < n; ++c) {
            const double akc = A_(k, c);
            if (akc == 0.0) continue;
            for (int r = k + 1; r < n; ++r) A_(r, c) -= A_(r, k) * akc;
        }
    }
    for (int r = 0; r < n; ++r) { double s = x[r]; for (int c = 0; c < r; ++c) s -= A_(c, r) * x[c]; x[r] = s / A_(r, r); }
    for (int r = n - 1; r >= 0; --r) { double s = x[r]; for (int c = r + 1; c < n; ++c) s -= A_(c, r) * x[c]; x[r] = s; }
    for (int k = n - 1; k >= 0; --k) { const int p = ipiv[k] - 1; if (p != k) std::swap(x[k], x[p]); }
#undef A_
}

// One epsilon system over the markers of `set`, concatenated in order:
// a single body as ibm_findEpsilon builds it, or every body of a level as
// one system under L_UNIVERSAL_EPSILON_CALC (ibm_universalEpsilonGather /
// Scatter, :1067-1142), which couples bodies whose supports overlap.
// Entry (I, J) sums over I's supports the kernel of J at the support; a
// pair of markers further apart on an axis than their two kernel reaches
// (1.5 dilations each) has only exact-zero terms, so the entry stays +0
// without evaluating them.  With a stream the LU and the solve run on the
// device (the same arithmetic); the host-only set-up solves on the host.
int find_epsilon_set(const GridView &g, const std::vector<IbmBody *> &set, cudaStream_t *device) {
    const int D = g.dims;
    const double dh = g.dh;
    std::vector<std::pair<IbmBody *, int>> mk;  // global marker -> (body, marker)
    for (IbmBody *b : set)
        for (int m = 0; m < b->nm; ++m) mk.emplace_back(b, m);
    const int n = (int)mk.size();
    if (n == 0) return LUMA_OK;
    std::vector<double> A((size_t)n * n, 0.0);  // row-major A[I][J]
    int band = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(max : band) if (n > 256)
    for (int I = 0; I < n; ++I) {
        const IbmBody &bi = *mk[I].first;
        const int mi = mk[I].second;
        for (int J = 0; J < n; ++J) {
            const IbmBody &bj = *mk[J].first;
            const int mj = mk[J].second;
            const double reach = (1.5 * (bi.dil[mi] + bj.dil[mj]) + 1e-6) * dh;
            bool near = true;
            for (int d = 0; d < D; ++d) near = near && std::fabs(bi.pos[3 * mi + d] - bj.pos[3 * mj + d]) <= reach;
            if (!near) continue;
            double aij = 0.0;
            for (int s = bi.off[mi]; s < bi.off[mi + 1]; ++s) {
                const double dI = bi.delta[s];
                double dJ = delta_kernel((bj.pos[3 * mj + 0] - bi.sx[s]) / dh, bj.dil[mj]) *
                            delta_kernel((bj.pos[3 * mj + 1] - bi.sy[s]) / dh, bj.dil[mj]);
                if (D == 3) dJ = dJ * delta_kernel((bj.pos[3 * mj + 2] - bi.sz[s]) / dh, bj.dil[mj]);
                aij += dI * dJ * bi.area[mi];
            }
            A[(size_t)I * n + J] = aij * bj.ds[mj];
            if (A[(size_t)I * n + J] != 0.0) band = std::max(band, I > J ? I - J : J - I);
        }
    }
    std::vector<double> x(n, 1.0);
    int rc = device ? luma_eps_solve_device(n, band, A, x, *device) : LUMA_E_INVALID;
    if (rc == LUMA_E_INVALID) {   // host-only set-up, or a band too wide for the device solve
        std::fill(x.begin(), x.end(), 1.0);
        lu_solve_transposed(n, A, x);
    } else if (rc) {
        return rc;
    }
    for (int I = 0; I < n; ++I) mk[I].first->eps[mk[I].second] = x[I];
    return LUMA_OK;
}

// Supports, spacing and epsilon of rigid bodies on one grid, in the order
// ObjectManager::ibm_initialise runs them (:190-246).
int setup_bodies(const GridView &v, std::vector<IbmBody> &bodies, bool universal, cudaStream_t *device) {
    for (IbmBody &b : bodies) {
        int rc = find_support(v, b);
        if (rc) return rc;
    }
    for (IbmBody &b : bodies) compute_ds(v, b);
    if (universal) {
        std::vector<IbmBody *> all;
        for (IbmBody &b : bodies) all.push_back(&b);
        return find_epsilon_set(v, all, device);
    }
    for (IbmBody &b : bodies)
        if (int rc = find_epsilon_set(v, {&b}, device)) return rc;
    return LUMA_OK;
}

template <class T>
int dalloc_copy(T **dst, const std::vector<T> &src) {
    cudaFree(*dst);
    *dst = nullptr;
    const size_t bytes = std::max<size_t>(1, src.size()) * sizeof(T);
    if (cudaMalloc(dst, bytes) != cudaSuccess) return luma_set_error(LUMA_E_NOMEM, "IBM device allocation failed");
    if (!src.empty() && cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return luma_set_error(LUMA_E_CUDA, "IBM upload failed");
    return LUMA_OK;
}

void free_device(IbmDevice &d) {
    cudaFree(d.vel); cudaFree(d.eps); cudaFree(d.ds); cudaFree(d.area);
    cudaFree(d.F); cudaFree(d.irho); cudaFree(d.imom);
    cudaFree(d.moff); cudaFree(d.msite); cudaFree(d.smarker); cudaFree(d.mdelta);
    cudaFree(d.usite); cudaFree(d.uoff); cudaFree(d.uref);
    d = IbmDevice();
}

// Concatenate the grid's bodies and build the site-major view of the supports.
int upload_bodies(luma_gpu_grid *g) {
    IbmState &st = *g->ibm;
    std::vector<double> vel, eps, ds, area, mdelta;
    std::vector<int> moff(1, 0), msite, smarker;
    int mbase = 0;
    for (size_t bi = 0; bi < st.bodies.size(); ++bi) {
        const IbmBody &b = st.bodies[bi];
        bool flexible = false;
        for (int fbi : st.flex_body) flexible |= (fbi == (int)bi);
        if (flexible) continue;  // moving markers live in the FEM/flex arrays
        for (int m = 0; m < b.nm; ++m) {
            for (int d = 0; d < 3; ++d) vel.push_back(b.vel[3 * m + d]);
            eps.push_back(b.eps[m]);
            ds.push_back(b.ds[m]);
            area.push_back(b.area[m]);
            for (int s = b.off[m]; s < b.off[m + 1]; ++s) {
                msite.push_back(b.sk[s] + b.sj[s] * g->d.K + b.si[s] * g->d.K * g->d.M);
                mdelta.push_back(b.delta[s]);
                smarker.push_back(mbase + m);
            }
            moff.push_back((int)msite.size());
        }
        mbase += b.nm;
    }
    const int nsup = (int)msite.size();
    // distinct sites in first-appearance order, each with its supports in order
    std::vector<int> usite, uoff, uref, first(g->n, -1), count;
    for (int s = 0; s < nsup; ++s) {
        const int id = msite[s];
        if (first[id] < 0) {
            first[id] = (int)usite.size();
            usite.push_back(id);
            count.push_back(0);
        }
        count[first[id]]++;
    }
    uoff.assign(usite.size() + 1, 0);
    for (size_t u = 0; u < usite.size(); ++u) uoff[u + 1] = uoff[u] + count[u];
    uref.assign(nsup, 0);
    std::vector<int> fill(usite.size(), 0);
    for (int s = 0; s < nsup; ++s) {
        const int u = first[msite[s]];
        uref[uoff[u] + fill[u]++] = s;
    }
    IbmDevice &dv = st.dev;
    free_device(dv);
    int rc;
    if ((rc = dalloc_copy(&dv.vel, vel)) || (rc = dalloc_copy(&dv.eps, eps)) || (rc = dalloc_copy(&dv.ds, ds)) ||
        (rc = dalloc_copy(&dv.area, area)) || (rc = dalloc_copy(&dv.mdelta, mdelta)) ||
        (rc = dalloc_copy(&dv.moff, moff)) || (rc = dalloc_copy(&dv.msite, msite)) ||
        (rc = dalloc_copy(&dv.smarker, smarker)) || (rc = dalloc_copy(&dv.usite, usite)) ||
        (rc = dalloc_copy(&dv.uoff, uoff)) || (rc = dalloc_copy(&dv.uref, uref)))
        return rc;
    std::vector<double> zeros3(3 * (size_t)mbase, 0.0), zeros1(mbase, 0.0);
    if ((rc = dalloc_copy(&dv.F, zeros3)) || (rc = dalloc_copy(&dv.imom, zeros3)) || (rc = dalloc_copy(&dv.irho, zeros1)))
        return rc;
    dv.nm = mbase;
    dv.nsup = nsup;
    dv.nu = (int)usite.size();
    return LUMA_OK;
}

IbmArgs make_ibm_args(const luma_gpu_grid *g) {
    const IbmDevice &d = g->ibm->dev;
    IbmArgs b;
    b.nm = d.nm; b.nu = d.nu; b.dims = g->d.dims;
    b.moff = d.moff; b.msite = d.msite; b.smarker = d.smarker;
    b.usite = d.usite; b.uoff = d.uoff; b.uref = d.uref;
    b.mdelta = d.mdelta; b.vel = d.vel; b.eps = d.eps; b.ds = d.ds; b.area = d.area;
    b.F = d.F; b.irho = d.irho; b.imom = d.imom;
    return b;
}

int grids_on_level(const luma_gpu_grid *g, int level) {
    if (g->d.level == level) return 1;
    int n = 0;
    for (const luma_gpu_grid *c : g->kids) n += grids_on_level(c, level);
    return n;
}

int init_tree(luma_gpu_grid *g) {
    if (g->ibm && g->ibm->has_bodies) {
        IbmState &st = *g->ibm;
        const bool universal = (g->d.flags & LUMA_FLAG_UNIVERSAL_EPSILON) != 0;
        if (universal && st.has_flexible)
            return luma_set_error(LUMA_E_INVALID, "universal epsilon with flexible bodies: the reference re-solves "
                                                  "the coupled system every sub-iteration (not reproduced)");
        if (universal && grids_on_level(root_of(g), g->d.level) > 1)
            return luma_set_error(LUMA_E_INVALID, "universal epsilon couples the bodies of a level: one region "
                                                  "per level only");
        int rc = setup_bodies(view_of(g), st.bodies, universal, &g->stream);
        if (rc) return rc;
        rc = upload_bodies(g);
        if (rc) return rc;
        if (st.has_flexible) {
            if ((rc = luma_fem_upload(g))) return rc;
            if ((rc = luma_fem_supports(g, nullptr))) return rc;
            if ((rc = luma_fem_take_error(g))) return rc;
        }
        st.ready = true;
        if ((rc = luma_update_defer(g))) return rc;
    }
    for (luma_gpu_grid *c : g->kids) {
        int rc = init_tree(c);
        if (rc) return rc;
    }
    return LUMA_OK;
}

}  // namespace

int luma_ibm_reset_forces(luma_gpu_grid *g, const StepArgs &a) {
    if (!g->force) return luma_set_error(LUMA_E_STATE, "IB bodies on a grid without a force field");
    const luma_grid_desc &d = g->d;
    cudaError_t e = d.precision == LUMA_PREC_FP64
                        ? launch_reset_forces<P64>(a, d.dims, d.gravity, d.gravity_dir, d.refinement_ratio, g->stream)
                        : launch_reset_forces<P32>(a, d.dims, d.gravity, d.gravity_dir, d.refinement_ratio, g->stream);
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "reset forces: %s", cudaGetErrorString(e));
    return LUMA_OK;
}

static int ibm_pass(luma_gpu_grid *g, const StepArgs &a) {
    const IbmArgs b = make_ibm_args(g);
    FlexArgs f{};
    if (g->ibm->has_flexible) f = g->ibm->fem.flex;
    cudaError_t e = dispatch(g->d.Q, g->d.precision, [&](auto q, auto p) {
        return launch_ibm_pass<decltype(q)::value, decltype(p)>(a, b, f, g->stream);
    });
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "IBM pass: %s", cudaGetErrorString(e));
    return LUMA_OK;
}

// ObjectManager::ibm_apply(g, true) (:33-54) with ibm_moveBodies (:61-104)
// and the FSI sub-iterations (:111-185): u_n, the start-of-step velocity,
// was saved by the caller's first loop; each sub-iteration restores it,
// resets the forces, re-runs the pass and the FEM, and checks the marker
// velocity change against 1e-4 (at most 10 iterations).  All ten
// sub-iterations are enqueued; the device-side loop test makes the ones
// after convergence return at once, so the host never waits in the loop.
constexpr int kFsiMaxIterations = 10;

int luma_ibm_apply(luma_gpu_grid *g, const StepArgs &a) {
    IbmState &st = *g->ibm;
    if (!st.ready) return luma_set_error(LUMA_E_STATE, "luma_gpu_ibm_initialise was not called");
    int rc;
    const size_t ubytes = g->n * g->d.dims * (g->d.precision == LUMA_PREC_FP64 ? 8 : 4);
    if (st.has_flexible && cudaMemcpyAsync(st.u_n, g->u, ubytes, cudaMemcpyDeviceToDevice, g->stream) != cudaSuccess)
        return luma_set_error(LUMA_E_CUDA, "u_n copy failed");
    if ((rc = ibm_pass(g, a))) return rc;
    if (!st.has_flexible) return LUMA_OK;
    if ((rc = luma_fem_move_bodies(g, nullptr, true))) return rc;
    if ((rc = luma_fem_fsi_begin(g))) return rc;
    StepArgs b = a;
    b.skip = luma_fem_fsi_flag(g);
    for (int it = 0; it < kFsiMaxIterations; ++it) {
        if ((rc = luma_fem_restore_u(g))) return rc;
        if ((rc = luma_ibm_reset_forces(g, b))) return rc;
        if ((rc = ibm_pass(g, b))) return rc;
        if ((rc = luma_fem_move_bodies(g, b.skip, false))) return rc;
        if ((rc = luma_fem_fsi_check(g))) return rc;
    }
    return luma_fem_commit(g);
}

void luma_ibm_free(luma_gpu_grid *g) {
    if (g->ibm && g->ibm->has_flexible) luma_fem_free(g);
    if (g->ibm) free_device(g->ibm->dev);
    delete g->ibm;
    g->ibm = nullptr;
}

extern "C" {

int luma_ibm_setup_host(const luma_grid_desc *desc, int nbodies, const int *nmarkers, const double *positions,
                        int universal, double *eps, double *ds, int *nsupports) {
    if (!desc || nbodies <= 0 || !nmarkers || !positions || !eps || !ds)
        return luma_set_error(LUMA_E_INVALID, "luma_ibm_setup_host: null argument or no bodies");
    const luma_grid_desc &d = *desc;
    if (!((d.dims == 2 && d.K == 1) || d.dims == 3) || d.N <= 0 || d.M <= 0 || d.K <= 0 || !(d.dh > 0.0))
        return luma_set_error(LUMA_E_INVALID, "luma_ibm_setup_host: bad grid size or spacing");
    if (!d.xpos || !d.ypos || !d.zpos)
        return luma_set_error(LUMA_E_INVALID, "luma_ibm_setup_host: the grid's site positions are required");
    const GridView v{d.dims, d.N, d.M, d.K, d.level, d.dh, d.xpos, d.ypos, d.zpos, d.global_edges};
    std::vector<IbmBody> bodies(nbodies);
    size_t off = 0;
    for (int ib = 0; ib < nbodies; ++ib) {
        if (nmarkers[ib] <= 0) return luma_set_error(LUMA_E_INVALID, "luma_ibm_setup_host: body %d has no markers", ib);
        IbmBody &b = bodies[ib];
        b.nm = nmarkers[ib];
        b.pos.assign(positions + 3 * off, positions + 3 * (off + b.nm));
        b.eps.assign(b.nm, 0.0);
        b.ds.assign(b.nm, 1.0);
        b.dil.assign(b.nm, 1.0);
        b.area.assign(b.nm, 1.0);
        off += b.nm;
    }
    if (int rc = setup_bodies(v, bodies, universal != 0, nullptr)) return rc;
    off = 0;
    for (const IbmBody &b : bodies) {
        for (int m = 0; m < b.nm; ++m) {
            eps[off + m] = b.eps[m];
            ds[off + m] = b.ds[m];
            if (nsupports) nsupports[off + m] = b.off[m + 1] - b.off[m];
        }
        off += b.nm;
    }
    return LUMA_OK;
}

int luma_gpu_ibm_add_body(luma_gpu_grid *g, int nmarkers, const double *positions, const double *velocities,
                          int *body_index) {
    if (!g || !positions || nmarkers <= 0) return luma_set_error(LUMA_E_INVALID, "bad IB body arguments");
    if (!(g->d.flags & LUMA_FLAG_IBM))
        return luma_set_error(LUMA_E_INVALID, "IB bodies need a grid created with LUMA_FLAG_IBM");
    if (g->hx.empty() || g->hy.empty() || g->hz.empty())
        return luma_set_error(LUMA_E_INVALID, "IB bodies need the grid's site positions");
    if (!g->ibm) g->ibm = new IbmState();
    static std::atomic<long long> next_seq{0};
    IbmBody b;
    b.nm = nmarkers;
    b.seq = next_seq++;
    b.pos.assign(positions, positions + 3 * (size_t)nmarkers);
    if (velocities) b.vel.assign(velocities, velocities + 3 * (size_t)nmarkers);
    else b.vel.assign(3 * (size_t)nmarkers, 0.0);
    b.eps.assign(nmarkers, 0.0);
    b.ds.assign(nmarkers, 1.0);
    b.dil.assign(nmarkers, 1.0);
    b.area.assign(nmarkers, 1.0);
    g->ibm->bodies.push_back(b);
    g->ibm->has_bodies = true;
    g->ibm->ready = false;
    if (body_index) *body_index = (int)g->ibm->bodies.size() - 1;
    return LUMA_OK;
}

int luma_gpu_ibm_initialise(luma_gpu_grid *root) {
    if (!root) return luma_set_error(LUMA_E_INVALID, "null grid");
    return init_tree(root);
}

int luma_gpu_ibm_get_markers(luma_gpu_grid *g, int body, double *out) {
    if (!g || !out) return luma_set_error(LUMA_E_INVALID, "null argument");
    if (!g->ibm || body < 0 || body >= (int)g->ibm->bodies.size())
        return luma_set_error(LUMA_E_INVALID, "no IB body %d on this grid", body);
    const IbmState &st = *g->ibm;
    int base = 0;
    for (int b = 0; b < body; ++b) base += st.bodies[b].nm;
    const IbmBody &bd = st.bodies[body];
    int flex_index = -1, flex_base = 0, rigid_base = 0;
    for (size_t k = 0; k < st.flex_body.size(); ++k)
        if (st.flex_body[k] == body) flex_index = (int)k;
    for (int b = 0; b < body; ++b) {
        bool fl = false;
        for (int fbi : st.flex_body) fl |= (fbi == b);
        if (!fl) rigid_base += st.bodies[b].nm;
    }
    for (int k = 0; k < flex_index; ++k) flex_base += st.flex[k].nm;
    (void)base;
    std::vector<double> F(3 * (size_t)bd.nm, 0.0);
    if (flex_index >= 0 && st.ready) {
        const FlexArgs &x = st.fem.flex;
        std::vector<double> pos(3 * (size_t)bd.nm), eps(bd.nm), ds(bd.nm);
        std::vector<int> ns(bd.nm);
        cudaStreamSynchronize(g->stream);
        if (cudaMemcpy(F.data(), x.F + 3 * (size_t)flex_base, F.size() * 8, cudaMemcpyDeviceToHost) ||
            cudaMemcpy(pos.data(), x.pos + 3 * (size_t)flex_base, pos.size() * 8, cudaMemcpyDeviceToHost) ||
            cudaMemcpy(eps.data(), x.eps + flex_base, eps.size() * 8, cudaMemcpyDeviceToHost) ||
            cudaMemcpy(ds.data(), x.ds + flex_base, ds.size() * 8, cudaMemcpyDeviceToHost) ||
            cudaMemcpy(ns.data(), x.nsupp + flex_base, ns.size() * 4, cudaMemcpyDeviceToHost))
            return luma_set_error(LUMA_E_CUDA, "filament marker download failed");
        for (int m = 0; m < bd.nm; ++m) {
            double *o = out + 9 * (size_t)m;
            o[0] = pos[3 * m]; o[1] = pos[3 * m + 1]; o[2] = pos[3 * m + 2];
            o[3] = F[3 * m]; o[4] = F[3 * m + 1]; o[5] = g->d.dims == 3 ? F[3 * m + 2] : 0.0;
            o[6] = eps[m]; o[7] = ds[m]; o[8] = ns[m];
        }
        return LUMA_OK;
    }
    if (st.ready && cudaMemcpy(F.data(), st.dev.F + 3 * (size_t)rigid_base, F.size() * sizeof(double),
                               cudaMemcpyDeviceToHost) != cudaSuccess)
        return luma_set_error(LUMA_E_CUDA, "marker force download failed");
    for (int m = 0; m < bd.nm; ++m) {
        double *o = out + 9 * (size_t)m;
        o[0] = bd.pos[3 * m]; o[1] = bd.pos[3 * m + 1]; o[2] = bd.pos[3 * m + 2];
        o[3] = F[3 * m]; o[4] = F[3 * m + 1]; o[5] = g->d.dims == 3 ? F[3 * m + 2] : 0.0;
        o[6] = bd.eps[m]; o[7] = bd.ds[m];
        o[8] = bd.off.empty() ? 0.0 : double(bd.off[m + 1] - bd.off[m]);
    }
    return LUMA_OK;
}

int luma_gpu_ibm_body_force(luma_gpu_grid *g, int body, double force[3]) {
    if (!g || !force) return luma_set_error(LUMA_E_INVALID, "null argument");
    if (!g->ibm || body < 0 || body >= (int)g->ibm->bodies.size())
        return luma_set_error(LUMA_E_INVALID, "no IB body %d on this grid", body);
    const IbmBody &bd = g->ibm->bodies[body];
    std::vector<double> m(9 * (size_t)bd.nm);
    int rc = luma_gpu_ibm_get_markers(g, body, m.data());
    if (rc) return rc;
    force[0] = force[1] = force[2] = 0.0;
    for (int k = 0; k < bd.nm; ++k) {
        const double *o = &m[9 * (size_t)k];
        const double volDepth = g->d.dims == 3 ? o[7] : 1.0;
        for (int d = 0; d < g->d.dims; ++d) force[d] += o[3 + d] * o[6] * volDepth * o[7];
    }
    return LUMA_OK;
}

}  // extern "C"
