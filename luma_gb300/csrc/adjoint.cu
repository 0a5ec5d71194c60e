// Discrete adjoint of the time-averaged drag of an immersed body.
//
// J = (1/T) sum_t sum_{m in body} F_m,x(t) * eps_m * ds_m (* ds_m in 3D):
// the body's marker forces integrated as ObjectManager::io_writeLiftDrag
// integrates them (LUMA src/ObjectManager_ops_io.cpp:105-121, before its
// physical scaling), averaged over the T steps of the forward run.  The
// gradient is taken with respect to the scale s of the inlet velocity
// (u = s * u_in at every velocity site) and the body's marker positions X.
//
// Forward (luma_gpu_adj_forward): T ordinary device steps, with the
// population state saved every K steps and J accumulated in FP64.
// Backward (luma_gpu_adj_backward): for each K-step segment, last first,
// restore its checkpoint, re-run the segment once while taping the
// post-stream populations and the marker forces of each step (one segment
// of K states resident; the force field is rebuilt from the marker forces),
// then apply the reverse of each step, newest first.  Full segments run as
// CUDA graphs captured once.  One step of the forward is
//   stream   g = S f          periodic pull, half-way bounce-back,
//                             extrapolate-right, forced-equilibrium inlet
//                             feq(rho_v, s u_v)
//   IBM      F_m = 2 A_m sum_s delta_ms (j_s - rho_s V_m)
//            F(s) = -sum_m delta_ms w_m F_m,  w_m = eps_m ds_m (* ds_m in 3D)
//   collide  f' = (1-omega) g + omega feq(rho, u) + Guo(u, F),
//            rho = sum g, u = (j + F/2)/rho
// (the 3D half-force quirk of the reference's macroscopic step, F_z/2
// added to x, is followed unless LUMA_FLAG_FIX_MACRO3D).  The support sets
// are the forward's: the Roma kernel and its derivative vanish on the edge
// of the support cage, so J is C1 across support changes.  Epsilon (the
// dense system A eps = 1) and ds (minimum marker distance) depend on X; that
// part of the chain rule runs on the host in FP64 from the per-marker and
// per-support sensitivities the device accumulates.
//
// Scope: one grid (no refinement), BGK, rigid IB bodies; site types fluid,
// solid, velocity and extrapolate-right; no regularised BCs, gravity or
// velocity ramp.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "dispatch.hpp"
#include "grid.hpp"
#include "kernels.hpp"

using namespace luma;

namespace luma {

struct AdjState {
    int body = -1, T = 0, K = 0, nseg = 0;
    int mode = 0;           // 0 idle, 1 accumulate J, 2 tape
    bool valid = false;     // a forward is recorded and not yet reversed
    int t0 = 0;
    int body_base = 0, body_nm = 0, body_sup = 0;  // body's first marker / support in the rigid arrays
    double *d_J = nullptr, *d_gs = nullptr;
    std::vector<void *> ckpt;
    void *fin_f[2] = {nullptr, nullptr};
    void *fin_u = nullptr, *fin_rho = nullptr;
    int fin_cur = 0, fin_t = 0;
    void *tape_g = nullptr;
    double *tape_Fm = nullptr;
    void *tape_Fs = nullptr;  // per step: the spread force at the distinct support sites (R)
    double *drag_terms = nullptr;  // per step of a forward segment: the body's F_x w per marker
    int tape_pos = 0;
    int *site_u = nullptr;  // per site: index of the distinct support site, or -1
    void *lam = nullptr;                       // adjoint of f at segment boundaries
    void *lamg[2] = {nullptr, nullptr};       // adjoint of the post-stream f, steps t and t-1
    void *lamF = nullptr;
    double *mu = nullptr, *Gw = nullptr, *Gd = nullptr, *w = nullptr;
    size_t bytes = 0;
    // full K-step segments run as CUDA graphs captured once (K even)
    cudaStream_t own = nullptr;
    cudaGraphExec_t seg_fwd = nullptr, seg_bwd = nullptr;
    // the reverse IBM pass runs on `side`, beside the reverse stream of the
    // sites whose gathers touch no support site (`near` marks the others,
    // listed in near_ids, which follow once both are done)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    uint8_t *near = nullptr;
    int *near_ids = nullptr;
    int nnear = 0;
    // kept for the next forward of the same length, segments and body while
    // the grid's launch signature and its support sites stay the same: the
    // buffers and the captured segment graphs are reused
    std::vector<uintptr_t> sig;
    std::vector<int> usite_host;
    bool graphs = true;
};

}  // namespace luma

namespace {

struct AdjArgs {
    int N, M, K, ncell, nm, nu, nsup, body_base, body_nm;
    int quirk;                 // 3D: F_z/2 enters u_x
    double omega, rho0, invT;
    const uint8_t *typ;
    const int *site_u;         // per site: distinct support index or -1
    const uint8_t *near;       // per site: its reverse stream reads a support site
    const int *near_ids;       // the marked sites
    int nnear;
    const void *g;             // taped post-stream populations (S)
    const double *Fm;          // taped marker forces (3 per marker)
    const void *Fs;            // taped force at the distinct support sites (R, D x nu)
    const void *lam_in;        // adjoint of the post-collision f (R)
    void *lam_out;             // adjoint of the pre-stream f (R)
    void *lamg, *lamF;         // R scratch
    const void *rho_field, *u_field;  // constant rho/u of non-fluid sites (R)
    // rigid IB arrays of the grid
    const int *moff, *msite, *smarker, *usite, *uoff, *uref;
    const double *mdelta, *vel, *area, *w;
    double *mu, *Gw, *Gd, *gs;
};

// The taped populations of site id and the step's force there: zero after
// the reset, the spread marker forces (taped) at support sites.
template <int Q, class P>
__device__ __forceinline__ void adj_collide_load(const AdjArgs &a, int id, typename P::R *gv, typename P::R *F) {
    using R = typename P::R;
    const size_t n = (size_t)a.ncell;
#pragma unroll
    for (int v = 0; v < Q; ++v) gv[v] = ld<P>(a.g, (size_t)v * n + id);
    F[0] = F[1] = F[2] = R(0);
    const int su = a.site_u[id];
    if (su >= 0)
        for (int d = 0; d < Lattice<Q>::D; ++d) F[d] = static_cast<const R *>(a.Fs)[(size_t)d * a.nu + su];
}

// Reverse of macroscopic + forcing + collision at fluid site id, given the
// adjoint lam' of the collided populations, the taped populations gv and
// the force F (registers): writes lam_g = d(lam'.f')/dg and
// lam_F = d(lam'.f')/dF of the site.
template <int Q, class P>
__device__ __forceinline__ void adj_collide_at(const AdjArgs &a, int id, const typename P::R *lam,
                                               const typename P::R *gv, const typename P::R *F, typename P::R *lg,
                                               typename P::R *lF) {
    using L = Lattice<Q>;
    using R = typename P::R;
    constexpr int D = L::D;
    const size_t n = (size_t)a.ncell;
    R rho = R(0), j[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        rho += gv[v];
        for (int d = 0; d < D; ++d) j[d] += R(L::c(v, d)) * gv[v];
    }
    if (P::shifted) rho += R(a.rho0);
    R u[3] = {R(0), R(0), R(0)};
    u[0] = (j[0] + R(0.5) * F[0] + (a.quirk ? R(0.5) * F[2] : R(0))) / rho;
    u[1] = (j[1] + R(0.5) * F[1]) / rho;
    if (D == 3) u[2] = (j[2] + (a.quirk ? R(0) : R(0.5) * F[2])) / rho;
    const R om = R(a.omega), g3 = R(3) * (R(1) - R(0.5) * om);
    const R usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    R arho = R(0), au[3] = {R(0), R(0), R(0)}, aF[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        const R w = R(L::w(v));
        R cu = R(0), Fc = R(0);
        for (int d = 0; d < D; ++d) {
            cu += R(L::c(v, d)) * u[d];
            Fc += R(L::c(v, d)) * F[d];
        }
        const R lv = lam[v];
        arho += lv * om * w * (R(1) + R(3) * cu + R(4.5) * cu * cu - R(1.5) * usq);
        for (int d = 0; d < D; ++d) {
            const R c = R(L::c(v, d));
            au[d] += lv * w * (om * rho * (R(3) * c + R(9) * cu * c - R(3) * u[d]) + g3 * (R(3) * Fc * c - F[d]));
            aF[d] += lv * g3 * w * (c * (R(1) + R(3) * cu) - u[d]);
        }
    }
    R aus = R(0);
    for (int d = 0; d < D; ++d) aus += au[d] * u[d];
    const R lrho = arho - aus / rho;
    R lj[3] = {R(0), R(0), R(0)};
    for (int d = 0; d < D; ++d) lj[d] = au[d] / rho;
    const R h = R(0.5) / rho;
    lF[id] = aF[0] + au[0] * h;
    lF[n + id] = aF[1] + au[1] * h;
    if (D == 3) lF[2 * n + id] = aF[2] + (a.quirk ? au[0] : au[2]) * h;
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        R s = (R(1) - om) * lam[v] + lrho;
        for (int d = 0; d < D; ++d) s += R(L::c(v, d)) * lj[d];
        lg[(size_t)v * n + id] = s;
    }
}

// Collided values of sites other than fluid ones never reach a fluid site.
template <int Q, class P>
__device__ __forceinline__ void adj_collide_zero(const AdjArgs &a, int id, typename P::R *lg, typename P::R *lF) {
    using R = typename P::R;
    const size_t n = (size_t)a.ncell;
    for (int v = 0; v < Q; ++v) lg[(size_t)v * n + id] = R(0);
    for (int d = 0; d < Lattice<Q>::D; ++d) lF[(size_t)d * n + id] = R(0);
}

// The reverse collision of a step from the adjoint in memory (lam_in).
template <int Q, class P>
__global__ void __launch_bounds__(128) k_adj_collide(AdjArgs a) {
    using R = typename P::R;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= a.ncell) return;
    R *lg = static_cast<R *>(a.lamg);
    R *lF = static_cast<R *>(a.lamF);
    if (a.typ[id] != LUMA_SITE_FLUID) {
        adj_collide_zero<Q, P>(a, id, lg, lF);
        return;
    }
    const size_t n = (size_t)a.ncell;
    const R *lin = static_cast<const R *>(a.lam_in);
    R lam[Q], gv[Q], F[3];
#pragma unroll
    for (int v = 0; v < Q; ++v) lam[v] = lin[(size_t)v * n + id];
    adj_collide_load<Q, P>(a, id, gv, F);
    adj_collide_at<Q, P>(a, id, lam, gv, F, lg, lF);
}

// Density and momentum at a support site as the IBM interpolation saw them:
// from the taped populations at fluid sites, from the (constant) fields
// elsewhere.
template <int Q, class P>
__device__ __forceinline__ void support_moments(const AdjArgs &a, int id, double &rho, double j[3]) {
    constexpr int D = Lattice<Q>::D;
    const size_t n = (size_t)a.ncell;
    j[0] = j[1] = j[2] = 0.0;
    if (a.typ[id] == LUMA_SITE_FLUID) {
        double r = 0.0;
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            const double gv = double(ld<P>(a.g, (size_t)v * n + id));
            r += gv;
            for (int d = 0; d < D; ++d) j[d] += Lattice<Q>::c(v, d) * gv;
        }
        rho = P::shifted ? r + a.rho0 : r;
    } else {
        using R = typename P::R;
        rho = double(static_cast<const R *>(a.rho_field)[id]);
        for (int d = 0; d < D; ++d) j[d] = rho * double(static_cast<const R *>(a.u_field)[(size_t)d * n + id]);
    }
}

// Reverse of the marker force and the spread for marker m:
// mu_m = dJ/dF_m, and the sensitivities to the spreading weight w_m and to
// each support's delta value.
template <int Q, class P>
__device__ __forceinline__ void adj_marker(const AdjArgs &a, int m) {
    using R = typename P::R;
    constexpr int D = Lattice<Q>::D;
    const size_t n = (size_t)a.ncell;
    const R *lF = static_cast<const R *>(a.lamF);
    const bool inbody = m >= a.body_base && m < a.body_base + a.body_nm;
    double sl[3] = {0, 0, 0};
    for (int s = a.moff[m]; s < a.moff[m + 1]; ++s)
        for (int d = 0; d < D; ++d) sl[d] += a.mdelta[s] * double(lF[(size_t)d * n + a.msite[s]]);
    const double wm = a.w[m];
    const double *Fm = a.Fm + 3 * m;
    double mu[3] = {0, 0, 0}, gw = 0.0;
    for (int d = 0; d < D; ++d) {
        mu[d] = -wm * sl[d];
        gw -= Fm[d] * sl[d];
    }
    if (inbody) {
        mu[0] += a.invT * wm;
        gw += a.invT * Fm[0];
    }
    a.Gw[m] += gw;
    for (int d = 0; d < 3; ++d) a.mu[3 * m + d] = mu[d];
    const double A2 = 2.0 * a.area[m];
    double Vmu = 0.0;
    for (int d = 0; d < D; ++d) Vmu += a.vel[3 * m + d] * mu[d];
    for (int s = a.moff[m]; s < a.moff[m + 1]; ++s) {
        const int id = a.msite[s];
        double rho, j[3];
        support_moments<Q, P>(a, id, rho, j);
        double t = -A2 * rho * Vmu;
        for (int d = 0; d < D; ++d) t += A2 * mu[d] * j[d] - wm * Fm[d] * double(lF[(size_t)d * n + id]);
        a.Gd[s] += t;
    }
}

// Adjoint of the interpolated density and momentum at distinct support
// site u, gathered in the forward's order and added to lam_g through
// rho = sum_v g_v and j = sum_v c_v g_v.
template <int Q, class P>
__device__ __forceinline__ void adj_support(const AdjArgs &a, int u) {
    using R = typename P::R;
    constexpr int D = Lattice<Q>::D;
    const size_t n = (size_t)a.ncell;
    const int id = a.usite[u];
    if (a.typ[id] != LUMA_SITE_FLUID) return;  // moments of other sites are constants
    double lj[3] = {0, 0, 0}, lr = 0.0;
    for (int q = a.uoff[u]; q < a.uoff[u + 1]; ++q) {
        const int s = a.uref[q];
        const int m = a.smarker[s];
        const double c = 2.0 * a.area[m] * a.mdelta[s];
        for (int d = 0; d < D; ++d) {
            lj[d] += c * a.mu[3 * m + d];
            lr -= c * a.vel[3 * m + d] * a.mu[3 * m + d];
        }
    }
    R *lg = static_cast<R *>(a.lamg);
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        double c = lr;
        for (int d = 0; d < D; ++d) c += Lattice<Q>::c(v, d) * lj[d];
        lg[(size_t)v * n + id] += R(c);
    }
}

template <int Q, class P>
__global__ void k_adj_marker(AdjArgs a) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < a.nm) adj_marker<Q, P>(a, m);
}

template <int Q, class P>
__global__ void k_adj_support(AdjArgs a) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u < a.nu) adj_support<Q, P>(a, u);
}

// Density and momentum at a support site in the policy's arithmetic (the
// FP32 path sums its shifted populations in FP32).
template <int Q, class P>
__device__ __forceinline__ void support_moments_r(const AdjArgs &a, int id, double &rho, double j[3]) {
    using R = typename P::R;
    constexpr int D = Lattice<Q>::D;
    const size_t n = (size_t)a.ncell;
    j[0] = j[1] = j[2] = 0.0;
    if (a.typ[id] == LUMA_SITE_FLUID) {
        R r = R(0), jr[3] = {R(0), R(0), R(0)};
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            const R gv = ld<P>(a.g, (size_t)v * n + id);
            r += gv;
            for (int d = 0; d < D; ++d) jr[d] += R(Lattice<Q>::c(v, d)) * gv;
        }
        rho = P::shifted ? double(r) + a.rho0 : double(r);
        for (int d = 0; d < D; ++d) j[d] = double(jr[d]);
    } else {
        rho = double(static_cast<const R *>(a.rho_field)[id]);
        for (int d = 0; d < D; ++d) j[d] = rho * double(static_cast<const R *>(a.u_field)[(size_t)d * n + id]);
    }
}

// Both IBM reverse passes in one block, for bodies small enough that one
// block covers them.  Everything the passes read is staged in shared memory
// first, in one round of independent loads (the per-support lam_F, moments
// and weights, the per-marker data, the support-site lists and the adjoint
// at the support sites); then, separated by block barriers: the per-marker
// sums in support order (as adj_marker), the per-support delta
// sensitivities, and the per-site gathers in the forward's order (as
// adj_support), which write the updated adjoint back.
constexpr int kIbmBlock = 512;
constexpr size_t kIbmBlockMaxSmem = 160 * 1024;

size_t ibm_block_smem(int nsup, int nm, int nu, int Q, size_t rs) {
    const size_t dbl = (size_t)nsup * 8 + (size_t)nm * 11;
    const size_t ints = (size_t)nu + (nu + 1) + 2 * (size_t)nsup + (nm + 1);
    return dbl * 8 + (size_t)nu * Q * rs + ints * 4;
}

template <int Q, class P>
__global__ void __launch_bounds__(kIbmBlock) k_adj_ibm_block(AdjArgs a) {
    using R = typename P::R;
    constexpr int D = Lattice<Q>::D;
    extern __shared__ double sm[];
    const int ns = a.nsup, nm = a.nm, nu = a.nu;
    double *dlf = sm;               // 3 per support: delta * lam_F at its site
    double *qs = dlf + 3 * ns;      // 3 per support: 2 area (j - rho V) at its site
    double *c0 = qs + 3 * ns;       // per support: G_delta so far - w F . lam_F
    double *cs = c0 + ns;           // per support: 2 area delta
    double *mu = cs + ns;           // 3 per marker: dJ/dF
    double *mk = mu + 3 * nm;       // 8 per marker: V, w, F, G_w so far
    R *lgo = reinterpret_cast<R *>(mk + 8 * nm);                 // Q per support site: lam_g before the pass
    int *usid = reinterpret_cast<int *>(lgo + (size_t)Q * nu);  // support site, -1 unless fluid
    int *uoff = usid + nu;
    int *uref = uoff + nu + 1;
    int *ms = uref + ns;            // marker of each support
    int *moff = ms + ns;
    const size_t n = (size_t)a.ncell;
    const R *lF = static_cast<const R *>(a.lamF);
    R *lg = static_cast<R *>(a.lamg);
    for (int s = threadIdx.x; s < ns; s += blockDim.x) {
        const int id = a.msite[s], m = a.smarker[s];
        const double dl = a.mdelta[s], wm = a.w[m], A2 = 2.0 * a.area[m];
        double rho, j[3];
        support_moments_r<Q, P>(a, id, rho, j);
        double c = a.Gd[s];
        for (int d = 0; d < 3; ++d) {
            const double l = d < D ? double(lF[(size_t)d * n + id]) : 0.0;
            dlf[3 * s + d] = dl * l;
            qs[3 * s + d] = d < D ? A2 * (j[d] - rho * a.vel[3 * m + d]) : 0.0;
            if (d < D) c -= wm * a.Fm[3 * m + d] * l;
        }
        c0[s] = c;
        cs[s] = A2 * dl;
        ms[s] = m;
        uref[s] = a.uref[s];
    }
    for (int m = threadIdx.x; m <= nm; m += blockDim.x) {
        moff[m] = a.moff[m];
        if (m == nm) continue;
        for (int d = 0; d < 3; ++d) {
            mk[8 * m + d] = a.vel[3 * m + d];
            mk[8 * m + 4 + d] = a.Fm[3 * m + d];
        }
        mk[8 * m + 3] = a.w[m];
        mk[8 * m + 7] = a.Gw[m];
    }
    for (int u = threadIdx.x; u <= nu; u += blockDim.x) {
        uoff[u] = a.uoff[u];
        if (u == nu) continue;
        const int id = a.usite[u];
        const bool fluid = a.typ[id] == LUMA_SITE_FLUID;
        usid[u] = fluid ? id : -1;
        if (fluid)
#pragma unroll
            for (int v = 0; v < Q; ++v) lgo[(size_t)v * nu + u] = lg[(size_t)v * n + id];
    }
    __syncthreads();
    for (int m = threadIdx.x; m < nm; m += blockDim.x) {
        const bool inbody = m >= a.body_base && m < a.body_base + a.body_nm;
        double sl[3] = {0, 0, 0};
        for (int s = moff[m]; s < moff[m + 1]; ++s)
            for (int d = 0; d < D; ++d) sl[d] += dlf[3 * s + d];
        const double wm = mk[8 * m + 3];
        const double *Fm = mk + 8 * m + 4;
        double mv[3] = {0, 0, 0}, gw = 0.0;
        for (int d = 0; d < D; ++d) {
            mv[d] = -wm * sl[d];
            gw -= Fm[d] * sl[d];
        }
        if (inbody) {
            mv[0] += a.invT * wm;
            gw += a.invT * Fm[0];
        }
        a.Gw[m] = mk[8 * m + 7] + gw;
        for (int d = 0; d < 3; ++d) mu[3 * m + d] = mv[d];
    }
    __syncthreads();
    for (int s = threadIdx.x; s < ns; s += blockDim.x) {
        const int m = ms[s];
        double t = c0[s];
        for (int d = 0; d < D; ++d) t += mu[3 * m + d] * qs[3 * s + d];
        a.Gd[s] = t;
    }
    for (int u = threadIdx.x; u < nu; u += blockDim.x) {
        const int id = usid[u];
        if (id < 0) continue;  // moments of other sites are constants
        double lj[3] = {0, 0, 0}, lr = 0.0;
        for (int q = uoff[u]; q < uoff[u + 1]; ++q) {
            const int s = uref[q];
            const int m = ms[s];
            const double c = cs[s];
            for (int d = 0; d < D; ++d) {
                lj[d] += c * mu[3 * m + d];
                lr -= c * mk[8 * m + d] * mu[3 * m + d];
            }
        }
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            double c = lr;
            for (int d = 0; d < D; ++d) c += Lattice<Q>::c(v, d) * lj[d];
            lg[(size_t)v * n + id] = lgo[(size_t)v * nu + u] + R(c);
        }
    }
}

__device__ __forceinline__ bool pulls(int t) {
    return t == LUMA_SITE_FLUID || t == LUMA_SITE_EXTRAPOLATE_RIGHT;
}

// Reverse of the stream (the transpose of the pull, gathered per source
// site) and the inlet-scale sensitivity of the forced-equilibrium inflow.
// FUSE: the adjoint of the pre-stream populations of step t stays in
// registers and feeds the reverse collision of step t-1 at the same site
// (arguments b); otherwise it goes to a.lam_out.
// SEL: 0 every site, 1 the sites not marked near, 2 the near list.
template <int Q, class P, bool FUSE, int SEL>
__global__ void __launch_bounds__(256) k_adj_stream(AdjArgs a, AdjArgs b) {
    using L = Lattice<Q>;
    using R = typename P::R;
    constexpr int D = L::D;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    int id = x;
    if (SEL == 1 && id < a.ncell && a.near[id]) id = -1;
    if (SEL == 2) id = x < a.nnear ? a.near_ids[x] : -1;
    const size_t n = (size_t)a.ncell;
    double gs_local = 0.0;
    if (id >= 0 && id < a.ncell) {
        const int K = a.K, M = a.M, N = a.N;
        const int k = id % K, j = (id / K) % M, i = id / (K * M);
        const R *lg = static_cast<const R *>(a.lamg);
        R *out = static_cast<R *>(a.lam_out);
        auto wrapid = [&](int x, int y, int z) {
            x = x < 0 ? x + N : (x >= N ? x - N : x);
            y = y < 0 ? y + M : (y >= M ? y - M : y);
            if (D == 3) z = z < 0 ? z + K : (z >= K ? z - K : z);
            else z = 0;
            return z + y * K + x * K * M;
        };
        const int yt = a.typ[id];
        // the reverse collision's inputs, loaded before the gathers
        R gv[Q], F[3];
        if (FUSE && yt == LUMA_SITE_FLUID) adj_collide_load<Q, P>(b, id, gv, F);
        const bool regular_source = yt == LUMA_SITE_FLUID;  // solid, velocity, extrapolate sources are replaced
        const bool extrap_source = i + 2 < N && a.typ[wrapid(i + 2, j, k)] == LUMA_SITE_EXTRAPOLATE_RIGHT;
        R lam[Q];
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            const int cx = L::c(v, 0), cy = L::c(v, 1), cz = L::c(v, 2);
            R s = R(0);
            // x = y + c_v pulls f_v(y)
            const int xid = wrapid(i + cx, j + cy, k + cz);
            if (regular_source && pulls(a.typ[xid])) s += lg[(size_t)v * n + xid];
            // bounce-back at y: g_opp(v)(y) = f_v(y) when y + c_v is solid
            if (pulls(yt) && a.typ[xid] == LUMA_SITE_SOLID) s += lg[(size_t)L::opp(v) * n + id];
            // extrapolate-right: x pulls f_v(e - 2 e_x) from the outlet site e = y + 2 e_x
            if (extrap_source) {
                const int x2 = wrapid(i + 2 + cx, j + cy, k + cz);
                if (pulls(a.typ[x2])) s += lg[(size_t)v * n + x2];
            }
            if (FUSE) lam[v] = s;
            else out[(size_t)v * n + id] = s;
            // inflow: y pulls feq_v(rho_e, s u_e) from the velocity site e = y - c_v
            if (yt == LUMA_SITE_FLUID) {
                const int sid = wrapid(i - cx, j - cy, k - cz);
                if (a.typ[sid] == LUMA_SITE_VELOCITY) {
                    const R *rf = static_cast<const R *>(a.rho_field);
                    const R *uf = static_cast<const R *>(a.u_field);
                    const double rs = double(rf[sid]);
                    double cu = 0.0, usq = 0.0;
                    for (int d = 0; d < D; ++d) {
                        const double ud = double(uf[(size_t)d * n + sid]);
                        cu += L::c(v, d) * ud;
                        usq += ud * ud;
                    }
                    const double dfeq = rs * L::w(v) * (3.0 * cu + 9.0 * cu * cu - 3.0 * usq);  // d/ds at s = 1
                    gs_local += double(lg[(size_t)v * n + id]) * dfeq;
                }
            }
        }
        if (FUSE) {
            R *lgb = static_cast<R *>(b.lamg);
            R *lFb = static_cast<R *>(b.lamF);
            if (yt == LUMA_SITE_FLUID) adj_collide_at<Q, P>(b, id, lam, gv, F, lgb, lFb);
            else adj_collide_zero<Q, P>(b, id, lgb, lFb);
        }
    }
    __shared__ double red[8];
    for (int o = 16; o > 0; o >>= 1) gs_local += __shfl_xor_sync(0xffffffffu, gs_local, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = gs_local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        if (t != 0.0) atomicAdd(a.gs, t);
    }
}

// J over one forward segment: per step the body's drag terms (recorded by
// the IBM interpolation), reduced in a fixed order by one block, scaled by
// 1/T and added to J step after step.
__global__ void k_drag_segment(const double *terms, int steps, int nm, double invT, double *J) {
    __shared__ double sh[256];
    // J gains one term per step, in step order, whatever the segmentation
    double acc = *J;
    for (int t = 0; t < steps; ++t) {
        double s = 0.0;
        for (int m = threadIdx.x; m < nm; m += blockDim.x) s += terms[(size_t)t * nm + m];
        sh[threadIdx.x] = s;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) acc += sh[0] * invT;
        __syncthreads();
    }
    if (threadIdx.x == 0) *J = acc;
}

template <class T>
int dmalloc(T **p, size_t bytes, AdjState &st) {
    if (cudaMalloc((void **)p, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return luma_set_error(LUMA_E_NOMEM, "adjoint: device allocation of %zu bytes failed", bytes);
    }
    st.bytes += bytes;
    return LUMA_OK;
}

size_t rsize(const luma_gpu_grid *g) { return g->d.precision == LUMA_PREC_FP64 ? 8 : 4; }

void free_state(AdjState *st) {
    if (!st) return;
    for (void *p : st->ckpt) cudaFree(p);
    cudaFree(st->fin_f[0]); cudaFree(st->fin_f[1]); cudaFree(st->fin_u); cudaFree(st->fin_rho);
    cudaFree(st->tape_g); cudaFree(st->tape_Fm); cudaFree(st->tape_Fs); cudaFree(st->site_u); cudaFree(st->drag_terms);
    if (st->seg_fwd) cudaGraphExecDestroy(st->seg_fwd);
    if (st->seg_bwd) cudaGraphExecDestroy(st->seg_bwd);
    if (st->own) cudaStreamDestroy(st->own);
    if (st->side) cudaStreamDestroy(st->side);
    if (st->ev_fork) cudaEventDestroy(st->ev_fork);
    if (st->ev_join) cudaEventDestroy(st->ev_join);
    cudaFree(st->near); cudaFree(st->near_ids);
    cudaFree(st->lam); cudaFree(st->lamg[0]); cudaFree(st->lamg[1]); cudaFree(st->lamF); cudaFree(st->mu);
    cudaFree(st->Gw); cudaFree(st->Gd); cudaFree(st->w); cudaFree(st->d_J); cudaFree(st->d_gs);
    delete st;
}

int check_scope(const luma_gpu_grid *g, int body) {
    const luma_grid_desc &d = g->d;
    if (g->parent || !g->kids.empty()) return luma_set_error(LUMA_E_INVALID, "adjoint: single-grid hierarchies only");
    if (!(d.flags & LUMA_FLAG_IBM) || !g->ibm || !g->ibm->ready || !g->ibm->has_bodies)
        return luma_set_error(LUMA_E_STATE, "adjoint: needs IB bodies, initialised (luma_gpu_ibm_initialise)");
    if (g->ibm->has_flexible) return luma_set_error(LUMA_E_INVALID, "adjoint: rigid bodies only");
    if (d.collision != LUMA_COLL_BGK) return luma_set_error(LUMA_E_INVALID, "adjoint: BGK collision only");
    if (d.flags & (LUMA_FLAG_REGULARISED | LUMA_FLAG_GRAVITY))
        return luma_set_error(LUMA_E_INVALID, "adjoint: no regularised BCs or gravity");
    if (d.velocity_ramp > 0.0 || d.reynolds_ramp > 0.0)
        return luma_set_error(LUMA_E_INVALID, "adjoint: no velocity or Reynolds ramp");
    if (d.flags & LUMA_FLAG_TIME_AVERAGES) return luma_set_error(LUMA_E_INVALID, "adjoint: no time averages");
    if (body < 0 || body >= (int)g->ibm->bodies.size()) return luma_set_error(LUMA_E_INVALID, "adjoint: bad body %d", body);
    std::vector<uint8_t> typ(g->n);
    if (cudaMemcpy(typ.data(), g->typ, g->n, cudaMemcpyDeviceToHost) != cudaSuccess)
        return luma_set_error(LUMA_E_CUDA, "adjoint: site labels");
    for (size_t i = 0; i < g->n; ++i) {
        const int t = typ[i];
        if (!(t == LUMA_SITE_FLUID || t == LUMA_SITE_SOLID || t == LUMA_SITE_VELOCITY || t == LUMA_SITE_EXTRAPOLATE_RIGHT))
            return luma_set_error(LUMA_E_INVALID, "adjoint: site type %d not supported (fluid, solid, velocity, "
                                                  "extrapolate-right only)", t);
    }
    return LUMA_OK;
}

AdjArgs make_adj_args(luma_gpu_grid *g, AdjState &st, int slot, int gbuf) {
    const IbmDevice &dv = g->ibm->dev;
    AdjArgs a;
    memset(&a, 0, sizeof a);
    a.N = g->d.N; a.M = g->d.M; a.K = g->d.K; a.ncell = (int)g->n; a.nm = dv.nm; a.nu = dv.nu; a.nsup = dv.nsup;
    a.body_base = st.body_base; a.body_nm = st.body_nm;
    a.quirk = g->d.dims == 3 && !(g->d.flags & LUMA_FLAG_FIX_MACRO3D);
    a.omega = g->d.omega; a.rho0 = g->d.rho_in; a.invT = 1.0 / st.T;
    a.typ = g->typ;
    a.site_u = st.site_u;
    a.near = st.near;
    a.near_ids = st.near_ids;
    a.nnear = st.nnear;
    const size_t rs = rsize(g);
    a.g = static_cast<char *>(st.tape_g) + (size_t)slot * g->n * g->d.Q * rs;
    a.Fm = st.tape_Fm + (size_t)slot * 3 * dv.nm;
    a.Fs = static_cast<char *>(st.tape_Fs) + (size_t)slot * g->d.dims * dv.nu * rs;
    a.lam_in = st.lam;
    a.lam_out = st.lam;
    a.lamg = st.lamg[gbuf];
    a.lamF = st.lamF;
    a.rho_field = g->rho;
    a.u_field = g->u;
    a.moff = dv.moff; a.msite = dv.msite; a.smarker = dv.smarker; a.usite = dv.usite; a.uoff = dv.uoff;
    a.uref = dv.uref; a.mdelta = dv.mdelta; a.vel = dv.vel; a.area = dv.area; a.w = st.w;
    a.mu = st.mu; a.Gw = st.Gw; a.Gd = st.Gd; a.gs = st.d_gs;
    return a;
}

template <int Q, class P>
cudaError_t launch_adj_collide(const AdjArgs &a, cudaStream_t s) {
    k_adj_collide<Q, P><<<(a.ncell + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
}

// The reverse IBM pass and the reverse stream of step t (a); with a
// previous step (b, prev) the reverse collision of step t-1 rides on the
// reverse stream.  With a near list, the one-block IBM pass runs on the side
// stream while the sites away from the supports stream back; the near sites
// follow once both are done (forked and joined by events, so the order holds
// in a captured graph as in direct launches).
template <int Q, class P>
cudaError_t launch_adj_step(const AdjArgs &a, const AdjArgs &b, bool prev, cudaStream_t s, const AdjState &st) {
    const size_t smem = ibm_block_smem(a.nsup, a.nm, a.nu, Q, sizeof(typename P::R));
    const bool block = a.nm > 0 && smem <= kIbmBlockMaxSmem;
    if (block && smem > 48 * 1024)
        cudaFuncSetAttribute(k_adj_ibm_block<Q, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const unsigned grid = (unsigned)((a.ncell + 255) / 256);
    if (block && prev && st.side && a.near_ids) {
        if (cudaEventRecord(st.ev_fork, s) != cudaSuccess || cudaStreamWaitEvent(st.side, st.ev_fork, 0) != cudaSuccess)
            return cudaGetLastError();
        k_adj_ibm_block<Q, P><<<1, kIbmBlock, smem, st.side>>>(a);
        if (cudaEventRecord(st.ev_join, st.side) != cudaSuccess) return cudaGetLastError();
        k_adj_stream<Q, P, true, 1><<<grid, 256, 0, s>>>(a, b);
        if (cudaStreamWaitEvent(s, st.ev_join, 0) != cudaSuccess) return cudaGetLastError();
        if (a.nnear > 0) k_adj_stream<Q, P, true, 2><<<(a.nnear + 63) / 64, 64, 0, s>>>(a, b);
        return cudaGetLastError();
    }
    if (block) {
        k_adj_ibm_block<Q, P><<<1, kIbmBlock, smem, s>>>(a);
    } else if (a.nm > 0) {
        k_adj_marker<Q, P><<<(a.nm + 63) / 64, 64, 0, s>>>(a);
        k_adj_support<Q, P><<<(a.nu + 127) / 128, 128, 0, s>>>(a);
    }
    if (prev) k_adj_stream<Q, P, true, 0><<<grid, 256, 0, s>>>(a, b);
    else k_adj_stream<Q, P, false, 0><<<grid, 256, 0, s>>>(a, b);
    return cudaGetLastError();
}

// Roma et al. (1999) 3-point kernel phi(r) and phi'(r) (r in units of the
// dilated spacing), as ibm_deltakernel evaluates phi.
double roma(double r) {
    const double a = std::fabs(r);
    if (a > 1.5) return 0.0;
    if (a > 0.5) return (5.0 - 3.0 * a - std::sqrt(1.0 - 3.0 * (1.0 - a) * (1.0 - a))) / 6.0;
    return (1.0 + std::sqrt(1.0 - 3.0 * a * a)) / 3.0;
}
double roma_d(double r) {
    const double a = std::fabs(r), sg = r < 0 ? -1.0 : 1.0;
    if (a > 1.5) return 0.0;
    if (a > 0.5) {
        const double q = 1.0 - a;
        return sg * (-3.0 - 3.0 * q / std::sqrt(1.0 - 3.0 * q * q)) / 6.0;
    }
    return -r / std::sqrt(1.0 - 3.0 * r * r);
}

// delta(x_s - X) of a marker with dilation `dil` and its gradient in X.
void delta_grad(const double xs[3], const double *X, double dh, double dil, int D, double *val, double grad[3]) {
    double p[3], dp[3];
    for (int d = 0; d < 3; ++d) {
        const double r = (xs[d] - X[d]) / dh / dil;
        p[d] = d < D ? roma(r) : 1.0;
        dp[d] = d < D ? roma_d(r) : 0.0;
    }
    *val = p[0] * p[1] * p[2];
    const double sc = -1.0 / (dh * dil);
    grad[0] = sc * dp[0] * p[1] * p[2];
    grad[1] = sc * p[0] * dp[1] * p[2];
    grad[2] = D == 3 ? sc * p[0] * p[1] * dp[2] : 0.0;
}

// Solve A^T x = b (A row-major n x n) by Gaussian elimination with partial
// pivoting.
void solve_transposed(int n, const std::vector<double> &A, std::vector<double> &x) {
    std::vector<double> a((size_t)n * n);
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) a[(size_t)r * n + c] = A[(size_t)c * n + r];
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int r = k + 1; r < n; ++r)
            if (std::fabs(a[(size_t)r * n + k]) > std::fabs(a[(size_t)p * n + k])) p = r;
        if (p != k) {
            for (int c = 0; c < n; ++c) std::swap(a[(size_t)k * n + c], a[(size_t)p * n + c]);
            std::swap(x[k], x[p]);
        }
        const double piv = a[(size_t)k * n + k];
        if (piv == 0.0) continue;
        for (int r = k + 1; r < n; ++r) {
            const double f = a[(size_t)r * n + k] / piv;
            if (f == 0.0) continue;
            for (int c = k; c < n; ++c) a[(size_t)r * n + c] -= f * a[(size_t)k * n + c];
            x[r] -= f * x[k];
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = x[r];
        for (int c = r + 1; c < n; ++c) s -= a[(size_t)r * n + c] * x[c];
        x[r] = a[(size_t)r * n + r] != 0.0 ? s / a[(size_t)r * n + r] : 0.0;
    }
}

// dJ/dX of one body from the device sensitivities: Gd (per support of the
// body, dJ/d delta_ms) and Gw (per marker, dJ/dw_m).  Follows the body's
// set-up: ds (first strict minimum of the marker distances), epsilon
// (A eps = 1, A_IJ = S_IJ area_I ds_J, S_IJ = sum over the supports q of I
// of delta_I(x_q) delta_J(x_q)).
void marker_gradient(const luma_gpu_grid *g, const IbmBody &bd, const double *Gd, const double *Gw, double *gX) {
    const int n = bd.nm, D = g->d.dims;
    const double dh = g->d.dh;
    std::fill(gX, gX + 3 * (size_t)n, 0.0);
    // (1) delta values of the supports
    for (int m = 0; m < n; ++m)
        for (int q = bd.off[m]; q < bd.off[m + 1]; ++q) {
            const double xs[3] = {bd.sx[q], bd.sy[q], bd.sz[q]};
            double val, gr[3];
            delta_grad(xs, &bd.pos[3 * m], dh, bd.dil[m], D, &val, gr);
            for (int d = 0; d < D; ++d) gX[3 * m + d] += Gd[q] * gr[d];
        }
    // (2) w_m = eps_m ds_m (* ds_m in 3D)
    std::vector<double> deps(n), dds(n);
    for (int m = 0; m < n; ++m) {
        const double ds = bd.ds[m], eps = bd.eps[m];
        deps[m] = Gw[m] * (D == 3 ? ds * ds : ds);
        dds[m] = Gw[m] * (D == 3 ? 2.0 * eps * ds : eps);
    }
    // (3) epsilon
    std::vector<double> S((size_t)n * n, 0.0), A((size_t)n * n);
    for (int I = 0; I < n; ++I)
        for (int J = 0; J < n; ++J) {
            double sij = 0.0;
            for (int q = bd.off[I]; q < bd.off[I + 1]; ++q) {
                const double xs[3] = {bd.sx[q], bd.sy[q], bd.sz[q]};
                double vJ, gJ[3];
                delta_grad(xs, &bd.pos[3 * J], dh, bd.dil[J], D, &vJ, gJ);
                sij += bd.delta[q] * vJ;
            }
            S[(size_t)I * n + J] = sij;
            A[(size_t)I * n + J] = sij * bd.area[I] * bd.ds[J];
        }
    std::vector<double> nu(deps);
    solve_transposed(n, A, nu);
    for (int I = 0; I < n; ++I)
        for (int J = 0; J < n; ++J) {
            const double sij = S[(size_t)I * n + J];
            if (sij == 0.0) continue;  // no overlap: the entry and its gradient vanish
            const double gA = -nu[I] * bd.eps[J];
            dds[J] += gA * sij * bd.area[I];
            const double gS = gA * bd.area[I] * bd.ds[J];
            for (int q = bd.off[I]; q < bd.off[I + 1]; ++q) {
                const double xs[3] = {bd.sx[q], bd.sy[q], bd.sz[q]};
                double vI, gI[3], vJ, gJ[3];
                delta_grad(xs, &bd.pos[3 * I], dh, bd.dil[I], D, &vI, gI);
                delta_grad(xs, &bd.pos[3 * J], dh, bd.dil[J], D, &vJ, gJ);
                for (int d = 0; d < D; ++d) {
                    gX[3 * I + d] += gS * gI[d] * vJ;
                    gX[3 * J + d] += gS * vI * gJ[d];
                }
            }
        }
    // (4) ds_m = min over n != m of |X_m - X_n| / dh
    for (int m = 0; m < n; ++m) {
        double best = 10.0;
        int arg = -1;
        for (int q = 0; q < n; ++q) {
            if (q == m) continue;
            double r = 0.0;
            for (int d = 0; d < 3; ++d) r += (bd.pos[3 * m + d] - bd.pos[3 * q + d]) * (bd.pos[3 * m + d] - bd.pos[3 * q + d]);
            const double dist = std::sqrt(r) / dh;
            if (dist < best) { best = dist; arg = q; }
        }
        if (arg < 0) continue;
        for (int d = 0; d < D; ++d) {
            const double gd = (bd.pos[3 * m + d] - bd.pos[3 * arg + d]) / (best * dh * dh);
            gX[3 * m + d] += dds[m] * gd;
            gX[3 * arg + d] -= dds[m] * gd;
        }
    }
}

}  // namespace

int luma_adj_step_hook(luma_gpu_grid *g, const StepArgs &a) {
    AdjState &st = *g->adj;
    (void)a;
    // the step's records went where luma_adj_redirect pointed them
    if (st.mode == 1 || st.mode == 2) st.tape_pos++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "adjoint hook: %s", cudaGetErrorString(e));
    return LUMA_OK;
}

// While taping, the step streams into the tape slot of the step and its
// collision writes the next state to the usual buffer, so the post-stream
// populations stay on the tape without a copy.
// The forward's step records its body's drag terms for the segment's J
// reduction; the taping step also records the marker forces.
void luma_adj_redirect(luma_gpu_grid *g, StepArgs &a) {
    const AdjState &st = *g->adj;
    if (st.mode == 1) {
        a.ibm_drag_out = st.drag_terms + (size_t)st.tape_pos * st.body_nm;
        a.ibm_drag_w = st.w;
        a.ibm_drag_base = st.body_base;
        a.ibm_drag_nm = st.body_nm;
    } else if (st.mode == 2) {
        a.fNew = static_cast<char *>(st.tape_g) + (size_t)st.tape_pos * g->n * g->d.Q * rsize(g);
        a.ibm_f_out = st.tape_Fm + (size_t)st.tape_pos * 3 * g->ibm->dev.nm;
        a.ibm_sf_out = static_cast<char *>(st.tape_Fs) + (size_t)st.tape_pos * g->d.dims * g->ibm->dev.nu * rsize(g);
    }
}

void luma_adj_free(luma_gpu_grid *g) {
    free_state(g->adj);
    g->adj = nullptr;
}

namespace {

// The adjoint's work runs on its own stream (capturable, unlike the legacy
// default stream); the caller's stream is drained first and put back after.
struct OwnStream {
    luma_gpu_grid *g;
    cudaStream_t saved;
    OwnStream(luma_gpu_grid *g_, AdjState &st) : g(g_), saved(g_->stream) {
        cudaStreamSynchronize(saved);
        g->stream = st.own;
    }
    ~OwnStream() { g->stream = saved; }
};

// Enqueues fn()'s work as a CUDA graph: captured and instantiated on first
// use, replayed after.  fn's host-side effects happen at capture only;
// `replay_effects` repeats the ones that matter on each later replay.  On a
// capture failure the work runs uncaptured and graphs are switched off.
template <class F, class H>
int run_graph(luma_gpu_grid *g, AdjState &st, cudaGraphExec_t *exec, F &&fn, H &&replay_effects) {
    cudaStream_t s = g->stream;
    if (!st.graphs) return fn();
    if (*exec) {
        if (cudaGraphLaunch(*exec, s) != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "adjoint: graph launch failed");
        replay_effects();
        return LUMA_OK;
    }
    const int t0 = g->t, cur0 = g->cur;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        st.graphs = false;
        return fn();
    }
    const int rc = fn();
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s, &graph);
    cudaError_t ei = cudaErrorUnknown;
    if (rc == LUMA_OK && e == cudaSuccess && graph) ei = cudaGraphInstantiate(exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        cudaGetLastError();
        *exec = nullptr;
        st.graphs = false;
        g->t = t0;
        g->cur = cur0;
        return fn();
    }
    if (cudaGraphLaunch(*exec, s) != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "adjoint: graph launch failed");
    return LUMA_OK;
}

// Per-site index of the distinct support site (or -1), for the force-field
// reconstruction in the reverse collide.
int build_site_map(luma_gpu_grid *g, AdjState &st, const std::vector<int> &usite) {
    const IbmDevice &dv = g->ibm->dev;
    std::vector<int> map(g->n, -1);
    for (int u = 0; u < dv.nu; ++u) map[usite[u]] = u;
    int rc = dmalloc(&st.site_u, g->n * sizeof(int), st);
    if (rc) return rc;
    if (cudaMemcpy(st.site_u, map.data(), g->n * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        return luma_set_error(LUMA_E_CUDA, "adjoint: site map upload");
    // Sites whose reverse stream reads the adjoint at a support site u: the
    // pull sources u - c_v, u itself (bounce-back, inflow) and the
    // extrapolate-right sources u - c_v - 2 e_x, periodic like the gathers.
    const int N = g->d.N, M = g->d.M, K = g->d.K, D = g->d.dims;
    std::vector<uint8_t> near(g->n, 0);
    for (int u = 0; u < dv.nu; ++u) {
        const int id = usite[u];
        const int k = id % K, j = (id / K) % M, i = id / (K * M);
        for (int di = -3; di <= 1; ++di)
            for (int dj = -1; dj <= 1; ++dj)
                for (int dk = (D == 3 ? -1 : 0); dk <= (D == 3 ? 1 : 0); ++dk) {
                    const int x = ((i + di) % N + N) % N, y = ((j + dj) % M + M) % M, z = ((k + dk) % K + K) % K;
                    near[(size_t)z + (size_t)y * K + (size_t)x * K * M] = 1;
                }
    }
    std::vector<int> ids;
    for (size_t id = 0; id < g->n; ++id)
        if (near[id]) ids.push_back((int)id);
    st.nnear = (int)ids.size();
    if ((rc = dmalloc(&st.near, g->n, st)) || (rc = dmalloc(&st.near_ids, ids.size() * sizeof(int), st))) return rc;
    if (cudaMemcpy(st.near, near.data(), g->n, cudaMemcpyHostToDevice) != cudaSuccess ||
        (!ids.empty() && cudaMemcpy(st.near_ids, ids.data(), ids.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess))
        return luma_set_error(LUMA_E_CUDA, "adjoint: near-site upload");
    return LUMA_OK;
}

}  // namespace

extern "C" {

int luma_gpu_adj_forward(luma_gpu_grid *g, int nsteps, int checkpoint_every, int body, double *J) {
    if (!g || !J || nsteps <= 0 || checkpoint_every <= 0)
        return luma_set_error(LUMA_E_INVALID, "luma_gpu_adj_forward: null pointer or non-positive step counts");
    int rc = check_scope(g, body);
    if (rc) return rc;
    const IbmState &ib = *g->ibm;
    const IbmDevice &dv = ib.dev;
    std::vector<int> usite(dv.nu);
    if (dv.nu && cudaMemcpy(usite.data(), dv.usite, dv.nu * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return luma_set_error(LUMA_E_CUDA, "adjoint: support sites");
    const int K = std::min(checkpoint_every, nsteps);
    AdjState *st = g->adj;
    bool reuse = false;
    if (st && st->T == nsteps && st->K == K && st->body == body && st->usite_host == usite) {
        std::vector<uintptr_t> sig;
        luma_tree_signature(g, sig);
        reuse = sig == st->sig;
    }
    auto fail = [&](int code) { luma_adj_free(g); return code; };
    const size_t rs = rsize(g);
    const size_t fbytes = g->n * g->d.Q * rs;
    const size_t ub = g->n * g->d.dims * rs, rb = g->n * rs;
    if (!reuse) {
        luma_adj_free(g);
        st = new AdjState();
        g->adj = st;
        if (cudaStreamCreateWithFlags(&st->own, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&st->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&st->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&st->ev_join, cudaEventDisableTiming) != cudaSuccess)
            return fail(luma_set_error(LUMA_E_CUDA, "adjoint: stream creation failed"));
        st->body = body;
        st->T = nsteps;
        st->K = K;
        st->nseg = (nsteps + K - 1) / K;
        st->usite_host = usite;
        if ((rc = dmalloc(&st->w, (size_t)dv.nm * 8, *st)) || (rc = dmalloc(&st->d_J, 8, *st)) ||
            (rc = dmalloc(&st->d_gs, 8, *st)) || (rc = build_site_map(g, *st, usite)))
            return fail(rc);
        int bnm = 0;
        for (size_t b = 0; b < ib.bodies.size(); ++b)
            if ((int)b == body) bnm = ib.bodies[b].nm;
        if ((rc = dmalloc(&st->drag_terms, (size_t)K * std::max(1, bnm) * 8, *st))) return fail(rc);
        st->ckpt.assign(st->nseg, nullptr);
        for (int k = 0; k < st->nseg; ++k)
            if ((rc = dmalloc(&st->ckpt[k], fbytes, *st))) return fail(rc);
        if ((rc = dmalloc(&st->fin_f[0], fbytes, *st)) || (rc = dmalloc(&st->fin_f[1], fbytes, *st)) ||
            (rc = dmalloc(&st->fin_u, ub, *st)) || (rc = dmalloc(&st->fin_rho, rb, *st)))
            return fail(rc);
        st->graphs = (K % 2) == 0;  // a graph replays a fixed buffer parity
        luma_tree_signature(g, st->sig);
    }
    st->valid = false;
    std::vector<double> w;
    int base = 0, sbase = 0;
    for (size_t b = 0; b < ib.bodies.size(); ++b) {
        const IbmBody &bd = ib.bodies[b];
        if ((int)b == body) {
            st->body_base = base;
            st->body_nm = bd.nm;
            st->body_sup = sbase;
        }
        for (int m = 0; m < bd.nm; ++m) w.push_back(bd.eps[m] * (g->d.dims == 3 ? bd.ds[m] : 1.0) * bd.ds[m]);
        base += bd.nm;
        sbase += bd.off.back();
    }
    if (cudaMemcpy(st->w, w.data(), w.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(luma_set_error(LUMA_E_CUDA, "adjoint: weights upload"));
    double h = 0.0;
    {
        OwnStream guard(g, *st);
        cudaStream_t s = g->stream;
        cudaMemsetAsync(st->d_J, 0, 8, s);
        st->t0 = g->t;
        st->mode = 1;
        // one forward segment: its steps record the drag terms, one block
        // folds them into J
        auto segment = [&](int steps) -> int {
            st->tape_pos = 0;
            int r = luma_gpu_step(g, steps);
            if (r) return r;
            k_drag_segment<<<1, 256, 0, g->stream>>>(st->drag_terms, steps, st->body_nm, 1.0 / st->T, st->d_J);
            const cudaError_t e = cudaGetLastError();
            return e == cudaSuccess ? LUMA_OK : luma_set_error(LUMA_E_CUDA, "adjoint drag: %s", cudaGetErrorString(e));
        };
        for (int k = 0; k < st->nseg; ++k) {
            if (cudaMemcpyAsync(st->ckpt[k], g->f[g->cur], fbytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                return fail(luma_set_error(LUMA_E_CUDA, "adjoint: checkpoint copy failed"));
            const int steps = std::min(st->K, st->T - k * st->K);
            if (steps == st->K)
                rc = run_graph(g, *st, &st->seg_fwd, [&] { return segment(steps); }, [&] { g->t += steps; });
            else
                rc = segment(steps);
            if (rc) {
                st->mode = 0;
                return fail(rc);
            }
        }
        st->mode = 0;
        // the state after the forward, put back after the backward sweep
        cudaMemcpyAsync(st->fin_f[0], g->f[0], fbytes, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(st->fin_f[1], g->f[1], fbytes, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(st->fin_u, g->u, ub, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(st->fin_rho, g->rho, rb, cudaMemcpyDeviceToDevice, s);
        st->fin_cur = g->cur;
        st->fin_t = g->t;
        cudaMemcpyAsync(&h, st->d_J, 8, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail(luma_set_error(LUMA_E_CUDA, "adjoint forward: %s", cudaGetErrorString(e)));
    }
    *J = h;
    st->valid = true;
    return LUMA_OK;
}

int luma_gpu_adj_backward(luma_gpu_grid *g, double dJ, double *grad_inlet_scale, double *grad_markers) {
    if (!g || !g->adj || !g->adj->valid)
        return luma_set_error(LUMA_E_STATE, "luma_gpu_adj_backward needs a preceding luma_gpu_adj_forward (once each)");
    AdjState &st = *g->adj;
    const IbmDevice &dv = g->ibm->dev;
    const int D = g->d.dims, Q = g->d.Q;
    const size_t rs = rsize(g);
    const size_t fbytes = g->n * Q * rs;
    int rc;
    if (!st.tape_g) {
        if ((rc = dmalloc(&st.tape_g, (size_t)st.K * fbytes, st)) ||
            (rc = dmalloc(&st.tape_Fm, (size_t)st.K * 3 * dv.nm * 8, st)) || (rc = dmalloc(&st.lam, fbytes, st)) ||
            (rc = dmalloc(&st.tape_Fs, (size_t)st.K * D * dv.nu * rs, st)) ||
            (rc = dmalloc(&st.lamg[0], fbytes, st)) || (rc = dmalloc(&st.lamg[1], fbytes, st)) ||
            (rc = dmalloc(&st.lamF, g->n * D * rs, st)) || (rc = dmalloc(&st.mu, 3 * (size_t)dv.nm * 8, st)) ||
            (rc = dmalloc(&st.Gw, (size_t)dv.nm * 8, st)) || (rc = dmalloc(&st.Gd, (size_t)dv.nsup * 8, st)))
            return rc;
        // the recompute's second loop also collides sites the stream skips
        // (solid, velocity) from the tape: keep that memory defined
        if (cudaMemset(st.tape_g, 0, (size_t)st.K * fbytes) != cudaSuccess)
            return luma_set_error(LUMA_E_CUDA, "adjoint: tape clear");
    }
    std::vector<double> Gw(dv.nm), Gd(dv.nsup);
    double gs = 0.0;
    {
        OwnStream guard(g, st);
        cudaStream_t s = g->stream;
        cudaMemsetAsync(st.lam, 0, fbytes, s);
        cudaMemsetAsync(st.Gw, 0, (size_t)dv.nm * 8, s);
        cudaMemsetAsync(st.Gd, 0, (size_t)dv.nsup * 8, s);
        cudaMemsetAsync(st.d_gs, 0, 8, s);
        // one segment: recompute with the tape on, then the reverse steps:
        // the reverse collision of the last step from the adjoint in
        // memory, then per step the reverse IBM pass and the reverse stream,
        // which carries the reverse collision of the step before it; the
        // segment's first step leaves the adjoint of its start in memory
        auto segment = [&](int steps) -> int {
            st.mode = 2;
            st.tape_pos = 0;
            int r = luma_gpu_step(g, steps);
            st.mode = 0;
            if (r) return r;
            int gb = 0;
            cudaError_t e = dispatch(Q, g->d.precision, [&](auto q, auto p) {
                return launch_adj_collide<decltype(q)::value, decltype(p)>(make_adj_args(g, st, steps - 1, gb), s);
            });
            for (int t = steps - 1; t >= 0 && e == cudaSuccess; --t) {
                const AdjArgs a = make_adj_args(g, st, t, gb);
                const AdjArgs b = make_adj_args(g, st, t > 0 ? t - 1 : 0, gb ^ 1);
                e = dispatch(Q, g->d.precision, [&](auto q, auto p) {
                    return launch_adj_step<decltype(q)::value, decltype(p)>(a, b, t > 0, s, st);
                });
                gb ^= 1;
            }
            if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "adjoint step: %s", cudaGetErrorString(e));
            return LUMA_OK;
        };
        for (int k = st.nseg - 1; k >= 0; --k) {
            const int steps = std::min(st.K, st.T - k * st.K);
            cudaMemcpyAsync(g->f[g->cur], st.ckpt[k], fbytes, cudaMemcpyDeviceToDevice, s);
            g->t = st.t0 + k * st.K;
            if (steps == st.K)
                rc = run_graph(g, st, &st.seg_bwd, [&] { return segment(steps); }, [&] { g->t += steps; });
            else
                rc = segment(steps);
            if (rc) return rc;
        }
        cudaMemcpyAsync(Gw.data(), st.Gw, (size_t)dv.nm * 8, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(Gd.data(), st.Gd, (size_t)dv.nsup * 8, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&gs, st.d_gs, 8, cudaMemcpyDeviceToHost, s);
        // put back the state after the forward
        cudaMemcpyAsync(g->f[0], st.fin_f[0], fbytes, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(g->f[1], st.fin_f[1], fbytes, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(g->u, st.fin_u, g->n * D * rs, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(g->rho, st.fin_rho, g->n * rs, cudaMemcpyDeviceToDevice, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "adjoint backward: %s", cudaGetErrorString(e));
    }
    g->cur = st.fin_cur;
    g->t = st.fin_t;
    st.valid = false;
    if (grad_inlet_scale) *grad_inlet_scale = dJ * gs;
    if (grad_markers) {
        const IbmBody &bd = g->ibm->bodies[st.body];
        std::vector<double> gX(3 * (size_t)bd.nm);
        marker_gradient(g, bd, Gd.data() + st.body_sup, Gw.data() + st.body_base, gX.data());
        for (int m = 0; m < bd.nm; ++m)
            for (int d = 0; d < D; ++d) grad_markers[(size_t)D * m + d] = dJ * gX[3 * m + d];
    }
    return LUMA_OK;
}

int luma_gpu_adj_memory(const luma_gpu_grid *g, size_t *bytes) {
    if (!g || !bytes) return luma_set_error(LUMA_E_INVALID, "luma_gpu_adj_memory: null argument");
    *bytes = g->adj ? g->adj->bytes : 0;
    return LUMA_OK;
}

}  // extern "C"
