// General two-buffer LBM step: every site type of the reference's stream,
// macroscopic, forcing and collision operators, with the reference's
// update order.  Used for grids with boundaries, refinement or IBM; the
// all-periodic fast path lives in k_bulk.cu.
//
// One step of a grid (GridObj::LBM_multi_opt, src/GridObj_ops_lbm_optimised.cpp:36-193):
//   phase A  k_stream_macro   stream (:206-297) + macroscopic (:800-919)
//                             [+ forcing and collision when the reference runs
//                             a single loop, i.e. without L_IBM_ON]
//   phase B  k_regularised    regularised velocity/pressure sites (:313-510);
//                             they read the interior macroscopic values of
//                             phase A (extrapolation, :1353-1412)
//   phase V  k_velocity_u     the u written into velocity sites by the
//                             forced-equilibrium BC under a velocity ramp (:255-265)
//   [IBM pass]
//   phase C  k_force_collide  forcing (:928-990) + collision (:765-790,
//                             :1122-1305) when the reference splits the loop
// followed by a swap of the two population buffers (:159).
#include <cuda_runtime.h>

#include <type_traits>

#include "device.cuh"
#include "grid.hpp"
#include "kernels.hpp"

namespace luma {

namespace {

template <int Q>
__device__ __forceinline__ int child_at(const StepArgs &a, int i, int j, int k) {
    constexpr int D = Lattice<Q>::D;
    if (a.level > 0) return a.nchild ? 0 : -1;
    int found = -1;
    // unrolled over the argument array (a run-time index would copy it to
    // local memory); the first child holding the site wins
#pragma unroll
    for (int s = kMaxChildren - 1; s >= 0; --s) {
        const int *L = a.child[s].lims;
        if (s < a.nchild && i >= L[0] && i <= L[1] && j >= L[2] && j <= L[3] && (D == 2 || (k >= L[4] && k <= L[5])))
            found = s;
    }
    return found;
}

// The 2^d fine sites under coarse site (i, j, k) in its child grid
// (GridUtils::getFineIndices): the child's populations, their per-direction
// stride, the first site and the steps along j and i.  False when no child
// holds the site.
template <int Q>
__device__ __forceinline__ bool coalesce_base(const StepArgs &a, int i, int j, int k, const void *&cf, size_t &cn,
                                              size_t &c0, size_t &cdj, size_t &cdi) {
    constexpr int D = Lattice<Q>::D;
    const int cs = child_at<Q>(a, i, j, k);
    bool ok = false;
#pragma unroll
    for (int q = 0; q < kMaxChildren; ++q)
        if (q == cs) {
            const ChildView &cg = a.child[q];
            const int ci = 2 * (i - cg.lims[0] + 1) - 2;
            const int cj = 2 * (j - cg.lims[2] + 1) - 2;
            const int ck = D == 3 ? 2 * (k - cg.lims[4] + 1) - 2 : 0;
            cf = cg.f;
            cn = (size_t)cg.N * cg.M * cg.K;
            c0 = (size_t)ck + (size_t)cj * cg.K + (size_t)ci * cg.K * cg.M;
            cdj = cg.K;
            cdi = (size_t)cg.K * cg.M;
            ok = true;
        }
    return ok;
}

// The direction tables in constant memory, for code that picks the
// direction at run time (one thread per population); fully unrolled loops
// use Lattice<Q>'s constexpr accessors, which fold to immediates.
template <int Q>
struct DirTable {
    int c[Q][3];
    int opp[Q];
    int refl[3][Q];
};
template <int Q>
constexpr DirTable<Q> dir_table() {
    DirTable<Q> t{};
    for (int v = 0; v < Q; ++v) {
        for (int d = 0; d < 3; ++d) t.c[v][d] = Lattice<Q>::c(v, d);
        t.opp[v] = Lattice<Q>::opp(v);
        for (int p = 0; p < 3; ++p) t.refl[p][v] = Lattice<Q>::reflect(p, v);
    }
    return t;
}
__constant__ DirTable<LUMA_GEN_Q> kDirs = dir_table<LUMA_GEN_Q>();

template <int Q, bool RT>
__device__ __forceinline__ int dir_c(int v, int d) {
    static_assert(!RT || Q == LUMA_GEN_Q, "run-time direction tables exist for this unit's lattice only");
    if constexpr (RT) return kDirs.c[v][d];
    else return Lattice<Q>::c(v, d);
}
template <int Q, bool RT>
__device__ __forceinline__ int dir_opp(int v) {
    if constexpr (RT) return kDirs.opp[v];
    else return Lattice<Q>::opp(v);
}
template <int Q, bool RT>
__device__ __forceinline__ int dir_reflect(int plane, int v) {
    if constexpr (RT) return kDirs.refl[plane][v];
    else return Lattice<Q>::reflect(plane, v);
}

// The pull from a forced-equilibrium velocity site (_LBM_stream_opt's
// velocity branch): the equilibrium of the source's rho and u (the inlet
// profile times the ramp while a ramp runs).
template <int Q, class P>
__device__ __forceinline__ typename P::R velocity_pull(const StepArgs &a, int j, int sid, int v) {
    using R = typename P::R;
    constexpr int D = Lattice<Q>::D;
    const size_t n = (size_t)a.ncell;
    const R rs = ldr<P>(a.rho, sid);
    R ux, uy, uz = R(0);
    if (a.has_ramp) {
        ux = R(a.ux_in[j] * a.ramp_stream);
        uy = R(a.uy_in[j] * a.ramp_stream);
        if (D == 3) uz = R(a.uz_in[j] * a.ramp_stream);
    } else {
        ux = ldr<P>(a.u, sid);
        uy = ldr<P>(a.u, n + sid);
        if (D == 3) uz = ldr<P>(a.u, 2 * n + sid);
    }
    return feq_s<Q, P>(v, rs, rs - rho0_of<P>(a), ux, uy, uz, cs2_of<P>(a));
}

// _LBM_stream_opt (:206-297) for one direction v of one site: the streamed
// population in the stored representation.  RT: v is a run-time value.
template <int Q, class P, bool RT>
__device__ __forceinline__ typename P::R stream_dir(const StepArgs &a, const int8_t *wall, int i, int j, int k,
                                                    int id, int type, int v) {
    using L = Lattice<Q>;
    using R = typename P::R;
    constexpr int D = L::D;
    const int N = a.N, M = a.M, K = a.K;
    const size_t n = (size_t)a.ncell;
    const int cx = dir_c<Q, RT>(v, 0), cy = dir_c<Q, RT>(v, 1), cz = dir_c<Q, RT>(v, 2);
    int sx = i - cx, sy = j - cy, sz = k - cz;
    sx = sx < 0 ? sx + N : (sx >= N ? sx - N : sx);
    sy = sy < 0 ? sy + M : (sy >= M ? sy - M : sy);
    if (D == 3) sz = sz < 0 ? sz + K : (sz >= K ? sz - K : sz);
    else sz = 0;
    const int sid = sz + sy * K + sx * K * M;
    const int stype = a.typ[sid];
    if (type == LUMA_SITE_BFL || stype == LUMA_SITE_BFL) {
        // _LBM_applyBFL_opt (:1010-1113) through the link tables
        // (kinds in bfl.cu); links without a wall stream as usual
        if (!a.bfl_rec) {
            *a.unsupported = 1;
            return R(0);
        }
        const int r = a.bfl_rec[id];
        const uint32_t lm = r >= 0 ? a.bfl_mask[r] : 0u;
        if ((lm >> v) & 1u) {
            const int l = a.bfl_first[r] + __popc(lm & ((1u << v) - 1u));
            const int kind = a.bfl_kind[l];
            const R fo = ld<P>(a.f, (size_t)dir_opp<Q, RT>(v) * n + id);
            R out;
            if (kind == 0) {
                out = fo;
            } else if (kind == 1) {
                out = ld<P>(a.fNew, (size_t)v * n + id);
            } else {
                const double q = a.bfl_q[l];
                const R fv = ld<P>(a.f, (size_t)v * n + id);
                out = add_rn(mul_rn(R(1 - 2 * q), R((fv - fo) / R(2 - 2 * q))), fo);
            }
            if (kind != 1) {
                const double sh = P::shifted ? L::w(v) * a.rho0 : 0.0;  // w_opp(v) = w_v
                a.bfl_val[l] = (double(fo) + sh) + (double(out) + sh);
            }
            return out;
        }
    }
    if (type == LUMA_SITE_SLIP) {
        // _LBM_applySpecReflect_opt (:527-581): first matching wall wins.
        const int8_t nv0 = wall[4 * (size_t)id + 0], nv1 = wall[4 * (size_t)id + 1], nv2 = wall[4 * (size_t)id + 2];
        int plane = -1;
        if (nv0 == 1 && cx == 1) plane = 0;
        else if (nv0 == -1 && cx == -1) plane = 0;
        else if (nv1 == 1 && cy == 1) plane = 1;
        else if (nv1 == -1 && cy == -1) plane = 1;
        else if (nv2 == 1 && cz == 1) plane = 2;
        else if (nv2 == -1 && cz == -1) plane = 2;
        if (plane >= 0) return ld<P>(a.f, (size_t)dir_reflect<Q, RT>(plane, v) * n + id);
    }
    if (stype == LUMA_SITE_SOLID) return ld<P>(a.f, (size_t)dir_opp<Q, RT>(v) * n + id);
    if (stype == LUMA_SITE_EXTRAPOLATE_RIGHT) return ld<P>(a.f, (size_t)v * n + (sid - 2 * (K * M)));
    if (stype == LUMA_SITE_VELOCITY && !(a.flags & LUMA_FLAG_REGULARISED)) return velocity_pull<Q, P>(a, j, sid, v);
    if (a.parent_f && stype == LUMA_SITE_TL_TO_COARSER && a.subcycle == 0) {
        // _LBM_explode_opt (:646-663) with GridUtils::getCoarseIndices.
        int fx = sx, fy = sy, fz = sz;
        if (fx % 2 != 0) fx -= 1;
        if (fy % 2 != 0) fy -= 1;
        if (fz % 2 != 0) fz -= 1;
        const int pi = fx / 2 + a.lims[0];
        const int pj = fy / 2 + a.lims[2];
        const int pk = D == 3 ? fz / 2 + a.lims[4] : 0;
        const size_t pn = (size_t)a.pN * a.pM * a.pK;
        return ld<P>(a.parent_f, (size_t)v * pn + pk + (size_t)pj * a.pK + (size_t)pi * a.pK * a.pM);
    }
    if (a.nchild && stype == LUMA_SITE_REFINED && type == LUMA_SITE_TL_TO_FINER) {
        // _LBM_coalesce_opt (:591-636) with GridUtils::getFineIndices.
        const void *cf;
        size_t cn, c0, cdj, cdi;
        if (!coalesce_base<Q>(a, i, j, k, cf, cn, c0, cdj, cdi)) {
            *a.unsupported = 2;
            return R(0);
        }
        R acc = R(0);
#pragma unroll
        for (int ii = 0; ii < 2; ++ii)
#pragma unroll
            for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk)
                    acc += ld<P>(cf, (size_t)v * cn + c0 + (size_t)kk + jj * cdj + ii * cdi);
        return acc / (D == 3 ? R(8) : R(4));
    }
    return ld<P>(a.f, (size_t)v * n + sid);
}

// _LBM_macro_opt (:800-891): density and velocity of fluid-like sites from
// the streamed populations, + 0.5*F when forcing; the 3D reference adds the
// z half-force to x (:833) unless LUMA_FLAG_FIX_MACRO3D.
// TAV: the kernel carries the running-mean update (a compile-time choice:
// the lean interior kernels do without its registers).
template <int Q, class P, bool STORE = true, bool TAV = true>
__device__ __forceinline__ void macro_site(const StepArgs &a, int i, int j, int k, int id, int type,
                                           const typename P::R *fn, typename P::R &rho, typename P::R &drho,
                                           typename P::R &ux, typename P::R &uy, typename P::R &uz,
                                           int tav_reps = 1) {
    using L = Lattice<Q>;
    using R = typename P::R;
    constexpr int D = L::D;
    const size_t n = (size_t)a.ncell;
    if (type == LUMA_SITE_FLUID || type == LUMA_SITE_BFL || type == LUMA_SITE_TL_TO_FINER ||
        type == LUMA_SITE_SLIP) {
        R r = R(0), mx = R(0), my = R(0), mz = R(0);
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            r += fn[v];
            mx += R(L::c(v, 0)) * fn[v];
            my += R(L::c(v, 1)) * fn[v];
            if (D == 3) mz += R(L::c(v, 2)) * fn[v];
        }
        if (a.forcing) {
            const R Fx = ldr<P>(a.force, id), Fy = ldr<P>(a.force, n + id);
            mx += R(0.5) * Fx;
            my += R(0.5) * Fy;
            if (D == 3) {
                const R Fz = ldr<P>(a.force, 2 * n + id);
                if (a.flags & LUMA_FLAG_FIX_MACRO3D) mz += R(0.5) * Fz;
                else mx += R(0.5) * Fz;
            }
        }
        if (P::shifted) {
            drho = r;
            rho = rho0_of<P>(a) + r;
        } else {
            rho = r;
            drho = r - rho0_of<P>(a);
        }
        ux = mx / rho;
        uy = my / rho;
        uz = D == 3 ? mz / rho : R(0);
        if (STORE) {
            str<P>(a.u, id, ux);
            str<P>(a.u, n + id, uy);
            if (D == 3) str<P>(a.u, 2 * n + id, uz);
            str<P>(a.rho, id, rho);
        }
    } else {
        rho = ldr<P>(a.rho, id);
        drho = rho - rho0_of<P>(a);
        ux = ldr<P>(a.u, id);
        uy = ldr<P>(a.u, n + id);
        uz = D == 3 ? ldr<P>(a.u, 2 * n + id) : R(0);
    }
    // time-averaged quantities (:895-917), tav_reps times (an IB support
    // site is re-macroed once per marker it supports)
    if (TAV && a.tav_rho) {
        const double t = (double)a.tav_t, t1 = (double)(a.tav_t + 1);
        const double uu[3] = {double(ux), double(uy), double(uz)};
        for (int rep = 0; rep < tav_reps; ++rep) {
            a.tav_rho[id] = __ddiv_rn(__dadd_rn(__dmul_rn(a.tav_rho[id], t), double(rho)), t1);
            int pq = 0;
            for (int p = 0; p < D; ++p) {
                double *up = a.tav_u + (size_t)p * n + id;
                *up = __ddiv_rn(__dadd_rn(__dmul_rn(*up, t), uu[p]), t1);
                for (int q = p; q < D; ++q) {
                    double *w = a.tav_uu + (size_t)pq * n + id;
                    *w = __ddiv_rn(__dadd_rn(__dmul_rn(*w, t), __dmul_rn(uu[p], uu[q])), t1);
                    ++pq;
                }
            }
        }
    }
    if (type == LUMA_SITE_TL_TO_FINER) {
        const int s = child_at<Q>(a, i, j, k);
#pragma unroll
        for (int q = 0; q < kMaxChildren; ++q) {
        if (q != s) continue;  // the child by unrolled selection (no local copy of the argument array)
        const ChildView &cg = a.child[q];
        const int ci = 2 * (i - cg.lims[0] + 1) - 2;
        const int cj = 2 * (j - cg.lims[2] + 1) - 2;
        const int ck = D == 3 ? 2 * (k - cg.lims[4] + 1) - 2 : 0;
        const size_t cn = (size_t)cg.N * cg.M * cg.K;
        for (int ii = 0; ii < 2; ++ii)
            for (int jj = 0; jj < 2; ++jj)
                for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk) {
                    const size_t cid = (size_t)(ck + kk) + (size_t)(cj + jj) * cg.K + (size_t)(ci + ii) * cg.K * cg.M;
                    str<P>(cg.u, cid, ux);
                    str<P>(cg.u, cn + cid, uy);
                    if (D == 3) str<P>(cg.u, 2 * cn + cid, uz);
                    str<P>(cg.rho, cid, rho);
                }
        }
    }
}

// _LBM_smag (:717-756): Smagorinsky-modified relaxation frequency.
template <int Q, class P>
__device__ __forceinline__ typename P::R smag_omega(const StepArgs &a, const typename P::R *fn, typename P::R rho,
                                                    typename P::R drho, typename P::R ux, typename P::R uy,
                                                    typename P::R uz) {
    using L = Lattice<Q>;
    using R = typename P::R;
    constexpr int D = L::D;
    R S00 = 0, S01 = 0, S02 = 0, S11 = 0, S12 = 0, S22 = 0;
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        const R fneq = fn[v] - feq_s<Q, P>(v, rho, drho, ux, uy, uz, cs2_of<P>(a));
        S00 += R(L::c(v, 0) * L::c(v, 0)) * fneq;
        S01 += R(L::c(v, 0) * L::c(v, 1)) * fneq;
        S11 += R(L::c(v, 1) * L::c(v, 1)) * fneq;
        if (D == 3) {
            S02 += R(L::c(v, 0) * L::c(v, 2)) * fneq;
            S12 += R(L::c(v, 1) * L::c(v, 2)) * fneq;
            S22 += R(L::c(v, 2) * L::c(v, 2)) * fneq;
        }
    }
    const R r0 = S00 * S00 + S01 * S01 + S02 * S02;
    const R r1 = S01 * S01 + S11 * S11 + S12 * S12;
    const R r2 = S02 * S02 + S12 * S12 + S22 * S22;
    const R Qs = sqrt(R(2) * (r0 + r1 + r2));
    const R tau = R(1) / omega_of<P>(a);
    const R cs2 = cs2_of<P>(a);
    const R tau_t = R(0.5) * (sqrt(tau * tau + R(2) * R(1.4142135623730950488016887242097) * csmag2_of<P>(a) *
                                                   rho0_of<P>(a) * cs2 * cs2 * Qs) - tau);
    return R(1) / (tau + tau_t);
}

// Collision of one site in place on fn (BGK / BGK-Smagorinsky / KBC), with
// the Guo term when forcing.  The reference's KBC reads the pre-stream f of
// the site (:1147, :1296).  COLL fixes the operator at compile time (-1:
// a.collision at run time).
template <int Q, class P, int COLL = -1>
__device__ __forceinline__ void collide_site(const StepArgs &a, int id, typename P::R *fn, typename P::R rho,
                                             typename P::R drho, typename P::R ux, typename P::R uy,
                                             typename P::R uz) {
    using L = Lattice<Q>;
    using R = typename P::R;
    constexpr int D = L::D;
    const size_t n = (size_t)a.ncell;
    const R cs2 = cs2_of<P>(a);
    R Fx = R(0), Fy = R(0), Fz = R(0);
    if (a.forcing) {
        Fx = ldr<P>(a.force, id);
        Fy = ldr<P>(a.force, n + id);
        if (D == 3) Fz = ldr<P>(a.force, 2 * n + id);
    }
    const int coll = COLL >= 0 ? COLL : a.collision;
    if (coll != LUMA_COLL_KBC) {
        const R om = coll == LUMA_COLL_BGK_SMAG ? smag_omega<Q, P>(a, fn, rho, drho, ux, uy, uz) : omega_of<P>(a);
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            const R eq = feq_s<Q, P>(v, rho, drho, ux, uy, uz, cs2);
            if (a.forcing) fn[v] = fn[v] + (om * (eq - fn[v]) + guo<Q, R>(v, omega_of<P>(a), cs2, ux, uy, uz, Fx, Fy, Fz));
            else fn[v] = fn[v] + om * (eq - fn[v]);
        }
        return;
    }
    // KBC-N4 (3D) / KBC-D (2D), _LBM_kbcCollide_opt (:1122-1305).
    const bool fixed = (a.flags & LUMA_FLAG_FIX_KBC) != 0;
    R src[Q], fe[Q], fneq[Q];
    R M[13];
#pragma unroll
    for (int m = 0; m < 13; ++m) M[m] = R(0);
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        src[v] = fixed ? fn[v] : ld<P>(a.f, (size_t)v * n + id);
        fe[v] = feq_s<Q, P>(v, rho, drho, ux, uy, uz, cs2);
        fneq[v] = src[v] - fe[v];
        const int cx = L::c(v, 0), cy = L::c(v, 1), cz = L::c(v, 2);
        if (D == 3) {
            // moment order: xx, xxy, xxz, xy, xyy, xyz, xz, xzz, yy, yyz, yz, yzz, zz
            M[0] += fneq[v] * R(cx * cx);
            M[1] += fneq[v] * R(cx * cx * cy);
            M[2] += fneq[v] * R(cx * cx * cz);
            M[3] += fneq[v] * R(cx * cy);
            M[4] += fneq[v] * R(cx * cy * cy);
            M[5] += fneq[v] * R(cx * cy * cz);
            M[6] += fneq[v] * R(cx * cz);
            M[7] += fneq[v] * R(cx * cz * cz);
            M[8] += fneq[v] * R(cy * cy);
            M[9] += fneq[v] * R(cy * cy * cz);
            M[10] += fneq[v] * R(cy * cz);
            M[11] += fneq[v] * R(cy * cz * cz);
            M[12] += fneq[v] * R(cz * cz);
        } else {
            M[0] += fneq[v] * R(cx * cx);
            M[1] += fneq[v] * R(cx * cy);
            M[2] += fneq[v] * R(cy * cy);
        }
    }
    // FP32 (shifted) path: the divisions by 6 and by the equilibrium as
    // products with reciprocals (an FP32 division is a multi-instruction
    // sequence, ~60 per site here); FP64 keeps the reference's divisions.
    auto sixth = [](R x) -> R {
        if constexpr (P::shifted) return x * R(1.0 / 6.0);
        else return x / R(6);
    };
    R ds[Q];
    R top = R(0), bot = R(0);
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        const int cx = L::c(v, 0), cy = L::c(v, 1), cz = L::c(v, 2);
        R s;
        if (D == 3) {
            if (cx == 0) {
                if (cy == 0) {
                    if (cz == 0) s = (-(M[0] + M[8] + M[12]));
                    else
                        s = (sixth((-(M[0] - M[12]) - (M[8] - M[12]))) + sixth(M[0] + M[8] + M[12]) -
                             R(cz) * R(0.5) * (M[2] + M[9]));
                } else {
                    if (cz == 0)
                        s = (sixth((-(M[0] - M[12]) + R(2) * (M[8] - M[12]))) + sixth(M[0] + M[8] + M[12]) -
                             R(cy) * R(0.5) * (M[1] + M[11]));
                    else
                        s = (R(cy * cz) * R(0.25) * M[10] + (R(cz) * R(0.25) * M[9] + R(cy) * R(0.25) * M[11]));
                }
            } else {
                if (cy == 0) {
                    if (cz == 0)
                        s = (sixth((R(2) * (M[0] - M[12]) - (M[8] - M[12]))) + sixth(M[0] + M[8] + M[12]) -
                             R(cx) * R(0.5) * (M[4] + M[7]));
                    else
                        s = (R(cx * cz) * R(0.25) * M[6] + (R(cz) * R(0.25) * M[2] + R(cx) * R(0.25) * M[7]));
                } else {
                    if (cz == 0)
                        s = (R(cx * cy) * R(0.25) * M[3] + (R(cy) * R(0.25) * M[1] + R(cx) * R(0.25) * M[4]));
                    else
                        s = (R(cx * cy * cz) * M[5] / R(8));
                }
            }
        } else {
            if (cx == 0) s = cy == 0 ? R(0) : R(-0.25) * (M[0] - M[2]);
            else s = cy == 0 ? R(0.25) * (M[0] - M[2]) : R(0.25) * R(cx * cy) * M[1];
        }
        ds[v] = s;
        const R dh = fneq[v] - s;
        const R feq_true = P::shifted ? fe[v] + R(L::w(v)) * rho0_of<P>(a) : fe[v];
        if constexpr (P::shifted) {
            const R rf = __frcp_rn(feq_true);
            top += s * dh * rf;
            bot += dh * dh * rf;
        } else {
            top += s * dh / feq_true;
            bot += dh * dh / feq_true;
        }
    }
    const R beta_m1 = R(2) / omega_of<P>(a);
    const R gamma = bot == R(0) ? R(2) : beta_m1 - (R(2) - beta_m1) * (top / bot);
    const R inv_b = R(1) / beta_m1;
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        const R dh = fneq[v] - ds[v];
        const R base = src[v] - inv_b * (R(2) * ds[v] + gamma * dh);
        fn[v] = a.forcing ? base + guo<Q, R>(v, omega_of<P>(a), cs2, ux, uy, uz, Fx, Fy, Fz) : base;
    }
}

// _LBM_stream_opt for one listed site.  Per direction (compile-time
// constants) the source's label picks the source: a plain pull, the
// bounce-back of a solid source, the extrapolation two planes back, the
// parent's population at the coarse site (explode), or the equilibrium of
// a velocity source; the rules that need more (coalesce, slip and BFL
// sites) take the full rule, one run-time-indexed copy of the code.  The
// values are those of stream_dir.
template <int Q, class P>
__device__ __forceinline__ void stream_site_split(const StepArgs &a, const int8_t *wall, int i, int j, int k, int id,
                                                  int type, typename P::R *fn) {
    using L = Lattice<Q>;
    using R = typename P::R;
    constexpr int D = L::D;
    const int N = a.N, M = a.M, K = a.K;
    const size_t n = (size_t)a.ncell;
    const bool reg = (a.flags & LUMA_FLAG_REGULARISED) != 0;
    const bool explode = a.parent_f && a.subcycle == 0;
    const bool coalesce = a.nchild && type == LUMA_SITE_TL_TO_FINER;
    // slip sites take the full rule in every direction; at BFL sites (or
    // next to them) only the directions with a BFL link do: the others stream
    // as usual (stream_dir's BFL branch falls through for them)
    const bool generic = type == LUMA_SITE_SLIP;
    uint32_t links = 0xffffffffu;  // without link tables every BFL-touched direction goes to the full rule
    if (a.bfl_rec) {
        const int r = a.bfl_rec[id];
        links = r >= 0 ? a.bfl_mask[r] : 0u;
    }
    const size_t pn = explode ? (size_t)a.pN * a.pM * a.pK : 0;
    unsigned special = generic ? 0xffffffffu : 0u;
    // coalesce (_LBM_coalesce_opt, :591-636, GridUtils::getFineIndices):
    // every direction averages the child's populations at the same 2^d fine
    // sites, so they are found once
    const void *cf = nullptr;
    size_t cn = 0, c0 = 0, cdi = 0, cdj = 0;
    if (coalesce && !generic && !coalesce_base<Q>(a, i, j, k, cf, cn, c0, cdj, cdi)) cf = nullptr;
    // every source's label first, with no branch between the loads: a
    // branch on a label right after its load would serialise the Q loads
    int sidv[Q], stv[Q];
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        int sx = i - L::c(v, 0), sy = j - L::c(v, 1), sz = k - L::c(v, 2);
        sx = sx < 0 ? sx + N : (sx >= N ? sx - N : sx);
        sy = sy < 0 ? sy + M : (sy >= M ? sy - M : sy);
        if (D == 3) sz = sz < 0 ? sz + K : (sz >= K ? sz - K : sz);
        else sz = 0;
        sidv[v] = sz + sy * K + sx * K * M;
        stv[v] = a.typ[sidv[v]];
    }
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        const int sid = sidv[v], st = stv[v];
        if (generic || ((type == LUMA_SITE_BFL || st == LUMA_SITE_BFL) && ((links >> v) & 1u)) ||
            (coalesce && st == LUMA_SITE_REFINED && !cf)) {
            special |= 1u << v;
            fn[v] = R(0);
        } else if (coalesce && st == LUMA_SITE_REFINED) {
            R acc = R(0);
#pragma unroll
            for (int ii = 0; ii < 2; ++ii)
#pragma unroll
                for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                    for (int kk = 0; kk < (D == 3 ? 2 : 1); ++kk)
                        acc += ld<P>(cf, (size_t)v * cn + c0 + (size_t)kk + jj * cdj + ii * cdi);
            fn[v] = acc / (D == 3 ? R(8) : R(4));
        } else if (st == LUMA_SITE_VELOCITY && !reg) {
            fn[v] = velocity_pull<Q, P>(a, j, sid, v);
        } else {
            const void *src = a.f;
            size_t q = (size_t)v * n + sid;
            if (st == LUMA_SITE_SOLID) {
                q = (size_t)L::opp(v) * n + id;
            } else if (st == LUMA_SITE_EXTRAPOLATE_RIGHT) {
                q = (size_t)v * n + (sid - 2 * (K * M));
            } else if (explode && st == LUMA_SITE_TL_TO_COARSER) {
                // GridUtils::getCoarseIndices on the wrapped source (even index down)
                int sx = i - L::c(v, 0), sy = j - L::c(v, 1), sz = D == 3 ? k - L::c(v, 2) : 0;
                sx = sx < 0 ? sx + N : (sx >= N ? sx - N : sx);
                sy = sy < 0 ? sy + M : (sy >= M ? sy - M : sy);
                if (D == 3) sz = sz < 0 ? sz + K : (sz >= K ? sz - K : sz);
                const int pi = (sx >> 1) + a.lims[0], pj = (sy >> 1) + a.lims[2];
                const int pk = D == 3 ? (sz >> 1) + a.lims[4] : 0;
                src = a.parent_f;
                q = (size_t)v * pn + pk + (size_t)pj * a.pK + (size_t)pi * a.pK * a.pM;
            }
            fn[v] = ld<P>(src, q);
        }
    }
    for (unsigned b = special & ((Q == 32 ? 0u : (1u << Q)) - 1u); b; b &= b - 1) {
        const int v = __ffs(b) - 1;
        const R val = stream_dir<Q, P, true>(a, wall, i, j, k, id, type, v);
#pragma unroll
        for (int w = 0; w < Q; ++w)
            if (w == v) fn[w] = val;
    }
}

// Sites phase A leaves alone: velocity/pressure sites of regularised grids
// are phase B's.
__device__ __forceinline__ bool phaseA_skips(const StepArgs &a, int type) {
    const bool reg = (a.flags & LUMA_FLAG_REGULARISED) != 0;
    return type == LUMA_SITE_REFINED || type == LUMA_SITE_SOLID || type == LUMA_SITE_VELOCITY ||
           (reg && type == LUMA_SITE_PRESSURE);
}

// Phase A after the stream: macroscopic step, collision where it belongs
// to phase A, stores.
template <int Q, class P, bool TAV, int COLL = -1>
__device__ __forceinline__ void finish_site(const StepArgs &a, int i, int j, int k, int id, int type,
                                            typename P::R *fn) {
    using R = typename P::R;
    R rho, drho, ux, uy, uz;
    macro_site<Q, P, true, TAV>(a, i, j, k, id, type, fn, rho, drho, ux, uy, uz);
    const size_t n = (size_t)a.ncell;
    if (a.ibm_split && a.defer && !a.defer[id] && type != LUMA_SITE_TL_TO_COARSER) {
        // IBM grid, site outside every support: its force is the reset's zero,
        // so its second-loop collision happens here (fOut != fNew keeps the
        // streamed values in fNew as well)
        if (a.fOut != a.fNew) {
#pragma unroll
            for (int v = 0; v < Q; ++v) st<P>(a.fNew, (size_t)v * n + id, fn[v]);
        }
        collide_site<Q, P, COLL>(a, id, fn, rho, drho, ux, uy, uz);
#pragma unroll
        for (int v = 0; v < Q; ++v) st<P>(a.fOut, (size_t)v * n + id, fn[v]);
        return;
    }
    if (!a.ibm_split && type != LUMA_SITE_TL_TO_COARSER) collide_site<Q, P, COLL>(a, id, fn, rho, drho, ux, uy, uz);
#pragma unroll
    for (int v = 0; v < Q; ++v) st<P>(a.fNew, (size_t)v * n + id, fn[v]);
}

template <int Q, class P, bool TAV>
__device__ __forceinline__ void stream_macro_site(const StepArgs &a, const int8_t *wall, int id) {
    using R = typename P::R;
    const int type = a.typ[id];
    if (phaseA_skips(a, type)) return;
    const int k = id % a.K;
    const int j = (id / a.K) % a.M;
    const int i = id / (a.K * a.M);
    R fn[Q];
    stream_site_split<Q, P>(a, wall, i, j, k, id, type, fn);
    finish_site<Q, P, TAV>(a, i, j, k, id, type, fn);
}

template <int Q, class P, bool TAV>
__global__ void __launch_bounds__(128) k_stream_macro(StepArgs a, const int8_t *wall) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id < a.ncell) stream_macro_site<Q, P, TAV>(a, wall, id);
}

// The same over the listed sites (those the interior kernel leaves), one
// thread per site, the collision operator fixed at compile time and the
// stream split into plain pulls and flagged rules (short code: the
// full-logic kernel's instruction fetch, not its loads, bounded it).
template <int Q, class P, int COLL, bool TAV>
__global__ void __launch_bounds__(128) k_stream_macro_list(StepArgs a, const int8_t *wall, const int *ids, int nids) {
    using R = typename P::R;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nids) return;
    const int id = ids[t];
    const int type = a.typ[id];
    if (phaseA_skips(a, type)) return;
    const int k = id % a.K, j = (id / a.K) % a.M, i = id / (a.K * a.M);
    R fn[Q];
    stream_site_split<Q, P>(a, wall, i, j, k, id, type, fn);
    finish_site<Q, P, TAV, COLL>(a, i, j, k, id, type, fn);
}

// The same for a short list of coalescing sites (transition sites to finer
// grids, after the sub-grids' steps), direction-parallel: a block takes
// 128/Q sites, one thread per (site, direction) streams one population into
// shared memory (a coalesce's 2^d loads per thread, every direction's in
// flight at once), then one thread per site finishes it.
template <int Q>
constexpr int late_sites() { return 128 / Q; }

template <int Q, class P, int COLL, bool TAV>
__global__ void __launch_bounds__(128) k_stream_macro_late(StepArgs a, const int8_t *wall, const int *ids, int nids) {
    using R = typename P::R;
    constexpr int S = late_sites<Q>();
    __shared__ R fs[S * Q];
    const int t = threadIdx.x;
    const int s = t / Q, v = t - s * Q;
    const int idx = blockIdx.x * S + s;
    if (s < S && idx < nids) {
        const int id = ids[idx];
        const int type = a.typ[id];
        if (!phaseA_skips(a, type)) {
            const int k = id % a.K, j = (id / a.K) % a.M, i = id / (a.K * a.M);
            fs[t] = stream_dir<Q, P, true>(a, wall, i, j, k, id, type, v);
        }
    }
    __syncthreads();
    if (t >= S) return;
    const int idx2 = blockIdx.x * S + t;
    if (idx2 >= nids) return;
    const int id = ids[idx2];
    const int type = a.typ[id];
    if (phaseA_skips(a, type)) return;
    const int k = id % a.K, j = (id / a.K) % a.M, i = id / (a.K * a.M);
    R fn[Q];
#pragma unroll
    for (int w = 0; w < Q; ++w) fn[w] = fs[t * Q + w];
    finish_site<Q, P, TAV, COLL>(a, i, j, k, id, type, fn);
}

// Interior fluid sites (every pull source a fluid site, so every direction
// is a plain pull): stream, macroscopic and collision of the same operators
// as stream_macro_site with the branches resolved at compile time, for a
// lean register budget and all Q loads in flight at once.  Under the IBM
// split, deferred sites stop after the macroscopic step (phase C collides
// them); the others carry the reset's zero force, whose Guo term and half
// force add exact zeros, so their force is not read.
template <int Q, class P, int COLL, bool TAV>
__global__ void __launch_bounds__(128) k_interior(StepArgs a, const uint8_t *fast) {
    using L = Lattice<Q>;
    using R = typename P::R;
    constexpr int D = L::D;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= a.ncell || !fast[id]) return;
    const int N = a.N, M = a.M, K = a.K;
    const int k = id % K, j = (id / K) % M, i = id / (K * M);
    const size_t n = (size_t)a.ncell;
    R fn[Q];
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        int sx = i - L::c(v, 0), sy = j - L::c(v, 1), sz = k - L::c(v, 2);
        sx = sx < 0 ? sx + N : (sx >= N ? sx - N : sx);
        sy = sy < 0 ? sy + M : (sy >= M ? sy - M : sy);
        if (D == 3) sz = sz < 0 ? sz + K : (sz >= K ? sz - K : sz);
        else sz = 0;
        fn[v] = ld<P>(a.f, (size_t)v * n + (sz + sy * K + sx * K * M));
    }
    const bool deferred = a.ibm_split && (!a.defer || a.defer[id]);
    StepArgs b = a;
    if (a.ibm_split && !deferred) b.forcing = 0;  // zero force: exact same sums
    R rho, drho, ux, uy, uz;
    // u and rho go to memory where something reads them later in the step
    // or after it (macro_out) or the IBM pass needs them (deferred sites)
    if (a.macro_out || deferred) macro_site<Q, P, true, TAV>(b, i, j, k, id, LUMA_SITE_FLUID, fn, rho, drho, ux, uy, uz);
    else macro_site<Q, P, false, TAV>(b, i, j, k, id, LUMA_SITE_FLUID, fn, rho, drho, ux, uy, uz);
    if (deferred || (a.ibm_split && a.fOut != a.fNew)) {
#pragma unroll
        for (int v = 0; v < Q; ++v) st<P>(a.fNew, (size_t)v * n + id, fn[v]);
        if (deferred) return;
    }
    if constexpr (!P::shifted && COLL == LUMA_COLL_BGK) {
        // FP64 BGK with the constants of cs^2 = 1/3 written out (3, 4.5,
        // 1.5) instead of the reference's divisions by cs^2: FP64 division
        // is the costliest operation of the step on this part, and the
        // results differ from the reference's expression by rounding only.
        const R om = omega_of<P>(a);
        const R usq15 = R(1.5) * (ux * ux + uy * uy + uz * uz);
        R Fx = R(0), Fy = R(0), Fz = R(0);
        if (b.forcing) {
            Fx = ldr<P>(a.force, id);
            Fy = ldr<P>(a.force, n + id);
            if (D == 3) Fz = ldr<P>(a.force, 2 * n + id);
        }
        const R g3 = R(3) * (R(1) - R(0.5) * om);
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            const R c0 = R(L::c(v, 0)), c1 = R(L::c(v, 1)), c2 = R(L::c(v, 2));
            const R cu = c0 * ux + c1 * uy + (D == 3 ? c2 * uz : R(0));
            const R w = R(L::w(v));
            const R eq = w * rho * (R(1) + R(3) * cu + R(4.5) * cu * cu - usq15);
            R f = fn[v] + om * (eq - fn[v]);
            if (b.forcing) {
                const R b1 = R(1) + R(3) * cu;
                R s = Fx * (c0 * b1 - ux) + Fy * (c1 * b1 - uy);
                if (D == 3) s += Fz * (c2 * b1 - uz);
                f += w * (g3 * s);
            }
            fn[v] = f;
        }
    } else {
        collide_site<Q, P, COLL>(b, id, fn, rho, drho, ux, uy, uz);
    }
    void *out = a.ibm_split ? a.fOut : a.fNew;
#pragma unroll
    for (int v = 0; v < Q; ++v) st<P>(out, (size_t)v * n + id, fn[v]);
}

// _LBM_regularised_opt (:313-510) for one velocity/pressure site of a
// regularised grid, preceded by its stream and followed (single-loop
// reference) by its collision.  Interior macroscopic values used for
// extrapolation come from phase A.
template <int Q, class P>
__global__ void __launch_bounds__(128) k_regularised(StepArgs a, const int8_t *wall, const RegSite *sites, int nsites) {
    using L = Lattice<Q>;
    using R = typename P::R;
    constexpr int D = L::D;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsites) return;
    const RegSite rs = sites[s];
    const int id = rs.id, i = rs.i, j = rs.j, k = rs.k;
    const int type = a.typ[id];
    const size_t n = (size_t)a.ncell;
    const R cs2 = cs2_of<P>(a);
    R fn[Q];
    stream_site_split<Q, P>(a, wall, i, j, k, id, type, fn);
    R vel[3] = {R(a.ux_in[j] * a.ramp_reg), R(a.uy_in[j] * a.ramp_reg), R(a.uz_in[j] * a.ramp_reg)};
    const int nd = rs.ndir;
    const int nv[3] = {rs.nvec[0], rs.nvec[1], rs.nvec[2]};
    R dens = rho0_of<P>(a) + R(a.pdelta);
    R drho;
    if (rs.edges > 1) {
        // First-order extrapolation of rho along the inward normal.
        const int i1 = i + nv[0], j1 = j + nv[1], k1 = k + nv[2];
        const int i2 = i1 + nv[0], j2 = j1 + nv[1], k2 = k1 + nv[2];
        const int id1 = k1 + j1 * a.K + i1 * a.K * a.M;
        const int id2 = k2 + j2 * a.K + i2 * a.K * a.M;
        dens = R(2) * ldr<P>(a.rho, id1) - ldr<P>(a.rho, id2);
        drho = dens - rho0_of<P>(a);
    } else {
        R fp = R(0), f0 = R(0);
        R wp = R(0), w0 = R(0);
#pragma unroll
        for (int v = 0; v < Q; ++v) {
            const int cn = nd == 0 ? L::c(v, 0) : (nd == 1 ? L::c(v, 1) : L::c(v, 2));
            if (cn == -nv[nd]) { fp += fn[v]; wp += R(L::w(v)); }
            else if (cn == 0) { f0 += fn[v]; w0 += R(L::w(v)); }
        }
        if (P::shifted) {
            // On a face the weights satisfy 2*sum(w_plus) + sum(w_zero) = 1, so
            // 2 f+ + f0 = rho0 + (2 g+ + g0): work with the small shifted sum X
            // and the density offset directly, as the unshifted formulas would
            // lose it to cancellation in FP32.
            (void)wp;
            (void)w0;
            const R X = R(2) * fp + f0;
            if (type == LUMA_SITE_PRESSURE) {
                for (int d = 0; d < D; d++)
                    if (d != nd) {
                        const int i1 = i + nv[0], j1 = j + nv[1], k1 = k + nv[2];
                        const int i2 = i1 + nv[0], j2 = j1 + nv[1], k2 = k1 + nv[2];
                        const int id1 = k1 + j1 * a.K + i1 * a.K * a.M;
                        const int id2 = k2 + j2 * a.K + i2 * a.K * a.M;
                        vel[d] = R(2) * ldr<P>(a.u, (size_t)d * n + id1) - ldr<P>(a.u, (size_t)d * n + id2);
                    }
                drho = R(a.pdelta);
                // u_n = 1 - (rho0 + X)/dens = (drho - X)/dens
                vel[nd] = (drho - X) / dens;
                if (nv[nd] == -1) vel[nd] *= R(-1);
            } else {
                R nvel = vel[nd];
                if (nv[nd] == -1) nvel *= R(-1);
                // dens = (rho0 + X)/(1 - un)  =>  dens - rho0 = (X + rho0*un)/(1 - un)
                drho = (X + rho0_of<P>(a) * nvel) / (R(1) - nvel);
                dens = rho0_of<P>(a) + drho;
            }
        } else if (type == LUMA_SITE_PRESSURE) {
            for (int d = 0; d < D; d++)
                if (d != nd) {
                    const int i1 = i + nv[0], j1 = j + nv[1], k1 = k + nv[2];
                    const int i2 = i1 + nv[0], j2 = j1 + nv[1], k2 = k1 + nv[2];
                    const int id1 = k1 + j1 * a.K + i1 * a.K * a.M;
                    const int id2 = k2 + j2 * a.K + i2 * a.K * a.M;
                    vel[d] = R(2) * ldr<P>(a.u, (size_t)d * n + id1) - ldr<P>(a.u, (size_t)d * n + id2);
                }
            vel[nd] = R(1) - ((R(1) / dens) * (R(2) * fp + f0));
            if (nv[nd] == -1) vel[nd] *= R(-1);
        } else {
            R nvel = vel[nd];
            if (nv[nd] == -1) nvel *= R(-1);
            dens = (R(1) / (R(1) - nvel)) * (R(2) * fp + f0);
        }
        if (!P::shifted) drho = dens - rho0_of<P>(a);
    }
    const R ux = vel[0], uy = vel[1], uz = D == 3 ? vel[2] : R(0);
    str<P>(a.rho, id, dens);
    str<P>(a.u, id, ux);
    str<P>(a.u, n + id, uy);
    if (D == 3) str<P>(a.u, 2 * n + id, uz);
    R Sxx = 0, Syy = 0, Sxy = 0, Szz = 0, Sxz = 0, Syz = 0;
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        const int c0 = L::c(v, 0), c1 = L::c(v, 1), c2 = L::c(v, 2);
        const int cn = nd == 0 ? c0 : (nd == 1 ? c1 : c2);
        const R eqv = feq_s<Q, P>(v, dens, drho, ux, uy, uz, cs2);
        if (rs.edges == 1 && cn == nv[nd]) {
            fn[v] = eqv + (fn[L::opp(v)] - feq_s<Q, P>(L::opp(v), dens, drho, ux, uy, uz, cs2));
        } else if (rs.edges > 1 && (c0 == nv[0] || c1 == nv[1] || (D == 3 && c2 == nv[2]))) {
            const int dp = c0 * nv[0] + c1 * nv[1] + (D == 3 ? c2 * nv[2] : 0);
            const int mag2 = c0 * c0 + c1 * c1 + (D == 3 ? c2 * c2 : 0);
            if (dp == 0 && mag2 > 1) fn[v] = eqv;
            else fn[v] = eqv + (fn[L::opp(v)] - feq_s<Q, P>(L::opp(v), dens, drho, ux, uy, uz, cs2));
        }
        const R fneq = fn[v] - eqv;
        Sxx += R(c0 * c0) * fneq;
        Syy += R(c1 * c1) * fneq;
        Sxy += R(c0 * c1) * fneq;
        if (D == 3) {
            Szz += R(c2 * c2) * fneq;
            Sxz += R(c0 * c2) * fneq;
            Syz += R(c1 * c2) * fneq;
        }
    }
#pragma unroll
    for (int v = 0; v < Q; v++) {
        const int c0 = L::c(v, 0), c1 = L::c(v, 1), c2 = L::c(v, 2);
        if constexpr (P::shifted) {
            // w/(2 cs^4) (c_a c_b - cs^2 delta_ab) S_ab with cs^2 = 1/3 and integer coefficients
            fn[v] = feq_s<Q, P>(v, dens, drho, ux, uy, uz, cs2) +
                    wmul<Q>(v, R(1.5) * (R(3 * c0 * c0 - 1) * Sxx + R(3 * c1 * c1 - 1) * Syy +
                                         R(3 * c2 * c2 - 1) * Szz + R(6 * c0 * c1) * Sxy + R(6 * c0 * c2) * Sxz +
                                         R(6 * c1 * c2) * Syz));
        } else {
            fn[v] = feq_s<Q, P>(v, dens, drho, ux, uy, uz, cs2) +
                    (R(L::w(v)) / (R(2) * cs2 * cs2)) *
                        (((R(c0 * c0) - cs2) * Sxx) + ((R(c1 * c1) - cs2) * Syy) + ((R(c2 * c2) - cs2) * Szz) +
                         (R(2 * c0 * c1) * Sxy) + (R(2 * c0 * c2) * Sxz) + (R(2 * c1 * c2) * Syz));
        }
    }
    if (!a.ibm_split) collide_site<Q, P>(a, id, fn, dens, drho, ux, uy, uz);
#pragma unroll
    for (int v = 0; v < Q; ++v) st<P>(a.fNew, (size_t)v * n + id, fn[v]);
}

// The velocity that the forced-equilibrium BC leaves in a velocity site's u
// under a velocity ramp: the inlet value of the row of the last site (in the
// reference's loop order) that pulled from it (:258-265).
template <class P>
__global__ void k_velocity_u(StepArgs a, int dims, const int2 *sites, int nsites) {
    using R = typename P::R;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsites) return;
    const int2 e = sites[s];  // (site id, row of its last writer)
    const size_t n = (size_t)a.ncell;
    str<P>(a.u, e.x, R(a.ux_in[e.y] * a.ramp_stream));
    str<P>(a.u, n + e.x, R(a.uy_in[e.y] * a.ramp_stream));
    if (dims == 3) str<P>(a.u, 2 * n + e.x, R(a.uz_in[e.y] * a.ramp_stream));
}

// Second loop of the reference under L_IBM_ON (:125-156): forcing at every
// non-solid site and collision at every site but transition-to-coarser,
// using the macroscopic values after the IBM pass.
template <int Q, class P>
__device__ __forceinline__ void force_collide_site(const StepArgs &a, int id) {
    using R = typename P::R;
    constexpr int D = Lattice<Q>::D;
    const int type = a.typ[id];
    if (type == LUMA_SITE_TL_TO_COARSER) return;
    const size_t n = (size_t)a.ncell;
    R fn[Q];
#pragma unroll
    for (int v = 0; v < Q; ++v) fn[v] = ld<P>(a.fNew, (size_t)v * n + id);
    const R rho = ldr<P>(a.rho, id);
    const R ux = ldr<P>(a.u, id), uy = ldr<P>(a.u, n + id);
    const R uz = D == 3 ? ldr<P>(a.u, 2 * n + id) : R(0);
    StepArgs b = a;
    if (type == LUMA_SITE_SOLID) b.forcing = 0;  // solid sites are collided without the Guo term
    collide_site<Q, P>(b, id, fn, rho, rho - rho0_of<P>(a), ux, uy, uz);
#pragma unroll
    for (int v = 0; v < Q; ++v) st<P>(a.fOut, (size_t)v * n + id, fn[v]);
}

template <int Q, class P>
__global__ void __launch_bounds__(128) k_force_collide(StepArgs a) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id < a.ncell) force_collide_site<Q, P>(a, id);
}

// The same over the listed sites only (the sites phase A left uncollided).
template <int Q, class P>
__global__ void __launch_bounds__(128) k_force_collide_list(StepArgs a, const int *ids, int nids) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nids) force_collide_site<Q, P>(a, ids[t]);
}

// ---- immersed boundary pass (ObjectManager::ibm_apply, src/ObjectManager_ops_ibm.cpp:33-54) ----

// ibm_interpolate (:498-591) + ibm_computeForce (:598-614) for 32 markers
// per block.  GB300 runs an FP64 instruction of a warp in 64 cycles of its
// SM sub-partition whatever the number of active lanes, so the kernel keeps
// every FP64 instruction dense: each warp forms the products of 8 markers
// with its lanes over a marker's supports (each term rs*dl*A and rs*u*dl*A
// rounded as the reference rounds it, no fused multiply-add) and parks them
// in shared memory; then warp q sums quantity q (rho, then each momentum
// component) for the 32 markers, lane = marker, in support order, so the
// sums are the reference's FP64 sums.  Supports beyond 32 per marker come
// in further rounds of the same two phases.
constexpr int kInterpMarkers = 32;

template <int Q, class P>
__global__ void __launch_bounds__(128) k_ibm_interp_force(StepArgs a, IbmArgs b) {
    if (a.skip && *a.skip) return;  // a converged FSI loop: later sub-iterations do nothing
    constexpr int D = Lattice<Q>::D;
    __shared__ double prod[kInterpMarkers][32][4];
    __shared__ double sums[4][kInterpMarkers];
    __shared__ int rounds;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int m0 = blockIdx.x * kInterpMarkers;
    const size_t n = (size_t)a.ncell;
    if (threadIdx.x < 32) {
        const int m = m0 + lane;
        const int cnt = m < b.nm ? b.moff[m + 1] - b.moff[m] : 0;
        int mx = cnt;
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) rounds = (mx + 31) / 32;
    }
    __syncthreads();
    double acc = 0.0;  // quantity w of marker m0 + lane
    for (int r = 0; r < rounds; ++r) {
#pragma unroll 2
        for (int i = 0; i < kInterpMarkers / 4; ++i) {
            const int ml = (kInterpMarkers / 4) * w + i, m = m0 + ml;
            if (m >= b.nm) break;
            const int s = b.moff[m] + 32 * r + lane;
            if (s < b.moff[m + 1]) {
                const int id = b.msite[s];
                const double rs = double(ldr<P>(a.rho, id));
                const double dl = b.mdelta[s];
                const double A = b.area[m];
                prod[ml][lane][0] = __dmul_rn(__dmul_rn(rs, dl), A);
                for (int d = 0; d < D; ++d)
                    prod[ml][lane][1 + d] = __dmul_rn(__dmul_rn(__dmul_rn(rs, double(ldr<P>(a.u, (size_t)d * n + id))), dl), A);
            }
        }
        __syncthreads();
        const int m = m0 + lane;
        if (w <= D && m < b.nm) {
            const int cnt = b.moff[m + 1] - b.moff[m] - 32 * r;
            for (int t = 0; t < (cnt < 32 ? cnt : 32); ++t) acc = __dadd_rn(acc, prod[lane][t][w]);
        }
        __syncthreads();
    }
    if (w <= D) sums[w][lane] = acc;
    __syncthreads();
    const int m = m0 + lane;
    if (w != 0 || m >= b.nm) return;
    const double rsum = sums[0][lane];
    b.irho[m] = rsum;
    for (int d = 0; d < D; ++d) {
        const double mom = sums[1 + d][lane];
        b.imom[3 * m + d] = mom;
        b.F[3 * m + d] = 2.0 * (mom - rsum * b.vel[3 * m + d]) / 1.0;
    }
    if (a.ibm_f_out)
        for (int d = 0; d < 3; ++d) a.ibm_f_out[3 * m + d] = b.F[3 * m + d];
    if (a.ibm_drag_out && m >= a.ibm_drag_base && m < a.ibm_drag_base + a.ibm_drag_nm)
        a.ibm_drag_out[m - a.ibm_drag_base] = b.F[3 * m] * a.ibm_drag_w[m];
}

// ibm_spread (:621-689) as a gather: one thread per distinct support site
// applies every (marker, support) contribution to it in the reference's
// (body, marker, support) order, so no atomics and a deterministic sum.
template <int Q, class P>
__global__ void k_ibm_spread(StepArgs a, IbmArgs b) {
    if (a.skip && *a.skip) return;  // a converged FSI loop: later sub-iterations do nothing
    constexpr int D = Lattice<Q>::D;
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= b.nu) return;
    const size_t n = (size_t)a.ncell;
    const int id = b.usite[u];
    double f[3];
    for (int d = 0; d < D; ++d) f[d] = double(ldr<P>(a.force, (size_t)d * n + id));
    for (int q = b.uoff[u]; q < b.uoff[u + 1]; ++q) {
        const int s = b.uref[q];
        const int m = b.smarker[s];
        const double volWidth = b.eps[m];
        const double volDepth = D == 3 ? b.ds[m] : 1.0;
        for (int d = 0; d < D; ++d) f[d] -= b.mdelta[s] * b.F[3 * m + d] * volWidth * volDepth * b.ds[m];
    }
    for (int d = 0; d < D; ++d) str<P>(const_cast<void *>(a.force), (size_t)d * n + id, typename P::R(f[d]));
    if (a.ibm_sf_out)
        for (int d = 0; d < D; ++d) static_cast<typename P::R *>(a.ibm_sf_out)[(size_t)d * b.nu + u] = typename P::R(f[d]);
}

// ibm_updateMacroscopic (:696-766): the macroscopic step again at every
// support site, now with the spread force.
template <int Q, class P>
__global__ void k_ibm_remacro(StepArgs a, IbmArgs b) {
    if (a.skip && *a.skip) return;  // a converged FSI loop: later sub-iterations do nothing
    using R = typename P::R;
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= b.nu) return;
    const size_t n = (size_t)a.ncell;
    const int id = b.usite[u];
    const int k = id % a.K, j = (id / a.K) % a.M, i = id / (a.K * a.M);
    const int type = a.typ[id];
    R fn[Q];
#pragma unroll
    for (int v = 0; v < Q; ++v) fn[v] = ld<P>(a.fNew, (size_t)v * n + id);
    R rho, drho, ux, uy, uz;
    // ibm_updateMacroscopic (:696-766) re-runs the macroscopic step once per
    // (marker, support) pair: the running means see each repetition
    macro_site<Q, P>(a, i, j, k, id, type, fn, rho, drho, ux, uy, uz, b.uoff[u + 1] - b.uoff[u]);
}

// _LBM_resetForces (:1327-1337): zero the force field, or, under gravity,
// set only the gravity component to rho*g*refinement_ratio (the other
// components keep their values, as in the reference).
template <class P>
__global__ void k_reset_forces(StepArgs a, int dims, double gravity, int gdir, double rr) {
    if (a.skip && *a.skip) return;  // a converged FSI loop: later sub-iterations do nothing
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)a.ncell) return;
    const size_t n = (size_t)a.ncell;
    if (a.flags & LUMA_FLAG_GRAVITY) {
        str<P>(const_cast<void *>(a.force), (size_t)gdir * n + id,
               typename P::R(double(ldr<P>(a.rho, id)) * gravity * rr));
    } else {
        for (int d = 0; d < dims; ++d) str<P>(const_cast<void *>(a.force), (size_t)d * n + id, typename P::R(0));
    }
}

// ---- flexible (moving) markers: fixed-capacity supports, atomic spread ----

template <int Q, class P>
__global__ void k_flex_interp_force(StepArgs a, FlexArgs f) {
    if (a.skip && *a.skip) return;  // a converged FSI loop: later sub-iterations do nothing
    constexpr int D = Lattice<Q>::D;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= f.nm) return;
    const size_t n = (size_t)a.ncell;
    double r = 0.0, mom[3] = {0.0, 0.0, 0.0};
    for (int s = 0; s < f.nsupp[m]; ++s) {
        const int id = f.supp[m * kFlexMaxSupp + s];
        const double rs = double(ldr<P>(a.rho, id));
        const double dl = f.delta[m * kFlexMaxSupp + s];
        r += rs * dl * 1.0;
        for (int d = 0; d < D; ++d) mom[d] += rs * double(ldr<P>(a.u, (size_t)d * n + id)) * dl * 1.0;
    }
    f.irho[m] = r;
    for (int d = 0; d < D; ++d) {
        f.imom[3 * m + d] = mom[d];
        f.F[3 * m + d] = 2.0 * (mom[d] - r * f.vel[3 * m + d]) / 1.0;
    }
}

// Spread of moving markers: supports change every FSI iteration, so the
// contributions are added with atomics (summation order differs from the
// reference's serial loop at the level of FP64 rounding).
template <int Q, class P>
__global__ void k_flex_spread(StepArgs a, FlexArgs f) {
    if (a.skip && *a.skip) return;  // a converged FSI loop: later sub-iterations do nothing
    constexpr int D = Lattice<Q>::D;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = t / kFlexMaxSupp, s = t % kFlexMaxSupp;
    if (m >= f.nm || s >= f.nsupp[m]) return;
    const size_t n = (size_t)a.ncell;
    const int id = f.supp[m * kFlexMaxSupp + s];
    const double volDepth = D == 3 ? f.ds[m] : 1.0;
    for (int d = 0; d < D; ++d) {
        const double c = f.delta[m * kFlexMaxSupp + s] * f.F[3 * m + d] * f.eps[m] * volDepth * f.ds[m];
        atomicAdd(static_cast<typename P::R *>(const_cast<void *>(a.force)) + (size_t)d * n + id,
                  typename P::R(-c));
    }
}

template <int Q, class P>
__global__ void k_flex_remacro(StepArgs a, FlexArgs f) {
    if (a.skip && *a.skip) return;  // a converged FSI loop: later sub-iterations do nothing
    using R = typename P::R;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = t / kFlexMaxSupp, s = t % kFlexMaxSupp;
    if (m >= f.nm || s >= f.nsupp[m]) return;
    const size_t n = (size_t)a.ncell;
    const int id = f.supp[m * kFlexMaxSupp + s];
    const int k = id % a.K, j = (id / a.K) % a.M, i = id / (a.K * a.M);
    R fn[Q];
#pragma unroll
    for (int v = 0; v < Q; ++v) fn[v] = ld<P>(a.fNew, (size_t)v * n + id);
    R rho, drho, ux, uy, uz;
    macro_site<Q, P>(a, i, j, k, id, a.typ[id], fn, rho, drho, ux, uy, uz);
}

}  // namespace

// The four passes of ibm_apply, each over every body of the grid: rigid
// bodies (ordered gather) and flexible markers (fixed slots, atomics).
template <int Q, class P>
cudaError_t launch_ibm_pass(const StepArgs &a, const IbmArgs &b, const FlexArgs &f, cudaStream_t s) {
    const int nt = f.nm * kFlexMaxSupp;
    if (b.nm > 0) k_ibm_interp_force<Q, P><<<(b.nm + kInterpMarkers - 1) / kInterpMarkers, 128, 0, s>>>(a, b);
    if (f.nm > 0) k_flex_interp_force<Q, P><<<(f.nm + 127) / 128, 128, 0, s>>>(a, f);
    if (b.nm > 0) k_ibm_spread<Q, P><<<(b.nu + 127) / 128, 128, 0, s>>>(a, b);
    if (f.nm > 0) k_flex_spread<Q, P><<<(nt + 127) / 128, 128, 0, s>>>(a, f);
    if (b.nm > 0) k_ibm_remacro<Q, P><<<(b.nu + 127) / 128, 128, 0, s>>>(a, b);
    if (f.nm > 0) k_flex_remacro<Q, P><<<(nt + 127) / 128, 128, 0, s>>>(a, f);
    return cudaGetLastError();
}
template <class P>
cudaError_t launch_reset_forces(const StepArgs &a, int dims, double gravity, int gdir, double rr, cudaStream_t s) {
    k_reset_forces<P><<<(a.ncell + 255) / 256, 256, 0, s>>>(a, dims, gravity, gdir, rr);
    return cudaGetLastError();
}

template <int Q, class P>
cudaError_t launch_general_phaseA(const StepArgs &a, const int8_t *wall, const uint8_t *fast, const int *gen_ids,
                                  int ngen, cudaStream_t s, int part) {
    const int bs = 128;
    const bool tav = a.tav_rho != nullptr;
    if (!fast) {
        if (tav) k_stream_macro<Q, P, true><<<(a.ncell + bs - 1) / bs, bs, 0, s>>>(a, wall);
        else k_stream_macro<Q, P, false><<<(a.ncell + bs - 1) / bs, bs, 0, s>>>(a, wall);
        return cudaGetLastError();
    }
    const int nb = (a.ncell + bs - 1) / bs;
    auto interior = [&](auto tv) {
        constexpr bool T = decltype(tv)::value;
        if (part != kPhaseAList && part != kPhaseALate) {
            if (a.collision == LUMA_COLL_KBC) k_interior<Q, P, LUMA_COLL_KBC, T><<<nb, bs, 0, s>>>(a, fast);
            else if (a.collision == LUMA_COLL_BGK_SMAG) k_interior<Q, P, LUMA_COLL_BGK_SMAG, T><<<nb, bs, 0, s>>>(a, fast);
            else k_interior<Q, P, LUMA_COLL_BGK, T><<<nb, bs, 0, s>>>(a, fast);
        }
        if (part == kPhaseALate) {
            if (ngen > 0) {
                const int lb = (ngen + late_sites<Q>() - 1) / late_sites<Q>();
                if (a.collision == LUMA_COLL_KBC)
                    k_stream_macro_late<Q, P, LUMA_COLL_KBC, T><<<lb, bs, 0, s>>>(a, wall, gen_ids, ngen);
                else if (a.collision == LUMA_COLL_BGK_SMAG)
                    k_stream_macro_late<Q, P, LUMA_COLL_BGK_SMAG, T><<<lb, bs, 0, s>>>(a, wall, gen_ids, ngen);
                else k_stream_macro_late<Q, P, LUMA_COLL_BGK, T><<<lb, bs, 0, s>>>(a, wall, gen_ids, ngen);
            }
            return;
        }
        if (part != kPhaseAInterior && ngen > 0) {
            // a list shorter than one 128-thread block per SM goes in 32-thread
            // blocks: its sites' scattered loads (coalesce: 2^d per direction)
            // then spread over every SM instead of queueing on a few
            const int lbs = ngen < kSMs * bs ? 32 : bs;
            const int lb = (ngen + lbs - 1) / lbs;
            if (a.collision == LUMA_COLL_KBC)
                k_stream_macro_list<Q, P, LUMA_COLL_KBC, T><<<lb, lbs, 0, s>>>(a, wall, gen_ids, ngen);
            else if (a.collision == LUMA_COLL_BGK_SMAG)
                k_stream_macro_list<Q, P, LUMA_COLL_BGK_SMAG, T><<<lb, lbs, 0, s>>>(a, wall, gen_ids, ngen);
            else k_stream_macro_list<Q, P, LUMA_COLL_BGK, T><<<lb, lbs, 0, s>>>(a, wall, gen_ids, ngen);
        }
    };
    if (tav) interior(std::true_type{});
    else interior(std::false_type{});
    return cudaGetLastError();
}
template <int Q, class P>
cudaError_t launch_general_phaseB(const StepArgs &a, const int8_t *wall, const RegSite *sites, int nsites,
                                  cudaStream_t s) {
    if (nsites <= 0) return cudaSuccess;
    const int bs = 128;
    k_regularised<Q, P><<<(nsites + bs - 1) / bs, bs, 0, s>>>(a, wall, sites, nsites);
    return cudaGetLastError();
}
template <class P>
cudaError_t launch_velocity_u(const StepArgs &a, int dims, const int2 *sites, int nsites, cudaStream_t s) {
    if (nsites <= 0) return cudaSuccess;
    k_velocity_u<P><<<(nsites + 127) / 128, 128, 0, s>>>(a, dims, sites, nsites);
    return cudaGetLastError();
}
template <int Q, class P>
cudaError_t launch_general_phaseC(const StepArgs &a, const int *ids, int nids, cudaStream_t s) {
    const int bs = 128;
    if (ids) {
        if (nids > 0) k_force_collide_list<Q, P><<<(nids + bs - 1) / bs, bs, 0, s>>>(a, ids, nids);
    } else {
        k_force_collide<Q, P><<<(a.ncell + bs - 1) / bs, bs, 0, s>>>(a);
    }
    return cudaGetLastError();
}

#define LUMA_INST(Q, P)                                                                                        \
    template cudaError_t launch_general_phaseA<Q, P>(const StepArgs &, const int8_t *, const uint8_t *, const int *, \
                                                     int, cudaStream_t, int);                                  \
    template cudaError_t launch_general_phaseB<Q, P>(const StepArgs &, const int8_t *, const RegSite *, int,   \
                                                     cudaStream_t);                                            \
    template cudaError_t launch_general_phaseC<Q, P>(const StepArgs &, const int *, int, cudaStream_t);
#define LUMA_INST_IBM(Q, P) \
    template cudaError_t launch_ibm_pass<Q, P>(const StepArgs &, const IbmArgs &, const FlexArgs &, cudaStream_t);

// This unit is compiled once per (lattice, precision) pair, with
// -DLUMA_GEN_Q=<9|19|27> -DLUMA_GEN_FP64=<0|1> (luma_gb300/build.py), so
// the six sets of instantiations build in parallel; the lattice-free
// launchers come with the D2Q9 objects.
#if !defined(LUMA_GEN_Q) || !defined(LUMA_GEN_FP64)
#error "k_general.cu is compiled per lattice and precision: define LUMA_GEN_Q and LUMA_GEN_FP64"
#endif
#if LUMA_GEN_FP64
#define LUMA_GEN_P P64
#else
#define LUMA_GEN_P P32
#endif
LUMA_INST(LUMA_GEN_Q, LUMA_GEN_P)
LUMA_INST_IBM(LUMA_GEN_Q, LUMA_GEN_P)
#if LUMA_GEN_Q == 9
template cudaError_t launch_reset_forces<LUMA_GEN_P>(const StepArgs &, int, double, int, double, cudaStream_t);
template cudaError_t launch_velocity_u<LUMA_GEN_P>(const StepArgs &, int, const int2 *, int, cudaStream_t);
#endif

}  // namespace luma
