// Device-side grid state, precision policies and the per-site physics shared
// by the LBM kernels.
//
// Populations live on the device as structure-of-arrays, f[v*ncell + id],
// with the reference's site index id = k + j*K + i*K*M (z fastest; LUMA
// src/GridObj_ops_lbm_optimised.cpp:79), so consecutive threads touch
// consecutive addresses for every direction.  Macroscopic fields are SoA too
// (u[d*ncell + id]).
//
// Two precision policies:
//  * P64: FP64 storage and arithmetic (the reference's arithmetic);
//  * P32: shifted FP32 storage g_i = f_i - w_i*rho0 with FP32 arithmetic.
//    Every operation of the step is linear in the populations with weights
//    that respect w_i = w_opp(i), so it acts on g exactly as on f once the
//    equilibrium is shifted the same way: g_eq_i = w_i*(rho - rho0) +
//    w_i*rho*(c_i.u/cs^2 + ...).  Keeping rho - rho0 = sum_i g_i as the
//    primary density variable removes the O(1) offset that costs FP32
//    populations their significant bits.
#pragma once

#include <cstdint>

#include "lattice.cuh"
#include "../../include/luma_gpu.h"

namespace luma {

struct P64 {
    using S = double;  // storage
    using R = double;  // arithmetic
    static constexpr bool shifted = false;
};
struct P32 {
    using S = float;
    using R = float;
    static constexpr bool shifted = true;
};

constexpr int kMaxChildren = 4;

// A sub-grid as seen by its parent (coalesce and the transition-layer
// macroscopic copy, :591-636 and :850-891).
struct ChildView {
    const void *f;     // child's current population buffer (S*)
    void *u, *rho;     // child's macroscopic fields (R*)
    int N, M, K;
    int lims[6];       // child's CoarseLims on this grid
};

// Everything a step kernel reads about one grid.  Passed by value.
struct StepArgs {
    int N, M, K, ncell;
    const uint8_t *typ;
    const void *f;          // populations before the step (S*)
    void *fNew;             // populations after the step (S*)
    void *fOut;             // where the split collision writes: fNew, or another buffer when fNew is kept
    const uint8_t *defer;   // IBM grids: per-site "collide in phase C" flag (null: phase C collides all)
    int macro_out;          // interior sites store u and rho (0: nothing reads them before the next step)
    // recording for the adjoint (null when off): the rigid markers' forces
    // (3 per marker), the spread force at the distinct support sites (R,
    // component-major over the supports) and one body's per-marker drag
    // terms F_x w of the step
    double *ibm_f_out, *ibm_drag_out;
    void *ibm_sf_out;
    // BFL links (null without a BFL body): per site a record or -1, per
    // record the linked directions and first link, per link q, kind and the
    // recorded f_opp + fNew_v of the step
    const int *bfl_rec;
    const uint32_t *bfl_mask;
    const int *bfl_first;
    const double *bfl_q;
    const uint8_t *bfl_kind;
    double *bfl_val;
    // running means (LUMA_FLAG_TIME_AVERAGES; null otherwise): rho, u_p and
    // u_p u_q (p <= q), SoA, FP64; tav_t = the grid's completed steps
    double *tav_rho, *tav_u, *tav_uu;
    int tav_t;
    const double *ibm_drag_w;
    int ibm_drag_base, ibm_drag_nm;
    void *u, *rho;          // R*, SoA
    const void *force;      // R*, SoA force_xyz (null when no forcing)
    const double *ux_in, *uy_in, *uz_in;
    double omega, rho0, cs2, csmag;
    // the same rounded to FP32 on the host (csmag2f = (float)(csmag * csmag)):
    // FP32 kernels take these instead of converting per thread, since a
    // conversion from FP64 occupies the FP64 unit
    float omegaf, rho0f, cs2f, csmag2f;
    double pdelta;          // GridUnits::pd2dlbm(L_PRESSURE_DELTA)
    double ramp_stream;     // velocity-ramp coefficient at t*dt (0 => no ramp write)
    double ramp_reg;        // ramp coefficient at (t+1)*dt (regularised BCs)
    int has_ramp;
    int flags, collision, subcycle;
    int forcing;            // IBM or gravity forcing active
    int ibm_split;          // reference compiled with L_IBM_ON: collide in a second pass
    // explode source (parent grid), :646-663
    const void *parent_f;
    int pN, pM, pK;
    int lims[6];            // this grid's CoarseLims on the parent
    int level;
    int nchild;
    ChildView child[kMaxChildren];
    // this grid's device flag: a site that needs an operation outside the
    // GPU path writes a non-zero code (read and cleared by luma_gpu_synchronize)
    int *unsupported;
    // FSI sub-iterations: the reset-forces and IBM kernels return at once
    // while *skip is non-zero (the loop has converged); null outside the loop
    const int *skip;
};

// The step's constants in the kernel's arithmetic type.
template <class P>
__device__ __forceinline__ typename P::R omega_of(const StepArgs &a) {
    if constexpr (sizeof(typename P::R) == 4) return a.omegaf; else return a.omega;
}
template <class P>
__device__ __forceinline__ typename P::R rho0_of(const StepArgs &a) {
    if constexpr (sizeof(typename P::R) == 4) return a.rho0f; else return a.rho0;
}
template <class P>
__device__ __forceinline__ typename P::R cs2_of(const StepArgs &a) {
    if constexpr (sizeof(typename P::R) == 4) return a.cs2f; else return a.cs2;
}
template <class P>
__device__ __forceinline__ typename P::R csmag2_of(const StepArgs &a) {
    if constexpr (sizeof(typename P::R) == 4) return a.csmag2f; else return a.csmag * a.csmag;
}

// Per regularised site: inward normal, normal direction and edge count from
// GridUtils::isWithinDomainWall (src/GridUtils.cpp:1369-1430), computed on
// the host from the site positions.
struct RegSite {
    int id, i, j, k;
    int8_t nvec[3];
    int8_t ndir;
    int8_t edges;
};

// Rounded products and sums the compiler may not fuse into an FMA (where an
// expression must round as the reference's does).
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <class P>
__device__ __forceinline__ typename P::R ld(const void *p, size_t idx) {
    return static_cast<typename P::R>(static_cast<const typename P::S *>(p)[idx]);
}
template <class P>
__device__ __forceinline__ void st(void *p, size_t idx, typename P::R v) {
    static_cast<typename P::S *>(p)[idx] = static_cast<typename P::S>(v);
}
template <class P>
__device__ __forceinline__ typename P::R ldr(const void *p, size_t idx) {
    return static_cast<const typename P::R *>(p)[idx];
}
template <class P>
__device__ __forceinline__ void str(void *p, size_t idx, typename P::R v) {
    static_cast<typename P::R *>(p)[idx] = v;
}

// The non-constant part of the equilibrium, A/cs^2 + B/(2 cs^4), in the
// reference's expression order (_LBM_equilibrium_opt, :674-705).
template <int Q, class R>
__device__ __forceinline__ R eq_poly(int v, R ux, R uy, R uz, R cs2) {
    using L = Lattice<Q>;
    const R c0 = R(L::c(v, 0)), c1 = R(L::c(v, 1)), c2 = R(L::c(v, 2));
    R A, B;
    if (L::D == 3) {
        A = (c0 * ux) + (c1 * uy) + (c2 * uz);
        B = (R(L::c(v, 0) * L::c(v, 0)) - cs2) * (ux * ux) + (R(L::c(v, 1) * L::c(v, 1)) - cs2) * (uy * uy) +
            (R(L::c(v, 2) * L::c(v, 2)) - cs2) * (uz * uz) + R(2 * L::c(v, 0) * L::c(v, 1)) * ux * uy +
            R(2 * L::c(v, 0) * L::c(v, 2)) * ux * uz + R(2 * L::c(v, 1) * L::c(v, 2)) * uy * uz;
    } else {
        A = (c0 * ux) + (c1 * uy);
        B = (R(L::c(v, 0) * L::c(v, 0)) - cs2) * (ux * ux) + (R(L::c(v, 1) * L::c(v, 1)) - cs2) * (uy * uy) +
            R(2 * L::c(v, 0) * L::c(v, 1)) * ux * uy;
    }
    return (A / cs2) + (B / (R(2) * cs2 * cs2));
}

// x * w_v for FP32 with the exact (FP64) lattice weight: w = hi + lo with hi
// the nearest float, so fma(x, hi, x*lo) is x*w to within an ulp.  The
// weights 1/18, 1/36, 1/3 ... are not floats; rounding them once biases every
// equilibrium the same way each step (sum_v w_v != 1 and sum_v w_v c_v c_v !=
// cs^2 I in FP32), which drifts mass and momentum.  With the split weight
// only unbiased rounding of the product remains.
template <int Q>
__device__ __forceinline__ float wmul(int v, float x) {
    const double w = Lattice<Q>::w(v);
    const float hi = float(w);
    const float lo = float(w - double(hi));
    return fmaf(x, hi, x * lo);
}

// The FP32 equilibrium polynomial with the exact constants of cs^2 = 1/3:
// 3 c.u + 4.5 (c.u)^2 - 1.5 u.u (the reference's A/cs^2 + B/(2 cs^4)).
template <int Q>
__device__ __forceinline__ float eq_poly32(int v, float ux, float uy, float uz) {
    using L = Lattice<Q>;
    float cu = 0.f;
    if (L::c(v, 0)) cu += L::c(v, 0) > 0 ? ux : -ux;
    if (L::c(v, 1)) cu += L::c(v, 1) > 0 ? uy : -uy;
    if (L::D == 3 && L::c(v, 2)) cu += L::c(v, 2) > 0 ? uz : -uz;
    const float usq = ux * ux + uy * uy + (L::D == 3 ? uz * uz : 0.f);
    return 3.f * cu + 4.5f * cu * cu - 1.5f * usq;
}

// Equilibrium in the stored representation: f_eq (P64, the reference's
// expression) or g_eq = f_eq - w*rho0 = w*(drho + rho*poly) (P32).
template <int Q, class P>
__device__ __forceinline__ typename P::R feq_s(int v, typename P::R rho, typename P::R drho, typename P::R ux,
                                                typename P::R uy, typename P::R uz, typename P::R cs2) {
    using R = typename P::R;
    if constexpr (P::shifted) {
        (void)cs2;
        return wmul<Q>(v, drho + rho * eq_poly32<Q>(v, ux, uy, uz));
    } else {
        const R w = R(Lattice<Q>::w(v));
        return rho * w * (R(1) + eq_poly<Q, R>(v, ux, uy, uz, cs2));
    }
}

// w_v * X in the arithmetic of the policy (exact-weight product in FP32).
template <int Q, class P>
__device__ __forceinline__ typename P::R wtimes(int v, typename P::R x) {
    if constexpr (P::shifted) return wmul<Q>(v, x);
    else return typename P::R(Lattice<Q>::w(v)) * x;
}

// Guo forcing term of direction v (_LBM_forceGrid_opt, :928-990).  FP64
// keeps the reference's expression; FP32 uses 1/cs^2 = 3 and the
// exact-weight product.
template <int Q, class R>
__device__ __forceinline__ R guo(int v, R omega, R cs2, R ux, R uy, R uz, R Fx, R Fy, R Fz) {
    using L = Lattice<Q>;
    if constexpr (sizeof(R) == 4) {
        R beta = R(L::c(v, 0)) * ux + R(L::c(v, 1)) * uy;
        if (L::D == 3) beta += R(L::c(v, 2)) * uz;
        beta = R(3) * beta;
        R s = R(0);
        s += Fx * (R(L::c(v, 0)) * (R(1) + beta) - ux);
        s += Fy * (R(L::c(v, 1)) * (R(1) + beta) - uy);
        if (L::D == 3) s += Fz * (R(L::c(v, 2)) * (R(1) + beta) - uz);
        return wmul<Q>(v, R(3) * (R(1) - R(0.5) * omega) * s);
    } else {
        const R lambda = (R(1) - R(0.5) * omega) * (R(L::w(v)) / cs2);
        R beta = R(L::c(v, 0)) * ux + R(L::c(v, 1)) * uy;
        if (L::D == 3) beta += R(L::c(v, 2)) * uz;
        beta = beta * (R(1) / cs2);
        R s = R(0);
        s += Fx * (R(L::c(v, 0)) * (R(1) + beta) - ux);
        s += Fy * (R(L::c(v, 1)) * (R(1) + beta) - uy);
        if (L::D == 3) s += Fz * (R(L::c(v, 2)) * (R(1) + beta) - uz);
        return s * lambda;
    }
}

}  // namespace luma
