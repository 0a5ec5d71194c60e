// In-place (AA-pattern) fused stream + collide for periodic grids whose
// sites are all fluid: one population buffer, read and written once per
// step, 2*Q*sizeof(S) bytes of HBM traffic per lattice update.
//
// Storage states of the single buffer A[v][x] (SoA, x = reference site id):
//   E ("even"): A[opp(v)][x] = f_v(x)            (post-collision, not streamed)
//   O ("odd") : A[v][x]      = f_v(x - c_v)      (post-collision, streamed)
// A step from E reads the incoming population of direction v at x from
// A[opp(v)][x - c_v] and writes the new post-collision f_v(x) to
// A[v][x + c_v]; the only other access to either slot in that step is by
// the same thread, so the update is race-free in place.  A step from O
// reads A[v][x] and writes A[opp(v)][x].  Two steps restore state E.
//
// The step is the reference's stream (:206-297, periodic modulo wrap),
// macroscopic (:800-847) and BGK collision (:765-790) for all-fluid grids;
// the equilibrium is expanded as w*rho*(1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u^2),
// the same polynomial as _LBM_equilibrium_opt (:674-705) with cs^2 = 1/3
// folded and the (v, opp(v)) pairs sharing their even part.  Density and
// velocity are written only on the last step of a batch (WRITE_MACRO).
#include <cuda_runtime.h>

#include "device.cuh"
#include "kernels.hpp"

namespace luma {

namespace {

template <int Q, class P, bool FROM_E, bool WRITE_MACRO>
__global__ void __launch_bounds__(256) k_aa(typename P::S *__restrict__ A, typename P::R *__restrict__ u,
                                            typename P::R *__restrict__ rho_out, int N, int M, int K,
                                            typename P::R omega, typename P::R rho0) {
    using L = Lattice<Q>;
    using R = typename P::R;
    using S = typename P::S;
    constexpr int D = L::D;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const int j = blockIdx.y;
    const int i = blockIdx.z;
    const size_t n = (size_t)N * M * K;
    const size_t x = (size_t)k + (size_t)K * ((size_t)j + (size_t)M * i);

    // Neighbour offsets with periodic wrap, per axis and sign.
    int dxp = 0, dxm = 0, dyp = 0, dym = 0, dzp = 0, dzm = 0;
    if (FROM_E) {
        const int KM = K * M;
        dxp = (i + 1 == N) ? -(N - 1) * KM : KM;
        dxm = (i == 0) ? (N - 1) * KM : -KM;
        dyp = (j + 1 == M) ? -(M - 1) * K : K;
        dym = (j == 0) ? (M - 1) * K : -K;
        if (D == 3) {
            dzp = (k + 1 == K) ? -(K - 1) : 1;
            dzm = (k == 0) ? (K - 1) : -1;
        }
    }
    auto off = [&](int cx, int cy, int cz) -> long long {
        long long o = 0;
        o += cx > 0 ? dxp : (cx < 0 ? dxm : 0);
        o += cy > 0 ? dyp : (cy < 0 ? dym : 0);
        o += cz > 0 ? dzp : (cz < 0 ? dzm : 0);
        return o;
    };

    R g[Q];
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        if (FROM_E) {
            // incoming f_v(x) = f_v(x - c_v), stored at A[opp(v)][x - c_v]
            const long long o = off(-L::c(v, 0), -L::c(v, 1), -L::c(v, 2));
            g[v] = R(A[(size_t)L::opp(v) * n + (size_t)((long long)x + o)]);
        } else {
            g[v] = R(A[(size_t)v * n + x]);
        }
    }

    // Moments.  Pair sums keep the FP32 sums of small shifted values short.
    R drho = R(0), jx = R(0), jy = R(0), jz = R(0);
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        drho += g[v];
        if (L::c(v, 0)) jx += L::c(v, 0) > 0 ? g[v] : -g[v];
        if (L::c(v, 1)) jy += L::c(v, 1) > 0 ? g[v] : -g[v];
        if (D == 3 && L::c(v, 2)) jz += L::c(v, 2) > 0 ? g[v] : -g[v];
    }
    R rho;
    if (P::shifted) rho = rho0 + drho;
    else { rho = drho; drho = rho - rho0; }
    const R inv = R(1) / rho;
    const R ux = jx * inv, uy = jy * inv, uz = D == 3 ? jz * inv : R(0);
    if (WRITE_MACRO) {
        u[x] = ux;
        u[n + x] = uy;
        if (D == 3) u[2 * n + x] = uz;
        rho_out[x] = rho;
    }
    const R usq15 = R(1.5) * (ux * ux + uy * uy + uz * uz);
    // rho*u.u from the momentum itself: 1.5 j.u
    const R ju15 = R(1.5) * (jx * ux + jy * uy + jz * uz);
    // Equilibrium, (v, opp(v)) pairs sharing their even part:
    //   shifted  g_eq = w*(drho + 3 c.j + 4.5 (c.j)(c.u) - 1.5 j.u), exact-weight product
    //   plain    f_eq = w*rho*(1 + 3cu + 4.5cu^2 - 1.5u^2)
    // The shifted form takes the odd part 3 w c.j from the momentum sums
    // directly, not as rho * (j/rho): in FP32 the rounded quotient times rho
    // differs from j by a bias fixed by the (nearly steady) density field,
    // which the collision would turn into a steady momentum leak.
#pragma unroll
    for (int v = 0; v < Q; ++v) {
        const int o = L::opp(v);
        if (o < v) continue;  // handled with its partner
        if (o == v) {  // rest population
            R eq;
            if constexpr (P::shifted) eq = wmul<Q>(v, drho - ju15);
            else eq = R(L::w(v)) * rho * (R(1) - usq15);
            g[v] = g[v] + omega * (eq - g[v]);
            continue;
        }
        R cu = R(0);
        if (L::c(v, 0)) cu += L::c(v, 0) > 0 ? ux : -ux;
        if (L::c(v, 1)) cu += L::c(v, 1) > 0 ? uy : -uy;
        if (D == 3 && L::c(v, 2)) cu += L::c(v, 2) > 0 ? uz : -uz;
        R eqv, eqo;
        if constexpr (P::shifted) {
            R cj = R(0);
            if (L::c(v, 0)) cj += L::c(v, 0) > 0 ? jx : -jx;
            if (L::c(v, 1)) cj += L::c(v, 1) > 0 ? jy : -jy;
            if (D == 3 && L::c(v, 2)) cj += L::c(v, 2) > 0 ? jz : -jz;
            const R even = drho + (R(4.5) * cj * cu - ju15);
            const R odd = R(3) * cj;
            eqv = wmul<Q>(v, even + odd);
            eqo = wmul<Q>(v, even - odd);
        } else {
            const R wr = R(L::w(v)) * rho;
            const R sym = wr * (R(1) + R(4.5) * cu * cu - usq15);
            const R asym = R(3) * wr * cu;
            eqv = sym + asym;
            eqo = sym - asym;
        }
        g[v] = g[v] + omega * (eqv - g[v]);
        g[o] = g[o] + omega * (eqo - g[o]);
    }

#pragma unroll
    for (int v = 0; v < Q; ++v) {
        if (FROM_E) {
            // post-collision f_v(x) streams to x + c_v, slot v
            const long long o = off(L::c(v, 0), L::c(v, 1), L::c(v, 2));
            A[(size_t)v * n + (size_t)((long long)x + o)] = S(g[v]);
        } else {
            A[(size_t)L::opp(v) * n + x] = S(g[v]);
        }
    }
}

}  // namespace

template <int Q, class P>
cudaError_t launch_aa(void *A, void *u, void *rho, int N, int M, int K, double omega, double rho0, bool from_e,
                      bool write_macro, cudaStream_t s) {
    using S = typename P::S;
    using R = typename P::R;
    const int bs = K >= 256 ? 256 : ((K + 31) / 32) * 32;
    dim3 grid((K + bs - 1) / bs, M, N);
    S *a = static_cast<S *>(A);
    R *uu = static_cast<R *>(u), *rr = static_cast<R *>(rho);
    const R om = R(omega), r0 = R(rho0);
    if (from_e) {
        if (write_macro) k_aa<Q, P, true, true><<<grid, bs, 0, s>>>(a, uu, rr, N, M, K, om, r0);
        else k_aa<Q, P, true, false><<<grid, bs, 0, s>>>(a, uu, rr, N, M, K, om, r0);
    } else {
        if (write_macro) k_aa<Q, P, false, true><<<grid, bs, 0, s>>>(a, uu, rr, N, M, K, om, r0);
        else k_aa<Q, P, false, false><<<grid, bs, 0, s>>>(a, uu, rr, N, M, K, om, r0);
    }
    return cudaGetLastError();
}

#define LUMA_INST_AA(Q, P) \
    template cudaError_t launch_aa<Q, P>(void *, void *, void *, int, int, int, double, double, bool, bool, cudaStream_t);
LUMA_INST_AA(9, P64)
LUMA_INST_AA(19, P64)
LUMA_INST_AA(27, P64)
LUMA_INST_AA(9, P32)
LUMA_INST_AA(19, P32)
LUMA_INST_AA(27, P32)

}  // namespace luma
