// Flexible filaments on the device: the co-rotational Euler-Bernoulli beam
// of FEMBody/FEMElement (LUMA src/FEMBody.cpp:136-424,
// src/FEMElement.cpp:109-302) and the FSI coupling of ObjectManager
// (src/ObjectManager_ops_ibm.cpp:61-185, :988-1032).
//
// One CTA per filament runs dynamicFEM: Newmark-beta (alpha 0.25, delta
// 0.5) with Newton-Raphson (tol 1e-10, <= 20 iterations); each iteration
// assembles the element force vectors and the mass and stiffness matrices
// with the reference's summation order (every global entry sums its element
// contributions in element order), forms the effective system and solves it
// with partial-pivot LU.  A second per-filament kernel rebuilds the moving
// markers' supports, spacing and epsilon.  This translation unit is built
// with FMA contraction off so the FP64 operation sequence is the
// reference's.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "dispatch.hpp"
#include "grid.hpp"
#include "kernels.hpp"
#include "quotient.cuh"

using namespace luma;

namespace {

constexpr double kNbAlpha = 0.25;
constexpr double kNbDelta = 0.5;
constexpr double kRelax = 0.5;
constexpr double kPi = 3.14159265358979323846;

// Shared memory budget for a filament's stiffness matrix (static shared
// arrays of the kernel take the rest of the 227 KB).
constexpr size_t kFemSmemMax = 200 * 1024;

struct FemKernelArgs {
    int nfil, maxdof, maxmk;
    int k_in_smem;              // K of the filament in dynamic shared memory
    int lu32;                   // Newton steps solved with FP32 factors of the scaled matrix (shifted-FP32
                                // grids; the matrix's FP32 copy follows K in dynamic shared memory)
    int eps_in_smem;            // the epsilon matrix of the filament in dynamic shared memory
    const int *node_off, *el_off, *dof_off, *mk_off, *bc;
    const double *dm, *velscale;
    const double *pos0, *ang0;
    const double *len0, *area, *I, *E, *rho;
    const int *child_off, *child_node;
    const double *child_z1, *child_z2;
    double *U, *U_n, *Ud, *Ud_n, *Udd, *Udd_n, *R, *Fv, *delU;
    double *M, *K, *epsA;
    double *elF, *elM, *elK, *elang, *ellen, *npos, *nang, *tmp;
    const int *parent_el;
    const double *parent_zeta, *mpos0;
    int *it;
    // first Newton iteration of a step (the state is the step's start in every
    // FSI sub-iteration): factored matrix, pivots, L extents, internal force
    // and mass term, kept by the step's first FEM call (cache_mode 1) and
    // reused by its later ones (cache_mode 2)
    double *Kc, *Fc, *MFc;
    int *ipc, *limc;
    int cache_mode;
    double *res, *fsi_res;      // per filament NR residual; FSI residual: [0] running max, [1] last
    int *fsi_state;             // FSI loop of the step: [0] converged, [1] sub-iterations run
    const int *skip;            // while *skip (the loop converged) the kernels return at once; may be null
    double dt, dh;
    FlexArgs flex;
    // grid for the support search
    int N, M_, K_, dims, level;
    const double *hx, *hy, *hz;
    double gstart[3];
    double edges[6];
    int *error;
};

__device__ __forceinline__ void Tmat(double ang, double T[6][6]) {
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) T[i][j] = 0.0;
    const double c = cos(ang), s = sin(ang);
    T[0][0] = T[1][1] = T[3][3] = T[4][4] = c;
    T[0][1] = T[3][4] = s;
    T[1][0] = T[4][3] = -s;
    T[2][2] = T[5][5] = 1.0;
}

// FEMBody::updateFEMValues (:297-325) for filament f.
__device__ void update_values(const FemKernelArgs &a, int f) {
    const int n0 = a.node_off[f], nn = a.node_off[f + 1] - n0;
    const int e0 = a.el_off[f], ne = a.el_off[f + 1] - e0;
    const int d0 = a.dof_off[f];
    for (int n = threadIdx.x; n < nn; n += blockDim.x) {
        for (int d = 0; d < 2; d++) a.npos[3 * (n0 + n) + d] = a.pos0[3 * (n0 + n) + d] + a.U[d0 + n * 3 + d];
        a.npos[3 * (n0 + n) + 2] = a.pos0[3 * (n0 + n) + 2];
        a.nang[n0 + n] = a.ang0[n0 + n] + a.U[d0 + n * 3 + 2];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
        double v[3];
        for (int d = 0; d < 3; ++d) v[d] = a.npos[3 * (n0 + e + 1) + d] - a.npos[3 * (n0 + e) + d];
        a.elang[e0 + e] = atan2(v[1], v[0]);
        double r = 0.0;
        for (int d = 0; d < 3; ++d) r += v[d] * v[d];
        a.ellen[e0 + e] = sqrt(r);
    }
    __syncthreads();
}

// Partial-pivot LU of the n x n block whose column-major element (r, c)
// is A[(off + c) * lda + (off + r)] (a row-major matrix read column-major,
// as GridUtils::solveLinearSystem hands it to dgetrf_), then the transposed
// solve for x (length n), n <= 512 (dgetrs_ with trans = 'T': U^T y = x,
// then L^T z = y, then the row interchanges in reverse).  Every element sees
// the operations of the dense serial algorithm in the same order; the ones
// that are exact no-ops (a zero multiplier, a zero matrix entry in the
// triangular sums, a swap of two zeros) are skipped, which is what makes the
// banded beam and epsilon systems cheap.  One warp does the work (warp
// barriers only); the pivot is the first row of largest magnitude (ties to
// the lower row).  Called by the whole block; returns after a block barrier.
// Zero tests and magnitude order on the bit patterns (integer pipe): +-0
// are the only doubles whose bits shifted left by one are 0, and |x| of
// non-NaN doubles orders like its bits read as unsigned.
__device__ __forceinline__ bool is_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }
__device__ __forceinline__ unsigned long long mag_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
// (32-bit index arithmetic: lda and n are at most 512)
#define AC(r, c) A[(off + (c)) * lda + (off + (r))]

// `band`: no entry of the matrix lies more than `band` rows below or
// columns right of the diagonal (n for a dense matrix).  Partial pivoting
// keeps the multipliers of column k in rows k+1..k+band and the pivot row's
// entries in columns up to k+2*band (a row at position r >= k holds
// original entries up to column r+band and fill from earlier steps j up to
// j+2*band), so the scans stop there; the entries they skip are exact
// zeros, which the dense elimination would leave as they are.

// The banded case (band <= NB, NB = 7 or 15), one warp.  GB300 gives an
// FP64 instruction of a warp 64 cycles of its sub-partition however many
// lanes are active, so a step issues as few as it can, each dense: the
// pivot's reciprocal, one multiply for all the multipliers (lane i: row
// k+1+i), and the rank-1 update over the (row, column) pairs of non-zero
// multiplier and pivot-row entry, 32 pairs per multiply-subtract.  The pivot
// search is integer work on every lane (the candidates' magnitude bits);
// the row interchange moves the rows' entries left of the window's right
// end (further right both rows hold zeros).  lim[c] bounds the last row
// holding a non-zero of L's column c (set by the multipliers, raised when
// an interchange moves a non-zero down), so the backward solve needs no
// scan.
// `progress` (may be null): after step k's row interchange, row k of U is
// final; the step count is published there (shared memory) for a forward
// solve running beside the factorisation on another warp.
template <int NB>
__device__ __forceinline__ void lu_factor_banded(double *A, int lda, int off, int n, int *ipiv, int band, int *lim,
                                                 int *rl, int *cl, volatile int *progress = nullptr,
                                                 bool l_swaps = true) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    for (int r = lane; r < n; r += 32) lim[r] = r;
    __syncwarp();
    for (int k = 0; k < n; ++k) {
        const int nr = min(n, k + band + 1) - k - 1;  // window rows below the diagonal
        const int cend = min(n, k + 2 * band + 1);
        // the candidates as bit patterns (integer registers and selects)
        long long cv[NB + 1];
#pragma unroll
        for (int i = 0; i <= NB; ++i) cv[i] = i <= nr ? __double_as_longlong(AC(k + i, k)) : 0ll;
        int pi = 0;
        unsigned long long best = (unsigned long long)cv[0] & 0x7fffffffffffffffull;
#pragma unroll
        for (int i = 1; i <= NB; ++i) {
            const unsigned long long v = (unsigned long long)cv[i] & 0x7fffffffffffffffull;
            if (i <= nr && v > best) {
                best = v;
                pi = i;
            }
        }
        const int p = k + pi;
        if (lane == 0) ipiv[k] = p + 1;
        if (best == 0) {  // a zero column: no interchange, no elimination
            if (progress && lane == 0) {
                __threadfence_block();
                *progress = k + 1;
            }
            continue;
        }
        long long pvb = cv[0], mineb = 0;
#pragma unroll
        for (int i = 1; i <= NB; ++i) {
            if (pi == i) pvb = cv[i];
            if (lane == i - 1) mineb = pi == i ? cv[0] : cv[i];  // row k+1+lane after the interchange
        }
        const double pv = __longlong_as_double(pvb), mine = __longlong_as_double(mineb);
        if (pi) {
            // the interchange in the window's columns (k .. cend-1); the rows'
            // L parts (left of k) follow after the factorisation
            __syncwarp();  // every lane's candidate reads before the interchange writes
            const int c = k + lane;
            if (c < cend) {
                const double t = AC(k, c);
                AC(k, c) = AC(p, c);
                AC(p, c) = t;
            }
            __syncwarp();
        }
        if (progress && lane == 0) {
            __threadfence_block();
            *progress = k + 1;
        }
        const double inv = 1.0 / pv;
        const double m = mine * inv;
        const bool mrow = lane < nr && !is_zero(m);
        if (lane < nr) AC(k + 1 + lane, k) = m;
        const int c = k + 1 + lane;
        const bool mcol = c < cend && !is_zero(AC(k, c));
        const unsigned rmask = __ballot_sync(full, mrow), cmask = __ballot_sync(full, mcol);
        // the non-zero rows and columns listed in order (ballot prefixes)
        if (mrow) rl[__popc(rmask & below)] = lane;
        if (mcol) cl[__popc(cmask & below)] = lane;
        if (lane == 0 && rmask) lim[k] = k + 32 - __clz(rmask);
        __syncwarp();
        const int nrl = __popc(rmask), npairs = nrl * __popc(cmask);
        if (npairs) {
            // pair t -> (row t mod nrl, column t div nrl); the quotient as a
            // multiply-shift, exact for t < 2^20 / nrl^2
            const unsigned magic = (1048576u + nrl - 1) / nrl;
            for (int t = lane; t < npairs; t += 32) {
                const int ci = (int)(((unsigned)t * magic) >> 20), ri = t - ci * nrl;
                const int rr = k + 1 + rl[ri], cc = k + 1 + cl[ci];
                AC(rr, cc) -= AC(rr, k) * AC(k, cc);
            }
        }
        __syncwarp();
    }
    // the row interchanges in the L part: column c takes, in step order, the
    // interchanges of the steps after it (nothing above reads these columns);
    // or lu_l_swaps on another warp, beside the factorisation
    if (!l_swaps) return;
    for (int c = lane; c < n; c += 32) {
        int lc = lim[c];
        for (int k = c + 1; k < n; ++k) {
            const int p = ipiv[k] - 1;
            if (p != k) {
                const double t = AC(k, c);
                AC(k, c) = AC(p, c);
                AC(p, c) = t;
                if (!is_zero(t) && p > lc) lc = p;
            }
        }
        lim[c] = lc;
    }
    __syncwarp();
}

// The L-part row interchanges of lu_factor_banded on another warp, step by
// step as the factorisation publishes them: step k's interchange of rows k
// and p in the columns left of k touches nothing the factorisation still
// reads (its steps read and write columns >= their own index), and column c
// of L is complete (its multipliers written at step c) before step k > c is
// published.  lim of those columns is raised here as in the serial pass.
__device__ __forceinline__ void lu_l_swaps(double *A, int lda, int off, int n, const volatile int *ipiv, int *lim,
                                           const volatile int *progress, int *err);

// Iterations a warp waits for the factorisation's next step before it
// gives up (and records code 3): far beyond any step's duration.
constexpr int kLuWaitLimit = 1 << 24;

__device__ __forceinline__ void lu_l_swaps(double *A, int lda, int off, int n, const volatile int *ipiv, int *lim,
                                           const volatile int *progress, int *err) {
    const int lane = threadIdx.x & 31;
    for (int k = 1; k < n; ++k) {
        int spins = 0;
        while (*progress <= k)
            if (++spins > kLuWaitLimit) {
                if (lane == 0 && err) atomicExch(err, 3);
                break;
            }
        __threadfence_block();
        const int p = ipiv[k] - 1;
        if (p == k) continue;
        for (int c = lane; c < k; c += 32) {
            const double t = AC(k, c);
            AC(k, c) = AC(p, c);
            AC(p, c) = t;
            if (!is_zero(t) && p > lim[c]) lim[c] = p;
        }
    }
}

// Forward U^T y = x (into xs), one warp.  U's rows reach 2*band right of the
// diagonal, so each lane keeps one pending row and subtracts a term as soon
// as its unknown is known, in ascending order (the serial order); the
// divisions use the diagonal's reciprocals (all formed at once beforehand,
// or per column when `progress` is given: then column c waits until the
// factorisation has published step c, and `err` takes code 3 if a wait
// runs out).
__device__ __forceinline__ void lu_forward(const double *A, int lda, int off, int n, const double *x, int band,
                                           double *xs, double *rd, const volatile int *progress, int *err) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (int r = lane; r < n; r += 32) {
        xs[r] = x[r];
        if (!progress) rd[r] = 1.0 / AC(r, r);
    }
    __syncwarp();
    double s = lane < n ? xs[lane] : 0.0;
    int row = lane;
    for (int c = 0; c < n; ++c) {
        if (progress) {
            int spins = 0;
            while (*progress <= c)
                if (++spins > kLuWaitLimit) {
                    if (lane == 0 && err) atomicExch(err, 3);
                    break;
                }
            __threadfence_block();
        }
        const double dc = AC(c, c), rc = progress ? 1.0 / dc : rd[c];
        const double v = row < n ? AC(c, row) : 0.0;
        double y = 0.0;
        if (row == c) y = quotient(s, dc, rc);
        y = __shfl_sync(full, y, c & 31);
        if (row == c) {
            xs[c] = y;
            row += 32;
            s = row < n ? xs[row] : 0.0;
        } else if (row < n && row <= c + 2 * band && !is_zero(v)) {
            s -= v * y;
        }
    }
    __syncwarp();
}

// Backward L^T z = y (y in xs), the row interchanges in reverse, the result
// into x; one warp.
__device__ __forceinline__ void lu_backward(const double *A, int lda, int off, int n, const int *ipiv, double *x,
                                            const int *lim, double *xs) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // backward L^T z = y, rows from the last: z_r = y_r - sum over c = r+1..lim[r]
    // of L(c, r) z_c, in ascending c.  Every lane carries the running sum;
    // lane j holds z_{r+1+j} (a window shifted by one lane per row) and forms
    // its product off the critical path; the sum takes the non-zero terms in
    // order, the first one from z_{r+1} itself.  A row's entries are loaded
    // while the row before it is summed.
    double zw = 0.0, zr = 0.0;
    int tn = lim[n - 1] - (n - 1);
    double yn = xs[n - 1];
    double Ln = 0.0;
    for (int r = n - 1; r >= 0; --r) {
        const int t = tn;
        const double yr = yn, L = Ln;
        if (r > 0) {
            tn = lim[r - 1] - (r - 1);
            yn = xs[r - 1];
            Ln = lane < tn ? AC(r + lane, r - 1) : 0.0;
        }
        zw = __shfl_up_sync(full, zw, 1);
        double zn;
        if (t <= 32) {
            const unsigned nzm = __ballot_sync(full, !is_zero(L));
            const double L0 = __shfl_sync(full, L, 0);
            const double prod = L * zw;
            double acc = yr;
            if (nzm & 1u) acc -= L0 * zr;
            for (unsigned b = nzm & ~1u; b; b &= b - 1) acc -= __shfl_sync(full, prod, __ffs(b) - 1);
            zn = acc;
        } else {
            // long columns (interchanges carried L far down): the plain sum
            double acc = yr;
            for (int cc = r + 1; cc <= lim[r]; ++cc) {
                const double v = AC(cc, r);
                if (!is_zero(v)) acc -= v * xs[cc];
            }
            zn = acc;
        }
        if (lane == 0) {
            zw = zr;  // z_{r+1} enters the window for the next row's shift
            if (r + 1 < n) xs[r + 1] = zr;
        }
        zr = zn;
        if (r > 0 && tn > 32) {
            if (lane == 0) xs[r] = zr;
            __syncwarp();
        }
    }
    if (lane == 0) {
        xs[0] = zr;
        for (int k = n - 1; k >= 0; --k) {
            const int p = ipiv[k] - 1;
            if (p != k) {
                const double t = xs[k];
                xs[k] = xs[p];
                xs[p] = t;
            }
        }
    }
    __syncwarp();
    for (int r = lane; r < n; r += 32) x[r] = xs[r];
}

// The transposed solve with the factors of lu_factor_banded (lim included),
// one warp.
__device__ __forceinline__ void lu_solve_factored(const double *A, int lda, int off, int n, const int *ipiv, double *x,
                                                  int band, const int *lim, double *xs, double *rd) {
    lu_forward(A, lda, off, n, x, band, xs, rd, nullptr, nullptr);
    lu_backward(A, lda, off, n, ipiv, x, lim, xs);
}

// The general case, one warp: lanes over rows / columns, the rank-1 update
// over (row, column) pairs of non-zero multiplier and pivot-row entry.
__device__ void lu_solve_dense(double *A, int lda, int off, int n, int *ipiv, double *x, int band, int *nzr,
                               int *nzc, int *lim, double *xs) {
    const int lane = threadIdx.x & 31;
    for (int k = 0; k < n; ++k) {
        unsigned long long best = 0;
        int p = n;
        const int rend = min(n, k + band + 1), cend = min(n, k + 2 * band + 1);
        for (int r = k + lane; r < rend; r += 32) {
            const unsigned long long v = mag_bits(AC(r, k));
            if (p == n || v > best) { best = v; p = r; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int op = __shfl_xor_sync(0xffffffffu, p, o);
            if (op < n && (p == n || ob > best || (ob == best && op < p))) { best = ob; p = op; }
        }
        if (lane == 0) ipiv[k] = p + 1;
        if (is_zero(AC(p, k))) continue;  // same value on every lane
        __syncwarp();
        if (p != k)
            for (int c = lane; c < n; c += 32) {
                const double t = AC(k, c);
                AC(k, c) = AC(p, c);
                AC(p, c) = t;
            }
        __syncwarp();
        // rows with a non-zero multiplier and columns with a non-zero
        // pivot-row entry, listed by warp ballots (every lane keeps the
        // counts)
        const double inv = 1.0 / AC(k, k);
        const unsigned below = (1u << lane) - 1u;
        int cr = 0, cc = 0;
        for (int r0 = k + 1; r0 < rend; r0 += 32) {
            const int r = r0 + lane;
            bool nz = false;
            if (r < rend) {
                const double m = AC(r, k) * inv;
                AC(r, k) = m;
                nz = !is_zero(m);
            }
            const unsigned b = __ballot_sync(0xffffffffu, nz);
            if (nz) nzr[cr + __popc(b & below)] = r;
            cr += __popc(b);
        }
        for (int c0 = k + 1; c0 < cend; c0 += 32) {
            const int c = c0 + lane;
            const bool nz = c < cend && !is_zero(AC(k, c));
            const unsigned b = __ballot_sync(0xffffffffu, nz);
            if (nz) nzc[cc + __popc(b & below)] = c;
            cc += __popc(b);
        }
        __syncwarp();
        for (int t = lane; t < cr * cc; t += 32) {
            const int r = nzr[t % cr], c = nzc[t / cr];
            AC(r, c) -= AC(r, k) * AC(k, c);
        }
        __syncwarp();
    }
    for (int r = lane; r < n; r += 32) xs[r] = x[r];
    // forward sums start at the first non-zero of each row's range
    for (int r = lane; r < n; r += 32) {
        int c = 0;
        while (c < r && is_zero(AC(c, r))) ++c;
        lim[r] = c;
    }
    __syncwarp();
    if (lane == 0)
        for (int r = 0; r < n; ++r) {
            double s = xs[r];
            for (int c = lim[r]; c < r; ++c) {
                const double v = AC(c, r);
                if (!is_zero(v)) s -= v * xs[c];
            }
            xs[r] = s / AC(r, r);
        }
    __syncwarp();
    // backward sums end at the last non-zero
    for (int r = lane; r < n; r += 32) {
        int c = n - 1;
        while (c > r && is_zero(AC(c, r))) --c;
        lim[r] = c;
    }
    __syncwarp();
    if (lane == 0) {
        for (int r = n - 1; r >= 0; --r) {
            double s = xs[r];
            for (int c = r + 1; c <= lim[r]; ++c) {
                const double v = AC(c, r);
                if (!is_zero(v)) s -= v * xs[c];
            }
            xs[r] = s;
        }
        for (int k = n - 1; k >= 0; --k) { const int p = ipiv[k] - 1; if (p != k) { const double t = xs[k]; xs[k] = xs[p]; xs[p] = t; } }
    }
    __syncwarp();
    for (int r = lane; r < n; r += 32) x[r] = xs[r];
}

#undef AC

// ---- FP32 factors for the shifted-FP32 path ----
// The Newmark matrix K + a0 M of a filament is well conditioned once its
// rows and columns are scaled by 1/sqrt|diagonal|: condition 7-44 against
// 1.6e5-3.2e5 unscaled over the filament-array workload's rigidities
// (EI 1e-3 .. 1e-1, a0 M / K 6e-2 .. 6 on the diagonal).  FP32 factors of
// the scaled matrix then solve a Newton step to ~1e-6 relative, and the
// iteration, whose residual and update stay FP64, converges to the same
// 1e-10 tolerance.  The algorithm is the FP64 path's (the partial-pivot LU
// and transposed solve of lu_factor / lu_solve_t), in FP32 with FMAs, on
// one warp: an FP32 operation does not hold a sub-partition the 64 cycles
// an FP64 one does, so the shuffles and shared-memory round trips of a
// pivot step set its length.
#define AF(r, c) A[(c) * lda + (r)]

// A (n x n, column-major, lda) in place; whole-row interchanges; lim[c] =
// last row of L's column c holding a non-zero.  band as lu_factor_banded's.
__device__ __forceinline__ void lu32_factor(float *A, int lda, int n, int *ipiv, int band, int *lim) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (int r = lane; r < n; r += 32) lim[r] = r;
    __syncwarp();
    for (int k = 0; k < n; ++k) {
        const int nr = min(n, k + band + 1) - k;  // candidate rows k .. k+nr-1 (nr <= 32)
        const int cend = min(n, k + 2 * band + 1);
        float v = lane < nr ? fabsf(AF(k + lane, k)) : -1.0f;
        int idx = lane;
        for (int o = 16; o > 0; o >>= 1) {  // the largest magnitude, the first row on ties
            const float ov = __shfl_xor_sync(full, v, o);
            const int oi = __shfl_xor_sync(full, idx, o);
            if (ov > v || (ov == v && oi < idx)) {
                v = ov;
                idx = oi;
            }
        }
        const int p = k + idx;
        if (lane == 0) ipiv[k] = p + 1;
        if (!(v > 0.0f)) continue;  // a zero column: no interchange, no elimination
        if (p != k) {
            __syncwarp();
            for (int c = lane; c < cend; c += 32) {
                const float t = AF(k, c);
                AF(k, c) = AF(p, c);
                AF(p, c) = t;
                if (c < k && t != 0.0f && p > lim[c]) lim[c] = p;
            }
            __syncwarp();
        }
        const float inv = 1.0f / AF(k, k);
        float m = 0.0f;
        if (lane >= 1 && lane < nr) {
            m = AF(k + lane, k) * inv;
            AF(k + lane, k) = m;
        }
        const unsigned nzm = __ballot_sync(full, m != 0.0f);
        if (lane == 0 && nzm) lim[k] = k + 31 - __clz(nzm);
        __syncwarp();
        const int nrows = nr - 1, ncols = cend - k - 1;
        for (int t = lane; t < nrows * ncols; t += 32) {
            const int j = t / nrows, i = t - j * nrows;
            const int r = k + 1 + i, c = k + 1 + j;
            AF(r, c) = fmaf(-AF(r, k), AF(k, c), AF(r, c));
        }
        __syncwarp();
    }
}

// A^T x = b with the factors of lu32_factor (b in x), one warp.  Forward
// U^T y = b: each lane keeps one pending row (lane, lane + 32, ...) and
// subtracts a column's term as soon as its unknown is known (U's rows reach
// 2*band < 32 right of the diagonal); backward L^T z = y and the
// interchanges on one lane.
__device__ __forceinline__ void lu32_solve_t(const float *A, int lda, int n, const int *ipiv, int band,
                                             const int *lim, float *x) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    float s = lane < n ? x[lane] : 0.0f;
    int row = lane;
    for (int c = 0; c < n; ++c) {
        const float v = row < n ? AF(c, row) : 0.0f;
        float y = 0.0f;
        if (row == c) y = s / AF(c, c);
        y = __shfl_sync(full, y, c & 31);
        if (row == c) {
            x[c] = y;
            row += 32;
            s = row < n ? x[row] : 0.0f;
        } else if (row < n && row <= c + 2 * band) {
            s = fmaf(-v, y, s);
        }
    }
    __syncwarp();
    if (lane == 0) {
        for (int r = n - 1; r >= 0; --r) {
            float z = x[r];
            for (int c = r + 1; c <= lim[r]; ++c) z = fmaf(-AF(c, r), x[c], z);
            x[r] = z;
        }
        for (int k = n - 1; k >= 0; --k) {
            const int p = ipiv[k] - 1;
            if (p != k) {
                const float t = x[k];
                x[k] = x[p];
                x[p] = t;
            }
        }
    }
    __syncwarp();
}

#undef AF

__device__ void lu_solve_block(double *A, int lda, int off, int n, int *ipiv, double *x, int band,
                               int *err = nullptr) {
    __shared__ int nzr[512], nzc[512];
    __shared__ int lim[512];
    __shared__ double xs[512], rd[512];
    __shared__ volatile int progress;
    if (band <= 15 && blockDim.x >= 96) {
        // warp 0 factors, warp 1 runs the forward solve one column behind,
        // warp 2 applies the L-part interchanges; warp 0 then solves backward
        if (threadIdx.x == 0) progress = 0;
        __syncthreads();
        if (threadIdx.x < 32) {
            if (band <= 7) lu_factor_banded<7>(A, lda, off, n, ipiv, band, lim, nzr, nzc, &progress, false);
            else lu_factor_banded<15>(A, lda, off, n, ipiv, band, lim, nzr, nzc, &progress, false);
        } else if (threadIdx.x < 64) {
            lu_forward(A, lda, off, n, x, band, xs, rd, &progress, err);
        } else if (threadIdx.x < 96) {
            lu_l_swaps(A, lda, off, n, ipiv, lim, &progress, err);
        }
        __syncthreads();
        if (threadIdx.x < 32) lu_backward(A, lda, off, n, ipiv, x, lim, xs);
    } else if (threadIdx.x < 32) {
        if (band <= 15) {
            if (band <= 7) lu_factor_banded<7>(A, lda, off, n, ipiv, band, lim, nzr, nzc);
            else lu_factor_banded<15>(A, lda, off, n, ipiv, band, lim, nzr, nzc);
            lu_solve_factored(A, lda, off, n, ipiv, x, band, lim, xs, rd);
        } else {
            lu_solve_dense(A, lda, off, n, ipiv, x, band, nzr, nzc, lim, xs);
        }
    }
    __syncthreads();
}

// 0.0 + v: v itself, except that -0 becomes +0 (integer work).
__device__ __forceinline__ double plus_zero(double v) {
    const long long b = __double_as_longlong(v);
    return __longlong_as_double(b == (long long)0x8000000000000000ull ? 0ll : b);
}

// sum over k = 0..5, from +0, of T[k][r] * g(k) in ascending k.  T (Tmat)
// is block diagonal: rotation blocks {0,1} and {3,4}, ones at 2 and 5.  A
// term with one of its zeros is an exact zero, and adding an exact zero to
// the running sum (which starts at +0 and so is never -0) leaves it as it
// is; a term with one of its ones is g(k) itself.  So the sum is the first
// block term (+0 + it) plus the second, or g(r) with -0 made +0.
template <class G>
__device__ __forceinline__ double tsum(const double T[6][6], int r, G g) {
    if (r == 2 || r == 5) return plus_zero(g(r));
    const int k1 = r < 2 ? 0 : 3;
    return plus_zero(T[k1][r] * g(k1)) + T[k1 + 1][r] * g(k1 + 1);
}

// Element matrices of FEMElement::forceVector/massMatrix/stiffMatrix
// (:273-302, :178-213, :218-268), in global coordinates.  Four threads per
// element, `part` 0 and 1 forming rows 0-2 and 3-5 of the mass matrix
// T^T M T (part 0 also the force vector T^T F), parts 2 and 3 those of the
// stiffness matrix (a row of T^T X T needs only the same row of T^T X).
// The caller gives a warp one part, so the FP64 work of a warp does not
// diverge.
template <int PART>
__device__ __forceinline__ void element_matrices(const FemKernelArgs &a, int f, int e) {
    const int e0 = a.el_off[f], n0 = a.node_off[f];
    const int ge = e0 + e;
    const double ang = a.elang[ge], L0 = a.len0[ge];
    const double EE = a.E[ge], A = a.area[ge], I = a.I[ge];
    double T[6][6];
    Tmat(ang, T);
    double F[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (PART != 1) {
        const double L = a.ellen[ge];
        const double a1 = a.nang[n0 + e], a2 = a.nang[n0 + e + 1];
        const double u = (L * L - L0 * L0) / (L + L0);
        const double t1 = atan2(cos(ang) * sin(a1) - sin(ang) * cos(a1), cos(ang) * cos(a1) + sin(ang) * sin(a1));
        const double t2 = atan2(cos(ang) * sin(a2) - sin(ang) * cos(a2), cos(ang) * cos(a2) + sin(ang) * sin(a2));
        const double F0 = (EE * A / L0) * u;
        const double M1 = (2 * EE * I / L0) * (2.0 * t1 + t2);
        const double M2 = (2 * EE * I / L0) * (t1 + 2.0 * t2);
        F[0] = -F0; F[1] = (1.0 / L0) * (M1 + M2); F[2] = M1; F[3] = F0; F[4] = -(1.0 / L0) * (M1 + M2); F[5] = M2;
    }
    if (PART == 0)
        // internal force in global coordinates, T^T F (the assembly's product)
#pragma unroll
        for (int i = 0; i < 6; ++i) a.elF[6 * ge + i] = tsum(T, i, [&](int c) { return F[c]; });
    double X[6][6] = {};
    if (PART < 2) {
        // mass
        const double C1 = a.rho[ge] * A * L0 / 420.0;
        X[0][0] = C1 * 140.0; X[0][3] = C1 * 70.0; X[1][1] = C1 * 156.0; X[1][2] = C1 * 22.0 * L0;
        X[1][4] = C1 * 54; X[1][5] = C1 * (-13.0 * L0); X[2][2] = C1 * 4.0 * (L0 * L0); X[2][4] = C1 * 13.0 * L0;
        X[2][5] = C1 * (-3.0 * (L0 * L0)); X[3][3] = C1 * 140.0; X[4][4] = C1 * 156.0; X[4][5] = C1 * (-22.0 * L0);
        X[5][5] = C1 * 4.0 * (L0 * L0);
    } else {
        // stiffness (linear + geometric)
        X[0][0] = EE * A / L0; X[0][3] = -EE * A / L0;
        X[1][1] = 12.0 * EE * I / (L0 * L0 * L0); X[1][2] = 6.0 * EE * I / (L0 * L0);
        X[1][4] = -12.0 * EE * I / (L0 * L0 * L0); X[1][5] = 6.0 * EE * I / (L0 * L0);
        X[2][2] = 4.0 * EE * I / L0; X[2][4] = -6.0 * EE * I / (L0 * L0); X[2][5] = 2.0 * EE * I / L0;
        X[3][3] = EE * A / L0; X[4][4] = 12.0 * EE * I / (L0 * L0 * L0); X[4][5] = -6.0 * EE * I / (L0 * L0);
        X[5][5] = 4.0 * EE * I / L0;
    }
#pragma unroll
    for (int i = 1; i < 6; i++)
#pragma unroll
        for (int j = 0; j < i; j++) X[i][j] = X[j][i];
    if (PART >= 2) {
        const double Fa = -F[0], V0 = F[4];
        X[0][1] += -V0 / L0; X[0][4] += V0 / L0; X[1][0] += -V0 / L0; X[1][1] += Fa / L0;
        X[1][3] += V0 / L0; X[1][4] += -Fa / L0; X[3][1] += V0 / L0; X[3][4] += -V0 / L0;
        X[4][0] += V0 / L0; X[4][1] += -Fa / L0; X[4][3] += -V0 / L0; X[4][4] += Fa / L0;
    }
    // rows r0..r0+2 of T^T X T with the reference's k-ordered products
    constexpr int r0 = 3 * (PART & 1);
    double *out = (PART < 2 ? a.elM : a.elK) + 36 * (size_t)ge;
#pragma unroll
    for (int rr = 0; rr < 3; ++rr) {
        const int r = r0 + rr;
        double P[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) P[c] = tsum(T, r, [&](int k) { return X[k][c]; });
#pragma unroll
        for (int c = 0; c < 6; ++c) out[6 * r + c] = tsum(T, c, [&](int k) { return P[k]; });
    }
}

// Load vector entry of DOF d (FEMElement::loadVector, :133-173), summing the
// (element, IB child) contributions in the reference's order.
__device__ double load_entry(const FemKernelArgs &a, int f, int d, double forceScale) {
    const int e0 = a.el_off[f], ne = a.el_off[f + 1] - e0, mk0 = a.mk_off[f];
    double val = 0.0;
    const int elo = d / 3 - 1 < 0 ? 0 : d / 3 - 1;
    const int ehi = d / 3 > ne - 1 ? ne - 1 : d / 3;
    for (int e = elo; e <= ehi; ++e) {
        const int i = d - 3 * e;
        if (i < 0 || i > 5) continue;
        const int ge = e0 + e;
        double T[6][6];
        Tmat(a.elang[ge], T);
        const double L = a.ellen[ge];
        for (int q = a.child_off[ge]; q < a.child_off[ge + 1]; ++q) {
            const int node = a.child_node[q];
            const double za = a.child_z1[q], zb = a.child_z2[q];
            const double sc = a.flex.eps[mk0 + node] * 1.0 * forceScale;
            const double fx[2] = {a.flex.F[3 * (mk0 + node)] * sc, a.flex.F[3 * (mk0 + node) + 1] * sc};
            double fv[2];
            for (int r = 0; r < 2; ++r) {
                double s = 0.0;
                for (int c = 0; c < 2; ++c) s += T[r][c] * fx[c];
                fv[r] = s;
            }
            double Rl[6];
            const double a2 = za * za, b2 = zb * zb;
            Rl[0] = fv[0] * 0.5 * L * (0.5 * zb - 0.5 * za + 0.25 * a2 - 0.25 * b2);
            Rl[1] = fv[1] * 0.5 * L * (0.5 * zb - 0.5 * za - a2 * a2 / 16.0 + b2 * b2 / 16.0 + 3.0 * a2 / 8.0 - 3.0 * b2 / 8.0);
            Rl[2] = fv[1] * 0.5 * L * (L * (-a2 * a2 + b2 * b2) / 32.0 - L * (-(za * za * za) + (zb * zb * zb)) / 24.0 - L * (-a2 + b2) / 16.0 + L * (zb - za) / 8.0);
            Rl[3] = fv[0] * 0.5 * L * (-0.25 * a2 + 0.25 * b2 + 0.5 * zb - 0.5 * za);
            Rl[4] = fv[1] * 0.5 * L * (0.5 * zb - 0.5 * za + a2 * a2 / 16.0 - b2 * b2 / 16.0 - 3.0 * a2 / 8.0 + 3.0 * b2 / 8.0);
            Rl[5] = fv[1] * 0.5 * L * (L * (-a2 * a2 + b2 * b2) / 32.0 + L * (-(za * za * za) + (zb * zb * zb)) / 24.0 - L * (-a2 + b2) / 16.0 - L * (zb - za) / 8.0);
            double s = 0.0;
            for (int c = 0; c < 6; ++c) s += T[c][i] * Rl[c];
            val += s;
        }
    }
    return val;
}

__global__ void k_fem_dynamic(FemKernelArgs a) {
    const int f = blockIdx.x;
    if (f >= a.nfil || (a.skip && *a.skip)) return;
    const int d0 = a.dof_off[f], nd = a.dof_off[f + 1] - d0;
    const int e0 = a.el_off[f], ne = a.el_off[f + 1] - e0;
    const int mk0 = a.mk_off[f], nmk = a.mk_off[f + 1] - mk0;
    const int bc = a.bc[f];
    extern __shared__ double fem_smem[];
    double *M = a.M + (size_t)f * a.maxdof * a.maxdof;
    double *K = a.k_in_smem ? fem_smem : a.K + (size_t)f * a.maxdof * a.maxdof;
    double *Meff = a.tmp + 2 * (size_t)d0, *MF = a.tmp + 2 * (size_t)d0 + nd;
    __shared__ int ipiv[512], lim[512], rl[32], cl[32];
    __shared__ double sq[512], xs[512], rd[512];
    __shared__ float sdf[512], yf[512];  // FP32 factors: the scale and the solve's vector
    __shared__ volatile int lu_progress;
    __shared__ int go;
    const int n32 = nd - bc;
    float *Kf = reinterpret_cast<float *>(fem_smem + (size_t)a.maxdof * a.maxdof);  // lu32 only
    const double Dt = a.dt;
    double *Kc = a.Kc + (size_t)f * a.maxdof * a.maxdof;
    int *ipc = a.ipc + (size_t)f * a.maxdof, *limc = a.limc + (size_t)f * a.maxdof;
    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
        a.U[d0 + i] = a.U_n[d0 + i];
        a.Ud[d0 + i] = a.Ud_n[d0 + i];
        a.Udd[d0 + i] = a.Udd_n[d0 + i];
    }
    __syncthreads();
    update_values(a, f);
    const double forceScale = a.dm[f] / (Dt * Dt);
    for (int d = threadIdx.x; d < nd; d += blockDim.x) a.R[d0 + d] = load_entry(a, f, d, forceScale);
    __syncthreads();
    const double a0 = 1.0 / (kNbAlpha * (Dt * Dt)), a2 = 1.0 / (kNbAlpha * Dt), a3 = 1.0 / (2.0 * kNbAlpha) - 1.0;
    int it = 0;
    double res = 0.0;
    do {
        if (it == 0 && a.cache_mode == 2 && a.lu32) {
            // as below, with the FP32 factors and the scale kept after them
            const float *Kcf = reinterpret_cast<const float *>(Kc);
            for (int q = threadIdx.x; q < n32 * n32; q += blockDim.x) Kf[q] = Kcf[q];
            for (int i = threadIdx.x; i < n32; i += blockDim.x) {
                sdf[i] = Kcf[(size_t)n32 * n32 + i];
                ipiv[i] = ipc[i];
                lim[i] = limc[i];
            }
            for (int i = threadIdx.x; i < nd; i += blockDim.x) {
                const double v = a.R[d0 + i] - a.Fc[d0 + i] + a.MFc[d0 + i];
                a.Fv[d0 + i] = v;
                a.delU[d0 + i] = v;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < n32; i += blockDim.x) yf[i] = (float)(sdf[i] * a.delU[d0 + bc + i]);
            __syncthreads();
            if (threadIdx.x < 32) lu32_solve_t(Kf, n32, n32, ipiv, 5, lim, yf);
            __syncthreads();
            for (int i = threadIdx.x; i < n32; i += blockDim.x) a.delU[d0 + bc + i] = (double)sdf[i] * (double)yf[i];
            __syncthreads();
        } else if (it == 0 && a.cache_mode == 2) {
            // the step's first Newton iteration again: its factors, internal
            // force and mass term from the step's first call, this call's load
            for (int q = threadIdx.x; q < nd * nd; q += blockDim.x) K[q] = Kc[q];
            for (int i = threadIdx.x; i < nd - bc; i += blockDim.x) {
                ipiv[i] = ipc[i];
                lim[i] = limc[i];
            }
            for (int i = threadIdx.x; i < nd; i += blockDim.x) {
                const double v = a.R[d0 + i] - a.Fc[d0 + i] + a.MFc[d0 + i];
                a.Fv[d0 + i] = v;
                a.delU[d0 + i] = v;
            }
            __syncthreads();
            if (threadIdx.x < 32) lu_solve_factored(K, nd, bc, nd - bc, ipiv, a.delU + d0 + bc, 5, lim, xs, rd);
            __syncthreads();
        } else {
        for (int t = threadIdx.x; t < 4 * ne; t += blockDim.x) {
            const int part = t / ne, e = t - part * ne;
            if (part == 0) element_matrices<0>(a, f, e);
            else if (part == 1) element_matrices<1>(a, f, e);
            else if (part == 2) element_matrices<2>(a, f, e);
            else element_matrices<3>(a, f, e);
        }
        for (int q = threadIdx.x; q < nd * nd; q += blockDim.x) {
            M[q] = 0.0;
            K[q] = 0.0;
        }
        __syncthreads();
        // F, M, K assembly (assembleGlobalMat into zeroed arrays): an entry
        // gets at most two element terms (adjacent elements share one node),
        // and a sum of two terms does not depend on their order, so the
        // element blocks are added even elements first, then odd ones
        for (int d = threadIdx.x; d < nd; d += blockDim.x) {
            double s = 0.0;
            for (int e = (d / 3 - 1 < 0 ? 0 : d / 3 - 1); e <= (d / 3 > ne - 1 ? ne - 1 : d / 3); ++e) {
                const int i = d - 3 * e;
                if (i < 0 || i > 5) continue;
                s += a.elF[6 * (e0 + e) + i];
            }
            a.Fv[d0 + d] = s;
        }
        for (int pass = 0; pass < 2; ++pass) {
            const int nb = (ne + 1 - pass) / 2;
            for (int t = threadIdx.x; t < nb * 36; t += blockDim.x) {
                const int e = 2 * (t / 36) + pass, ij = t % 36;
                const size_t q = (size_t)(3 * e + ij / 6) * nd + (3 * e + ij % 6);
                M[q] += a.elM[36 * (size_t)(e0 + e) + ij];
                K[q] += a.elK[36 * (size_t)(e0 + e) + ij];
            }
            __syncthreads();
        }
        // FEMBody::setNewmark (:264-293)
        for (int i = threadIdx.x; i < nd; i += blockDim.x)
            Meff[i] = a0 * (a.U_n[d0 + i] - a.U[d0 + i]) + a2 * a.Ud[d0 + i] + a3 * a.Udd[d0 + i];
        __syncthreads();
        // M is zero outside the three node columns around row i's node
        for (int i = threadIdx.x; i < nd; i += blockDim.x) {
            const int jlo = 3 * (i / 3) - 3 < 0 ? 0 : 3 * (i / 3) - 3;
            const int jhi = 3 * (i / 3) + 6 > nd ? nd : 3 * (i / 3) + 6;
            double s = 0.0;
            for (int j = jlo; j < jhi; ++j) s += M[(size_t)i * nd + j] * Meff[j];
            MF[i] = s;
        }
        __syncthreads();
        const bool keep = it == 0 && a.cache_mode == 1;
        for (int i = threadIdx.x; i < nd; i += blockDim.x) {
            if (keep) {
                a.Fc[d0 + i] = a.Fv[d0 + i];
                a.MFc[d0 + i] = MF[i];
            }
            a.Fv[d0 + i] = a.R[d0 + i] - a.Fv[d0 + i] + MF[i];
        }
        for (int t = threadIdx.x; t < nd * 9; t += blockDim.x) {
            const int i = t / 9, j = 3 * (i / 3) - 3 + t % 9;
            if (j < 0 || j >= nd) continue;
            K[(size_t)i * nd + j] += a0 * M[(size_t)i * nd + j];
        }
        for (int i = threadIdx.x; i < nd; i += blockDim.x) a.delU[d0 + i] = a.Fv[d0 + i];
        __syncthreads();
        if (a.lu32) {
            // scale rows and columns by 1/sqrt|K_ii| (the diagonal holds
            // a0 M_ii > 0), factor and solve in FP32 (the column-major view
            // of K, transposed solve, as below), unscale the update
            for (int i = threadIdx.x; i < n32; i += blockDim.x) {
                const double kii = fabs(K[(size_t)(bc + i) * nd + bc + i]);
                sdf[i] = kii > 0.0 ? (float)(1.0 / sqrt(kii)) : 1.0f;
            }
            for (int q = threadIdx.x; q < n32 * n32; q += blockDim.x) Kf[q] = 0.0f;
            __syncthreads();
            // K is zero more than 5 off the diagonal (an element couples
            // the DOFs of two adjacent nodes): only the band is converted
            for (int t = threadIdx.x; t < n32 * 11; t += blockDim.x) {
                const int c = t / 11, r = c - 5 + (t - c * 11);  // Kf(r, c) = s_r K[bc+c][bc+r] s_c
                if (r < 0 || r >= n32) continue;
                const double v = K[(size_t)(bc + c) * nd + bc + r];
                Kf[c * n32 + r] = (float)((double)sdf[r] * v * (double)sdf[c]);
            }
            for (int i = threadIdx.x; i < n32; i += blockDim.x) yf[i] = (float)(sdf[i] * a.delU[d0 + bc + i]);
            __syncthreads();
            if (threadIdx.x < 32) {
                lu32_factor(Kf, n32, n32, ipiv, 5, lim);
                lu32_solve_t(Kf, n32, n32, ipiv, 5, lim, yf);
            }
            __syncthreads();
            for (int i = threadIdx.x; i < n32; i += blockDim.x) a.delU[d0 + bc + i] = (double)sdf[i] * (double)yf[i];
            if (keep) {
                float *Kcf = reinterpret_cast<float *>(Kc);
                for (int q = threadIdx.x; q < n32 * n32; q += blockDim.x) Kcf[q] = Kf[q];
                for (int i = threadIdx.x; i < n32; i += blockDim.x) {
                    Kcf[(size_t)n32 * n32 + i] = sdf[i];
                    ipc[i] = ipiv[i];
                    limc[i] = lim[i];
                }
            }
            __syncthreads();
        } else {
        // an element couples the 6 DOFs of its two nodes: half-bandwidth 5.
        // Warp 0 factors; warp 1 (another FP64 unit) runs the forward solve
        // one column behind it; warp 0 then solves backward.
        if (threadIdx.x == 0) lu_progress = 0;
        __syncthreads();
        if (threadIdx.x < 32)
            lu_factor_banded<7>(K, nd, bc, nd - bc, ipiv, 5, lim, rl, cl, &lu_progress, false);
        else if (threadIdx.x < 64)
            lu_forward(K, nd, bc, nd - bc, a.delU + d0 + bc, 5, xs, rd, &lu_progress, a.error);
        else if (threadIdx.x < 96)
            lu_l_swaps(K, nd, bc, nd - bc, ipiv, lim, &lu_progress, a.error);
        __syncthreads();
        if (threadIdx.x < 32) lu_backward(K, nd, bc, nd - bc, ipiv, a.delU + d0 + bc, lim, xs);
        __syncthreads();
        if (keep) {
            for (int q = threadIdx.x; q < nd * nd; q += blockDim.x) Kc[q] = K[q];
            for (int i = threadIdx.x; i < nd - bc; i += blockDim.x) {
                ipc[i] = ipiv[i];
                limc[i] = lim[i];
            }
        }
        }
        }
        for (int i = threadIdx.x; i < bc; i += blockDim.x) a.delU[d0 + i] = 0.0;
        __syncthreads();
        // the squares of the residual's sum formed densely beforehand; one
        // thread adds them in order
        for (int i = threadIdx.x; i < nd; i += blockDim.x) {
            const double du = a.delU[d0 + i];
            a.U[d0 + i] = a.U[d0 + i] + du;
            sq[i] = du * du;
        }
        __syncthreads();
        update_values(a, f);
        if (threadIdx.x == 0) {
            double dp = 0.0;
            for (int i = 0; i < nd; i++) dp += sq[i];
            const double L = a.len0[e0] * ne;
            res = sqrt(dp / (double)nd) / L;
            go = (res > 1e-10 && it + 1 < 20) ? 1 : 0;
        }
        __syncthreads();
        ++it;
    } while (go);
    // FEMBody::finishNewmark (:236-255)
    const double a6 = 1.0 / (kNbAlpha * (Dt * Dt)), a7 = -1.0 / (kNbAlpha * Dt), a8 = -(1.0 / (2.0 * kNbAlpha) - 1.0);
    const double a9 = Dt * (1.0 - kNbDelta), a10 = kNbDelta * Dt;
    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
        const double s = a6 * (a.U[d0 + i] - a.U_n[d0 + i]) + a7 * a.Ud[d0 + i] + a8 * a.Udd[d0 + i];
        a.Ud[d0 + i] = a.Ud[d0 + i] + a9 * a.Udd[d0 + i] + a10 * s;
        a.Udd[d0 + i] = s;
    }
    if (threadIdx.x == 0) {
        a.it[f] = it;
        a.res[f] = res;
    }
    __syncthreads();
    // FEMBody::updateIBMarkers (:329-370)
    for (int m = threadIdx.x; m < nmk; m += blockDim.x) {
        const int e = a.parent_el[mk0 + m];
        const int ge = e0 + e;
        const double z = a.parent_zeta[mk0 + m];
        double T[6][6];
        Tmat(a.elang[ge], T);
        double lU[6], lV[6];
        for (int r = 0; r < 6; ++r) {
            double s1 = 0.0, s2 = 0.0;
            for (int c = 0; c < 6; ++c) {
                s1 += T[r][c] * a.U[d0 + e * 3 + c];
                s2 += T[r][c] * a.Ud[d0 + e * 3 + c];
            }
            lU[r] = s1;
            lV[r] = s2;
        }
        const double zz = (z + 1.0) / 2.0, L = a.ellen[ge];
        const double N0 = 1.0 - (z + 1.0) / 2.0;
        const double N1 = 1.0 - 3.0 * (zz * zz) + 2.0 * (zz * zz * zz);
        const double N2 = (zz - 2.0 * (zz * zz) + (zz * zz * zz)) * L;
        const double N3 = (z + 1.0) / 2.0;
        const double N4 = 3.0 * (zz * zz) - 2.0 * (zz * zz * zz);
        const double N5 = (-(zz * zz) + (zz * zz * zz)) * L;
        const double su[2] = {lU[0] * N0 + lU[3] * N3, lU[1] * N1 + lU[2] * N2 + lU[4] * N4 + lU[5] * N5};
        const double sv[2] = {lV[0] * N0 + lV[3] * N3, lV[1] * N1 + lV[2] * N2 + lV[4] * N4 + lV[5] * N5};
        const double Tt[2][2] = {{T[0][0], T[1][0]}, {T[0][1], T[1][1]}};
        const int g = mk0 + m;
        for (int r = 0; r < 2; ++r) {
            double s1 = 0.0, s2 = 0.0;
            for (int c = 0; c < 2; ++c) { s1 += Tt[r][c] * su[c]; s2 += Tt[r][c] * sv[c]; }
            const double gv = s2 * (a.dt / a.dh);
            a.flex.pos[3 * g + r] = a.mpos0[3 * g + r] + s1;
            a.flex.vel_km1[3 * g + r] = a.flex.vel[3 * g + r];
            a.flex.vel[3 * g + r] = kRelax * gv + (1.0 - kRelax) * a.flex.vel_km1[3 * g + r];
        }
    }
}

// The Roma kernel at dilation 1 with its two divisions (by 6 and by 3)
// formed as correctly rounded quotients from the constants' reciprocals
// (quotient(): the same bits as the division, fewer FP64 operations).
__device__ __forceinline__ double roma(double radius) {
    const double mag_r = fabs(radius);  // |r| / 1.0
    if (mag_r > 1.5) return 0.0;
    if (mag_r > 0.5) return quotient(5.0 - (3.0 * mag_r) - sqrt(-3.0 * ((1.0 - mag_r) * (1.0 - mag_r)) + 1.0), 6.0, 1.0 / 6.0);
    return quotient(1.0 + sqrt(1.0 - 3.0 * (mag_r * mag_r)), 3.0, 1.0 / 3.0);
}


// Supports, ds and epsilon of one filament's markers (ibm_findSupport,
// ibm_computeDs, ibm_findEpsilon for a moving body).
//
// A marker's supports are the nodes of its cage: per axis the five
// candidate coordinates around its near node (offsets -2..2), each with the
// cage test |X - x|/dh < 1.5, the domain test and its kernel value; a
// support node's coordinates, tests and delta are combinations of these.
// So the kernel first forms every marker's cage record (x.cage: the 15
// coordinates and 15 kernel values; x.cagei: the near node and the test
// bits), one thread per (marker, axis, offset); then lists each marker's
// supports in the reference's order (the near node, then the cage nodes in
// (i, j, k) order); then forms ds over marker pairs; then each epsilon entry
// (I, J) evaluates J's kernel at I's candidate coordinates and sums
// delta_I * phi_J over I's supports in the same order.  Every value is the
// same expression on the same operands as node by node.
constexpr int kEpsChunk = 2048;  // epsilon entries tested per round

__device__ __forceinline__ bool cage_ok(unsigned fl, int d, int o) { return ((fl >> (5 * d + o)) & 1u) != 0; }

__global__ void k_flex_support(FemKernelArgs a) {
    const int f = blockIdx.x;
    if (f >= a.nfil || (a.skip && *a.skip)) return;
    const int mk0 = a.mk_off[f], nmk = a.mk_off[f + 1] - mk0;
    const int D = a.dims;
    const double dh = a.dh, rdh = 1.0 / dh;  // divisions by dh as quotient(., dh, rdh)
    const FlexArgs &x = a.flex;
    // near node per (marker, axis); the test bits start clear, ds at 10
    for (int q = threadIdx.x; q < 3 * nmk; q += blockDim.x) {
        const int m = q / 3, d = q % 3, g = mk0 + m;
        x.cagei[4 * g + d] = d < D ? (int)floor(quotient(x.pos[3 * g + d] - a.gstart[d], dh, rdh)) : 0;
        if (d == 0) {
            x.cagei[4 * g + 3] = 0;
            x.ds[g] = 10.0;
        }
    }
    __syncthreads();
    // cage record per (marker, axis, offset)
    for (int q = threadIdx.x; q < 15 * nmk; q += blockDim.x) {
        const int m = q / 15, w = q % 15, d = w / 5, o = w % 5, g = mk0 + m;
        const int *ni = &x.cagei[4 * g];
        if (ni[0] < 0 || ni[1] < 0 || ni[2] < 0 || ni[0] >= a.N || ni[1] >= a.M_ || ni[2] >= a.K_) continue;
        const bool act = d < D;
        const double *h = d == 0 ? a.hx : d == 1 ? a.hy : a.hz;
        const double nearp = act ? h[ni[d]] : 0.0;
        const double p = x.pos[3 * g + d];
        const double e = act ? nearp + (o - 2) * dh : nearp;
        const bool cage = !act || quotient(fabs(p - e), dh, rdh) < 1.5;
        const bool dom = !act || !(e < a.edges[2 * d] || e > a.edges[2 * d + 1]);
        x.cage[32 * (size_t)g + w] = e;
        x.cage[32 * (size_t)g + 15 + w] = act ? roma(quotient(e - p, dh, rdh)) : 1.0;
        if (cage && dom) atomicOr(&x.cagei[4 * g + 3], 1 << w);
    }
    __syncthreads();
    // support lists
    for (int m = threadIdx.x; m < nmk; m += blockDim.x) {
        const int g = mk0 + m;
        const int in = x.cagei[4 * g], jn = x.cagei[4 * g + 1], kn = x.cagei[4 * g + 2];
        const unsigned fl = (unsigned)x.cagei[4 * g + 3];
        if (in < 0 || jn < 0 || kn < 0 || in >= a.N || jn >= a.M_ || kn >= a.K_) {
            atomicExch(a.error, 1);
            x.nsupp[g] = 0;
            continue;
        }
        const double *rec = &x.cage[32 * (size_t)g];
        int ns = 0;
        auto add = [&](int i, int j, int k, int oi, int oj, int ok) {
            if (ns >= kFlexMaxSupp) { atomicExch(a.error, 2); return; }
            const int s = g * kFlexMaxSupp + ns;
            x.supp[s] = k + j * a.K_ + i * a.K_ * a.M_;
            x.sx[s] = rec[oi]; x.sy[s] = rec[5 + oj]; x.sz[s] = rec[10 + ok];
            double v = rec[15 + oi] * rec[20 + oj];
            if (D == 3) v = v * rec[25 + ok];
            x.delta[s] = v;
            ++ns;
        };
        add(in, jn, kn, 2, 2, 2);
        // the reference scans +-5 nodes; every cage node (< 1.5 dh from the
        // marker, which is < 1 dh from the near node) lies within +-2, met
        // in the same (i, j, k) order
        for (int oi = 0; oi < 5; oi++)
            for (int oj = 0; oj < 5; oj++)
                for (int ok = (D == 3 ? 0 : 2); ok <= (D == 3 ? 4 : 2); ok++) {
                    const int i = in + oi - 2, j = jn + oj - 2, k = kn + ok - 2;
                    if (cage_ok(fl, 0, oi) && cage_ok(fl, 1, oj) && cage_ok(fl, 2, ok) && (oi != 2 || oj != 2 || ok != 2)) {
                        if (i < 0 || j < 0 || k < 0 || i >= a.N || j >= a.M_ || k >= a.K_) {
                            atomicExch(a.error, 1);
                            continue;
                        }
                        add(i, j, k, oi, oj, ok);
                    }
                }
        x.nsupp[g] = ns;
    }
    // ds: the smallest distance to another marker of the filament, in dh
    // (10 when none is nearer); a minimum of non-negative doubles is the
    // minimum of their bit patterns
    for (int q = threadIdx.x; q < nmk * nmk; q += blockDim.x) {
        const int m = q / nmk, o = q % nmk;
        if (m == o) continue;
        const int g = mk0 + m, h = mk0 + o;
        double r = 0.0;
        for (int d = 0; d < 3; ++d) {
            const double v = x.pos[3 * g + d] - x.pos[3 * h + d];
            r += v * v;
        }
        const double dist = quotient(sqrt(r), dh, rdh);
        if (dist < 10.0)
            atomicMin(reinterpret_cast<unsigned long long *>(&x.ds[g]), (unsigned long long)__double_as_longlong(dist));
    }
    __syncthreads();
    extern __shared__ double flex_smem[];
    double *A = a.eps_in_smem ? flex_smem : a.epsA + (size_t)f * a.maxmk * a.maxmk;
    // Entries in chunks: each thread tests its share of a chunk, writes the
    // entries of markers more than 3 dh apart on an axis (they share no
    // support node: every term is an exact zero and the entry stays +0)
    // and lists the others, which are then evaluated one per lane, densely.
    __shared__ int near_list[kEpsChunk];
    __shared__ int near_count;
    for (int q0 = 0; q0 < nmk * nmk; q0 += kEpsChunk) {
        if (threadIdx.x == 0) near_count = 0;
        __syncthreads();
        for (int q = q0 + threadIdx.x; q < min(nmk * nmk, q0 + kEpsChunk); q += blockDim.x) {
            const int I = q / nmk, J = q % nmk;
            const int gI = mk0 + I, gJ = mk0 + J;
            bool near = x.nsupp[gI] > 0;
            for (int d = 0; d < D; ++d) near = near && fabs(x.pos[3 * gI + d] - x.pos[3 * gJ + d]) <= 3.01 * dh;
            if (near) near_list[atomicAdd(&near_count, 1)] = q;
            else A[(size_t)I * nmk + J] = 0.0 * x.ds[gJ];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < near_count; t += blockDim.x) {
            const int q = near_list[t];
            const int I = q / nmk, J = q % nmk;
            const int gI = mk0 + I, gJ = mk0 + J;
            double aij = 0.0;
            const double *rec = &x.cage[32 * (size_t)gI];
            const unsigned fl = (unsigned)x.cagei[4 * gI + 3];
            const int ni[3] = {x.cagei[4 * gI], x.cagei[4 * gI + 1], x.cagei[4 * gI + 2]};
            double ph[15], fj[15];
#pragma unroll
            for (int w = 0; w < 15; ++w) ph[w] = rec[15 + w];
            // J's kernel at I's candidate coordinates (those a support uses)
#pragma unroll
            for (int w = 0; w < 15; ++w) {
                const int d = w / 5;
                fj[w] = 0.0;
                if (d < D && (w % 5 == 2 || cage_ok(fl, d, w % 5)))
                    fj[w] = roma(quotient(x.pos[3 * gJ + d] - rec[w], dh, rdh));
            }
            int ns = 0;
            auto term = [&](int oi, int oj, int ok) {
                if (ns >= kFlexMaxSupp) return;
                double dl = ph[oi] * ph[5 + oj];
                if (D == 3) dl = dl * ph[10 + ok];
                double dJ = fj[oi] * fj[5 + oj];
                if (D == 3) dJ = dJ * fj[10 + ok];
                aij += dl * dJ * 1.0;
                ++ns;
            };
            term(2, 2, 2);
#pragma unroll
            for (int oi = 0; oi < 5; oi++)
#pragma unroll
                for (int oj = 0; oj < 5; oj++)
#pragma unroll
                    for (int ok = 0; ok < 5; ok++) {
                        if (D != 3 && ok != 2) continue;
                        const int i = ni[0] + oi - 2, j = ni[1] + oj - 2, k = ni[2] + ok - 2;
                        if (cage_ok(fl, 0, oi) && cage_ok(fl, 1, oj) && cage_ok(fl, 2, ok) &&
                            (oi != 2 || oj != 2 || ok != 2) && !(i < 0 || j < 0 || k < 0 || i >= a.N ||
                                                                 j >= a.M_ || k >= a.K_))
                            term(oi, oj, ok);
                    }
            A[(size_t)I * nmk + J] = aij * x.ds[gJ];
        }
        __syncthreads();
    }
    __shared__ int ipiv[512];
    __shared__ int band;
    if (threadIdx.x == 0) band = 0;
    for (int m = threadIdx.x; m < nmk; m += blockDim.x) x.eps[mk0 + m] = 1.0;
    __syncthreads();
    // markers share support nodes only within a few dh of each other: along
    // a filament the system is banded, which bounds the solver's scans
    for (int q = threadIdx.x; q < nmk * nmk; q += blockDim.x) {
        const int off = q / nmk - q % nmk;
        if (!is_zero(A[q])) atomicMax(&band, off < 0 ? -off : off);
    }
    __syncthreads();
    lu_solve_block(A, nmk, 0, nmk, ipiv, x.eps + mk0, band < nmk ? band : nmk, a.error);
}

// max over flexible markers of |U - U_km1| / (L_UX0 dt/dh)  (ibm_checkVelDiff)
__global__ void k_fsi_residual(FemKernelArgs a) {
    const int f = blockIdx.x;
    if (f >= a.nfil || (a.skip && *a.skip)) return;
    const int mk0 = a.mk_off[f], nmk = a.mk_off[f + 1] - mk0;
    for (int m = threadIdx.x; m < nmk; m += blockDim.x) {
        const int g = mk0 + m;
        double r = 0.0;
        for (int d = 0; d < 3; ++d) {
            const double v = a.flex.vel[3 * g + d] - a.flex.vel_km1[3 * g + d];
            r += v * v;
        }
        const double v = fabs(sqrt(r) / a.velscale[f]);
        atomicMax(reinterpret_cast<unsigned long long *>(a.fsi_res), (unsigned long long)__double_as_longlong(v));
    }
}

// The FSI sub-iterations of a step (ibm_subIterate, src/ObjectManager_ops_ibm.cpp:
// 111-185) run without the host: all ten are enqueued, and after each one
// k_fsi_decide applies the loop test (another iteration while the residual
// is above 1e-4); once it fails, every kernel of the later iterations
// returns at once.  Nothing waits on the flag.
__global__ void k_fsi_begin(int *state, double *res) {
    state[0] = 0;
    state[1] = 0;
    res[0] = 0.0;
}
__global__ void k_fsi_decide(int *state, double *res) {
    if (state[0]) return;
    state[1] += 1;
    res[1] = res[0];
    res[0] = 0.0;
    if (!(res[1] > 1e-4)) state[0] = 1;
}
// u <- u_n (the velocity at the start of the step) for the next
// sub-iteration, unless the loop has converged; 4-byte words, 16 at a time.
__global__ void k_restore_u(const int *skip, uint32_t *__restrict__ dst, const uint32_t *__restrict__ src,
                            size_t words) {
    if (*skip) return;
    const size_t nv = words / 4;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride)
        reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(src)[i];
    for (size_t i = 4 * nv + (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += stride) dst[i] = src[i];
}

__global__ void k_fem_commit(FemKernelArgs a, int ndof_total) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ndof_total) return;
    a.U_n[i] = a.U[i];
    a.Ud_n[i] = a.Ud[i];
    a.Udd_n[i] = a.Udd[i];
}

FemKernelArgs make_fem_args(luma_gpu_grid *g) {
    FemDevice &d = g->ibm->fem;
    FemKernelArgs a;
    memset(&a, 0, sizeof a);
    a.nfil = d.nfil; a.maxdof = d.maxdof; a.maxmk = d.maxmk;
    a.node_off = d.node_off; a.el_off = d.el_off; a.dof_off = d.dof_off; a.mk_off = d.mk_off; a.bc = d.bc;
    a.dm = d.dm; a.velscale = d.velscale;
    a.pos0 = d.pos0; a.ang0 = d.ang0;
    a.len0 = d.len0; a.area = d.area; a.I = d.I; a.E = d.E; a.rho = d.rho;
    a.child_off = d.child_off; a.child_node = d.child_node; a.child_z1 = d.child_z1; a.child_z2 = d.child_z2;
    a.U = d.U; a.U_n = d.U_n; a.Ud = d.Ud; a.Ud_n = d.Ud_n; a.Udd = d.Udd; a.Udd_n = d.Udd_n;
    a.R = d.R; a.Fv = d.Fv; a.delU = d.delU;
    a.M = d.M; a.K = d.K; a.epsA = d.epsA;
    a.parent_el = d.parent_el; a.parent_zeta = d.parent_zeta; a.mpos0 = d.mpos0;
    a.it = d.it; a.res = d.res; a.fsi_res = d.fsi_res; a.fsi_state = d.fsi_state;
    a.Kc = d.Kc; a.Fc = d.Fc; a.MFc = d.MFc; a.ipc = d.ipc; a.limc = d.limc;
    a.dt = g->d.dt; a.dh = g->d.dh;
    a.flex = d.flex;
    a.N = g->d.N; a.M_ = g->d.M; a.K_ = g->d.K; a.dims = g->d.dims; a.level = g->d.level;
    return a;
}

}  // namespace

// ---- host side -------------------------------------------------------------

struct FemScratch {
    double *elF = nullptr, *elM = nullptr, *elK = nullptr, *elang = nullptr, *ellen = nullptr;
    double *npos = nullptr, *nang = nullptr, *tmp = nullptr;
    double *hx = nullptr, *hy = nullptr, *hz = nullptr;
    int *error = nullptr;
};
static std::vector<std::pair<luma_gpu_grid *, FemScratch>> g_scratch;

static FemScratch *scratch_of(luma_gpu_grid *g) {
    for (auto &p : g_scratch)
        if (p.first == g) return &p.second;
    return nullptr;
}

template <class T>
static int up(T **dst, const std::vector<T> &src) {
    cudaFree(*dst);
    *dst = nullptr;
    if (cudaMalloc(dst, std::max<size_t>(1, src.size()) * sizeof(T)) != cudaSuccess)
        return luma_set_error(LUMA_E_NOMEM, "FEM device allocation failed");
    if (!src.empty() && cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return luma_set_error(LUMA_E_CUDA, "FEM upload failed");
    return LUMA_OK;
}
template <class T>
static int zeros(T **dst, size_t n) {
    return up(dst, std::vector<T>(n, T(0)));
}

// Upload every filament of the grid (called once by luma_gpu_ibm_initialise).
// A kernel's dynamic shared-memory limit holds for every launch on its
// device: grids set up later with smaller matrices must not lower it under
// earlier ones, so it only ever rises (per device and kernel, under a lock).
static bool raise_smem_limit(const void *kernel, size_t bytes) {
    struct Limit {
        int dev;
        const void *kernel;
        size_t bytes;
    };
    static std::mutex mu;
    static std::vector<Limit> set;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    std::lock_guard<std::mutex> lock(mu);
    for (Limit &e : set)
        if (e.dev == dev && e.kernel == kernel) {
            if (bytes <= e.bytes) return true;
            if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
                return false;
            e.bytes = bytes;
            return true;
        }
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) return false;
    set.push_back({dev, kernel, bytes});
    return true;
}

int luma_fem_upload(luma_gpu_grid *g) {
    IbmState &st = *g->ibm;
    FemDevice &d = st.fem;
    std::vector<int> node_off(1, 0), el_off(1, 0), dof_off(1, 0), mk_off(1, 0), bc, child_off(1, 0), child_node,
        parent_el;
    std::vector<double> dm, vs, pos0, ang0, len0, area, I, E, rho, cz1, cz2, pz, mpos0, mvel, mpos;
    int maxdof = 0, maxmk = 0;
    for (size_t k = 0; k < st.flex.size(); ++k) {
        const FlexBody &fb = st.flex[k];
        const IbmBody &ib = st.bodies[st.flex_body[k]];
        bc.push_back(fb.bc);
        dm.push_back(fb.dm);
        vs.push_back(fb.velscale);
        pos0.insert(pos0.end(), fb.pos0.begin(), fb.pos0.end());
        ang0.insert(ang0.end(), fb.ang0.begin(), fb.ang0.end());
        for (int e = 0; e < fb.nel; ++e) {
            len0.push_back(fb.len0[e]); area.push_back(fb.area[e]); I.push_back(fb.I[e]); E.push_back(fb.E[e]);
            rho.push_back(fb.rho[e]);
            for (int q = fb.child_off[e]; q < fb.child_off[e + 1]; ++q) {
                child_node.push_back(fb.child_node[q]);
                cz1.push_back(fb.child_z1[q]);
                cz2.push_back(fb.child_z2[q]);
            }
            child_off.push_back((int)child_node.size());
        }
        parent_el.insert(parent_el.end(), fb.parent_el.begin(), fb.parent_el.end());
        pz.insert(pz.end(), fb.parent_zeta.begin(), fb.parent_zeta.end());
        mpos0.insert(mpos0.end(), fb.mpos0.begin(), fb.mpos0.end());
        mpos.insert(mpos.end(), ib.pos.begin(), ib.pos.end());
        mvel.insert(mvel.end(), ib.vel.begin(), ib.vel.end());
        node_off.push_back(node_off.back() + fb.nel + 1);
        el_off.push_back(el_off.back() + fb.nel);
        dof_off.push_back(dof_off.back() + 3 * (fb.nel + 1));
        mk_off.push_back(mk_off.back() + fb.nm);
        maxdof = std::max(maxdof, 3 * (fb.nel + 1));
        maxmk = std::max(maxmk, fb.nm);
    }
    if (maxdof > 512 || maxmk > 512) return luma_set_error(LUMA_E_INVALID, "filament too large for the device solver");
    d.nfil = (int)st.flex.size();
    d.maxdof = maxdof;
    d.maxmk = maxmk;
    const int ndof = dof_off.back(), nmk = mk_off.back(), nel = el_off.back(), nnode = node_off.back();
    int rc;
    if ((rc = up(&d.node_off, node_off)) || (rc = up(&d.el_off, el_off)) || (rc = up(&d.dof_off, dof_off)) ||
        (rc = up(&d.mk_off, mk_off)) || (rc = up(&d.bc, bc)) || (rc = up(&d.dm, dm)) || (rc = up(&d.velscale, vs)) ||
        (rc = up(&d.pos0, pos0)) || (rc = up(&d.ang0, ang0)) || (rc = up(&d.len0, len0)) || (rc = up(&d.area, area)) ||
        (rc = up(&d.I, I)) || (rc = up(&d.E, E)) || (rc = up(&d.rho, rho)) || (rc = up(&d.child_off, child_off)) ||
        (rc = up(&d.child_node, child_node)) || (rc = up(&d.child_z1, cz1)) || (rc = up(&d.child_z2, cz2)) ||
        (rc = up(&d.parent_el, parent_el)) || (rc = up(&d.parent_zeta, pz)) || (rc = up(&d.mpos0, mpos0)))
        return rc;
    if ((rc = zeros(&d.U, ndof)) || (rc = zeros(&d.U_n, ndof)) || (rc = zeros(&d.Ud, ndof)) ||
        (rc = zeros(&d.Ud_n, ndof)) || (rc = zeros(&d.Udd, ndof)) || (rc = zeros(&d.Udd_n, ndof)) ||
        (rc = zeros(&d.R, ndof)) || (rc = zeros(&d.Fv, ndof)) || (rc = zeros(&d.delU, ndof)) ||
        (rc = zeros(&d.M, (size_t)d.nfil * maxdof * maxdof)) || (rc = zeros(&d.K, (size_t)d.nfil * maxdof * maxdof)) ||
        (rc = zeros(&d.epsA, (size_t)d.nfil * maxmk * maxmk)) || (rc = zeros(&d.it, d.nfil)) ||
        (rc = zeros(&d.res, d.nfil)) || (rc = zeros(&d.fsi_res, 2)) ||
        (rc = zeros(&d.fsi_state, 2)) || (rc = zeros(&d.Kc, (size_t)d.nfil * maxdof * maxdof)) ||
        (rc = zeros(&d.Fc, ndof)) || (rc = zeros(&d.MFc, ndof)) || (rc = zeros(&d.ipc, (size_t)d.nfil * maxdof)) ||
        (rc = zeros(&d.limc, (size_t)d.nfil * maxdof)))
        return rc;
    FlexArgs &x = d.flex;
    x.nm = nmk;
    x.dims = g->d.dims;
    if ((rc = up(&x.pos, mpos)) || (rc = up(&x.vel, mvel)) || (rc = zeros(&x.vel_km1, 3 * (size_t)nmk)) ||
        (rc = zeros(&x.F, 3 * (size_t)nmk)) || (rc = zeros(&x.eps, nmk)) || (rc = zeros(&x.ds, nmk)) ||
        (rc = zeros(&x.irho, nmk)) || (rc = zeros(&x.imom, 3 * (size_t)nmk)) || (rc = zeros(&x.nsupp, nmk)) ||
        (rc = zeros(&x.supp, (size_t)nmk * kFlexMaxSupp)) || (rc = zeros(&x.delta, (size_t)nmk * kFlexMaxSupp)) ||
        (rc = zeros(&x.sx, (size_t)nmk * kFlexMaxSupp)) || (rc = zeros(&x.sy, (size_t)nmk * kFlexMaxSupp)) ||
        (rc = zeros(&x.sz, (size_t)nmk * kFlexMaxSupp)) || (rc = zeros(&x.cage, 32 * (size_t)nmk)) ||
        (rc = zeros(&x.cagei, 4 * (size_t)nmk)))
        return rc;
    FemScratch sc;
    if ((rc = zeros(&sc.elF, 6 * (size_t)nel)) || (rc = zeros(&sc.elM, 36 * (size_t)nel)) ||
        (rc = zeros(&sc.elK, 36 * (size_t)nel)) || (rc = zeros(&sc.elang, nel)) || (rc = zeros(&sc.ellen, nel)) ||
        (rc = zeros(&sc.npos, 3 * (size_t)nnode)) || (rc = zeros(&sc.nang, nnode)) ||
        (rc = zeros(&sc.tmp, 2 * (size_t)ndof)) || (rc = up(&sc.hx, g->hx)) || (rc = up(&sc.hy, g->hy)) ||
        (rc = up(&sc.hz, g->hz)) || (rc = zeros(&sc.error, 1)))
        return rc;
    g_scratch.push_back({g, sc});
    // a filament's stiffness and epsilon matrices in shared memory when they
    // fit; on shifted-FP32 grids the stiffness matrix's FP32 copy after it
    const size_t kb = (size_t)maxdof * maxdof * sizeof(double), eb = (size_t)maxmk * maxmk * sizeof(double);
    const size_t kb32 = kb + (size_t)maxdof * maxdof * sizeof(float);
    d.lu32 = g->d.precision == LUMA_PREC_FP32_SHIFTED && kb32 <= kFemSmemMax &&
             raise_smem_limit(reinterpret_cast<const void *>(k_fem_dynamic), kb32);
    d.k_in_smem = d.lu32 || (kb <= kFemSmemMax && raise_smem_limit(reinterpret_cast<const void *>(k_fem_dynamic), kb));
    d.eps_in_smem = eb <= kFemSmemMax && raise_smem_limit(reinterpret_cast<const void *>(k_flex_support), eb);
    cudaGetLastError();
    st.u_n = nullptr;
    const size_t rs = g->d.precision == LUMA_PREC_FP64 ? 8 : 4;
    if (cudaMalloc(&st.u_n, g->n * g->d.dims * rs) != cudaSuccess)
        return luma_set_error(LUMA_E_NOMEM, "u_n allocation failed");
    return LUMA_OK;
}

static FemKernelArgs full_args(luma_gpu_grid *g) {
    FemKernelArgs a = make_fem_args(g);
    FemScratch *sc = scratch_of(g);
    a.elF = sc->elF; a.elM = sc->elM; a.elK = sc->elK; a.elang = sc->elang; a.ellen = sc->ellen;
    a.npos = sc->npos; a.nang = sc->nang; a.tmp = sc->tmp;
    a.hx = sc->hx; a.hy = sc->hy; a.hz = sc->hz; a.error = sc->error;
    const luma_gpu_grid *r = g;
    while (r->parent) r = r->parent;
    for (int q = 0; q < 6; ++q) a.edges[q] = r->d.global_edges[q];
    for (int ax = 0; ax < 3; ++ax) {
        const std::vector<double> &p = ax == 0 ? g->hx : (ax == 1 ? g->hy : g->hz);
        a.gstart[ax] = g->d.level == 0 ? 0.0 : p[0] - g->d.dh / 2.0;
    }
    return a;
}

// Supports/ds/epsilon of the filaments' markers (initialise and after FEM).
int luma_fem_supports(luma_gpu_grid *g, const int *skip) {
    FemKernelArgs a = full_args(g);
    a.skip = skip;
    const FemDevice &d = g->ibm->fem;
    a.eps_in_smem = d.eps_in_smem;
    const size_t eb = (size_t)a.maxmk * a.maxmk * sizeof(double);
    k_flex_support<<<a.nfil, 256, a.eps_in_smem ? eb : 0, g->stream>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "flex support: %s", cudaGetErrorString(e));
    return LUMA_OK;
}

// ObjectManager::ibm_moveBodies (:61-104) for the filaments of a grid.
// `first`: the step's first FEM call (it keeps its first Newton iteration's
// factors); later calls of the step reuse them.
int luma_fem_move_bodies(luma_gpu_grid *g, const int *skip, bool first) {
    FemKernelArgs a = full_args(g);
    a.skip = skip;
    a.cache_mode = first ? 1 : 2;
    a.k_in_smem = g->ibm->fem.k_in_smem;
    a.lu32 = g->ibm->fem.lu32;
    const size_t kb = (size_t)a.maxdof * a.maxdof * (a.lu32 ? sizeof(double) + sizeof(float) : sizeof(double));
    k_fem_dynamic<<<a.nfil, 128, a.k_in_smem ? kb : 0, g->stream>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "FEM: %s", cudaGetErrorString(e));
    return luma_fem_supports(g, skip);
}

const int *luma_fem_fsi_flag(luma_gpu_grid *g) { return g->ibm->fem.fsi_state; }

int luma_fem_fsi_begin(luma_gpu_grid *g) {
    FemDevice &d = g->ibm->fem;
    k_fsi_begin<<<1, 1, 0, g->stream>>>(d.fsi_state, d.fsi_res);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "FSI begin: %s", cudaGetErrorString(e));
    return LUMA_OK;
}

int luma_fem_restore_u(luma_gpu_grid *g) {
    const size_t bytes = g->n * g->d.dims * (g->d.precision == LUMA_PREC_FP64 ? 8 : 4);
    k_restore_u<<<152 * 4, 256, 0, g->stream>>>(g->ibm->fem.fsi_state, static_cast<uint32_t *>(g->u),
                                                 reinterpret_cast<const uint32_t *>(g->ibm->u_n), bytes / 4);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "FSI u restore: %s", cudaGetErrorString(e));
    return LUMA_OK;
}

// The loop test of one sub-iteration (ibm_checkVelDiff, :988-1032, then
// the while condition of ibm_subIterate), on the device.
int luma_fem_fsi_check(luma_gpu_grid *g) {
    FemKernelArgs a = full_args(g);
    a.skip = a.fsi_state;
    k_fsi_residual<<<a.nfil, 128, 0, g->stream>>>(a);
    k_fsi_decide<<<1, 1, 0, g->stream>>>(a.fsi_state, a.fsi_res);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "FSI residual: %s", cudaGetErrorString(e));
    return LUMA_OK;
}

// A filament marker that left its grid (or overflowed its support slots)
// since the last check: reads and clears the record (blocks on the stream).
int luma_fem_take_error(luma_gpu_grid *g) {
    FemScratch *sc = scratch_of(g);
    if (!sc) return LUMA_OK;
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, sc->error, sizeof(int), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "FEM error read: %s", cudaGetErrorString(e));
    if (!err) return LUMA_OK;
    cudaMemsetAsync(sc->error, 0, sizeof(int), g->stream);
    if (err == 3)
        return luma_set_error(LUMA_E_CUDA, "grid L%d R%d: FEM solve gave up waiting for its factorisation", g->d.level,
                              g->d.region);
    return luma_set_error(LUMA_E_DOMAIN, "grid L%d R%d: a filament marker left its grid (code %d)", g->d.level,
                          g->d.region, err);
}

int luma_fem_commit(luma_gpu_grid *g) {
    FemKernelArgs a = full_args(g);
    int ndof = 0;
    for (const FlexBody &fb : g->ibm->flex) ndof += 3 * (fb.nel + 1);
    k_fem_commit<<<(ndof + 127) / 128, 128, 0, g->stream>>>(a, ndof);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return luma_set_error(LUMA_E_CUDA, "FEM commit: %s", cudaGetErrorString(e));
    return LUMA_OK;
}

void luma_fem_free(luma_gpu_grid *g) {
    for (size_t i = 0; i < g_scratch.size(); ++i)
        if (g_scratch[i].first == g) {
            FemScratch &s = g_scratch[i].second;
            cudaFree(s.elF); cudaFree(s.elM); cudaFree(s.elK); cudaFree(s.elang); cudaFree(s.ellen);
            cudaFree(s.npos); cudaFree(s.nang); cudaFree(s.tmp); cudaFree(s.hx); cudaFree(s.hy); cudaFree(s.hz);
            cudaFree(s.error);
            g_scratch.erase(g_scratch.begin() + i);
            break;
        }
    if (!g->ibm) return;
    FemDevice &d = g->ibm->fem;
    void *ptrs[] = {d.node_off, d.el_off, d.dof_off, d.mk_off, d.bc, d.dm, d.velscale, d.pos0, d.ang0, d.len0,
                    d.area, d.I, d.E, d.rho, d.child_off, d.child_node, d.child_z1, d.child_z2, d.U, d.U_n, d.Ud,
                    d.Ud_n, d.Udd, d.Udd_n, d.R, d.Fv, d.delU, d.M, d.K, d.epsA, d.parent_el, d.parent_zeta,
                    d.mpos0, d.it, d.res, d.fsi_res, d.fsi_state, d.Kc, d.Fc, d.MFc, d.ipc, d.limc, d.flex.pos, d.flex.vel, d.flex.vel_km1, d.flex.F, d.flex.eps,
                    d.flex.ds, d.flex.irho, d.flex.imom, d.flex.nsupp, d.flex.supp, d.flex.delta, d.flex.sx,
                    d.flex.sy, d.flex.sz, d.flex.cage, d.flex.cagei, g->ibm->u_n};
    for (void *p : ptrs) cudaFree(p);
    d = FemDevice();
    g->ibm->u_n = nullptr;
}

// A flexible filament as the reference's FILAMENT_ARRAY reader builds it
// (inc/Body.h:143-187 markers, src/FEMBody.cpp:48-130 beam,
// :378-424 IB <-> FEM mapping).  The beam is planar (x-y) as the
// reference's; on a 3D grid its load and marker update use the x and y
// components and markers keep their z.
extern "C" int luma_gpu_ibm_add_filament(luma_gpu_grid *g, const double start[3], double length, double height,
                                         double depth, double angle_v, int nel, int clamped, double density,
                                         double E, double dm, double fsi_vel_scale, int *body_index) {
    if (!g || !start || nel <= 0 || length <= 0) return luma_set_error(LUMA_E_INVALID, "bad filament arguments");
    if (g->d.dims == 3 && !(depth > 0))
        return luma_set_error(LUMA_E_INVALID, "a filament on a 3D grid needs a positive depth");
    const double dh = g->d.dh;
    const int nmk = (int)std::floor(length / dh) + 1;
    const double spacing = length / (nmk - 1);
    const double spacing_h = spacing * std::cos(angle_v * kPi / 180);
    std::vector<double> xyz(3 * (size_t)nmk);
    for (int i = 0; i < nmk; i++) {
        xyz[3 * i + 0] = start[0] + i * spacing_h * std::cos(0.0 * kPi / 180.0);
        xyz[3 * i + 1] = start[1] + i * spacing * std::sin(angle_v * kPi / 180.0);
        xyz[3 * i + 2] = start[2] + i * spacing_h * std::sin(0.0 * kPi / 180.0);
    }
    int ib = -1;
    int rc = luma_gpu_ibm_add_body(g, nmk, xyz.data(), nullptr, &ib);
    if (rc) return rc;
    FlexBody fb;
    fb.nel = nel;
    fb.nm = nmk;
    fb.bc = clamped ? 3 : 2;
    fb.dm = dm;
    fb.velscale = fsi_vel_scale;
    const double fs = length / nel, fs_h = fs * std::cos(angle_v * kPi / 180);
    for (int i = 0; i < nel + 1; i++) {
        fb.pos0.push_back(start[0] + i * fs_h * std::cos(0.0 * kPi / 180.0));
        fb.pos0.push_back(start[1] + i * fs * std::sin(angle_v * kPi / 180.0));
        fb.pos0.push_back(start[2] + i * fs_h * std::sin(0.0 * kPi / 180.0));
        fb.ang0.push_back(angle_v * kPi / 180.0);
    }
    if (g->d.dims == 2) depth = dh;  // 2D: unit lattice depth (src/FEMBody.cpp:103-105)
    for (int e = 0; e < nel; ++e) {
        fb.len0.push_back(fs);
        fb.area.push_back(height * depth);
        fb.I.push_back(depth * (height * height * height) / 12.0);
        fb.E.push_back(E);
        fb.rho.push_back(density);
    }
    const int nI = nmk, nF = nel + 1;
    fb.parent_el.assign(nI, 0);
    fb.parent_zeta.assign(nI, -1.0);
    for (int i = 1; i < nI; i++) {
        const double q = i * ((nF - 1.0) / (nI - 1.0));
        if (std::fmod(q, 1.0) == 0.0) {
            fb.parent_el[i] = (int)std::floor(q) - 1;
            fb.parent_zeta[i] = 1.0;
        } else {
            fb.parent_el[i] = (int)std::floor(q);
            fb.parent_zeta[i] = std::fmod(q, 1.0) * 2.0 - 1.0;
        }
    }
    fb.child_off.assign(1, 0);
    for (int e = 0; e < nel; ++e) {
        for (int node = 0; node < nI; ++node) {
            double n1 = -1 + 2.0 * ((node - 0.5) * ((nF - 1.0) / (nI - 1.0)) - e) / 1.0;
            double n2 = -1 + 2.0 * ((node + 0.5) * ((nF - 1.0) / (nI - 1.0)) - e) / 1.0;
            if ((n1 > -1.0 && n1 < 1.0) || (n2 > -1.0 && n2 < 1.0)) {
                if (n1 < -1.0) n1 = -1.0;
                if (n2 > 1.0) n2 = 1.0;
                fb.child_node.push_back(node);
                fb.child_z1.push_back(n1);
                fb.child_z2.push_back(n2);
            }
        }
        fb.child_off.push_back((int)fb.child_node.size());
    }
    fb.mpos0 = xyz;
    g->ibm->flex.push_back(fb);
    g->ibm->flex_body.push_back(ib);
    g->ibm->has_flexible = true;
    if (body_index) *body_index = ib;
    return LUMA_OK;
}
