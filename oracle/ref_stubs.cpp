/* Oracle test infrastructure: the symbols a serial build of the reference
 * needs but does not define once main_lbm.cpp, the MPI manager sources and
 * the HDF5 writer are left out of the oracle build.
 *
 *  - GridUtils::path_str (defined by the reference in src/main_lbm.cpp:55).
 *  - MpiManager singleton and neighbour table: unreachable in a serial build
 *    (every use sits under L_BUILD_FOR_MPI or behind a rank count of 1); the
 *    methods abort if ever reached.
 *  - LAPACK dgetrf_/dgetrs_ (declared in inc/GridUtils.h:30-31, called from
 *    GridUtils::solveLinearSystem, src/GridUtils.cpp:356-395).  LAPACK is
 *    linked unpinned by the reference (makefile:26) and is not installed
 *    here, so this file restates the published algorithm: unblocked
 *    right-looking LU with partial (row) pivoting on a column-major matrix,
 *    1-based pivot indices, and the transposed solve A^T x = b for
 *    TRANS='T'.  Results agree with a blocked LAPACK LU to rounding only.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "../inc/stdafx.h"
#include "../inc/GridUtils.h"
#include "../inc/MpiManager.h"

std::string GridUtils::path_str;
MpiManager *MpiManager::me = nullptr;
const int MpiManager::neighbour_vectors[3][26] = {{0}};

static void oracle_unreachable(const char *what) {
    std::fprintf(stderr, "oracle: serial build reached MPI routine %s\n", what);
    std::abort();
}

MpiManager *MpiManager::getInstance() { oracle_unreachable("getInstance"); return nullptr; }
void MpiManager::destroyInstance() { oracle_unreachable("destroyInstance"); }

extern "C" void dgetrf_(int *m_, int *n_, double *a, int *lda_, int *ipiv, int *info) {
    const int m = *m_, n = *n_, lda = *lda_;
    const int kmax = m < n ? m : n;
    *info = 0;
#define A_(r, c) a[(size_t)(c) * lda + (r)]
    for (int k = 0; k < kmax; ++k) {
        int p = k;
        double best = std::fabs(A_(k, k));
        for (int r = k + 1; r < m; ++r) {
            double v = std::fabs(A_(r, k));
            if (v > best) { best = v; p = r; }
        }
        ipiv[k] = p + 1;
        if (A_(p, k) == 0.0) { if (*info == 0) *info = k + 1; continue; }
        if (p != k)
            for (int c = 0; c < n; ++c) { double t = A_(k, c); A_(k, c) = A_(p, c); A_(p, c) = t; }
        const double inv = 1.0 / A_(k, k);
        for (int r = k + 1; r < m; ++r) A_(r, k) *= inv;
        for (int c = k + 1; c < n; ++c) {
            const double akc = A_(k, c);
            if (akc == 0.0) continue;
            for (int r = k + 1; r < m; ++r) A_(r, c) -= A_(r, k) * akc;
        }
    }
#undef A_
}

extern "C" void dgetrs_(char *trans, int *n_, int *nrhs_, double *a, int *lda_, int *ipiv,
                        double *b, int *ldb_, int *info) {
    const int n = *n_, nrhs = *nrhs_, lda = *lda_, ldb = *ldb_;
    *info = 0;
#define A_(r, c) a[(size_t)(c) * lda + (r)]
    for (int j = 0; j < nrhs; ++j) {
        double *x = b + (size_t)j * ldb;
        if (*trans == 'N' || *trans == 'n') {
            for (int k = 0; k < n; ++k) { int p = ipiv[k] - 1; if (p != k) { double t = x[k]; x[k] = x[p]; x[p] = t; } }
            for (int r = 0; r < n; ++r) { double s = x[r]; for (int c = 0; c < r; ++c) s -= A_(r, c) * x[c]; x[r] = s; }
            for (int r = n - 1; r >= 0; --r) { double s = x[r]; for (int c = r + 1; c < n; ++c) s -= A_(r, c) * x[c]; x[r] = s / A_(r, r); }
        } else {
            /* A = P L U  =>  A^T = U^T L^T P^T */
            for (int r = 0; r < n; ++r) { double s = x[r]; for (int c = 0; c < r; ++c) s -= A_(c, r) * x[c]; x[r] = s / A_(r, r); }
            for (int r = n - 1; r >= 0; --r) { double s = x[r]; for (int c = r + 1; c < n; ++c) s -= A_(c, r) * x[c]; x[r] = s; }
            for (int k = n - 1; k >= 0; --k) { int p = ipiv[k] - 1; if (p != k) { double t = x[k]; x[k] = x[p]; x[p] = t; } }
        }
    }
#undef A_
}

void MpiManager::mpi_buildMarkerComms(int) { oracle_unreachable("mpi_buildMarkerComms"); }
void MpiManager::mpi_buildSupportComms(int) { oracle_unreachable("mpi_buildSupportComms"); }
void MpiManager::mpi_interpolateComm(int, std::vector<std::vector<double>> &) { oracle_unreachable("mpi_interpolateComm"); }
void MpiManager::mpi_spreadComm(int, std::vector<std::vector<double>> &) { oracle_unreachable("mpi_spreadComm"); }
void MpiManager::mpi_spreadNewMarkers(int, std::vector<std::vector<int>> &,
                                      std::vector<std::vector<std::vector<double>>> &,
                                      std::vector<std::vector<std::vector<double>>> &) {
    oracle_unreachable("mpi_spreadNewMarkers");
}
