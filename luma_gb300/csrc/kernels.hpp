// Launch entry points of the device kernels (host-callable, stream-ordered).
#pragma once

#include <cuda_runtime.h>

#include "device.cuh"

namespace luma {

// k_general.cu
// Phase A of a split grid launches the interior kernel and the list kernel
// of the other streamed sites; `part` selects both or one of them.
// kPhaseALate: a list of transition sites to finer grids (coalesce), run
// one thread per (site, direction)
enum { kPhaseAAll = 0, kPhaseAInterior = 1, kPhaseAList = 2, kPhaseALate = 3 };
template <int Q, class P>
cudaError_t launch_general_phaseA(const StepArgs &a, const int8_t *wall, const uint8_t *fast, const int *gen_ids,
                                  int ngen, cudaStream_t s, int part = kPhaseAAll);
template <int Q, class P>
cudaError_t launch_general_phaseB(const StepArgs &a, const int8_t *wall, const RegSite *sites, int nsites,
                                  cudaStream_t s);
template <class P>
cudaError_t launch_velocity_u(const StepArgs &a, int dims, const int2 *sites, int nsites, cudaStream_t s);
template <int Q, class P>
cudaError_t launch_general_phaseC(const StepArgs &a, const int *ids, int nids, cudaStream_t s);
struct IbmArgs;
struct FlexArgs;
template <int Q, class P>
cudaError_t launch_ibm_pass(const StepArgs &a, const IbmArgs &b, const FlexArgs &f, cudaStream_t s);
template <class P>
cudaError_t launch_reset_forces(const StepArgs &a, int dims, double gravity, int gdir, double rr, cudaStream_t s);


// k_bulk.cu
template <int Q, class P>
cudaError_t launch_aa(void *A, void *u, void *rho, int N, int M, int K, double omega, double rho0, bool from_e,
                      bool write_macro, cudaStream_t s);

// k_transfer.cu
enum PopLayout { kPopPlain = 0, kPopAAE = 1, kPopAAO = 2 };
template <int Q, class P>
cudaError_t launch_pop_in(const double *aos, void *soa, int N, int M, int K, int layout, double rho0,
                          cudaStream_t s);
template <int Q, class P>
cudaError_t launch_pop_out(const void *soa, double *aos, int N, int M, int K, int layout, double rho0,
                           cudaStream_t s);
template <class P>
cudaError_t launch_vec_in(const double *aos, void *soa, size_t n, int dims, cudaStream_t s);
template <class P>
cudaError_t launch_vec_out(const void *soa, double *aos, size_t n, int dims, cudaStream_t s);
// Blocks of the FP64 field reduction; its device buffer holds
// (kReduceBlocks + 1) * 8 doubles: the result (mass, mx, my, mz, ke, max|u|,
// nonfinite, spare) followed by one slot of partials per block.
constexpr int kSMs = 152;  // streaming multiprocessors of a GB300
constexpr int kReduceBlocks = kSMs * 4;
template <class P>
cudaError_t launch_reduce(const uint8_t *typ, const void *rho, const void *u, size_t n, int dims, double *acc,
                          cudaStream_t s);

}  // namespace luma
