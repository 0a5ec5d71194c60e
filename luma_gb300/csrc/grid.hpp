// Host-side state of one grid of the hierarchy behind a luma_gpu_grid handle.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <vector>

#include "device.cuh"
#include "../../include/luma_gpu.h"

namespace luma {
struct IbmState;
struct AdjState;
struct StepGraph;
struct BflState;
struct IoJobs;
}

struct luma_gpu_grid;

struct luma_gpu_grid {
    luma_grid_desc d{};         // copy of the descriptor (array pointers cleared)
    size_t n = 0;               // sites
    double cs2 = 0;             // (1/sqrt(3))^2 as the reference computes it
    uint8_t *typ = nullptr;     // site labels
    void *f[2] = {nullptr, nullptr};  // population buffers (S*, SoA)
    int cur = 0;                // index of the buffer holding f
    void *u = nullptr, *rho = nullptr, *force = nullptr;  // R*, SoA
    double *uxin = nullptr, *uyin = nullptr, *uzin = nullptr;
    int8_t *wall = nullptr;     // slip-site wall normals (4 bytes per site) or null
    luma::RegSite *reg = nullptr;
    int nreg = 0;
    int2 *velu = nullptr;       // (velocity site, row of last writer) under a ramp
    int nvelu = 0;
    double *acc = nullptr;      // reduction accumulators
    int *unsup = nullptr;       // device flag: non-zero when a site needed an operation outside the GPU path
    double *tav = nullptr;      // running means (rho, u_p, u_p u_q; SoA, FP64) or null
    int t = 0;
    bool bulk = false;          // in-place AA path
    bool bulk_fixed = false;    // state uploaded: path can no longer change
    int aa_odd = 0;             // AA storage state: 0 = E, 1 = O
    // IBM grids: sites whose collision waits for the IBM pass (phase C);
    // every other site is collided in phase A (fuse = true)
    bool fuse = false;
    uint8_t *defer = nullptr;   // per-site flag
    int *defer_ids = nullptr;   // the flagged sites
    int ndefer = 0;
    std::vector<uint8_t> htyp;  // site labels (host copy)
    // general path: interior fluid sites (plain pulls only) run a lean
    // kernel; the listed others run the full site logic
    uint8_t *fast = nullptr;
    int *gen_ids = nullptr;
    int ngen = 0;
    int ngen_early = 0;         // gen_ids[0, ngen_early): sites other than transition sites to finer grids
    luma_gpu_grid *parent = nullptr;
    std::vector<luma_gpu_grid *> kids;
    cudaStream_t stream = nullptr;
    // grids with sub-grids: the sub-grids' steps run on kid_stream (high
    // priority) beside this grid's interior kernel; fork/join events
    cudaStream_t kid_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the listed sites' kernel runs on list_stream (high priority) beside
    // the interior kernel: both pull from the same populations and write
    // only their own sites; fork/join events
    cudaStream_t list_stream = nullptr;
    cudaEvent_t ev_lfork = nullptr, ev_ljoin = nullptr;
    luma::IbmState *ibm = nullptr;
    luma::AdjState *adj = nullptr;   // discrete-adjoint tape (adjoint.cu)
    luma::StepGraph *graph = nullptr;  // level 0: two steps of the tree as a CUDA graph (capi.cu)
    luma::BflState *bfl = nullptr;     // BFL link tables (bfl.cu)
    luma::IoJobs *io = nullptr;        // level 0: pending file writers (io.cu)
    size_t nbfl_sites = 0;             // eBFL-labelled sites
    std::vector<double> hx, hy, hz;  // site positions (host copy, for IB support search)
};

int luma_set_error(int code, const char *fmt, ...);

// capi.cu
int luma_update_defer(luma_gpu_grid *g);
int luma_build_interior(luma_gpu_grid *g);
void luma_tree_signature(const luma_gpu_grid *g, std::vector<uintptr_t> &sig);
// ibm.cu
int luma_ibm_reset_forces(luma_gpu_grid *g, const luma::StepArgs &a);
int luma_ibm_apply(luma_gpu_grid *g, const luma::StepArgs &a);
void luma_ibm_free(luma_gpu_grid *g);
// adjoint.cu
int luma_adj_step_hook(luma_gpu_grid *g, const luma::StepArgs &a);
void luma_adj_redirect(luma_gpu_grid *g, luma::StepArgs &a);
void luma_adj_free(luma_gpu_grid *g);
// bfl.cu
void luma_bfl_free(luma_gpu_grid *g);
void luma_bfl_args(const luma_gpu_grid *g, luma::StepArgs &a);
void luma_bfl_signature(const luma_gpu_grid *g, std::vector<uintptr_t> &sig);
// io.cu
void luma_io_free(luma_gpu_grid *g);
// epsilon.cu
int luma_eps_solve_device(int n, int band, const std::vector<double> &a, std::vector<double> &x, cudaStream_t s);
// fem.cu
int luma_fem_upload(luma_gpu_grid *g);
int luma_fem_supports(luma_gpu_grid *g, const int *skip);
int luma_fem_move_bodies(luma_gpu_grid *g, const int *skip, bool first);
const int *luma_fem_fsi_flag(luma_gpu_grid *g);
int luma_fem_fsi_begin(luma_gpu_grid *g);
int luma_fem_restore_u(luma_gpu_grid *g);
int luma_fem_fsi_check(luma_gpu_grid *g);
int luma_fem_take_error(luma_gpu_grid *g);
int luma_fem_commit(luma_gpu_grid *g);
void luma_fem_free(luma_gpu_grid *g);

namespace luma {

// One rigid immersed-boundary body on the host: marker state and the
// support lists built by ibm_findSupport (FP64, reference order).
struct IbmBody {
    int nm = 0;
    long long seq = 0;          // creation order over the process (the restart file lists bodies in it)
    std::vector<double> pos, vel, eps, ds, dil, area;  // per marker (pos/vel: 3 per marker)
    std::vector<int> off;                               // CSR offsets, nm + 1
    std::vector<int> si, sj, sk;                        // support site indices
    std::vector<double> sx, sy, sz, delta;              // support positions and delta values
};

// Device arrays of all bodies owned by one grid, concatenated in body order.
struct IbmDevice {
    int nm = 0, nsup = 0, nu = 0;
    double *vel = nullptr, *eps = nullptr, *ds = nullptr, *area = nullptr;
    double *F = nullptr, *irho = nullptr, *imom = nullptr;   // per marker (F, imom: 3 per marker)
    int *moff = nullptr, *msite = nullptr, *smarker = nullptr;
    double *mdelta = nullptr;
    int *usite = nullptr, *uoff = nullptr, *uref = nullptr;  // unique support sites -> supports in order
};

// Flexible filaments: markers with fixed-capacity support slots (supports
// move every FSI iteration) and the FEM beam state, all device resident.
// The support cage |x - X|/dh < 1.5 holds 3 nodes per axis, but a marker
// within rounding of a half-node offset can pass the test on 4 (both ends
// at 1.5 minus an ulp): 4^3 slots cover every case in 3D.
constexpr int kFlexMaxSupp = 64;

struct FlexArgs {
    int nm;                     // flexible markers on this grid (all filaments)
    int dims;
    double *pos, *vel, *vel_km1, *F, *eps, *ds, *irho, *imom;  // per marker (3 for pos/vel/F/imom)
    int *nsupp, *supp;          // supp[m*kFlexMaxSupp + s] = site id
    double *delta, *sx, *sy, *sz;
    double *cage;               // per marker: 15 candidate coordinates, 15 kernel values (axis-major, offsets -2..2)
    int *cagei;                 // per marker: near node (3), cage-and-domain test bits (bit 5*axis + offset)
};

struct FemDevice {
    int nfil = 0, maxdof = 0, maxmk = 0;
    // per filament offsets
    int *node_off = nullptr, *el_off = nullptr, *dof_off = nullptr, *mk_off = nullptr, *bc = nullptr;
    double *dm = nullptr, *velscale = nullptr;
    // nodes
    double *pos0 = nullptr, *ang0 = nullptr;
    // elements
    double *len0 = nullptr, *area = nullptr, *I = nullptr, *E = nullptr, *rho = nullptr;
    int *child_off = nullptr, *child_node = nullptr;
    double *child_z1 = nullptr, *child_z2 = nullptr;
    // state per DOF
    double *U = nullptr, *U_n = nullptr, *Ud = nullptr, *Ud_n = nullptr, *Udd = nullptr, *Udd_n = nullptr;
    double *R = nullptr, *Fv = nullptr, *delU = nullptr;
    // scratch: dense M, K per filament (maxdof^2 each), element matrices
    double *M = nullptr, *K = nullptr, *epsA = nullptr;
    // the step's first Newton iteration: factors, pivots, L extents (per
    // filament maxdof^2 / maxdof), internal force and mass term (per DOF)
    double *Kc = nullptr, *Fc = nullptr, *MFc = nullptr;
    int *ipc = nullptr, *limc = nullptr;
    // markers
    int *parent_el = nullptr;
    double *parent_zeta = nullptr, *mpos0 = nullptr;
    // outputs
    int *it = nullptr;
    double *res = nullptr, *fsi_res = nullptr;  // FSI residual: [0] running max, [1] last
    int *fsi_state = nullptr;                   // FSI loop of the step: [0] converged, [1] iterations
    int k_in_smem = 0, eps_in_smem = 0;         // the filament matrices fit in shared memory
    int lu32 = 0;                               // Newton steps with FP32 factors (shifted-FP32 grids)
    // flexible IB marker arrays
    FlexArgs flex{};
};

struct FlexBody {                // host description of one filament
    int nel = 0, nm = 0, bc = 3;
    double dm = 0, velscale = 1;
    std::vector<double> pos0, ang0;          // nodes
    std::vector<double> len0, area, I, E, rho;  // elements
    std::vector<int> child_off, child_node;
    std::vector<double> child_z1, child_z2;
    std::vector<int> parent_el;
    std::vector<double> parent_zeta, mpos0;  // markers
};

struct IbmState {
    bool has_bodies = false;
    bool has_flexible = false;
    bool ready = false;
    std::vector<IbmBody> bodies;
    IbmDevice dev;
    std::vector<FlexBody> flex;      // filaments (their markers are bodies too, in order)
    std::vector<int> flex_body;      // IB body index of each filament
    FemDevice fem;
    double *u_n = nullptr;           // start-of-step velocity (R*), for FSI resets
};

// Marker-side arguments of the IBM kernels.
struct IbmArgs {
    int nm, nu, dims;
    const int *moff, *msite, *smarker, *usite, *uoff, *uref;
    const double *mdelta, *vel, *eps, *ds, *area;
    double *F, *irho, *imom;
};

}
