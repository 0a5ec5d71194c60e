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
    int t = 0;
    bool bulk = false;          // in-place AA path
    bool bulk_fixed = false;    // state uploaded: path can no longer change
    int aa_odd = 0;             // AA storage state: 0 = E, 1 = O
    luma_gpu_grid *parent = nullptr;
    std::vector<luma_gpu_grid *> kids;
    cudaStream_t stream = nullptr;
    luma::IbmState *ibm = nullptr;
    std::vector<double> hx, hy, hz;  // site positions (host copy, for IB support search)
};

int luma_set_error(int code, const char *fmt, ...);

// ibm.cu
int luma_ibm_reset_forces(luma_gpu_grid *g, const luma::StepArgs &a);
int luma_ibm_apply(luma_gpu_grid *g, const luma::StepArgs &a);
void luma_ibm_free(luma_gpu_grid *g);

namespace luma {

// One rigid immersed-boundary body on the host: marker state and the
// support lists built by ibm_findSupport (FP64, reference order).
struct IbmBody {
    int nm = 0;
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

struct IbmState {
    bool has_bodies = false;
    bool has_flexible = false;
    bool ready = false;
    std::vector<IbmBody> bodies;
    IbmDevice dev;
};

// Marker-side arguments of the IBM kernels.
struct IbmArgs {
    int nm, nu, dims;
    const int *moff, *msite, *smarker, *usite, *uoff, *uref;
    const double *mdelta, *vel, *eps, *ds, *area;
    double *F, *irho, *imom;
};

}
