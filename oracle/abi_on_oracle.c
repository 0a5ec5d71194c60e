/* ORACLE — test infrastructure only.  The entry points of include/luma_gpu.h
 * that the LUMA-side shim (luma_gb300/shim/gridobj_gpu.cpp) calls, carried
 * out by the oracle (lbm_oracle.c) on the host instead of the GPU library.
 * Linked in place of libluma_gpu.so into a build of the reference with the
 * shim, it lets a CPU test run the reference's own initialisation, hand its
 * GridObj tree and IB bodies through the shim and compare the state the
 * shim brings back with the reference's own LBM_multi_opt: a check of the
 * shim's mapping (descriptor fields, layouts, grid tree, bodies, counters),
 * the GPU library's side of each call being checked by the GPU tests. */
#include <stddef.h>
#include <string.h>

#include "../include/luma_gpu.h"

typedef struct oracle_grid oracle_grid;
oracle_grid *oracle_grid_create(const luma_grid_desc *d, oracle_grid *parent);
void oracle_grid_destroy(oracle_grid *g);
int oracle_upload_state(oracle_grid *g, const double *f, const double *u, const double *rho,
                        const double *force_xyz, int t);
int oracle_download_state(const oracle_grid *g, double *f, double *u, double *rho, double *force_xyz);
int oracle_download_time_averages(const oracle_grid *g, double *rho_ta, double *ui_ta, double *uiuj_ta);
int oracle_step(oracle_grid *root, int nsteps);
int oracle_get_time(const oracle_grid *g);
int oracle_ibm_add_body(oracle_grid *g, int nm, const double *xyz);
int oracle_ibm_initialise(void);
void oracle_ibm_set_universal(int on);
const char *oracle_last_error(void);

static oracle_grid *O(luma_gpu_grid *g) { return (oracle_grid *)g; }

int luma_gpu_abi_version(void) { return LUMA_GPU_ABI_VERSION; }
const char *luma_gpu_last_error_string(void) { return oracle_last_error(); }

int luma_gpu_grid_create(const luma_grid_desc *desc, luma_gpu_grid *parent, luma_gpu_grid **out) {
    if (!desc || !out) return LUMA_E_INVALID;
    if (desc->flags & LUMA_FLAG_UNIVERSAL_EPSILON) oracle_ibm_set_universal(1);
    *out = (luma_gpu_grid *)oracle_grid_create(desc, O(parent));
    return *out ? LUMA_OK : LUMA_E_INVALID;
}

int luma_gpu_grid_destroy(luma_gpu_grid *g) {
    oracle_grid_destroy(O(g));
    return LUMA_OK;
}

int luma_gpu_upload_state(luma_gpu_grid *g, const double *f, const double *u, const double *rho,
                          const double *force_xyz, int t) {
    return oracle_upload_state(O(g), f, u, rho, force_xyz, t) ? LUMA_E_INVALID : LUMA_OK;
}

int luma_gpu_download_state(luma_gpu_grid *g, double *f, double *u, double *rho, double *force_xyz) {
    return oracle_download_state(O(g), f, u, rho, force_xyz) ? LUMA_E_INVALID : LUMA_OK;
}

int luma_gpu_download_time_averages(luma_gpu_grid *g, double *rho_ta, double *ui_ta, double *uiuj_ta) {
    return oracle_download_time_averages(O(g), rho_ta, ui_ta, uiuj_ta) ? LUMA_E_STATE : LUMA_OK;
}

int luma_gpu_get_time(const luma_gpu_grid *g, int *t) {
    *t = oracle_get_time((const oracle_grid *)g);
    return LUMA_OK;
}

int luma_gpu_step(luma_gpu_grid *root, int nsteps) {
    return oracle_step(O(root), nsteps) ? LUMA_E_INVALID : LUMA_OK;
}

int luma_gpu_synchronize(luma_gpu_grid *root) {
    (void)root;
    return LUMA_OK;
}

int luma_gpu_ibm_add_body(luma_gpu_grid *g, int nmarkers, const double *positions, const double *velocities,
                          int *body_index) {
    (void)velocities;  /* the oracle's rigid bodies are at rest, as the test's are */
    const int b = oracle_ibm_add_body(O(g), nmarkers, positions);
    if (body_index) *body_index = b;
    return b < 0 ? LUMA_E_INVALID : LUMA_OK;
}

int oracle_ibm_markers(int ib, double *out);

int luma_gpu_ibm_get_markers(luma_gpu_grid *grid, int body, double *out) {
    (void)grid;  /* the oracle numbers bodies over all grids, as the shim kept them */
    return oracle_ibm_markers(body, out) ? LUMA_E_INVALID : LUMA_OK;
}

int luma_gpu_ibm_initialise(luma_gpu_grid *root) {
    (void)root;
    return oracle_ibm_initialise() ? LUMA_E_INVALID : LUMA_OK;
}
