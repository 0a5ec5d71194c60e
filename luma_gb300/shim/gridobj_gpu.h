/*
 * gridobj_gpu.h — LUMA-side binding of the GB300 time step.
 *
 * Compiled into LUMA itself (LUMA's inc/ on the include path, its
 * definitions.h in force) together with gridobj_gpu.cpp, and linked with
 * libluma_gpu.so.  It builds a device twin of LUMA's GridObj tree through
 * the C ABI (include/luma_gpu.h), hands over the ObjectManager's rigid IB
 * bodies, runs GridObj::LBM_multi_opt on the device and brings the state
 * back into the GridObj members for LUMA's writers.
 *
 * LUMA's side of the integration is three edits:
 *   inc/GridObj.h, inside class GridObj:   friend class LumaGpuShim;
 *   src/GridObj_ops_lbm_optimised.cpp, first lines of LBM_multi_opt
 *     (src/GridObj_ops_lbm_optimised.cpp:36):
 *       #ifdef L_GPU_PATH
 *       if (level == 0) { LumaGpuShim::step_or_exit(this, 1); return; }
 *       #endif
 *   src/main_lbm.cpp: LumaGpuShim::create_or_exit(Grids, L_GPU_PRECISION)
 *     after ibm_initialise (:291) and LumaGpuShim::sync_or_exit(Grids)
 *     before each output writer.
 */
#ifndef LUMA_GRIDOBJ_GPU_H
#define LUMA_GRIDOBJ_GPU_H

class GridObj;
struct luma_gpu_grid;

class LumaGpuShim {
public:
    /* Device twins of the tree under `root` (level 0; each sub-grid after
     * its parent, in region order), its state uploaded (f, u, rho,
     * force_xyz, t), the rigid IB bodies of the ObjectManager handed over
     * and initialised on the device (ObjectManager::ibm_initialise,
     * src/ObjectManager_ops_ibm.cpp:190-246).  `precision` is a
     * LUMA_PREC_* value.  Returns a LUMA_OK / LUMA_E_* status. */
    static int create(GridObj *root, int precision);
    /* `nsteps` calls of GridObj::LBM_multi_opt on the device; the host
     * counters t of the tree advance with them. */
    static int step(GridObj *root, int nsteps);
    /* f, u, rho, force_xyz (and the time averages when LUMA keeps them)
     * of every grid back into the GridObj members, with t, and the rigid
     * IB markers' force, epsilon and ds into the ObjectManager's bodies. */
    static int sync_to_host(GridObj *root);
    /* Releases the device twins of the tree. */
    static void destroy(GridObj *root);
    /* The twin of a grid, or null. */
    static luma_gpu_grid *twin(const GridObj *g);

    /* The same three calls for LUMA's code paths, which have no status to
     * return: a failure goes to L_ERROR (log and exit, inc/stdafx.h:127-149)
     * with luma_gpu_last_error_string(). */
    static void create_or_exit(GridObj *root, int precision);
    static void step_or_exit(GridObj *root, int nsteps);
    static void sync_or_exit(GridObj *root);
};

#endif
