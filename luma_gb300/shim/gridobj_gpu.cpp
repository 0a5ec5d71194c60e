// LUMA-side binding of the GB300 time step (see gridobj_gpu.h).  Built
// inside LUMA: GridObj, GridManager, ObjectManager and the definitions.h
// switches are LUMA's own.  Every GridObj member read or written here is
// named as LUMA declares it (inc/GridObj.h:54-127); the descriptor fields
// are documented in include/luma_gpu.h.
#include <iterator>
#include <map>
#include <string>
#include <vector>

// LUMA's headers in LUMA's own order (stdafx.h first, as its sources do)
#include "stdafx.h"
#include "GridObj.h"
#include "GridManager.h"
#include "GridUnits.h"
#include "ObjectManager.h"
#include "IBBody.h"

#include "../../include/luma_gpu.h"
#include "gridobj_gpu.h"

namespace {

std::map<const GridObj *, luma_gpu_grid *> g_twins;
struct BodyTwin {
    size_t body;         // index in ObjectManager::iBody
    luma_gpu_grid *grid; // twin of the owning grid
    int index;           // the body's index on that twin
};
std::vector<BodyTwin> g_bodies;
std::string g_err;   // the shim's own refusals (the library's are in luma_gpu_last_error_string)

int refuse(const char *msg) {
    g_err = msg;
    return LUMA_E_INVALID;
}

// GridObj -> luma_grid_desc (the fields GridObj::LBM_multi_opt reads).
void describe(const GridObj *g, int precision, luma_grid_desc &d, std::vector<int32_t> &typ) {
    GridManager *gm = GridManager::getInstance();
    d = luma_grid_desc();
    d.abi_version = LUMA_GPU_ABI_VERSION;
    d.level = g->level;
    d.region = g->region_number;
    d.dims = L_DIMS;
    d.Q = L_NUM_VELS;
    d.N = g->N_lim;
    d.M = g->M_lim;
    d.K = g->K_lim;
    d.precision = precision;
#if defined L_USE_KBC_COLLISION
    d.collision = LUMA_COLL_KBC;
#elif defined L_USE_BGKSMAG
    d.collision = LUMA_COLL_BGK_SMAG;
#else
    d.collision = LUMA_COLL_BGK;
#endif
    d.flags = 0;
#ifdef L_REGULARISED_BOUNDARIES
    d.flags |= LUMA_FLAG_REGULARISED;
#endif
#ifdef L_IBM_ON
    d.flags |= LUMA_FLAG_IBM;
#endif
#ifdef L_GRAVITY_ON
    d.flags |= LUMA_FLAG_GRAVITY;
#endif
#ifdef L_COMPUTE_TIME_AVERAGED_QUANTITIES
    d.flags |= LUMA_FLAG_TIME_AVERAGES;
#endif
#ifdef L_UNIVERSAL_EPSILON_CALC
    d.flags |= LUMA_FLAG_UNIVERSAL_EPSILON;
#endif
    d.omega = g->omega;
    d.dt = g->dt;
    d.dh = g->dh;
    d.refinement_ratio = g->refinement_ratio;
    d.rho_in = L_RHOIN;
#ifdef L_VELOCITY_RAMP
    d.velocity_ramp = L_VELOCITY_RAMP;
#endif
#ifdef L_REYNOLDS_RAMP
    d.reynolds_ramp = L_REYNOLDS_RAMP;
#endif
#ifdef L_RE
    d.re = L_RE;
#endif
    d.pressure_delta = GridUnits::pd2dlbm(L_PRESSURE_DELTA, const_cast<GridObj *>(g));
    d.gravity = g->gravity;
    d.gravity_dir = L_GRAVITY_DIRECTION;
    d.csmag = L_CSMAG;
    for (int e = 0; e < 6; ++e) d.global_edges[e] = gm->global_edges[e][0];
    const double wt[6] = {L_WALL_THICKNESS_LEFT, L_WALL_THICKNESS_RIGHT, L_WALL_THICKNESS_BOTTOM,
                          L_WALL_THICKNESS_TOP, L_WALL_THICKNESS_FRONT, L_WALL_THICKNESS_BACK};
    for (int e = 0; e < 6; ++e) d.wall_thickness[e] = wt[e];
    if (g->level > 0) {
        d.coarse_lims[0] = g->CoarseLimsX[eMinimum];
        d.coarse_lims[1] = g->CoarseLimsX[eMaximum];
        d.coarse_lims[2] = g->CoarseLimsY[eMinimum];
        d.coarse_lims[3] = g->CoarseLimsY[eMaximum];
        d.coarse_lims[4] = g->CoarseLimsZ[eMinimum];
        d.coarse_lims[5] = g->CoarseLimsZ[eMaximum];
    }
    typ.assign(g->LatTyp.begin(), g->LatTyp.end());
    d.lattyp = typ.data();
    d.xpos = g->XPos.data();
    d.ypos = g->YPos.data();
    d.zpos = g->ZPos.data();
    d.ux_in = g->ux_in.data();
    d.uy_in = g->uy_in.data();
    d.uz_in = g->uz_in.data();
}

int create_tree(GridObj *g, luma_gpu_grid *parent, int precision) {
    luma_grid_desc d;
    std::vector<int32_t> typ;
    describe(g, precision, d, typ);
    luma_gpu_grid *h = nullptr;
    if (int rc = luma_gpu_grid_create(&d, parent, &h)) return rc;
    g_twins[g] = h;
    for (GridObj *sg : g->subGrid)
        if (int rc = create_tree(sg, h, precision)) return rc;
    return LUMA_OK;
}

int upload_tree(GridObj *g) {
    luma_gpu_grid *h = g_twins.at(g);
    if (int rc = luma_gpu_upload_state(h, g->f.data(), g->u.data(), g->rho.data(),
                                       g->force_xyz.empty() ? nullptr : g->force_xyz.data(), g->t))
        return rc;
    for (GridObj *sg : g->subGrid)
        if (int rc = upload_tree(sg)) return rc;
    return LUMA_OK;
}

int download_tree(GridObj *g) {
    luma_gpu_grid *h = g_twins.at(g);
    if (int rc = luma_gpu_download_state(h, g->f.data(), g->u.data(), g->rho.data(),
                                         g->force_xyz.empty() ? nullptr : g->force_xyz.data()))
        return rc;
    if (int rc = luma_gpu_get_time(h, &g->t)) return rc;
#ifdef L_COMPUTE_TIME_AVERAGED_QUANTITIES
    if (int rc = luma_gpu_download_time_averages(h, g->rho_timeav.data(), g->ui_timeav.data(),
                                                 g->uiuj_timeav.data()))
        return rc;
#endif
    for (GridObj *sg : g->subGrid)
        if (int rc = download_tree(sg)) return rc;
    return LUMA_OK;
}

void advance_t(GridObj *g, int steps) {
    g->t += steps;
    for (GridObj *sg : g->subGrid) advance_t(sg, 2 * steps);
}

#ifdef L_IBM_ON
// The ObjectManager's rigid bodies (ObjectManager::iBody, inc/ObjectManager.h:
// 104) as LUMA's geometry reader built them, on the grid that owns each
// (Body::_Owner, inc/Body.h:66), then the device set-up.
int hand_over_bodies(GridObj *root) {
    ObjectManager *om = ObjectManager::getInstance();
    bool any = false;
    for (IBBody &b : om->iBody) {
        if (b.isFlexible)   // FEM filaments enter through luma_gpu_ibm_add_filament with the
                            // FILAMENT_ARRAY reader's parameters, which the built body no longer holds
            return refuse("a flexible IB body is not handed over by this shim");
        auto it = g_twins.find(b._Owner);
        if (it == g_twins.end()) return refuse("an IB body's owning grid has no device twin");
        std::vector<double> pos, vel;
        for (IBMarker &m : b.markers) {
            pos.insert(pos.end(), {m.position[0], m.position[1], m.position[2]});
            vel.insert(vel.end(), {m.markerVel[0], m.markerVel[1], L_DIMS == 3 ? m.markerVel[2] : 0.0});
        }
        int idx = -1;
        if (int rc = luma_gpu_ibm_add_body(it->second, (int)b.markers.size(), pos.data(), vel.data(), &idx))
            return rc;
        g_bodies.push_back({(size_t)(&b - om->iBody.data()), it->second, idx});
        any = true;
    }
    return any ? luma_gpu_ibm_initialise(g_twins.at(root)) : LUMA_OK;
}

// The markers' IBM force, epsilon and ds back into ObjectManager::iBody
// (IBMarker::force_xyz, epsilon, ds, inc/IBMarker.h:56-70): what LUMA's
// lift/drag writer reads (src/ObjectManager_ops_io.cpp:65-128).
int sync_bodies() {
    ObjectManager *om = ObjectManager::getInstance();
    std::vector<double> mk;
    for (const BodyTwin &t : g_bodies) {
        IBBody &b = om->iBody[t.body];
        mk.resize(9 * b.markers.size());
        if (int rc = luma_gpu_ibm_get_markers(t.grid, t.index, mk.data())) return rc;
        for (size_t m = 0; m < b.markers.size(); ++m) {
            IBMarker &x = b.markers[m];
            for (size_t d = 0; d < x.force_xyz.size() && d < 3; ++d) x.force_xyz[d] = mk[9 * m + 3 + d];
            x.epsilon = mk[9 * m + 6];
            x.ds = mk[9 * m + 7];
        }
    }
    return LUMA_OK;
}
#endif

void fail(int rc) {
    if (rc != LUMA_OK)
        L_ERROR(std::string("GB300 step: ") + (g_err.empty() ? luma_gpu_last_error_string() : g_err),
                GridUtils::logfile);
}

}  // namespace

int LumaGpuShim::create(GridObj *root, int precision) {
    g_err.clear();
    destroy(root);
    if (int rc = create_tree(root, nullptr, precision)) return rc;
    if (int rc = upload_tree(root)) return rc;
#ifdef L_IBM_ON
    if (int rc = hand_over_bodies(root)) return rc;
#endif
    return LUMA_OK;
}

int LumaGpuShim::step(GridObj *root, int nsteps) {
    g_err.clear();
    luma_gpu_grid *h = twin(root);
    if (!h) return refuse("LumaGpuShim::create was not called for this grid");
    if (int rc = luma_gpu_step(h, nsteps)) return rc;
    advance_t(root, nsteps);
    return LUMA_OK;
}

int LumaGpuShim::sync_to_host(GridObj *root) {
    g_err.clear();
    if (!twin(root)) return refuse("LumaGpuShim::create was not called for this grid");
    if (int rc = luma_gpu_synchronize(twin(root))) return rc;
    if (int rc = download_tree(root)) return rc;
#ifdef L_IBM_ON
    if (int rc = sync_bodies()) return rc;
#endif
    return LUMA_OK;
}

void LumaGpuShim::destroy(GridObj *root) {
    auto it = g_twins.find(root);
    if (it == g_twins.end()) return;
    g_bodies.clear();
    luma_gpu_grid_destroy(it->second);   // the sub-grids' twins with it
    for (auto i = g_twins.begin(); i != g_twins.end();) {
        bool under = false;
        for (const GridObj *p = i->first; p; p = p->parentGrid) under = under || p == root;
        i = under ? g_twins.erase(i) : std::next(i);
    }
}

luma_gpu_grid *LumaGpuShim::twin(const GridObj *g) {
    auto it = g_twins.find(g);
    return it == g_twins.end() ? nullptr : it->second;
}

void LumaGpuShim::create_or_exit(GridObj *root, int precision) { fail(create(root, precision)); }
void LumaGpuShim::step_or_exit(GridObj *root, int nsteps) { fail(step(root, nsteps)); }
void LumaGpuShim::sync_or_exit(GridObj *root) { fail(sync_to_host(root)); }
