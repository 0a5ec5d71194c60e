/* Oracle test infrastructure: a driver for the reference's own serial build.
 *
 * It performs the initialisation sequence of the reference's main()
 * (src/main_lbm.cpp:170-291: GridManager, GridObj(0), LBM_addSubGrid per
 * region, setGridHierarchy, ObjectManager, geometry read, ibm_initialise),
 * optionally replaces the L0 velocity/density field with a field read from a
 * raw binary file (and re-initialises f = feq(rho, u) exactly as
 * LBM_initGrid does, src/GridObj_init_grids.cpp:316-333), then calls
 * GridObj::LBM_multi_opt() the requested number of times
 * (src/main_lbm.cpp:441) and dumps every grid of the hierarchy as raw
 * little-endian arrays in the reference's AoS layout.
 *
 * Usage:
 *   luma_ref --out DIR --steps N [--dump-every K] [--init-u FILE] [--init-rho FILE]
 *            [--workdir DIR] [--markers FILE] [--drag-out FILE] [--momex-out FILE]
 *            [--bfl-out FILE] [--bfl-forces FILE] [--io-at S] [--restart-read]
 *
 * With --momex-out (cases compiled with L_LD_OUT) FILE gets, per step s, the
 * momentum-exchange force ObjectManager::computeLiftDrag accumulated over
 * the solid sites during step s (from the populations before it).
 *
 * With --bfl-out FILE gets BFL body 0 as the stream looks it up: its
 * marker count and Q values (L_NUM_VELS per marker, BFLBody::Q) and, per L0
 * site in id order, the marker Body::getMarkerData finds for the site's
 * position (-1 for none).  With --bfl-forces (cases compiled with L_LD_OUT)
 * FILE gets, per step s and marker m, the momentum-exchange force
 * ObjectManager::computeLiftDrag(v, id, g, markerID) accumulated on the
 * marker during step s.
 *
 * With --io-at S the reference's own ASCII writers run after step S:
 * GridObj::io_lite(S, "") (files io_lite.Lev<l>.Reg<r>.Rnk0.<S>.dat) and
 * GridObj::io_restart(eWrite) (restart_LBM_Rnk0.out), into DIR.
 *
 * With --restart-read the grids are read back from
 * <workdir>/input/restart_LBM_Rnk0.out by GridObj::io_restart(eRead) before
 * the first dump.
 *
 * With --drag-out nothing is dumped; FILE gets the time average over the N
 * steps of body 0's lattice-unit drag and N.
 *
 * Builds with the LUMA-side shim (LUMA_HARNESS_SHIM, luma_gb300/shim/)
 * take --gpu-shim PREC: after the initialisation the shim builds the
 * device twin of the grid tree (LUMA_PREC_* PREC) and hands over the IB
 * bodies, each step is the shim's LBM_multi_opt, and every dump first
 * brings the state back into the GridObj tree through the shim.
 *
 * Output, per dump step s and grid (level l, region r):
 *   DIR/s<s>/L<l>R<r>_meta.txt   key value lines (sizes, omega, dt, dh, t, limits)
 *   DIR/s<s>/L<l>R<r>_<name>.bin f, u, rho, typ (int32), force (if allocated),
 *                                rho_ta, ui_ta, uiuj_ta (time-averaging builds)
 * and, if IBM bodies exist, DIR/s<s>/markers.txt.
 */
#include <sys/stat.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../inc/stdafx.h"
#include "../inc/GridObj.h"
#include "../inc/GridManager.h"
#include "../inc/ObjectManager.h"
#include "../inc/IBBody.h"
#ifdef LUMA_HARNESS_SHIM
#include "../include/luma_gpu.h"
#include "gridobj_gpu.h"
#endif

static void write_raw(const std::string &path, const void *data, size_t bytes) {
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp) { std::perror(path.c_str()); std::exit(2); }
    if (bytes && std::fwrite(data, 1, bytes, fp) != bytes) { std::perror(path.c_str()); std::exit(2); }
    std::fclose(fp);
}

static std::vector<double> read_raw(const std::string &path, size_t count) {
    std::vector<double> v(count);
    FILE *fp = std::fopen(path.c_str(), "rb");
    if (!fp) { std::perror(path.c_str()); std::exit(2); }
    if (std::fread(v.data(), sizeof(double), count, fp) != count) {
        std::fprintf(stderr, "short read %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(fp);
    return v;
}

static void dump_grid(GridObj *g, const std::string &dir) {
    char pre[64];
    std::snprintf(pre, sizeof pre, "/L%dR%d_", g->level, g->region_number);
    std::string p = dir + pre;
    FILE *m = std::fopen((p + "meta.txt").c_str(), "w");
    std::fprintf(m, "level %d\nregion %d\nN %d\nM %d\nK %d\nQ %d\ndims %d\nt %d\n", g->level,
                 g->region_number, g->N_lim, g->M_lim, g->K_lim, L_NUM_VELS, L_DIMS, g->t);
    std::fprintf(m, "omega %.17g\ndt %.17g\ndh %.17g\nnu %.17g\n", g->omega, g->dt, g->dh, g->nu);
    if (g->level > 0)
        std::fprintf(m, "coarse_lims %d %d %d %d %d %d\n", g->CoarseLimsX[0], g->CoarseLimsX[1],
                     g->CoarseLimsY[0], g->CoarseLimsY[1], g->CoarseLimsZ[0], g->CoarseLimsZ[1]);
    std::fclose(m);
    write_raw(p + "f.bin", g->f.data(), g->f.size() * sizeof(double));
    write_raw(p + "u.bin", g->u.data(), g->u.size() * sizeof(double));
    write_raw(p + "rho.bin", g->rho.data(), g->rho.size() * sizeof(double));
    std::vector<int> typ(g->LatTyp.size());
    for (size_t i = 0; i < typ.size(); ++i) typ[i] = static_cast<int>(g->LatTyp[i]);
    write_raw(p + "typ.bin", typ.data(), typ.size() * sizeof(int));
    write_raw(p + "uxin.bin", g->ux_in.data(), g->ux_in.size() * sizeof(double));
    write_raw(p + "xpos.bin", g->XPos.data(), g->XPos.size() * sizeof(double));
    write_raw(p + "ypos.bin", g->YPos.data(), g->YPos.size() * sizeof(double));
    write_raw(p + "zpos.bin", g->ZPos.data(), g->ZPos.size() * sizeof(double));
    if (!g->force_xyz.empty())
        write_raw(p + "force.bin", g->force_xyz.data(), g->force_xyz.size() * sizeof(double));
#ifdef L_COMPUTE_TIME_AVERAGED_QUANTITIES
    write_raw(p + "rho_ta.bin", g->rho_timeav.data(), g->rho_timeav.size() * sizeof(double));
    write_raw(p + "ui_ta.bin", g->ui_timeav.data(), g->ui_timeav.size() * sizeof(double));
    write_raw(p + "uiuj_ta.bin", g->uiuj_timeav.data(), g->uiuj_timeav.size() * sizeof(double));
#endif
    for (GridObj *sg : g->subGrid) dump_grid(sg, dir);
}

static void dump_markers(const std::string &dir) {
#ifdef L_IBM_ON
    ObjectManager *om = ObjectManager::getInstance();
    FILE *fp = std::fopen((dir + "/markers.txt").c_str(), "w");
    for (size_t b = 0; b < om->iBody.size(); ++b) {
        IBBody &body = om->iBody[b];
        for (size_t m = 0; m < body.markers.size(); ++m) {
            IBMarker &mk = body.markers[m];
            const double fz = mk.force_xyz.size() > 2 ? mk.force_xyz[2] : 0.0;
            std::fprintf(fp, "%zu %zu %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %zu\n",
                         b, m, mk.position[0], mk.position[1], mk.position[2], mk.force_xyz[0],
                         mk.force_xyz[1], fz, mk.epsilon, mk.ds, mk.markerVel[0],
                         mk.markerVel[1], mk.markerVel[2], mk.dilation, mk.supp_i.size());
        }
    }
    std::fclose(fp);
    fp = std::fopen((dir + "/supports.txt").c_str(), "w");
    for (size_t b = 0; b < om->iBody.size(); ++b) {
        IBBody &body = om->iBody[b];
        for (size_t m = 0; m < body.markers.size(); ++m) {
            IBMarker &mk = body.markers[m];
            for (size_t q = 0; q < mk.supp_i.size(); ++q)
                std::fprintf(fp, "%zu %zu %zu %d %d %d %.17g\n", b, m, q, mk.supp_i[q], mk.supp_j[q], mk.supp_k[q],
                             mk.deltaval[q]);
        }
    }
    std::fclose(fp);
#else
    (void)dir;
#endif
}

/* Lattice-unit drag of body 0 as io_writeLiftDrag sums it per marker
 * (src/ObjectManager_ops_io.cpp:105-121, before its physical scaling). */
static double body_drag() {
#ifdef L_IBM_ON
    ObjectManager *om = ObjectManager::getInstance();
    if (om->iBody.empty()) return 0.0;
    IBBody &body = om->iBody[0];
    double s = 0.0;
    for (size_t m = 0; m < body.markers.size(); ++m) {
        IBMarker &mk = body.markers[m];
        const double volDepth = L_DIMS == 3 ? mk.ds : 1.0;
        s += mk.force_xyz[0] * mk.epsilon * volDepth * mk.ds;
    }
    return s;
#else
    return 0.0;
#endif
}

static void dump_all(GridObj *root, const std::string &out, int step) {
    std::string dir = out + "/s" + std::to_string(step);
    mkdir(dir.c_str(), 0755);
    dump_grid(root, dir);
    dump_markers(dir);
}

#ifdef L_IBM_ON
/* Rigid IB bodies with explicit marker positions (the case's marker layout
 * is not one of the reference's prefab formulas).  File format:
 *   nbodies
 *   level region nmarkers      (per body, followed by nmarkers lines "x y z")
 * Each body is built as the reference's constructors build one
 * (inc/Body.h:197-255 then IBBody::initialise, src/IBBody.cpp:58-91). */
static void inject_markers(ObjectManager *om, GridObj *root, const std::string &path) {
    std::ifstream in(path.c_str());
    int nb = 0;
    in >> nb;
    for (int b = 0; b < nb; ++b) {
        int lev, reg, nm;
        in >> lev >> reg >> nm;
        GridObj *g = nullptr;
        GridUtils::getGrid(root, lev, reg, g);
        if (!g) { std::fprintf(stderr, "no grid L%d R%d\n", lev, reg); std::exit(2); }
        IBBody body;
        body._Owner = g;
        body.id = b;
        body.closed_surface = true;
        body.level = lev;
        body.owningRank = 0;
        for (int m = 0; m < nm; ++m) {
            double x, y, z;
            in >> x >> y >> z;
            body.markers.emplace_back(x, y, z, m, g);
        }
        body.initialise(eRigid);
        om->iBody.push_back(body);
        om->hasIBMBodies[lev] = true;
    }
    om->ibm_finaliseReadIn(nb);
}
#endif

static void dump_bfl(GridObj *g, const std::string &path) {
    ObjectManager *om = ObjectManager::getInstance();
    FILE *fp = std::fopen(path.c_str(), "w");
    if (om->pBody.empty()) {
        std::fprintf(fp, "0 %d\n", L_NUM_VELS);
        std::fclose(fp);
        return;
    }
    BFLBody &b = om->pBody[0];
    std::fprintf(fp, "%zu %d\n", b.markers.size(), L_NUM_VELS);
    for (size_t m = 0; m < b.markers.size(); ++m) {
        for (int v = 0; v < L_NUM_VELS; ++v) std::fprintf(fp, "%.17g ", b.Q[v + L_NUM_VELS * m]);
        std::fprintf(fp, "\n");
    }
    for (int i = 0; i < g->N_lim; ++i)
        for (int j = 0; j < g->M_lim; ++j)
            for (int k = 0; k < g->K_lim; ++k) {
                MarkerData *md = b.getMarkerData(g->XPos[i], g->YPos[j], g->ZPos[k]);
                std::fprintf(fp, "%d\n", md->isValid() ? md->ID : -1);
                delete md;
            }
    std::fclose(fp);
}

static void reinit_equilibrium(GridObj *g) {
    const int n = g->N_lim * g->M_lim * g->K_lim;
    for (int id = 0; id < n; ++id)
        for (int v = 0; v < L_NUM_VELS; ++v) g->f[v + id * L_NUM_VELS] = g->_LBM_equilibrium_opt(id, v);
    g->feq = g->f;
    g->fNew = g->f;
}

int main(int argc, char **argv) {
    std::string out = ".", init_u, init_rho, workdir, markers, drag_out, momex_out, bfl_out, bfl_forces;
    int steps = 0, dump_every = 0, io_at = -1;
    bool restart_read = false;
    int shim_prec = -1;
    for (int a = 1; a < argc; ++a) {
        std::string k = argv[a];
        auto next = [&]() -> std::string {
            if (a + 1 >= argc) { std::fprintf(stderr, "missing value for %s\n", k.c_str()); std::exit(2); }
            return argv[++a];
        };
        if (k == "--out") out = next();
        else if (k == "--steps") steps = std::atoi(next().c_str());
        else if (k == "--dump-every") dump_every = std::atoi(next().c_str());
        else if (k == "--init-u") init_u = next();
        else if (k == "--init-rho") init_rho = next();
        else if (k == "--workdir") workdir = next();
        else if (k == "--markers") markers = next();
        else if (k == "--drag-out") drag_out = next();
        else if (k == "--momex-out") momex_out = next();
        else if (k == "--bfl-out") bfl_out = next();
        else if (k == "--bfl-forces") bfl_forces = next();
        else if (k == "--io-at") io_at = std::atoi(next().c_str());
        else if (k == "--restart-read") restart_read = true;
        else if (k == "--gpu-shim") shim_prec = std::atoi(next().c_str());
        else { std::fprintf(stderr, "unknown argument %s\n", k.c_str()); return 2; }
    }
    mkdir(out.c_str(), 0755);
    char outabs[4096];
    if (!realpath(out.c_str(), outabs)) { std::perror("realpath"); return 2; }
    out = outabs;
    if (!workdir.empty() && chdir(workdir.c_str()) != 0) { std::perror("chdir"); return 2; }

    GridUtils::path_str = out;
    std::ofstream logfile((out + "/log.txt").c_str(), std::ios::out);
    GridUtils::logfile = &logfile;

    GridManager *gm = GridManager::getInstance();
    GridObj *const grids = new GridObj(0);
    if (L_NUM_LEVELS != 0)
        for (int reg = 0; reg < L_NUM_REGIONS; ++reg) grids->LBM_addSubGrid(reg);
    gm->setGridHierarchy(grids);

    const size_t ncell = (size_t)grids->N_lim * grids->M_lim * grids->K_lim;
    if (!init_u.empty()) {
        std::vector<double> u = read_raw(init_u, ncell * L_DIMS);
        for (size_t i = 0; i < u.size(); ++i) grids->u[i] = u[i];
    }
    if (!init_rho.empty()) {
        std::vector<double> r = read_raw(init_rho, ncell);
        for (size_t i = 0; i < r.size(); ++i) grids->rho[i] = r[i];
    }
    if (!init_u.empty() || !init_rho.empty()) {
        reinit_equilibrium(grids);
#ifdef L_IBM_ON
        grids->u_n = grids->u;
#endif
    }

    ObjectManager *om = ObjectManager::getInstance(grids);
#ifdef L_GEOMETRY_FILE
    om->io_readInGeomConfig();
#endif
#ifdef L_IBM_ON
    if (!markers.empty()) inject_markers(om, grids, markers);
#endif
#ifdef L_IBM_ON
    om->ibm_initialise();
#endif
    (void)om;
    if (restart_read) grids->io_restart(eRead);
    if (!bfl_out.empty()) dump_bfl(grids, bfl_out);
    FILE *bf = bfl_forces.empty() ? nullptr : std::fopen(bfl_forces.c_str(), "w");

#ifdef L_LD_OUT
    // Momentum-exchange force of the solid sites of L0, reset every step
    // (resetMomexBodyForces resets only the grid a bounce-back body was
    // read onto).
    FILE *mf = momex_out.empty() ? nullptr : std::fopen(momex_out.c_str(), "w");
    if (mf) {
        om->bbbOnGridLevel = 0;
        om->bbbOnGridReg = 0;
    }
#endif
#ifdef LUMA_HARNESS_SHIM
    if (shim_prec >= 0 && LumaGpuShim::create(grids, shim_prec) != 0) {
        std::fprintf(stderr, "shim create failed: %s\n", luma_gpu_last_error_string());
        return 3;
    }
    auto step_once = [&]() {
        if (shim_prec < 0) { grids->LBM_multi_opt(); return; }
        if (LumaGpuShim::step(grids, 1) != 0 || LumaGpuShim::sync_to_host(grids) != 0) {
            std::fprintf(stderr, "shim step failed: %s\n", luma_gpu_last_error_string());
            std::exit(3);
        }
    };
#else
    if (shim_prec >= 0) { std::fprintf(stderr, "--gpu-shim needs a build with the shim\n"); return 2; }
    auto step_once = [&]() { grids->LBM_multi_opt(); };
#endif
    if (drag_out.empty()) dump_all(grids, out, 0);
    double drag_sum = 0.0;
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 1; s <= steps; ++s) {
        step_once();
#ifdef L_LD_OUT
        if (mf)
            std::fprintf(mf, "%d %.17g %.17g %.17g\n", s, om->bbbForceOnObjectX, om->bbbForceOnObjectY,
                         om->bbbForceOnObjectZ);
#endif
        if (bf && !om->pBody.empty())
            for (size_t m = 0; m < om->pBody[0].markers.size(); ++m) {
                const BFLMarker &mk = om->pBody[0].markers[m];
                std::fprintf(bf, "%d %zu %.17g %.17g %.17g\n", s, m, mk.forceX, mk.forceY, mk.forceZ);
            }
        if (s == io_at) {
            // io_lite prefixes "./" to the output path: run it from / so
            // that the absolute path stays absolute
            char cwd[4096];
            if (!getcwd(cwd, sizeof cwd) || chdir("/") != 0) { std::perror("chdir"); return 2; }
            grids->io_lite(s, "");
            if (chdir(cwd) != 0) { std::perror("chdir"); return 2; }
            grids->io_restart(eWrite);
        }
        if (!drag_out.empty()) drag_sum += body_drag();
        else if ((dump_every > 0 && s % dump_every == 0) || s == steps) dump_all(grids, out, s);
    }
#ifdef L_LD_OUT
    if (mf) std::fclose(mf);
#endif
    if (bf) std::fclose(bf);
    if (!drag_out.empty()) {
        FILE *df = std::fopen(drag_out.c_str(), "w");
        std::fprintf(df, "%.17g %d\n", steps > 0 ? drag_sum / steps : 0.0, steps);
        std::fclose(df);
    }
    auto t1 = std::chrono::steady_clock::now();
    double sec = std::chrono::duration<double>(t1 - t0).count();
    FILE *tf = std::fopen((out + "/timing.txt").c_str(), "w");
    std::fprintf(tf, "steps %d\nseconds %.6f\ncells %zu\n", steps, sec, ncell);
    std::fclose(tf);
    logfile.close();
    return 0;
}
