// Output of grid state in the reference's ASCII formats, fed by device
// snapshots.
//
// GridObj::io_lite (LUMA src/GridObj_ops_io.cpp:706-810): one file per grid,
// <dir>/io_lite.Lev<l>.Reg<r>.Rnk<rank>.<(int)t>.dat, one line per site in
// (k, j, i) order (i fastest): rank, label, X, Y, Z, rho, u (a 0.000000
// z-column in 2D), f[Q], fNew[Q], every value followed by a tab, doubles in
// fixed notation with the writer's precision (L_OUTPUT_PRECISION).
//
// GridObj::io_restart(eWrite) (:406-490): <dir>/restart_LBM_Rnk<rank>.out,
// level 0 first and every sub-grid appended after its parent (depth first,
// region order), one line per site in (k, j, i) order: level, region, X, Y,
// Z, u in dimensionless units (u dh / dt), rho, and per direction the scaled
// non-equilibrium part ((f - feq) omega) / (feq dt), with feq from the
// site's rho and u as _LBM_equilibrium_opt (:674-705) evaluates it; values in
// the stream's default format (6 significant digits).
//
// The ostream insertions the reference uses format a double as printf's
// "%.*f" (fixed) and "%.6g" (default) do, so the writers use those.
//
// luma_gpu_io_lite / luma_gpu_io_restart take the snapshot on the calling
// thread (device -> host, reference layout, FP64) and leave the formatting
// and the file writes to a host thread: they return once the state is on
// the host, while the GPU steps on.  luma_gpu_io_wait joins the writers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "grid.hpp"
#include "lattice.cuh"
#include "dispatch.hpp"
#include "kernels.hpp"

using namespace luma;

namespace luma {
struct IoJobs {
    std::vector<std::thread> threads;
    std::mutex mu;
    int status = LUMA_OK;
    std::string message;
};
}  // namespace luma

namespace {

// One grid's state in the reference layout with what the writers print.
struct Snapshot {
    int level = 0, region = 0, N = 0, M = 0, K = 0, Q = 0, dims = 0;
    double dt = 0, dh = 0, omega = 0;
    std::vector<int> typ;
    std::vector<double> x, y, z, f, fnew, u, rho;
    std::vector<double> rho_ta, ui_ta, uiuj_ta;  // empty without time averages
};

void lattice_c(int Q, int v, int c[3]) {
    for (int d = 0; d < 3; ++d)
        c[d] = Q == 9 ? Lattice<9>::c(v, d) : (Q == 19 ? Lattice<19>::c(v, d) : Lattice<27>::c(v, d));
}
double lattice_w(int Q, int v) { return Q == 9 ? Lattice<9>::w(v) : (Q == 19 ? Lattice<19>::w(v) : Lattice<27>::w(v)); }

// _LBM_equilibrium_opt with the reference's expression structure (integer
// lattice products, cs = 1/sqrt(3) squared in place).
double feq(int Q, int dims, int v, double rho, const double *u) {
    int c[3];
    lattice_c(Q, v, c);
    const double cs = 1.0 / std::sqrt(3.0);
    double A, B;
    if (dims == 3) {
        A = (c[0] * u[0]) + (c[1] * u[1]) + (c[2] * u[2]);
        B = ((c[0] * c[0]) - (cs * cs)) * (u[0] * u[0]) + ((c[1] * c[1]) - (cs * cs)) * (u[1] * u[1]) +
            ((c[2] * c[2]) - (cs * cs)) * (u[2] * u[2]) + 2 * c[0] * c[1] * u[0] * u[1] +
            2 * c[0] * c[2] * u[0] * u[2] + 2 * c[1] * c[2] * u[1] * u[2];
    } else {
        A = (c[0] * u[0]) + (c[1] * u[1]);
        B = ((c[0] * c[0]) - (cs * cs)) * (u[0] * u[0]) + ((c[1] * c[1]) - (cs * cs)) * (u[1] * u[1]) +
            2 * c[0] * c[1] * u[0] * u[1];
    }
    return rho * lattice_w(Q, v) * (1.0 + (A / (cs * cs)) + (B / (2.0 * (cs * cs) * (cs * cs))));
}

struct Out {
    FILE *fp;
    std::string buf;
    char tmp[64];
    void d(int v) { buf += std::to_string(v); buf += '\t'; }
    void fixed(double v, int prec) {
        std::snprintf(tmp, sizeof tmp, "%.*f", prec, v);
        buf += tmp;
        buf += '\t';
    }
    void gen(double v) {
        std::snprintf(tmp, sizeof tmp, "%.6g", v);
        buf += tmp;
        buf += '\t';
    }
    void raw(const char *s) { buf += s; }
    bool flush(bool force = false) {
        if (!force && buf.size() < (1u << 20)) return true;
        const bool ok = std::fwrite(buf.data(), 1, buf.size(), fp) == buf.size();
        buf.clear();
        return ok;
    }
};

int write_lite(const Snapshot &s, const std::string &dir, double tval, int prec, int rank) {
    const std::string path = dir + "/io_lite.Lev" + std::to_string(s.level) + ".Reg" + std::to_string(s.region) +
                             ".Rnk" + std::to_string(rank) + "." + std::to_string((int)tval) + ".dat";
    FILE *fp = std::fopen(path.c_str(), "w");
    if (!fp) return luma_set_error(LUMA_E_INVALID, "io_lite: cannot open %s: %s", path.c_str(), std::strerror(errno));
    Out o{fp, {}, {}};
    o.buf.reserve(1u << 21);
    const char *zero = "0.000000\t";  // std::to_string(0.0)
    bool ok = true;
    for (int k = 0; k < s.K && ok; ++k)
        for (int j = 0; j < s.M && ok; ++j)
            for (int i = 0; i < s.N && ok; ++i) {
                const size_t id = (size_t)k + (size_t)j * s.K + (size_t)i * s.K * s.M;
                o.d(rank);
                o.d(s.typ[id]);
                o.fixed(s.x[i], prec);
                o.fixed(s.y[j], prec);
                o.fixed(s.z[k], prec);
                o.fixed(s.rho[id], prec);
                for (int d = 0; d < s.dims; ++d) o.fixed(s.u[id * s.dims + d], prec);
                if (s.dims != 3) o.raw(zero);
                for (int v = 0; v < s.Q; ++v) o.fixed(s.f[v + id * s.Q], prec);
                for (int v = 0; v < s.Q; ++v) o.fixed(s.fnew[v + id * s.Q], prec);
                if (!s.rho_ta.empty()) {
                    // the time-averaged columns (:764-791): rho, u (a zero
                    // z-column in 2D), then the u u products padded to six
                    const int npq = 3 * s.dims - 3;
                    const double *uu = &s.uiuj_ta[id * npq];
                    o.fixed(s.rho_ta[id], prec);
                    for (int d = 0; d < s.dims; ++d) o.fixed(s.ui_ta[id * s.dims + d], prec);
                    if (s.dims != 3) o.raw(zero);
                    o.fixed(uu[0], prec);
                    o.fixed(uu[1], prec);
                    if (s.dims == 3) {
                        for (int q = 2; q < 6; ++q) o.fixed(uu[q], prec);
                    } else {
                        o.raw(zero);
                        o.fixed(uu[2], prec);
                        o.raw(zero);
                        o.raw(zero);
                    }
                }
                o.raw("\n");
                ok = o.flush();
            }
    ok = ok && o.flush(true);
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? LUMA_OK : luma_set_error(LUMA_E_INVALID, "io_lite: write to %s failed", path.c_str());
}

int write_restart(const Snapshot &s, FILE *fp) {
    Out o{fp, {}, {}};
    o.buf.reserve(1u << 21);
    bool ok = true;
    for (int k = 0; k < s.K && ok; ++k)
        for (int j = 0; j < s.M && ok; ++j)
            for (int i = 0; i < s.N && ok; ++i) {
                const size_t id = (size_t)k + (size_t)j * s.K + (size_t)i * s.K * s.M;
                o.d(s.level);
                o.d(s.region);
                o.gen(s.x[i]);
                o.gen(s.y[j]);
                o.gen(s.z[k]);
                const double *u = &s.u[id * s.dims];
                for (int d = 0; d < s.dims; ++d) o.gen((u[d] * s.dh) / s.dt);
                o.gen(s.rho[id]);
                for (int v = 0; v < s.Q; ++v) {
                    const double fe = feq(s.Q, s.dims, v, s.rho[id], u);
                    o.gen(((s.f[v + id * s.Q] - fe) * s.omega) / (fe * s.dt));
                }
                o.raw("\n");
                ok = o.flush();
            }
    ok = ok && o.flush(true);
    return ok ? LUMA_OK : luma_set_error(LUMA_E_INVALID, "io_restart: write failed");
}

int from_desc(const luma_grid_desc *d, const double *f, const double *fnew, const double *u, const double *rho,
              Snapshot &s) {
    if (!d || !d->lattyp || !d->xpos || !d->ypos || !d->zpos || !f || !u || !rho)
        return luma_set_error(LUMA_E_INVALID, "writer: descriptor labels/positions and f, u, rho are required");
    const size_t n = (size_t)d->N * d->M * d->K;
    s.level = d->level; s.region = d->region; s.N = d->N; s.M = d->M; s.K = d->K; s.Q = d->Q; s.dims = d->dims;
    s.dt = d->dt; s.dh = d->dh; s.omega = d->omega;
    s.typ.assign(d->lattyp, d->lattyp + n);
    s.x.assign(d->xpos, d->xpos + d->N);
    s.y.assign(d->ypos, d->ypos + d->M);
    s.z.assign(d->zpos, d->zpos + d->K);
    s.f.assign(f, f + n * d->Q);
    s.fnew.assign(fnew ? fnew : f, (fnew ? fnew : f) + n * d->Q);
    s.u.assign(u, u + n * d->dims);
    s.rho.assign(rho, rho + n);
    return LUMA_OK;
}

int set_averages(Snapshot &s, const double *rho_ta, const double *ui_ta, const double *uiuj_ta) {
    if (!rho_ta && !ui_ta && !uiuj_ta) return LUMA_OK;
    if (!rho_ta || !ui_ta || !uiuj_ta) return luma_set_error(LUMA_E_INVALID, "writer: give all three time averages");
    const size_t n = (size_t)s.N * s.M * s.K;
    s.rho_ta.assign(rho_ta, rho_ta + n);
    s.ui_ta.assign(ui_ta, ui_ta + n * s.dims);
    s.uiuj_ta.assign(uiuj_ta, uiuj_ta + n * (3 * s.dims - 3));
    return LUMA_OK;
}

// Device -> host snapshot of one grid (reference layout, FP64).  fNew is the
// other population buffer of the two-buffer path (the state before the
// latest step, as the reference's fNew holds after its swap); the in-place
// path keeps one buffer and reports f there.
int take(luma_gpu_grid *g, Snapshot &s) {
    const luma_grid_desc &d = g->d;
    s.level = d.level; s.region = d.region; s.N = d.N; s.M = d.M; s.K = d.K; s.Q = d.Q; s.dims = d.dims;
    s.dt = d.dt; s.dh = d.dh; s.omega = d.omega;
    s.typ.assign(g->htyp.begin(), g->htyp.end());
    if (g->hx.size() != (size_t)d.N || g->hy.size() != (size_t)d.M || g->hz.size() != (size_t)d.K)
        return luma_set_error(LUMA_E_STATE, "writer: the grid was created without site positions");
    s.x = g->hx; s.y = g->hy; s.z = g->hz;
    s.f.resize(g->n * d.Q);
    s.u.resize(g->n * d.dims);
    s.rho.resize(g->n);
    int rc = luma_gpu_download_state(g, s.f.data(), s.u.data(), s.rho.data(), nullptr);
    if (rc) return rc;
    if (g->tav) {
        s.rho_ta.resize(g->n);
        s.ui_ta.resize(g->n * d.dims);
        s.uiuj_ta.resize(g->n * (3 * d.dims - 3));
        if ((rc = luma_gpu_download_time_averages(g, s.rho_ta.data(), s.ui_ta.data(), s.uiuj_ta.data()))) return rc;
    }
    if (g->bulk) {
        s.fnew = s.f;
        return LUMA_OK;
    }
    s.fnew.resize(g->n * d.Q);
    double *stage = nullptr;
    cudaStream_t st = g->stream;
    if (cudaMallocAsync(&stage, g->n * d.Q * sizeof(double), st) != cudaSuccess)
        return luma_set_error(LUMA_E_NOMEM, "writer: staging allocation failed");
    cudaError_t e = dispatch(d.Q, d.precision, [&](auto q, auto p) {
        return launch_pop_out<decltype(q)::value, decltype(p)>(g->f[g->cur ^ 1], stage, d.N, d.M, d.K, kPopPlain,
                                                              d.rho_in, st);
    });
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.fnew.data(), stage, g->n * d.Q * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(stage, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? LUMA_OK : luma_set_error(LUMA_E_CUDA, "writer snapshot: %s", cudaGetErrorString(e));
}

// The tree in the reference's recursion order (parent, then each sub-grid's
// subtree in region order).
int take_tree(luma_gpu_grid *g, std::vector<Snapshot> &out) {
    out.emplace_back();
    if (int rc = take(g, out.back())) return rc;
    for (luma_gpu_grid *c : g->kids)
        if (int rc = take_tree(c, out)) return rc;
    return LUMA_OK;
}

IoJobs &jobs(luma_gpu_grid *root) {
    if (!root->io) root->io = new IoJobs();
    return *root->io;
}

void record(IoJobs &J, int rc) {
    if (rc == LUMA_OK) return;
    std::lock_guard<std::mutex> lk(J.mu);
    if (J.status == LUMA_OK) {
        J.status = rc;
        J.message = luma_gpu_last_error_string();
    }
}

// ObjectManager::io_restart(eWrite) (src/ObjectManager_ops_io.cpp:136-190):
// the number of bodies and a newline, then per body a "\t/\t" separator,
// its marker count, "\t/\t", and per marker x, y, z (and, for a flexible
// body, the old position) each followed by a tab; no final newline.
int write_ibbody(const char *path, int nbodies, const int *nmarkers, const int *flexible, const double *positions,
                 const double *positions0) {
    FILE *fp = std::fopen(path, "w");
    if (!fp) return luma_set_error(LUMA_E_INVALID, "io_restart: cannot open %s", path);
    Out o{fp, {}, {}};
    o.buf += std::to_string(nbodies);
    o.buf += '\n';
    size_t m0 = 0;
    int rc = LUMA_OK;
    for (int b = 0; b < nbodies && rc == LUMA_OK; ++b) {
        const bool flex = flexible && flexible[b];
        if (flex && !positions0) {
            rc = luma_set_error(LUMA_E_INVALID, "io_restart: flexible body %d needs old positions", b);
            break;
        }
        o.raw("\t/\t");
        o.buf += std::to_string(nmarkers[b]);
        o.raw("\t/\t");
        for (int m = 0; m < nmarkers[b]; ++m) {
            const size_t g = m0 + (size_t)m;
            for (int d = 0; d < 3; ++d) o.gen(positions[3 * g + d]);
            if (flex)
                for (int d = 0; d < 3; ++d) o.gen(positions0[3 * g + d]);
        }
        m0 += (size_t)nmarkers[b];
    }
    const bool ok = o.flush(true);
    if (std::fclose(fp) != 0 || !ok) rc = rc ? rc : luma_set_error(LUMA_E_INVALID, "io_restart: write failed");
    return rc;
}

// The IB bodies of a tree for the restart file, in the order they were
// created (ObjectManager's iBody order): each body's current marker
// positions (a filament's from the device) and, for filaments, the
// markers' initial positions (IBMarker::position0); rigid bodies' entries
// of pos0 are zeros the writer does not read.
struct IbBodies {
    std::vector<int> nm, flex;
    std::vector<double> pos, pos0;
};

int take_ib_bodies(luma_gpu_grid *root, IbBodies &out) {
    struct Entry {
        long long seq;
        int nm, flex;
        std::vector<double> pos, pos0;
    };
    std::vector<Entry> all;
    std::vector<luma_gpu_grid *> todo{root};
    while (!todo.empty()) {
        luma_gpu_grid *g = todo.back();
        todo.pop_back();
        for (luma_gpu_grid *c : g->kids) todo.push_back(c);
        if (!g->ibm) continue;
        const luma::IbmState &st = *g->ibm;
        std::vector<int> fidx(st.bodies.size(), -1), fbase(st.bodies.size(), 0);
        int base = 0;
        for (size_t k = 0; k < st.flex_body.size(); ++k) {
            fidx[st.flex_body[k]] = (int)k;
            fbase[st.flex_body[k]] = base;
            base += st.flex[k].nm;
        }
        for (size_t b = 0; b < st.bodies.size(); ++b) {
            const luma::IbmBody &bd = st.bodies[b];
            Entry e{bd.seq, bd.nm, fidx[b] >= 0 ? 1 : 0, bd.pos, std::vector<double>(3 * (size_t)bd.nm, 0.0)};
            if (e.flex) {
                e.pos0 = st.flex[fidx[b]].mpos0;
                if (st.ready) {
                    cudaError_t err = cudaStreamSynchronize(g->stream);
                    if (err == cudaSuccess)
                        err = cudaMemcpy(e.pos.data(), st.fem.flex.pos + 3 * (size_t)fbase[b],
                                         e.pos.size() * sizeof(double), cudaMemcpyDeviceToHost);
                    if (err != cudaSuccess)
                        return luma_set_error(LUMA_E_CUDA, "io_restart: filament markers: %s", cudaGetErrorString(err));
                }
            }
            all.push_back(std::move(e));
        }
    }
    std::sort(all.begin(), all.end(), [](const Entry &a, const Entry &b) { return a.seq < b.seq; });
    for (const Entry &e : all) {
        out.nm.push_back(e.nm);
        out.flex.push_back(e.flex);
        out.pos.insert(out.pos.end(), e.pos.begin(), e.pos.end());
        out.pos0.insert(out.pos0.end(), e.pos0.begin(), e.pos0.end());
    }
    return LUMA_OK;
}
}  // namespace

void luma_io_free(luma_gpu_grid *g) {
    if (!g->io) return;
    for (std::thread &t : g->io->threads)
        if (t.joinable()) t.join();
    delete g->io;
    g->io = nullptr;
}

extern "C" {

int luma_gpu_io_lite(luma_gpu_grid *root, const char *dir, double tval, int precision, int rank) {
    if (!root || !dir || precision < 0 || precision > 30)
        return luma_set_error(LUMA_E_INVALID, "luma_gpu_io_lite: null argument or precision outside 0..30");
    if (root->parent) return luma_set_error(LUMA_E_INVALID, "luma_gpu_io_lite takes the level-0 grid");
    auto snaps = std::make_shared<std::vector<Snapshot>>();
    if (int rc = take_tree(root, *snaps)) return rc;
    IoJobs &J = jobs(root);
    const std::string d(dir);
    J.threads.emplace_back([snaps, d, tval, precision, rank, &J] {
        for (const Snapshot &s : *snaps) record(J, write_lite(s, d, tval, precision, rank));
    });
    return LUMA_OK;
}

int luma_gpu_io_restart(luma_gpu_grid *root, const char *dir, int rank) {
    if (!root || !dir) return luma_set_error(LUMA_E_INVALID, "luma_gpu_io_restart: null argument");
    if (root->parent) return luma_set_error(LUMA_E_INVALID, "luma_gpu_io_restart takes the level-0 grid");
    auto snaps = std::make_shared<std::vector<Snapshot>>();
    if (int rc = take_tree(root, *snaps)) return rc;
    IoJobs &J = jobs(root);
    // with IBM on (L_IBM_ON), level 0's GridObj::io_restart also has the
    // ObjectManager write every IB body (src/GridObj_ops_io.cpp:484-487)
    std::shared_ptr<IbBodies> ib;
    if (root->d.flags & LUMA_FLAG_IBM) {
        ib = std::make_shared<IbBodies>();
        if (int rc = take_ib_bodies(root, *ib)) return rc;
    }
    const std::string path = std::string(dir) + "/restart_LBM_Rnk" + std::to_string(rank) + ".out";
    const std::string ibpath = std::string(dir) + "/restart_IBBody_Rnk" + std::to_string(rank) + ".out";
    J.threads.emplace_back([snaps, ib, path, ibpath, &J] {
        FILE *fp = std::fopen(path.c_str(), "w");
        if (!fp) {
            record(J, luma_set_error(LUMA_E_INVALID, "io_restart: cannot open %s", path.c_str()));
            return;
        }
        for (const Snapshot &s : *snaps) record(J, write_restart(s, fp));
        if (std::fclose(fp) != 0) record(J, luma_set_error(LUMA_E_INVALID, "io_restart: close of %s failed", path.c_str()));
        if (ib)
            record(J, write_ibbody(ibpath.c_str(), (int)ib->nm.size(), ib->nm.data(), ib->flex.data(),
                                   ib->pos.data(), ib->pos0.data()));
    });
    return LUMA_OK;
}

int luma_gpu_io_wait(luma_gpu_grid *root) {
    if (!root) return luma_set_error(LUMA_E_INVALID, "null grid");
    if (!root->io) return LUMA_OK;
    IoJobs &J = *root->io;
    for (std::thread &t : J.threads)
        if (t.joinable()) t.join();
    J.threads.clear();
    const int rc = J.status;
    const std::string msg = J.message;
    J.status = LUMA_OK;
    J.message.clear();
    return rc == LUMA_OK ? LUMA_OK : luma_set_error(rc, "%s", msg.c_str());
}

int luma_io_lite_write(const luma_grid_desc *desc, const double *f, const double *fnew, const double *u,
                       const double *rho, const double *rho_ta, const double *ui_ta, const double *uiuj_ta,
                       const char *dir, double tval, int precision, int rank) {
    if (!dir || precision < 0 || precision > 30)
        return luma_set_error(LUMA_E_INVALID, "luma_io_lite_write: null directory or precision outside 0..30");
    Snapshot s;
    if (int rc = from_desc(desc, f, fnew, u, rho, s)) return rc;
    if (int rc = set_averages(s, rho_ta, ui_ta, uiuj_ta)) return rc;
    return write_lite(s, dir, tval, precision, rank);
}

// GridObj::io_restart(eRead) (:490-580) called on level 0: every line of
// the file sets u (dimensionless -> lattice: u dt / dh), rho and f of the
// site of its (level, region) grid that encloses its position, with
// f = feq (1 + dt f_neq / omega).  As the reference does, feq is level 0's
// equilibrium at the index (k + j K0 + i K0 M0) with level 0's rho and u,
// and omega is level 0's, whatever grid the line belongs to.  Lines whose
// position lies outside level 0's domain, or off their grid, are skipped.
int luma_io_restart_read(const char *path, int ngrids, const luma_grid_desc *const *descs, double *const *f,
                         double *const *u, double *const *rho) {
    if (!path || ngrids <= 0 || !descs || !f || !u || !rho)
        return luma_set_error(LUMA_E_INVALID, "luma_io_restart_read: null argument");
    for (int g = 0; g < ngrids; ++g)
        if (!descs[g] || !f[g] || !u[g] || !rho[g] || !descs[g]->xpos || !descs[g]->ypos || !descs[g]->zpos)
            return luma_set_error(LUMA_E_INVALID, "luma_io_restart_read: grid %d lacks arrays or positions", g);
    const luma_grid_desc &L0 = *descs[0];
    if (L0.level != 0) return luma_set_error(LUMA_E_INVALID, "luma_io_restart_read: descs[0] must be level 0");
    std::ifstream in(path);
    if (!in.is_open()) return luma_set_error(LUMA_E_INVALID, "io_restart: cannot open %s", path);
    const int D = L0.dims, Q = L0.Q;
    const double *E = L0.global_edges;
    std::string line;
    while (std::getline(in, line)) {
        const char *p = line.c_str();
        char *end;
        auto num = [&](double &v) -> bool {
            v = std::strtod(p, &end);
            if (end == p) return false;
            p = end;
            return true;
        };
        double lv, rg, x, y, z;
        if (!num(lv) || !num(rg) || !num(x) || !num(y) || !num(z)) continue;  // blank or short line
        int gi = -1;
        for (int g = 0; g < ngrids; ++g)
            if (descs[g]->level == (int)lv && descs[g]->region == (int)rg) gi = g;
        if (gi < 0)
            return luma_set_error(LUMA_E_INVALID, "io_restart: no grid level %d region %d", (int)lv, (int)rg);
        const luma_grid_desc &G = *descs[gi];
        // GridUtils::isOnThisRank (serial): inside level 0's edges, then the
        // enclosing voxel of the line's grid must be on that grid
        if (!(E[0] <= x && x < E[1] && E[2] <= y && y < E[3] && (D != 3 || (E[4] <= z && z < E[5])))) continue;
        const double sx = G.level == 0 ? E[0] : G.xpos[0] - 0.5 * G.dh;
        const double sy = G.level == 0 ? E[2] : G.ypos[0] - 0.5 * G.dh;
        const double sz = G.level == 0 ? E[4] : G.zpos[0] - 0.5 * G.dh;
        const int i = (int)std::floor((x - sx) / G.dh), j = (int)std::floor((y - sy) / G.dh);
        const int k = D == 3 ? (int)std::floor((z - sz) / G.dh) : 0;
        if (i < 0 || i >= G.N || j < 0 || j >= G.M || k < 0 || k >= G.K) continue;
        const size_t gid = (size_t)k + (size_t)j * G.K + (size_t)i * G.K * G.M;
        const size_t id0 = (size_t)k + (size_t)j * L0.K + (size_t)i * L0.K * L0.M;  // level 0's strides
        double vals[3 + 1 + 27];
        int nv = 0;
        for (; nv < D + 1 + Q; ++nv)
            if (!num(vals[nv])) break;
        if (nv < D + 1 + Q) return luma_set_error(LUMA_E_INVALID, "io_restart: short line in %s", path);
        for (int d = 0; d < D; ++d) u[gi][gid * D + d] = (vals[d] * G.dt) / G.dh;
        rho[gi][gid] = vals[D];
        for (int v = 0; v < Q; ++v) {
            const double fe = feq(Q, D, v, rho[0][id0], &u[0][id0 * D]);
            f[gi][gid * Q + v] = fe * (1 + (G.dt * vals[D + 1 + v]) / L0.omega);
        }
    }
    return LUMA_OK;
}

int luma_io_ibbody_restart_write(const char *path, int nbodies, const int *nmarkers, const int *flexible,
                                 const double *positions, const double *positions0) {
    if (!path || nbodies < 0 || (nbodies > 0 && (!nmarkers || !positions)))
        return luma_set_error(LUMA_E_INVALID, "luma_io_ibbody_restart_write: null argument");
    return write_ibbody(path, nbodies, nmarkers, flexible, positions, positions0);
}

int luma_io_restart_write(const luma_grid_desc *desc, const double *f, const double *u, const double *rho,
                          const char *path, int append) {
    if (!path) return luma_set_error(LUMA_E_INVALID, "luma_io_restart_write: null path");
    Snapshot s;
    if (int rc = from_desc(desc, f, nullptr, u, rho, s)) return rc;
    FILE *fp = std::fopen(path, append ? "a" : "w");
    if (!fp) return luma_set_error(LUMA_E_INVALID, "io_restart: cannot open %s", path);
    int rc = write_restart(s, fp);
    if (std::fclose(fp) != 0 && rc == LUMA_OK) rc = luma_set_error(LUMA_E_INVALID, "io_restart: close failed");
    return rc;
}

}  // extern "C"
