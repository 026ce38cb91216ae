// C ABI of the GB300 rans library (include/afx_rans.h) and the host
// orchestration of the device path: buffers, CUDA-graph capture of iteration
// chunks, the run_solver loop with a device-resident convergence test, and
// the reference-order <-> device-order state exchange.
#include "../../include/afx_rans.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "afx_host.hpp"
#include "afx_krylov.hpp"
#include "afx_launch.hpp"

namespace afx {
void enqueue_permute_in(int n, const int* cell_old, const void* src, void* dst, cudaStream_t s);
void enqueue_permute_out(int n, const int* cell_old, const void* src, void* dst, cudaStream_t s);
void enqueue_to_f32(int n, const void* src, void* dst, cudaStream_t s);
void enqueue_correction(int n, const void* R64, const void* R32, void* corr, cudaStream_t s);
double fp64_fma_peak(int reps);
long long noalloc_max_cells();
long long noalloc_max_faces();
cudaError_t noalloc_residual_f64(const StepArgs& a, const int* cell_old, const double* q_ref, double* R_ref,
                                 cudaStream_t s);
void enqueue_prolong(int nc, const double* cx, const double* cy, const double* ca, const void* coarse_full, int nf,
                     const double* fx, const double* fy, void* fine_q, cudaStream_t s);
void enqueue_full_state(int n, int nb, const int* cell_old, const int* owner_dev, const void* q, void* full,
                        cudaStream_t s);
void enqueue_wall_seg_dist(int nc, const double* cx, const double* cy, int nw, const double* seg, double* out,
                           cudaStream_t s);
void enqueue_wall_dist(int nc, const double* cx, const double* cy, int nw, const double* wx, const double* wy,
                       double* out, cudaStream_t s);
struct ImplicitEngine;
ImplicitEngine* implicit_create(const StepArgs& a, bool f32, bool graph, const std::vector<int>& colors,
                                const int* cslot, const int* cnbr, cudaStream_t s);
void implicit_destroy(ImplicitEngine* e);
void implicit_fill(ImplicitEngine* e, const StepArgs& a, int p, cudaStream_t s);
int implicit_solve_update(ImplicitEngine* e, const StepArgs& a, int p, const double* b, double relax,
                          cudaStream_t s);
void implicit_transpose(ImplicitEngine* e, cudaStream_t s);
int implicit_apply_inverse(ImplicitEngine* e, const StepArgs& a, const double* b, const double* area, double scale,
                           double* out, cudaStream_t s);
int implicit_apply_sweep(ImplicitEngine* e, const StepArgs& a, const double* b, const double* area, double scale,
                         double* out, cudaStream_t s);
}  // namespace afx

using namespace afx;

static thread_local std::string g_err;

#define AFX_CUDA(x)                                                                                      \
    do {                                                                                                 \
        cudaError_t e_ = (x);                                                                            \
        if (e_ != cudaSuccess) throw Error(AFX_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class F>
static int guarded(F&& f) {
    try {
        f();
        return AFX_OK;
    } catch (const Error& e) {
        g_err = e.what();
        return e.code;
    } catch (const std::out_of_range& e) {
        g_err = std::string("unknown name: ") + e.what();
        return AFX_ERR_ARG;
    } catch (const std::exception& e) {
        g_err = e.what();
        return AFX_ERR_ARG;
    }
}

struct afx_mesh_s {
    HostMesh m;
    DeviceLayout L;
    bool has_layout = false;
    const DeviceLayout& layout() {
        if (!has_layout) {
            L = build_layout(m);
            has_layout = true;
        }
        return L;
    }
};

struct afx_config_s {
    Settings s;
};

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void alloc(size_t n) {
        if (n == 0) n = 16;
        AFX_CUDA(cudaMalloc(&p, n));
        bytes = n;
    }
    void upload(const void* src, size_t n, cudaStream_t s) {
        alloc(n);
        AFX_CUDA(cudaMemcpyAsync(p, src, n, cudaMemcpyHostToDevice, s));
    }
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

template <class T>
std::vector<T> cast_vec(const std::vector<double>& v) {
    return std::vector<T>(v.begin(), v.end());
}

}  // namespace

static void lsq_weights(const HostMesh& m, const DeviceLayout& L, std::vector<double>& lsqw64,
                        std::vector<int>& code);

struct afx_solver_s {
    Settings st;
    // per boundary edge (reference order): patch, owner cell, edge centre, normal, length
    struct BoundaryEdge {
        std::string patch;
        int owner_dev;
        double ex, ey, nx, ny, L;
    };
    std::vector<BoundaryEdge> bedges;
    std::vector<int> cell_old;  // device cell -> reference cell
    std::vector<int32_t> h_fcell, h_cslot;  // device layout topology, for the tile lists
    struct TileData {
        DevBuf hstart, xptr, xlist, ctile;
        int maxnf = 0;
    };
    std::map<int, std::unique_ptr<TileData>> tiles;  // per block size
    bool fp64 = true;
    // FP32-mixed defect correction: an FP64 residual machine on the same FP64
    // master state (FP64 geometry and work arrays), refreshed every
    // corr_interval iterations
    int corr_interval = 0;
    StepArgs a64;
    void* R32buf = nullptr;

    // corr = R64(q) - R32(q) for the state of parity p.  Both residual
    // launches use a64's control block, which is never set to done, so a
    // refresh inside a run leaves the run's own control block alone.  The
    // FP32 gradient/limiter buffers are re-formed by the next iteration.
    void refresh_correction(int p) {
        enqueue_residual_f64(a64, p, stream);
        StepArgs r = a;
        r.Rq = R32buf;
        r.ctrl = a64.ctrl;
        enqueue_residual_f32(r, p, stream);
        enqueue_correction(a.n_cells, a64.Rq, R32buf, (void*)a.corr, stream);
    }

    // Tile lists for `B` cells per tile: faces sorted by their first device
    // cell make each tile's own faces one contiguous range; a face whose two
    // cells lie in different tiles is also listed by the later tile.
    void use_tiles(int B) {
        auto& td = tiles[B];
        if (!td) {
            td.reset(new TileData());
            const int N = a.n_cells, F = a.n_faces;
            const int nt = (N + B - 1) / B;
            std::vector<int> hstart(nt + 1, F), xcount(nt, 0), xidx(F, -1), home(F);
            for (int f = F - 1; f >= 0; --f) {
                const int c0 = h_fcell[2 * f], c1 = h_fcell[2 * f + 1];
                const int hc = c1 >= 0 ? std::min(c0, c1) : c0;
                home[f] = hc / B;
                hstart[home[f]] = f;
            }
            for (int t = nt - 1; t >= 0; --t)
                if (hstart[t] > hstart[t + 1]) hstart[t] = hstart[t + 1];
            for (int f = 0; f < F; ++f) {
                const int c0 = h_fcell[2 * f], c1 = h_fcell[2 * f + 1];
                if (c1 < 0) continue;
                const int t0 = c0 / B, t1 = c1 / B;
                if (t0 != t1) xidx[f] = xcount[std::max(t0, t1)]++;
            }
            std::vector<int> xptr(nt + 1, 0);
            for (int t = 0; t < nt; ++t) xptr[t + 1] = xptr[t] + xcount[t];
            std::vector<int> xlist(std::max(xptr[nt], 1));
            for (int f = 0; f < F; ++f) {
                if (xidx[f] < 0) continue;
                const int t = std::max(h_fcell[2 * f] / B, h_fcell[2 * f + 1] / B);
                xlist[xptr[t] + xidx[f]] = f;
            }
            int maxnf = 0;
            for (int t = 0; t < nt; ++t) maxnf = std::max(maxnf, hstart[t + 1] - hstart[t] + xcount[t]);
            if (maxnf >= 32767) throw Error(AFX_ERR_MESH, "tile face list too long");
            std::vector<short> ctile(4 * (size_t)N, 0);
            for (int i = 0; i < N; ++i) {
                const int t = i / B;
                for (int s = 0; s < 4; ++s) {
                    const int v = h_cslot[4 * (size_t)i + s];
                    if (v == 0) continue;
                    const int f = (v > 0 ? v : -v) - 1;
                    const int lf = home[f] == t ? f - hstart[t] : (hstart[t + 1] - hstart[t]) + xidx[f];
                    ctile[4 * (size_t)i + s] = (short)(v > 0 ? lf + 1 : -(lf + 1));
                }
            }
            td->hstart.upload(hstart.data(), hstart.size() * sizeof(int), stream);
            td->xptr.upload(xptr.data(), xptr.size() * sizeof(int), stream);
            td->xlist.upload(xlist.data(), xlist.size() * sizeof(int), stream);
            td->ctile.upload(ctile.data(), ctile.size() * sizeof(short), stream);
            td->maxnf = maxnf;
            AFX_CUDA(cudaStreamSynchronize(stream));
        }
        a.tile_hstart = (const int*)td->hstart.p;
        a.tile_xptr = (const int*)td->xptr.p;
        a.tile_xlist = (const int*)td->xlist.p;
        a.tile_ctile = td->ctile.p;
        a.tile_maxnf = td->maxnf;
    }

    void set_launch(int variant, int block) {
        a.variant = variant;
        a.block = block;
        if (variant == 2) use_tiles(block);
    }
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    StepArgs a;
    std::vector<std::unique_ptr<DevBuf>> bufs;
    Ctrl* h_ctrl = nullptr;  // pinned
    double* h_stage = nullptr;  // pinned staging for state exchange
    size_t h_stage_bytes = 0;
    DevBuf d_stage, d_cell_old;
    int parity = 0;
    int pending_last = -1;  // parity read by the last iteration whose qW is not materialised
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
    std::atomic<int> stop{0};
    std::vector<double> hist;
    double last_sec = 0;
    std::vector<int> boundary_type;           // per boundary edge
    std::vector<FarfieldVars> boundary_vars;  // solver.h:214-230
    struct PatchForces {
        DevBuf cell, geo, cp, sums;
        int n = 0;
        double xmin = 0, xmax = 0, x_moment = 0, y_moment = 0;
    };
    std::map<std::string, std::unique_ptr<PatchForces>> patches;
    // adjoint work arrays (allocated on first use) and the last adjoint state
    struct AdjointBufs {
        DevBuf v, fbar, gbx, gby, qbar, lw, lt, u, bqbar, g, q, lam[2], ls[2], partials;
        DevBuf lam_obj[2];  // the last implicit adjoint solution of C_L / C_D (initial guess of the next)
        int dirs = 4;       // input directions per pass of the face kernel
        AdjArgs args(const void* v_dev, void* u_dev) const {
            AdjArgs j;
            j.dirs_per_pass = dirs;
            j.v = v_dev;
            j.fbar = fbar.p;
            j.gbx = gbx.p;
            j.gby = gby.p;
            j.qbar = qbar.p;
            j.lw = lw.p;
            j.lt = lt.p;
            j.u = u_dev;
            j.bqbar = bqbar.p;
            return j;
        }
    };
    std::unique_ptr<AdjointBufs> adj;
    int adj_parity = 0;  // lam[adj_parity] holds the last adjoint solution
    std::string adj_patch, adj_objective;  // what the last adjoint solution is of
    // inverse-distance deformation of one boundary patch (afx_deform_patch)
    struct PatchDeform {
        std::string patch;
        double power = 0;
        std::vector<int> pnodes;      // the patch's nodes, ascending
        std::vector<double> pnx, pny; // their unit normals (undeformed mesh)
        std::vector<char> role;       // per node: 0 volume, 1 on the patch, 2 on another boundary (fixed)
        std::vector<double> W;        // per volume node: sum of the inverse-distance weights
    };
    std::unique_ptr<PatchDeform> pdef;
    AdjointBufs& adjoint() {
        if (!fp64) throw Error(AFX_ERR_CONFIG, "the adjoint needs an fp64 solver");
        if (a.visc > 1) throw Error(AFX_ERR_CONFIG, "the adjoint covers the inviscid and laminar fluxes");
        if (a.lsq) throw Error(AFX_ERR_CONFIG, "the adjoint covers the Green-Gauss gradient only");
        if (!adj) {
            const size_t N = a.n_cells, F = a.n_faces, B = std::max(a.n_bnd, 1);
            auto b = std::make_unique<AdjointBufs>();
            b->dirs = st.adjoint_directions;
            for (DevBuf* d : {&b->v, &b->gbx, &b->gby, &b->qbar, &b->u, &b->g, &b->q, &b->lam[0], &b->lam[1],
                              &b->ls[0], &b->ls[1]})
                d->alloc(N * 32);
            b->fbar.alloc(F * (a.visc == 1 ? 256 : 64));
            b->lw.alloc(N * 64);
            b->lt.alloc(N * 32);
            b->bqbar.alloc(B * 32);
            b->partials.alloc(((N + 255) / 256) * 8);
            for (DevBuf* d : {&b->gbx, &b->gby, &b->lw, &b->lt, &b->lam[0], &b->lam[1]})
                AFX_CUDA(cudaMemsetAsync(d->p, 0, d->bytes, stream));
            adj = std::move(b);
        }
        return *adj;
    }

    void* dalloc(size_t n) {
        bufs.emplace_back(new DevBuf());
        bufs.back()->alloc(n);
        AFX_CUDA(cudaMemsetAsync(bufs.back()->p, 0, bufs.back()->bytes, stream));
        return bufs.back()->p;
    }
    template <class T>
    const void* dupload(const std::vector<T>& v) {
        bufs.emplace_back(new DevBuf());
        bufs.back()->upload(v.data(), v.size() * sizeof(T), stream);
        return bufs.back()->p;
    }

    ~afx_solver_s() {
        if (stream) cudaStreamSynchronize(stream);
        implicit_destroy(imp);
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        for (auto& g : graphs64) cudaGraphExecDestroy(g.second);
        if (h_ctrl) cudaFreeHost(h_ctrl);
        if (h_stage) cudaFreeHost(h_stage);
        bufs.clear();
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    // host copies of the mesh and its device layout (the geometry can be
    // deformed: afx_deform_patch)
    HostMesh hm;
    DeviceLayout hl;
    std::vector<double> nodes0x, nodes0y;  // undeformed node coordinates

    // geometry kept on the host: boundary edges for the forces, centroids for
    // grid sequencing
    void host_geometry() {
        const HostMesh& m = hm;
        const DeviceLayout& L = hl;
        bedges.clear();
        for (size_t b = 0; b < m.boundaryEdges.size(); ++b) {
            const uint32_t e = m.boundaryEdges[b];
            bedges.push_back({m.boundaryEdgesPhysicals[b], L.cell_new[m.edgesCells[e][0]], m.edgesCentersX[e],
                              m.edgesCentersY[e], m.edgesNormalsX[e], m.edgesNormalsY[e], m.edgesLengths[e]});
        }
        patches.clear();
        geo_cx = m.cellsCentersX;
        geo_cy = m.cellsCentersY;
        geo_area = m.cellsAreas;
        dev_cx.resize(L.n_cells);
        dev_cy.resize(L.n_cells);
        for (int i = 0; i < L.n_cells; ++i) {
            dev_cx[i] = m.cellsCentersX[L.cell_old[i]];
            dev_cy[i] = m.cellsCentersY[L.cell_old[i]];
        }
        d_geo.reset();
        d_devc.reset();
    }

    // new node coordinates: metrics, device geometry, host geometry
    void set_nodes(const double* x, const double* y) {
        hm.update_nodes(x, y);
        fill_layout_geometry(hm, hl);
        auto put = [&](const void* dst, const std::vector<double>& v, bool f32) {
            if (f32) {
                std::vector<float> f(v.begin(), v.end());
                AFX_CUDA(cudaMemcpyAsync((void*)dst, f.data(), f.size() * 4, cudaMemcpyHostToDevice, stream));
                AFX_CUDA(cudaStreamSynchronize(stream));
            } else {
                AFX_CUDA(cudaMemcpyAsync((void*)dst, v.data(), v.size() * 8, cudaMemcpyHostToDevice, stream));
            }
        };
        std::vector<double> lw;
        std::vector<int> code;
        if (a.lsq) lsq_weights(hm, hl, lw, code);
        for (StepArgs* m : {&a, &a64}) {
            if (!m->fn) continue;
            const bool f32 = (m == &a) && !fp64;
            if (m == &a64 && a64.fn == a.fn) continue;
            put(m->area, hl.area, f32);
            put(m->fn, hl.fn, f32);
            put(m->fLg, hl.fLg, f32);
            put(m->fd0, hl.fd0, f32);
            put(m->fd1, hl.fd1, f32);
            put(m->ft, hl.ft, f32);
            if (m->lsq && m->lsqw) put(m->lsqw, lw, f32);
        }
        AFX_CUDA(cudaStreamSynchronize(stream));
        host_geometry();  // (captured iteration graphs read the arrays in place)
    }

    // grid sequencing (multigrid.h:99-178): centroids and areas of all cells
    // (ghosts included, reference order), real-cell centroids in device order
    std::vector<double> geo_cx, geo_cy, geo_area, dev_cx, dev_cy;
    DevBuf d_geo, d_devc, d_owner, d_full;

    // implicit solver (solver.h:852-1213), when settings.solver == "implicit"
    ImplicitEngine* imp = nullptr;
    void* imp_b = nullptr;  // FP64 right-hand side
    int imp_lin_iters = 0;
    // the FP64 machine of the implicit path: the solver itself (FP64) or its
    // FP64 residual machine (FP32-mixed: FP32 Jacobian and Krylov vectors)
    StepArgs& A64() { return fp64 ? a : a64; }

    // ||RhoVector|| of parity p (fillRhoRHS, solver.h:1094-1152) into imp_b
    double imp_rhs(int p) {
        StepArgs r = A64();
        r.Rq = imp_b;
        enqueue_rhs_f64(r, p, stream);
        if (r.n_cases > 0) {
            // a batch stops a case whose right-hand side is not finite; the
            // norm below is not used by the batch loop
            r.ctrl = a.ctrl;
            enqueue_case_nonfinite(r, imp_b, stream);
            return 0.0;
        }
        const int nb = (r.n_cells + r.block - 1) / r.block;
        std::vector<double> parts(nb);
        AFX_CUDA(cudaMemcpyAsync(parts.data(), r.partials, nb * 8, cudaMemcpyDeviceToHost, stream));
        AFX_CUDA(cudaStreamSynchronize(stream));
        double t = 0;
        for (double x : parts) t += x;
        return std::sqrt(t);
    }

    // fill + compute + solve(relaxation, tol, rhs_iterations) of
    // implicitSolver (solver.h:1000-1213) at the given CFL; returns the final
    // ||RhoVector||, or -1 if the system could not be solved
    // the mean-flow implicit iteration, then (Spalart-Allmaras) the
    // segregated point-implicit nu~ updates at the new state; the norm
    // returned is then that of the right-hand side with the updated eddy
    // viscosity, so a run converges only once nu~ has stopped moving too
    double implicit_iteration(double cfl, double tol_abs) {
        double r = implicit_iteration_mean(cfl, tol_abs);
        if (a.visc == 2 && r == r && r >= 0) {
            StepArgs m = A64();
            m.cfl = cfl;
            enqueue_sa_implicit_f64(m, parity, 3, stream);
            r = imp_rhs(parity);
        }
        return r;
    }

    double implicit_iteration_mean(double cfl, double tol_abs) {
        StepArgs m = A64();
        m.cfl = cfl;
        if (a.n_cases > 0) m.ctrl = a.ctrl;  // a case stopped during the fill is counted on the run's control block
        if (a.visc == 2) enqueue_sa_mut_f64(m, parity, stream);  // the frozen eddy viscosity of the fill
        implicit_fill(imp, m, parity, stream);
        imp_lin_iters = 0;
        auto solve_update = [&]() {
            const int it = implicit_solve_update(imp, A64(), parity, (const double*)imp_b, st.relaxation, stream);
            if (it < 0) return false;
            imp_lin_iters += it;
            return true;
        };
        const bool batch = a.n_cases > 0;  // per-case control instead of the global early exits
        double err = imp_rhs(parity);
        if (!batch) {
            if (!(err == err)) return err;
            if (err < tol_abs) return err;
        }
        const double err_ini = err;
        if (!solve_update()) return -1;
        for (int i = 0; i < st.rhs_iterations; ++i) {
            err = imp_rhs(parity);
            if (!batch) {
                if (!(err == err)) return err;
                if (err < tol_abs) return err;
                if (err > 10 * err_ini) return err;
            }
            if (!solve_update()) return -1;
        }
        return imp_rhs(parity);
    }

    // Spalart-Allmaras arrays of machine x (device cell order): the FP64
    // nu~ buffers are allocated once (own) and shared; the wall distance,
    // centroids, ghost centroids and mu_t are in x's arithmetic type.
    void sa_setup(StepArgs& x, bool f32, bool own) {
        const size_t N = hl.n_cells, B = hl.n_bnd;
        if (own) {
            for (int p = 0; p < 2; ++p) {
                x.sa_nu[p] = dalloc(N * 8);
                x.sa_nus[p] = dalloc(N * 8);
            }
            x.sa_nuW = dalloc(N * 8);
            double q[4];
            conservative(st, freestream(), q);
            x.sa_nu_far = 3. * st.mu_L / q[0];  // 3 nu_inf
            std::vector<double> nu(N, x.sa_nu_far);
            for (int p = 0; p < 2; ++p)
                AFX_CUDA(cudaMemcpyAsync(x.sa_nu[p], nu.data(), N * 8, cudaMemcpyHostToDevice, stream));
            AFX_CUDA(cudaStreamSynchronize(stream));
        }
        std::vector<double> wd_ref = sa_wall_distance();
        std::vector<double> wd(N), cxy(2 * N), gxy(2 * std::max<size_t>(B, 1));
        for (size_t i = 0; i < N; ++i) {
            wd[i] = wd_ref[hl.cell_old[i]];
            cxy[2 * i] = dev_cx[i];
            cxy[2 * i + 1] = dev_cy[i];
        }
        for (size_t b = 0; b < B; ++b) {  // the ghost of boundary edge b (mesh.h:744-787)
            const uint32_t g = hm.edgesCells[hm.boundaryEdges[b]][1];
            gxy[2 * b] = geo_cx[g];
            gxy[2 * b + 1] = geo_cy[g];
        }
        x.sa_mut = dalloc(N * (f32 ? 4 : 8));
        x.sa_wd = f32 ? dupload(cast_vec<float>(wd)) : dupload(wd);
        x.sa_cxy = f32 ? dupload(cast_vec<float>(cxy)) : dupload(cxy);
        x.sa_gxy = f32 ? dupload(cast_vec<float>(gxy)) : dupload(gxy);
    }

    // Spalart-Allmaras wall distance on the GPU: from each real cell's
    // centroid to the nearest no-slip wall face (a segment), reference order
    std::vector<double> sa_wall_distance() {
        const int nc = (int)hl.n_cells;
        std::vector<double> seg;  // ax, ay, bx, by per no-slip wall face, boundary order
        for (size_t b = 0; b < bedges.size(); ++b)
            if (boundary_type[b] == BC_WALL) {
                const auto& en = hm.edgesNodes[hm.boundaryEdges[b]];
                seg.insert(seg.end(), {hm.nodesX[en[0]], hm.nodesY[en[0]], hm.nodesX[en[1]], hm.nodesY[en[1]]});
            }
        const int nw = (int)(seg.size() / 4);
        std::vector<double> c(2 * (size_t)nc);
        std::copy(geo_cx.begin(), geo_cx.begin() + nc, c.begin());
        std::copy(geo_cy.begin(), geo_cy.begin() + nc, c.begin() + nc);
        DevBuf dc, dw, dout;
        dc.upload(c.data(), c.size() * 8, stream);
        dw.upload(seg.data(), std::max<size_t>(seg.size(), 1) * 8, stream);
        dout.alloc((size_t)nc * 8);
        const double* pc = (const double*)dc.p;
        enqueue_wall_seg_dist(nc, pc, pc + nc, nw, (const double*)dw.p, (double*)dout.p, stream);
        std::vector<double> out((size_t)nc);
        AFX_CUDA(cudaMemcpyAsync(out.data(), dout.p, (size_t)nc * 8, cudaMemcpyDeviceToHost, stream));
        AFX_CUDA(cudaStreamSynchronize(stream));
        return out;
    }

    // after FP64 updates of the master state, the FP32 shadow follows
    void imp_sync() {
        if (!fp64) sync_shadow(parity);
        pending_last = -1;
    }

    // get_boundary_variables, solver.h:597-611
    FarfieldVars freestream() const {
        for (size_t b = 0; b < boundary_type.size(); ++b)
            if (boundary_type[b] == BC_FARFIELD || boundary_type[b] == BC_INLET_OUTLET) return boundary_vars[b];
        return FarfieldVars();
    }

    // set_bcs (solver.h:200-247): per-boundary type and variables
    void set_bcs() {
        const size_t B = bedges.size();
        boundary_type.assign(B, BC_INTERNAL);
        boundary_vars.assign(B, FarfieldVars());
        for (size_t b = 0; b < B; ++b) {
            auto it = st.bcs.find(bedges[b].patch);
            if (it == st.bcs.end())
                throw Error(AFX_ERR_CONFIG, "no boundary condition for patch '" + bedges[b].patch + "'");
            boundary_type[b] = Settings::bc_code(it->second.type);
            if (boundary_type[b] == BC_FARFIELD) boundary_vars[b] = it->second.vars;
        }
    }

    // refill_bcs (solver.h:259-274): ghost states from the boundary variables
    void refill_bcs() {
        const size_t B = boundary_type.size();
        std::vector<double> bq(4 * B);
        for (size_t b = 0; b < B; ++b) conservative(st, boundary_vars[b], &bq[4 * b]);
        std::vector<int> bt(boundary_type.begin(), boundary_type.end());
        AFX_CUDA(cudaMemcpyAsync((void*)a.btype, bt.data(), B * sizeof(int), cudaMemcpyHostToDevice, stream));
        if (fp64) {
            AFX_CUDA(cudaMemcpyAsync((void*)a.bq, bq.data(), bq.size() * 8, cudaMemcpyHostToDevice, stream));
        } else {
            std::vector<float> f(bq.begin(), bq.end());
            AFX_CUDA(cudaMemcpyAsync((void*)a.bq, f.data(), f.size() * 4, cudaMemcpyHostToDevice, stream));
            if (a64.bq)
                AFX_CUDA(cudaMemcpyAsync((void*)a64.bq, bq.data(), bq.size() * 8, cudaMemcpyHostToDevice, stream));
            AFX_CUDA(cudaStreamSynchronize(stream));
        }
        AFX_CUDA(cudaStreamSynchronize(stream));
    }

    void sync_shadow(int p) {
        if (!fp64) enqueue_to_f32(a.n_cells, a.qm[p], a.qsh[p], stream);
    }

    void enqueue_iteration(int p) {
        if (fp64) enqueue_iteration_f64(a, p, stream);
        else enqueue_iteration_f32(a, p, stream);
    }

    // FP32-mixed with an FP64 finish: after the FP32 residual stops falling,
    // the run continues with FP64 iterations on the same FP64 master state.
    bool finish = false;
    StepArgs a64it;              // the FP64 machine set up for iterations (main control block)
    bool shadow_stale = false;   // FP64 iterations ran since the FP32 shadow was formed
    bool last_fp64 = false;      // the last iteration was an FP64 one
    // FP64-finish phase, kept across runs until the state or the boundary
    // conditions are reset (init, set_state, set_farfield)
    bool phase64 = false;
    long long iters_total = 0;
    std::vector<std::pair<long long, double>> fp32_samples;  // (iteration, norm) of the FP32 phase
    void reset_phase() {
        phase64 = false;
        iters_total = 0;
        fp32_samples.clear();
    }
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs64;

    void ensure_shadow() {
        if (shadow_stale) {
            sync_shadow(parity);
            shadow_stale = false;
        }
    }

    cudaGraphExec_t graph(int k, int p, bool g64 = false) {
        auto& cache = g64 ? graphs64 : graphs;
        auto key = std::make_pair(k, p);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
        cudaGraph_t g;
        AFX_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        int q = p;
        for (int i = 0; i < k; ++i) {
            if (g64) enqueue_iteration_f64(a64it, q, stream);
            else enqueue_iteration(q);
            q ^= 1;
        }
        AFX_CUDA(cudaStreamEndCapture(stream, &g));
        cudaGraphExec_t ex;
        AFX_CUDA(cudaGraphInstantiate(&ex, g, 0));
        cudaGraphDestroy(g);
        cache[key] = ex;
        return ex;
    }

    int chunk() const {
        if (a.n_cells >= 1000000) return 2;
        if (a.n_cells >= 100000) return 8;
        return 32;
    }

    void set_ctrl(int run_mode, int max_it, double tol) {
        std::memset(h_ctrl, 0, sizeof(Ctrl));
        h_ctrl->run_mode = run_mode;
        h_ctrl->max_it = max_it;
        h_ctrl->tol = tol;
        AFX_CUDA(cudaMemcpyAsync(a.ctrl, h_ctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, stream));
        if (a.n_cases > 0) {  // every case of a batch starts the run afresh
            AFX_CUDA(cudaMemsetAsync(a.cctrl, 0, a.n_cases * sizeof(CaseCtrl), stream));
            AFX_CUDA(cudaMemsetAsync(a.case_done, 0, a.n_cases * sizeof(int), stream));
        }
    }

    void read_ctrl() {
        AFX_CUDA(cudaMemcpyAsync(h_ctrl, a.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, stream));
        AFX_CUDA(cudaStreamSynchronize(stream));
    }

    void materialize_qW() {
        if (pending_last < 0) return;
        set_ctrl(0, 0, 0);  // the kernels skip their work while ctrl->done is set
        if (fp64) enqueue_last_stage_residual_f64(a, pending_last, stream);
        else if (last_fp64) enqueue_last_stage_residual_f64(a64it, pending_last, stream);
        else enqueue_last_stage_residual_f32(a, pending_last, stream);
        pending_last = -1;
    }

    // Runs n iterations (run_mode 0) or the run_solver loop (run_mode 1).
    // Returns the number of iterations executed.  With the FP64 finish
    // (run_mode 1 only), the FP32 phase ends when the residual norm has not
    // halved over the last 3000 iterations; FP64 iterations follow.
    int run(int n, int run_mode, double tol) {
        const int p0 = parity;
        ensure_shadow();
        AFX_CUDA(cudaEventRecord(ev0, stream));
        const int K = chunk();
        int launched = 0;
        bool stopped = false;
        last_fp64 = phase64;
        auto& samples = fp32_samples;
        int since = corr_interval;  // refresh the defect correction before the first chunk
        while (launched < n) {
            if (!phase64 && corr_interval > 0 && since >= corr_interval) {
                refresh_correction((p0 + launched) & 1);
                since = 0;
            }
            const int k = (n - launched >= K) ? K : 1;
            AFX_CUDA(cudaGraphLaunch(graph(k, (p0 + launched) & 1, phase64), stream));
            launched += k;
            since += k;
            if (run_mode == 1 || launched >= n || stop.load()) {
                read_ctrl();
                if (h_ctrl->done) break;
                if (stop.load()) {
                    stopped = true;
                    break;
                }
                const long long now = iters_total + launched;
                if (finish && !phase64 && run_mode == 1 && (samples.empty() || now - samples.back().first >= 1000)) {
                    samples.emplace_back(now, h_ctrl->last_norm);
                    for (const auto& sm : samples)
                        if (now - sm.first >= 3000 && now - sm.first < 4000 && h_ctrl->last_norm > 0.5 * sm.second) {
                            phase64 = true;  // FP32 floor reached
                            shadow_stale = true;
                            last_fp64 = true;
                            break;
                        }
                }
            }
        }
        AFX_CUDA(cudaEventRecord(ev1, stream));
        read_ctrl();
        float ms = 0;
        AFX_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        last_sec = ms * 1e-3;
        const int done = h_ctrl->iter;
        iters_total += done;
        if (phase64 && done > 0) shadow_stale = true;
        parity = p0 ^ (done & 1);
        // a batch keeps each case's last-stage qW in Rq as it goes
        if (done > 0 && a.n_cases == 0) pending_last = parity ^ 1;
        (void)tol;
        if (stopped) stop.store(0);
        return stopped ? -done - 1 : done;
    }
};

extern "C" {

const char* afx_last_error(void) { return g_err.c_str(); }
const char* afx_version(void) { return "afx-gb300 0.1 (sm_103a)"; }

// ------------------------------------------------------------------ mesh
int afx_mesh_load(const char* path, afx_mesh* out) {
    return guarded([&] {
        if (!path || !out) throw Error(AFX_ERR_ARG, "null argument");
        auto* m = new afx_mesh_s();
        try {
            m->m = load_gmsh(path);
        } catch (...) {
            delete m;
            throw;
        }
        *out = m;
    });
}

int afx_mesh_from_arrays(int n_nodes, const double* x, const double* y, int n_cells, const int* cell_nodes,
                         int n_bedges, const int* bedge_nodes, const int* bedge_patch, const char* patch_names,
                         afx_mesh* out) {
    return guarded([&] {
        if (!x || !y || !cell_nodes || !out || n_nodes <= 0 || n_cells <= 0 || n_bedges < 0)
            throw Error(AFX_ERR_ARG, "bad mesh arrays");
        std::vector<std::string> names;
        {
            std::string all(patch_names ? patch_names : "");
            size_t pos = 0;
            while (pos <= all.size()) {
                size_t nl = all.find('\n', pos);
                if (nl == std::string::npos) nl = all.size();
                if (nl > pos) names.push_back(all.substr(pos, nl - pos));
                pos = nl + 1;
            }
        }
        auto m = std::make_unique<afx_mesh_s>();
        HostMesh& h = m->m;
        h.nodesX.assign(x, x + n_nodes);
        h.nodesY.assign(y, y + n_nodes);
        h.cellsNodes.resize(n_cells);
        h.cellsIsTriangle.resize(n_cells);
        for (int c = 0; c < n_cells; ++c) {
            const int* cn = cell_nodes + 4 * (size_t)c;
            const bool tri = cn[3] < 0;
            for (int j = 0; j < (tri ? 3 : 4); ++j)
                if (cn[j] < 0 || cn[j] >= n_nodes) throw Error(AFX_ERR_MESH, "cell node index out of range");
            h.cellsNodes[c] = {(uint32_t)cn[0], (uint32_t)cn[1], (uint32_t)cn[2], tri ? 0u : (uint32_t)cn[3]};
            h.cellsIsTriangle[c] = tri;
        }
        for (int b = 0; b < n_bedges; ++b) {
            const int p = bedge_patch[b];
            if (p < 0 || p >= (int)names.size()) throw Error(AFX_ERR_MESH, "boundary patch index out of range");
            if (bedge_nodes[2 * b] < 0 || bedge_nodes[2 * b] >= n_nodes || bedge_nodes[2 * b + 1] < 0 ||
                bedge_nodes[2 * b + 1] >= n_nodes)
                throw Error(AFX_ERR_MESH, "boundary node index out of range");
            h.bnd0.push_back((uint32_t)bedge_nodes[2 * b]);
            h.bnd1.push_back((uint32_t)bedge_nodes[2 * b + 1]);
            h.bndName.push_back(names[p]);
        }
        h.finalize();
        *out = m.release();
    });
}

int afx_mesh_counts(afx_mesh m, long long counts[5]) {
    return guarded([&] {
        if (!m || !counts) throw Error(AFX_ERR_ARG, "null argument");
        counts[0] = m->m.nRealCells;
        counts[1] = (long long)m->m.cellsAreas.size();
        counts[2] = (long long)m->m.edgesCells.size();
        counts[3] = (long long)m->m.boundaryEdges.size();
        counts[4] = (long long)m->m.nodesX.size();
    });
}

int afx_mesh_get(afx_mesh mp, const char* what, double* out, long long cap, long long* n) {
    return guarded([&] {
        if (!mp || !what) throw Error(AFX_ERR_ARG, "null argument");
        HostMesh& m = mp->m;
        std::string w(what);
        const std::vector<double>* v = nullptr;
        if (w == "cx") v = &m.cellsCentersX;
        else if (w == "cy") v = &m.cellsCentersY;
        else if (w == "area") v = &m.cellsAreas;
        else if (w == "ex") v = &m.edgesCentersX;
        else if (w == "ey") v = &m.edgesCentersY;
        else if (w == "nx") v = &m.edgesNormalsX;
        else if (w == "ny") v = &m.edgesNormalsY;
        else if (w == "L") v = &m.edgesLengths;
        else if (w == "wall_dist") v = &m.wall_dist;
        else if (w == "node_x") v = &m.nodesX;
        else if (w == "node_y") v = &m.nodesY;
        if (!v) throw Error(AFX_ERR_ARG, "unknown mesh array '" + w + "'");
        if (n) *n = (long long)v->size();
        if (out) std::memcpy(out, v->data(), std::min<long long>(cap, (long long)v->size()) * sizeof(double));
    });
}

int afx_mesh_get_int(afx_mesh mp, const char* what, long long* out, long long cap, long long* n) {
    return guarded([&] {
        if (!mp || !what) throw Error(AFX_ERR_ARG, "null argument");
        HostMesh& m = mp->m;
        std::string w(what);
        std::vector<long long> v;
        if (w == "edges_cells") {
            for (auto& e : m.edgesCells) { v.push_back(e[0]); v.push_back(e[1]); }
        } else if (w == "edges_nodes") {
            for (auto& e : m.edgesNodes) { v.push_back(e[0]); v.push_back(e[1]); }
        } else if (w == "boundary_edges") {
            for (auto e : m.boundaryEdges) v.push_back(e);
        } else if (w == "cell_order") {
            for (auto c : mp->layout().cell_old) v.push_back(c);
        } else {
            throw Error(AFX_ERR_ARG, "unknown mesh array '" + w + "'");
        }
        if (n) *n = (long long)v.size();
        if (out) std::memcpy(out, v.data(), std::min<long long>(cap, (long long)v.size()) * sizeof(long long));
    });
}

int afx_mesh_boundary_name(afx_mesh mp, int b, char* out, int cap) {
    return guarded([&] {
        if (!mp || !out || cap <= 0) throw Error(AFX_ERR_ARG, "null argument");
        const std::string& s = mp->m.boundaryEdgesPhysicals.at(b);
        std::snprintf(out, cap, "%s", s.c_str());
    });
}

int afx_mesh_set_nodes(afx_mesh mp, const double* x, const double* y, long long n) {
    return guarded([&] {
        if (!mp || !x || !y) throw Error(AFX_ERR_ARG, "null argument");
        if (n != (long long)mp->m.nodesX.size()) throw Error(AFX_ERR_ARG, "node count mismatch");
        mp->m.update_nodes(x, y);
        if (mp->has_layout) fill_layout_geometry(mp->m, mp->L);
    });
}

void afx_mesh_free(afx_mesh m) { delete m; }

// ---------------------------------------------------------------- config
int afx_config_create(afx_config* out) {
    return guarded([&] {
        if (!out) throw Error(AFX_ERR_ARG, "null argument");
        *out = new afx_config_s();
    });
}

int afx_config_from_ini_string(const char* text, afx_config* out) {
    return guarded([&] {
        if (!text || !out) throw Error(AFX_ERR_ARG, "null argument");
        auto c = std::make_unique<afx_config_s>();
        import_ini(c->s, text);
        *out = c.release();
    });
}

int afx_config_from_ini(const char* path, afx_config* out) {
    return guarded([&] {
        if (!path || !out) throw Error(AFX_ERR_ARG, "null argument");
        std::ifstream f(path);
        if (!f) throw Error(AFX_ERR_IO, std::string("Config file: ") + path + " not found");
        std::stringstream ss;
        ss << f.rdbuf();
        auto c = std::make_unique<afx_config_s>();
        import_ini(c->s, ss.str());
        *out = c.release();
    });
}

static double* dfield(Settings& s, const std::string& k) {
    if (k == "gamma") return &s.gamma;
    if (k == "R") return &s.R;
    if (k == "mu_L") return &s.mu_L;
    if (k == "Pr_L") return &s.Pr_L;
    if (k == "Pr_T") return &s.Pr_T;
    if (k == "start_cfl") return &s.start_cfl;
    if (k == "slope_cfl") return &s.slope_cfl;
    if (k == "max_cfl") return &s.max_cfl;
    if (k == "relaxation") return &s.relaxation;
    if (k == "tolerance") return &s.tolerance;
    if (k == "limiter_k") return &s.limiter_k;
    if (k == "alpha_start") return &s.alpha_start;
    if (k == "alpha_end") return &s.alpha_end;
    if (k == "alpha_step") return &s.alpha_step;
    return nullptr;
}

int afx_config_set_double(afx_config c, const char* key, double v) {
    return guarded([&] {
        if (!c || !key) throw Error(AFX_ERR_ARG, "null argument");
        std::string k(key);
        if (k == "rhs_iterations") c->s.rhs_iterations = (int)v;
        else if (k == "max_iterations") c->s.max_iterations = (int)v;
        else if (k == "block_size") {
            const int b = (int)v;
            if (b != 0 && b != 32 && b != 64 && b != 128 && b != 256)
                throw Error(AFX_ERR_CONFIG, "block_size must be 0 (auto), 32, 64, 128 or 256");
            c->s.block_size = b;
        } else if (k == "fp64_correction_interval") {
            if (v < 0) throw Error(AFX_ERR_CONFIG, "fp64_correction_interval must be >= 0");
            c->s.fp64_correction_interval = (int)v;
        } else if (k == "fp64_finish") {
            c->s.fp64_finish = v != 0;
        } else if (k == "krylov_graph") {
            c->s.krylov_graph = v != 0;
        } else if (k == "krylov_preconditioner") {
            if (v != 0 && v != 1) throw Error(AFX_ERR_CONFIG, "krylov_preconditioner must be 0 or 1");
            c->s.krylov_preconditioner = (int)v;
        } else if (k == "adjoint_directions") {
            if (v != 1 && v != 2 && v != 4) throw Error(AFX_ERR_CONFIG, "adjoint_directions must be 1, 2 or 4");
            c->s.adjoint_directions = (int)v;
        }
        else if (k == "second_order") c->s.second_order = v != 0;
        else if (double* p = dfield(c->s, k)) *p = v;
        else throw Error(AFX_ERR_ARG, "unknown numeric setting '" + k + "'");
    });
}

int afx_config_get_double(afx_config c, const char* key, double* v) {
    return guarded([&] {
        if (!c || !key || !v) throw Error(AFX_ERR_ARG, "null argument");
        std::string k(key);
        if (k == "rhs_iterations") *v = c->s.rhs_iterations;
        else if (k == "max_iterations") *v = c->s.max_iterations;
        else if (k == "block_size") *v = c->s.block_size;
        else if (k == "fp64_correction_interval") *v = c->s.fp64_correction_interval;
        else if (k == "fp64_finish") *v = c->s.fp64_finish ? 1 : 0;
        else if (k == "krylov_graph") *v = c->s.krylov_graph ? 1 : 0;
        else if (k == "krylov_preconditioner") *v = c->s.krylov_preconditioner;
        else if (k == "adjoint_directions") *v = c->s.adjoint_directions;
        else if (k == "second_order") *v = c->s.second_order ? 1 : 0;
        else if (double* p = dfield(c->s, k)) *v = *p;
        else throw Error(AFX_ERR_ARG, "unknown numeric setting '" + k + "'");
    });
}

int afx_config_set_string(afx_config c, const char* key, const char* v) {
    return guarded([&] {
        if (!c || !key || !v) throw Error(AFX_ERR_ARG, "null argument");
        std::string k(key), s(v);
        auto check = [&](std::initializer_list<const char*> ok) {
            for (auto o : ok)
                if (s == o) return;
            throw Error(AFX_ERR_CONFIG, "invalid value '" + s + "' for " + k);
        };
        if (k == "solver") { check({"explicit", "implicit"}); c->s.solver = s; }
        else if (k == "gradient") { check({"green-gauss", "least-squares"}); c->s.gradient = s; }
        else if (k == "viscosity") {
            check({"inviscid", "laminar", "spalart-allmaras", "spallart-allmaras"});
            c->s.viscosity = s;
        } else if (k == "limiter") { check({"venkatakrishnan", "michalak"}); c->s.limiter = s; }
        else if (k == "precision") { check({"fp64", "fp32-mixed"}); c->s.precision = s; }
        else if (k == "kernel_variant") { check({"auto", "gather", "face", "tile"}); c->s.kernel_variant = s; }
        else if (k == "airfoil_name") c->s.airfoil_name = s;
        else throw Error(AFX_ERR_ARG, "unknown string setting '" + k + "'");
    });
}

int afx_config_get_string(afx_config c, const char* key, char* out, int cap) {
    return guarded([&] {
        if (!c || !key || !out || cap <= 0) throw Error(AFX_ERR_ARG, "null argument");
        std::string k(key), v;
        if (k == "solver") v = c->s.solver;
        else if (k == "gradient") v = c->s.gradient;
        else if (k == "viscosity") v = c->s.viscosity;
        else if (k == "limiter") v = c->s.limiter;
        else if (k == "precision") v = c->s.precision;
        else if (k == "kernel_variant") v = c->s.kernel_variant;
        else if (k == "airfoil_name") v = c->s.airfoil_name;
        else throw Error(AFX_ERR_ARG, "unknown string setting '" + k + "'");
        std::snprintf(out, cap, "%s", v.c_str());
    });
}

int afx_config_set_bc(afx_config c, const char* name, const char* type, double T, double mach, double angle,
                      double p) {
    return guarded([&] {
        if (!c || !name || !type) throw Error(AFX_ERR_ARG, "null argument");
        if (!c->s.bcs.count(name)) c->s.bc_order.push_back(name);
        auto& bc = c->s.bcs[name];
        bc.type = type;
        bc.vars = FarfieldVars();
        if (bc.type == "farfield") bc.vars = FarfieldVars{mach, angle, T, p};
    });
}

int afx_config_bc_count(afx_config c, int* n) {
    return guarded([&] {
        if (!c || !n) throw Error(AFX_ERR_ARG, "null argument");
        *n = (int)c->s.bcs.size();
    });
}

int afx_config_get_bc(afx_config c, const char* name, char* type, int cap, double* T, double* mach, double* angle,
                      double* p) {
    return guarded([&] {
        if (!c || !name) throw Error(AFX_ERR_ARG, "null argument");
        auto it = c->s.bcs.find(name);
        if (it == c->s.bcs.end()) throw Error(AFX_ERR_ARG, std::string("no boundary condition '") + name + "'");
        if (type && cap > 0) std::snprintf(type, cap, "%s", it->second.type.c_str());
        if (T) *T = it->second.vars.T;
        if (mach) *mach = it->second.vars.mach;
        if (angle) *angle = it->second.vars.angle;
        if (p) *p = it->second.vars.p;
    });
}

void afx_config_free(afx_config c) { delete c; }

// ---------------------------------------------------------------- solver
}  // extern "C"

// Least-squares gradient weights (solver.h:402-422) per real cell, over its
// local edges in their own order: M = (d^T d)^-1 (closed form), weights M d_j,
// and the cslot slot of each local edge.
static void lsq_weights(const HostMesh& m, const DeviceLayout& L, std::vector<double>& lsqw64,
                        std::vector<int>& code) {
    const size_t N = L.n_cells;
    std::vector<int> face_of_edge(L.n_faces);
    for (int f = 0; f < L.n_faces; ++f) face_of_edge[L.face_edge[f]] = f;
    lsqw64.assign(8 * N, 0.0);
    code.assign(N, 0);
    for (size_t i = 0; i < N; ++i) {
        const uint32_t c = (uint32_t)L.cell_old[i];
        const uint32_t nj = m.cellsIsTriangle[c] ? 3 : 4;
        double dx[4], dy[4], a00 = 0, a01 = 0, a11 = 0;
        int cd = (int)nj << 8;
        for (uint32_t j = 0; j < nj; ++j) {
            const uint32_t e = m.cellsEdges[c][j];
            const uint32_t cn = m.edgesCells[e][0] == c ? m.edgesCells[e][1] : m.edgesCells[e][0];
            dx[j] = m.cellsCentersX[cn] - m.cellsCentersX[c];
            dy[j] = m.cellsCentersY[cn] - m.cellsCentersY[c];
            a00 += dx[j] * dx[j];
            a01 += dx[j] * dy[j];
            a11 += dy[j] * dy[j];
            int slot = -1;
            for (int sl = 0; sl < 4; ++sl) {
                const int v = L.cslot[4 * i + sl];
                if (v != 0 && (v > 0 ? v : -v) - 1 == face_of_edge[e]) slot = sl;
            }
            if (slot < 0) throw Error(AFX_ERR_MESH, "least squares: cell edge not among its faces");
            cd |= slot << (2 * j);
        }
        const double invdet = 1.0 / (a00 * a11 - a01 * a01);
        const double M0 = a11 * invdet, M1 = -a01 * invdet, M2 = -a01 * invdet, M3 = a00 * invdet;
        for (uint32_t j = 0; j < nj; ++j) {
            lsqw64[8 * i + 2 * j] = M0 * dx[j] + M1 * dy[j];
            lsqw64[8 * i + 2 * j + 1] = M2 * dx[j] + M3 * dy[j];
        }
        code[i] = cd;
    }
}

// The device solver of one mesh (a single case, or the union of a batch's
// cases) with settings `st`.
static std::unique_ptr<afx_solver_s> make_solver(const HostMesh& m, const DeviceLayout& L, const Settings& st0) {
    {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
            throw Error(AFX_ERR_CUDA, "no CUDA device available");
        auto s = std::make_unique<afx_solver_s>();
        s->st = st0;
        s->hm = m;
        s->hl = L;
        s->host_geometry();
        s->cell_old = L.cell_old;
        s->h_fcell = L.fcell;
        s->h_cslot = L.cslot;
        s->fp64 = s->st.precision != "fp32-mixed";
        AFX_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        AFX_CUDA(cudaEventCreate(&s->ev0));
        AFX_CUDA(cudaEventCreate(&s->ev1));
        AFX_CUDA(cudaHostAlloc((void**)&s->h_ctrl, sizeof(Ctrl), cudaHostAllocDefault));
        s->set_bcs();
        StepArgs& a = s->a;
        a.n_cells = L.n_cells;
        a.n_faces = L.n_faces;
        a.n_bnd = L.n_bnd;
        const size_t N = L.n_cells, F = L.n_faces, B = L.n_bnd;
        a.cslot = s->dupload(L.cslot);
        a.cnbr = s->dupload(L.cnbr);
        a.fcell = s->dupload(L.fcell);
        if (s->fp64) {
            a.area = s->dupload(L.area);
            a.fn = s->dupload(L.fn);
            a.fLg = s->dupload(L.fLg);
            a.fd0 = s->dupload(L.fd0);
            a.fd1 = s->dupload(L.fd1);
            a.ft = s->dupload(L.ft);
        } else {
            a.area = s->dupload(cast_vec<float>(L.area));
            a.fn = s->dupload(cast_vec<float>(L.fn));
            a.fLg = s->dupload(cast_vec<float>(L.fLg));
            a.fd0 = s->dupload(cast_vec<float>(L.fd0));
            a.fd1 = s->dupload(cast_vec<float>(L.fd1));
            a.ft = s->dupload(cast_vec<float>(L.ft));
        }
        const size_t w = s->fp64 ? 8 : 4;
        a.btype = s->dalloc(std::max<size_t>(B, 1) * sizeof(int));
        a.bq = s->dalloc(std::max<size_t>(B, 1) * 4 * w);
        const Settings& st = s->st;
        a.gamma = st.gamma;
        a.R = st.R;
        a.mu = st.mu_L;
        a.kheat = 1. * st.mu_L / st.Pr_L;  // gas::k(), core.h:43-45
        a.limiter_k = st.limiter_k;
        a.cfl = st.start_cfl;
        a.relax = st.relaxation;
        const int vc = st.viscosity_code();
        a.visc = vc == VISC_LAMINAR ? 1 : (vc == VISC_SA ? 2 : 0);
        a.cp = st.cp;
        a.Pr_L = st.Pr_L;
        a.Pr_T = st.Pr_T;
        if (a.visc == 2 && (st.fp64_correction_interval > 0 || st.fp64_finish))
            throw Error(AFX_ERR_CONFIG, "spalart-allmaras: fp64_correction_interval and fp64_finish are not available");
        a.second = st.second_order ? 1 : 0;
        a.need_grad = (st.second_order || vc != VISC_INVISCID) ? 1 : 0;
        a.limiter = st.limiter == "michalak" ? 1 : 0;
        std::vector<double> lsqw64;
        if (st.gradient == "least-squares") {
            std::vector<int> code;
            lsq_weights(m, L, lsqw64, code);
            a.lsq = 1;
            a.lsqw = s->fp64 ? s->dupload(lsqw64) : s->dupload(cast_vec<float>(lsqw64));
            a.lsqs = (const int*)s->dupload(code);
        }
        // defaults from measurement on GB300: the FP64 path is FP64-pipe bound,
        // so each face flux is formed once; FP32-mixed re-forms fluxes in the
        // gather.  afx_autotune() times both on the actual mesh.
        const int variant = st.kernel_variant == "face" ? 1
                            : st.kernel_variant == "gather" ? 0
                            : st.kernel_variant == "tile" ? 2
                                                          : (s->fp64 ? 1 : 2);
        const int block = st.block_size ? st.block_size : (N >= 600 * 256 ? 256 : (N >= 300 * 128 ? 128 : 64));
        for (int p = 0; p < 2; ++p) {
            a.qm[p] = s->dalloc(N * 32);
            a.qsh[p] = s->fp64 ? a.qm[p] : s->dalloc(N * 16);
            a.qs[p] = s->dalloc(N * 4 * w);
        }
        a.gx = s->dalloc(N * 4 * w);
        a.gy = s->dalloc(N * 4 * w);
        a.phi = s->dalloc(N * 4 * w);
        a.dt = s->dalloc(N * w);
        a.Rq = s->dalloc(N * 32);
        // face buffers always exist so the autotuner may switch variants
        a.fflux = s->dalloc(F * 4 * w);
        a.feL = s->dalloc(F * w);
        a.n_partials = (int)((N + 31) / 32);  // enough for the smallest block size
        a.partials = (double*)s->dalloc(a.n_partials * sizeof(double));
        a.ctrl = (Ctrl*)s->dalloc(sizeof(Ctrl));
        a.hist = (double*)s->dalloc(HIST_CAP * sizeof(double));
        s->d_cell_old.upload(L.cell_old.data(), N * sizeof(int), s->stream);
        // Spalart-Allmaras has the face and tile variants (the gather variant
        // would re-form the eddy-viscous face terms on both sides)
        s->set_launch(a.visc == 2 && variant == 0 ? 1 : variant, block);
        if (a.visc == 2) s->sa_setup(a, !s->fp64, true);
        const bool implicit = st.solver == "implicit";
        if (!s->fp64 && (st.fp64_correction_interval > 0 || st.fp64_finish || implicit)) {
            // FP64 residual machine on the same FP64 master state
            s->corr_interval = st.fp64_correction_interval;
            StepArgs& b = s->a64;
            b = a;
            b.area = s->dupload(L.area);
            b.fn = s->dupload(L.fn);
            b.fLg = s->dupload(L.fLg);
            b.fd0 = s->dupload(L.fd0);
            b.fd1 = s->dupload(L.fd1);
            b.ft = s->dupload(L.ft);
            if (a.lsq) b.lsqw = s->dupload(lsqw64);
            b.bq = s->dalloc(std::max<size_t>(B, 1) * 32);
            for (int p = 0; p < 2; ++p) b.qsh[p] = b.qm[p];
            b.qs[0] = b.qs[1] = nullptr;  // residual launches read no stage state
            b.gx = s->dalloc(N * 32);
            b.gy = s->dalloc(N * 32);
            b.phi = s->dalloc(N * 32);
            b.dt = s->dalloc(N * 8);
            b.Rq = s->dalloc(N * 32);
            b.variant = 0;  // gather: no FP64 face buffers needed
            b.fflux = b.feL = nullptr;
            if (implicit) {
                // the implicit right-hand side is formed every chord step:
                // the face-flux variant (one FP64 flux per face)
                b.variant = 1;
                b.fflux = s->dalloc(F * 32);
                b.feL = s->dalloc(F * 8);
            }
            b.corr = nullptr;
            if (a.visc == 2) s->sa_setup(b, false, false);  // FP64 copies of the typed SA arrays
            b.ctrl = (Ctrl*)s->dalloc(sizeof(Ctrl));  // zeroed, never set to done
            s->R32buf = s->dalloc(N * 32);
            if (s->corr_interval > 0) a.corr = s->dalloc(N * 16);
            if (st.fp64_finish) {
                // the same machine, set up to iterate: FP64 stage states, the
                // face-flux variant (FP64-pipe bound: one flux per face), the
                // run's own control block, partial sums and history
                s->finish = true;
                StepArgs& c = s->a64it;
                c = b;
                c.qs[0] = s->dalloc(N * 32);
                c.qs[1] = s->dalloc(N * 32);
                c.variant = 1;
                c.fflux = s->dalloc(F * 32);
                c.feL = s->dalloc(F * 8);
                c.Rq = a.Rq;
                c.ctrl = a.ctrl;
                c.partials = a.partials;
                c.hist = a.hist;
                c.norms = a.norms;
                c.block = N >= 600 * 256 ? 256 : (N >= 300 * 128 ? 128 : 64);
            }
        }
        if (implicit) {
            // greedy colouring of the cell graph in device order (no two
            // face neighbours share a colour): the Gauss-Seidel preconditioner
            // updates one colour at a time
            std::vector<int> color(N, -1);
            for (size_t i = 0; i < N; ++i) {
                unsigned used = 0;
                for (int k = 0; k < 4; ++k) {
                    const int o = L.cnbr[4 * i + k];
                    if (L.cslot[4 * i + k] != 0 && o >= 0 && color[o] >= 0 && color[o] < 32) used |= 1u << color[o];
                }
                int c = 0;
                while (used & (1u << c)) ++c;
                color[i] = c;
            }
            s->imp_b = s->dalloc(N * 32);
            s->imp = implicit_create(s->A64(), !s->fp64, st.krylov_graph, color, L.cslot.data(), L.cnbr.data(),
                                     s->stream);
        }
        s->d_stage.alloc(N * 32);
        AFX_CUDA(cudaHostAlloc((void**)&s->h_stage, N * 32, cudaHostAllocDefault));
        s->h_stage_bytes = N * 32;
        s->refill_bcs();
        AFX_CUDA(cudaStreamSynchronize(s->stream));
        return s;
    }
}

extern "C" {

int afx_solver_create(afx_mesh mp, afx_config cp, afx_solver* out) {
    return guarded([&] {
        if (!mp || !cp || !out) throw Error(AFX_ERR_ARG, "null argument");
        *out = make_solver(mp->m, mp->layout(), cp->s).release();
    });
}

void afx_solver_free(afx_solver s) { delete s; }

int afx_init_freestream(afx_solver s) {
    return guarded([&] {
        if (!s) throw Error(AFX_ERR_ARG, "null argument");
        double q[4];
        conservative(s->st, s->freestream(), q);  // init(), solver.h:615-631
        const size_t N = s->a.n_cells;
        for (size_t i = 0; i < N; ++i) std::memcpy(s->h_stage + 4 * i, q, 32);
        AFX_CUDA(cudaMemcpyAsync(s->a.qm[s->parity], s->h_stage, N * 32, cudaMemcpyHostToDevice, s->stream));
        if (s->a.visc == 2) {  // nu~ = 3 nu_inf everywhere
            AFX_CUDA(cudaStreamSynchronize(s->stream));
            for (size_t i = 0; i < N; ++i) s->h_stage[i] = s->a.sa_nu_far;
            AFX_CUDA(cudaMemcpyAsync(s->a.sa_nu[s->parity], s->h_stage, N * 8, cudaMemcpyHostToDevice, s->stream));
        }
        s->sync_shadow(s->parity);
        s->shadow_stale = false;
        s->reset_phase();
        s->refill_bcs();
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    });
}

// The reference's nu array (solver.h:55), unused there: nu~ of the
// Spalart-Allmaras model per real cell, reference order.
int afx_set_turbulence(afx_solver s, const double* nu, long long n) {
    return guarded([&] {
        if (!s || !nu) throw Error(AFX_ERR_ARG, "null argument");
        if (s->a.visc != 2) throw Error(AFX_ERR_CONFIG, "not a spalart-allmaras solver");
        const size_t N = s->a.n_cells;
        if (n != (long long)N) throw Error(AFX_ERR_ARG, "size must be n_real_cells");
        AFX_CUDA(cudaMemcpyAsync(s->d_stage.p, nu, N * 8, cudaMemcpyDefault, s->stream));
        enqueue_permute_in1((int)N, (const int*)s->d_cell_old.p, s->d_stage.p, s->a.sa_nu[s->parity], s->stream);
        s->reset_phase();
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    });
}

int afx_get_turbulence(afx_solver s, double* nu, long long n) {
    return guarded([&] {
        if (!s || !nu) throw Error(AFX_ERR_ARG, "null argument");
        if (s->a.visc != 2) throw Error(AFX_ERR_CONFIG, "not a spalart-allmaras solver");
        const size_t N = s->a.n_cells;
        if (n != (long long)N) throw Error(AFX_ERR_ARG, "size must be n_real_cells");
        enqueue_permute_out1((int)N, (const int*)s->d_cell_old.p, s->a.sa_nu[s->parity], s->d_stage.p, s->stream);
        AFX_CUDA(cudaMemcpyAsync(nu, s->d_stage.p, N * 8, cudaMemcpyDefault, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    });
}

// nu~ residual R/A of the last evaluation (afx_residual: the current state;
// an iteration: its last stage), reference order.
int afx_turbulence_residual(afx_solver s, double* nuW, long long n) {
    return guarded([&] {
        if (!s || !nuW) throw Error(AFX_ERR_ARG, "null argument");
        if (s->a.visc != 2) throw Error(AFX_ERR_CONFIG, "not a spalart-allmaras solver");
        const size_t N = s->a.n_cells;
        if (n != (long long)N) throw Error(AFX_ERR_ARG, "size must be n_real_cells");
        enqueue_permute_out1((int)N, (const int*)s->d_cell_old.p, s->a.sa_nuW, s->d_stage.p, s->stream);
        AFX_CUDA(cudaMemcpyAsync(nuW, s->d_stage.p, N * 8, cudaMemcpyDefault, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    });
}

int afx_set_state(afx_solver s, const double* q, long long n) {
    return guarded([&] {
        if (!s || !q) throw Error(AFX_ERR_ARG, "null argument");
        const size_t N = s->a.n_cells;
        if (n != (long long)(4 * N)) throw Error(AFX_ERR_ARG, "state size must be 4*n_real_cells");
        AFX_CUDA(cudaMemcpyAsync(s->d_stage.p, q, N * 32, cudaMemcpyDefault, s->stream));
        enqueue_permute_in((int)N, (const int*)s->d_cell_old.p, s->d_stage.p, s->a.qm[s->parity], s->stream);
        s->sync_shadow(s->parity);
        s->shadow_stale = false;
        s->reset_phase();
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    });
}

int afx_get_state(afx_solver s, double* q, long long n) {
    return guarded([&] {
        if (!s || !q) throw Error(AFX_ERR_ARG, "null argument");
        const size_t N = s->a.n_cells;
        if (n != (long long)(4 * N)) throw Error(AFX_ERR_ARG, "state size must be 4*n_real_cells");
        enqueue_permute_out((int)N, (const int*)s->d_cell_old.p, s->a.qm[s->parity], s->d_stage.p, s->stream);
        AFX_CUDA(cudaMemcpyAsync(q, s->d_stage.p, N * 32, cudaMemcpyDefault, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    });
}

int afx_residual(afx_solver s, double* R, long long n) {
    return guarded([&] {
        if (!s) throw Error(AFX_ERR_ARG, "null argument");
        const size_t N = s->a.n_cells;
        if (R && n != (long long)(4 * N)) throw Error(AFX_ERR_ARG, "residual size must be 4*n_real_cells");
        s->ensure_shadow();
        s->set_ctrl(0, 0, 0);
        if (s->fp64) enqueue_residual_f64(s->a, s->parity, s->stream);
        else enqueue_residual_f32(s->a, s->parity, s->stream);
        s->pending_last = -1;
        if (R) {
            enqueue_permute_out((int)N, (const int*)s->d_cell_old.p, s->a.Rq, s->d_stage.p, s->stream);
            AFX_CUDA(cudaMemcpyAsync(R, s->d_stage.p, N * 32, cudaMemcpyDefault, s->stream));
        }
        AFX_CUDA(cudaStreamSynchronize(s->stream));
        AFX_CUDA(cudaGetLastError());
    });
}

// fillRhoRHS (solver.h:1079-1152) of the current state, for an implicit
// solver: the face sums of the second-order residual, not divided by the
// area, ghost rows zero.  rhs gets the real-cell rows (AoS FP64, reference
// cell order).
int afx_implicit_rhs(afx_solver s, double* rhs, long long n) {
    return guarded([&] {
        if (!s || !rhs) throw Error(AFX_ERR_ARG, "null argument");
        if (!s->imp) throw Error(AFX_ERR_CONFIG, "afx_implicit_rhs needs an implicit solver");
        const size_t N = s->a.n_cells;
        if (n != (long long)(4 * N)) throw Error(AFX_ERR_ARG, "size must be 4*n_real_cells");
        s->ensure_shadow();
        s->materialize_qW();
        s->set_ctrl(0, 0, 0);
        s->imp_rhs(s->parity);
        enqueue_permute_out((int)N, (const int*)s->d_cell_old.p, s->imp_b, s->d_stage.p, s->stream);
        AFX_CUDA(cudaMemcpyAsync(rhs, s->d_stage.p, N * 32, cudaMemcpyDefault, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
        AFX_CUDA(cudaGetLastError());
    });
}

// The implicit path of afx_iterate / afx_run_to_convergence: the loop of
// multigrid<implicitSolver>::run_solver (multigrid.h:240-293) with its CFL
// ramp min(start + (i+1) slope, max); run_mode 0 runs n iterations without
// the convergence test.
static int implicit_run(afx_solver_s* s, int n, int run_mode, double tol, double* last) {
    s->ensure_shadow();
    s->materialize_qW();
    if (s->a.n_cases > 0) {
        // batch: every case follows run_solver on its own (per-case err_0,
        // err/err_0, tolerance, iteration limit); the right-hand-side rows
        // of a case that has stopped are zero, so its state holds
        s->set_ctrl(run_mode, n, tol);
        StepArgs A = s->A64();
        A.ctrl = s->a.ctrl;
        if (run_mode == 1) {
            double qf[4] = {0, 0, 0, 0};
            enqueue_uniform_f64(A, s->parity, qf, s->stream);
        }
        AFX_CUDA(cudaEventRecord(s->ev0, s->stream));
        double cfl = s->st.start_cfl;
        int i = 0;
        bool stopped = false;
        while (i < n) {
            if (s->stop.load()) {
                stopped = true;
                break;
            }
            const double e = s->implicit_iteration(cfl, 0.0);
            if (e < 0) {
                s->imp_sync();
                throw Error(AFX_ERR_DIVERGED, "implicit solve failed (singular diagonal block)");
            }
            enqueue_case_control(A, s->stream);  // per-case norms of the last right-hand side
            cfl = std::min(s->st.start_cfl + (i + 1) * s->st.slope_cfl, s->st.max_cfl);
            ++i;
            s->read_ctrl();
            if (s->h_ctrl->done) break;
        }
        AFX_CUDA(cudaEventRecord(s->ev1, s->stream));
        AFX_CUDA(cudaEventSynchronize(s->ev1));
        float ms = 0;
        AFX_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
        s->last_sec = ms * 1e-3;
        s->imp_sync();
        if (last) *last = 0;
        if (stopped) {
            s->stop.store(0);
            throw Error(AFX_ERR_STOPPED, "stopped by request");
        }
        return i;
    }
    s->set_ctrl(0, 0, 0);
    StepArgs& A = s->A64();
    if (A.ctrl != s->a.ctrl) AFX_CUDA(cudaMemsetAsync(A.ctrl, 0, sizeof(Ctrl), s->stream));
    double err0 = 1.0;
    if (run_mode == 1) {
        double qf[4];
        conservative(s->st, s->freestream(), qf);
        enqueue_uniform_f64(A, s->parity, qf, s->stream);  // qW (last dQ) + freestream fluxes
        Ctrl c;
        AFX_CUDA(cudaMemcpyAsync(&c, A.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
        err0 = c.err0;
    }
    AFX_CUDA(cudaEventRecord(s->ev0, s->stream));
    double cfl = s->st.start_cfl, err = 0;
    int i = 0;
    s->hist.clear();
    bool stopped = false;
    do {
        if (s->stop.load()) {
            stopped = true;
            break;
        }
        const double e = s->implicit_iteration(cfl, run_mode == 1 ? err0 * tol : 0.0);
        if (!(e == e) || e > 1.7976931348623157e308) {
            s->imp_sync();
            throw Error(AFX_ERR_NONFINITE, "residual norm is not finite");
        }
        if (e < 0) {
            s->imp_sync();
            throw Error(AFX_ERR_DIVERGED, "implicit solve failed (singular diagonal block)");
        }
        err = e;
        if (run_mode == 1) {
            if (i == 0 && err > 2 * err0) err0 = err;
            err /= err0;
        }
        cfl = std::min(s->st.start_cfl + (i + 1) * s->st.slope_cfl, s->st.max_cfl);
        ++i;
        s->hist.push_back(err);
    } while ((run_mode == 0 ? i < n : (err > tol && i < n)));
    AFX_CUDA(cudaEventRecord(s->ev1, s->stream));
    AFX_CUDA(cudaEventSynchronize(s->ev1));
    float ms = 0;
    AFX_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->last_sec = ms * 1e-3;
    s->imp_sync();
    if (last) *last = err;
    if (stopped) {
        s->stop.store(0);
        throw Error(AFX_ERR_STOPPED, "stopped by request");
    }
    return i;
}

int afx_iterate(afx_solver s, int n_iters, double* res_norm) {
    return guarded([&] {
        if (!s || n_iters < 0) throw Error(AFX_ERR_ARG, "bad argument");
        if (s->imp) {
            double e = 0;
            if (n_iters > 0) implicit_run(s, n_iters, 0, 0, &e);
            if (res_norm) *res_norm = e;
            return;
        }
        s->set_ctrl(0, n_iters, 0);
        const int done = s->run(n_iters, 0, 0);
        AFX_CUDA(cudaGetLastError());
        if (res_norm) *res_norm = s->h_ctrl->last_norm;
        if (s->h_ctrl->status == 4) throw Error(AFX_ERR_NONFINITE, "residual norm is not finite");
        if (done < 0) throw Error(AFX_ERR_STOPPED, "stopped by request");
    });
}

// Newton-Krylov finish of an implicit solver (no counterpart in the
// reference, whose implicit iteration keeps a pseudo-time term): solve
// RHS(q) = 0 (fillRhoRHS, the flux balance of every real cell) by inexact
// Newton steps J dq = RHS(q), J = -dRHS/dq applied matrix-free as a
// one-sided difference of the right-hand side (step 1e-7 of the state's
// RMS over the direction's), each solved by flexible GMRES to lin_tol
// relative, preconditioned by the solver's own linear solve with its matrix
// at `cfl` (A/dt + the face Jacobians, formed at the Newton iterate).
// Rows are scaled by the cell's perimeter: the unscaled norm is dominated
// by the far field's large faces (and by their round-off, ~1e-11 of the
// freestream norm on a 100-chord hybrid mesh) while the wall's thin cells,
// which set the forces, hardly count; per unit face length every cell
// weighs alike.  Each step is backtracked (halved up to 8 times) until the
// scaled norm falls; a step that finds no decrease (the round-off floor)
// ends the solve at the step's start.  err is ||RHS / perimeter|| over the
// same norm of the freestream state's face fluxes.  record (cap rows of 4,
// may be null): per Newton step err after it, the step length, its Krylov
// steps and the linear residual reached.
static double newton_run(afx_solver_s* s, double tol, int max_newton, double cfl, double lin_tol, int max_krylov,
                         int* n_newton, int* n_krylov, double* record, int cap) {
    if (!s->imp) throw Error(AFX_ERR_CONFIG, "newton: needs an implicit solver");
    if (s->a.visc == 2) throw Error(AFX_ERR_CONFIG, "newton: the Spalart-Allmaras equation is not in its system");
    if (s->a.n_cases > 0) throw Error(AFX_ERR_CONFIG, "newton: not for batches");
    s->ensure_shadow();
    s->materialize_qW();
    s->set_ctrl(0, 0, 0);
    StepArgs A = s->A64();
    if (A.ctrl != s->a.ctrl) AFX_CUDA(cudaMemsetAsync(A.ctrl, 0, sizeof(Ctrl), s->stream));
    const int p = s->parity;
    const size_t N = A.n_cells;
    const long long n4 = 4LL * (long long)N;
    KrylovSpace ks(n4, 60);
    DevBuf q0, b, rp, pc, dq, wsc, psc, tmp;
    for (DevBuf* d : {&q0, &b, &rp, &pc, &dq, &wsc, &psc, &tmp}) d->alloc(N * 32);
    {
        // row scales: 1 / perimeter and perimeter per device cell, 4 rows each
        const HostMesh& hm = s->hm;
        std::vector<double> per(hm.nRealCells, 0.0);
        for (size_t e = 0; e < hm.edgesCells.size(); ++e)
            for (int k = 0; k < 2; ++k) {
                const uint32_t c = hm.edgesCells[e][k];
                if (c < hm.nRealCells) per[c] += hm.edgesLengths[e];
            }
        std::vector<double> w(4 * N), pv(4 * N);
        for (size_t i = 0; i < N; ++i)
            for (int k = 0; k < 4; ++k) {
                pv[4 * i + k] = per[s->hl.cell_old[i]];
                w[4 * i + k] = 1.0 / pv[4 * i + k];
            }
        AFX_CUDA(cudaMemcpyAsync(wsc.p, w.data(), N * 32, cudaMemcpyHostToDevice, s->stream));
        AFX_CUDA(cudaMemcpyAsync(psc.p, pv.data(), N * 32, cudaMemcpyHostToDevice, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    }
    const double* W = (const double*)wsc.p;
    const double* Pm = (const double*)psc.p;
    // ||RHS / perimeter|| of a right-hand side v
    auto scaled_norm = [&](const void* v) {
        kv_mul(ks, W, (const double*)v, (double*)tmp.p, s->stream);
        return std::sqrt(kv_dot(ks, (const double*)tmp.p, (const double*)tmp.p, s->stream));
    };
    double err0 = 1.0;
    {
        // the freestream state's face fluxes (qW, which run_solver adds, cleared)
        double qf[4];
        conservative(s->st, s->freestream(), qf);
        AFX_CUDA(cudaMemsetAsync(A.Rq, 0, (size_t)A.n_cells * 32, s->stream));
        enqueue_uniform_f64(A, p, qf, s->stream);
        const double e0 = scaled_norm(A.Rq);
        err0 = e0 > 0 ? e0 : 1.0;
    }
    double* qm = (double*)A.qm[p];
    StepArgs r = A;
    r.Rq = rp.p;  // right-hand sides of perturbed states
    int nn = 0, nk = 0;
    AFX_CUDA(cudaEventRecord(s->ev0, s->stream));
    s->imp_rhs(p);
    double e = scaled_norm(s->imp_b);
    bool have_q0 = false;  // q0 holds the current step's start (restored if the step fails)
    try {
        while (e / err0 > tol && nn < max_newton) {
            if (!(e == e)) throw Error(AFX_ERR_NONFINITE, "newton: residual norm is not finite");
            StepArgs m = A;
            m.cfl = cfl;
            implicit_fill(s->imp, m, p, s->stream);
            AFX_CUDA(cudaMemcpyAsync(q0.p, qm, N * 32, cudaMemcpyDeviceToDevice, s->stream));
            have_q0 = true;
            // the scaled system (W J) dq = W RHS, W = 1 / perimeter
            kv_mul(ks, W, (const double*)s->imp_b, (double*)b.p, s->stream);
            const double qrms = std::sqrt(kv_dot(ks, (const double*)q0.p, (const double*)q0.p, s->stream) / n4);
            const KrylovOp op = [&](const double* v, double* out) {
                const double vrms = std::sqrt(kv_dot(ks, v, v, s->stream) / n4);
                if (vrms == 0) {
                    AFX_CUDA(cudaMemsetAsync(out, 0, N * 32, s->stream));
                    return;
                }
                const double eps = 1e-7 * std::max(1.0, qrms) / vrms;
                kv_axpby(ks, eps, v, 1.0, (const double*)q0.p, qm, s->stream);
                enqueue_rhs_f64(r, p, s->stream);
                kv_mul(ks, W, (const double*)rp.p, (double*)rp.p, s->stream);
                kv_axpby(ks, -1.0 / eps, (const double*)rp.p, 1.0 / eps, (const double*)b.p, out, s->stream);
            };
            const KrylovOp pre = [&](const double* v, double* out) {
                kv_mul(ks, Pm, v, (double*)pc.p, s->stream);  // M^-1 (perimeter .* v)
                const int rc = s->st.krylov_preconditioner == 1
                                   ? implicit_apply_inverse(s->imp, A, (const double*)pc.p, nullptr, 1.0, out, s->stream)
                                   : implicit_apply_sweep(s->imp, A, (const double*)pc.p, nullptr, 1.0, out, s->stream);
                if (rc < 0) throw Error(AFX_ERR_DIVERGED, "newton: singular diagonal block");
            };
            const FgmresResult fr =
                fgmres(ks, (const double*)b.p, (double*)dq.p, true, lin_tol, max_krylov, op, pre, s->stream);
            nk += fr.iters;
            double lam = 1.0, en = 0;
            bool stalled = false;
            for (int ls = 0;; ++ls) {
                kv_axpby(ks, lam, (const double*)dq.p, 1.0, (const double*)q0.p, qm, s->stream);
                s->imp_rhs(p);
                en = scaled_norm(s->imp_b);
                if (en == en && en < e) break;
                if (ls == 8) {
                    AFX_CUDA(cudaMemcpyAsync(qm, q0.p, N * 32, cudaMemcpyDeviceToDevice, s->stream));
                    s->imp_rhs(p);
                    en = scaled_norm(s->imp_b);
                    stalled = true;
                    break;
                }
                lam *= 0.5;
            }
            if (record && nn < cap) {
                double* row = record + 4 * (size_t)nn;
                row[0] = en / err0;
                row[1] = stalled ? 0.0 : lam;
                row[2] = fr.iters;
                row[3] = fr.res / std::max(fr.b_norm, 1e-300);
            }
            e = en;
            ++nn;
            have_q0 = false;  // the step is taken (or undone): nothing to restore
            if (stalled) break;
        }
    } catch (...) {
        if (have_q0) cudaMemcpyAsync(qm, q0.p, N * 32, cudaMemcpyDeviceToDevice, s->stream);
        s->imp_sync();
        throw;
    }
    // qW (the implicit iteration's last update, which run_solver's err_0
    // adds to the freestream fluxes) is left at zero
    AFX_CUDA(cudaMemsetAsync(A.Rq, 0, (size_t)A.n_cells * 32, s->stream));
    AFX_CUDA(cudaEventRecord(s->ev1, s->stream));
    AFX_CUDA(cudaEventSynchronize(s->ev1));
    float ms = 0;
    AFX_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->last_sec = ms * 1e-3;
    s->imp_sync();
    if (n_newton) *n_newton = nn;
    if (n_krylov) *n_krylov = nk;
    return e / err0;
}

int afx_newton_solve(afx_solver s, double tol, int max_newton, double cfl, double lin_tol, int max_krylov,
                     int* newton_iters, int* krylov_iters, double* err, double* record, int record_cap) {
    return guarded([&] {
        if (!s) throw Error(AFX_ERR_ARG, "null argument");
        if (tol <= 0) tol = s->st.tolerance;
        if (max_newton <= 0) max_newton = 20;
        if (cfl <= 0) cfl = s->st.max_cfl;
        if (lin_tol <= 0) lin_tol = 1e-3;
        if (max_krylov <= 0) max_krylov = 300;
        const double e = newton_run(s, tol, max_newton, cfl, lin_tol, max_krylov, newton_iters, krylov_iters,
                                    record, record_cap);
        if (err) *err = e;
    });
}

int afx_run_to_convergence(afx_solver s, double tol, int max_it, int* iters, double* err) {
    return guarded([&] {
        if (!s) throw Error(AFX_ERR_ARG, "null argument");
        if (tol <= 0) tol = s->st.tolerance;
        if (max_it <= 0) max_it = s->st.max_iterations;
        if (s->imp) {
            double e = 0;
            const int n = implicit_run(s, max_it, 1, tol, &e);
            if (iters) *iters = n;
            if (err) *err = e;
            return;
        }
        s->materialize_qW();
        s->set_ctrl(1, max_it, tol);
        double qf[4];
        conservative(s->st, s->freestream(), qf);
        if (s->fp64) enqueue_uniform_f64(s->a, s->parity, qf, s->stream);
        else enqueue_uniform_f32(s->a, s->parity, qf, s->stream);
        const int done = s->run(max_it, 1, tol);
        AFX_CUDA(cudaGetLastError());
        if (iters) *iters = s->h_ctrl->iter;
        if (err) *err = s->h_ctrl->err;
        s->hist.resize(s->h_ctrl->hist_n);
        if (!s->hist.empty())
            AFX_CUDA(cudaMemcpy(s->hist.data(), s->a.hist, s->hist.size() * 8, cudaMemcpyDeviceToHost));
        if (s->h_ctrl->status == 4) throw Error(AFX_ERR_NONFINITE, "residual norm is not finite");
        if (done < 0) throw Error(AFX_ERR_STOPPED, "stopped by request");
    });
}

int afx_residual_history(afx_solver s, double* out, int cap, int* n) {
    return guarded([&] {
        if (!s || !n) throw Error(AFX_ERR_ARG, "null argument");
        *n = (int)s->hist.size();
        if (out)
            for (int i = 0; i < *n && i < cap; ++i) out[i] = s->hist[i];
    });
}

// get_wall_profile (post.h:301-387) over the boundary edges named `patch`,
// with the freestream `vf`.
// Force-integration arguments of the boundary edges named `patch` (their
// geometry is uploaded on first use), with the freestream `vf`.
static ForceArgs force_args(afx_solver_s* s, const std::string& patch, const FarfieldVars& vf) {
    {
        auto& pf = s->patches[patch];
        if (!pf) {
            pf.reset(new afx_solver_s::PatchForces());
            std::vector<int> cells;
            std::vector<double> geo;
            bool first = true;
            unsigned n_added = 0;
            for (const auto& be : s->bedges) {  // post.h:320-338
                if (be.patch != patch) continue;
                if (first) {
                    pf->xmin = pf->xmax = be.ex;
                    pf->y_moment = be.ey;
                    first = false;
                } else {
                    pf->xmin = std::min(pf->xmin, be.ex);
                    pf->xmax = std::max(pf->xmax, be.ex);
                    pf->y_moment += be.ey;
                }
                n_added += 1;
                cells.push_back(be.owner_dev);
                geo.insert(geo.end(), {be.ex, be.ey, be.nx, be.ny, be.L});
            }
            if (n_added == 0) {
                s->patches.erase(patch);
                throw Error(AFX_ERR_ARG, "no boundary edges on patch '" + patch + "'");
            }
            pf->y_moment /= (double)n_added;
            pf->x_moment = (pf->xmax - pf->xmin) * 0.25 + pf->xmin;
            pf->n = (int)n_added;
            pf->cell.upload(cells.data(), cells.size() * sizeof(int), s->stream);
            pf->geo.upload(geo.data(), geo.size() * 8, s->stream);
            pf->cp.alloc(n_added * 8);
            pf->sums.alloc(3 * 8);
        }
        ForceArgs f;
        f.n = pf->n;
        f.cell = (const int*)pf->cell.p;
        f.geo = (const double*)pf->geo.p;
        f.xmin = pf->xmin;
        f.xmax = pf->xmax;
        f.x_moment = pf->x_moment;
        f.y_moment = pf->y_moment;
        f.p_inf = vf.p;
        f.mach_inf = vf.mach;
        f.gamma = s->st.gamma;
        f.q = (const double*)s->a.qm[s->parity];
        f.cp = (double*)pf->cp.p;
        f.sums = (double*)pf->sums.p;
        return f;
    }
}

static void forces_impl(afx_solver_s* s, const std::string& patch, const FarfieldVars& vf, double* cl, double* cd,
                        double* cm, double* cp, int cap, int* n_cp) {
    {
        const ForceArgs f = force_args(s, patch, vf);
        enqueue_forces(f, s->stream);
        double sums[3];
        AFX_CUDA(cudaMemcpyAsync(sums, f.sums, 24, cudaMemcpyDeviceToHost, s->stream));
        std::vector<double> cph(f.n);
        AFX_CUDA(cudaMemcpyAsync(cph.data(), f.cp, f.n * 8, cudaMemcpyDeviceToHost, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
        const double fx = sums[0], fy = sums[1], aoa = vf.angle;  // post.h:379-384
        if (cd) *cd = fx * std::cos(aoa) + fy * std::sin(aoa);
        if (cl) *cl = -fx * std::sin(aoa) + fy * std::cos(aoa);
        if (cm) *cm = sums[2];
        if (n_cp) *n_cp = f.n;
        if (cp)
            for (int i = 0; i < f.n && i < cap; ++i) cp[i] = cph[i];
    }
}

int afx_forces(afx_solver s, const char* patch, double* cl, double* cd, double* cm, double* cp, int cap, int* n_cp) {
    return guarded([&] {
        if (!s || !patch) throw Error(AFX_ERR_ARG, "null argument");
        forces_impl(s, patch, s->freestream(), cl, cd, cm, cp, cap, n_cp);
    });
}

int afx_set_farfield(afx_solver s, const char* patch, double mach, double angle, double T, double p) {
    return guarded([&] {
        if (!s || !patch) throw Error(AFX_ERR_ARG, "null argument");
        auto it = s->st.bcs.find(patch);
        if (it == s->st.bcs.end() || it->second.type != "farfield")
            throw Error(AFX_ERR_ARG, std::string("no farfield patch '") + patch + "'");
        s->materialize_qW();
        it->second.vars = FarfieldVars{mach, angle, T, p};
        s->reset_phase();
        s->set_bcs();
        s->refill_bcs();
    });
}

int afx_profile_iterations(afx_solver s, int n_iters, double* ms, int* launches, int n_kinds) {
    return guarded([&] {
        if (!s || !ms || !launches || n_iters <= 0) throw Error(AFX_ERR_ARG, "bad argument");
        Prof prof;
        for (int i = 0; i <= Prof::CAP; ++i) AFX_CUDA(cudaEventCreate(&prof.ev[i]));
        for (int k = 0; k < n_kinds; ++k) {
            ms[k] = 0;
            launches[k] = 0;
        }
        s->ensure_shadow();
        s->set_ctrl(0, n_iters, 0);
        s->a.prof = &prof;
        try {
            for (int it = 0; it < n_iters; ++it) {
                prof.start(s->stream);
                s->enqueue_iteration(s->parity);
                AFX_CUDA(cudaStreamSynchronize(s->stream));
                for (int j = 0; j < prof.n; ++j) {
                    float t = 0;
                    AFX_CUDA(cudaEventElapsedTime(&t, prof.ev[j], prof.ev[j + 1]));
                    if (prof.kid[j] < n_kinds) {
                        ms[prof.kid[j]] += t;
                        launches[prof.kid[j]] += 1;
                    }
                }
                s->parity ^= 1;
            }
        } catch (...) {
            s->a.prof = nullptr;
            throw;
        }
        s->a.prof = nullptr;
        s->pending_last = s->parity ^ 1;
        for (int i = 0; i <= Prof::CAP; ++i) cudaEventDestroy(prof.ev[i]);
        s->read_ctrl();
        if (s->h_ctrl->status == 4) throw Error(AFX_ERR_NONFINITE, "residual norm is not finite");
    });
}

// Times every residual variant x block size over `iters` iterations from the
// current state and keeps the fastest; the state (and a batch's qW) is put
// back afterwards.
static void autotune_impl(afx_solver_s* s, int iters, char* variant, int cap, int* block, double* ms_per_iter) {
    {
        if (!s || iters <= 0) throw Error(AFX_ERR_ARG, "bad argument");
        StepArgs& a = s->a;
        const size_t N = a.n_cells;
        // qW of the last run is formed now: the timing runs overwrite its inputs
        s->materialize_qW();
        s->ensure_shadow();
        // keep the state: the timing runs start from it and it is put back after
        DevBuf save, saveR, saveNu;
        save.alloc(N * 32);
        AFX_CUDA(cudaMemcpyAsync(save.p, a.qm[s->parity], N * 32, cudaMemcpyDeviceToDevice, s->stream));
        if (a.visc == 2) {
            saveNu.alloc(N * 8);
            AFX_CUDA(cudaMemcpyAsync(saveNu.p, a.sa_nu[s->parity], N * 8, cudaMemcpyDeviceToDevice, s->stream));
        }
        if (a.n_cases > 0) {  // a batch's iterations write qW
            saveR.alloc(N * 32);
            AFX_CUDA(cudaMemcpyAsync(saveR.p, a.Rq, N * 32, cudaMemcpyDeviceToDevice, s->stream));
        }
        const int p0 = s->parity;
        cudaEvent_t e0, e1;
        AFX_CUDA(cudaEventCreate(&e0));
        AFX_CUDA(cudaEventCreate(&e1));
        double best = 1e300;
        int best_var = a.variant, best_block = a.block;
        const int blocks[3] = {64, 128, 256};
        for (int var = a.visc == 2 ? 1 : 0; var < 3; ++var) {
            for (int bi = 0; bi < 3; ++bi) {
                s->set_launch(var, blocks[bi]);
                s->set_ctrl(0, 0, 0);
                AFX_CUDA(cudaMemcpyAsync(a.qm[p0], save.p, N * 32, cudaMemcpyDeviceToDevice, s->stream));
                if (a.visc == 2)
                    AFX_CUDA(cudaMemcpyAsync(a.sa_nu[p0], saveNu.p, N * 8, cudaMemcpyDeviceToDevice, s->stream));
                s->sync_shadow(p0);
                int p = p0;
                s->enqueue_iteration(p);  // warm-up
                p ^= 1;
                AFX_CUDA(cudaEventRecord(e0, s->stream));
                for (int it = 0; it < iters; ++it) {
                    s->enqueue_iteration(p);
                    p ^= 1;
                }
                AFX_CUDA(cudaEventRecord(e1, s->stream));
                AFX_CUDA(cudaEventSynchronize(e1));
                float ms = 0;
                AFX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best) {
                    best = ms;
                    best_var = var;
                    best_block = blocks[bi];
                }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        s->set_launch(best_var, best_block);
        for (auto& g : s->graphs) cudaGraphExecDestroy(g.second);
        s->graphs.clear();
        AFX_CUDA(cudaMemcpyAsync(a.qm[p0], save.p, N * 32, cudaMemcpyDeviceToDevice, s->stream));
        if (a.visc == 2) AFX_CUDA(cudaMemcpyAsync(a.sa_nu[p0], saveNu.p, N * 8, cudaMemcpyDeviceToDevice, s->stream));
        if (a.n_cases > 0) AFX_CUDA(cudaMemcpyAsync(a.Rq, saveR.p, N * 32, cudaMemcpyDeviceToDevice, s->stream));
        s->sync_shadow(p0);
        s->set_ctrl(0, 0, 0);
        AFX_CUDA(cudaStreamSynchronize(s->stream));
        s->parity = p0;
        s->pending_last = -1;
        static const char* vnames[3] = {"gather", "face", "tile"};
        if (variant && cap > 0) std::snprintf(variant, cap, "%s", vnames[best_var]);
        if (block) *block = best_block;
        if (ms_per_iter) *ms_per_iter = best / iters;
    }
}

int afx_autotune(afx_solver s, int iters, char* variant, int cap, int* block, double* ms_per_iter) {
    return guarded([&] { autotune_impl(s, iters, variant, cap, block, ms_per_iter); });
}

int afx_measure_fp64_peak(int reps, double* tflops) {
    return guarded([&] {
        if (!tflops) throw Error(AFX_ERR_ARG, "null argument");
        const double t = fp64_fma_peak(reps > 0 ? reps : 5);
        if (t < 0) throw Error(AFX_ERR_CUDA, "FP64 peak kernel failed");
        *tflops = t;
    });
}

const char* afx_kernel_name(int k) {
    static const char* names[K_COUNT] = {"k_prep", "k_limiter", "k_face_flux", "k_cell_sum", "k_resid_gather",
                                         "k_control", "k_resid_tile"};
    return (k >= 0 && k < K_COUNT) ? names[k] : "";
}

// For callers that cannot let the library allocate device memory (see
// afx_noalloc.cu): the residual of a caller-owned device state, written to a
// caller-owned device array, with all scratch in the library's fixed device
// array.  No cudaMalloc/cudaFree or other allocating call is made here.  The
// work runs on the solver's own stream, which is synchronised before return.
int afx_residual_noalloc(afx_solver s, const double* q_dev, double* R_dev, long long n) {
    return guarded([&] {
        if (!s || !q_dev || !R_dev) throw Error(AFX_ERR_ARG, "null argument");
        const long long N = s->a.n_cells;
        if (n != 4 * N) throw Error(AFX_ERR_ARG, "state size must be 4*n_real_cells");
        if (!s->fp64) throw Error(AFX_ERR_CONFIG, "afx_residual_noalloc needs an fp64 solver");
        if (N > noalloc_max_cells() || s->a.n_faces > noalloc_max_faces())
            throw Error(AFX_ERR_ARG, "mesh too large for afx_residual_noalloc: " + std::to_string(N) + " cells, " +
                                         std::to_string(s->a.n_faces) + " faces (limits " +
                                         std::to_string(noalloc_max_cells()) + " cells, " +
                                         std::to_string(noalloc_max_faces()) + " faces)");
        for (const void* ptr : {(const void*)q_dev, (const void*)R_dev}) {
            cudaPointerAttributes at;
            if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess ||
                (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
                cudaGetLastError();
                throw Error(AFX_ERR_ARG, "afx_residual_noalloc takes device pointers");
            }
        }
        // the lazily formed last-stage qW of a previous iterate() reads the
        // gradient/limiter buffers that the residual below overwrites
        s->materialize_qW();
        s->set_ctrl(0, 0, 0);
        AFX_CUDA(noalloc_residual_f64(s->a, (const int*)s->d_cell_old.p, q_dev, R_dev, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    });
}

// ------------------------------------------------------------------ batch
// A batch is one device solver over the union of its cases' meshes: the
// meshes share no node, so every face, gradient and limiter stencil stays
// within its case, and one launch per kernel advances all cases.  Each
// case's cells are a contiguous device range (case_off); boundary patches are
// renamed "<case>/<patch>" inside the union.
}  // extern "C"

struct afx_batch_s {
    std::unique_ptr<afx_solver_s> s;
    int n = 0;
    std::vector<int> cell_off;  // reference-order (== device-order) cell range of each case
    std::vector<int> bnd_off;   // boundary-edge range of each case
    std::vector<FarfieldVars> far;  // freestream of each case (solver.h:597-611 per case)
    std::vector<std::vector<std::string>> patch_names;
    std::vector<CaseCtrl> h_cctrl;
    DevBuf case_of, case_off, case_done, cell_sq, cctrl, chist, qfar;

    // per-case freestream from the case's own boundaries; uploaded as state
    void set_freestream() {
        far.assign(n, FarfieldVars());
        for (int c = 0; c < n; ++c)
            for (int b = bnd_off[c]; b < bnd_off[c + 1]; ++b)
                if (s->boundary_type[b] == BC_FARFIELD || s->boundary_type[b] == BC_INLET_OUTLET) {
                    far[c] = s->boundary_vars[b];
                    break;
                }
        std::vector<double> q(4 * (size_t)n);
        for (int c = 0; c < n; ++c) conservative(s->st, far[c], &q[4 * c]);
        AFX_CUDA(cudaMemcpyAsync(qfar.p, q.data(), q.size() * 8, cudaMemcpyHostToDevice, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    }
    void read_cases() {
        h_cctrl.resize(n);
        AFX_CUDA(cudaMemcpyAsync(h_cctrl.data(), s->a.cctrl, n * sizeof(CaseCtrl), cudaMemcpyDeviceToHost,
                                 s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    }
    void check_case(int c) const {
        if (c < 0 || c >= n) throw Error(AFX_ERR_ARG, "case index out of range");
    }
};

extern "C" {

int afx_batch_create(int n_cases, const afx_mesh* meshes, const afx_config* configs, afx_batch* out) {
    return guarded([&] {
        if (n_cases <= 0 || !meshes || !configs || !out) throw Error(AFX_ERR_ARG, "bad argument");
        if (n_cases > 65535) throw Error(AFX_ERR_ARG, "at most 65535 cases in a batch");
        auto b = std::make_unique<afx_batch_s>();
        b->n = n_cases;
        // the scheme is shared: every case must agree with case 0 on it
        const Settings& s0 = configs[0] ? configs[0]->s : throw Error(AFX_ERR_ARG, "null config");
        if (s0.viscosity_code() == VISC_SA)
            throw Error(AFX_ERR_CONFIG, "spalart-allmaras cases run one solver each (no batch)");
        Settings st = s0;
        st.bcs.clear();
        st.bc_order.clear();
        if (st.fp64_correction_interval > 0 || st.fp64_finish)
            throw Error(AFX_ERR_CONFIG, "fp64_correction_interval and fp64_finish are single-case options");
        HostMesh u;
        b->cell_off.push_back(0);
        b->bnd_off.push_back(0);
        b->patch_names.resize(n_cases);
        for (int c = 0; c < n_cases; ++c) {
            if (!meshes[c] || !configs[c]) throw Error(AFX_ERR_ARG, "null mesh or config");
            const Settings& sc = configs[c]->s;
            if (sc.gamma != s0.gamma || sc.R != s0.R || sc.mu_L != s0.mu_L || sc.Pr_L != s0.Pr_L ||
                sc.viscosity != s0.viscosity || sc.gradient != s0.gradient || sc.limiter != s0.limiter ||
                sc.precision != s0.precision || sc.second_order != s0.second_order ||
                sc.start_cfl != s0.start_cfl || sc.relaxation != s0.relaxation || sc.limiter_k != s0.limiter_k)
                throw Error(AFX_ERR_CONFIG, "case " + std::to_string(c) +
                                                ": the scheme settings of a batch must match case 0's (only the "
                                                "mesh and the boundary conditions vary per case)");
            const HostMesh& m = meshes[c]->m;
            const uint32_t node0 = (uint32_t)u.nodesX.size();
            u.nodesX.insert(u.nodesX.end(), m.nodesX.begin(), m.nodesX.end());
            u.nodesY.insert(u.nodesY.end(), m.nodesY.begin(), m.nodesY.end());
            for (uint32_t i = 0; i < m.nRealCells; ++i) {
                auto cn = m.cellsNodes[i];
                const int k = m.cellsIsTriangle[i] ? 3 : 4;
                for (int j = 0; j < k; ++j) cn[j] += node0;
                u.cellsNodes.push_back(cn);
                u.cellsIsTriangle.push_back(m.cellsIsTriangle[i]);
            }
            const std::string pre = std::to_string(c) + "/";
            for (size_t e = 0; e < m.bnd0.size(); ++e) {
                u.bnd0.push_back(m.bnd0[e] + node0);
                u.bnd1.push_back(m.bnd1[e] + node0);
                u.bndName.push_back(pre + m.bndName[e]);
            }
            for (const auto& kv : sc.bcs) {
                st.bcs[pre + kv.first] = kv.second;
                b->patch_names[c].push_back(kv.first);
            }
            b->cell_off.push_back((int)u.cellsNodes.size());
            b->bnd_off.push_back((int)u.bnd0.size());
        }
        u.finalize();
        u.segments = b->cell_off;
        const DeviceLayout L = build_layout(u);
        b->s = make_solver(u, L, st);
        afx_solver_s& s = *b->s;
        // the union's boundary edges keep the cases' order: case c's are
        // bnd_off[c]..bnd_off[c+1]
        std::vector<int> cof(u.nRealCells);
        for (int c = 0; c < n_cases; ++c)
            for (int i = b->cell_off[c]; i < b->cell_off[c + 1]; ++i) cof[L.cell_new[i]] = c;
        for (int c = 0; c < n_cases; ++c)
            for (int i = b->cell_off[c]; i < b->cell_off[c + 1]; ++i)
                if (cof[i] != c) throw Error(AFX_ERR_MESH, "batch layout: a case's cells are not contiguous");
        b->case_of.upload(cof.data(), cof.size() * sizeof(int), s.stream);
        b->case_off.upload(b->cell_off.data(), b->cell_off.size() * sizeof(int), s.stream);
        b->case_done.alloc(n_cases * sizeof(int));
        b->cell_sq.alloc(u.nRealCells * sizeof(double));
        b->cctrl.alloc(n_cases * sizeof(CaseCtrl));
        b->chist.alloc((size_t)n_cases * CASE_HIST_CAP * sizeof(double));
        b->qfar.alloc(4 * (size_t)n_cases * sizeof(double));
        StepArgs& a = s.a;
        a.n_cases = n_cases;
        a.case_of = (const int*)b->case_of.p;
        a.case_off = (const int*)b->case_off.p;
        a.case_done = (int*)b->case_done.p;
        a.cell_sq = (double*)b->cell_sq.p;
        a.cctrl = (CaseCtrl*)b->cctrl.p;
        a.chist = (double*)b->chist.p;
        a.qfar_case = (const double*)b->qfar.p;
        if (s.a64.fn) {  // the FP64 machine (implicit right-hand sides) sees the cases too
            for (StepArgs* x : {&s.a64, &s.a64it}) {
                x->n_cases = a.n_cases;
                x->case_of = a.case_of;
                x->case_off = a.case_off;
                x->case_done = a.case_done;
                x->cell_sq = a.cell_sq;
                x->cctrl = a.cctrl;
                x->chist = a.chist;
                x->qfar_case = a.qfar_case;
            }
        }
        AFX_CUDA(cudaMemsetAsync(b->cell_sq.p, 0, u.nRealCells * sizeof(double), s.stream));
        s.set_ctrl(0, 0, 0);
        b->set_freestream();
        *out = b.release();
    });
}

void afx_batch_free(afx_batch b) { delete b; }

int afx_batch_counts(afx_batch b, int* n_cases, long long* n_cells_total) {
    return guarded([&] {
        if (!b) throw Error(AFX_ERR_ARG, "null argument");
        if (n_cases) *n_cases = b->n;
        if (n_cells_total) *n_cells_total = b->s->a.n_cells;
    });
}

int afx_batch_init_freestream(afx_batch b) {
    return guarded([&] {
        if (!b) throw Error(AFX_ERR_ARG, "null argument");
        afx_solver_s& s = *b->s;
        for (int c = 0; c < b->n; ++c) {
            double q[4];
            conservative(s.st, b->far[c], q);  // init(), solver.h:615-631, per case
            for (int i = b->cell_off[c]; i < b->cell_off[c + 1]; ++i) std::memcpy(s.h_stage + 4 * (size_t)i, q, 32);
        }
        // cases are contiguous device ranges in the same order: no permutation
        // is needed for a per-case uniform state
        AFX_CUDA(cudaMemcpyAsync(s.a.qm[s.parity], s.h_stage, (size_t)s.a.n_cells * 32, cudaMemcpyHostToDevice,
                                 s.stream));
        s.sync_shadow(s.parity);
        AFX_CUDA(cudaStreamSynchronize(s.stream));
    });
}

int afx_batch_set_state(afx_batch b, int c, const double* q, long long n) {
    return guarded([&] {
        if (!b || !q) throw Error(AFX_ERR_ARG, "null argument");
        b->check_case(c);
        afx_solver_s& s = *b->s;
        const size_t N = s.a.n_cells, c0 = b->cell_off[c], nc = b->cell_off[c + 1] - c0;
        if (n != (long long)(4 * nc)) throw Error(AFX_ERR_ARG, "state size must be 4*n_real_cells of the case");
        // whole state out in reference order, the case's slice replaced, back in
        enqueue_permute_out((int)N, (const int*)s.d_cell_old.p, s.a.qm[s.parity], s.d_stage.p, s.stream);
        AFX_CUDA(cudaMemcpyAsync((double*)s.d_stage.p + 4 * c0, q, nc * 32, cudaMemcpyDefault, s.stream));
        enqueue_permute_in((int)N, (const int*)s.d_cell_old.p, s.d_stage.p, s.a.qm[s.parity], s.stream);
        s.sync_shadow(s.parity);
        AFX_CUDA(cudaStreamSynchronize(s.stream));
    });
}

int afx_batch_get_state(afx_batch b, int c, double* q, long long n) {
    return guarded([&] {
        if (!b || !q) throw Error(AFX_ERR_ARG, "null argument");
        b->check_case(c);
        afx_solver_s& s = *b->s;
        const size_t N = s.a.n_cells, c0 = b->cell_off[c], nc = b->cell_off[c + 1] - c0;
        if (n != (long long)(4 * nc)) throw Error(AFX_ERR_ARG, "state size must be 4*n_real_cells of the case");
        enqueue_permute_out((int)N, (const int*)s.d_cell_old.p, s.a.qm[s.parity], s.d_stage.p, s.stream);
        AFX_CUDA(cudaMemcpyAsync(q, (const double*)s.d_stage.p + 4 * c0, nc * 32, cudaMemcpyDefault, s.stream));
        AFX_CUDA(cudaStreamSynchronize(s.stream));
    });
}

int afx_batch_iterate(afx_batch b, int n_iters, double* res_norms) {
    return guarded([&] {
        if (!b || n_iters < 0) throw Error(AFX_ERR_ARG, "bad argument");
        afx_solver_s& s = *b->s;
        int done = 0;
        if (s.imp) {
            implicit_run(&s, n_iters, 0, 0, nullptr);
        } else {
            s.set_ctrl(0, n_iters, 0);
            done = s.run(n_iters, 0, 0);
        }
        AFX_CUDA(cudaGetLastError());
        b->read_cases();
        bool bad = false;
        for (int c = 0; c < b->n; ++c) {
            if (res_norms) res_norms[c] = b->h_cctrl[c].last_norm;
            bad |= b->h_cctrl[c].status == 4;
        }
        if (bad) throw Error(AFX_ERR_NONFINITE, "residual norm is not finite in at least one case");
        if (done < 0) throw Error(AFX_ERR_STOPPED, "stopped by request");
    });
}

int afx_batch_run_to_convergence(afx_batch b, double tol, int max_it, int* iters, double* errs, int* status) {
    return guarded([&] {
        if (!b) throw Error(AFX_ERR_ARG, "null argument");
        afx_solver_s& s = *b->s;
        if (tol <= 0) tol = s.st.tolerance;
        if (max_it <= 0) max_it = s.st.max_iterations;
        int done = 0;
        if (s.imp) {
            implicit_run(&s, max_it, 1, tol, nullptr);
        } else {
            s.set_ctrl(1, max_it, tol);
            // get_uniform_residual per case: each cell's case freestream
            double qf[4] = {0, 0, 0, 0};
            if (s.fp64) enqueue_uniform_f64(s.a, s.parity, qf, s.stream);
            else enqueue_uniform_f32(s.a, s.parity, qf, s.stream);
            done = s.run(max_it, 1, tol);
        }
        AFX_CUDA(cudaGetLastError());
        b->read_cases();
        for (int c = 0; c < b->n; ++c) {
            if (iters) iters[c] = b->h_cctrl[c].iter;
            if (errs) errs[c] = b->h_cctrl[c].err;
            if (status) status[c] = b->h_cctrl[c].status == 4 ? AFX_ERR_NONFINITE : AFX_OK;
        }
        if (done < 0) throw Error(AFX_ERR_STOPPED, "stopped by request");
    });
}

int afx_batch_case_history(afx_batch b, int c, double* out, int cap, int* n) {
    return guarded([&] {
        if (!b || !n) throw Error(AFX_ERR_ARG, "null argument");
        b->check_case(c);
        b->read_cases();
        const int k = std::min(b->h_cctrl[c].hist_n, CASE_HIST_CAP);
        *n = k;
        if (out && cap > 0 && k > 0)
            AFX_CUDA(cudaMemcpy(out, b->s->a.chist + (size_t)c * CASE_HIST_CAP, std::min(k, cap) * 8,
                                cudaMemcpyDeviceToHost));
    });
}

int afx_batch_forces(afx_batch b, int c, const char* patch, double* cl, double* cd, double* cm) {
    return guarded([&] {
        if (!b || !patch) throw Error(AFX_ERR_ARG, "null argument");
        b->check_case(c);
        forces_impl(b->s.get(), std::to_string(c) + "/" + patch, b->far[c], cl, cd, cm, nullptr, 0, nullptr);
    });
}

int afx_batch_set_farfield(afx_batch b, int c, const char* patch, double mach, double angle, double T, double p) {
    return guarded([&] {
        if (!b || !patch) throw Error(AFX_ERR_ARG, "null argument");
        b->check_case(c);
        afx_solver_s& s = *b->s;
        auto it = s.st.bcs.find(std::to_string(c) + "/" + patch);
        if (it == s.st.bcs.end() || it->second.type != "farfield")
            throw Error(AFX_ERR_ARG, std::string("no farfield patch '") + patch + "' in case " + std::to_string(c));
        it->second.vars = FarfieldVars{mach, angle, T, p};
        s.set_bcs();
        s.refill_bcs();
        b->set_freestream();
    });
}

int afx_batch_autotune(afx_batch b, int iters, char* variant, int cap, int* block, double* ms_per_iter) {
    return guarded([&] {
        if (!b) throw Error(AFX_ERR_ARG, "null argument");
        autotune_impl(b->s.get(), iters, variant, cap, block, ms_per_iter);
    });
}

int afx_batch_last_device_seconds(afx_batch b, double* sec) {
    return guarded([&] {
        if (!b || !sec) throw Error(AFX_ERR_ARG, "null argument");
        *sec = b->s->last_sec;
    });
}

int afx_batch_linear_iterations(afx_batch b, int* iters, int n_cases) {
    return guarded([&] {
        if (!b || !iters) throw Error(AFX_ERR_ARG, "null argument");
        if (n_cases != b->n) throw Error(AFX_ERR_ARG, "n_cases must be the batch's case count");
        for (int c = 0; c < b->n; ++c) iters[c] = b->s->imp ? b->s->imp_lin_iters : 0;
    });
}

// ---------------------------------------------------------------- adjoint
int afx_residual_vjp(afx_solver s, const double* q, const double* v, double* u, double* bq_bar, long long n) {
    return guarded([&] {
        if (!s || !v || !u) throw Error(AFX_ERR_ARG, "null argument");
        const size_t N = s->a.n_cells, B = s->a.n_bnd;
        if (n != (long long)(4 * N)) throw Error(AFX_ERR_ARG, "state size must be 4*n_real_cells");
        auto& J = s->adjoint();
        s->materialize_qW();  // the prep below overwrites the last stage's gradients
        s->set_ctrl(0, 0, 0);
        StepArgs a = s->a;
        int p = s->parity;
        if (q) {  // the caller's state in a scratch buffer; the solver's own state is kept
            AFX_CUDA(cudaMemcpyAsync(s->d_stage.p, q, N * 32, cudaMemcpyDefault, s->stream));
            enqueue_permute_in((int)N, (const int*)s->d_cell_old.p, s->d_stage.p, J.q.p, s->stream);
            a.qm[0] = a.qsh[0] = J.q.p;
            p = 0;
        }
        AFX_CUDA(cudaMemcpyAsync(s->d_stage.p, v, N * 32, cudaMemcpyDefault, s->stream));
        enqueue_permute_in((int)N, (const int*)s->d_cell_old.p, s->d_stage.p, J.v.p, s->stream);
        enqueue_adjoint_prep(a, p, false, s->stream);
        enqueue_vjp(a, p, J.args(J.v.p, J.u.p), s->stream);
        enqueue_permute_out((int)N, (const int*)s->d_cell_old.p, J.u.p, s->d_stage.p, s->stream);
        AFX_CUDA(cudaMemcpyAsync(u, s->d_stage.p, N * 32, cudaMemcpyDefault, s->stream));
        if (bq_bar && B > 0) AFX_CUDA(cudaMemcpyAsync(bq_bar, J.bqbar.p, B * 32, cudaMemcpyDefault, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
        AFX_CUDA(cudaGetLastError());
    });
}

int afx_boundary_states(afx_solver s, double* bq, long long n) {
    return guarded([&] {
        if (!s || !bq) throw Error(AFX_ERR_ARG, "null argument");
        const size_t B = s->boundary_type.size();
        if (n != (long long)(4 * B)) throw Error(AFX_ERR_ARG, "size must be 4*n_boundary_edges");
        for (size_t b = 0; b < B; ++b) conservative(s->st, s->boundary_vars[b], bq + 4 * b);
    });
}

int afx_adjoint_solve(afx_solver s, const char* patch, const char* objective, double tol, int max_it, double* dJ,
                      int* iters, double* res) {
    return guarded([&] {
        if (!s || !patch || !objective || !dJ) throw Error(AFX_ERR_ARG, "null argument");
        const std::string obj = objective;
        if (obj != "cl" && obj != "cd") throw Error(AFX_ERR_ARG, "objective must be \"cl\" or \"cd\"");
        if (tol <= 0) tol = 1e-10;
        if (max_it <= 0) max_it = 100000;
        auto& J = s->adjoint();
        const size_t N = s->a.n_cells, B = s->a.n_bnd;
        s->materialize_qW();
        s->set_ctrl(0, 0, 0);
        const int p = s->parity;
        const StepArgs& a = s->a;
        const FarfieldVars vf = s->freestream();
        // forces at the converged state and dJ/dq of J = cx*fx + cy*fy
        double cl = 0, cd = 0;
        forces_impl(s, patch, vf, &cl, &cd, nullptr, nullptr, 0, nullptr);
        const double ca = std::cos(vf.angle), sa = std::sin(vf.angle);
        const double cx = obj == "cl" ? -sa : ca, cy = obj == "cl" ? ca : sa;
        ForceArgs f = force_args(s, patch, vf);
        AFX_CUDA(cudaMemsetAsync(J.g.p, 0, N * 32, s->stream));
        enqueue_objective_grad(f, cx, cy, J.g.p, s->stream);
        int q = 0, it = 0;
        double r0 = -1, r = 0;
        if (s->imp) {
            // an implicit solver: (dR/dq)^T lam = -dJ/dq by flexible GMRES on
            // the exact transposed Jacobian (the vJP kernel), preconditioned
            // by the solver's own linear solve with its matrix at max_cfl,
            // transposed: M^T d = v (GMRES, the transposed ILU(0)), then
            // -A .* d -- the primal's implicit iteration for the adjoint
            // equation (dR/dq = -M/A as the CFL grows), accelerated
            StepArgs m = a;
            m.cfl = s->st.max_cfl;
            implicit_fill(s->imp, m, p, s->stream);
            implicit_transpose(s->imp, s->stream);
            enqueue_adjoint_prep(a, p, false, s->stream);  // gradients and limiter of the state for the vJP
            const long long n4 = 4LL * (long long)N;
            KrylovSpace ks(n4, 60);
            DevBuf rhs, pc;
            rhs.alloc(N * 32);
            pc.alloc(N * 32);
            kv_axpby(ks, -1.0, (const double*)J.g.p, 0.0, nullptr, (double*)rhs.p, s->stream);
            DevBuf& last = J.lam_obj[obj == "cl" ? 0 : 1];
            const bool warm = last.p != nullptr;
            if (warm) AFX_CUDA(cudaMemcpyAsync(J.lam[0].p, last.p, N * 32, cudaMemcpyDeviceToDevice, s->stream));
            const KrylovOp op = [&](const double* v, double* out) {
                enqueue_vjp(a, p, J.args(v, out), s->stream);
            };
            const KrylovOp pre = [&](const double* v, double* out) {
                AFX_CUDA(cudaMemcpyAsync(pc.p, v, N * 32, cudaMemcpyDeviceToDevice, s->stream));
                const double* area = (const double*)a.area;
                const int rc = s->st.krylov_preconditioner == 1
                                   ? implicit_apply_inverse(s->imp, a, (const double*)pc.p, area, -1.0, out, s->stream)
                                   : implicit_apply_sweep(s->imp, a, (const double*)pc.p, area, -1.0, out, s->stream);
                if (rc < 0) throw Error(AFX_ERR_NONFINITE, "adjoint: singular diagonal block");
            };
            AFX_CUDA(cudaEventRecord(s->ev0, s->stream));
            const FgmresResult fr =
                fgmres(ks, (const double*)rhs.p, (double*)J.lam[0].p, !warm, tol, max_it, op, pre, s->stream);
            if (!last.p) last.alloc(N * 32);
            AFX_CUDA(cudaMemcpyAsync(last.p, J.lam[0].p, N * 32, cudaMemcpyDeviceToDevice, s->stream));
            if (!(fr.res == fr.res) || fr.res > 1.7976931348623157e308)
                throw Error(AFX_ERR_NONFINITE, "adjoint diverged");
            it = fr.iters;
            r0 = fr.b_norm > 0 ? fr.b_norm : 1.0;
            r = fr.res;
        } else {
            // gradients, limiter and local time step of the converged state
            enqueue_adjoint_prep(a, p, true, s->stream);
            // pseudo-time iteration lam <- lam + relax*dt*(J^T lam + dJ/dq) with
            // the solver's three stages (alpha = 1/4, 1/2, 1), from lam = 0
            AFX_CUDA(cudaMemsetAsync(J.lam[0].p, 0, N * 32, s->stream));
            static const double alpha[3] = {0.25, 0.5, 1.0};
            const int nparts = (int)((N + 255) / 256);
            std::vector<double> parts(nparts);
            const int chunk = 10;
            auto one = [&](int qq, bool norm) {
                const void* l0 = J.lam[qq].p;
                for (int st = 0; st < 3; ++st) {
                    const void* lk = st == 0 ? l0 : J.ls[st - 1].p;
                    enqueue_vjp(a, p, J.args(lk, J.u.p), s->stream);
                    void* out = st < 2 ? J.ls[st].p : J.lam[qq ^ 1].p;
                    enqueue_adjoint_update((int)N, l0, J.u.p, J.g.p, a.dt, alpha[st], a.relax, out,
                                           (st == 2 && norm) ? (double*)J.partials.p : nullptr, s->stream);
                }
            };
            // a graph of `chunk` iterations (even, so it starts and ends on lam[0])
            cudaGraph_t gr;
            cudaGraphExec_t ge;
            AFX_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            for (int k = 0; k < chunk; ++k) one(k & 1, k == chunk - 1);
            AFX_CUDA(cudaStreamEndCapture(s->stream, &gr));
            AFX_CUDA(cudaGraphInstantiate(&ge, gr, 0));
            cudaGraphDestroy(gr);
            AFX_CUDA(cudaEventRecord(s->ev0, s->stream));
            try {
                while (it < max_it) {
                    AFX_CUDA(cudaGraphLaunch(ge, s->stream));
                    it += chunk;
                    AFX_CUDA(cudaMemcpyAsync(parts.data(), J.partials.p, nparts * 8, cudaMemcpyDeviceToHost,
                                             s->stream));
                    AFX_CUDA(cudaStreamSynchronize(s->stream));
                    double t = 0;
                    for (double x : parts) t += x;
                    r = std::sqrt(t);
                    if (!(r == r) || r > 1.7976931348623157e308) throw Error(AFX_ERR_NONFINITE, "adjoint diverged");
                    if (r0 < 0) {
                        // the first chunk's residual stands in for ||dJ/dq|| (lam = 0)
                        std::vector<double> gh(4 * N);
                        AFX_CUDA(cudaMemcpy(gh.data(), J.g.p, N * 32, cudaMemcpyDeviceToHost));
                        double g2 = 0;
                        for (double x : gh) g2 += x * x;
                        r0 = std::sqrt(g2) > 0 ? std::sqrt(g2) : 1.0;
                    }
                    if (r / r0 < tol || s->stop.load()) break;
                }
            } catch (...) {
                cudaGraphExecDestroy(ge);
                throw;
            }
            cudaGraphExecDestroy(ge);
        }
        AFX_CUDA(cudaEventRecord(s->ev1, s->stream));
        AFX_CUDA(cudaEventSynchronize(s->ev1));
        float ms = 0;
        AFX_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
        s->last_sec = ms * 1e-3;
        s->adj_parity = q;
        s->adj_patch = patch;
        s->adj_objective = obj;
        if (iters) *iters = it;
        if (res) *res = r / r0;
        // dJ/dalpha, dJ/dM = explicit terms + lam . dR/dbq . dbq/d(alpha, M)
        enqueue_vjp(a, p, J.args(J.lam[q].p, J.u.p), s->stream);
        std::vector<double> bb(4 * B);
        if (B) AFX_CUDA(cudaMemcpyAsync(bb.data(), J.bqbar.p, B * 32, cudaMemcpyDeviceToHost, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
        const double Jv = obj == "cl" ? cl : cd;
        double da = obj == "cl" ? -cd : cl;  // d/dalpha of (cx, cy) at fixed forces
        double dm = -2.0 * Jv / vf.mach;      // cp ~ 1/M^2
        for (size_t b = 0; b < B; ++b) {
            if (s->boundary_type[b] != BC_FARFIELD) continue;
            double qb[4];
            conservative(s->st, s->boundary_vars[b], qb);
            const FarfieldVars& bv = s->boundary_vars[b];
            const double kin = qb[3] - bv.p / (s->st.gamma - 1);
            da += bb[4 * b + 1] * (-qb[2]) + bb[4 * b + 2] * qb[1];
            if (bv.mach != 0)
                dm += (bb[4 * b + 1] * qb[1] + bb[4 * b + 2] * qb[2] + bb[4 * b + 3] * 2.0 * kin) / bv.mach;
        }
        dJ[0] = da;
        dJ[1] = dm;
        if (s->stop.load()) {
            s->stop.store(0);
            throw Error(AFX_ERR_STOPPED, "stopped by request");
        }
    });
}

// Inverse-distance deformation data of `patch` with weights d^-power: the
// patch nodes (normals from the undeformed mesh), the nodes of the other
// boundary patches (held fixed), and each volume node's weight sum.
static afx_solver_s::PatchDeform& patch_deform(afx_solver_s* s, const std::string& patch, double power) {
    if (s->pdef && s->pdef->patch == patch && s->pdef->power == power) return *s->pdef;
    const HostMesh& m = s->hm;
    if (s->nodes0x.empty()) {
        s->nodes0x = m.nodesX;
        s->nodes0y = m.nodesY;
    }
    const std::vector<double>&X = s->nodes0x, &Y = s->nodes0y;
    auto d = std::make_unique<afx_solver_s::PatchDeform>();
    d->patch = patch;
    d->power = power;
    const size_t V = X.size();
    d->role.assign(V, 0);
    std::vector<double> nx(V, 0.), ny(V, 0.);
    // undeformed edge normals: the metrics of the undeformed nodes
    HostMesh m0 = m;
    m0.update_nodes(X.data(), Y.data());
    for (size_t b = 0; b < m0.boundaryEdges.size(); ++b) {
        const uint32_t e = m0.boundaryEdges[b];
        const bool on = m0.boundaryEdgesPhysicals[b] == patch;
        for (int k = 0; k < 2; ++k) {
            const uint32_t v = m0.edgesNodes[e][k];
            if (on) {
                d->role[v] = 1;
                nx[v] += m0.edgesNormalsX[e];
                ny[v] += m0.edgesNormalsY[e];
            } else if (d->role[v] != 1) {
                d->role[v] = 2;
            }
        }
    }
    std::vector<int> fixed;
    for (size_t v = 0; v < V; ++v) {
        if (d->role[v] == 1) {
            const double l = std::sqrt(nx[v] * nx[v] + ny[v] * ny[v]);
            d->pnodes.push_back((int)v);
            d->pnx.push_back(nx[v] / l);
            d->pny.push_back(ny[v] / l);
        } else if (d->role[v] == 2) {
            fixed.push_back((int)v);
        }
    }
    if (d->pnodes.empty()) throw Error(AFX_ERR_ARG, "no boundary edges on patch '" + patch + "'");
    d->W.assign(V, 0.);
#pragma omp parallel for
    for (long v = 0; v < (long)V; ++v) {
        if (d->role[v] != 0) continue;
        double w = 0;
        for (int k : d->pnodes) w += std::pow(std::hypot(X[v] - X[k], Y[v] - Y[k]), -power);
        for (int f : fixed) w += std::pow(std::hypot(X[v] - X[f], Y[v] - Y[f]), -power);
        d->W[v] = w;
    }
    s->pdef = std::move(d);
    return *s->pdef;
}

// Node displacement of a displacement (cx, cy) of patch node k (index into
// pnodes), added to (x, y): the node itself moves by (cx, cy), every volume
// node by its inverse-distance weight of node k times (cx, cy)
static void add_patch_vec(const afx_solver_s* s, const afx_solver_s::PatchDeform& d, int k, double cx, double cy,
                          std::vector<double>& x, std::vector<double>& y) {
    const std::vector<double>&X = s->nodes0x, &Y = s->nodes0y;
    const int vk = d.pnodes[k];
    const double p = d.power;
    const long V = (long)X.size();
#pragma omp parallel for
    for (long v = 0; v < V; ++v) {
        if (d.role[v] != 0) continue;
        const double w = std::pow(std::hypot(X[v] - X[vk], Y[v] - Y[vk]), -p) / d.W[v];
        x[v] += w * cx;
        y[v] += w * cy;
    }
    x[vk] += cx;
    y[vk] += cy;
}

// ... of a normal displacement c of patch node k (along its undeformed normal)
static void add_patch_mode(const afx_solver_s* s, const afx_solver_s::PatchDeform& d, int k, double c,
                           std::vector<double>& x, std::vector<double>& y) {
    add_patch_vec(s, d, k, c * d.pnx[k], c * d.pny[k], x, y);
}

int afx_patch_nodes(afx_solver s, const char* patch, long long* ids, double* nx, double* ny, int cap, int* n) {
    return guarded([&] {
        if (!s || !patch || !n) throw Error(AFX_ERR_ARG, "null argument");
        const auto& d = patch_deform(s, patch, s->pdef ? s->pdef->power : 2.0);
        *n = (int)d.pnodes.size();
        for (int k = 0; k < *n && k < cap; ++k) {
            if (ids) ids[k] = d.pnodes[k];
            if (nx) nx[k] = d.pnx[k];
            if (ny) ny[k] = d.pny[k];
        }
    });
}

int afx_deform_patch(afx_solver s, const char* patch, const double* a, int n, double power) {
    return guarded([&] {
        if (!s || !patch || !a) throw Error(AFX_ERR_ARG, "null argument");
        if (power <= 0) power = 2.0;
        const auto& d = patch_deform(s, patch, power);
        if (n != (int)d.pnodes.size())
            throw Error(AFX_ERR_ARG, "expected " + std::to_string(d.pnodes.size()) + " patch-node displacements");
        std::vector<double> x = s->nodes0x, y = s->nodes0y;
        for (int k = 0; k < n; ++k)
            if (a[k] != 0) add_patch_mode(s, d, k, a[k], x, y);
        s->materialize_qW();
        s->set_nodes(x.data(), y.data());
    });
}

int afx_deform_patch_xy(afx_solver s, const char* patch, const double* dx, const double* dy, int n, double power) {
    return guarded([&] {
        if (!s || !patch || !dx || !dy) throw Error(AFX_ERR_ARG, "null argument");
        if (power <= 0) power = 2.0;
        const auto& d = patch_deform(s, patch, power);
        if (n != (int)d.pnodes.size())
            throw Error(AFX_ERR_ARG, "expected " + std::to_string(d.pnodes.size()) + " patch-node displacements");
        std::vector<double> x = s->nodes0x, y = s->nodes0y;
        for (int k = 0; k < n; ++k)
            if (dx[k] != 0 || dy[k] != 0) add_patch_vec(s, d, k, dx[k], dy[k], x, y);
        s->materialize_qW();
        s->set_nodes(x.data(), y.data());
    });
}

// d/dt of the Lagrangian J(q; X(a0 + t c)) + lam . R(q; X(a0 + t c)) at t = 0
// for each direction c (one row of `dirs`, an entry per patch node), by
// central differences with step h about the current node positions, at the
// frozen converged state q: the adjoint's shape derivative along c.
static void shape_directional(afx_solver_s* s, const afx_solver_s::PatchDeform& d, const char* objective, double h,
                              const double* dirs, int n_dirs, bool xy, double* dJ) {
    const int n = (int)d.pnodes.size();
    auto& J = s->adjoint();
    const size_t N = s->a.n_cells;
    const std::string patch = d.patch;
    s->materialize_qW();
    // lambda (device order) to the host
    std::vector<double> lam(4 * N), R(4 * N);
    AFX_CUDA(cudaMemcpyAsync(lam.data(), J.lam[s->adj_parity].p, N * 32, cudaMemcpyDeviceToHost, s->stream));
    AFX_CUDA(cudaStreamSynchronize(s->stream));
    const std::vector<double> xc = s->hm.nodesX, yc = s->hm.nodesY;
    const size_t V = xc.size();
    const FarfieldVars vf = s->freestream();
    const bool cl_obj = std::string(objective) == "cl";
    StepArgs r = s->a;
    r.Rq = J.u.p;  // scratch: the solver's qW stays
    // J(q; X) + lambda . R(q; X) at the current state for nodes (x, y)
    auto lagr = [&](const std::vector<double>& x, const std::vector<double>& y) {
        s->set_nodes(x.data(), y.data());
        s->set_ctrl(0, 0, 0);
        r.area = s->a.area;
        enqueue_residual_f64(r, s->parity, s->stream);
        AFX_CUDA(cudaMemcpyAsync(R.data(), J.u.p, N * 32, cudaMemcpyDeviceToHost, s->stream));
        double cl = 0, cd = 0;
        forces_impl(s, patch, vf, &cl, &cd, nullptr, nullptr, 0, nullptr);
        double lr = 0;
        for (size_t i = 0; i < 4 * N; ++i) lr += lam[i] * R[i];
        return (cl_obj ? cl : cd) + lr;
    };
    try {
        std::vector<double> dx(V), dy(V), xp(V), yp(V), xm(V), ym(V);
        for (int j = 0; j < n_dirs; ++j) {
            std::fill(dx.begin(), dx.end(), 0.);
            std::fill(dy.begin(), dy.end(), 0.);
            if (xy) {
                const double* c = dirs + (size_t)j * 2 * n;
                for (int k = 0; k < n; ++k)
                    if (c[2 * k] != 0 || c[2 * k + 1] != 0) add_patch_vec(s, d, k, c[2 * k], c[2 * k + 1], dx, dy);
            } else {
                const double* c = dirs + (size_t)j * n;
                for (int k = 0; k < n; ++k)
                    if (c[k] != 0) add_patch_mode(s, d, k, c[k], dx, dy);
            }
            for (size_t v = 0; v < V; ++v) {
                xp[v] = xc[v] + h * dx[v];
                yp[v] = yc[v] + h * dy[v];
                xm[v] = xc[v] - h * dx[v];
                ym[v] = yc[v] - h * dy[v];
            }
            dJ[j] = (lagr(xp, yp) - lagr(xm, ym)) / (2 * h);
        }
    } catch (...) {
        s->set_nodes(xc.data(), yc.data());
        throw;
    }
    s->set_nodes(xc.data(), yc.data());
}

int afx_adjoint_patch(afx_solver s, const char* patch, const char* objective, double power, double h, double* dJ,
                      int n) {
    return guarded([&] {
        if (!s || !patch || !objective || !dJ) throw Error(AFX_ERR_ARG, "null argument");
        if (s->adj_patch != patch || s->adj_objective != objective)
            throw Error(AFX_ERR_ARG, "afx_adjoint_patch needs afx_adjoint_solve of the same patch and objective first");
        if (power <= 0) power = 2.0;
        if (h <= 0) h = 1e-7;
        const auto& d = patch_deform(s, patch, power);
        if (n != (int)d.pnodes.size())
            throw Error(AFX_ERR_ARG, "expected room for " + std::to_string(d.pnodes.size()) + " sensitivities");
        std::vector<double> dirs;  // unit vectors e_k
        for (int k = 0; k < n; ++k) {
            std::vector<double> e(n, 0.);
            e[k] = 1.0;
            dirs.insert(dirs.end(), e.begin(), e.end());
        }
        shape_directional(s, d, objective, h, dirs.data(), n, false, dJ);
    });
}

int afx_adjoint_patch_dirs(afx_solver s, const char* patch, const char* objective, double power, double h,
                           const double* dirs, int n_dirs, int n_patch, double* dJ) {
    return guarded([&] {
        if (!s || !patch || !objective || !dirs || !dJ || n_dirs < 0) throw Error(AFX_ERR_ARG, "bad argument");
        if (s->adj_patch != patch || s->adj_objective != objective)
            throw Error(AFX_ERR_ARG,
                        "afx_adjoint_patch_dirs needs afx_adjoint_solve of the same patch and objective first");
        if (power <= 0) power = 2.0;
        if (h <= 0) h = 1e-7;
        const auto& d = patch_deform(s, patch, power);
        if (n_patch != (int)d.pnodes.size())
            throw Error(AFX_ERR_ARG, "directions must have " + std::to_string(d.pnodes.size()) + " entries");
        shape_directional(s, d, objective, h, dirs, n_dirs, false, dJ);
    });
}

int afx_adjoint_patch_dirs_xy(afx_solver s, const char* patch, const char* objective, double power, double h,
                              const double* dirs, int n_dirs, int n_patch, double* dJ) {
    return guarded([&] {
        if (!s || !patch || !objective || !dirs || !dJ || n_dirs < 0) throw Error(AFX_ERR_ARG, "bad argument");
        if (s->adj_patch != patch || s->adj_objective != objective)
            throw Error(AFX_ERR_ARG,
                        "afx_adjoint_patch_dirs_xy needs afx_adjoint_solve of the same patch and objective first");
        if (power <= 0) power = 2.0;
        if (h <= 0) h = 1e-7;
        const auto& d = patch_deform(s, patch, power);
        if (n_patch != (int)d.pnodes.size())
            throw Error(AFX_ERR_ARG, "directions must have 2 x " + std::to_string(d.pnodes.size()) + " entries");
        shape_directional(s, d, objective, h, dirs, n_dirs, true, dJ);
    });
}

int afx_adjoint_state(afx_solver s, double* lam, long long n) {
    return guarded([&] {
        if (!s || !lam) throw Error(AFX_ERR_ARG, "null argument");
        const size_t N = s->a.n_cells;
        if (n != (long long)(4 * N)) throw Error(AFX_ERR_ARG, "size must be 4*n_real_cells");
        auto& J = s->adjoint();
        enqueue_permute_out((int)N, (const int*)s->d_cell_old.p, J.lam[s->adj_parity].p, s->d_stage.p, s->stream);
        AFX_CUDA(cudaMemcpyAsync(lam, s->d_stage.p, N * 32, cudaMemcpyDefault, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    });
}

// multigrid::run's level transfer (multigrid.h:316-321): coarse ghosts from
// their owners, fine state = mapper * coarse state, fine ghosts refilled.
int afx_prolongate(afx_solver coarse, afx_solver fine) {
    return guarded([&] {
        if (!coarse || !fine) throw Error(AFX_ERR_ARG, "null argument");
        afx_solver_s& c = *coarse;
        afx_solver_s& f = *fine;
        const int nc = (int)c.geo_area.size(), nr = c.a.n_cells, nb = nc - nr;
        if (!c.d_geo.p) {
            std::vector<double> g(3 * (size_t)nc);
            std::copy(c.geo_cx.begin(), c.geo_cx.end(), g.begin());
            std::copy(c.geo_cy.begin(), c.geo_cy.end(), g.begin() + nc);
            std::copy(c.geo_area.begin(), c.geo_area.end(), g.begin() + 2 * (size_t)nc);
            c.d_geo.upload(g.data(), g.size() * 8, c.stream);
            std::vector<int> owner(std::max(nb, 1), 0);
            for (int b = 0; b < nb; ++b) owner[b] = c.bedges[b].owner_dev;
            c.d_owner.upload(owner.data(), owner.size() * sizeof(int), c.stream);
            c.d_full.alloc((size_t)nc * 32);
        }
        if (!f.d_devc.p) {
            std::vector<double> g(2 * f.dev_cx.size());
            std::copy(f.dev_cx.begin(), f.dev_cx.end(), g.begin());
            std::copy(f.dev_cy.begin(), f.dev_cy.end(), g.begin() + f.dev_cx.size());
            f.d_devc.upload(g.data(), g.size() * 8, f.stream);
        }
        c.ensure_shadow();
        enqueue_full_state(nr, nb, (const int*)c.d_cell_old.p, (const int*)c.d_owner.p, c.a.qm[c.parity], c.d_full.p,
                           c.stream);
        AFX_CUDA(cudaStreamSynchronize(c.stream));
        AFX_CUDA(cudaStreamSynchronize(f.stream));
        const double* geo = (const double*)c.d_geo.p;
        const double* fc = (const double*)f.d_devc.p;
        enqueue_prolong(nc, geo, geo + nc, geo + 2 * (size_t)nc, c.d_full.p, f.a.n_cells, fc, fc + f.a.n_cells,
                        f.a.qm[f.parity], f.stream);
        f.sync_shadow(f.parity);
        f.shadow_stale = false;
        f.reset_phase();
        f.pending_last = -1;
        f.refill_bcs();
        AFX_CUDA(cudaStreamSynchronize(f.stream));
        AFX_CUDA(cudaGetLastError());
    });
}

// mesh::compute_wall_dist (mesh.h:794-830) with the solver's boundary
// conditions: every cell (ghosts included, reference order).
int afx_wall_distance(afx_solver s, double* out, long long n) {
    return guarded([&] {
        if (!s || !out) throw Error(AFX_ERR_ARG, "null argument");
        const int nc = (int)s->geo_area.size();
        if (n != nc) throw Error(AFX_ERR_ARG, "size must be n_real_cells + n_boundary_edges");
        std::vector<double> w;  // wall edge centres in boundary order, then x / y
        std::vector<double> wy;
        for (size_t b = 0; b < s->bedges.size(); ++b)
            if (s->boundary_type[b] == BC_WALL || s->boundary_type[b] == BC_SLIP_WALL) {
                w.push_back(s->bedges[b].ex);
                wy.push_back(s->bedges[b].ey);
            }
        const int nw = (int)w.size();
        w.insert(w.end(), wy.begin(), wy.end());
        std::vector<double> c(2 * (size_t)nc);
        std::copy(s->geo_cx.begin(), s->geo_cx.end(), c.begin());
        std::copy(s->geo_cy.begin(), s->geo_cy.end(), c.begin() + nc);
        DevBuf dc, dw, dout;
        dc.upload(c.data(), c.size() * 8, s->stream);
        dw.upload(w.data(), std::max<size_t>(w.size(), 1) * 8, s->stream);
        dout.alloc((size_t)nc * 8);
        const double* pc = (const double*)dc.p;
        const double* pw = (const double*)dw.p;
        enqueue_wall_dist(nc, pc, pc + nc, nw, pw, pw + nw, (double*)dout.p, s->stream);
        AFX_CUDA(cudaMemcpyAsync(out, dout.p, (size_t)nc * 8, cudaMemcpyDeviceToHost, s->stream));
        AFX_CUDA(cudaStreamSynchronize(s->stream));
    });
}

// rans::save (post.h:58-180) of a host state on a mesh
int afx_write_vtu(afx_mesh m, const double* q, const double* wall_dist, long long n, double gamma, double R,
                  const char* path) {
    return guarded([&] {
        if (!m || !q || !path) throw Error(AFX_ERR_ARG, "null argument");
        if (n != 4 * (long long)m->m.nRealCells) throw Error(AFX_ERR_ARG, "state size must be 4*n_real_cells");
        write_vtu(m->m, q, wall_dist, gamma, R, path);
    });
}

// save(filename, solver) of the solver's state, with the wall distance that
// multigrid.h:71 forms before a run (mesh::compute_wall_dist, on the GPU)
int afx_save_vtu(afx_solver s, const char* path) {
    return guarded([&] {
        if (!s || !path) throw Error(AFX_ERR_ARG, "null argument");
        const size_t N = s->a.n_cells;
        std::vector<double> q(4 * N), wd(s->geo_area.size());
        if (int rc = afx_get_state(s, q.data(), (long long)q.size())) throw Error(rc, afx_last_error());
        if (int rc = afx_wall_distance(s, wd.data(), (long long)wd.size())) throw Error(rc, afx_last_error());
        write_vtu(s->hm, q.data(), wd.data(), s->st.gamma, s->st.R, path);
    });
}

int afx_linear_iterations(afx_solver s, int* n) {
    return guarded([&] {
        if (!s || !n) throw Error(AFX_ERR_ARG, "null argument");
        *n = s->imp ? s->imp_lin_iters : 0;
    });
}

int afx_request_stop(afx_solver s) {
    if (!s) return AFX_ERR_ARG;
    s->stop.store(1);
    return AFX_OK;
}

int afx_last_device_seconds(afx_solver s, double* sec) {
    return guarded([&] {
        if (!s || !sec) throw Error(AFX_ERR_ARG, "null argument");
        *sec = s->last_sec;
    });
}

}  // extern "C"
