/*
 * afx_rans.h — C ABI of the GB300 rans residual library (libafx_rans.so).
 *
 * Drop-in boundary for AeroFLEX's `rans` module (header-only C++ in the
 * reference: the headers of src/rans/include/rans/).  Each entry point names the
 * reference interface it replaces.  Plain C types only: opaque handles,
 * pointers and sizes.  State arrays cross the boundary in the reference's
 * layout: AoS [rho, rhou, rhov, rhoE] per REAL cell, cells in the order the
 * mesh file (or the arrays) listed them.
 *
 * Every function returns an afx_status (0 = ok).  On failure the message is
 * in afx_last_error() (thread-local).  No C++ exception crosses the ABI.
 * Handles are not thread-safe individually; distinct handles may be used
 * from distinct threads.  afx_request_stop() may be called from any thread.
 */
#ifndef AFX_RANS_H
#define AFX_RANS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    AFX_OK = 0,
    AFX_ERR_IO = 1,        /* file missing / unreadable */
    AFX_ERR_CONFIG = 2,    /* bad INI content or setting (tinyconfig/Settings throws) */
    AFX_ERR_MESH = 3,      /* malformed mesh (mesh.h throws std::invalid_argument) */
    AFX_ERR_NONFINITE = 4, /* residual norm became NaN/Inf */
    AFX_ERR_DIVERGED = 5,  /* residual grew past the divergence guard */
    /* 6 is not used: no entry point waits on the device without a bound */
    AFX_ERR_CUDA = 7,      /* CUDA runtime error or no usable GPU */
    AFX_ERR_ARG = 8,       /* null handle / bad size / unknown name */
    AFX_ERR_STOPPED = 9    /* afx_request_stop() ended a run early (results are valid) */
} afx_status;

typedef struct afx_mesh_s* afx_mesh;
typedef struct afx_config_s* afx_config;
typedef struct afx_solver_s* afx_solver;
typedef struct afx_batch_s* afx_batch;

/* Thread-local text of the last error. */
const char* afx_last_error(void);
/* Library version string. */
const char* afx_version(void);

/* ------------------------------------------------------------- mesh ---- */
/* Replaces rans::mesh::mesh(std::string filename) / read_file
 * (src/rans/include/rans/mesh.h:250, 834-884): gmsh 4.1 ASCII. */
int afx_mesh_load(const char* path, afx_mesh* out);
/* Same mesh built from arrays (the generators' path).  cell_nodes holds 4
 * node indices per cell, -1 in slot 3 for a triangle; boundary edges are
 * node pairs with a patch index into patch_names ('\n'-separated). */
int afx_mesh_from_arrays(int n_nodes, const double* x, const double* y, int n_cells, const int* cell_nodes,
                         int n_bedges, const int* bedge_nodes, const int* bedge_patch, const char* patch_names,
                         afx_mesh* out);
/* counts[0..4] = real cells, cells incl. ghosts, edges, boundary edges, nodes
 * (mesh.h:209-246 sizes; nRealCells, mesh.h:869). */
int afx_mesh_counts(afx_mesh m, long long counts[5]);
/* Copies one FP64 metric in reference order: "cx","cy","area" (all cells incl.
 * ghosts), "ex","ey","nx","ny","L" (edges), "wall_dist" (cells), mesh.h:378-453;
 * "node_x","node_y" (the node coordinates, nodesX/nodesY, mesh.h:209-210). */
int afx_mesh_get(afx_mesh m, const char* what, double* out, long long cap, long long* n);
/* Integer topology: "edges_cells" (2/edge), "edges_nodes" (2/edge),
 * "boundary_edges" (edge id per boundary edge), "cell_order" (device
 * renumbering: reference cell id of each device cell). */
int afx_mesh_get_int(afx_mesh m, const char* what, long long* out, long long cap, long long* n);
/* Physical name of boundary edge b (mesh.h:783-785). */
int afx_mesh_boundary_name(afx_mesh m, int b, char* out, int cap);
/* New node coordinates for the same topology (a deformed shape): the
 * metrics and ghost cells are re-formed with the formulas of mesh.h:378-453,
 * 744-787.  Solvers created afterwards see the new geometry; a solver
 * deforms its own copy with afx_deform_patch.  n = number of nodes. */
int afx_mesh_set_nodes(afx_mesh m, const double* x, const double* y, long long n);
void afx_mesh_free(afx_mesh m);

/* ----------------------------------------------------------- config ---- */
/* Replaces rans::Settings defaults (src/rans/include/rans/core.h:166-199). */
int afx_config_create(afx_config* out);
/* Replaces Settings::import_config_file(tiny::config&) (core.h:238-272) over
 * tiny::config::read (libs/headeronly/tinyconfig.hpp:152-221). */
int afx_config_from_ini(const char* path, afx_config* out);
int afx_config_from_ini_string(const char* text, afx_config* out);
/* Numeric fields: gamma, R, mu_L, Pr_L, Pr_T, start_cfl, slope_cfl, max_cfl,
 * relaxation, tolerance, limiter_k, alpha_start, alpha_end, alpha_step,
 * rhs_iterations, max_iterations, second_order (0/1); this library's
 * block_size (0 auto | 32 | 64 | 128 | 256), fp64_correction_interval
 * (FP32-mixed: refresh an FP64 defect correction every n iterations, 0 off)
 * fp64_finish (FP32-mixed: afx_run_to_convergence continues with FP64
 * iterations once the FP32 residual stops falling, 0/1) and krylov_graph
 * (implicit solver: 1 = each GMRES solve is one CUDA graph with device-side
 * loops, 0 = the same kernels driven from a host loop, for profilers) and
 * krylov_preconditioner (the flexible GMRES of afx_newton_solve and of the
 * implicit adjoint: 1 = a GMRES solve with the implicit matrix, 0 = one
 * ILU(0) sweep with it) and adjoint_directions (input directions per pass
 * of the vJP's face kernel, 1, 2 or 4: vector dual numbers that share the
 * value's work; every choice gives the same bits). */
int afx_config_set_double(afx_config c, const char* key, double v);
int afx_config_get_double(afx_config c, const char* key, double* v);
/* String fields: solver ("explicit"/"implicit"), gradient ("green-gauss"/
 * "least-squares"), viscosity ("inviscid"/"laminar"/"spalart-allmaras"/
 * "spallart-allmaras"), limiter ("venkatakrishnan"/"michalak"),
 * precision ("fp64"/"fp32-mixed"), kernel_variant ("auto"/"gather"/"face"/
 * "tile"), airfoil_name. */
int afx_config_set_string(afx_config c, const char* key, const char* v);
int afx_config_get_string(afx_config c, const char* key, char* out, int cap);
/* One [rans-bc] entry (core.h:244-255): type "farfield"/"slip-wall"/"wall". */
int afx_config_set_bc(afx_config c, const char* name, const char* type, double T, double mach, double angle,
                      double p);
int afx_config_bc_count(afx_config c, int* n);
/* Read one [rans-bc] entry back (Settings::bcs[name], core.h:171). */
int afx_config_get_bc(afx_config c, const char* name, char* type, int cap, double* T, double* mach, double* angle,
                      double* p);
void afx_config_free(afx_config c);

/* ----------------------------------------------------------- solver ---- */
/* Replaces explicitSolver(mesh, gas, viscosity) + set_bcs / set_second_order /
 * set_gradient_scheme / set_limiter_k (solver.h:108, 131-162, 200-247;
 * multigrid.h:70-77).  Uploads the mesh to the GPU in its device layout. */
int afx_solver_create(afx_mesh m, afx_config c, afx_solver* out);
void afx_solver_free(afx_solver s);
/* init() + refill_bcs() (solver.h:615-631, 259-274). */
int afx_init_freestream(afx_solver s);
/* Overwrite the real-cell state (get_q() = ..., solver.h:255) from host
 * AoS FP64 [4*n_real]; ghost states keep their boundary values. */
int afx_set_state(afx_solver s, const double* q, long long n);
int afx_get_state(afx_solver s, double* q, long long n);
/* Spalart-Allmaras solvers (viscosity "spalart-allmaras"; the reference's
 * nu array, solver.h:55, which it leaves unused): nu~ per real cell,
 * reference order.  afx_init_freestream sets nu~ = 3 mu_L / rho_inf. */
int afx_set_turbulence(afx_solver s, const double* nu, long long n);
int afx_get_turbulence(afx_solver s, double* nu, long long n);
/* nu~ residual R/A of the last evaluation (afx_residual: the current state;
 * afx_iterate: the last stage of the last iteration), reference order. */
int afx_turbulence_residual(afx_solver s, double* nuW, long long n);
/* Residual of the current state as the first RK stage forms it: ghosts,
 * Green-Gauss gradient, limiter, face loop, /area (solver.h:745-799).
 * R gets AoS FP64 [4*n_real]. */
int afx_residual(afx_solver s, double* R, long long n);
/* Implicit solvers: fillRhoRHS (solver.h:1079-1152) of the current state —
 * the second-order face sums not divided by the area (RhoVector), real-cell
 * rows, AoS FP64 [4*n_real], reference cell order. */
int afx_implicit_rhs(afx_solver s, double* rhs, long long n);
/* n explicit iterations (explicitSolver::solve, solver.h:802-828); res_norm
 * gets ‖qW‖₂ of the last stage of the last iteration. */
int afx_iterate(afx_solver s, int n_iters, double* res_norm);
/* multigrid<explicitSolver>::run_solver (multigrid.h:182-237): err_0 from
 * get_uniform_residual (solver.h:636-690), iterate until err <= tolerance,
 * max_iterations, or afx_request_stop.  tol/max_it <= 0 take the config's. */
int afx_run_to_convergence(afx_solver s, double tol, int max_it, int* iters, double* err);
/* Newton-Krylov finish of an implicit solver (not in the reference, whose
 * implicit iteration keeps its pseudo-time term at max_cfl): inexact Newton
 * on the implicit right-hand side (fillRhoRHS) with matrix-free
 * Jacobian-vector products (one-sided differences of the right-hand side),
 * flexible GMRES to lin_tol relative (<= 0: 1e-3; at most max_krylov steps
 * per Newton step, <= 0: 300) preconditioned by the solver's own linear
 * solve with its matrix at `cfl` (<= 0: max_cfl).  Rows are scaled by the
 * cell perimeter (flux imbalance per unit face length: the wall's thin
 * cells weigh as much as the far field's large ones), and each step
 * backtracks on that scaled norm.  Stops at err <= tol (<= 0: the
 * settings' tolerance), err = ||RHS / perimeter|| over the same norm of the
 * freestream state's face fluxes, or after max_newton steps (<= 0: 20).
 * Leaves qW (the last-update term of afx_run_to_convergence's err_0) at 0.
 * A step that finds no decrease after 8 halvings (the round-off floor of
 * the right-hand side) ends the solve at its start; compare err with tol.
 * record (record_cap rows of 4, may be NULL): per Newton step err after it,
 * the step length taken (0: none), its Krylov steps, the relative linear
 * residual reached.  Start it from a state the implicit iteration has
 * brought near the solution.  Not for Spalart-Allmaras solvers or batches. */
int afx_newton_solve(afx_solver s, double tol, int max_newton, double cfl, double lin_tol, int max_krylov,
                     int* newton_iters, int* krylov_iters, double* err, double* record, int record_cap);
/* Residual history as run_solver stores it (every 10th iteration). */
int afx_residual_history(afx_solver s, double* out, int cap, int* n);
/* get_wall_profile(solver&, patch) (src/rans/include/rans/post.h:301-387):
 * pressure C_L, C_D, C_M and cp per patch edge (cap entries at most). */
int afx_forces(afx_solver s, const char* patch, double* cl, double* cd, double* cm, double* cp, int cap,
               int* n_cp);
/* settings.bcs[patch].vars_far = {...}; set_bcs(...) (rans.h:92-97). */
int afx_set_farfield(afx_solver s, const char* patch, double mach, double angle, double T, double p);
/* Atomic stop flag polled between device launch groups (GUIHandler::signal.stop,
 * src/common/common_aeroflex.hpp:11-19; multigrid.h:234). */
int afx_request_stop(afx_solver s);
/* Seconds of device time spent by the last afx_iterate/afx_run_to_convergence. */
int afx_last_device_seconds(afx_solver s, double* sec);

/* Measurement hooks (no counterpart in the reference, which has no
 * profiling): n iterations launched eagerly with a CUDA event after every
 * kernel on the solver's stream; ms[k] and launches[k] accumulate per kernel
 * kind k < n_kinds, named by afx_kernel_name(k).  The state advances by n
 * iterations exactly as afx_iterate would. */
int afx_profile_iterations(afx_solver s, int n_iters, double* ms, int* launches, int n_kinds);
const char* afx_kernel_name(int k);
/* FP64 arithmetic peak of the current GPU, measured (no counterpart in the
 * reference): independent fused multiply-add chains on every SM, best of
 * `reps` launches timed with CUDA events, 2 flops per FMA, in TFLOP/s.  The
 * denominator of the FP64 path's roofline, which the FP64 pipe bounds. */
int afx_measure_fp64_peak(int reps, double* tflops);
/* Launch autotuner (no counterpart in the reference): times `iters`
 * iterations of each residual-kernel variant ("gather": per-cell flux
 * re-formation; "face": one flux per face + ordered cell sum) at 64, 128 and
 * 256 threads per block on this solver's mesh, keeps the fastest, and puts
 * the state back.  Both variants give bit-identical results; the state and
 * the stored residual qW are as before the call. */
int afx_autotune(afx_solver s, int iters, char* variant, int cap, int* block, double* ms_per_iter);

/* Residual without device allocation.  No counterpart in the reference.
 * For callers that cannot let a library allocate device memory: a structural
 * or coupling code that owns all device memory through its own pool sized at
 * start-up (a library-side cudaMalloc/cudaFree would synchronise the whole
 * device and break that code's stream overlap, and could fail once the pool
 * holds the memory).  Same result as afx_residual (bit for bit) for the state
 * q_dev, but q_dev and R_dev are the caller's DEVICE arrays of 4*n_real
 * doubles in reference cell order, and the scratch lives in a fixed 24 MiB
 * device array inside the library: at most 262,144 cells and 524,288 faces
 * (larger meshes return AFX_ERR_ARG).  FP64 solvers only.
 * Ordering: the call reads q_dev on the solver's own stream, which is not
 * ordered after the caller's streams, so q_dev must be complete on the
 * device when the call is made (the caller synchronises the stream that
 * wrote it).  The call synchronises the solver's stream before it returns,
 * so R_dev is complete on return.
 * The solver's state is not changed; its gradient/limiter buffers are
 * overwritten as afx_residual does (a pending last-stage qW is formed first).
 * Calls share the fixed array, so calls that overlap on the GPU (two host
 * threads, two solvers) race: the caller serialises them.  On each device,
 * the first call looks up the array's device address with that device
 * current. */
int afx_residual_noalloc(afx_solver s, const double* q_dev, double* R_dev, long long n);

/* Grid sequencing: multigrid::run's transfer between levels (multigrid.h:
 * 316-321 with the mapper of gen_mapper, multigrid.h:99-178).  The fine
 * solver's state becomes mapper * the coarse state (ghost cells taking their
 * owner's state, bcs_from_internal, solver.h:276-287), and its ghost states
 * are refilled from its boundary conditions.  The mapper weights every coarse
 * cell j (ghosts included) within d^2 < 2 A_j of a fine cell by
 * 1/max(0.1 sqrt(A_j), d), normalised.  Both solvers on the same device. */
int afx_prolongate(afx_solver coarse, afx_solver fine);

/* mesh::compute_wall_dist (mesh.h:794-830) on the GPU with the solver's
 * boundary conditions: for every cell (real then ghost, reference order) the
 * least distance from its centroid to the centre of a wall or slip-wall
 * boundary edge; 1 when the mesh has none.  n = n_real_cells +
 * n_boundary_edges.  (The reference computes it for its Spalart-Allmaras
 * model, which it does not implement.) */
int afx_wall_distance(afx_solver s, double* out, long long n);

/* Implicit solver (settings solver = "implicit"): Krylov (GMRES)
 * iterations of the last implicit iteration, over its first solve and its
 * rhs_iterations chord solves (solver.h:1170-1213).  0 for the explicit
 * solver.  No counterpart in the reference (Eigen's iterations() is only
 * printed under RANS_DEBUG). */
int afx_linear_iterations(afx_solver s, int* n);
/* ---- Output.  Replaces rans::save (post.h:58-180): the ASCII VTU file,
 * byte for byte as the reference writes it (node coordinates, real cells as
 * VTK triangles 5 / quads 9, and per cell the wall distance, Mach, density,
 * pressure, temperature and velocity of solution, core.h:119-164). */
/* A host state q (4*n_real doubles, reference order) on mesh m; wall_dist:
 * n_real doubles or NULL (zeros: a mesh whose compute_wall_dist has not run);
 * gamma, R: the gas. */
int afx_write_vtu(afx_mesh m, const double* q, const double* wall_dist, long long n, double gamma, double R,
                  const char* path);
/* The solver's state on its (possibly deformed) mesh, with the wall distance
 * of its wall / slip-wall patches (mesh.h:794-830, as multigrid.h:71 forms
 * it before a run) and its gas. */
int afx_save_vtu(afx_solver s, const char* path);


/* ---- Adjoint of the FP64 residual.  No counterpart in the reference (it
 * has no adjoint).  R(q) is the residual afx_residual returns (first-stage
 * semantics: gradients and limiter formed from q, solver.h:745-799); bq are
 * the boundary states of the boundary edges (core.h:73-83 for farfield
 * patches).  Inviscid or laminar flux; first or second order; Green-Gauss
 * gradient; Venkatakrishnan or Michalak limiter (the derivative of the
 * active branch: min/max and limiter cases follow the state).  FP64 solvers
 * only (AFX_ERR_CONFIG otherwise).
 *
 * u = (dR/dq)^T v and, if bq_bar != NULL, bq_bar = (dR/dbq)^T v (4 per
 * boundary edge, boundary order).  q: the state to linearise about, or NULL
 * for the solver's state (the solver's state is not changed either way).
 * q, v, u: 4*n_real doubles in reference cell order, host or device. */
int afx_residual_vjp(afx_solver s, const double* q, const double* v, double* u, double* bq_bar, long long n);
/* Boundary states bq (4 per boundary edge, conservative variables). */
int afx_boundary_states(afx_solver s, double* bq, long long n);
/* Sensitivities of a force coefficient J ("cl" or "cd" over `patch`,
 * post.h:301-387) at the solver's (converged) state: solves
 * (dR/dq)^T lam = -(dJ/dq)^T until ||(dR/dq)^T lam + dJ/dq|| falls below
 * tol * ||dJ/dq|| (tol <= 0: 1e-10) or max_it iterations (<= 0: 100000).
 * An explicit solver iterates in pseudo-time with its own local time step
 * and three stages.  An implicit solver solves it by flexible GMRES
 * (restarts every 60 steps) on the exact transposed Jacobian (the vJP),
 * preconditioned by its own linear solve with its matrix at max_cfl and the
 * converged state, transposed with its ILU(0) factors (M^T d = v, then
 * -A .* d); iterations = Krylov steps, and the solve starts from the last
 * solution of the same objective on this solver.  dJ[0] = dJ/d(angle) per radian of the farfield angle,
 * dJ[1] = dJ/d(Mach), both for every farfield-type boundary together.
 * iters, res: iterations run and the final relative adjoint residual. */
int afx_adjoint_solve(afx_solver s, const char* patch, const char* objective, double tol, int max_it, double* dJ,
                      int* iters, double* res);
/* The adjoint state lam of the last afx_adjoint_solve (reference order). */
int afx_adjoint_state(afx_solver s, double* lam, long long n);

/* ---- Shape deformation and surface sensitivities.  No counterpart in the
 * reference.  A boundary patch (e.g. "wall") deforms by a normal
 * displacement a_k of each of its nodes (unit normals of the undeformed mesh:
 * the mean of the adjacent patch-edge normals, pointing out of the flow
 * domain); every other node moves by inverse-distance weighting
 * (weights d^-power) of the patch displacements, with the nodes of the other
 * boundary patches held fixed.  Displacements are relative to the
 * undeformed mesh (a = 0 restores it); the state is kept. */
/* The patch's nodes (ascending node index) and their unit normals. */
int afx_patch_nodes(afx_solver s, const char* patch, long long* ids, double* nx, double* ny, int cap, int* n);
/* Deform: n == number of patch nodes; power <= 0: 2. */
int afx_deform_patch(afx_solver s, const char* patch, const double* a, int n, double power);
/* dJ/da_k for every patch node k, J the objective of the last
 * afx_adjoint_solve on the same patch (call it first, at the converged
 * state): dJ/da_k = dJ/da_k|_q + lam . dR/da_k|_q, the geometric partials by
 * central differences of the residual and the forces with step h
 * (h <= 0: 1e-7), no re-convergence.  FP64 solvers. */
int afx_adjoint_patch(afx_solver s, const char* patch, const char* objective, double power, double h, double* dJ,
                      int n);
/* The same derivative along n_dirs directions at once: dJ[j] = dJ/dt of
 * a = a0 + t * dirs[j*n_patch .. (j+1)*n_patch), each by one central
 * difference (two residual evaluations per direction, not per node).  A
 * structural model with fewer degrees of freedom than patch nodes takes its
 * gradient this way (the directions are its modes' surface displacements).
 * n_patch must equal the number of patch nodes. */
int afx_adjoint_patch_dirs(afx_solver s, const char* patch, const char* objective, double power, double h,
                           const double* dirs, int n_dirs, int n_patch, double* dJ);
/* Displacement vectors instead of normal displacements: patch node k moves
 * by (dx[k], dy[k]), the volume by the same inverse-distance weights (a
 * structural model moving the wall along its own axes, e.g. a beam's
 * deflection), and the adjoint derivative along such directions, each row
 * of dirs holding (dx_k, dy_k) for every patch node (2 n_patch entries). */
int afx_deform_patch_xy(afx_solver s, const char* patch, const double* dx, const double* dy, int n, double power);
int afx_adjoint_patch_dirs_xy(afx_solver s, const char* patch, const char* objective, double power, double h,
                              const double* dirs, int n_dirs, int n_patch, double* dJ);

/* ---- Batched load cases.  No single counterpart in the reference: its
 * polar sweep runs one case after another (src/rans/include/rans/rans.h:
 * 92-105 loops over the angles, multigrid.h:183-234 run_solver per case).  A
 * batch advances many independent cases -- each with its own mesh, angle,
 * Mach and farfield -- in one launch per kernel, one device solver over the
 * union of the meshes.  Every case follows the reference's run_solver logic
 * on its own (err_0, err/err_0 < tol, max iterations, history every 10th
 * iteration); a case that stops holds its state while the others go on.
 * In FP64 each case's state, iteration count and history are bit-identical
 * to a single afx_solver on that case alone (norms: same to ~1e-15).
 *
 * All configs must share the scheme (gamma, R, mu, Pr, viscosity, gradient,
 * limiter, precision, second_order, start_cfl, relaxation, limiter_k); the
 * boundary conditions come from each case's own config, keyed by the case
 * mesh's patch names.  Launch settings (kernel_variant, block_size) are case
 * 0's.  fp64_correction_interval and fp64_finish are single-case options. */
int afx_batch_create(int n_cases, const afx_mesh* meshes, const afx_config* configs, afx_batch* out);
void afx_batch_free(afx_batch b);
int afx_batch_counts(afx_batch b, int* n_cases, long long* n_cells_total);
/* init() (solver.h:615-631) of every case with its own freestream. */
int afx_batch_init_freestream(afx_batch b);
/* State of case c in the case mesh's reference cell order (4*n_real doubles). */
int afx_batch_set_state(afx_batch b, int c, const double* q, long long n);
int afx_batch_get_state(afx_batch b, int c, double* q, long long n);
/* n iterations of every case; res_norms[c] = ||qW||_2 of case c's last
 * stage (may be NULL).  AFX_ERR_NONFINITE if any case's norm is not finite
 * (that case stops where it went non-finite; the others complete). */
int afx_batch_iterate(afx_batch b, int n_iters, double* res_norms);
/* run_solver of every case at once; per case: iterations, final err/err_0
 * and status (AFX_OK or AFX_ERR_NONFINITE).  tol <= 0 / max_it <= 0: case
 * 0's config values.  Returns when every case has stopped. */
int afx_batch_run_to_convergence(afx_batch b, double tol, int max_it, int* iters, double* errs, int* status);
/* err/err_0 every 10th iteration of case c's last run (up to 4096 entries). */
int afx_batch_case_history(afx_batch b, int c, double* out, int cap, int* n);
/* get_wall_profile (post.h:301-387) of case c over its patch `patch`. */
int afx_batch_forces(afx_batch b, int c, const char* patch, double* cl, double* cd, double* cm);
/* rans.h:92-98 for case c: new farfield conditions, state kept. */
int afx_batch_set_farfield(afx_batch b, int c, const char* patch, double mach, double angle, double T, double p);
/* afx_autotune over the whole batch (state and qW put back). */
int afx_batch_autotune(afx_batch b, int iters, char* variant, int cap, int* block, double* ms_per_iter);
int afx_batch_last_device_seconds(afx_batch b, double* sec);
/* Krylov iterations of each case in the last implicit iteration (0 for the
 * explicit solver); iters holds n_cases entries. */
int afx_batch_linear_iterations(afx_batch b, int* iters, int n_cases);

#ifdef __cplusplus
}
#endif

#endif /* AFX_RANS_H */
