"""Config 5: adjoint sensitivities on the hybrid boundary-layer mesh and the
aeroelastic coupling they drive (aeroflex_gb300/coupling.py).

- CPU: the beam against the closed-form cantilever, the load-vector size
  rule of set_Load_Vector_From_Vector (model.hpp:94-100), the rank-one
  Newton update against a dense solve, the loads' wall-face geometry
  against the library's metrics of the deflected wall, and the C++ beam
  (include/afx_coupling.hpp) against this one.
- GPU, the config 2 generator at 8k cells (Euler, first order, M 0.15,
  AoA 10 deg, implicit solver then its Newton-Krylov finish to 3e-12,
  just above the round-off floor of the right-hand side's norm there):
  dC_L/dalpha, dC_D/dalpha and the normal-displacement gradients of C_L
  and C_D along 16 random unit directions (seed 3) against central
  differences of converged solutions (steps 2e-5 and 1e-5: at the
  converged objectives' round-off floor, ~5e-13, a step of 1e-7 leaves
  the difference uncertain by ~1e-4 relative), 1e-6 relative plus the two
  steps' disagreement taken twice (the disagreement is itself a noisy
  estimate of the difference's error); then 5 coupling iterations with the
  50-element beam (EI = 1e4 N m^2) at sea-level dynamic pressure.
- GPU, config 2's full 201k-cell mesh: the vJP kernel against central
  differences (step 1e-7) along 16 random unit directions (seed 3).
"""
import math

import numpy as np
import pytest

from aeroflex_gb300 import coupling, meshgen

MACH, AOA = 0.15, 10.0 * math.pi / 180


def test_beam_matches_the_cantilever_formulas():
    EI, L = 1e4, 1.0
    b = coupling.Beam(50, EI, L)
    # uniform load q = 1 N/m as consistent nodal loads (midpoint rule, fine)
    xs = (np.arange(40000) + 0.5) / 40000 * L
    F = b.shape_matrix(xs).T @ np.full(xs.size, L / xs.size)
    u = b.solve(F)
    assert abs(u[-2] - L ** 4 / (8 * EI)) <= 1e-9 * L ** 4 / (8 * EI) + 1e-15
    assert abs(u[-1] - L ** 3 / (6 * EI)) <= 1e-9 * L ** 3 / (6 * EI) + 1e-15
    x = b.xn
    w = x * x * (6 * L * L - 4 * L * x + x * x) / (24 * EI)
    np.testing.assert_allclose(u[0::2], w, rtol=1e-8, atol=1e-15)
    # tip force P
    F = np.zeros(b.n_dof)
    F[-2] = 3.0
    u = b.solve(F)
    assert abs(u[-2] - 3.0 * L ** 3 / (3 * EI)) <= 1e-12
    assert abs(u[-1] - 3.0 * L ** 2 / (2 * EI)) <= 1e-12
    # the clamp holds whatever the load there
    F[:2] = 5.0
    assert np.all(b.solve(F)[:2] == 0)


def test_load_vector_of_another_size_is_ignored():
    b = coupling.Beam(10)
    f = np.arange(b.n_dof, dtype=float)
    assert b.set_load_vector_from_vector(f)
    assert not b.set_load_vector_from_vector(np.ones(b.n_dof + 2))
    np.testing.assert_array_equal(b.forces, f)


def test_rank_one_newton_solves_the_linearised_beam():
    b = coupling.Beam(20, 3e3)
    rng = np.random.default_rng(1)
    F = rng.standard_normal(b.n_dof)
    s = rng.standard_normal(b.n_dof)
    g = 1e-4 * rng.standard_normal(b.n_dof)
    g[b.clamped] = 0
    u = 1e-3 * rng.standard_normal(b.n_dof)
    u[b.clamped] = 0
    x = coupling.rank_one_newton(b, F, s, g, u)
    A = b.K_final - np.outer(b.apply_spc(s), g)
    want = np.linalg.solve(A, b.apply_spc(F - s * (g @ u)))
    np.testing.assert_allclose(x, want, rtol=1e-10, atol=1e-14)


def test_coupling_wall_faces_are_the_mesh_metrics_of_the_deflected_wall(afx):
    # the loads' face geometry for a deflected wall equals the metrics the
    # library forms for those node positions (order, normals into the body,
    # lengths, centres); host code only
    m = _small_mesh()
    M = afx.mesh.from_arrays(m)
    names = M.boundary_names()
    be = M.get_int("boundary_edges")
    wall = np.array([n == "wall" for n in names])
    ids = np.unique(M.get_int("edges_nodes").reshape(-1, 2)[be[wall]].ravel())

    class Patch:  # the node list a solver's afx_patch_nodes returns
        def patch_nodes(self, patch):
            return ids, np.zeros(len(ids)), np.ones(len(ids))

    beam = coupling.Beam(50, 1e4)
    cpl = coupling.Coupling(Patch(), M, m, beam, 1000.0)
    u = np.zeros(beam.n_dof)
    u[0::2] = 3e-4 * beam.xn ** 2  # 0.3 mm at the trailing edge: no cell of the first layer inverts
    a = cpl.surface_displacement(u)
    xc, nx, ny, L = cpl.wall_faces(a)
    y = np.array(m["y"], np.float64)
    y[ids] += a
    M2 = afx.mesh.from_arrays(dict(m, y=y))
    e = be[wall]
    for got, key in ((xc, "ex"), (nx, "nx"), (ny, "ny"), (L, "L")):
        np.testing.assert_allclose(got, M2.get(key)[e], rtol=0, atol=1e-15)


def test_cpp_beam_matches_the_python_beam(afx, tmp_path):
    # include/afx_coupling.hpp's beam (dense LU) against coupling.Beam
    # (numpy), and the whole header, coupling loop included, compiles and
    # links against the library
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "beam_coupling")
    lib = os.path.dirname(afx.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(root, "include"),
                           os.path.join(root, "aeroflex_gb300", "cpp", "beam_coupling.cpp"), "-o", exe,
                           "-L", lib, "-lafx_rans", "-Wl,-rpath," + lib])
    out = subprocess.run([exe, "beam"], capture_output=True, text=True, check=True).stdout.split("\n")
    uniform, tip = (np.array(list(map(float, l.split()))) for l in out[:2])
    b = coupling.Beam(50, 1e4, 1.0)
    xs = (np.arange(40000) + 0.5) / 40000
    F = b.shape_matrix(xs).T @ np.full(xs.size, 1.0 / xs.size)
    # two LU factorisations of a stiffness whose entries span 1 (the
    # clamped rows) to 1.25e9 (EI/L_e^3), and loads summed in another order:
    # they agree to ~1e-10, not to the last bit
    np.testing.assert_allclose(uniform, b.solve(F), rtol=1e-9, atol=1e-20)
    P = np.zeros(b.n_dof)
    P[-2] = 3.0
    np.testing.assert_allclose(tip, b.solve(P), rtol=1e-9, atol=1e-20)


def _small_mesh():
    return meshgen.hybrid_airfoil(n_surf=128, bl_layers=16, first=1e-3, growth=1.2, r_far=20.0, fill_cells=6000)


def _solver(afx, M, angle=AOA):
    st = afx.Settings().set("solver", "implicit").set("precision", "fp64").set("viscosity", "inviscid")
    st.set("second_order", 0.0).set("start_cfl", 10.0).set("slope_cfl", 20.0).set("max_cfl", 200.0)
    st.set_bc("farfield", "farfield", 1.0, MACH, angle, 1.0).set_bc("wall", "slip-wall")
    g = afx.Solver(M, st)
    g.init()
    return g


def _converge(g, tol=3e-12):
    g.run_solver(1e-6, 2000)
    nn, nk, err = g.newton_solve(tol, 30)
    assert err <= tol, (nn, nk, err)
    return err


@pytest.mark.gpu
def test_newton_finish_reaches_the_implicit_iteration_s_solution(afx):
    # an O-mesh the implicit iteration itself converges to 1e-12: the
    # Newton finish from its 1e-6 state lands on the same solution, in a
    # few steps that each take the full Newton step
    m = meshgen.airfoil_omesh(32, 24, split=False, m=0.02, p=0.4, t=0.12)
    M = afx.mesh.from_arrays(m)
    a = _solver(afx, M)
    it, err = a.run_solver(1e-12, 3000)
    assert err <= 1e-12, (it, err)
    b = _solver(afx, M)
    _converge(b)
    assert len(b.newton_record) <= 6 and b.newton_record[0, 1] == 1.0, b.newton_record
    fa, fb = afx.get_wall_profile(a), afx.get_wall_profile(b)
    for k in ("cl", "cd", "cm"):
        assert abs(fa[k] - fb[k]) <= 1e-10, (k, fa[k], fb[k])
    # and the hybrid mesh, where the implicit iteration alone stalls
    g = _solver(afx, afx.mesh.from_arrays(_small_mesh()))
    _converge(g)


def _fd(afx, g, deform, objectives, steps=(1e-7, 1e-6)):
    """Central differences of converged objectives for deform(t): (mean of
    the two steps, their disagreement) per objective."""
    out = {o: [] for o in objectives}
    for h in steps:
        v = {}
        for sg in (1, -1):
            deform(sg * h)
            _converge(g)
            v[sg] = afx.get_wall_profile(g)
        for o in objectives:
            out[o].append((v[1][o] - v[-1][o]) / (2 * h))
    return {o: (0.5 * (d[0] + d[1]), abs(d[0] - d[1])) for o, d in out.items()}


@pytest.mark.gpu
def test_config5_gradients_match_converged_differences(afx):
    m = _small_mesh()
    M = afx.mesh.from_arrays(m)
    g = _solver(afx, M)
    _converge(g)
    ids, nx, ny = g.patch_nodes("wall")
    assert len(ids) == 128
    rng = np.random.default_rng(3)
    D = rng.standard_normal((16, len(ids)))
    D /= np.linalg.norm(D, axis=1)[:, None]
    grad, dalpha = {}, {}
    for obj in ("cl", "cd"):
        (da, dm), it, res = g.adjoint_solve("wall", obj, tol=1e-12, max_it=600)
        assert res <= 1e-12, (obj, it, res)
        dalpha[obj] = da
        grad[obj] = g.adjoint_patch_dirs(D, "wall", obj)

    def angle(t):
        g.set_farfield("farfield", MACH, AOA + t)

    fd = _fd(afx, g, angle, ("cl", "cd"), steps=(1e-5, 2e-5))
    angle(0.0)
    for obj in ("cl", "cd"):
        ref, unc = fd[obj]
        assert abs(dalpha[obj] - ref) <= 1e-6 * abs(ref) + 2 * unc + 1e-9, (obj, dalpha[obj], ref, unc)
    for j in range(16):
        fd = _fd(afx, g, lambda t: g.deform_patch(t * D[j], "wall"), ("cl", "cd"), steps=(2e-5, 1e-5))
        for obj in ("cl", "cd"):
            ref, unc = fd[obj]
            assert abs(grad[obj][j] - ref) <= 1e-6 * abs(ref) + 2 * unc + 1e-9, (j, obj, grad[obj][j], ref, unc)


@pytest.mark.gpu
def test_config5_coupling_iterations(afx):
    m = _small_mesh()
    M = afx.mesh.from_arrays(m)
    g = _solver(afx, M)
    _converge(g)
    beam = coupling.Beam(50, 1e4)
    cpl = coupling.Coupling(g, M, m, beam, coupling.sea_level_dynamic_pressure(MACH), tol=3e-12)
    hist, final = cpl.run(AOA, 5)
    assert len(hist) == 5
    for e in hist:
        # the loads' face sums are the solver's force integration
        assert abs(e["cy"] - e["cy_solver"]) <= 1e-12 * abs(e["cy_solver"]), e
        assert e["flow_residual"] <= 3e-12
        assert e["adjoint_cl"]["residual"] <= 1e-12 and e["adjoint_cd"]["residual"] <= 1e-12
    # the wing section bends up and the lift falls (trailing edge up)
    assert 1e-4 < final["tip_deflection_m"] < 5e-2, final
    assert final["cl"] < hist[0]["cl"]
    # Newton: the steps shrink fast, and each step's predicted lift and drag
    # changes (adjoint gradients) match the next solve's to first order
    steps = [e["step_norm_m"] for e in hist]
    assert steps[-1] <= 1e-3 * steps[0], steps
    cls = [e["cl"] for e in hist] + [final["cl"]]
    cds = [e["cd"] for e in hist] + [final["cd"]]
    for k in range(5):
        dcl, dcd = cls[k + 1] - cls[k], cds[k + 1] - cds[k]
        assert abs(hist[k]["dcl_pred"] - dcl) <= 0.05 * abs(dcl) + 1e-9, (k, hist[k]["dcl_pred"], dcl)
        assert abs(hist[k]["dcd_pred"] - dcd) <= 0.05 * abs(dcd) + 1e-9, (k, hist[k]["dcd_pred"], dcd)


@pytest.mark.gpu
def test_config5_vjp_on_the_full_mesh(afx):
    m = meshgen.hybrid_airfoil()
    M = afx.mesh.from_arrays(m)
    assert M.nRealCells > 190000
    st = afx.Settings().set("solver", "explicit").set("precision", "fp64").set("viscosity", "inviscid")
    st.set("second_order", 0.0).set("start_cfl", 1.0)
    st.set_bc("farfield", "farfield", 1.0, MACH, AOA, 1.0).set_bc("wall", "slip-wall")
    g = afx.Solver(M, st)
    g.init()
    g.iterate(20)
    rng = np.random.default_rng(3)
    q = g.get_q()
    q = q * (1 + 1e-3 * rng.standard_normal(q.size))  # generic: no ties
    v = rng.standard_normal(q.size)
    u, _ = g.residual_vjp(v, q=q)
    for j in range(16):
        e = rng.standard_normal(q.size)
        e /= np.linalg.norm(e)
        d = []
        for h in (1e-7, 1e-6):
            g.set_q(q + h * e)
            Rp = g.residual()
            g.set_q(q - h * e)
            Rm = g.residual()
            d.append(float(v @ (Rp - Rm)) / (2 * h))
        lhs = float(u @ e)
        unc = abs(d[0] - d[1])
        assert abs(lhs - d[0]) <= 1e-6 * abs(d[0]) + unc, (j, lhs, d)
