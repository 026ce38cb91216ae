"""Batched load cases (afx_batch_*) against the oracle, case by case.

A batch is one device solver over the union of the cases' meshes; each case
must behave exactly as the reference's solver on that case alone: FP64
states, iteration counts and convergence histories bit-identical (norms are
sums in another order: relative 1e-12), forces to 1e-12.
"""
import numpy as np
import pytest

from tests.cases import DEG, batch_cases, gpu_settings, gpu_solver, oracle_solver, rel_l2

pytestmark = pytest.mark.gpu


def _batch(afx, cases, precision="fp64", **st):
    meshes = [afx.mesh.from_arrays(m) for m, _ in cases]
    sets = [gpu_settings(afx, bcs, precision, **dict(st)) for _, bcs in cases]
    return afx.Batch(meshes, sets)


@pytest.mark.parametrize("kv", ["face", "tile", "gather"])
def test_batch_iterations_bitexact(afx, orc, kv):
    cases = batch_cases()
    b = _batch(afx, cases, kernel_variant=kv)
    b.init()
    refs = []
    for m, bcs in cases:
        so = oracle_solver(orc, m, bcs)
        so.init()
        refs.append(so)
    for c, so in enumerate(refs):
        np.testing.assert_array_equal(b.get_q(c), so.q())
    norms = b.iterate(7)
    for c, so in enumerate(refs):
        no = so.iterate(7)
        np.testing.assert_array_equal(b.get_q(c), so.q())
        assert abs(norms[c] - no[-1]) <= 1e-12 * no[-1]


def test_batch_run_solver_matches_each_case(afx, orc):
    cases = batch_cases()
    # three cases converge (at 139, 161 and 430 iterations), the channel
    # stops at the iteration limit
    st = dict(tolerance=3e-2, max_iterations=600)
    b = _batch(afx, cases, **st)
    b.init()
    it_b, err_b, status = b.run_solver()
    assert (status == 0).all()
    iters = []
    for c, (m, bcs) in enumerate(cases):
        so = oracle_solver(orc, m, bcs, **st)
        so.init()
        it_o, err_o, hist_o = so.run_solver()
        assert it_b[c] == it_o, (c, it_b[c], it_o)
        assert abs(err_b[c] - err_o) <= 1e-10 * abs(err_o)
        np.testing.assert_allclose(b.history(c), hist_o, rtol=1e-10)
        np.testing.assert_array_equal(b.get_q(c), so.q())
        wo = so.wall_profile("wall")
        fb = b.forces(c, "wall")
        for k in ("cl", "cd", "cm"):
            assert abs(fb[k] - wo[k]) <= 1e-12 * max(abs(wo[k]), 1e-12), (c, k, fb[k], wo[k])
        iters.append(it_o)
    # the cases stop at different iterations: early ones held their state
    assert len(set(iters)) > 1


def test_batch_warm_restart_one_case(afx, orc):
    # rans.h:92-98 on one case of the batch: new angle, state kept, err_0 of
    # the next run includes that case's last-stage qW (solver.h:643-649)
    cases = batch_cases()[:3]
    st = dict(tolerance=1e-2, max_iterations=300)
    b = _batch(afx, cases, **st)
    b.init()
    b.run_solver()
    refs = []
    for m, bcs in cases:
        so = oracle_solver(orc, m, bcs, **st)
        so.init()
        so.run_solver()
        refs.append(so)
    b.set_farfield(1, "farfield", 0.35, 6.0 * DEG)
    refs[1].set_farfield("farfield", 0.35, 6.0 * DEG)
    it_b, err_b, _ = b.run_solver()
    for c, so in enumerate(refs):
        it_o, err_o, _ = so.run_solver()
        assert it_b[c] == it_o, (c, it_b[c], it_o)
        assert abs(err_b[c] - err_o) <= 1e-10 * abs(err_o)
        np.testing.assert_array_equal(b.get_q(c), so.q())


def test_batch_set_state_roundtrip(afx, orc):
    cases = batch_cases()
    b = _batch(afx, cases)
    b.init()
    rng = np.random.default_rng(3)
    qs = [b.get_q(c) * (1 + 1e-3 * rng.standard_normal(4 * b.n_real[c])) for c in range(len(cases))]
    for c in (2, 0, 3, 1):
        b.set_q(c, qs[c])
    for c in range(len(cases)):
        np.testing.assert_array_equal(b.get_q(c), qs[c])
    b.iterate(2)
    for c, (m, bcs) in enumerate(cases):
        so = oracle_solver(orc, m, bcs)
        so.init()
        so.set_q(qs[c])
        so.iterate(2)
        np.testing.assert_array_equal(b.get_q(c), so.q())


def test_batch_fp32_mixed_equals_single_case_solvers(afx):
    # the FP32-mixed batch runs the same per-cell arithmetic as a single
    # FP32-mixed solver on each case with the same kernel variant
    cases = batch_cases()
    b = _batch(afx, cases, "fp32-mixed", kernel_variant="tile", block_size=128)
    b.init()
    b.iterate(20)
    for c, (m, bcs) in enumerate(cases):
        g = gpu_solver(afx, m, bcs, "fp32-mixed", kernel_variant="tile", block_size=128)
        g.init()
        g.iterate(20)
        assert rel_l2(b.get_q(c), g.get_q()) < 1e-12


def test_batch_autotune_keeps_results(afx, orc):
    cases = batch_cases()
    b = _batch(afx, cases)
    b.init()
    b.iterate(3)
    t = b.autotune(2)
    assert t["variant"] in ("gather", "face", "tile") and t["ms_per_iter"] > 0
    b.iterate(2)
    for c, (m, bcs) in enumerate(cases):
        so = oracle_solver(orc, m, bcs)
        so.init()
        so.iterate(5)
        np.testing.assert_array_equal(b.get_q(c), so.q())


def test_batch_rejects_mixed_schemes(afx):
    cases = batch_cases()[:2]
    meshes = [afx.mesh.from_arrays(m) for m, _ in cases]
    sets = [gpu_settings(afx, cases[0][1]), gpu_settings(afx, cases[1][1], limiter="michalak")]
    with pytest.raises(afx.AfxError) as ei:
        afx.Batch(meshes, sets)
    assert ei.value.code == 2


@pytest.mark.parametrize("precision", ["fp64", "fp32-mixed"])
def test_batch_implicit_polar_converges_per_case(afx, precision):
    # an implicit batch (FP32-mixed: FP32 Jacobians and Krylov vectors, FP64
    # right-hand side) reaches each case's FP64 fixed point: converged C_L /
    # C_D of every case within 1e-8 of the same case solved alone in FP64
    from aeroflex_gb300 import meshgen
    imp = dict(solver="implicit", start_cfl=40.0, slope_cfl=50.0, max_cfl=100.0)
    cases = []
    for ns, nr, mach, aoa, kw in [(32, 24, 0.5, 1.25, {}), (40, 20, 0.3, 4.0, dict(m=0.04)),
                                  (24, 24, 0.6, -2.0, dict(t=0.15))]:
        m = meshgen.airfoil_omesh(ns, nr, split=False, **kw)
        bcs = {"farfield": dict(type="farfield", T=1.0, mach=mach, angle=aoa * DEG, p=1.0),
               "wall": dict(type="slip-wall")}
        cases.append((m, bcs))
    b = _batch(afx, cases, precision, **imp)
    b.init()
    it, err, st = b.run_solver(1e-11, 300)
    assert (st == 0).all() and (err <= 1e-11).all(), (it, err)
    for c, (m, bcs) in enumerate(cases):
        g = gpu_solver(afx, m, bcs, "fp64", **imp)
        g.init()
        g.run_solver(1e-11, 300)
        wg = afx.get_wall_profile(g, "wall")
        fb = b.forces(c, "wall")
        for k in ("cl", "cd"):
            assert abs(fb[k] - wg[k]) <= 1e-8 * max(abs(wg[k]), 1e-3), (c, k, fb[k], wg[k])


def test_batch_implicit_isolates_a_failed_case(afx):
    # a case whose state is not finite stops with status NONFINITE; the other
    # cases of the implicit batch still reach their own fixed points
    from aeroflex_gb300 import meshgen
    imp = dict(solver="implicit", start_cfl=40.0, slope_cfl=50.0, max_cfl=100.0)
    cases = []
    for ns, nr, mach, aoa in [(32, 24, 0.5, 1.25), (24, 16, 0.4, 3.0), (40, 20, 0.3, -1.0)]:
        m = meshgen.airfoil_omesh(ns, nr, split=False)
        bcs = {"farfield": dict(type="farfield", T=1.0, mach=mach, angle=aoa * DEG, p=1.0),
               "wall": dict(type="slip-wall")}
        cases.append((m, bcs))
    b = _batch(afx, cases, "fp32-mixed", **imp)
    b.init()
    q = b.get_q(1)
    q[::4] = np.nan
    b.set_q(1, q)
    it, err, st = b.run_solver(1e-11, 300)
    assert st[1] == 4 and st[0] == 0 and st[2] == 0, (it, err, st)
    for c in (0, 2):
        m, bcs = cases[c]
        g = gpu_solver(afx, m, bcs, "fp64", **imp)
        g.init()
        g.run_solver(1e-11, 300)
        wg = afx.get_wall_profile(g, "wall")
        fb = b.forces(c, "wall")
        assert abs(fb["cl"] - wg["cl"]) <= 1e-8 * max(abs(wg["cl"]), 1e-3), (c, fb, wg)
