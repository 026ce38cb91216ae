"""Implicit solver (settings.solver = "implicit"): the reference's
implicitSolver + run_solver loop on the GPU.  Its iterates are not pinned
(the reference's own trajectory depends on Eigen's ILUT + GMRES), so the
checks are on the fixed point: it must converge to the same R(q) = 0 as the
explicit path, whose residual is bit-exact to the oracle -- converged C_L /
C_D within 1e-8 relative, state within 1e-8 -- in far fewer iterations, in
FP64 and in FP32-mixed (FP32 Jacobian and Krylov vectors, FP64 residual)."""
import numpy as np
import pytest

from aeroflex_gb300 import meshgen
from tests.cases import DEG, gpu_solver, rel_l2

pytestmark = pytest.mark.gpu

BCS = {"farfield": dict(type="farfield", T=1.0, mach=0.5, angle=1.25 * DEG, p=1.0), "wall": dict(type="slip-wall")}


def _explicit_reference(afx, m):
    g = gpu_solver(afx, m, BCS, cfl=1.5)
    g.init()
    g.run_solver(1e-12, 300000)
    return g


@pytest.mark.parametrize("precision", ["fp64", "fp32-mixed"])
def test_implicit_reaches_the_explicit_fixed_point(afx, precision):
    from aeroflex_gb300.rans import get_wall_profile
    m = meshgen.airfoil_omesh(32, 32, split=False)
    ge = _explicit_reference(afx, m)
    we = get_wall_profile(ge, "wall")
    gi = gpu_solver(afx, m, BCS, precision, solver="implicit", start_cfl=40.0, slope_cfl=50.0, max_cfl=100.0)
    gi.init()
    it, err = gi.run_solver(1e-12, 300)
    assert err <= 1e-12, (it, err)
    assert it < 300
    wi = get_wall_profile(gi, "wall")
    for k in ("cl", "cd"):
        assert abs(wi[k] - we[k]) <= 1e-8 * max(abs(we[k]), 1e-3), (k, wi[k], we[k])
    assert rel_l2(gi.get_q(), ge.get_q()) < 1e-8
    h = gi.history()
    assert len(h) == it and h[-1] == pytest.approx(err)


def test_implicit_iterate_and_stop_semantics(afx):
    m = meshgen.airfoil_omesh(24, 16, split=False)
    g = gpu_solver(afx, m, BCS, solver="implicit", start_cfl=40.0)
    g.init()
    r1 = g.iterate(3)
    r2 = g.iterate(3)
    assert np.isfinite(r1) and np.isfinite(r2) and r2 < r1


@pytest.mark.parametrize("precision", ["fp64", "fp32-mixed"])
def test_krylov_host_loop_equals_the_solve_graph(afx, precision):
    # krylov_graph = 0 drives the same kernels from a host loop: same Krylov
    # iterations, bit-identical states
    m = meshgen.airfoil_omesh(32, 24, split=False)
    out = []
    for graph in (1, 0):
        g = gpu_solver(afx, m, BCS, precision, solver="implicit", start_cfl=40.0, krylov_graph=graph)
        g.init()
        g.iterate(3)
        out.append((g.get_q(), g.linear_iterations()))
    assert out[0][1] == out[1][1] and out[0][1] > 0
    assert np.array_equal(out[0][0], out[1][0])
