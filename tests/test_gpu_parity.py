"""GPU parity: the CUDA path through the C ABI against the CPU oracle on the
same seeded inputs.

FP64: bit-exact (every face flux, gradient, limiter and time step is formed
with the reference's operand order, and per-cell sums visit faces in the
reference's edge order).  Residual norms are sums in a different order:
relative 1e-12.  Forces use a tree reduction: relative 1e-12.
FP32-mixed: tolerances stated per test.
"""
import numpy as np
import pytest

from tests.cases import channel_case, gpu_solver, omesh_case, oracle_solver, rel_l2

pytestmark = pytest.mark.gpu


def _warm_state(orc, m, bcs, n, **st):
    s = oracle_solver(orc, m, bcs, **st)
    s.init()
    s.iterate(n)
    return s


@pytest.mark.parametrize("variant", [
    dict(),
    dict(second_order=False),
    dict(limiter="michalak"),
    dict(viscosity="laminar"),
    dict(viscosity="laminar", second_order=False),
    dict(viscosity="spallart-allmaras"),
    dict(gradient="least-squares"),
    dict(gradient="least-squares", viscosity="laminar"),
])
def test_residual_bitexact_omesh(afx, orc, variant):
    m, bcs = omesh_case(48, 24)
    so = _warm_state(orc, m, bcs, 15, **variant)
    q = so.q()
    Ro = so.residual()
    g = gpu_solver(afx, m, bcs, **variant)
    g.init()
    g.set_q(q)
    Rg = g.residual()
    assert np.isfinite(Rg).all()
    np.testing.assert_array_equal(Rg, Ro)


@pytest.mark.parametrize("kv", ["gather", "face", "tile", "lsq"])
def test_residual_bitexact_shuffled_channel(afx, orc, kv):
    m, bcs, q = channel_case(64, 32)
    extra = dict(gradient="least-squares") if kv == "lsq" else {}
    kv = "face" if kv == "lsq" else kv
    so = oracle_solver(orc, m, bcs, **extra)
    so.init()
    so.set_q(q)
    Ro = so.residual()
    g = gpu_solver(afx, m, bcs, kernel_variant=kv, **extra)
    g.init()
    g.set_q(q)
    np.testing.assert_array_equal(g.residual(), Ro)


@pytest.mark.parametrize("variant", [
    dict(), dict(viscosity="laminar"), dict(second_order=False),
    dict(kernel_variant="gather"), dict(kernel_variant="gather", viscosity="laminar"),
    dict(kernel_variant="face", block_size=64), dict(kernel_variant="gather", block_size=32),
    dict(kernel_variant="tile"), dict(kernel_variant="tile", block_size=64),
    dict(kernel_variant="tile", block_size=256, viscosity="laminar"),
    dict(kernel_variant="tile", second_order=False),
    dict(gradient="least-squares"), dict(gradient="least-squares", kernel_variant="tile"),
    dict(gradient="least-squares", kernel_variant="gather", limiter="michalak"),
])
def test_iterations_bitexact(afx, orc, variant):
    m, bcs = omesh_case(48, 24)
    so = oracle_solver(orc, m, bcs, **variant)
    so.init()
    g = gpu_solver(afx, m, bcs, **variant)
    g.init()
    np.testing.assert_array_equal(g.get_q(), so.q())
    norms = so.iterate(7)
    r = g.iterate(7)
    np.testing.assert_array_equal(g.get_q(), so.q())
    assert abs(r - norms[-1]) <= 1e-12 * norms[-1]
    # an odd count then an even count exercises both state buffers
    so.iterate(2)
    g.iterate(2)
    np.testing.assert_array_equal(g.get_q(), so.q())


@pytest.mark.parametrize("kv", ["face", "tile"])
def test_large_channel_iterations_bitexact(afx, orc, kv):
    m, bcs, q = channel_case(256, 128)
    so = oracle_solver(orc, m, bcs)
    so.init()
    so.set_q(q)
    g = gpu_solver(afx, m, bcs, kernel_variant=kv)
    g.init()
    g.set_q(q)
    so.iterate(3)
    g.iterate(3)
    np.testing.assert_array_equal(g.get_q(), so.q())


def test_run_solver_matches(afx, orc):
    m, bcs = omesh_case(32, 16)
    st = dict(tolerance=1e-3, max_iterations=400)
    so = oracle_solver(orc, m, bcs, **st)
    so.init()
    it_o, err_o, hist_o = so.run_solver()
    g = gpu_solver(afx, m, bcs, **st)
    g.init()
    it_g, err_g = g.run_solver()
    assert it_g == it_o
    assert abs(err_g - err_o) <= 1e-10 * abs(err_o)
    np.testing.assert_allclose(g.history(), hist_o, rtol=1e-10)
    np.testing.assert_array_equal(g.get_q(), so.q())
    # warm restart at a new angle (rans.h:92-98): err_0 of the second run
    # includes the previous run's qW (solver.h:643-649)
    so.set_farfield("farfield", 0.5, 3.0 * 0.01745)
    g.set_farfield("farfield", 0.5, 3.0 * 0.01745)
    it_o2, err_o2, _ = so.run_solver()
    it_g2, err_g2 = g.run_solver()
    assert it_g2 == it_o2
    assert abs(err_g2 - err_o2) <= 1e-10 * abs(err_o2)
    np.testing.assert_array_equal(g.get_q(), so.q())


def test_forces_match(afx, orc):
    m, bcs = omesh_case(48, 24)
    so = _warm_state(orc, m, bcs, 30)
    g = gpu_solver(afx, m, bcs)
    g.init()
    g.set_q(so.q())
    wo = so.wall_profile("wall")
    from aeroflex_gb300.rans import get_wall_profile
    wg = get_wall_profile(g, "wall")
    np.testing.assert_array_equal(wg["cp"], wo["cp"])
    for k in ("cl", "cd", "cm"):
        assert abs(wg[k] - wo[k]) <= 1e-12 * max(abs(wo[k]), 1e-12), (k, wg[k], wo[k])


def test_fp32_mixed_residual_close(afx, orc):
    m, bcs = omesh_case(48, 24)
    so = _warm_state(orc, m, bcs, 15)
    q = so.q()
    Ro = so.residual()
    g = gpu_solver(afx, m, bcs, precision="fp32-mixed")
    g.init()
    g.set_q(q)
    Rg = g.residual()
    # FP32 face fluxes: the residual is a sum of O(1) fluxes cancelling to
    # O(1e-2), so its relative error is ~1e-7 * |F|/|R|.
    assert rel_l2(Rg, Ro) < 2e-3


def test_fp32_mixed_iterations_track_fp64(afx, orc):
    m, bcs = omesh_case(48, 24)
    so = oracle_solver(orc, m, bcs)
    so.init()
    so.iterate(50)
    g = gpu_solver(afx, m, bcs, precision="fp32-mixed")
    g.init()
    g.iterate(50)
    assert rel_l2(g.get_q(), so.q()) < 1e-5


def test_autotune_keeps_state_and_parity(afx, orc):
    m, bcs, q = channel_case(128, 64)
    so = oracle_solver(orc, m, bcs)
    so.init()
    so.set_q(q)
    g = gpu_solver(afx, m, bcs)
    g.init()
    g.set_q(q)
    t = g.autotune(2)
    assert t["variant"] in ("gather", "face") and t["block"] in (64, 128, 256) and t["ms_per_iter"] > 0
    np.testing.assert_array_equal(g.get_q(), q)
    so.iterate(2)
    g.iterate(2)
    np.testing.assert_array_equal(g.get_q(), so.q())


def test_fp32_mixed_variants_agree(afx):
    m, bcs, q = channel_case(128, 64)
    out = []
    for kv in ("gather", "face", "tile"):
        g = gpu_solver(afx, m, bcs, precision="fp32-mixed", kernel_variant=kv)
        g.init()
        g.set_q(q)
        g.iterate(3)
        out.append(g.get_q())
    # different FP32 summation contexts (fast-math contraction) only
    assert rel_l2(out[0], out[1]) < 1e-6
    assert rel_l2(out[0], out[2]) < 1e-6


def test_fp32_defect_correction_tracks_fp64(afx, orc):
    # after a refresh at the start of the run the corrected FP32 residual is
    # R64 up to FP32 rounding of the correction: the first iteration matches
    # the FP64 oracle to ~1e-7 of the state update, closer than pure FP32
    m, bcs = omesh_case(48, 24)
    so = oracle_solver(orc, m, bcs)
    so.init()
    so.iterate(20)
    q = so.q()
    so.iterate(1)
    ref = so.q()
    errs = []
    for corr in (0, 50):
        g = gpu_solver(afx, m, bcs, precision="fp32-mixed", fp64_correction_interval=corr)
        g.init()
        g.set_q(q)
        g.iterate(1)
        errs.append(rel_l2(g.get_q() - q, ref - q))
    assert errs[1] < errs[0] and errs[1] < 1e-4, errs


def test_fp64_finish_switches_and_converges(afx):
    # FP32-mixed run_to_convergence with the FP64 finish ends below what the
    # FP32 residual alone can reach, and its last iterations are FP64 ones
    m = __import__("aeroflex_gb300.meshgen", fromlist=["x"]).airfoil_omesh(32, 32, split=False)
    bcs = {"farfield": dict(type="farfield", T=1.0, mach=0.5, angle=1.25 * 0.01745, p=1.0),
           "wall": dict(type="slip-wall")}
    errs = []
    for fin in (0, 1):
        g = gpu_solver(afx, m, bcs, precision="fp32-mixed", cfl=1.5, fp64_finish=fin)
        g.init()
        it, err = g.run_solver(1e-11, 60000)
        errs.append(err)
    assert errs[1] < 1e-2 * errs[0], errs


def test_nonfinite_flagged(afx):
    m, bcs = omesh_case(32, 16)
    g = gpu_solver(afx, m, bcs, cfl=1e6)
    g.init()
    from aeroflex_gb300.rans import AfxError
    with pytest.raises(AfxError) as ei:
        g.iterate(50)
    assert ei.value.code == 4


def test_prolongate_bitexact(afx, orc):
    # multigrid::run's coarse -> fine transfer (multigrid.h:99-178, 316-321)
    from aeroflex_gb300 import meshgen
    from tests.cases import DEG
    bcs = {"farfield": dict(type="farfield", T=1.0, mach=0.5, angle=1.25 * DEG, p=1.0),
           "wall": dict(type="slip-wall")}
    mc = meshgen.airfoil_omesh(32, 16, split=False)
    mf = meshgen.airfoil_omesh(64, 32, split=False)
    oc = oracle_solver(orc, mc, bcs)
    oc.init()
    oc.iterate(30)
    of = oracle_solver(orc, mf, bcs)
    of.init()
    of.prolongate_from(oc)
    gc = gpu_solver(afx, mc, bcs)
    gc.init()
    gc.set_q(oc.q())
    gf = gpu_solver(afx, mf, bcs)
    gf.init()
    gf.prolongate_from(gc)
    np.testing.assert_array_equal(gf.get_q(), of.q())
    of.iterate(3)
    gf.iterate(3)
    np.testing.assert_array_equal(gf.get_q(), of.q())


@pytest.mark.parametrize("case", ["omesh", "channel"])
def test_wall_distance_bitexact(afx, orc, case):
    # mesh::compute_wall_dist (mesh.h:794-830), ghosts included
    if case == "omesh":
        m, bcs = omesh_case(48, 24)
    else:
        m, bcs, _ = channel_case(64, 32)
    so = oracle_solver(orc, m, bcs)
    g = gpu_solver(afx, m, bcs)
    np.testing.assert_array_equal(g.wall_distance(), so.wall_distance())


def test_full_size_channel_fp64_bitexact(afx, orc):
    """The benchmark's workload at full size (2048 x 1024 quads -> 4,194,304
    shuffled triangles, density bump): the FP64 residual and one explicit
    iteration bit for bit against the oracle, face-flux and tile variants."""
    m, bcs, q = channel_case(2048, 1024)
    so = oracle_solver(orc, m, bcs)
    so.init()
    so.set_q(q)
    R0 = so.residual()
    so.iterate(1)
    q1 = so.q()
    for kv in ("face", "tile"):
        g = gpu_solver(afx, m, bcs, kernel_variant=kv)
        g.init()
        g.set_q(q)
        assert np.array_equal(g.residual(), R0), kv
        g.iterate(1)
        assert np.array_equal(g.get_q(), q1), kv
        del g
