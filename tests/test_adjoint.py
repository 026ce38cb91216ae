"""Adjoint of the FP64 residual: u = (dR/dq)^T v and (dR/dbq)^T v from the
GPU (afx_residual_vjp) against central finite differences of the CPU
oracle's residual, and force-coefficient sensitivities from the adjoint solve
(afx_adjoint_solve) against finite differences of converged GPU solutions.

Tolerances: 1e-6 relative, as stated for the adjoint, plus the uncertainty
of the finite difference itself.  The residual is only piecewise smooth (the
limiter's min(1, .) and its min over faces, the neighbour max/min, the
entropy fix and the boundary cases switch branch), so a central difference
with a step that crosses a switch is wrong by O(1) in that term.  The
states are made generic (1e-3 random perturbation: no ties between
neighbours), the difference is taken at steps 1e-5 ... 1e-8, and the
reference is the pair of consecutive steps that agree best; their
disagreement is added to the tolerance.
"""
import numpy as np
import pytest

from tests.cases import DEG, channel_case, gpu_solver, omesh_case, oracle_solver

pytestmark = pytest.mark.gpu


def _fd_ref(f, steps=(1e-5, 1e-6, 1e-7, 1e-8)):
    """(value, uncertainty) of df/dh at 0 from central differences of f at
    the steps: the consecutive pair that agrees best."""
    d = [(f(h) - f(-h)) / (2 * h) for h in steps]
    k = min(range(len(d) - 1), key=lambda i: abs(d[i] - d[i + 1]))
    return 0.5 * (d[k] + d[k + 1]), abs(d[k] - d[k + 1])


def _generic(q, seed):
    return q * (1 + 1e-3 * np.random.default_rng(seed).standard_normal(q.size))


def _vR(orc_s, q, e, v):
    def f(h):
        orc_s.set_q(q + h * e)
        return float(v @ orc_s.residual())
    return f


@pytest.mark.parametrize("variant", [dict(), dict(limiter="michalak"), dict(second_order=False),
                                     dict(viscosity="laminar"), dict(viscosity="laminar", second_order=False)])
def test_vjp_matches_oracle_finite_differences(afx, orc, variant):
    m, bcs = omesh_case(48, 24)
    so = oracle_solver(orc, m, bcs, **variant)
    so.init()
    so.iterate(40)
    q = _generic(so.q(), 3)
    g = gpu_solver(afx, m, bcs, **variant)
    g.init()
    rng = np.random.default_rng(11)
    for trial in range(3):
        v = rng.standard_normal(q.size)
        e = rng.standard_normal(q.size) * np.abs(q)
        u, _ = g.residual_vjp(v, q=q)
        lhs = float(u @ e)
        rhs, unc = _fd_ref(_vR(so, q, e, v))
        assert unc <= 1e-5 * abs(rhs) and abs(lhs - rhs) <= 1e-6 * abs(rhs) + unc, (trial, lhs, rhs, unc)


@pytest.mark.parametrize("variant", [dict(), dict(viscosity="laminar", second_order=False)])
def test_vector_duals_give_the_single_direction_bits(afx, variant):
    # 1, 2 or 4 input directions per pass of the face kernel: each direction
    # is formed by the same operations, so the vJP is bit for bit the same
    m, bcs = omesh_case(48, 24)
    rng = np.random.default_rng(7)
    out = []
    for k in (1, 2, 4):
        g = gpu_solver(afx, m, bcs, adjoint_directions=float(k), **variant)
        g.init()
        g.iterate(30)
        q = g.get_q()
        v = rng.standard_normal(q.size) if not out else out[0][2]
        u, b = g.residual_vjp(v)
        out.append((u, b, v))
    for u, b, _ in out[1:]:
        np.testing.assert_array_equal(u, out[0][0])
        np.testing.assert_array_equal(b, out[0][1])


def test_vjp_shuffled_channel_all_boundaries(afx, orc):
    # slip walls + farfield on a shuffled, jittered triangle mesh
    m, bcs, q = channel_case(48, 24)
    so = oracle_solver(orc, m, bcs)
    so.init()
    so.set_q(q)
    so.iterate(10)
    q = _generic(so.q(), 4)
    g = gpu_solver(afx, m, bcs)
    g.init()
    rng = np.random.default_rng(5)
    v = rng.standard_normal(q.size)
    e = rng.standard_normal(q.size) * np.abs(q)
    u, _ = g.residual_vjp(v, q=q)
    rhs, unc = _fd_ref(_vR(so, q, e, v))
    assert unc <= 1e-5 * abs(rhs) and abs(float(u @ e) - rhs) <= 1e-6 * abs(rhs) + unc, (float(u @ e), rhs, unc)


def test_boundary_state_adjoint_matches_angle_fd(afx, orc):
    # (dR/dbq)^T v contracted with dbq/dalpha = (0, -rho*v, rho*u, 0) equals
    # the derivative of v.R with respect to the farfield angle
    m, bcs = omesh_case(48, 24, mach=0.5, aoa_deg=2.0)
    so = oracle_solver(orc, m, bcs)
    so.init()
    so.iterate(40)
    q = _generic(so.q(), 6)
    so.set_q(q)
    g = gpu_solver(afx, m, bcs)
    g.init()
    g.set_q(q)
    rng = np.random.default_rng(2)
    v = rng.standard_normal(q.size)
    _, bqbar = g.residual_vjp(v)
    bq = g.boundary_states()
    far = np.array([n == "farfield" for n in g.mesh_boundary_names])
    dbq = np.zeros_like(bq)
    dbq[far, 1] = -bq[far, 2]
    dbq[far, 2] = bq[far, 1]
    lhs = float((bqbar * dbq).sum())
    a0 = 2.0 * DEG

    def f(h):
        so.set_farfield("farfield", 0.5, a0 + h)
        return float(v @ so.residual())
    rhs, unc = _fd_ref(f)
    assert unc <= 1e-5 * abs(rhs) and abs(lhs - rhs) <= 1e-6 * abs(rhs) + unc, (lhs, rhs, unc)


def test_torch_gradcheck_harness(afx):
    torch = pytest.importorskip("torch")
    from tests.adjoint_harness import ResidualFn
    m, bcs = omesh_case(16, 8)
    g = gpu_solver(afx, m, bcs)
    g.init()
    g.iterate(20)
    q = torch.from_numpy(g.get_q()).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x: ResidualFn.apply(x, g), (q,), eps=1e-6, atol=1e-7, rtol=1e-6,
                                    fast_mode=True)


def _converged(afx, m, bcs, mach, aoa):
    b = dict(bcs)
    b["farfield"] = dict(b["farfield"], mach=mach, angle=aoa)
    g = gpu_solver(afx, m, b, cfl=1.5)
    g.init()
    g.run_solver(1e-12, 200000)
    return g


def test_adjoint_alpha_mach_sensitivities_match_fd(afx):
    from aeroflex_gb300.rans import get_wall_profile
    from aeroflex_gb300 import meshgen
    m = meshgen.airfoil_omesh(48, 32, split=False, m=0.02, p=0.4, t=0.12)
    bcs = {"farfield": dict(type="farfield", T=1.0, mach=0.5, angle=2.0 * DEG, p=1.0), "wall": dict(type="slip-wall")}
    M0, a0 = 0.5, 2.0 * DEG
    g = _converged(afx, m, bcs, M0, a0)
    out = {}
    for obj in ("cl", "cd"):
        d, iters, res = g.adjoint_solve("wall", obj, tol=1e-12, max_it=200000)
        assert res < 1e-10
        out[obj] = d
    for k, (dM, da) in ((0, (0.0, 1e-5)), (1, (1e-5, 0.0))):
        gp = _converged(afx, m, bcs, M0 + dM, a0 + da)
        gm = _converged(afx, m, bcs, M0 - dM, a0 - da)
        h = dM + da
        for obj in ("cl", "cd"):
            fd = (get_wall_profile(gp, "wall")[obj] - get_wall_profile(gm, "wall")[obj]) / (2 * h)
            ad = out[obj][k]
            assert abs(ad - fd) <= 1e-6 * abs(fd) + 1e-9, (obj, k, ad, fd)


@pytest.mark.parametrize("viscosity,wall,second", [("inviscid", "slip-wall", True), ("laminar", "wall", False)])
def test_implicit_adjoint_alpha_mach_sensitivities_match_fd(afx, viscosity, wall, second):
    # an implicit solver's adjoint: its implicit iteration transposed (the
    # ILU(0)-preconditioned GMRES on M^T), with the exact vJP in the defect.
    # The laminar case runs first order: on this coarse mesh the second-order
    # limiter switches within the angle step of the difference (the adjoint
    # then differs from it by ~1e-4), while on 48 x 32 both agree to 2e-9.
    from aeroflex_gb300.rans import get_wall_profile
    from aeroflex_gb300 import meshgen
    m = meshgen.airfoil_omesh(32, 24, split=False, m=0.02, p=0.4, t=0.12)
    bcs = {"farfield": dict(type="farfield", T=1.0, mach=0.5, angle=2.0 * DEG, p=1.0), "wall": dict(type=wall)}
    M0, a0 = 0.5, 2.0 * DEG

    def conv(M, a):
        b = dict(bcs)
        b["farfield"] = dict(b["farfield"], mach=M, angle=a)
        g = gpu_solver(afx, m, b, viscosity=viscosity, second_order=second, solver="implicit", start_cfl=40.0,
                       slope_cfl=50.0, max_cfl=100.0)
        g.init()
        g.run_solver(1e-12, 3000)
        return g

    g = conv(M0, a0)
    out = {}
    for obj in ("cl", "cd"):
        d, iters, res = g.adjoint_solve("wall", obj, tol=1e-12, max_it=5000)
        assert res < 1e-11 and iters < 5000, (obj, iters, res)
        out[obj] = d
    for k, (dM, da) in ((0, (0.0, 1e-5)), (1, (1e-5, 0.0))):
        gp, gm = conv(M0 + dM, a0 + da), conv(M0 - dM, a0 - da)
        h = dM + da
        for obj in ("cl", "cd"):
            fd = (get_wall_profile(gp, "wall")[obj] - get_wall_profile(gm, "wall")[obj]) / (2 * h)
            ad = out[obj][k]
            assert abs(ad - fd) <= 1e-6 * abs(fd) + 1e-9, (obj, k, ad, fd)


def _implicit(afx, m, bcs, a=None, **kw):
    g = gpu_solver(afx, m, bcs, solver="implicit", start_cfl=40.0, slope_cfl=50.0, max_cfl=100.0, **kw)
    g.init()
    if a is not None:
        g.deform_patch(a, "wall", 2.0)
    it, err = g.run_solver(1e-13, 600)
    assert err <= 1e-12, (it, err)
    return g


@pytest.mark.parametrize("order,steps,rtol", [
    # first order: smooth in the shape, steps of 1e-6
    ("first", (2e-6, 1e-6), 1e-6),
    # second order: the limiter (min over faces of min(1, .)) switches within
    # displacements of ~1e-6, so the check takes the step 1e-7; the converged
    # C_L is good to ~1e-13, which bounds the difference's accuracy near 1e-6
    ("second", (2e-7, 1e-7), 1e-5),
])
def test_adjoint_surface_sensitivities_match_fd(afx, order, steps, rtol):
    # dJ/da for the normal displacements a of the wall nodes (displacement
    # spread into the volume by inverse-distance weighting), against central
    # differences of converged solutions (to 1e-13) on deformed meshes
    from aeroflex_gb300 import meshgen
    from aeroflex_gb300.rans import get_wall_profile
    m = meshgen.airfoil_omesh(32, 24, split=False, m=0.02, p=0.4, t=0.12)
    bcs = {"farfield": dict(type="farfield", T=1.0, mach=0.5, angle=2.0 * DEG, p=1.0), "wall": dict(type="slip-wall")}
    kw = dict(second_order=(order == "second"))
    g = _implicit(afx, m, bcs, **kw)
    ids, nx, ny = g.patch_nodes("wall")
    assert len(ids) == 32 and np.allclose(np.hypot(nx, ny), 1.0)
    rng = np.random.default_rng(3)
    c = rng.standard_normal(len(ids))
    dirs = [c / np.linalg.norm(c)]
    for obj in ("cl", "cd"):
        g.adjoint_solve("wall", obj, tol=1e-13, max_it=400000)
        dJ = g.adjoint_patch("wall", obj)
        for c in dirs:
            pred = float(c @ dJ)
            fds = []
            for eps in steps:
                Jp = get_wall_profile(_implicit(afx, m, bcs, eps * c, **kw), "wall")[obj]
                Jm = get_wall_profile(_implicit(afx, m, bcs, -eps * c, **kw), "wall")[obj]
                fds.append((Jp - Jm) / (2 * eps))
            fd, unc = 0.5 * (fds[0] + fds[1]), abs(fds[0] - fds[1])
            assert abs(pred - fd) <= rtol * abs(fd) + unc + 1e-9, (obj, pred, fd, unc)
