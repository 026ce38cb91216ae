"""Spalart-Allmaras (SA-neg) turbulence model.

The reference has no SA model (physics.h:259-261, an empty branch), so the
FP64 oracle (oracle/sa_oracle.cpp, the published model restated) is the
checker:
- CPU: the source term's analytic derivative against central differences,
  and the hybrid boundary-layer mesh generator;
- GPU (FP64): residuals (mean flow with mu_t and wall shear, and nu~) and
  explicit iterations bit for bit against the oracle; FP32-mixed within
  stated tolerances; the implicit solver's converged state is a zero of the
  oracle's residual; a turbulent flat plate's skin friction against the
  1/5-power turbulent correlation.
"""
import numpy as np
import pytest

from aeroflex_gb300 import meshgen
from tests.cases import DEG, gpu_solver, rel_l2


def _sa_settings(**kw):
    st = dict(viscosity="spalart-allmaras", mu_L=1.4 * 0.3 / 1e5, cfl=0.5)
    st.update(kw)
    return st


def _airfoil(n_surf=48, n_rad=24, split=False, first=2e-4, mach=0.3, aoa=2.0):
    m = meshgen.airfoil_omesh(n_surf, n_rad, split=split, first=first)
    bcs = {"farfield": dict(type="farfield", T=1.0, mach=mach, angle=aoa * DEG, p=1.0), "wall": dict(type="wall")}
    return m, bcs


def test_sa_source_derivative_matches_finite_differences(orc):
    """d(P - D)/dnu~ (the implicit diagonal) against central differences,
    both branches; samples where two step sizes disagree straddle a branch
    switch of the model and are skipped."""
    rng = np.random.default_rng(3)
    checked = 0
    for _ in range(3000):
        nul = 10 ** rng.uniform(-6, -3)
        nut = nul * 10 ** rng.uniform(-2, 3) * (1 if rng.random() < 0.8 else -1)
        om, d = 10 ** rng.uniform(-2, 3), 10 ** rng.uniform(-5, 0)
        _, ds = orc.sa_source(nut, nul, om, d)
        fd = []
        for h in (1e-6 * abs(nut), 1e-7 * abs(nut)):
            sp, _ = orc.sa_source(nut + h, nul, om, d)
            sm, _ = orc.sa_source(nut - h, nul, om, d)
            fd.append((sp - sm) / (2 * h))
        if abs(fd[0] - fd[1]) > 1e-5 * max(abs(fd[0]), 1e-300):
            continue
        assert abs(fd[0] - ds) <= 1e-6 * max(abs(ds), 1e-300), (nut, nul, om, d, ds, fd)
        checked += 1
    assert checked > 2500


def test_hybrid_mesh_generator(orc):
    """Config 2's mesh: 513 surface nodes (512 distinct), 60 quad layers from
    1e-6 chord at growth 1.1, a conforming triangular fill to 100 chords,
    about 200k cells."""
    m = meshgen.hybrid_airfoil()
    assert m["n_bl_quads"] == 512 * 60
    assert abs(m["bl_thickness"] - 1e-6 * (1.1 ** 60 - 1) / 0.1) < 1e-12
    assert 190000 <= len(m["cells"]) <= 210000
    om = orc.Mesh.from_arrays(m)
    a = om.get("area")[: om.n_real]
    assert (a > 0).all()
    assert om.boundary_names().count("wall") == 512
    r = np.hypot(om.get("ex") - 0.5, om.get("ey"))
    far = np.array([n == "farfield" for n in om.boundary_names()])
    be = om.get_int("boundary_edges")
    assert np.allclose(r[be[far]], 100.0, rtol=1e-3)


def _warm(orc, m, bcs, n, **kw):
    so = orc.Solver(orc.Mesh.from_arrays(m), orc.default_settings(**_sa_settings(**kw)), bcs)
    so.init()
    so.iterate(n)
    return so


def _gpu(afx, m, bcs, precision="fp64", **kw):
    return gpu_solver(afx, m, bcs, precision=precision, **_sa_settings(**kw))


@pytest.mark.gpu
@pytest.mark.parametrize("kv", ["face", "tile"])
@pytest.mark.parametrize("split", [False, True])
def test_sa_residual_and_iterations_bitexact(afx, orc, kv, split):
    m, bcs = _airfoil(split=split)
    so = _warm(orc, m, bcs, 40)
    q, nu = so.q(), so.nu()
    R = so.residual()
    nuW = so.nu_residual()
    g = _gpu(afx, m, bcs, kernel_variant=kv)
    g.init()
    g.set_q(q)
    g.set_nu(nu)
    np.testing.assert_array_equal(g.residual(), R)
    np.testing.assert_array_equal(g.nu_residual(), nuW)
    so.iterate(5)
    g.iterate(5)
    np.testing.assert_array_equal(g.get_q(), so.q())
    np.testing.assert_array_equal(g.nu(), so.nu())


@pytest.mark.gpu
def test_sa_fp32_mixed_tracks_fp64(afx, orc):
    m, bcs = _airfoil()
    so = _warm(orc, m, bcs, 40)
    g = _gpu(afx, m, bcs, precision="fp32-mixed")
    g.init()
    g.set_q(so.q())
    g.set_nu(so.nu())
    so.iterate(20)
    g.iterate(20)
    assert rel_l2(g.get_q(), so.q()) < 1e-5
    assert rel_l2(g.nu(), so.nu()) < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32-mixed"])
def test_sa_implicit_converges_to_a_zero_of_the_oracle_residual(afx, orc, precision):
    m, bcs = _airfoil(n_surf=64, n_rad=32, first=1e-4)
    g = _gpu(afx, m, bcs, precision=precision, solver="implicit", cfl=10.0, slope_cfl=10.0, max_cfl=200.0,
             tolerance=1e-10, max_iterations=800)
    g.init()
    q0 = g.get_q()
    it, err = g.run_solver()
    assert err <= 1e-10, (it, err)
    so = orc.Solver(orc.Mesh.from_arrays(m), orc.default_settings(**_sa_settings()), bcs)
    so.init()
    R0 = np.linalg.norm(so.residual())
    W0 = np.linalg.norm(so.nu_residual())
    so.set_q(g.get_q())
    so.set_nu(g.nu())
    assert np.linalg.norm(so.residual()) <= 1e-8 * R0
    assert np.linalg.norm(so.nu_residual()) <= 1e-6 * W0
    assert np.abs(g.get_q() - q0).max() > 0


def flat_plate(nx=96, ny=64, L=1.0, H=0.5, first=2e-5, lead=0.25):
    """Flat plate of length L from x = 0 (no-slip "wall"), far field on the
    stretch of length `lead` before it, above and at the ends; quads
    clustered at the wall (first height `first`) and at the leading edge."""
    xs_lead = -lead * (1 - np.linspace(0, 1, nx // 6 + 1)) ** 1.5
    xs_plate = L * (np.linspace(0, 1, nx + 1) ** 1.5)
    xs = np.concatenate([xs_lead[:-1], xs_plate])
    lo, hi = 1.0 + 1e-9, 2.0
    for _ in range(200):  # geometric growth ratio reaching H in ny layers
        r = 0.5 * (lo + hi)
        lo, hi = (r, hi) if first * (r ** ny - 1) / (r - 1) < H else (lo, r)
    ys = first * (r ** np.arange(ny + 1) - 1) / (r - 1)
    ys *= H / ys[-1]
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    nxn, nyn = len(xs), len(ys)
    x, y = X.reshape(-1), Y.reshape(-1)
    ii, jj = np.meshgrid(np.arange(nxn - 1), np.arange(nyn - 1), indexing="ij")
    a = ii * nyn + jj
    cells = np.stack([a, a + nyn, a + nyn + 1, a + 1], -1).reshape(-1, 4).astype(np.int32)
    i = np.arange(nxn - 1)
    j = np.arange(nyn - 1)
    bottom = np.stack([i * nyn, (i + 1) * nyn], -1)
    plate = xs[:-1] >= 0
    top = np.stack([i * nyn + nyn - 1, (i + 1) * nyn + nyn - 1], -1)
    left = np.stack([j, j + 1], -1)
    right = np.stack([(nxn - 1) * nyn + j, (nxn - 1) * nyn + j + 1], -1)
    bedges = np.concatenate([bottom[plate], bottom[~plate], top, left, right]).astype(np.int32)
    bpatch = np.concatenate([np.zeros(plate.sum()), np.ones(len(bedges) - plate.sum())]).astype(np.int32)
    return dict(x=x, y=y, cells=cells, bedges=bedges, bpatch=bpatch, names=["wall", "farfield"])


@pytest.mark.gpu
def test_sa_flat_plate_skin_friction(afx, orc):
    """Turbulent flat plate at M 0.2, Re_L = 5e6: the converged implicit
    solution is turbulent over 0.3 <= x/L <= 0.9 (skin friction at least 3
    times Blasius' 0.664 Re_x^-1/2, between 0.75 and 1.6 times the 1/5-power
    turbulent correlation 0.0592 Re_x^-0.2, falling with x as Re_x^-b,
    0.1 <= b <= 0.35).  The scheme gives 1.37-1.42 times the correlation: the
    reference's Roe flux keeps a Harten floor of 0.025 c on the shear wave
    (physics.h:215-217), which near the wall is an order of magnitude above
    nu + nu_t on these cells."""
    mach, re = 0.2, 5e6
    m = flat_plate()
    rho, u = 1.4, mach
    mu = rho * u * 1.0 / re
    bcs = {"wall": dict(type="wall"), "farfield": dict(type="farfield", T=1.0, mach=mach, angle=0.0, p=1.0)}
    g = gpu_solver(afx, m, bcs, viscosity="spalart-allmaras", mu_L=mu, solver="implicit", cfl=5.0, slope_cfl=5.0,
                   max_cfl=100.0, tolerance=1e-8, max_iterations=3000)
    g.init()
    it, err = g.run_solver()
    assert err <= 1e-8, (it, err)
    om = orc.Mesh.from_arrays(m)  # the same numbering as the solver's
    q = g.get_q().reshape(-1, 4)
    cy = om.get("cy")
    names = om.boundary_names()
    be = om.get_int("boundary_edges")
    ec = om.get_int("edges_cells").reshape(-1, 2)
    ex, ey = om.get("ex"), om.get("ey")
    xs, cfs = [], []
    for b, nm in enumerate(names):
        if nm != "wall":
            continue
        e = be[b]
        c = ec[e, 0]
        delta = abs(ey[e] - cy[c])
        cfs.append(mu * (q[c, 1] / q[c, 0]) / delta / (0.5 * rho * u * u))
        xs.append(ex[e])
    xs, cfs = np.array(xs), np.array(cfs)
    sel = (xs >= 0.3) & (xs <= 0.9)
    ratio = cfs[sel] / (0.0592 * (re * xs[sel]) ** -0.2)
    assert np.all((ratio > 0.75) & (ratio < 1.6)), ratio
    assert np.all(cfs[sel] > 3 * 0.664 / np.sqrt(re * xs[sel]))
    b = -np.polyfit(np.log(xs[sel]), np.log(cfs[sel]), 1)[0]
    assert 0.1 <= b <= 0.35, b
