"""The oracle pinned to the reference's own code.

oracle/_ref is the reference's rans code compiled from its unmodified
headers (oracle/build_ref.py, with the Eigen-API stand-in of
oracle/eigen_api).  tests/golden/ref_pins.json holds what it computed
(tests/golden/make_ref_golden.py).  Here, on the CPU:

- the oracle restatement reproduces every committed reference pin bit for
  bit (runs anywhere: it needs only the committed fixture);
- where the reference tree is present: the pins regenerate identically from
  the reference, and the reference and the oracle agree directly on more
  inputs (the example meshes, face fluxes on random states, grid sequencing).
"""
import json
import os

import numpy as np
import pytest

from aeroflex_gb300 import meshgen
from oracle import refsrc
from tests import refpins

with open(refpins.PINS_JSON) as f:
    PINS = json.load(f)

needs_ref = pytest.mark.skipif(not refsrc.available(), reason="reference source tree not present")


def test_oracle_reproduces_the_reference_pins(orc):
    got = refpins.explicit_pins(refpins.OracleDriver(orc))
    want = PINS["explicit"]
    assert sorted(got) == sorted(want)
    for k in want:
        assert got[k] == want[k], k  # hashes, and sequential sums in both


@needs_ref
def test_reference_pins_regenerate():
    from oracle import ref
    assert ref.available()
    got = refpins.explicit_pins(refpins.RefDriver())
    assert got == PINS["explicit"]
    assert refpins.implicit_rhs_pins(refpins.RefDriver()) == PINS["implicit_rhs"]


@needs_ref
@pytest.mark.parametrize("name", ["naca0012q_coarse", "naca0012q_mid", "naca0012_coarse", "naca0012_mid",
                                  "airfoil_demo_coarse", "airfoil_API2_coarse", "flat_plate"])
def test_reference_example_meshes_read_alike(orc, afx, name):
    """The reference's reader, the oracle's and the product's on the
    reference's own example meshes: same numbering, same metrics."""
    from oracle import ref
    path = refsrc.path("examples", "rans", name + ".msh")
    rm, om, gm = ref.Mesh(path), orc.Mesh.load(path), afx.mesh(path)
    assert (rm.n_real, rm.n_tot, rm.n_edges, rm.n_boundary) == (om.n_real, om.n_tot, om.n_edges, om.n_boundary)
    for k in ("cx", "cy", "area", "ex", "ey", "nx", "ny", "L"):
        np.testing.assert_array_equal(om.get(k), rm.get(k), err_msg=k)
        np.testing.assert_array_equal(gm.get(k), rm.get(k), err_msg=k)
    np.testing.assert_array_equal(om.get_int("edges_cells"), rm.get_int("edges_cells"))
    assert om.boundary_names() == rm.boundary_names()


@needs_ref
def test_reference_face_fluxes_equal_the_oracle(orc):
    """Every flux functor (physics.h:160-530), inviscid and laminar, on
    random states and normals."""
    from oracle import ref
    rng = np.random.default_rng(7)
    for _ in range(200):
        q = []
        for _ in range(2):
            rho = rng.uniform(0.5, 2.0)
            u, v = rng.uniform(-0.8, 0.8, 2)
            p = rng.uniform(0.5, 1.5)
            q.append(np.array([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)]))
        th = rng.uniform(0, 2 * np.pi)
        nx, ny = np.cos(th), np.sin(th)
        gx, gy = rng.normal(size=4), rng.normal(size=4)
        for bc in ("internal", "farfield", "slip-wall", "wall"):
            for visc in (0, 1):
                a = ref.face_flux(q[0], q[1], nx, ny, visc=visc, bc=bc, gx=gx, gy=gy)
                b = orc.face_flux(q[0], q[1], nx, ny, visc=visc, bc=bc, gx=gx, gy=gy)
                np.testing.assert_array_equal(a, b, err_msg="%s visc=%d" % (bc, visc))


@needs_ref
def test_reference_grid_sequencing_equals_the_oracle(orc):
    """multigrid::run over two levels (multigrid.h:295-363): run_solver on
    the coarse mesh, the inverse-distance transfer, run_solver on the fine
    mesh."""
    coarse, fine = meshgen.airfoil_omesh(16, 8, split=False), meshgen.airfoil_omesh(32, 16, split=False)
    bcs = refpins.airfoil_bcs(0.5, 2.0)
    st = dict(start_cfl=1.5, tolerance=1e-2, max_iterations=300)
    drv = refpins.RefDriver()
    c = drv.levels([coarse, fine], bcs, **st)
    hist = c.run(reinit=True)
    oc = refpins.OracleDriver(orc).solver(coarse, bcs, **st).s
    of = refpins.OracleDriver(orc).solver(fine, bcs, **st).s
    oc.init()
    _, _, h1 = oc.run_solver()
    of.prolongate_from(oc)
    _, _, h2 = of.run_solver()
    np.testing.assert_array_equal(hist, np.concatenate([h1, h2]))
    np.testing.assert_array_equal(c.q(-1), of.q())


def test_c1_split_mesh_diverges_in_the_reference():
    """Config 1 as configured (split triangles): the reference's implicit
    solver stops with status 1 after its residual grew, as recorded by the
    fixture script; on the same mesh with whole quads it converges."""
    d = PINS["c1_split_diverges"]
    assert d["status"] == 1
    h = np.array(d["history"])
    assert h[-1] > 10 * h.min()
    c1 = PINS["implicit"]["c1_quads"]["polar"][0]
    assert c1["status"] == 0 and c1["final_residual"] <= 1e-10
