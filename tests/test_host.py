"""Host-side checks that need no GPU: the C-ABI library loads and exports
every symbol include/afx_rans.h declares, the mesh loader reproduces the
reference's numbering and metrics bit for bit (against the oracle), and the
INI reader follows tiny::config + Settings::import_config_file."""
import os
import re

import numpy as np
import pytest

from aeroflex_gb300 import meshgen
from oracle import refsrc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_MESHES = refsrc.path("examples", "rans")
METRICS = ["cx", "cy", "area", "ex", "ey", "nx", "ny", "L"]


def test_abi_exports_every_declared_symbol(afx):
    decl = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            decl |= set(re.findall(r"\b(afx_[a-z0-9_]+)\s*\(", txt))
    assert decl, "no declarations found"
    L = afx.lib()
    missing = [d for d in sorted(decl) if not hasattr(L, d)]
    assert not missing, missing
    assert set(afx.ABI_SYMBOLS) == decl


def _compare_mesh(gm, om):
    assert gm.nRealCells == om.n_real and gm.n_edges == om.n_edges and gm.n_boundary == om.n_boundary
    for k in METRICS:
        np.testing.assert_array_equal(gm.get(k), om.get(k), err_msg=k)
    for k in ("edges_cells", "edges_nodes", "boundary_edges"):
        np.testing.assert_array_equal(gm.get_int(k), om.get_int(k), err_msg=k)
    assert gm.boundary_names() == om.boundary_names()


@pytest.mark.parametrize("gen", [
    lambda: meshgen.airfoil_omesh(64, 32),
    lambda: meshgen.airfoil_omesh(32, 16, split=False),
    lambda: meshgen.airfoil_omesh(40, 20, m=0.04, p=0.4, t=0.15),
    lambda: meshgen.channel(48, 24),
])
def test_mesh_arrays_match_oracle(afx, orc, gen):
    m = gen()
    _compare_mesh(afx.mesh.from_arrays(m), orc.Mesh.from_arrays(m))


def test_gmsh_roundtrip_matches_arrays(afx, orc, tmp_path):
    m = meshgen.airfoil_omesh(48, 24)
    p = tmp_path / "o.msh"
    meshgen.write_gmsh(str(p), m)
    gf = afx.mesh(str(p))
    _compare_mesh(gf, orc.Mesh.from_arrays(m))
    _compare_mesh(gf, orc.Mesh.load(str(p)))


@pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference examples not mounted")
@pytest.mark.parametrize("name", ["naca0012q_coarse.msh", "naca0012_coarse.msh", "flat_plate.msh",
                                  "airfoil_demo_coarse.msh"])
def test_reference_example_meshes(afx, orc, name):
    path = os.path.join(REF_MESHES, name)
    _compare_mesh(afx.mesh(path), orc.Mesh.load(path))


def test_layout_is_a_permutation(afx):
    m = afx.mesh.from_arrays(meshgen.channel(32, 16))
    order = m.get_int("cell_order")
    assert sorted(order.tolist()) == list(range(m.nRealCells))


def test_mesh_errors(afx, tmp_path):
    with pytest.raises(afx.AfxError) as e:
        afx.mesh(str(tmp_path / "missing.msh"))
    assert e.value.code == 1
    m = meshgen.airfoil_omesh(16, 8)
    bad = dict(m)
    bad["bedges"] = m["bedges"][:-1]  # one boundary edge left unlisted
    bad["bpatch"] = m["bpatch"][:-1]
    with pytest.raises(afx.AfxError) as e:
        afx.mesh.from_arrays(bad)
    assert e.value.code == 3
    bad = dict(m)
    bad["cells"] = m["cells"].copy()
    bad["cells"][0, 0] = 10 ** 7
    with pytest.raises(afx.AfxError) as e:
        afx.mesh.from_arrays(bad)
    assert e.value.code == 3


CONF = """[rans-gas]
gamma = 1.4
R = 0.71428571428

[rans-bc]
<
    name = farfield,
    type = farfield,
    T = 1,
    mach = 0.2,
    angle = 420.0,
    p = 1,
>
<name = wall, type = slip-wall>

[rans-alphas]
alpha_start = 1.0
alpha_end = 7.0
alpha_step = 3.0

[rans-solver]
solver = implicit
viscosity = inviscid
gradient = green-gauss
second_order = true
relaxation = 0.9
start_cfl = 40.0
slope_cfl = 50.0
max_cfl = 100.0
tolerance = 1e-4
rhs_iterations = 5
max_iterations = 300
limiter_k = 5.0
"""


def test_config_ini(afx):
    c = afx.Settings.from_ini_string(CONF)
    assert c.get("solver") == "implicit"
    assert c.get("gamma") == 1.4 and c.get("max_cfl") == 100.0 and c.get("max_iterations") == 300
    assert c.get("second_order") == 1.0 and c.get("alpha_step") == 3.0
    assert c.bc_count() == 2
    assert c.get("precision") == "fp64"
    c2 = afx.Settings.from_ini_string(CONF.replace("viscosity = inviscid", "viscosity = spallart-allmaras")
                                      .replace("solver = implicit", "solver = explicit"))
    assert c2.get("viscosity") == "spallart-allmaras" and c2.get("solver") == "explicit"
    c3 = afx.Settings.from_ini_string(CONF.replace("viscosity = inviscid", "viscosity = bogus"))
    assert c3.get("viscosity") == "inviscid"  # unknown strings leave the setting unchanged (core.h:218-227)


def test_library_settings_roundtrip(afx):
    # this library's own numeric settings: defaults, set, read back
    c = afx.Settings()
    assert c.get("krylov_graph") == 1.0 and c.get("fp64_finish") == 0.0 and c.get("block_size") == 0.0
    c.set("krylov_graph", 0).set("fp64_finish", 1).set("block_size", 128).set("fp64_correction_interval", 20)
    assert c.get("krylov_graph") == 0.0 and c.get("fp64_finish") == 1.0
    assert c.get("block_size") == 128.0 and c.get("fp64_correction_interval") == 20.0
    with pytest.raises(afx.AfxError) as e:
        c.set("block_size", 100)
    assert e.value.code == 2


@pytest.mark.parametrize("mutate,msg", [
    (lambda t: t.replace("<name = wall, type = slip-wall>\n", ""), "Invalid number of boundary conditions"),
    (lambda t: t.replace("[rans-alphas]", "[rans-alphaz]"), "Section [rans-alphas] not found"),
    (lambda t: t.replace("second_order = true", "second_order = maybe"), "not a valid boolean"),
    (lambda t: t.replace("limiter_k = 5.0\n", ""), "Setting (limiter_k) not found"),
    (lambda t: t.replace("[rans-gas]", "[rans-gas"), "Closing character is missing"),
])
def test_config_errors(afx, mutate, msg):
    with pytest.raises(afx.AfxError) as e:
        afx.Settings.from_ini_string(mutate(CONF))
    assert e.value.code == 2 and msg in str(e.value)


@pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference examples not mounted")
def test_reference_configs(afx):
    c = afx.Settings.from_ini(refsrc.path("examples", "conf.ini"))
    assert c.get("max_cfl") == 100.0 and c.get("tolerance") == 1e-4
    # examples/rans/config.ini has no [rans-alphas]: import fails as in the reference (core.h:269)
    with pytest.raises(afx.AfxError) as e:
        afx.Settings.from_ini(os.path.join(REF_MESHES, "config.ini"))
    assert "rans-alphas" in str(e.value)


def test_solver_without_gpu_fails_loudly(afx):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    m = afx.mesh.from_arrays(meshgen.airfoil_omesh(16, 8))
    with pytest.raises(afx.AfxError) as e:
        afx.Solver(m, afx.Settings())
    assert e.value.code == 7


def test_batch_checks_schemes_then_fails_loudly_without_gpu(afx):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    meshes = [afx.mesh.from_arrays(meshgen.airfoil_omesh(16, 8)), afx.mesh.from_arrays(meshgen.airfoil_omesh(20, 8))]
    sets = [afx.Settings(), afx.Settings().set("limiter", "michalak")]
    with pytest.raises(afx.AfxError) as e:
        afx.Batch(meshes, sets)
    assert e.value.code == 2 and "case 1" in str(e.value)
    with pytest.raises(afx.AfxError) as e:
        afx.Batch(meshes, [afx.Settings(), afx.Settings()])
    assert e.value.code == 7


def test_mesh_set_nodes_matches_a_fresh_mesh(afx):
    # deformed coordinates on an existing mesh give exactly the metrics of a
    # mesh built from the deformed coordinates
    m0 = meshgen.airfoil_omesh(24, 12, split=False, m=0.02)
    rng = np.random.default_rng(7)
    x = m0["x"] * (1 + 1e-3 * rng.standard_normal(m0["x"].size))
    y = m0["y"] * (1 + 1e-3 * rng.standard_normal(m0["y"].size))
    a = afx.mesh.from_arrays(m0)
    a.set_nodes(x, y)
    b = afx.mesh.from_arrays(dict(m0, x=x, y=y))
    for what in ("cx", "cy", "area", "ex", "ey", "nx", "ny", "L"):
        np.testing.assert_array_equal(a.get(what), b.get(what), err_msg=what)
    np.testing.assert_array_equal(a.get("node_x"), x)
    np.testing.assert_array_equal(a.get("node_y"), y)
    with pytest.raises(afx.AfxError):
        a.set_nodes(x[:-1], y[:-1])


def test_polar_sweep_meshes_do_not_fold():
    # every cell of the 256 polar-sweep O-meshes keeps the orientation of
    # the mesh (no folded cell near the far field)
    for c in meshgen.polar_sweep_cases(256, seed=4):
        m = c["mesh"]
        X, Y = m["x"][m["cells"]], m["y"][m["cells"]]
        sa = 0.5 * sum(X[:, k] * Y[:, (k + 1) % 4] - X[:, (k + 1) % 4] * Y[:, k] for k in range(4))
        assert (sa < 0).all() or (sa > 0).all(), (c["n_cells"], int((sa > 0).sum()))
