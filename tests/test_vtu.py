"""VTU output (`rans::save`, post.h:58-180): the library's writer
(afx_write_vtu, formatted in parallel chunks) against the oracle's
restatement (one string, std::to_string and a fixed 16-digit stream, as the
reference assembles it), byte for byte, on the same mesh and state."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from tests.cases import channel_case, omesh_case
from oracle import refsrc

REF_MESHES = refsrc.path("examples", "rans")


def _oracle_state(orc, m, bcs, iters=12):
    om = orc.Mesh.from_arrays(m)
    s = orc.Solver(om, orc.default_settings(), bcs)
    s.init()
    s.iterate(iters)
    return om, s


@pytest.mark.parametrize("case", ["omesh_quads", "channel_triangles"])
def test_vtu_bytes_match_oracle(afx, orc, tmp_path, case):
    if case == "omesh_quads":
        m, bcs = omesh_case(40, 20, split=False)
    else:
        m, bcs, _ = channel_case(30, 14)
    om, s = _oracle_state(orc, m, bcs)
    q = s.q()
    wd = s.wall_distance()[: om.n_real]
    gm = afx.mesh.from_arrays(m)
    mine, ref = tmp_path / "afx.vtu", tmp_path / "orc.vtu"
    gm.write_vtu(mine, q, wd)
    om.save_vtu(ref, q, wd)
    a, b = mine.read_bytes(), ref.read_bytes()
    assert len(a) > 1000 and a == b


def test_vtu_without_wall_distance_and_gas(afx, orc, tmp_path):
    # no wall distance: zeros, as a mesh whose compute_wall_dist never ran;
    # another gas changes pressure-derived fields only through gamma and R
    m, bcs = omesh_case(24, 12, split=True)
    om, s = _oracle_state(orc, m, bcs, iters=3)
    q = s.q()
    gm = afx.mesh.from_arrays(m)
    gm.write_vtu(tmp_path / "a.vtu", q, None, gamma=1.3, R=0.5)
    om.save_vtu(tmp_path / "b.vtu", q, None, gamma=1.3, R=0.5)
    assert (tmp_path / "a.vtu").read_bytes() == (tmp_path / "b.vtu").read_bytes()


def test_vtu_structure(afx, tmp_path):
    # an independent reading of the file: counts, offsets, cell types, fields
    m, bcs = omesh_case(16, 8, split=True)
    gm = afx.mesh.from_arrays(m)
    n = gm.nRealCells
    q = np.tile([1.4, 0.7, 0.1, 2.7], n)
    gm.write_vtu(tmp_path / "s.vtu", q)
    root = ET.parse(tmp_path / "s.vtu").getroot()
    piece = root.find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfCells")) == n and int(piece.get("NumberOfPoints")) == len(m["x"])
    arrays = {a.get("Name"): np.array(a.text.split(), float) for a in piece.iter("DataArray") if a.get("Name")}
    ntri = int((np.asarray(m["cells"])[:, 3] < 0).sum())
    assert len(arrays["types"]) == n and int((arrays["types"] == 5).sum()) == ntri
    assert arrays["offsets"][-1] == 3 * ntri + 4 * (n - ntri) == len(arrays["connectivity"])
    assert np.allclose(arrays["Density"], 1.4) and np.allclose(arrays["Wall Distance"], 0.0)
    p = 0.4 * (2.7 - 0.5 / 1.4 * (0.7 ** 2 + 0.1 ** 2))
    assert np.allclose(arrays["Pressure"], p) and np.allclose(arrays["Temperature"], p / (0.71428571428 * 1.4))
    assert np.allclose(arrays["Velocity"].reshape(-1, 3), [0.5, 0.1 / 1.4, 0.0])


def test_vtu_rejects_bad_sizes(afx, tmp_path):
    m, _ = omesh_case(16, 8)
    gm = afx.mesh.from_arrays(m)
    with pytest.raises(afx.AfxError) as e:
        gm.write_vtu(tmp_path / "x.vtu", np.zeros(5))
    assert e.value.code == 8
    with pytest.raises(afx.AfxError) as e:
        gm.write_vtu(tmp_path / "no_such_dir" / "x.vtu", np.ones(4 * gm.nRealCells))
    assert e.value.code == 1


@pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference examples not mounted")
@pytest.mark.parametrize("name", ["naca0012q_coarse.msh", "airfoil_demo_coarse.msh"])
def test_vtu_reference_meshes(afx, orc, tmp_path, name):
    # the reference's own gmsh files through both loaders, a generic state
    path = os.path.join(REF_MESHES, name)
    gm, om = afx.mesh(path), orc.Mesh.load(path)
    n = gm.nRealCells
    rng = np.random.default_rng(2)
    q = np.tile([1.4, 0.7, 0.05, 2.8], n) * (1 + 0.01 * rng.standard_normal(4 * n))
    wd = rng.uniform(0, 3, n)
    gm.write_vtu(tmp_path / "a.vtu", q, wd)
    om.save_vtu(tmp_path / "b.vtu", q, wd)
    assert (tmp_path / "a.vtu").read_bytes() == (tmp_path / "b.vtu").read_bytes()


@pytest.mark.gpu
def test_save_vtu_of_a_solver_matches_oracle(afx, orc, tmp_path):
    # save(filename, solver): the GPU state after FP64 iterations (bit-exact
    # to the oracle's) and the GPU wall distance (mesh.h:794-830)
    from tests.cases import gpu_solver
    m, bcs = omesh_case(32, 16, split=False)
    g = gpu_solver(afx, m, bcs)
    g.init()
    g.iterate(10)
    afx.save(tmp_path / "g.vtu", g)
    om, s = _oracle_state(orc, m, bcs, iters=10)
    om.save_vtu(tmp_path / "o.vtu", s.q(), s.wall_distance()[: om.n_real])
    assert (tmp_path / "g.vtu").read_bytes() == (tmp_path / "o.vtu").read_bytes()


def test_vtu_extreme_values_match_oracle(afx, orc, tmp_path):
    # long fixed-notation numbers (1e300 has 301 integer digits), tiny ones,
    # negative zero: the library's formatting equals the stream formatting
    m, bcs = omesh_case(16, 8, split=True)
    gm, om = afx.mesh.from_arrays(m), orc.Mesh.from_arrays(m)
    n = gm.nRealCells
    q = np.tile([1.4, 0.7, 0.05, 2.8], n)
    q[0::4][:3] = [1e300, 1e-300, 3.0]
    q[1::4][:3] = [-0.0, 1e150, -1e-200]
    wd = np.full(n, 0.0)
    wd[:4] = [-0.0, 1e300, 5e-324, 0.1]
    gm.write_vtu(tmp_path / "a.vtu", q, wd)
    om.save_vtu(tmp_path / "b.vtu", q, wd)
    assert (tmp_path / "a.vtu").read_bytes() == (tmp_path / "b.vtu").read_bytes()
