"""The C++ layer (include/afx_rans.hpp) compiles and links against the
library, and on the GPU its alpha sweep gives the same polar as the Python
mirror of the same calls."""
import os
import subprocess

import numpy as np
import pytest

from aeroflex_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

INI = """[rans-gas]
gamma = 1.4
R = 0.71428571428

[rans-bc]
<
    name = farfield,
    type = farfield,
    T = 1,
    mach = 0.5,
    angle = 0.0,
    p = 1,
>
<name = wall, type = slip-wall>

[rans-alphas]
alpha_start = 0.0
alpha_end = 2.0
alpha_step = 2.0

[rans-solver]
solver = explicit
viscosity = inviscid
gradient = green-gauss
second_order = true
relaxation = 0.9
start_cfl = 1.5
slope_cfl = 0.0
max_cfl = 1.5
tolerance = 1e-3
rhs_iterations = 5
max_iterations = 300
limiter_k = 5.0
"""


def _build(afx, tmp_path):
    exe = str(tmp_path / "polar_sweep")
    lib = os.path.dirname(afx.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "aeroflex_gb300", "cpp", "polar_sweep.cpp"), "-o", exe,
                           "-L", lib, "-lafx_rans", "-Wl,-rpath," + lib])
    return exe


def test_cpp_layer_builds(afx, tmp_path):
    assert os.path.exists(_build(afx, tmp_path))


@pytest.mark.gpu
def test_cpp_polar_matches_python(afx, tmp_path):
    exe = _build(afx, tmp_path)
    m = meshgen.airfoil_omesh(48, 24, split=False)
    msh = str(tmp_path / "o.msh")
    meshgen.write_gmsh(msh, m)
    ini = tmp_path / "c.ini"
    ini.write_text(INI)
    out = subprocess.run([exe, str(ini), msh], capture_output=True, text=True, check=True).stdout.split("\n")
    rows = [list(map(float, l.split())) for l in out if l and not l.startswith("iterations")]
    st = afx.Settings.from_ini(str(ini))
    g = afx.Solver(afx.mesh(msh), st)
    g.set_farfield("farfield", 0.5, 0.0)
    g.init()
    for a, cl, cd, cm in rows:
        g.set_farfield("farfield", 0.5, a * 0.01745)
        g.run_solver()
        w = afx.get_wall_profile(g, "wall")
        np.testing.assert_array_equal([cl, cd, cm], [w["cl"], w["cd"], w["cm"]])


@pytest.mark.gpu
def test_cpp_two_level_polar_matches_python(afx, tmp_path):
    # the reference's coarse -> mid sequence (rans.h:84-85, multigrid.h:295-363)
    exe = _build(afx, tmp_path)
    paths = []
    for k, (ns, nr) in enumerate(((24, 12), (48, 24))):
        p = str(tmp_path / ("l%d.msh" % k))
        meshgen.write_gmsh(p, meshgen.airfoil_omesh(ns, nr, split=False))
        paths.append(p)
    ini = tmp_path / "c.ini"
    ini.write_text(INI)
    out = subprocess.run([exe, str(ini)] + paths, capture_output=True, text=True, check=True).stdout.split("\n")
    rows = [list(map(float, l.split())) for l in out if l and not l.startswith("iterations")]
    st = afx.Settings.from_ini(str(ini))
    lv = [afx.Solver(afx.mesh(p), st) for p in paths]
    lv[0].set_farfield("farfield", 0.5, 0.0)
    lv[0].init()
    for a, cl, cd, cm in rows:
        for g in lv:
            g.set_farfield("farfield", 0.5, a * 0.01745)
        lv[0].run_solver()
        lv[1].prolongate_from(lv[0])
        lv[1].run_solver()
        w = afx.get_wall_profile(lv[1], "wall")
        np.testing.assert_array_equal([cl, cd, cm], [w["cl"], w["cd"], w["cm"]])
