"""Pins of the reference's own results (tests/golden/ref_pins.json).

Each pin is a small seeded run — generated mesh, boundary conditions,
settings, a sequence of calls — whose results the reference's own code
produced (oracle/_ref, built from the unmodified rans headers; fixture
script tests/golden/make_ref_golden.py).  The same runs are repeated through
three drivers with one interface:

- ``RefDriver``: the reference's code (where its source tree is present);
- ``OracleDriver``: the CPU restatement;
- ``GpuDriver``: the CUDA library through its C ABI.

Arrays are pinned by the SHA-256 of their little-endian float64 bytes
(bit-exact); norms, histories and forces, which the GPU sums in another
order, are pinned by value.
"""
import hashlib
import os
import tempfile

import numpy as np

from aeroflex_gb300 import meshgen

DEG = 0.01745  # the reference's degree factor (rans.h:88,94)
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PINS_JSON = os.path.join(GOLDEN, "ref_pins.json")
MID_MESH_NPZ = os.path.join(GOLDEN, "naca0012q_mid_arrays.npz")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, "<f8").tobytes()).hexdigest()


def airfoil_bcs(mach, aoa_deg, wall="slip-wall"):
    return {"farfield": dict(type="farfield", T=1.0, mach=mach, angle=aoa_deg * DEG, p=1.0), "wall": dict(type=wall)}


def mid_mesh_arrays():
    """The reference's examples/rans/naca0012q_mid.msh as its reader numbers
    it (nodes, cells, boundary edges and patches), from the committed
    fixture."""
    z = np.load(MID_MESH_NPZ)
    return dict(x=z["x"], y=z["y"], cells=z["cells"], bedges=z["bedges"], bpatch=z["bpatch"],
                names=[str(s) for s in z["names"]])


# ---------------------------------------------------------------- drivers
class RefDriver:
    """The reference's own code (oracle/ref.py); meshes go through a gmsh 4.1
    file and the reference's reader, settings through its INI reader."""
    name = "reference"

    def __init__(self):
        from oracle import ref
        self.ref = ref
        self.dir = tempfile.mkdtemp()
        self.n = 0

    def _msh(self, m):
        self.n += 1
        p = os.path.join(self.dir, "m%d.msh" % self.n)
        meshgen.write_gmsh(p, m)
        return p

    def solver(self, m, bcs, limiter="venkatakrishnan", mu_L=None, **st):
        old = self.ref.use_variant("michalak" if limiter == "michalak" else "")
        try:
            c = self.ref.Case(self.ref.ini_text(bcs, **st), self._msh(m), mu_L=mu_L or 0.0)
        finally:
            self.ref.use_variant(old)
        return RefSolver(c)

    def levels(self, meshes, bcs, **st):
        c = self.ref.Case(self.ref.ini_text(bcs, **st), [self._msh(m) for m in meshes])
        return c


class RefSolver:
    def __init__(self, c):
        self.c = c

    def init(self):
        self.c.init()

    def set_q(self, q):
        self.c.set_q(q)

    def q(self):
        return self.c.q()

    def residual(self):
        return self.c.residual()

    def iterate(self, n):
        return float(self.c.iterate(n)[-1])

    def wall_profile(self, patch="wall"):
        return self.c.wall_profile(patch)

    def run_solver(self):
        st, h = self.c.run_solver()
        return st, h

    def uniform_residual(self):
        return self.c.uniform_residual()

    def rhs(self):
        return self.c.residual()  # fillRhoRHS for an implicit case

    def wall_distance(self):
        return self.c.wall_distance()


class OracleDriver:
    name = "oracle"

    def __init__(self, orc):
        self.orc = orc

    def solver(self, m, bcs, mu_L=None, start_cfl=1.0, solver="explicit", **st):
        if mu_L:
            st["mu_L"] = mu_L
        s = self.orc.Solver(self.orc.Mesh.from_arrays(m), self.orc.default_settings(cfl=start_cfl, **st), bcs)
        return OracleSolver(s)


class OracleSolver:
    def __init__(self, s):
        self.s = s

    def init(self):
        self.s.init()

    def set_q(self, q):
        self.s.set_q(q)

    def q(self):
        return self.s.q()

    def residual(self):
        return self.s.residual()

    def iterate(self, n):
        return float(self.s.iterate(n)[-1])

    def wall_profile(self, patch="wall"):
        return self.s.wall_profile(patch)

    def run_solver(self):
        _, _, h = self.s.run_solver()
        return 0, h

    def uniform_residual(self):
        return self.s.uniform_residual()

    def wall_distance(self):
        return self.s.wall_distance()


class GpuDriver:
    name = "gpu"

    def __init__(self, afx, precision="fp64", **extra):
        self.afx = afx
        self.precision = precision
        self.extra = extra

    def solver(self, m, bcs, mu_L=None, solver="explicit", **st):
        s = self.afx.Settings()
        s.set("solver", solver)
        s.set("precision", self.precision)
        if mu_L:
            s.set("mu_L", mu_L)
        for k, v in list(st.items()) + list(self.extra.items()):
            s.set(k, (1.0 if v else 0.0) if isinstance(v, bool) else v)
        for name, b in bcs.items():
            s.set_bc(name, b["type"], b.get("T", 1.0), b.get("mach", 0.2), b.get("angle", 0.0), b.get("p", 1.0))
        return GpuSolver(self.afx, self.afx.Solver(self.afx.mesh.from_arrays(m), s))


class GpuSolver:
    def __init__(self, afx, s):
        self.afx = afx
        self.s = s

    def init(self):
        self.s.init()

    def set_q(self, q):
        self.s.set_q(q)

    def q(self):
        return self.s.get_q()

    def residual(self):
        return self.s.residual()

    def iterate(self, n):
        return self.s.iterate(n)

    def wall_profile(self, patch="wall"):
        return self.afx.get_wall_profile(self.s, patch)

    def run_solver(self):
        self.s.run_solver()
        return 0, self.s.history()

    def uniform_residual(self):
        return None

    def rhs(self):
        return self.s.implicit_rhs()

    def wall_distance(self):
        return self.s.wall_distance()


# ------------------------------------------------------------------- pins
def _forces(w):
    return [float(w["cl"]), float(w["cd"]), float(w["cm"])]


def explicit_pins(drv):
    """The explicit path (residual, iterations, forces, run_solver, wall
    distance) on small generated meshes."""
    out = {}
    # a C1-shaped airfoil case in miniature: split-triangle O-mesh
    m = meshgen.airfoil_omesh(32, 16)
    bcs = airfoil_bcs(0.5, 1.25)
    s = drv.solver(m, bcs, start_cfl=1.0)
    s.init()
    out["omesh_split_R0"] = sha(s.residual())
    norms = {}
    done = 0
    for n in (1, 2, 10, 100):
        norms[str(n)] = s.iterate(n - done)
        done = n
        out["omesh_split_q%d" % n] = sha(s.q())
    out["omesh_split_R100"] = sha(s.residual())
    out["omesh_split_norms"] = norms
    w = s.wall_profile("wall")
    out["omesh_split_forces100"] = _forces(w)
    out["omesh_split_cp100"] = sha(w["cp"])
    # shuffled jittered channel with the density bump
    m = meshgen.channel(32, 16, jitter=0.2, seed=1, shuffle_seed=2)
    bcs = {"farfield": dict(type="farfield", T=1.0, mach=0.3, angle=0.0, p=1.0), "wall": dict(type="slip-wall")}
    s = drv.solver(m, bcs, start_cfl=1.0)
    s.init()
    s.set_q(meshgen.density_bump_state(m, mach=0.3))
    out["channel_R0"] = sha(s.residual())
    s.iterate(10)
    out["channel_q10"] = sha(s.q())
    out["channel_R10"] = sha(s.residual())
    # scheme variants on quads and triangles
    for tag, kw, wall in [("laminar", dict(viscosity="laminar", mu_L=1e-3), "wall"),
                          ("lsq", dict(gradient="least-squares"), "slip-wall"),
                          ("first_order", dict(second_order=False), "slip-wall"),
                          ("laminar_lsq", dict(viscosity="laminar", gradient="least-squares", mu_L=1e-3), "wall"),
                          ("michalak", dict(limiter="michalak"), "slip-wall"),
                          ("michalak_laminar", dict(limiter="michalak", viscosity="laminar", mu_L=1e-3), "wall")]:
        for shape, mm in (("tri", meshgen.airfoil_omesh(24, 12)), ("quad", meshgen.airfoil_omesh(24, 12, split=False))):
            s = drv.solver(mm, airfoil_bcs(0.4, 3.0, wall), start_cfl=1.0, **kw)
            s.init()
            s.iterate(10)
            out["%s_%s_q10" % (tag, shape)] = sha(s.q())
            out["%s_%s_R10" % (tag, shape)] = sha(s.residual())
    # run_solver: convergence loop, history, uniform-residual normaliser
    m = meshgen.airfoil_omesh(24, 12, split=False)
    s = drv.solver(m, airfoil_bcs(0.5, 2.0), start_cfl=1.5, tolerance=1e-3, max_iterations=1500)
    s.init()
    u = s.uniform_residual()
    if u is not None:
        out["run_solver_uniform_residual"] = u
    _, h = s.run_solver()
    out["run_solver_history"] = [float(v) for v in h]
    out["run_solver_q"] = sha(s.q())
    out["run_solver_forces"] = _forces(s.wall_profile("wall"))
    # wall distance (mesh.h:794-830) to a no-slip wall
    m = meshgen.airfoil_omesh(32, 16)
    s = drv.solver(m, airfoil_bcs(0.5, 1.25, "wall"), start_cfl=1.0)
    out["wall_distance"] = sha(s.wall_distance())
    # the reference's own example mesh, explicit path
    m = mid_mesh_arrays()
    s = drv.solver(m, airfoil_bcs(0.2, 4.0), start_cfl=1.0)
    s.init()
    out["naca0012q_mid_R0"] = sha(s.residual())
    out["naca0012q_mid_norm5"] = s.iterate(5)
    out["naca0012q_mid_q5"] = sha(s.q())
    out["naca0012q_mid_R5"] = sha(s.residual())
    return out


# implicit runs: the converged fixed point of the reference's default
# (implicit) solver; conf.ini's CFL ramp (start 40, slope 50, max 100) and
# tolerance tightened to 1e-10 so that the converged state does not depend
# on the linear solver's iterates
IMPLICIT = dict(solver="implicit", start_cfl=40.0, slope_cfl=50.0, max_cfl=100.0, tolerance=1e-10,
                rhs_iterations=5, relaxation=0.9)


def c1_quad_mesh():
    """Config 1's O-mesh (129 cosine-spaced surface nodes x 65 layers to 20
    chords) with its quads kept whole: on the 2-triangle split the
    reference's second-order scheme diverges (its explicit and implicit
    solvers both)."""
    return meshgen.airfoil_omesh(128, 64, split=False)


def implicit_polar_cases():
    """(tag, mesh arrays, Mach, angles in degrees): config 1 on quads, and
    the reference's examples/rans/naca0012q_mid.msh at examples/conf.ini's
    Mach 0.2 and angles 1, 4, 7 (warm-started from one angle to the next, as
    Rans::run_airfoil does)."""
    return [("c1_quads", c1_quad_mesh(), 0.5, [1.25]),
            ("naca0012q_mid", mid_mesh_arrays(), 0.2, [1.0, 4.0, 7.0])]


def perturbed(q, amp=0.02):
    """A deterministic non-uniform state near q: each entry scaled by
    1 + amp sin(0.37 i)."""
    i = np.arange(q.size, dtype=np.float64)
    return q * (1.0 + amp * np.sin(0.37 * i))


def implicit_rhs_pins(drv):
    """fillRhoRHS (solver.h:1079-1152) of perturbed states: second order
    (Green-Gauss, least squares) and first order, inviscid and laminar."""
    out = {}
    for tag, kw, wall in [("gg", {}, "slip-wall"), ("lsq", dict(gradient="least-squares"), "slip-wall"),
                          ("first_order", dict(second_order=False), "slip-wall"),
                          ("laminar", dict(viscosity="laminar", mu_L=1e-3), "wall")]:
        for shape, mm in (("tri", meshgen.airfoil_omesh(24, 12)), ("quad", meshgen.airfoil_omesh(24, 12, split=False))):
            s = drv.solver(mm, airfoil_bcs(0.4, 3.0, wall), solver="implicit", start_cfl=40.0, **kw)
            s.init()
            s.set_q(perturbed(s.q()))
            out["rhs_%s_%s" % (tag, shape)] = sha(s.rhs())
    return out
