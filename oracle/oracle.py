"""ctypes wrapper over the CPU oracle (test infrastructure only).

Used by tests/ as the checker, by __graft_entry__.smoke() and by the
CPU-baseline leg of bench.py.  Never imported by the product package.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

BC_TYPES = {"farfield": 1, "slip-wall": 2, "wall": 3, "inlet-outlet": 4}
VISCOSITY = {"inviscid": 0, "laminar": 1, "spalart-allmaras": 2, "spallart-allmaras": 3}


class OrcSettings(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("R", ctypes.c_double), ("mu_L", ctypes.c_double),
                ("Pr_L", ctypes.c_double), ("Pr_T", ctypes.c_double),
                ("viscosity", ctypes.c_int), ("gradient", ctypes.c_int), ("second_order", ctypes.c_int),
                ("limiter", ctypes.c_int),
                ("limiter_k", ctypes.c_double), ("cfl", ctypes.c_double), ("relaxation", ctypes.c_double),
                ("tolerance", ctypes.c_double), ("max_iterations", ctypes.c_int)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, cp, ip, dp = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
        L.orc_last_error.restype = cp
        L.orc_mesh_load.restype = vp
        L.orc_mesh_load.argtypes = [cp]
        L.orc_mesh_from_arrays.restype = vp
        L.orc_mesh_from_arrays.argtypes = [ip, vp, vp, ip, vp, ip, vp, vp, cp]
        L.orc_mesh_free.argtypes = [vp]
        L.orc_mesh_counts.argtypes = [vp, vp]
        L.orc_mesh_get.restype = ctypes.c_longlong
        L.orc_mesh_get.argtypes = [vp, cp, vp]
        L.orc_mesh_get_int.restype = ctypes.c_longlong
        L.orc_mesh_get_int.argtypes = [vp, cp, vp]
        L.orc_mesh_boundary_name.restype = cp
        L.orc_mesh_boundary_name.argtypes = [vp, ip]
        L.orc_solver_create.restype = vp
        L.orc_solver_create.argtypes = [vp, ctypes.POINTER(OrcSettings), ip, vp, vp, vp]
        L.orc_solver_free.argtypes = [vp]
        L.orc_init.argtypes = [vp]
        L.orc_refill_bcs.argtypes = [vp]
        L.orc_set_farfield.argtypes = [vp, cp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_set_q.argtypes = [vp, vp]
        L.orc_set_nu.argtypes = [vp, vp]
        L.orc_sa_source.argtypes = [ctypes.c_double] * 4 + [vp, vp]
        L.orc_prolongate.argtypes = [vp, vp]
        L.orc_set_threads.argtypes = [ip]
        L.orc_wall_distance.restype = ctypes.c_longlong
        L.orc_wall_distance.argtypes = [vp, vp]
        L.orc_get.restype = ctypes.c_longlong
        L.orc_get.argtypes = [vp, cp, vp]
        L.orc_residual.argtypes = [vp, vp]
        L.orc_iterate.argtypes = [vp, ip, vp]
        L.orc_uniform_residual.restype = ctypes.c_double
        L.orc_uniform_residual.argtypes = [vp]
        L.orc_run_solver.argtypes = [vp, vp, vp, vp, ip, vp]
        L.orc_wall_profile.argtypes = [vp, cp, vp, vp, ip, vp]
        L.orc_time_iterations.restype = ctypes.c_double
        L.orc_time_iterations.argtypes = [vp, ip]
        L.orc_time_residuals.restype = ctypes.c_double
        L.orc_time_residuals.argtypes = [vp, ip]
        d = ctypes.c_double
        L.orc_face_flux.argtypes = [d, ip, ip, d, d, vp, vp, vp, vp, vp]
        L.orc_save_vtu.argtypes = [vp, vp, vp, d, d, cp]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def face_flux(qL, qR, nx, ny, gamma=1.4, visc=0, bc="internal", gx=None, gy=None):
    """One restated face flux F (physics.h:160-530), not multiplied by length."""
    qL = np.ascontiguousarray(qL, np.float64)
    qR = np.ascontiguousarray(qR, np.float64)
    gx = np.zeros(4) if gx is None else np.ascontiguousarray(gx, np.float64)
    gy = np.zeros(4) if gy is None else np.ascontiguousarray(gy, np.float64)
    f = np.empty(4)
    t = 0 if bc == "internal" else BC_TYPES[bc]
    lib().orc_face_flux(gamma, visc, t, nx, ny, _ptr(qL), _ptr(qR), _ptr(gx), _ptr(gy), _ptr(f))
    return f


class Mesh:
    """Restated `rans::mesh` (mesh.h:198-273)."""

    def __init__(self, handle):
        if not handle:
            raise RuntimeError("oracle mesh: " + lib().orc_last_error().decode())
        self.h = handle
        c = np.zeros(5, np.int64)
        lib().orc_mesh_counts(self.h, _ptr(c))
        self.n_real, self.n_tot, self.n_edges, self.n_boundary, self.n_nodes = (int(v) for v in c)

    @classmethod
    def load(cls, path):
        return cls(lib().orc_mesh_load(str(path).encode()))

    @classmethod
    def from_arrays(cls, m):
        x = np.ascontiguousarray(m["x"], np.float64)
        y = np.ascontiguousarray(m["y"], np.float64)
        cells = np.ascontiguousarray(m["cells"], np.int32)
        be = np.ascontiguousarray(m["bedges"], np.int32)
        bp = np.ascontiguousarray(m["bpatch"], np.int32)
        names = "\n".join(m["names"]).encode()
        h = lib().orc_mesh_from_arrays(len(x), _ptr(x), _ptr(y), len(cells), _ptr(cells), len(be), _ptr(be),
                                       _ptr(bp), names)
        return cls(h)

    def get(self, what):
        n = lib().orc_mesh_get(self.h, what.encode(), None)
        if n < 0:
            raise KeyError(what)
        out = np.empty(n, np.float64)
        lib().orc_mesh_get(self.h, what.encode(), _ptr(out))
        return out

    def get_int(self, what):
        n = lib().orc_mesh_get_int(self.h, what.encode(), None)
        if n < 0:
            raise KeyError(what)
        out = np.empty(n, np.int64)
        lib().orc_mesh_get_int(self.h, what.encode(), _ptr(out))
        return out

    def boundary_names(self):
        return [lib().orc_mesh_boundary_name(self.h, b).decode() for b in range(self.n_boundary)]

    def save_vtu(self, path, q, wall_dist=None, gamma=1.4, R=0.71428571428):
        """save (post.h:58-180) of state q (4 per real cell) on this mesh."""
        q = np.ascontiguousarray(q, np.float64)
        wd = None if wall_dist is None else np.ascontiguousarray(wall_dist, np.float64)
        if lib().orc_save_vtu(self.h, _ptr(q), None if wd is None else _ptr(wd), float(gamma), float(R),
                              str(path).encode()):
            raise OSError("oracle: cannot write " + str(path))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_mesh_free(self.h)
            self.h = None


def default_settings(**kw):
    """Settings defaults of core.h:166-199, explicit solver."""
    s = dict(gamma=1.4, R=0.71428571428, mu_L=1e-5, Pr_L=0.72, Pr_T=0.9, viscosity="inviscid",
             gradient="green-gauss", second_order=True, limiter="venkatakrishnan", limiter_k=5.0, cfl=1.0,
             relaxation=0.9, tolerance=1e-4, max_iterations=300)
    s.update(kw)
    return s


class Solver:
    """Restated `rans::explicitSolver` (solver.h:721-828) plus run_solver and get_wall_profile."""

    def __init__(self, mesh, settings, bcs):
        self.mesh = mesh
        st = OrcSettings(settings["gamma"], settings["R"], settings["mu_L"], settings["Pr_L"], settings["Pr_T"],
                         VISCOSITY[settings["viscosity"]],
                         0 if settings["gradient"] == "least-squares" else 1,
                         1 if settings["second_order"] else 0,
                         1 if settings["limiter"] == "michalak" else 0,
                         settings["limiter_k"], settings["cfl"], settings["relaxation"], settings["tolerance"],
                         settings["max_iterations"])
        names = (ctypes.c_char_p * len(bcs))(*[n.encode() for n in bcs])
        types = np.array([BC_TYPES.get(b["type"], 0) for b in bcs.values()], np.int32)
        vals = np.array([[b.get("T", 1.0), b.get("mach", 0.2), b.get("angle", 0.0), b.get("p", 1.0)]
                         for b in bcs.values()], np.float64).reshape(-1)
        h = lib().orc_solver_create(mesh.h, ctypes.byref(st), len(bcs), ctypes.cast(names, ctypes.c_void_p),
                                    _ptr(types), _ptr(vals))
        if not h:
            raise RuntimeError("oracle solver: " + lib().orc_last_error().decode())
        self.h = h
        self.n_real = mesh.n_real

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_solver_free(self.h)
            self.h = None

    def init(self):
        lib().orc_init(self.h)

    def refill_bcs(self):
        lib().orc_refill_bcs(self.h)

    def set_farfield(self, patch, mach, angle, T=1.0, p=1.0):
        if lib().orc_set_farfield(self.h, patch.encode(), mach, angle, T, p):
            raise RuntimeError(lib().orc_last_error().decode())

    def wall_distance(self):
        """mesh::compute_wall_dist (mesh.h:794-830), all cells."""
        n = lib().orc_wall_distance(self.h, None)
        out = np.empty(n, np.float64)
        lib().orc_wall_distance(self.h, _ptr(out))
        return out

    def prolongate_from(self, coarse):
        """Grid-sequencing transfer (multigrid.h:99-178, 295-363): this
        solver's state from the coarse solver's."""
        lib().orc_prolongate(coarse.h, self.h)

    def set_q(self, q):
        q = np.ascontiguousarray(q, np.float64).reshape(-1)
        assert q.size == 4 * self.n_real
        lib().orc_set_q(self.h, _ptr(q))

    def get(self, what):
        n = lib().orc_get(self.h, what.encode(), None)
        out = np.empty(n, np.float64)
        lib().orc_get(self.h, what.encode(), _ptr(out))
        return out

    def q(self):
        return self.get("q")[: 4 * self.n_real].copy()

    def set_nu(self, nu):
        """nu~ of the real cells (Spalart-Allmaras)."""
        nu = np.ascontiguousarray(nu, np.float64).reshape(-1)
        assert nu.size == self.n_real
        lib().orc_set_nu(self.h, _ptr(nu))

    def nu(self):
        return self.get("nu")[: self.n_real].copy()

    def nu_residual(self):
        """nuW of the last residual or stage (per real cell)."""
        return self.get("nuW")[: self.n_real].copy()

    def residual(self):
        R = np.empty(4 * self.n_real, np.float64)
        if lib().orc_residual(self.h, _ptr(R)):
            raise RuntimeError(lib().orc_last_error().decode())
        return R

    def iterate(self, n):
        norms = np.empty(n, np.float64)
        if lib().orc_iterate(self.h, n, _ptr(norms)):
            raise RuntimeError(lib().orc_last_error().decode())
        return norms

    def uniform_residual(self):
        return lib().orc_uniform_residual(self.h)

    def run_solver(self, hist_cap=100000):
        it = ctypes.c_int()
        err = ctypes.c_double()
        hist = np.empty(hist_cap, np.float64)
        nh = ctypes.c_int()
        if lib().orc_run_solver(self.h, ctypes.byref(it), ctypes.byref(err), _ptr(hist), hist_cap,
                                ctypes.byref(nh)):
            raise RuntimeError(lib().orc_last_error().decode())
        return it.value, err.value, hist[: min(nh.value, hist_cap)].copy()

    def wall_profile(self, patch="wall", cap=1 << 20):
        out = np.empty(3, np.float64)
        cp = np.empty(cap, np.float64)
        n = ctypes.c_int()
        if lib().orc_wall_profile(self.h, patch.encode(), _ptr(out), _ptr(cp), cap, ctypes.byref(n)):
            raise RuntimeError(lib().orc_last_error().decode())
        return dict(cl=out[0], cd=out[1], cm=out[2], cp=cp[: n.value].copy())

    def time_iterations(self, n):
        return lib().orc_time_iterations(self.h, n)

    def time_residuals(self, n):
        return lib().orc_time_residuals(self.h, n)


def sa_source(nut, nul, omega, d):
    """Spalart-Allmaras source P - D of one cell and its derivative in nu~."""
    src, dsrc = ctypes.c_double(), ctypes.c_double()
    lib().orc_sa_source(float(nut), float(nul), float(omega), float(d), ctypes.byref(src), ctypes.byref(dsrc))
    return src.value, dsrc.value


def set_threads(n):
    """OpenMP threads of the oracle's per-cell loops (0: all host threads)."""
    lib().orc_set_threads(int(n))
