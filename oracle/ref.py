"""ctypes wrapper over oracle/_ref/libref.so: the reference's own rans code
built from its unmodified headers (test infrastructure only; see
oracle/ref_capi.cpp and oracle/build_ref.py).

Used by tests/ to pin the oracle restatement and the committed golden
fixtures to the reference itself, and by tests/golden/make_ref_golden.py.
``available()`` is False where the reference tree is absent; the tests that
need it then skip.
"""
import ctypes
import os
import tempfile

import numpy as np

from . import build_ref as _build

_libs = {}
_variant = ""


def available():
    try:
        lib()
        return True
    except Exception:
        return False


def use_variant(variant):
    """Selects the build the next objects use: "" (the reference's default
    Venkatakrishnan limiter) or "michalak" (its RANS_MICHALAK_LIMITER
    build).  Returns the previous selection."""
    global _variant
    old, _variant = _variant, variant
    return old


def lib(variant=None):
    variant = _variant if variant is None else variant
    if variant not in _libs:
        path = _build.build(variant=variant)
        if not path:
            raise RuntimeError("the reference tree is not available")
        L = ctypes.CDLL(path)
        vp, cp, ip, d = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_double
        L.ref_last_error.restype = cp
        L.ref_mesh_load.restype = vp
        L.ref_mesh_load.argtypes = [cp]
        L.ref_mesh_free.argtypes = [vp]
        L.ref_mesh_counts.argtypes = [vp, vp]
        L.ref_mesh_get.restype = ctypes.c_longlong
        L.ref_mesh_get.argtypes = [vp, cp, vp]
        L.ref_mesh_get_int.restype = ctypes.c_longlong
        L.ref_mesh_get_int.argtypes = [vp, cp, vp]
        L.ref_mesh_boundary_name.restype = cp
        L.ref_mesh_boundary_name.argtypes = [vp, ip]
        L.ref_case_create.restype = vp
        L.ref_case_create.argtypes = [cp, cp, d]
        L.ref_case_free.argtypes = [vp]
        L.ref_case_levels.argtypes = [vp, vp]
        L.ref_init.argtypes = [vp, ip]
        L.ref_refill_bcs.argtypes = [vp, ip]
        L.ref_set_q.argtypes = [vp, ip, vp]
        L.ref_get.restype = ctypes.c_longlong
        L.ref_get.argtypes = [vp, ip, cp, vp]
        L.ref_wall_distance.restype = ctypes.c_longlong
        L.ref_wall_distance.argtypes = [vp, ip, vp]
        L.ref_residual.argtypes = [vp, ip, vp]
        L.ref_iterate.argtypes = [vp, ip, ip, vp]
        L.ref_uniform_residual.restype = d
        L.ref_uniform_residual.argtypes = [vp, ip]
        L.ref_run_solver.argtypes = [vp, ip, vp, vp, ip, vp]
        L.ref_run.argtypes = [vp, ip, vp, ip, vp]
        L.ref_set_angle.argtypes = [vp, cp, d]
        L.ref_wall_profile.argtypes = [vp, ip, cp, vp, vp, ip, vp]
        L.ref_implicit_block.argtypes = [vp, ip, d, ip, ip, vp, ip]
        L.ref_face_flux.argtypes = [d, ip, ip, d, d, vp, vp, vp, vp, vp]
        _libs[variant] = L
    return _libs[variant]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(rc):
    if rc:
        raise RuntimeError("reference: " + lib().ref_last_error().decode())


def face_flux(qL, qR, nx, ny, gamma=1.4, visc=0, bc="internal", gx=None, gy=None):
    """One face flux of the reference's functors (physics.h:160-530)."""
    types = {"internal": 0, "farfield": 1, "slip-wall": 2, "wall": 3}
    a = [np.ascontiguousarray(v, np.float64) for v in (qL, qR, np.zeros(4) if gx is None else gx,
                                                      np.zeros(4) if gy is None else gy)]
    f = np.empty(4)
    lib().ref_face_flux(gamma, visc, types[bc], nx, ny, *[_ptr(v) for v in a], _ptr(f))
    return f


class Mesh:
    """rans::mesh read by the reference's own gmsh 4.1 reader (mesh.h:250)."""

    def __init__(self, path):
        self.L = lib()
        h = self.L.ref_mesh_load(str(path).encode())
        if not h:
            raise RuntimeError("reference mesh: " + self.L.ref_last_error().decode())
        self.h = h
        c = np.zeros(5, np.int64)
        self.L.ref_mesh_counts(self.h, _ptr(c))
        self.n_real, self.n_tot, self.n_edges, self.n_boundary, self.n_nodes = (int(v) for v in c)

    def get(self, what):
        n = self.L.ref_mesh_get(self.h, what.encode(), None)
        if n < 0:
            raise KeyError(what)
        out = np.empty(n, np.float64)
        self.L.ref_mesh_get(self.h, what.encode(), _ptr(out))
        return out

    def get_int(self, what):
        n = self.L.ref_mesh_get_int(self.h, what.encode(), None)
        if n < 0:
            raise KeyError(what)
        out = np.empty(n, np.int64)
        self.L.ref_mesh_get_int(self.h, what.encode(), _ptr(out))
        return out

    def boundary_names(self):
        return [self.L.ref_mesh_boundary_name(self.h, b).decode() for b in range(self.n_boundary)]

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_mesh_free(self.h)
            self.h = None


def ini_text(bcs, solver="explicit", gradient="green-gauss", viscosity="inviscid", second_order=True,
             relaxation=0.9, start_cfl=1.0, slope_cfl=50.0, max_cfl=100.0, tolerance=1e-4, rhs_iterations=5,
             max_iterations=300, limiter_k=5.0, gamma=1.4, R=0.71428571428):
    """The reference's INI layout (core.h:238-272) for these settings; bcs
    maps a patch name to dict(type=..., T, mach, angle, p)."""
    lines = ["[rans-gas]", "gamma = %r" % gamma, "R = %r" % R, "", "[rans-bc]"]
    for name, b in bcs.items():
        if b["type"] == "farfield":
            lines.append("<name = %s, type = farfield, T = %r, mach = %r, angle = %r, p = %r>"
                         % (name, b.get("T", 1.0), b.get("mach", 0.2), b.get("angle", 0.0), b.get("p", 1.0)))
        else:
            lines.append("<name = %s, type = %s>" % (name, b["type"]))
    lines += ["", "[rans-alphas]", "alpha_start = 1.0", "alpha_end = 7.0", "alpha_step = 3.0", "",
              "[rans-solver]", "solver = " + solver, "viscosity = " + viscosity, "gradient = " + gradient,
              "second_order = " + ("true" if second_order else "false"), "relaxation = %r" % relaxation,
              "start_cfl = %r" % start_cfl, "slope_cfl = %r" % slope_cfl, "max_cfl = %r" % max_cfl,
              "tolerance = %r" % tolerance, "rhs_iterations = %d" % rhs_iterations,
              "max_iterations = %d" % max_iterations, "limiter_k = %r" % limiter_k, ""]
    return "\n".join(lines)


class Case:
    """The reference's Settings (from an INI file), meshes and multigrid
    object (multigrid.h:58-97), one solver per grid level."""

    def __init__(self, ini, mesh_paths, mu_L=0.0):
        """ini: an INI file path, or INI text (written to a temporary file)."""
        tmp = None
        if "\n" in ini:
            fd, tmp = tempfile.mkstemp(suffix=".ini")
            with os.fdopen(fd, "w") as f:
                f.write(ini)
            ini = tmp
        try:
            paths = "\n".join(str(p) for p in ([mesh_paths] if isinstance(mesh_paths, (str, os.PathLike))
                                               else mesh_paths))
            self.L = lib()
            h = self.L.ref_case_create(str(ini).encode(), paths.encode(), float(mu_L))
        finally:
            if tmp:
                os.unlink(tmp)
        if not h:
            raise RuntimeError("reference case: " + self.L.ref_last_error().decode())
        self.h = h
        imp = ctypes.c_int()
        self.n_levels = self.L.ref_case_levels(self.h, ctypes.byref(imp))
        self.implicit = bool(imp.value)
        self.meshes = [Mesh(p) for p in paths.split("\n")]

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_case_free(self.h)
            self.h = None

    def _check(self, rc):
        if rc:
            raise RuntimeError("reference: " + self.L.ref_last_error().decode())

    def n_real(self, lvl=-1):
        return self.meshes[lvl].n_real

    def _lvl(self, lvl):
        return lvl % self.n_levels

    def init(self, lvl=-1):
        self._check(self.L.ref_init(self.h, self._lvl(lvl)))

    def refill_bcs(self, lvl=-1):
        self._check(self.L.ref_refill_bcs(self.h, self._lvl(lvl)))

    def set_q(self, q, lvl=-1):
        q = np.ascontiguousarray(q, np.float64).reshape(-1)
        assert q.size == 4 * self.n_real(lvl)
        self._check(self.L.ref_set_q(self.h, self._lvl(lvl), _ptr(q)))

    def get(self, what, lvl=-1):
        n = self.L.ref_get(self.h, self._lvl(lvl), what.encode(), None)
        if n < 0:
            raise KeyError(what)
        out = np.empty(n, np.float64)
        self.L.ref_get(self.h, self._lvl(lvl), what.encode(), _ptr(out))
        return out

    def q(self, lvl=-1):
        return self.get("q", lvl)[: 4 * self.n_real(lvl)].copy()

    def wall_distance(self, lvl=-1):
        n = self.L.ref_wall_distance(self.h, self._lvl(lvl), None)
        out = np.empty(n, np.float64)
        self.L.ref_wall_distance(self.h, self._lvl(lvl), _ptr(out))
        return out

    def residual(self, lvl=-1):
        R = np.empty(4 * self.n_real(lvl), np.float64)
        self._check(self.L.ref_residual(self.h, self._lvl(lvl), _ptr(R)))
        return R

    def iterate(self, n, lvl=-1):
        norms = np.empty(max(n, 1), np.float64)
        self._check(self.L.ref_iterate(self.h, self._lvl(lvl), n, _ptr(norms)))
        return norms[:n]

    def uniform_residual(self, lvl=-1):
        return self.L.ref_uniform_residual(self.h, self._lvl(lvl))

    def run_solver(self, lvl=-1, hist_cap=200000):
        st = ctypes.c_int()
        hist = np.empty(hist_cap, np.float64)
        nh = ctypes.c_int()
        self._check(self.L.ref_run_solver(self.h, self._lvl(lvl), ctypes.byref(st), _ptr(hist), hist_cap,
                                    ctypes.byref(nh)))
        return st.value, hist[: min(nh.value, hist_cap)].copy()

    def run(self, reinit=True, hist_cap=200000):
        hist = np.empty(hist_cap, np.float64)
        nh = ctypes.c_int()
        self._check(self.L.ref_run(self.h, 1 if reinit else 0, _ptr(hist), hist_cap, ctypes.byref(nh)))
        return hist[: min(nh.value, hist_cap)].copy()

    def set_angle(self, angle, patch="farfield"):
        self._check(self.L.ref_set_angle(self.h, patch.encode(), float(angle)))

    def wall_profile(self, patch="wall", lvl=-1, cap=1 << 20):
        out = np.empty(3, np.float64)
        cp = np.empty(cap, np.float64)
        n = ctypes.c_int()
        self._check(self.L.ref_wall_profile(self.h, self._lvl(lvl), patch.encode(), _ptr(out), _ptr(cp), cap,
                                      ctypes.byref(n)))
        return dict(cl=out[0], cd=out[1], cm=out[2], cp=cp[: n.value].copy())

    def implicit_block(self, i, j, cfl=None, lvl=-1, fill=True):
        blk = np.empty(16, np.float64)
        self._check(self.L.ref_implicit_block(self.h, self._lvl(lvl), float(cfl or 0.0), int(i), int(j), _ptr(blk),
                                        1 if fill else 0))
        return blk.reshape(4, 4)
