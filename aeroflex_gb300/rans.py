"""Python host mirror of AeroFLEX's `rans` interface over the C ABI.

Names follow the reference (src/rans/include/rans/*.h): ``mesh`` (mesh.h),
``Settings`` (core.h), ``Solver`` (solver.h explicitSolver + multigrid.h
run_solver) and ``get_wall_profile`` (post.h).  Every call goes through
libafx_rans.so; there is no Python or CPU fallback — a missing library is
an ImportError.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libafx_rans.so")

AFX_ERRORS = {1: "IO", 2: "CONFIG", 3: "MESH", 4: "NONFINITE", 5: "DIVERGED", 7: "CUDA", 8: "ARG",
              9: "STOPPED"}

# Symbols declared in include/afx_rans.h.
ABI_SYMBOLS = [
    "afx_last_error", "afx_version", "afx_mesh_load", "afx_mesh_from_arrays", "afx_mesh_counts", "afx_mesh_get",
    "afx_mesh_get_int", "afx_mesh_boundary_name", "afx_mesh_free", "afx_config_create", "afx_config_from_ini",
    "afx_config_from_ini_string", "afx_config_set_double", "afx_config_get_double", "afx_config_set_string",
    "afx_config_get_string", "afx_config_set_bc", "afx_config_bc_count", "afx_config_get_bc", "afx_config_free",
    "afx_solver_create",
    "afx_solver_free", "afx_init_freestream", "afx_set_state", "afx_get_state", "afx_residual", "afx_iterate",
    "afx_run_to_convergence", "afx_residual_history", "afx_forces", "afx_set_farfield", "afx_request_stop",
    "afx_last_device_seconds", "afx_profile_iterations", "afx_kernel_name", "afx_autotune",
    "afx_residual_noalloc", "afx_implicit_rhs", "afx_set_turbulence", "afx_get_turbulence",
    "afx_turbulence_residual", "afx_measure_fp64_peak", "afx_newton_solve", "afx_batch_create", "afx_batch_free",
    "afx_batch_counts", "afx_batch_init_freestream",
    "afx_batch_set_state", "afx_batch_get_state", "afx_batch_iterate", "afx_batch_run_to_convergence",
    "afx_batch_case_history", "afx_batch_forces", "afx_batch_set_farfield", "afx_batch_autotune",
    "afx_batch_last_device_seconds", "afx_residual_vjp", "afx_boundary_states", "afx_adjoint_solve",
    "afx_adjoint_state", "afx_linear_iterations", "afx_prolongate", "afx_patch_nodes", "afx_deform_patch",
    "afx_adjoint_patch", "afx_adjoint_patch_dirs", "afx_deform_patch_xy", "afx_adjoint_patch_dirs_xy",
    "afx_wall_distance", "afx_mesh_set_nodes", "afx_batch_linear_iterations",
    "afx_write_vtu", "afx_save_vtu",
]
N_KERNEL_KINDS = 7


class AfxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("AFX_ERR_%s: %s" % (AFX_ERRORS.get(code, code), msg))
        self.code = code


_lib = None


def lib():
    """Load libafx_rans.so (built by __graft_entry__.build() / aeroflex_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libafx_rans.so is not built (run `python -m aeroflex_gb300.build`)")
    L = ctypes.CDLL(LIB_PATH)
    vp, cp, i, d, ll = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    P = ctypes.POINTER
    sig = {
        "afx_last_error": (cp, []),
        "afx_version": (cp, []),
        "afx_mesh_load": (i, [cp, P(vp)]),
        "afx_mesh_from_arrays": (i, [i, vp, vp, i, vp, i, vp, vp, cp, P(vp)]),
        "afx_mesh_counts": (i, [vp, vp]),
        "afx_mesh_get": (i, [vp, cp, vp, ll, P(ll)]),
        "afx_mesh_get_int": (i, [vp, cp, vp, ll, P(ll)]),
        "afx_mesh_boundary_name": (i, [vp, i, ctypes.c_char_p, i]),
        "afx_mesh_free": (None, [vp]),
        "afx_config_create": (i, [P(vp)]),
        "afx_config_from_ini": (i, [cp, P(vp)]),
        "afx_config_from_ini_string": (i, [cp, P(vp)]),
        "afx_config_set_double": (i, [vp, cp, d]),
        "afx_config_get_double": (i, [vp, cp, P(d)]),
        "afx_config_set_string": (i, [vp, cp, cp]),
        "afx_config_get_string": (i, [vp, cp, ctypes.c_char_p, i]),
        "afx_config_set_bc": (i, [vp, cp, cp, d, d, d, d]),
        "afx_config_bc_count": (i, [vp, P(i)]),
        "afx_config_get_bc": (i, [vp, cp, ctypes.c_char_p, i, P(d), P(d), P(d), P(d)]),
        "afx_config_free": (None, [vp]),
        "afx_solver_create": (i, [vp, vp, P(vp)]),
        "afx_solver_free": (None, [vp]),
        "afx_init_freestream": (i, [vp]),
        "afx_set_state": (i, [vp, vp, ll]),
        "afx_get_state": (i, [vp, vp, ll]),
        "afx_residual": (i, [vp, vp, ll]),
        "afx_iterate": (i, [vp, i, P(d)]),
        "afx_run_to_convergence": (i, [vp, d, i, P(i), P(d)]),
        "afx_residual_history": (i, [vp, vp, i, P(i)]),
        "afx_forces": (i, [vp, cp, P(d), P(d), P(d), vp, i, P(i)]),
        "afx_set_farfield": (i, [vp, cp, d, d, d, d]),
        "afx_request_stop": (i, [vp]),
        "afx_last_device_seconds": (i, [vp, P(d)]),
        "afx_profile_iterations": (i, [vp, i, vp, vp, i]),
        "afx_kernel_name": (cp, [i]),
        "afx_autotune": (i, [vp, i, ctypes.c_char_p, i, P(i), P(d)]),
        "afx_residual_noalloc": (i, [vp, vp, vp, ll]),
        "afx_implicit_rhs": (i, [vp, vp, ll]),
        "afx_set_turbulence": (i, [vp, vp, ll]),
        "afx_get_turbulence": (i, [vp, vp, ll]),
        "afx_turbulence_residual": (i, [vp, vp, ll]),
        "afx_measure_fp64_peak": (i, [ctypes.c_int, vp]),
        "afx_batch_create": (i, [i, vp, vp, P(vp)]),
        "afx_batch_free": (None, [vp]),
        "afx_batch_counts": (i, [vp, P(i), P(ll)]),
        "afx_batch_init_freestream": (i, [vp]),
        "afx_batch_set_state": (i, [vp, i, vp, ll]),
        "afx_batch_get_state": (i, [vp, i, vp, ll]),
        "afx_batch_iterate": (i, [vp, i, vp]),
        "afx_batch_run_to_convergence": (i, [vp, d, i, vp, vp, vp]),
        "afx_batch_case_history": (i, [vp, i, vp, i, P(i)]),
        "afx_batch_forces": (i, [vp, i, cp, P(d), P(d), P(d)]),
        "afx_batch_set_farfield": (i, [vp, i, cp, d, d, d, d]),
        "afx_batch_autotune": (i, [vp, i, ctypes.c_char_p, i, P(i), P(d)]),
        "afx_batch_last_device_seconds": (i, [vp, P(d)]),
        "afx_residual_vjp": (i, [vp, vp, vp, vp, vp, ll]),
        "afx_boundary_states": (i, [vp, vp, ll]),
        "afx_adjoint_solve": (i, [vp, cp, cp, d, i, vp, P(i), P(d)]),
        "afx_adjoint_state": (i, [vp, vp, ll]),
        "afx_linear_iterations": (i, [vp, P(i)]),
        "afx_batch_linear_iterations": (i, [vp, vp, i]),
        "afx_prolongate": (i, [vp, vp]),
        "afx_patch_nodes": (i, [vp, cp, vp, vp, vp, i, P(i)]),
        "afx_deform_patch": (i, [vp, cp, vp, i, d]),
        "afx_adjoint_patch": (i, [vp, cp, cp, d, d, vp, i]),
        "afx_adjoint_patch_dirs": (i, [vp, cp, cp, d, d, vp, i, i, vp]),
        "afx_newton_solve": (i, [vp, d, i, d, d, i, P(i), P(i), P(d), vp, i]),
        "afx_deform_patch_xy": (i, [vp, cp, vp, vp, i, d]),
        "afx_adjoint_patch_dirs_xy": (i, [vp, cp, cp, d, d, vp, i, i, vp]),
        "afx_wall_distance": (i, [vp, vp, ll]),
        "afx_mesh_set_nodes": (i, [vp, vp, vp, ll]),
        "afx_write_vtu": (i, [vp, vp, vp, ll, d, d, cp]),
        "afx_save_vtu": (i, [vp, cp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise AfxError(rc, lib().afx_last_error().decode())


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class mesh:
    """`rans::mesh` (mesh.h:198-273): gmsh 4.1 file or generator arrays."""

    def __init__(self, filename=None, arrays=None):
        h = ctypes.c_void_p()
        if filename is not None:
            _check(lib().afx_mesh_load(str(filename).encode(), ctypes.byref(h)))
        else:
            m = arrays
            x = np.ascontiguousarray(m["x"], np.float64)
            y = np.ascontiguousarray(m["y"], np.float64)
            cells = np.ascontiguousarray(m["cells"], np.int32)
            be = np.ascontiguousarray(m["bedges"], np.int32)
            bp = np.ascontiguousarray(m["bpatch"], np.int32)
            _check(lib().afx_mesh_from_arrays(len(x), _ptr(x), _ptr(y), len(cells), _ptr(cells), len(be), _ptr(be),
                                              _ptr(bp), "\n".join(m["names"]).encode(), ctypes.byref(h)))
        self.h = h
        c = np.zeros(5, np.int64)
        _check(lib().afx_mesh_counts(self.h, _ptr(c)))
        self.nRealCells, self.n_tot, self.n_edges, self.n_boundary, self.n_nodes = (int(v) for v in c)

    @classmethod
    def from_arrays(cls, m):
        return cls(arrays=m)

    def get(self, what):
        n = ctypes.c_longlong()
        _check(lib().afx_mesh_get(self.h, what.encode(), None, 0, ctypes.byref(n)))
        out = np.empty(n.value, np.float64)
        _check(lib().afx_mesh_get(self.h, what.encode(), _ptr(out), n.value, ctypes.byref(n)))
        return out

    def get_int(self, what):
        n = ctypes.c_longlong()
        _check(lib().afx_mesh_get_int(self.h, what.encode(), None, 0, ctypes.byref(n)))
        out = np.empty(n.value, np.int64)
        _check(lib().afx_mesh_get_int(self.h, what.encode(), _ptr(out), n.value, ctypes.byref(n)))
        return out

    def set_nodes(self, x, y):
        """New node coordinates, same topology: metrics re-formed."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        _check(lib().afx_mesh_set_nodes(self.h, _ptr(x), _ptr(y), x.size))

    def write_vtu(self, path, q, wall_dist=None, gamma=1.4, R=0.71428571428):
        """`save` (post.h:58-180) of host state q (4 per real cell, reference
        order) on this mesh; wall_dist per real cell (None: zeros)."""
        q = np.ascontiguousarray(q, np.float64).ravel()
        wd = None if wall_dist is None else np.ascontiguousarray(wall_dist, np.float64)
        _check(lib().afx_write_vtu(self.h, _ptr(q), None if wd is None else _ptr(wd), q.size, float(gamma), float(R),
                                   str(path).encode()))

    def boundary_names(self):
        buf = ctypes.create_string_buffer(256)
        out = []
        for b in range(self.n_boundary):
            _check(lib().afx_mesh_boundary_name(self.h, b, buf, 256))
            out.append(buf.value.decode())
        return out

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.afx_mesh_free(self.h)
            self.h = None


class Settings:
    """`rans::Settings` (core.h:166-232); ``from_ini`` = import_config_file."""

    def __init__(self, handle=None):
        if handle is None:
            handle = ctypes.c_void_p()
            _check(lib().afx_config_create(ctypes.byref(handle)))
        self.h = handle

    @classmethod
    def from_ini(cls, path):
        h = ctypes.c_void_p()
        _check(lib().afx_config_from_ini(str(path).encode(), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def from_ini_string(cls, text):
        h = ctypes.c_void_p()
        _check(lib().afx_config_from_ini_string(text.encode(), ctypes.byref(h)))
        return cls(h)

    def set(self, key, value):
        if isinstance(value, str):
            _check(lib().afx_config_set_string(self.h, key.encode(), value.encode()))
        else:
            _check(lib().afx_config_set_double(self.h, key.encode(), float(value)))
        return self

    def get(self, key):
        v = ctypes.c_double()
        rc = lib().afx_config_get_double(self.h, key.encode(), ctypes.byref(v))
        if rc == 0:
            return v.value
        buf = ctypes.create_string_buffer(256)
        _check(lib().afx_config_get_string(self.h, key.encode(), buf, 256))
        return buf.value.decode()

    def set_bc(self, name, type, T=1.0, mach=0.2, angle=0.0, p=1.0):
        _check(lib().afx_config_set_bc(self.h, name.encode(), type.encode(), T, mach, angle, p))
        return self

    def bc_count(self):
        n = ctypes.c_int()
        _check(lib().afx_config_bc_count(self.h, ctypes.byref(n)))
        return n.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.afx_config_free(self.h)
            self.h = None


class Solver:
    """Explicit solver on the GPU: `explicitSolver` (solver.h:721-828) +
    `multigrid<explicitSolver>::run_solver` (multigrid.h:182-237)."""

    def __init__(self, m, settings):
        h = ctypes.c_void_p()
        _check(lib().afx_solver_create(m.h, settings.h, ctypes.byref(h)))
        self.h = h
        self.n_real = m.nRealCells
        self.n_boundary = m.n_boundary
        self.mesh_boundary_names = m.boundary_names()

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.afx_solver_free(self.h)
            self.h = None

    def init(self):
        _check(lib().afx_init_freestream(self.h))

    def set_q(self, q):
        q = np.ascontiguousarray(q, np.float64).reshape(-1)
        _check(lib().afx_set_state(self.h, _ptr(q), q.size))

    def get_q(self, out=None):
        if out is None:
            out = np.empty(4 * self.n_real, np.float64)
        _check(lib().afx_get_state(self.h, _ptr(out), out.size))
        return out

    def residual(self):
        R = np.empty(4 * self.n_real, np.float64)
        _check(lib().afx_residual(self.h, _ptr(R), R.size))
        return R

    def set_nu(self, nu):
        """nu~ of the Spalart-Allmaras model per real cell (reference order)."""
        nu = np.ascontiguousarray(nu, np.float64).reshape(-1)
        _check(lib().afx_set_turbulence(self.h, _ptr(nu), nu.size))

    def nu(self):
        out = np.empty(self.n_real, np.float64)
        _check(lib().afx_get_turbulence(self.h, _ptr(out), out.size))
        return out

    def nu_residual(self):
        """nu~ residual R/A of the last evaluation."""
        out = np.empty(self.n_real, np.float64)
        _check(lib().afx_turbulence_residual(self.h, _ptr(out), out.size))
        return out

    def implicit_rhs(self):
        """fillRhoRHS (solver.h:1079-1152) of the current state (implicit
        solvers): face sums not divided by the area."""
        R = np.empty(4 * self.n_real, np.float64)
        _check(lib().afx_implicit_rhs(self.h, _ptr(R), R.size))
        return R

    def iterate(self, n):
        r = ctypes.c_double()
        _check(lib().afx_iterate(self.h, int(n), ctypes.byref(r)))
        return r.value

    def run_solver(self, tol=0.0, max_it=0):
        it = ctypes.c_int()
        err = ctypes.c_double()
        _check(lib().afx_run_to_convergence(self.h, tol, max_it, ctypes.byref(it), ctypes.byref(err)))
        return it.value, err.value

    def history(self):
        n = ctypes.c_int()
        _check(lib().afx_residual_history(self.h, None, 0, ctypes.byref(n)))
        out = np.empty(n.value, np.float64)
        _check(lib().afx_residual_history(self.h, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def newton_solve(self, tol=0.0, max_newton=0, cfl=0.0, lin_tol=0.0, max_krylov=0):
        """Newton-Krylov finish of an implicit solver: (Newton steps,
        Krylov steps, err), err = ||RHS|| / err_0; the per-step record
        (err, step length, Krylov steps, linear residual) is kept in
        self.newton_record."""
        nn, nk, err = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        cap = max(int(max_newton), 20)
        rec = np.zeros((cap, 4), np.float64)
        _check(lib().afx_newton_solve(self.h, float(tol), int(max_newton), float(cfl), float(lin_tol),
                                      int(max_krylov), ctypes.byref(nn), ctypes.byref(nk), ctypes.byref(err),
                                      _ptr(rec), cap))
        self.newton_record = rec[: min(nn.value, cap)].copy()
        return nn.value, nk.value, err.value

    def set_farfield(self, patch, mach, angle, T=1.0, p=1.0):
        _check(lib().afx_set_farfield(self.h, patch.encode(), mach, angle, T, p))

    def request_stop(self):
        _check(lib().afx_request_stop(self.h))

    def last_device_seconds(self):
        s = ctypes.c_double()
        _check(lib().afx_last_device_seconds(self.h, ctypes.byref(s)))
        return s.value

    def autotune(self, iters=5):
        """Pick the fastest residual-kernel variant and block size on this mesh."""
        buf = ctypes.create_string_buffer(16)
        blk = ctypes.c_int()
        ms = ctypes.c_double()
        _check(lib().afx_autotune(self.h, int(iters), buf, 16, ctypes.byref(blk), ctypes.byref(ms)))
        return dict(variant=buf.value.decode(), block=blk.value, ms_per_iter=ms.value)

    def save_vtu(self, path):
        """`save(filename, solver)` (post.h:58-180): the solver's state, its
        wall distance and gas."""
        _check(lib().afx_save_vtu(self.h, str(path).encode()))

    def wall_distance(self):
        """mesh::compute_wall_dist (mesh.h:794-830) on the GPU: all cells."""
        out = np.empty(self.n_real + self.n_boundary, np.float64)
        _check(lib().afx_wall_distance(self.h, _ptr(out), out.size))
        return out

    def prolongate_from(self, coarse):
        """Grid-sequencing transfer (multigrid.h:99-178, 316-321): this
        solver's state from the coarse solver's."""
        _check(lib().afx_prolongate(coarse.h, self.h))

    def linear_iterations(self):
        """Krylov iterations of the last implicit iteration (0: explicit solver)."""
        n = ctypes.c_int()
        _check(lib().afx_linear_iterations(self.h, ctypes.byref(n)))
        return n.value

    def residual_vjp(self, v, q=None):
        """((dR/dq)^T v, (dR/dbq)^T v) at state q (default: the solver's);
        the second is (n_boundary, 4)."""
        v = np.ascontiguousarray(v, np.float64).reshape(-1)
        u = np.empty_like(v)
        bq = np.empty((self.n_boundary, 4), np.float64)
        qp = None
        if q is not None:
            q = np.ascontiguousarray(q, np.float64).reshape(-1)
            qp = _ptr(q)
        _check(lib().afx_residual_vjp(self.h, qp, _ptr(v), _ptr(u), _ptr(bq) if self.n_boundary else None, v.size))
        return u, bq

    def boundary_states(self):
        bq = np.empty((self.n_boundary, 4), np.float64)
        _check(lib().afx_boundary_states(self.h, _ptr(bq), bq.size))
        return bq

    def adjoint_solve(self, patch="wall", objective="cl", tol=0.0, max_it=0):
        """(dJ/dangle, dJ/dMach), iterations, relative adjoint residual."""
        dJ = np.zeros(2, np.float64)
        it = ctypes.c_int()
        res = ctypes.c_double()
        _check(lib().afx_adjoint_solve(self.h, patch.encode(), objective.encode(), float(tol), int(max_it), _ptr(dJ),
                                       ctypes.byref(it), ctypes.byref(res)))
        return (float(dJ[0]), float(dJ[1])), it.value, res.value

    def patch_nodes(self, patch="wall"):
        """(node ids, unit normals nx, ny) of a boundary patch."""
        n = ctypes.c_int()
        _check(lib().afx_patch_nodes(self.h, patch.encode(), None, None, None, 0, ctypes.byref(n)))
        ids = np.empty(n.value, np.int64)
        nx = np.empty(n.value, np.float64)
        ny = np.empty(n.value, np.float64)
        _check(lib().afx_patch_nodes(self.h, patch.encode(), _ptr(ids), _ptr(nx), _ptr(ny), n.value, ctypes.byref(n)))
        return ids, nx, ny

    def deform_patch(self, a, patch="wall", power=2.0):
        a = np.ascontiguousarray(a, np.float64)
        _check(lib().afx_deform_patch(self.h, patch.encode(), _ptr(a), a.size, float(power)))

    def adjoint_patch(self, patch="wall", objective="cl", power=2.0, h=0.0):
        """dJ/da_k for every patch node (after adjoint_solve of the same J)."""
        n = len(self.patch_nodes(patch)[0])
        out = np.empty(n, np.float64)
        _check(lib().afx_adjoint_patch(self.h, patch.encode(), objective.encode(), float(power), float(h), _ptr(out),
                                       n))
        return out

    def adjoint_patch_dirs(self, dirs, patch="wall", objective="cl", power=2.0, h=0.0):
        """dJ/dt along each row c of `dirs` (a = a0 + t c over the patch
        nodes), after adjoint_solve of the same J: two residual evaluations
        per direction."""
        dirs = np.ascontiguousarray(np.atleast_2d(dirs), np.float64)
        out = np.empty(dirs.shape[0], np.float64)
        _check(lib().afx_adjoint_patch_dirs(self.h, patch.encode(), objective.encode(), float(power), float(h),
                                            _ptr(dirs), dirs.shape[0], dirs.shape[1], _ptr(out)))
        return out

    def deform_patch_xy(self, dx, dy, patch="wall", power=2.0):
        """Patch node k displaced by (dx[k], dy[k]), relative to the
        undeformed mesh; the volume follows by inverse-distance weighting."""
        dx = np.ascontiguousarray(dx, np.float64)
        dy = np.ascontiguousarray(dy, np.float64)
        _check(lib().afx_deform_patch_xy(self.h, patch.encode(), _ptr(dx), _ptr(dy), dx.size, float(power)))

    def adjoint_patch_dirs_xy(self, dirs, patch="wall", objective="cl", power=2.0, h=0.0):
        """dJ/dt along displacement-vector directions: dirs (n_dirs,
        n_patch, 2), (dx_k, dy_k) per patch node."""
        dirs = np.ascontiguousarray(dirs, np.float64)
        if dirs.ndim == 2:
            dirs = dirs[None]
        out = np.empty(dirs.shape[0], np.float64)
        _check(lib().afx_adjoint_patch_dirs_xy(self.h, patch.encode(), objective.encode(), float(power), float(h),
                                               _ptr(dirs), dirs.shape[0], dirs.shape[1], _ptr(out)))
        return out

    def adjoint_state(self):
        lam = np.empty(4 * self.n_real, np.float64)
        _check(lib().afx_adjoint_state(self.h, _ptr(lam), lam.size))
        return lam

    def profile_iterations(self, n):
        """Per-kernel device time (CUDA events on the solver's stream) over n
        eager iterations: {kernel name: (total ms, launches)}."""
        ms = np.zeros(N_KERNEL_KINDS, np.float64)
        cnt = np.zeros(N_KERNEL_KINDS, np.int32)
        _check(lib().afx_profile_iterations(self.h, int(n), _ptr(ms), _ptr(cnt), N_KERNEL_KINDS))
        return {lib().afx_kernel_name(k).decode(): (float(ms[k]), int(cnt[k])) for k in range(N_KERNEL_KINDS)
                if cnt[k] > 0}


def save(filename, s):
    """`rans::save` (post.h:58-180): the VTU file of solver s."""
    s.save_vtu(filename)


def measure_fp64_peak(reps=5):
    """FP64 FMA-chain peak of the current GPU in TFLOP/s (afx_measure_fp64_peak)."""
    t = ctypes.c_double()
    _check(lib().afx_measure_fp64_peak(int(reps), ctypes.byref(t)))
    return t.value


def get_wall_profile(s, patch="wall", cap=1 << 20):
    """`get_wall_profile` (post.h:301-387): dict(cl, cd, cm, cp)."""
    cl, cd, cm = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    n = ctypes.c_int()
    cp = np.empty(cap, np.float64)
    _check(lib().afx_forces(s.h, patch.encode(), ctypes.byref(cl), ctypes.byref(cd), ctypes.byref(cm), _ptr(cp), cap,
                            ctypes.byref(n)))
    return dict(cl=cl.value, cd=cd.value, cm=cm.value, cp=cp[: n.value].copy())


class Batch:
    """Many independent load cases (own mesh, angle, Mach) advanced together:
    each case follows `multigrid<explicitSolver>::run_solver`
    (multigrid.h:183-234) on its own, one launch per kernel for all of them."""

    def __init__(self, meshes, settings):
        meshes, settings = list(meshes), list(settings)
        if len(meshes) != len(settings):
            raise ValueError("one Settings per mesh")
        self._keep = (meshes, settings)
        mh = (ctypes.c_void_p * len(meshes))(*[m.h.value for m in meshes])
        sh = (ctypes.c_void_p * len(settings))(*[s.h.value for s in settings])
        h = ctypes.c_void_p()
        _check(lib().afx_batch_create(len(meshes), ctypes.cast(mh, ctypes.c_void_p), ctypes.cast(sh, ctypes.c_void_p),
                                      ctypes.byref(h)))
        self.h = h
        self.n = len(meshes)
        self.n_real = [m.nRealCells for m in meshes]

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.afx_batch_free(self.h)
            self.h = None

    def __len__(self):
        return self.n

    def n_cells_total(self):
        n = ctypes.c_longlong()
        _check(lib().afx_batch_counts(self.h, None, ctypes.byref(n)))
        return n.value

    def init(self):
        _check(lib().afx_batch_init_freestream(self.h))

    def set_q(self, c, q):
        q = np.ascontiguousarray(q, np.float64).reshape(-1)
        _check(lib().afx_batch_set_state(self.h, int(c), _ptr(q), q.size))

    def get_q(self, c):
        out = np.empty(4 * self.n_real[c], np.float64)
        _check(lib().afx_batch_get_state(self.h, int(c), _ptr(out), out.size))
        return out

    def iterate(self, n, raise_nonfinite=True):
        """n iterations of every case; returns each case's last norm.  With
        raise_nonfinite=False a case whose norm went non-finite (that case
        then holds its state) shows as a non-finite entry instead of raising."""
        r = np.zeros(self.n, np.float64)
        rc = lib().afx_batch_iterate(self.h, int(n), _ptr(r))
        if rc != 0 and not (rc == 4 and not raise_nonfinite):
            _check(rc)
        return r

    def run_solver(self, tol=0.0, max_it=0):
        """Returns (iterations, err/err_0, status) arrays, one entry per case."""
        it = np.zeros(self.n, np.int32)
        err = np.zeros(self.n, np.float64)
        st = np.zeros(self.n, np.int32)
        _check(lib().afx_batch_run_to_convergence(self.h, float(tol), int(max_it), _ptr(it), _ptr(err), _ptr(st)))
        return it, err, st

    def history(self, c):
        n = ctypes.c_int()
        _check(lib().afx_batch_case_history(self.h, int(c), None, 0, ctypes.byref(n)))
        out = np.empty(n.value, np.float64)
        _check(lib().afx_batch_case_history(self.h, int(c), _ptr(out), n.value, ctypes.byref(n)))
        return out

    def forces(self, c, patch="wall"):
        cl, cd, cm = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(lib().afx_batch_forces(self.h, int(c), patch.encode(), ctypes.byref(cl), ctypes.byref(cd),
                                      ctypes.byref(cm)))
        return dict(cl=cl.value, cd=cd.value, cm=cm.value)

    def set_farfield(self, c, patch, mach, angle, T=1.0, p=1.0):
        _check(lib().afx_batch_set_farfield(self.h, int(c), patch.encode(), mach, angle, T, p))

    def autotune(self, iters=5):
        buf = ctypes.create_string_buffer(16)
        blk = ctypes.c_int()
        ms = ctypes.c_double()
        _check(lib().afx_batch_autotune(self.h, int(iters), buf, 16, ctypes.byref(blk), ctypes.byref(ms)))
        return dict(variant=buf.value.decode(), block=blk.value, ms_per_iter=ms.value)

    def last_device_seconds(self):
        s = ctypes.c_double()
        _check(lib().afx_batch_last_device_seconds(self.h, ctypes.byref(s)))
        return s.value

    def linear_iterations(self):
        """Krylov iterations of each case in the last implicit iteration."""
        out = np.zeros(self.n, np.int32)
        _check(lib().afx_batch_linear_iterations(self.h, _ptr(out), self.n))
        return out
