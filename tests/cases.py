"""Shared workload definitions for the tests (small versions of the
benchmark configurations) and helpers that run the oracle and the GPU
library on identical inputs."""
import math

import numpy as np

from aeroflex_gb300 import meshgen

DEG = 0.01745  # the reference's degree -> radian factor (rans.h:88,94)


def omesh_case(n_surf=64, n_rad=32, mach=0.5, aoa_deg=1.25, **kw):
    m = meshgen.airfoil_omesh(n_surf=n_surf, n_rad=n_rad, **kw)
    bcs = {"farfield": dict(type="farfield", T=1.0, mach=mach, angle=aoa_deg * DEG, p=1.0),
           "wall": dict(type="slip-wall")}
    return m, bcs


def channel_case(nx=64, ny=32, mach=0.3, seed=1):
    m = meshgen.channel(nx, ny, jitter=0.2, seed=seed, shuffle_seed=seed + 1)
    bcs = {"farfield": dict(type="farfield", T=1.0, mach=mach, angle=0.0, p=1.0), "wall": dict(type="slip-wall")}
    q = meshgen.density_bump_state(m, mach=mach)
    return m, bcs, q


def oracle_solver(orc, m, bcs, **settings):
    om = orc.Mesh.from_arrays(m)
    st = orc.default_settings(**settings)
    s = orc.Solver(om, st, bcs)
    return s


def gpu_solver(afx, m, bcs, precision="fp64", **settings):
    st = gpu_settings(afx, bcs, precision, **settings)
    gm = afx.mesh.from_arrays(m)
    return afx.Solver(gm, st)


def gpu_settings(afx, bcs, precision="fp64", **settings):
    st = afx.Settings()
    st.set("solver", "explicit")
    st.set("precision", precision)
    cfl = settings.pop("cfl", 1.0)
    st.set("start_cfl", cfl)
    for k, v in settings.items():
        if isinstance(v, bool):
            v = 1.0 if v else 0.0
        st.set(k, v)
    for name, b in bcs.items():
        st.set_bc(name, b["type"], b.get("T", 1.0), b.get("mach", 0.2), b.get("angle", 0.0), b.get("p", 1.0))
    return st


def batch_cases():
    """Four small cases of uneven size, shape and flow (a polar-sweep batch
    in miniature): O-meshes of different resolution and camber, and a
    jittered channel."""
    out = []
    for (ns, nr, mach, aoa, kw) in [(32, 16, 0.5, 1.25, {}), (48, 24, 0.3, 4.0, dict(m=0.04, p=0.4, t=0.10)),
                                    (40, 20, 0.6, -2.0, dict(t=0.15))]:
        out.append(omesh_case(ns, nr, mach=mach, aoa_deg=aoa, **kw))
    m, bcs, _ = channel_case(24, 12, mach=0.4, seed=5)
    out.append((m, bcs))
    return out


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
