"""Regenerate tests/golden/ref_pins.json and naca0012q_mid_arrays.npz from
the reference's own code (oracle/_ref, built from its unmodified headers by
oracle/build_ref.py).  Needs the reference source tree.  Run from the
repository root:

    python tests/golden/make_ref_golden.py

ref_pins.json holds:
- "explicit": the pins of tests/refpins.explicit_pins run by the
  reference (hashes of states and residuals, norms, histories, forces);
- "implicit_rhs": hashes of the implicit right-hand side (fillRhoRHS) of
  perturbed states (tests/refpins.implicit_rhs_pins);
- "implicit": converged C_L, C_D, C_M of the reference's implicit solver
  (tests/refpins.implicit_polar_cases);
- "c1_split_diverges": the reference's implicit solver on config 1's
  split-triangle mesh as configured: its run_solver status and history.
naca0012q_mid_arrays.npz holds the node, cell and boundary arrays of the
reference's examples/rans/naca0012q_mid.msh as its own reader numbers them,
so that runs on that mesh need no reference tree.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from aeroflex_gb300 import meshgen  # noqa: E402
from oracle import ref, refsrc  # noqa: E402
from tests import refpins  # noqa: E402


def write_mid_mesh():
    rm = ref.Mesh(refsrc.path("examples", "rans", "naca0012q_mid.msh"))
    names = rm.boundary_names()
    uniq = sorted(set(names))
    np.savez_compressed(refpins.MID_MESH_NPZ, x=rm.get("node_x"), y=rm.get("node_y"),
                        cells=rm.get_int("cells_nodes").reshape(-1, 4).astype(np.int32),
                        bedges=rm.get_int("boundary_nodes").reshape(-1, 2).astype(np.int32),
                        bpatch=np.array([uniq.index(n) for n in names], np.int32), names=np.array(uniq))


def implicit_pins(drv):
    out = {}
    for tag, m, mach, angles in refpins.implicit_polar_cases():
        s = drv.solver(m, refpins.airfoil_bcs(mach, angles[0]), max_iterations=400, **refpins.IMPLICIT)
        s.c.init()
        res = []
        for a in angles:
            s.c.set_angle(a * refpins.DEG)
            s.c.refill_bcs()  # multigrid::run(false) starts with refill_bcs (multigrid.h:332)
            t = time.time()
            st, h = s.c.run_solver()
            w = s.c.wall_profile("wall")
            res.append(dict(angle_deg=a, status=st, iterations=len(h), final_residual=float(h[-1]),
                            cl=float(w["cl"]), cd=float(w["cd"]), cm=float(w["cm"])))
            print(tag, res[-1], "%.0fs" % (time.time() - t), flush=True)
        out[tag] = dict(mach=mach, polar=res)
    return out


def c1_split(drv):
    m = meshgen.airfoil_omesh(128, 64)
    s = drv.solver(m, refpins.airfoil_bcs(0.5, 1.25), max_iterations=200, **refpins.IMPLICIT)
    s.c.init()
    st, h = s.c.run_solver()
    return dict(status=st, iterations=len(h), history=[float(v) for v in h])


if __name__ == "__main__":
    write_mid_mesh()
    drv = refpins.RefDriver()
    out = {"generator": "tests/golden/make_ref_golden.py",
           "source": "the reference's rans headers compiled unmodified (oracle/build_ref.py)",
           "explicit": refpins.explicit_pins(drv),
           "implicit_rhs": refpins.implicit_rhs_pins(drv)}
    out["c1_split_diverges"] = c1_split(drv)
    print("c1 split:", out["c1_split_diverges"]["status"], out["c1_split_diverges"]["iterations"], flush=True)
    out["implicit"] = implicit_pins(drv)
    with open(refpins.PINS_JSON, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", refpins.PINS_JSON)
