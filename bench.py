"""Benchmark of the rans residual path on one GB300.

Workload: the throughput channel mesh — unit square, 2048 x 1024 quads split
into 4,194,304 triangles, interior nodes jittered by +-0.2 h (seed 1), cells
shuffled (seed 2), freestream M = 0.3 with a Gaussian density bump
(amplitude 0.05, width 0.1).  Patches: "farfield" (left/right), "wall"
(slip, bottom/top).  Explicit second-order scheme (Green-Gauss gradient,
Venkatakrishnan limiter K = 5, Roe flux), CFL 1, relaxation 0.9.

One step = one explicit iteration (three RK stages); metric = cell-residual
evaluations per second = N_cells * 3 / seconds per step.  The headline
``value`` is the FP32-mixed path (FP32 fluxes, FP64 state update / norm);
the FP64 path (bit-identical to the reference arithmetic) is measured beside
it under "fp64".  Inputs are larger than L2 (state, gradients, limiter and
face records are ~1 GB), so no extra L2 flush is needed between steps.

``--impl reference`` times the CPU oracle (the project's plain-C++
restatement of the reference's explicit path: serial face loops, OpenMP on
per-cell loops, as the reference) on the machine's host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY = 2048, 1024
MACH = 0.3
SAMPLE_NX, SAMPLE_NY = 512, 256  # CPU sample of the same generator


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def _setup_gpu(precision, m, q0, variant="auto"):
    from aeroflex_gb300 import rans
    st = rans.Settings()
    st.set("solver", "explicit").set("precision", precision).set("start_cfl", 1.0).set("relaxation", 0.9)
    st.set("kernel_variant", variant)
    st.set_bc("farfield", "farfield", 1.0, MACH, 0.0, 1.0).set_bc("wall", "slip-wall")
    g = rans.Solver(m, st)
    g.init()
    g.set_q(q0)
    return g


def algorithmic_bytes(kernel, n, f, precision):
    """Compulsory HBM bytes of one launch of ``kernel`` (every array it
    touches counted once).  w = bytes of the arithmetic type."""
    w = 8 if precision == "fp64" else 4
    cell_vec = 4 * w
    face_geo = 8 + 8 * w  # c0,c1 + n, (L,g), d0, d1
    if kernel == "k_resid_gather":
        # reads: cslot, area, qk, gx, gy, phi, q0 (FP64), dt; faces; writes next stage state
        # (stage 2 writes the FP64 state + FP32 shadow: counted as the average over the 3 stages)
        writes = (cell_vec + cell_vec + (32 + cell_vec)) / 3.0
        return n * (16 + w + 4 * cell_vec + 32 + w + writes) + f * face_geo
    if kernel == "k_resid_tile":
        # faces once (40/72 B records), cell vectors q, gx, gy, phi of every cell once, per-cell tile
        # slots (8), area, dt, FP64 q0, stage writes; tile lists are < 1% and not counted
        writes = (cell_vec + cell_vec + (32 + cell_vec)) / 3.0
        return n * (4 * cell_vec + 8 + w + w + 32 + writes) + f * face_geo
    if kernel == "k_face_flux":
        return n * 4 * cell_vec + f * (face_geo + 4 * w)
    if kernel == "k_cell_sum":
        writes = (cell_vec + cell_vec + 32) / 3.0
        return n * (16 + w + 32 + w + writes) + f * (8 + 4 * w)
    if kernel == "k_prep":
        return n * (16 + w + cell_vec + 3 * cell_vec + w) + f * face_geo
    if kernel == "k_limiter":
        return n * (16 + w + 4 * cell_vec) + f * face_geo
    return 0


def run_lean(args):
    """Warm-up + K iterations and nothing else (the command profiled by ncu)."""
    from aeroflex_gb300 import meshgen, rans

    marr = meshgen.channel(args.nx, args.ny, jitter=0.2, seed=1, shuffle_seed=2)
    q0 = meshgen.density_bump_state(marr, mach=MACH)
    m = rans.mesh.from_arrays(marr)
    for precision in args.precision.split(","):
        g = _setup_gpu(precision, m, q0, args.variant)
        g.iterate(args.warmup)
        g.iterate(args.steps)
        print(json.dumps({"precision": precision, "cells": m.nRealCells, "steps": args.steps,
                          "ms_per_step": g.last_device_seconds() / args.steps * 1e3}))
        del g


def run_gpu(args):
    import torch  # device plumbing only: pinned host memory for the end-to-end leg
    from aeroflex_gb300 import meshgen, rans

    t0 = time.time()
    marr = meshgen.channel(args.nx, args.ny, jitter=0.2, seed=1, shuffle_seed=2)
    q0 = meshgen.density_bump_state(marr, mach=MACH)
    m = rans.mesh.from_arrays(marr)
    N, F = m.nRealCells, m.n_edges
    setup_s = time.time() - t0
    hbm_peak, peak_kind = _peaks()
    result = {}
    for precision in ("fp32-mixed", "fp64"):
        g = _setup_gpu(precision, m, q0)
        tuned = g.autotune(3 if precision == "fp32-mixed" else 1)
        K = args.steps if precision == "fp32-mixed" else max(3, min(args.steps, 50))
        clocks = Clocks()
        clocks.start() if precision == "fp32-mixed" else None
        g.set_q(q0)
        g.iterate(args.warmup)
        g.set_q(q0)
        g.iterate(K)
        sec = g.last_device_seconds()
        ck = clocks.stop() if precision == "fp32-mixed" else None
        evals = N * 3 * K / sec
        # per-kernel device times (CUDA events on the solver's stream)
        prof = g.profile_iterations(min(5, K))
        n_prof = min(5, K)
        tot = sum(v[0] for v in prof.values())
        top = max(prof.items(), key=lambda kv: kv[1][0])
        kname, (kms, kn) = top
        per_launch_s = kms / kn * 1e-3
        ab = algorithmic_bytes(kname, N, F, precision)
        achieved = ab / per_launch_s / 1e9
        launches_per_iter = sum(v[1] for v in prof.values()) / n_prof
        entry = dict(value=evals, ms_per_step=sec / K * 1e3, steps=K, tuned=tuned,
                     kernels={k: dict(ms_total=v[0], launches=v[1], share=v[0] / tot) for k, v in prof.items()},
                     roofline=dict(kernel=kname, bound="hbm", achieved=achieved, peak=hbm_peak, unit="GB/s",
                                   frac=achieved / hbm_peak, peak_source=peak_kind, traffic=None,
                                   algorithmic_bytes_per_launch=ab, launch_ms=per_launch_s * 1e3),
                     gpu_launches=int(round(launches_per_iter * K)))
        if precision == "fp32-mixed":
            entry["clocks"] = ck
            # end-to-end through the C ABI: host state -> device, iterate, norm back
            qh = torch.from_numpy(q0.copy()).pin_memory().numpy() if torch.cuda.is_available() else q0.copy()
            Ke = max(3, min(args.steps, 20))
            g.set_q(qh)
            g.iterate(1)
            t1 = time.perf_counter()
            for _ in range(Ke):
                g.set_q(qh)
                g.iterate(1)
            e2e_s = (time.perf_counter() - t1) / Ke
            entry["e2e"] = dict(value=N * 3 / e2e_s, unit="cell-residual evals/s", h2d_bytes_per_step=N * 32,
                                d2h_bytes_per_step=8, ms_per_step=e2e_s * 1e3, steps=Ke)
        result[precision] = entry
        del g
    return dict(N=N, F=F, setup_s=setup_s, res=result)


def cpu_baseline(budget_s=12.0):
    """The oracle (plain-C++ restatement of the reference's explicit solver)
    on a 512 x 256 sample of the same generator, all host threads."""
    from aeroflex_gb300 import meshgen
    from oracle import oracle

    marr = meshgen.channel(SAMPLE_NX, SAMPLE_NY, jitter=0.2, seed=1, shuffle_seed=2)
    s = oracle.Solver(oracle.Mesh.from_arrays(marr), oracle.default_settings(cfl=1.0), {
        "farfield": dict(type="farfield", T=1.0, mach=MACH, angle=0.0, p=1.0), "wall": dict(type="slip-wall")})
    s.init()
    s.set_q(meshgen.density_bump_state(marr, mach=MACH))
    s.time_iterations(1)
    its, sec = 0, 0.0
    while sec < budget_s:
        sec += s.time_iterations(1)
        its += 1
    n = SAMPLE_NX * SAMPLE_NY * 2
    return dict(value=n * 3 * its / sec, unit="cell-residual evals/s", cores=os.cpu_count(), kind="port",
                sample="%d explicit iterations on the %dx%d channel (%d cells), OMP_NUM_THREADS=%s" %
                       (its, SAMPLE_NX, SAMPLE_NY, n, os.environ.get("OMP_NUM_THREADS", str(os.cpu_count()))))


def run_reference(args):
    from aeroflex_gb300 import meshgen
    from oracle import oracle

    marr = meshgen.channel(SAMPLE_NX, SAMPLE_NY, jitter=0.2, seed=1, shuffle_seed=2)
    s = oracle.Solver(oracle.Mesh.from_arrays(marr), oracle.default_settings(cfl=1.0), {
        "farfield": dict(type="farfield", T=1.0, mach=MACH, angle=0.0, p=1.0), "wall": dict(type="slip-wall")})
    s.init()
    s.set_q(meshgen.density_bump_state(marr, mach=MACH))
    n = SAMPLE_NX * SAMPLE_NY * 2
    for _ in range(args.warmup):
        s.time_residuals(1)
    sec = s.time_residuals(args.steps)
    v = n * args.steps / sec
    line = {"metric": "cell-residual evals/s", "value": v, "unit": "cell-residual evals/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": "channel 2048x1024 -> 4,194,304 shuffled triangles, M 0.3 density bump; "
                                   "reference step = one second-order residual evaluation (dt, gradient, "
                                   "limiter, face loop) on the %dx%d sample (%d cells)" % (SAMPLE_NX, SAMPLE_NY, n)},
            "cpu_baseline": {"value": v, "unit": "cell-residual evals/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "%d residual evaluations on the %dx%d channel sample" %
                                       (args.steps, SAMPLE_NX, SAMPLE_NY)},
            "e2e": {"value": v, "unit": "cell-residual evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--nx", type=int, default=NX)
    ap.add_argument("--ny", type=int, default=NY)
    ap.add_argument("--lean", action="store_true", help="warm-up + timed iterations only (for ncu)")
    ap.add_argument("--precision", default="fp32-mixed", help="--lean: comma-separated precisions")
    ap.add_argument("--variant", default="auto", help="--lean: residual kernel variant (auto|gather|face|tile)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    import __graft_entry__
    __graft_entry__.build()
    if args.lean:
        run_lean(args)
        return
    # replicas only: each rank runs the full workload on its own GPU
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    r = run_gpu(args)
    f32 = r["res"]["fp32-mixed"]
    f64 = r["res"]["fp64"]
    value, ms = f32["value"], f32["ms_per_step"]
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        value = r["N"] * 3 / (ms * 1e-3) * world
    if rank != 0:
        return
    line = {
        "metric": "cell-residual evals/s", "value": value, "unit": "cell-residual evals/s", "n_gpus": world,
        "steps": f32["steps"], "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-mixed (f32 flux/gradient/limiter, f64 update/norm)",
        "data": "synthetic",
        "config": {"workload": "channel 2048x1024 quads -> %d shuffled triangles, M 0.3 density bump, explicit "
                               "RK3 second order, CFL 1" % r["N"], "cells": r["N"], "faces": r["F"],
                   "precision": "fp32-mixed", "l2": "inputs larger than L2 (~1 GB touched per step)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {k: f32["roofline"][k] for k in ("bound", "achieved", "peak", "unit", "frac", "traffic")},
        "roofline_kernel": f32["roofline"],
        "kernels": f32["kernels"],
        "clocks": f32["clocks"],
        "e2e": f32["e2e"],
        "gpu_launches": f32["gpu_launches"],
        "tuned": f32["tuned"],
        "fp64": {"value": f64["value"], "ms_per_step": f64["ms_per_step"], "steps": f64["steps"],
                 "tuned": f64["tuned"],
                 "roofline_kernel": f64["roofline"], "kernels": f64["kernels"], "gpu_launches": f64["gpu_launches"]},
        "setup_s": r["setup_s"],
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline()
    print(json.dumps(line))


if __name__ == "__main__":
    main()
