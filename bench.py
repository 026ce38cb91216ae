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


def _setup_gpu(precision, m, q0, variant="auto", block=0, adjoint_directions=4):
    from aeroflex_gb300 import rans
    st = rans.Settings()
    st.set("solver", "explicit").set("precision", precision).set("start_cfl", 1.0).set("relaxation", 0.9)
    st.set("kernel_variant", variant).set("block_size", block).set("adjoint_directions", adjoint_directions)
    st.set_bc("farfield", "farfield", 1.0, MACH, 0.0, 1.0).set_bc("wall", "slip-wall")
    g = rans.Solver(m, st)
    g.init()
    g.set_q(q0)
    return g


def stage_cell_bytes(precision, variant_reads):
    """Per-cell bytes of the three RK stages' epilogues (average over the
    stages): stage 1 reads nothing extra and writes dt + the next stage
    state; stage 2 reads the FP32 shadow of q (FP64: q) + dt and writes the
    next stage state; stage 3 reads the FP64 q + dt and writes q (+ the FP32
    shadow).  ``variant_reads`` = the variant's own per-cell reads."""
    w = 8 if precision == "fp64" else 4
    cv = 4 * w
    shadow_w = 0 if precision == "fp64" else cv
    s0 = variant_reads + w + cv
    s1 = variant_reads + cv + w + cv
    s2 = variant_reads + 32 + w + 32 + shadow_w
    return (s0 + s1 + s2) / 3.0


def algorithmic_bytes(kernel, n, f, precision):
    """Compulsory HBM bytes of one launch of ``kernel``: every array element
    the launch must touch, counted once (neighbour re-reads are not counted).
    w = bytes of the arithmetic type; a cell vector is 4w; a face record is
    c0,c1 (8 B) + n, (L, g), d0, d1 (8w)."""
    w = 8 if precision == "fp64" else 4
    cv = 4 * w
    face_geo = 8 + 8 * w
    if kernel == "k_resid_tile":
        # q, gx, gy, phi of every cell, 4 x int16 tile slots, area; faces once
        return n * stage_cell_bytes(precision, 4 * cv + 8 + w) + f * face_geo
    if kernel == "k_resid_gather":
        # q, gx, gy, phi, cslot + cnbr (32), area; face records without c0,c1
        return n * stage_cell_bytes(precision, 4 * cv + 32 + w) + f * 8 * w
    if kernel == "k_face_flux":
        # q, gx, gy, phi of every cell; face records; F*L written (+ eig*L in stage 1)
        return n * 4 * cv + f * (face_geo + 4 * w + w / 3.0)
    if kernel == "k_cell_sum":
        # cslot + cnbr, area, F*L of every face (+ eig*L in stage 1), epilogue
        return n * stage_cell_bytes(precision, 32 + w) + f * (4 * w + w / 3.0)
    if kernel == "k_prep":
        # q, cslot + cnbr, area; n, (L, g), d0, d1; writes gx, gy, phi (+dt for the gather variant)
        return n * (cv + 32 + w + 3 * cv) + f * 8 * w
    if kernel == "k_limiter":
        # qk, gx, gy, cslot + cnbr, area; d0, d1; writes phi
        return n * (4 * cv + 32 + w) + f * 4 * w
    return 0


def kernel_rooflines(prof, n, f, precision, peak):
    """Each profiled kernel's algorithmic bytes per launch over its mean
    CUDA-event launch time, against the HBM peak (the kernels the launch
    list shows beside the dominant one)."""
    out = {}
    for k, (ms, launches) in prof.items():
        ab = algorithmic_bytes(k, n, f, precision)
        if ab <= 0 or launches <= 0 or ms <= 0:
            continue
        gbs = ab / (ms / launches * 1e-3) / 1e9
        out[k] = dict(algorithmic_bytes_per_launch=ab, launch_ms=ms / launches, achieved=gbs, unit="GB/s",
                      frac=gbs / peak)
    return out


def measured_traffic(kernel, precision, n, f):
    """DRAM bytes per launch of ``kernel`` from the committed ncu summary
    (profiles/traffic.json: measured on a smaller channel, per cell and per
    face), scaled to this launch's cells and faces; None if not recorded."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            t = json.load(fh)
        e = t[precision][kernel]
        return e["bytes_per_cell"] * n + e["bytes_per_face"] * f
    except Exception:
        return None


def evaluation_bytes(n, g, f, precision):
    """Compulsory HBM bytes of one cell-residual evaluation of the whole
    mesh (gradient + limiter + flux, one RK stage), each array counted once:
    (N+G)(4 w_s + 3 w_geo) + N (16 w_g + 8 w_phi + 4 w_r) + F (8 + 5 w_geo)
    -- q of every cell and ghost; area and centroid; gx, gy written and read;
    the limiter written and read; R written; per face two cell ids and
    (n_x, n_y, L, x_f, y_f).  FP64: every w = 8; FP32-mixed: w = 4 except
    the FP64 residual (w_r = 8)."""
    w = 8 if precision == "fp64" else 4
    return (n + g) * (4 * w + 3 * w) + n * (16 * w + 8 * w + 4 * 8) + f * (8 + 5 * w)


# FP64 operations (add, sub, mul, div, sqrt each 1) of the explicit scheme,
# hand-counted from the reference's expressions (physics.h:160-264,
# solver.h:308-356, 428-469, 517-593, 745-828), per interior face and per
# cell of ONE iteration (three RK stages) as the GPU path forms it: the
# gradient (formed from the stage-0 state, the same in every stage) and the
# time step once per iteration; limiter, reconstruction and flux per stage.
FLUX_OPS = 207        # internal_flux, inviscid: 18 divisions, 6 square roots
RECON_OPS = 44        # q +- phi (grad q . d), both sides
FLUX_SCATTER_OPS = 12  # F*L and the two accumulations
LIMITER_OPS = 230     # Venkatakrishnan, both sides of the face
GRADIENT_OPS = 73     # Green-Gauss face term (weights, vars(), 4 x 13)
DT_OPS = 38           # spectral radius of both sides, accumulation
CELL_OPS = 70         # gradient / area, dt, 3 x (residual / area + update)


def fp64_ops_per_iteration(n, f):
    per_face = 3 * (FLUX_OPS + RECON_OPS + FLUX_SCATTER_OPS + LIMITER_OPS) + GRADIENT_OPS + DT_OPS
    return f * per_face + n * CELL_OPS


def run_lean(args):
    """Warm-up + K iterations and nothing else (the command profiled by ncu)."""
    from aeroflex_gb300 import meshgen, rans

    marr = meshgen.channel(args.nx, args.ny, jitter=0.2, seed=1, shuffle_seed=2)
    q0 = meshgen.density_bump_state(marr, mach=MACH)
    m = rans.mesh.from_arrays(marr)
    if args.implicit and args.implicit_batch > 0:
        # implicit iterations of a batch of subsonic polar-sweep cases from freestream
        cases = [c for c in meshgen.polar_sweep_cases(256, seed=4) if c["mach"] <= 0.5 and c["aoa_deg"] <= 8.0]
        cases = cases[:args.implicit_batch]
        meshes = [rans.mesh.from_arrays(c["mesh"]) for c in cases]
        for precision in args.precision.split(","):
            sts = []
            for c in cases:
                st = rans.Settings().set("solver", "implicit").set("precision", precision).set("start_cfl", 40.0)
                st.set("slope_cfl", 50.0).set("max_cfl", 100.0).set("krylov_graph", 0 if args.krylov_host_loop else 1)
                st.set_bc("farfield", "farfield", 1.0, c["mach"], c["aoa_deg"] * 0.01745, 1.0).set_bc("wall", "slip-wall")
                sts.append(st)
            b = rans.Batch(meshes, sts)
            b.init()
            b.iterate(args.steps, raise_nonfinite=False)
            print(json.dumps({"implicit_batch": precision, "cases": len(cases), "cells": b.n_cells_total(),
                              "iterations": args.steps, "krylov_last_iteration": int(b.linear_iterations()[0]),
                              "device_s": b.last_device_seconds()}))
            del b
        return
    if args.implicit:
        # two implicit iterations on the 128 x 128 airfoil O-mesh from freestream, CFL 40
        am = rans.mesh.from_arrays(meshgen.airfoil_omesh(128, 128, split=False))
        for precision in args.precision.split(","):
            st = rans.Settings().set("solver", "implicit").set("precision", precision).set("start_cfl", 40.0)
            st.set("krylov_graph", 0 if args.krylov_host_loop else 1)
            st.set_bc("farfield", "farfield", 1.0, 0.5, 1.25 * 0.01745, 1.0).set_bc("wall", "slip-wall")
            g = rans.Solver(am, st)
            g.init()
            g.iterate(args.steps)
            print(json.dumps({"implicit": precision, "cells": am.nRealCells, "iterations": args.steps,
                              "krylov_last_iteration": g.linear_iterations(),
                              "device_s": g.last_device_seconds()}))
            del g
        return
    if args.adjoint:
        # transpose-Jacobian products of the FP64 residual (afx_residual_vjp),
        # for each number of input directions per pass of the face kernel
        v = np.random.default_rng(1).standard_normal(4 * m.nRealCells)
        for k in [int(x) for x in args.adjoint_directions.split(",")]:
            g = _setup_gpu("fp64", m, q0, "face", args.block, k)
            for _ in range(args.warmup):
                g.residual_vjp(v)
            t = time.perf_counter()
            for _ in range(args.steps):
                g.residual_vjp(v)
            print(json.dumps({"adjoint_vjp": True, "directions_per_pass": k, "cells": m.nRealCells,
                              "steps": args.steps,
                              "ms_per_vjp_host": (time.perf_counter() - t) / args.steps * 1e3}))
            del g
        return
    for precision in args.precision.split(","):
        g = _setup_gpu(precision, m, q0, args.variant, args.block)
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
    G = m.n_boundary
    setup_s = time.time() - t0
    hbm_peak, peak_kind = _peaks()
    fp64_peak = rans.measure_fp64_peak(5)
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
                     # the FP64 path is bound by the FP64 pipe (87% active under
                     # ncu): its HBM fraction is reported for reference only
                     roofline=dict(kernel=kname, bound="hbm" if precision == "fp32-mixed" else "fp64-pipe",
                                   achieved=achieved, peak=hbm_peak, unit="GB/s",
                                   frac=achieved / hbm_peak, peak_source=peak_kind,
                                   traffic=measured_traffic(kname, precision, N, F),
                                   algorithmic_bytes_per_launch=ab, launch_ms=per_launch_s * 1e3),
                     gpu_launches=int(round(launches_per_iter * K)))
        try:
            entry["roofline_kernels"] = kernel_rooflines(prof, N, F, precision, hbm_peak)
        except Exception as ex:  # a report, never a reason to lose the line
            entry["roofline_kernels"] = {"error": repr(ex)}
        if precision == "fp32-mixed":
            entry["clocks"] = ck
        # end-to-end through the C ABI, every step: the host state (pinned)
        # to the device, one iteration, the updated state and the residual
        # norm back to pinned host memory
        qh = torch.from_numpy(q0.copy()).pin_memory().numpy() if torch.cuda.is_available() else q0.copy()
        qo = torch.empty(q0.size, dtype=torch.float64).pin_memory().numpy() if torch.cuda.is_available() \
            else np.empty_like(q0)
        Ke = max(3, min(args.steps if precision == "fp32-mixed" else K, 20))
        g.set_q(qh)
        g.iterate(1)
        g.get_q(qo)
        t1 = time.perf_counter()
        for _ in range(Ke):
            g.set_q(qh)
            g.iterate(1)
            g.get_q(qo)
        e2e_s = (time.perf_counter() - t1) / Ke
        entry["e2e"] = dict(value=N * 3 / e2e_s, unit="cell-residual evals/s", h2d_bytes_per_step=N * 32,
                            d2h_bytes_per_step=N * 32 + 8, ms_per_step=e2e_s * 1e3, steps=Ke)
        # the whole evaluation against the compulsory bytes of one evaluation
        eb = evaluation_bytes(N, G, F, precision)
        entry["roofline_evaluation"] = dict(bytes_per_evaluation=eb, achieved=eb * 3 / (sec / K) / 1e9,
                                            peak=hbm_peak, unit="GB/s",
                                            frac=eb * 3 / (sec / K) / 1e9 / hbm_peak, peak_source=peak_kind)
        if precision == "fp64":
            ops = fp64_ops_per_iteration(N, F)
            entry["fp64_ops"] = dict(ops_per_iteration=ops, achieved_tflops=ops / (sec / K) / 1e12,
                                     peak_tflops=fp64_peak, frac=ops / (sec / K) / 1e12 / fp64_peak if fp64_peak else None,
                                     peak_source="measured live: FP64 FMA chains (afx_measure_fp64_peak), "
                                                 "2 flops per FMA; the bit-exact path is compiled without FMA "
                                                 "contraction, so at most half of it is reachable")
        result[precision] = entry
        del g
    return dict(N=N, F=F, setup_s=setup_s, res=result, fp64_peak=fp64_peak)


def time_to_cl(budget_s=60.0):
    """Time to C_L within 1e-6 on the 2-D airfoil case: NACA0012, M 0.5,
    AoA 1.25 deg (0.01745 rad/deg), O-mesh 128 surface x 128 radial quads =
    16,384 cells, far field 20 chords, explicit second-order scheme, CFL 1.5.
    FP64 runs until C_L moves less than 1e-10 between 5000-iteration samples:
    that C_L is the reference.  FP32-mixed C_L, once the FP32 residual floor
    is reached, random-walks by ~1e-6, so its C_L is the mean of the last 10
    samples taken every 1000 iterations; its time-to-C_L is the first time
    that mean is within 1e-6 of the FP64 value and stays so to the end of
    the run.  Times are device seconds (CUDA events) of the iterations;
    force evaluations between samples are not counted."""
    from aeroflex_gb300 import meshgen, rans

    m = rans.mesh.from_arrays(meshgen.airfoil_omesh(128, 128, split=False))

    def solver(prec):
        st = rans.Settings().set("solver", "explicit").set("precision", prec).set("start_cfl", 1.5)
        st.set_bc("farfield", "farfield", 1.0, 0.5, 1.25 * 0.01745, 1.0).set_bc("wall", "slip-wall")
        s = rans.Solver(m, st)
        s.init()
        return s

    t_start = time.time()
    s = solver("fp64")
    samples, dev, last, its = [], 0.0, None, 0
    while its < 200000 and time.time() - t_start < budget_s:
        s.iterate(5000)
        its += 5000
        dev += s.last_device_seconds()
        cl = rans.get_wall_profile(s, "wall")["cl"]
        samples.append((its, dev, cl))
        if last is not None and abs(cl - last) < 1e-10:
            break
        last = cl
    cl64 = samples[-1][2]
    hit64 = next((x for i, x in enumerate(samples) if all(abs(y[2] - cl64) < 1e-6 for y in samples[i:])), None)
    cd64 = rans.get_wall_profile(s, "wall")["cd"]
    del s
    s = solver("fp32-mixed")
    fs, dev, its = [], 0.0, 0
    t1 = time.time()
    while its < 200000 and time.time() - t1 < budget_s / 2:
        s.iterate(1000)
        its += 1000
        dev += s.last_device_seconds()
        w = rans.get_wall_profile(s, "wall")
        fs.append((its, dev, w["cl"], w["cd"]))
    means = [(fs[i][0], fs[i][1], float(np.mean([x[2] for x in fs[max(0, i - 9):i + 1]]))) for i in range(len(fs))]
    hit32 = next((x for i, x in enumerate(means) if i >= 9 and all(abs(y[2] - cl64) < 1e-6 for y in means[i:])), None)
    del s
    # FP32-mixed with the FP64 finish: run_to_convergence in 1000-iteration
    # calls (the FP32 -> FP64 switch persists across calls)
    st = rans.Settings().set("solver", "explicit").set("precision", "fp32-mixed").set("start_cfl", 1.5)
    st.set("fp64_finish", 1)
    st.set_bc("farfield", "farfield", 1.0, 0.5, 1.25 * 0.01745, 1.0).set_bc("wall", "slip-wall")
    s = rans.Solver(m, st)
    s.init()
    ff, dev, its = [], 0.0, 0
    t2 = time.time()
    while its < 200000 and time.time() - t2 < budget_s / 2:
        n_it, _ = s.run_solver(1e-14, 1000)
        its += n_it
        dev += s.last_device_seconds()
        ff.append((its, dev, rans.get_wall_profile(s, "wall")["cl"]))
        if its >= 20000 and abs(ff[-1][2] - cl64) < 1e-8:
            break
    hitf = next((x for i, x in enumerate(ff) if all(abs(y[2] - cl64) < 1e-6 for y in ff[i:])), None)
    out = {"case": "NACA0012 O-mesh 128x128 quads (16,384 cells), M 0.5, AoA 1.25 deg, CFL 1.5",
           "fp64": {"cl": cl64, "cd": cd64, "iterations": samples[-1][0],
                    "time_to_cl_1e-6_s": None if hit64 is None else hit64[1],
                    "iterations_to_cl_1e-6": None if hit64 is None else hit64[0]},
           "fp32_mixed": {"cl_window_mean": means[-1][2], "cl_error": abs(means[-1][2] - cl64),
                          "cl_last_sample_error": abs(fs[-1][2] - cl64), "cd_error": abs(fs[-1][3] - cd64),
                          "iterations": fs[-1][0],
                          "time_to_cl_1e-6_s": None if hit32 is None else hit32[1],
                          "iterations_to_cl_1e-6": None if hit32 is None else hit32[0]}}
    out["fp32_mixed_fp64_finish"] = {"cl": ff[-1][2], "cl_error": abs(ff[-1][2] - cl64), "iterations": ff[-1][0],
                                     "time_to_cl_1e-6_s": None if hitf is None else hitf[1],
                                     "iterations_to_cl_1e-6": None if hitf is None else hitf[0]}
    if hit64 and hit32:
        out["speedup_time_to_cl_fp32_mixed"] = hit64[1] / hit32[1]
    if hit64 and hitf:
        out["speedup_time_to_cl_fp32_mixed_fp64_finish"] = hit64[1] / hitf[1]
    # the implicit solver (the reference's default), FP64 and FP32-mixed
    # (FP32 Jacobian and Krylov vectors, FP64 residual): run_solver in
    # 10-iteration calls, each restarting the CFL ramp 40 -> 90 -> 100
    for prec in ("fp64", "fp32-mixed"):
        st = rans.Settings().set("solver", "implicit").set("precision", prec).set("start_cfl", 40.0)
        st.set("slope_cfl", 50.0).set("max_cfl", 100.0)
        st.set_bc("farfield", "farfield", 1.0, 0.5, 1.25 * 0.01745, 1.0).set_bc("wall", "slip-wall")
        s = rans.Solver(m, st)
        s.init()
        im, dev, its = [], 0.0, 0
        t3 = time.time()
        while its < 2000 and time.time() - t3 < budget_s / 2:
            n_it, _ = s.run_solver(1e-14, 10)
            its += n_it
            dev += s.last_device_seconds()
            im.append((its, dev, rans.get_wall_profile(s, "wall")["cl"]))
            if abs(im[-1][2] - cl64) < 1e-9 or n_it == 0:
                break
        hiti = next((x for i, x in enumerate(im) if all(abs(y[2] - cl64) < 1e-6 for y in im[i:])), None)
        key = "implicit_" + prec.replace("-", "_")
        out[key] = {"cl": im[-1][2], "cl_error": abs(im[-1][2] - cl64), "iterations": im[-1][0],
                    "time_to_cl_1e-6_s": None if hiti is None else hiti[1],
                    "iterations_to_cl_1e-6": None if hiti is None else hiti[0]}
        if hit64 and hiti:
            out["speedup_time_to_cl_" + key] = hit64[1] / hiti[1]
        del s
    return out


def batch_sweep(n_cases=256, K=100, K64=10, warmup=3):
    """Batched polar sweep: ``n_cases`` NACA 4-digit cases (camber U[0,6]%,
    thickness U[8,18]%, camber position U[0.2,0.6], log-uniform 5k-200k
    quad cells, AoA U[-4,12] deg, Mach U[0.1,0.7], seed 4), Euler, CFL 1.
    FP32-mixed batch (one launch per kernel for all cases, autotuned
    variant/block) against the FP64 path run case by case, and the FP64
    batch.  Rate = cells x 3 stages x iterations / device seconds."""
    from aeroflex_gb300 import meshgen, rans

    t0 = time.time()
    cases = meshgen.polar_sweep_cases(n_cases, seed=4)
    meshes = [rans.mesh.from_arrays(c["mesh"]) for c in cases]
    ncell = np.array([m.nRealCells for m in meshes])
    N = int(ncell.sum())

    def settings(c, prec):
        st = rans.Settings().set("solver", "explicit").set("precision", prec).set("start_cfl", 1.0)
        st.set_bc("farfield", "farfield", 1.0, c["mach"], c["aoa_deg"] * 0.01745, 1.0).set_bc("wall", "slip-wall")
        return st

    out = {"cases": n_cases, "cells_total": N, "cells_min": int(ncell.min()), "cells_max": int(ncell.max()),
           "workload": "polar sweep: %d NACA 4-digit O-meshes (quads, log-uniform 5k-200k cells), AoA U[-4,12] deg, "
                       "Mach U[0.1,0.7], Euler, CFL 1, seed 4" % n_cases}
    for prec, k in (("fp32-mixed", K), ("fp64", K64)):
        b = rans.Batch(meshes, [settings(c, prec) for c in cases])
        b.init()
        tuned = b.autotune(2)
        b.init()
        b.iterate(warmup, raise_nonfinite=False)
        b.init()
        norms = b.iterate(k, raise_nonfinite=False)
        sec = b.last_device_seconds()
        out["batch_" + prec.replace("-", "_")] = {
            "value": N * 3 * k / sec, "unit": "cell-residual evals/s", "ms_per_iteration": sec / k * 1e3,
            "iterations": k, "tuned": tuned, "finite_cases": int(np.isfinite(norms).sum())}
        del b
    # the FP64 path case by case (the reference's polar loop, one solver per case)
    dev, its = 0.0, K64
    for c, m in zip(cases, meshes):
        s = rans.Solver(m, settings(c, "fp64"))
        s.init()
        s.iterate(warmup)
        s.init()
        try:
            s.iterate(its)
        except rans.AfxError as e:  # a diverging case: its iterations still ran
            if e.code != 4:
                raise
        dev += s.last_device_seconds()
        del s
    out["per_case_fp64"] = {"value": N * 3 * its / dev, "unit": "cell-residual evals/s",
                            "ms_per_sweep_iteration": dev / its * 1e3, "iterations": its}
    out["speedup_batch_fp32_mixed_vs_per_case_fp64"] = out["batch_fp32_mixed"]["value"] / out["per_case_fp64"]["value"]
    out["speedup_batch_fp64_vs_per_case_fp64"] = out["batch_fp64"]["value"] / out["per_case_fp64"]["value"]
    out["wall_s"] = time.time() - t0
    return out


def batch_converge(n_cases=16, tol=1e-10, max_it=300, max_cells=40000):
    """Batched polar sweep to convergence (the same implicit solver in every
    arm): ``n_cases`` subsonic cases (M <= 0.5, AoA <= 8 deg) of the
    polar-sweep generator (seed 4) with at most ``max_cells`` cells each,
    solved to err/err_0 <= tol as one FP32-mixed batch (FP32 Jacobians and
    Krylov vectors, FP64 residual), as one FP64 batch, and as the FP64
    per-case loop (the reference's polar loop).  Reports device times, the
    FP32-mixed batch's speed-up over the FP64 batch (same algorithm) and
    over the per-case loop, and the largest C_L / C_D difference to the FP64
    batch."""
    from aeroflex_gb300 import meshgen, rans

    cases = [c for c in meshgen.polar_sweep_cases(256, seed=4)
             if c["mach"] <= 0.5 and c["aoa_deg"] <= 8.0 and c["n_cells"] <= max_cells][:n_cases]
    meshes = [rans.mesh.from_arrays(c["mesh"]) for c in cases]

    def settings(c, prec):
        st = rans.Settings().set("solver", "implicit").set("precision", prec).set("start_cfl", 40.0)
        st.set("slope_cfl", 50.0).set("max_cfl", 100.0)
        st.set_bc("farfield", "farfield", 1.0, c["mach"], c["aoa_deg"] * 0.01745, 1.0).set_bc("wall", "slip-wall")
        return st

    t0 = time.time()
    out = {"cases": len(cases), "cells_total": int(sum(m.nRealCells for m in meshes)), "tolerance": tol,
           "workload": "first %d cases with M <= 0.5, AoA <= 8 deg and <= %d cells of the polar-sweep generator "
                       "(seed 4), Euler, implicit solver, CFL 40 -> 100, to err/err_0 <= %g" % (n_cases, max_cells, tol)}
    forces = {}
    for prec in ("fp32-mixed", "fp64"):
        b = rans.Batch(meshes, [settings(c, prec) for c in cases])
        b.init()
        it_b, err_b, st_b = b.run_solver(tol, max_it)
        key = "batch_" + prec.replace("-", "_")
        out[key] = {"device_s": b.last_device_seconds(), "iterations": [int(x) for x in it_b],
                    "converged": int(sum(1 for e in err_b if e <= tol))}
        forces[prec] = [b.forces(k, "wall") for k in range(len(cases))]
        del b
    t64 = 0.0
    its64 = []
    for c, m in zip(cases, meshes):
        s = rans.Solver(m, settings(c, "fp64"))
        s.init()
        try:
            n, e = s.run_solver(tol, max_it)
        except rans.AfxError:
            n = max_it
        t64 += s.last_device_seconds()
        its64.append(int(n))
        del s
    out["per_case_fp64"] = {"device_s": t64, "iterations": its64}
    f32, f64 = forces["fp32-mixed"], forces["fp64"]
    out["max_abs_dcl_fp32_mixed_vs_fp64"] = max(abs(a["cl"] - b["cl"]) for a, b in zip(f32, f64))
    out["max_abs_dcd_fp32_mixed_vs_fp64"] = max(abs(a["cd"] - b["cd"]) for a, b in zip(f32, f64))
    t32 = out["batch_fp32_mixed"]["device_s"]
    out["speedup_batch_fp32_mixed_vs_batch_fp64"] = out["batch_fp64"]["device_s"] / t32 if t32 > 0 else None
    out["speedup_batch_fp32_mixed_vs_per_case_fp64"] = t64 / t32 if t32 > 0 else None
    out["wall_s"] = time.time() - t0
    return out


def c2_time_to_cl(budget32=150.0, budget64=330.0, sample=100):
    """Config 2: NACA0012 on the hybrid boundary-layer mesh (512 x 60 quads,
    first height 1e-6 chord, growth 1.1, Delaunay fill to 100 chords, 201k
    cells), Spalart-Allmaras, Re 6e6, M 0.15, AoA 10 deg, implicit solver
    (first order: the reference's second-order reconstruction diverges on
    this mesh at every CFL tried), CFL 5 -> 200.  The FP32-mixed path runs
    until err/err_0 <= 1e-9 and gives C_L* (within about 3e-8 of the fully
    converged value); the FP64 path runs until its C_L has stayed within 1e-6
    of C_L* for three samples.  Time to C_L within
    1e-6 of C_L* (C_L sampled every ``sample`` iterations, device seconds)
    for both, and the FP32-mixed speed-up."""
    from aeroflex_gb300 import meshgen, rans

    t0 = time.time()
    m = rans.mesh.from_arrays(meshgen.hybrid_airfoil())
    mach, aoa = 0.15, 10.0
    mu = 1.4 * mach / 6e6

    def run(prec, budget, stop):
        st = rans.Settings().set("solver", "implicit").set("precision", prec).set("viscosity", "spalart-allmaras")
        st.set("mu_L", mu).set("second_order", 0.0).set("start_cfl", 5.0).set("slope_cfl", 5.0).set("max_cfl", 200.0)
        st.set_bc("farfield", "farfield", 1.0, mach, aoa * 0.01745, 1.0).set_bc("wall", "wall")
        g = rans.Solver(m, st)
        g.init()
        samples, dev, its, t1, err = [], 0.0, 0, time.time(), 1.0
        while time.time() - t1 < budget:
            n, err = g.run_solver(1e-9, sample)
            its += n
            dev += g.last_device_seconds()
            w = rans.get_wall_profile(g, "wall")
            samples.append((its, dev, w["cl"], w["cd"]))
            if n < sample or stop(samples):
                break
        del g
        return samples, err

    s32, e32 = run("fp32-mixed", budget32, lambda s: False)
    cl_ref = s32[-1][2]
    s64, e64 = run("fp64", budget64,
                   lambda s: len(s) >= 3 and all(abs(x[2] - cl_ref) <= 1e-6 for x in s[-3:]))

    def hit(samples):
        return next((x for i, x in enumerate(samples) if all(abs(y[2] - cl_ref) <= 1e-6 for y in samples[i:])),
                    None)

    h32, h64 = hit(s32), hit(s64)
    out = {"case": "config 2: hybrid mesh %d cells, SA, Re 6e6, M 0.15, AoA 10 deg, implicit first order" %
                   m.nRealCells,
           "cl_converged_fp32_mixed": cl_ref, "err_fp32_mixed": e32, "iterations_fp32_mixed": s32[-1][0],
           "cl_fp64_last": s64[-1][2], "cd_fp64_last": s64[-1][3], "err_fp64": e64, "iterations_fp64": s64[-1][0],
           "cl_error_fp64_vs_fp32_mixed": abs(s64[-1][2] - cl_ref),
           "cd_error_fp64_vs_fp32_mixed": abs(s64[-1][3] - s32[-1][3]),
           "time_to_cl_1e-6_s_fp32_mixed": None if h32 is None else h32[1],
           "time_to_cl_1e-6_s_fp64": None if h64 is None else h64[1],
           "iterations_to_cl_1e-6_fp32_mixed": None if h32 is None else h32[0],
           "iterations_to_cl_1e-6_fp64": None if h64 is None else h64[0]}
    if h32 and h64:
        out["speedup_time_to_cl_fp32_mixed_vs_fp64"] = h64[1] / h32[1]
    out["wall_s"] = time.time() - t0
    return out


def c5_adjoint_coupling(n_fd_dirs=4):
    """Config 5: adjoint sensitivities of C_L and C_D and the aeroelastic
    coupling they drive (Euler, first order, M 0.15, AoA 10 deg).

    - Config 2's full hybrid mesh (201k cells): the FP64 vJP kernel against
      central differences of the residual (steps 1e-7 and 1e-6) along 16
      random unit directions (seed 3) at a generic state.
    - The config 2 generator at 8k cells: the flow to the round-off floor
      (implicit iteration to 1e-6, then the Newton-Krylov finish), both
      adjoints, dC_L/dalpha and the normal-displacement gradients along the
      first ``n_fd_dirs`` of 16 random unit directions (seed 3) against
      central differences (step 1e-7) of converged solutions, then 5
      coupling iterations with the 50-element Euler-Bernoulli beam
      (EI = 1e4 N m^2, clamped at the leading edge) at sea-level q_inf."""
    import math as _m

    import numpy as np

    from aeroflex_gb300 import coupling, meshgen, rans

    t0 = time.time()
    mach, aoa = 0.15, 10.0 * _m.pi / 180
    out = {"case": "config 5: Euler, first order, M 0.15, AoA 10 deg"}

    def settings(solver, prec="fp64"):
        st = rans.Settings().set("solver", solver).set("precision", prec).set("viscosity", "inviscid")
        st.set("second_order", 0.0).set("start_cfl", 10.0 if solver == "implicit" else 1.0)
        st.set("slope_cfl", 20.0).set("max_cfl", 200.0)
        st.set_bc("farfield", "farfield", 1.0, mach, aoa, 1.0).set_bc("wall", "slip-wall")
        return st

    # full mesh: vJP against differences of the residual
    m = meshgen.hybrid_airfoil()
    M = rans.mesh.from_arrays(m)
    g = rans.Solver(M, settings("explicit"))
    g.init()
    g.iterate(20)
    rng = np.random.default_rng(3)
    q = g.get_q()
    q = q * (1 + 1e-3 * rng.standard_normal(q.size))
    v = rng.standard_normal(q.size)
    t = time.time()
    u, _ = g.residual_vjp(v, q=q)
    t_vjp = time.time() - t
    errs, uncs = [], []
    for _ in range(16):
        e = rng.standard_normal(q.size)
        e /= np.linalg.norm(e)
        d = []
        for h in (1e-7, 1e-6):
            g.set_q(q + h * e)
            Rp = g.residual()
            g.set_q(q - h * e)
            Rm = g.residual()
            d.append(float(v @ (Rp - Rm)) / (2 * h))
        errs.append(abs(float(u @ e) - d[0]) / abs(d[0]))
        uncs.append(abs(d[0] - d[1]) / abs(d[0]))
    out["vjp_full_mesh"] = {"cells": M.nRealCells, "directions": 16, "fd_step": 1e-7,
                            "max_rel_diff_vs_fd": max(errs), "max_rel_fd_step_disagreement": max(uncs),
                            "vjp_call_s": t_vjp}
    del g

    # reduced mesh: converged gradients and the coupling
    ms = meshgen.hybrid_airfoil(n_surf=128, bl_layers=16, first=1e-3, growth=1.2, r_far=20.0, fill_cells=6000)
    Ms = rans.mesh.from_arrays(ms)

    def solver():
        g = rans.Solver(Ms, settings("implicit"))
        g.init()
        return g

    def converge(g):
        it, _ = g.run_solver(1e-6, 2000)
        d0 = g.last_device_seconds()
        nn, nk, err = g.newton_solve(3e-12, 30)
        return it, nn, nk, err, d0 + g.last_device_seconds()

    g = solver()
    it, nn, nk, err, dev = converge(g)
    red = {"cells": Ms.nRealCells, "implicit_iterations": it, "newton_steps": nn, "krylov_steps": nk,
           "err": err, "flow_device_s": dev}
    D = rng.standard_normal((16, len(g.patch_nodes("wall")[0])))
    D = D / np.linalg.norm(D, axis=1)[:, None]
    adj = {}
    for obj in ("cl", "cd"):
        (da, dm), ait, ares = g.adjoint_solve("wall", obj, tol=1e-12, max_it=600)
        adj[obj] = {"dalpha": da, "dmach": dm, "krylov_steps": ait, "residual": ares,
                    "device_s": g.last_device_seconds(),
                    "dirs": g.adjoint_patch_dirs(D[:n_fd_dirs], "wall", obj).tolist()}
    fd = {"cl": [], "cd": []}

    def central(deform, h):
        vals = []
        for sg in (1, -1):
            deform(sg * h)
            converge(g)
            vals.append(rans.get_wall_profile(g))
        return {o: (vals[0][o] - vals[1][o]) / (2 * h) for o in ("cl", "cd")}

    da = central(lambda t_: g.set_farfield("farfield", mach, aoa + t_), 1e-5)
    g.set_farfield("farfield", mach, aoa)
    fd5 = {"cl": [], "cd": []}
    for j in range(n_fd_dirs):
        r = central(lambda t_: g.deform_patch(t_ * D[j], "wall"), 1e-7)
        r5 = central(lambda t_: g.deform_patch(t_ * D[j], "wall"), 1e-5)
        for o in ("cl", "cd"):
            fd[o].append(r[o])
            fd5[o].append(r5[o])
    g.deform_patch(np.zeros(D.shape[1]), "wall")
    converge(g)
    red["adjoint"] = {o: {k: adj[o][k] for k in ("dalpha", "dmach", "krylov_steps", "residual", "device_s")}
                      for o in adj}
    red["dalpha_vs_fd"] = {o: {"adjoint": adj[o]["dalpha"], "fd_step_1e-5": da[o],
                               "rel_diff": abs(adj[o]["dalpha"] - da[o]) / abs(da[o])} for o in ("cl", "cd")}
    red["surface_gradient_vs_fd"] = {
        o: {"directions": n_fd_dirs,
            "max_rel_diff_fd_step_1e-7": max(abs(a - b) / abs(b) for a, b in zip(adj[o]["dirs"], fd[o])),
            "max_rel_diff_fd_step_1e-5": max(abs(a - b) / abs(b) for a, b in zip(adj[o]["dirs"], fd5[o]))}
        for o in ("cl", "cd")}
    red["note"] = ("the converged objectives carry a round-off floor of ~5e-13 (the right-hand side's norm "
                   "stops at ~1e-12 of its freestream value), so a central difference with step 1e-7 is "
                   "uncertain by ~1e-4 relative; step 1e-5 brings that to ~1e-6")
    # coupling
    t = time.time()
    cpl = coupling.Coupling(g, Ms, ms, coupling.Beam(50, 1e4), coupling.sea_level_dynamic_pressure(mach),
                            tol=3e-12)
    hist, final = cpl.run(aoa, 5)
    keep = ("cl", "cd", "cy", "tip_deflection_m", "dcl_pred", "dcd_pred", "alpha_equivalent_deg", "step_norm_m",
            "flow_residual", "load_N_per_m")
    red["coupling"] = {"beam": "50 Euler-Bernoulli elements, EI 1e4 N m^2, clamped at the leading edge",
                       "q_inf_Pa": coupling.sea_level_dynamic_pressure(mach),
                       "history": [{k: e[k] for k in keep} for e in hist], "final": final,
                       "wall_s": time.time() - t}
    out["reduced"] = red
    out["wall_s"] = time.time() - t0
    return out


def c5_full(iterations=5, n_fd_dirs=2, smooth=True):
    """Config 5 at its stated size: config 2's hybrid mesh (201k cells),
    Euler, first order, M 0.15, AoA 10 deg.  The primal on an FP32-mixed
    implicit solver (its right-hand side, update and Newton finish are FP64,
    so it converges to the FP64 solution: implicit iteration to 1e-6, then
    the Newton-Krylov finish with its matrix at CFL 2000 to 3e-11, the
    round-off floor there), the adjoints on an FP64 solver of the same mesh
    (FGMRES preconditioned with the transposed matrix at CFL 2e4) from that
    state; gradients of C_L and C_D along 16 random unit normal-displacement
    directions (seed 3).  Central differences of converged solutions check
    them two ways: along the first ``n_fd_dirs`` random directions with
    steps 1e-6 and 3e-7 (node-to-node random displacements of a step of
    1e-5 already reach 40% of the boundary layer's first cell height, 1e-6
    chord, and the cell metrics' curvature then puts ~1e-3 of truncation
    error in the difference), and (``smooth``) along two smooth
    vertical-displacement directions (random sine series over the chord,
    unit norm) with steps 1e-3 and 3e-4; then ``iterations`` coupling
    iterations with the 50-element beam."""
    import math as _m

    import numpy as np

    from aeroflex_gb300 import coupling, meshgen, rans

    t0 = time.time()
    mach, aoa = 0.15, 10.0 * _m.pi / 180

    def solver(M, prec, max_cfl):
        st = rans.Settings().set("solver", "implicit").set("precision", prec).set("viscosity", "inviscid")
        st.set("second_order", 0.0).set("start_cfl", 10.0).set("slope_cfl", 20.0).set("max_cfl", max_cfl)
        st.set_bc("farfield", "farfield", 1.0, mach, aoa, 1.0).set_bc("wall", "slip-wall")
        g = rans.Solver(M, st)
        g.init()
        return g

    m = meshgen.hybrid_airfoil()
    M = rans.mesh.from_arrays(m)
    s32 = solver(M, "fp32-mixed", 200.0)
    s64 = solver(M, "fp64", 2e4)
    out = {"case": "config 5 at size: hybrid mesh %d cells, Euler, first order, M 0.15, AoA 10 deg" % M.nRealCells}

    def converge():
        it, _ = s32.run_solver(1e-6, 3000)
        d0 = s32.last_device_seconds()
        nn, nk, err = s32.newton_solve(3e-11, 30, 2000.0)
        s64.set_q(s32.get_q())
        return {"implicit": it, "newton": nn, "krylov": nk, "err": err,
                "device_s": d0 + s32.last_device_seconds()}

    out["flow"] = converge()
    ids = s64.patch_nodes("wall")[0]
    rng = np.random.default_rng(3)
    D = rng.standard_normal((16, len(ids)))
    D = D / np.linalg.norm(D, axis=1)[:, None]
    xk = m["x"][ids]
    S = np.zeros((2, len(ids), 2))
    for j in range(2):
        c = rng.standard_normal(6)
        S[j, :, 1] = sum(c[k] * np.sin((k + 1) * np.pi * xk) for k in range(6))
        S[j] /= np.linalg.norm(S[j])
    grads, gsm = {}, {}
    for obj in ("cl", "cd"):
        (da, dm), it, res = s64.adjoint_solve("wall", obj, tol=1e-10, max_it=600)
        t = time.time()
        grads[obj] = s64.adjoint_patch_dirs(D, "wall", obj)
        t_dirs = time.time() - t
        gsm[obj] = s64.adjoint_patch_dirs_xy(S, "wall", obj)
        out["adjoint_" + obj] = {"dalpha": da, "dmach": dm, "krylov_steps": it, "residual": res,
                                 "device_s": s64.last_device_seconds(), "gradient_16_dirs_s": t_dirs}

    def central(deform, h):
        vals = []
        for sg in (1, -1):
            for g in (s32, s64):
                deform(g, sg * h)
            converge()
            vals.append(rans.get_wall_profile(s64))
        return {o: (vals[0][o] - vals[1][o]) / (2 * h) for o in ("cl", "cd")}

    rnd = []
    for j in range(n_fd_dirs):
        r6 = central(lambda g, t_: g.deform_patch(t_ * D[j], "wall"), 1e-6)
        r7 = central(lambda g, t_: g.deform_patch(t_ * D[j], "wall"), 3e-7)
        rnd.append({o: {"adjoint": float(grads[o][j]), "fd_step_1e-6": r6[o], "fd_step_3e-7": r7[o],
                        "rel_diff_vs_fd_1e-6": abs(grads[o][j] - r6[o]) / abs(r6[o]),
                        "rel_fd_step_disagreement": abs(r6[o] - r7[o]) / abs(r6[o])} for o in r6})
    sm = []
    for j in range(2 if smooth else 0):
        r3 = central(lambda g, t_: g.deform_patch_xy(0 * S[j, :, 0], t_ * S[j, :, 1], "wall"), 1e-3)
        r4 = central(lambda g, t_: g.deform_patch_xy(0 * S[j, :, 0], t_ * S[j, :, 1], "wall"), 3e-4)
        sm.append({o: {"adjoint": float(gsm[o][j]), "fd_step_1e-3": r3[o], "fd_step_3e-4": r4[o],
                           "rel_diff_vs_fd_3e-4": abs(gsm[o][j] - r4[o]) / abs(r4[o]),
                           "rel_fd_step_disagreement": abs(r3[o] - r4[o]) / abs(r4[o])} for o in r3})
    for g in (s32, s64):
        g.deform_patch(np.zeros(len(ids)), "wall")
    converge()
    out["gradient_vs_fd"] = {"random_normal_directions": rnd, "smooth_vertical_directions": sm}
    if iterations <= 0:
        out["wall_s"] = time.time() - t0
        return out
    t = time.time()
    cpl = coupling.Coupling(s64, M, m, coupling.Beam(50, 1e4), coupling.sea_level_dynamic_pressure(mach),
                            tol=3e-11, adjoint_tol=1e-10, flow_solver=s32, newton_cfl=2000.0)
    hist, final = cpl.run(aoa, iterations)
    keep = ("cl", "cd", "cy", "tip_deflection_m", "dcl_pred", "dcd_pred", "alpha_equivalent_deg", "step_norm_m",
            "flow_iterations", "flow_residual", "adjoint_cl", "adjoint_cd")
    out["coupling"] = {"history": [{k: e[k] for k in keep} for e in hist], "final": final,
                       "wall_s": time.time() - t}
    out["wall_s"] = time.time() - t0
    return out


def cpu_baseline(budget_s=12.0):
    """The oracle (plain-C++ restatement of the reference's explicit solver:
    serial face loops, OpenMP per-cell loops as the reference) on a 512 x 256
    sample of the same generator, with all host threads and with one thread,
    plus its time per iteration on the 128 x 128 airfoil case, from which the
    CPU time to C_L within 1e-6 is extrapolated with the FP64 GPU path's
    iteration count (same arithmetic, so the same iterations)."""
    from aeroflex_gb300 import meshgen
    from oracle import oracle

    marr = meshgen.channel(SAMPLE_NX, SAMPLE_NY, jitter=0.2, seed=1, shuffle_seed=2)
    s = oracle.Solver(oracle.Mesh.from_arrays(marr), oracle.default_settings(cfl=1.0), {
        "farfield": dict(type="farfield", T=1.0, mach=MACH, angle=0.0, p=1.0), "wall": dict(type="slip-wall")})
    s.init()
    s.set_q(meshgen.density_bump_state(marr, mach=MACH))
    n = SAMPLE_NX * SAMPLE_NY * 2
    out = {}
    for threads, budget in ((0, budget_s), (1, budget_s / 2)):
        oracle.set_threads(threads)
        s.time_iterations(1)
        its, sec = 0, 0.0
        while sec < budget:
            sec += s.time_iterations(1)
            its += 1
        out[threads] = (n * 3 * its / sec, its)
    # the airfoil case of the time-to-C_L leg
    am = meshgen.airfoil_omesh(128, 128, split=False)
    a = oracle.Solver(oracle.Mesh.from_arrays(am), oracle.default_settings(cfl=1.5), {
        "farfield": dict(type="farfield", T=1.0, mach=0.5, angle=1.25 * 0.01745, p=1.0), "wall": dict(type="slip-wall")})
    a.init()
    oracle.set_threads(0)
    a.time_iterations(2)
    t_it = a.time_iterations(20) / 20
    oracle.set_threads(0)
    return {"value": out[0][0], "unit": "cell-residual evals/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "%d explicit iterations on the %dx%d channel (%d cells), all %d host threads" %
                      (out[0][1], SAMPLE_NX, SAMPLE_NY, n, os.cpu_count()),
            "one_thread": {"value": out[1][0], "iterations": out[1][1]},
            "airfoil_ms_per_iteration": t_it * 1e3,
            "airfoil_time_to_cl_1e-6_s_extrapolated": t_it * 35000,
            "airfoil_note": "128x128 quad O-mesh, CFL 1.5: 35,000 iterations to C_L within 1e-6 (the FP64 GPU "
                            "path's count, bit-identical arithmetic) x the measured time per iteration"}


def workload_config(n, f, world=1):
    """The config object both arms print (the same workload)."""
    return {"workload": "channel 2048x1024 quads -> %d shuffled triangles, M 0.3 density bump, explicit "
                        "second-order residual (Green-Gauss, Venkatakrishnan K 5, Roe), CFL 1" % n,
            "cells": n, "faces": f, "l2": "inputs larger than L2 (~1 GB touched per step)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def run_reference(args):
    """The reference's CPU implementation of the path on the machine's host
    cores: the oracle port (bit-identical to the reference's own code on the
    committed pins; the reference's tree is not on the box), all host
    threads, on the full channel mesh of the GPU arm.  One step = one
    second-order residual evaluation of every cell (time step, gradient,
    limiter, face loop), the unit the GPU arm counts three times per
    iteration."""
    from aeroflex_gb300 import meshgen
    from oracle import oracle

    marr = meshgen.channel(args.nx, args.ny, jitter=0.2, seed=1, shuffle_seed=2)
    om = oracle.Mesh.from_arrays(marr)
    s = oracle.Solver(om, oracle.default_settings(cfl=1.0), {
        "farfield": dict(type="farfield", T=1.0, mach=MACH, angle=0.0, p=1.0), "wall": dict(type="slip-wall")})
    s.init()
    s.set_q(meshgen.density_bump_state(marr, mach=MACH))
    n, f = om.n_real, om.n_edges
    oracle.set_threads(0)
    t_first = s.time_residuals(1)
    for _ in range(args.warmup - 1):
        s.time_residuals(1)
    # a step is a full-mesh evaluation (about 2 s on 16 cores): large step
    # counts are cut to what fits in about two minutes, and the line says so
    steps = max(1, min(args.steps, int(120.0 / max(t_first, 1e-3))))
    sec = s.time_residuals(steps)
    v = n * steps / sec
    line = {"metric": "cell-residual evals/s", "value": v, "unit": "cell-residual evals/s", "n_gpus": args.gpus,
            "steps": steps, "steps_requested": args.steps, "warmup": args.warmup,
            "ms_per_step": sec / steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": workload_config(n, f),
            "cpu_baseline": {"value": v, "unit": "cell-residual evals/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "%d second-order residual evaluations of the full %d-cell channel, all %d "
                                       "host threads (OpenMP per-cell loops, serial face loops, as the reference)"
                                       % (steps, n, os.cpu_count())},
            "e2e": {"value": v, "unit": "cell-residual evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-cl", action="store_true", help="skip the time-to-C_L leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched polar-sweep leg")
    ap.add_argument("--batch-cases", type=int, default=256)
    ap.add_argument("--no-batch-converge", action="store_true",
                    help="skip the batched polar sweep to convergence (FP32-mixed batch vs FP64 batch vs per case)")
    ap.add_argument("--no-c2", action="store_true", help="skip the config 2 (SA, hybrid mesh) time-to-C_L leg")
    ap.add_argument("--no-c5", action="store_true", help="skip the config 5 (adjoint + coupling) leg")
    ap.add_argument("--c5-only", action="store_true", help="run the config 5 leg alone and print it")
    ap.add_argument("--c5-full", action="store_true",
                    help="run config 5 at its stated size (201k cells; about 10 minutes) alone and print it")
    ap.add_argument("--c5-full-iterations", type=int, default=5,
                    help="--c5-full: coupling iterations (0: the gradients and their checks only)")
    ap.add_argument("--c5-full-no-smooth", action="store_true",
                    help="--c5-full: skip the differences along smooth directions")
    ap.add_argument("--nx", type=int, default=NX)
    ap.add_argument("--ny", type=int, default=NY)
    ap.add_argument("--lean", action="store_true", help="warm-up + timed iterations only (for ncu)")
    ap.add_argument("--precision", default="fp32-mixed", help="--lean: comma-separated precisions")
    ap.add_argument("--variant", default="auto", help="--lean: residual kernel variant (auto|gather|face|tile)")
    ap.add_argument("--block", type=int, default=0, help="--lean: threads per block (0: the library's default)")
    ap.add_argument("--adjoint", action="store_true", help="--lean: FP64 residual vJP calls instead of iterations")
    ap.add_argument("--adjoint-directions", default="4",
                    help="--lean --adjoint: comma-separated input directions per pass of the face kernel (1, 2, 4)")
    ap.add_argument("--implicit", action="store_true",
                    help="--lean: implicit iterations on the 128x128 airfoil O-mesh (--steps of them)")
    ap.add_argument("--implicit-batch", type=int, default=0,
                    help="--lean --implicit: a batch of this many subsonic polar-sweep cases instead")
    ap.add_argument("--krylov-host-loop", action="store_true",
                    help="--lean --implicit: GMRES loops on the host, every kernel a plain launch (for ncu)")
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
    if args.c5_only:
        print(json.dumps({"c5_adjoint_coupling": c5_adjoint_coupling()}))
        return
    if args.c5_full:
        print(json.dumps({"c5_full": c5_full(args.c5_full_iterations, smooth=not args.c5_full_no_smooth)}))
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
        "config": workload_config(r["N"], r["F"], world),
        "roofline": {k: f32["roofline"][k] for k in ("bound", "achieved", "peak", "unit", "frac", "traffic")},
        "roofline_kernel": f32["roofline"],
        "roofline_evaluation": f32["roofline_evaluation"],
        "roofline_kernels": f32["roofline_kernels"],
        "kernels": f32["kernels"],
        "clocks": f32["clocks"],
        "e2e": f32["e2e"],
        "gpu_launches": f32["gpu_launches"],
        "tuned": f32["tuned"],
        # the bit-exact FP64 path (the reference's arithmetic), same workload
        "fp64": {"value": f64["value"], "unit": "cell-residual evals/s", "ms_per_step": f64["ms_per_step"],
                 "steps": f64["steps"], "dtype": "f64", "e2e": f64["e2e"], "tuned": f64["tuned"],
                 "fp64_ops": f64["fp64_ops"], "roofline_evaluation": f64["roofline_evaluation"],
                 "roofline_kernel": f64["roofline"], "roofline_kernels": f64["roofline_kernels"],
                 "kernels": f64["kernels"], "gpu_launches": f64["gpu_launches"]},
        "setup_s": r["setup_s"],
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline()
    if not args.no_cl:
        line["time_to_cl"] = time_to_cl()
    if not args.no_batch:
        line["batch"] = batch_sweep(args.batch_cases)
    if not args.no_batch_converge:
        line["batch_converge"] = batch_converge()
    if not args.no_c2:
        line["c2_time_to_cl"] = c2_time_to_cl()
    if not args.no_c5:
        line["c5_adjoint_coupling"] = c5_adjoint_coupling()
    print(json.dumps(line))


if __name__ == "__main__":
    main()
