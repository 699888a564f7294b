#!/usr/bin/env python
"""Forward + adjoint solves per second on one GB300 (the headline metric).

Workload C2 (the reference's "plain FP64 forward solve on GPU"
configuration, driven to the gradient as an inversion iteration does): a
0.5 ohm-m block in a 10/100/1000 ohm-m three-layer earth, octree min/max
level 6/7 (1.69M edges), 121 stations on an 11x11 grid at 1 km, 8
frequencies log-spaced 0.01-100 Hz, both polarisations.  One step = forward
solves for all 16 (frequency, polarisation) right-hand sides, weighted
residual, 16 adjoint solves and the J^T r sensitivity: 32 solves, each driven
to ||b - A x|| / ||b|| <= 1e-7 checked in FP64 (InversionFV::compute_gradient_
of the reference for every frequency).  Synthetic data: seeded 5 % noise on
the 1-D 100 ohm-m halfspace impedance.

  value   : solves/s, device-event time of the step with sigma resident
  e2e     : solves/s through the public C ABI with host buffers (set_sigma +
            gradient call, host<->device copies inside the timed region)
  plain   : the same step as the plain FP64 GPU solve (one frequency per call,
            complex128 SSOR-BiCGStab, Jacobi divergence correction), measured
            in the same run: the denominator of the batched-vs-plain ratio
  cpu_baseline : the reference's CPU algorithm (the C restatement in oracle/)
            on the host cores, converged solves of a stated sample

`--impl reference` times the reference's CPU algorithm alone on all host
cores (complete adjoint solves of the two highest frequencies, one process
per core as the reference's frequency-parallel MPI groups), with its mesh read
from the committed leaf list (oracle/leaves/) so that the GPU library is never
loaded.  Under torchrun (N > 1) frequencies are split round-robin over the
ranks (freq_parallel.cpp:99-117) and the gradient is summed once.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+adjoint solves/sec per GB300, learned+batched vs plain, at 1e-7 rel residual"
UNIT = "solves/s"
TOL = 1e-7


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c2", "c3", "c5"],
                    help="c2: the headline workload; c3: one mesh per frequency (16 meshes of 0.9-3.0 M "
                         "edges, 0.001-1000 Hz), forward + per-station adjoint gradients, meshes run "
                         "concurrently; c5: the inversion iteration at scale (levels 6/8, "
                         "3.1 M edges, 400 stations, 24 frequencies 0.001-1000 Hz, data from a random model)")
    ap.add_argument("--c3-freqs", type=int, default=16, help="c3: frequencies (meshes) of the 16, evenly spread")
    ap.add_argument("--c3-sources", type=int, default=8,
                    help="c3: station sources per mesh (2 adjoint solves each; the full workload has 121)")
    ap.add_argument("--c3-concurrent", type=int, default=4, help="c3: handles run at once (0: all)")
    ap.add_argument("--c3-replicas", type=int, default=1,
                    help="c3: handles per mesh, the mesh's station sources split across them (each also solves "
                         "the mesh's forward problem; those repeated forward solves are not counted)")
    # profiling runs only: a smaller mesh of the same survey (octree levels)
    ap.add_argument("--min-level", type=int, default=0, help="override the configuration's min octree level")
    ap.add_argument("--max-level", type=int, default=0, help="override the configuration's max octree level")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--forward", default="reference", choices=["interleaved", "reference"])
    # profiling runs only (a capped solve is not a bench number): Krylov
    # iteration cap per solve
    ap.add_argument("--maxiter", type=int, default=5000)
    ap.add_argument("--arm", default="batched", choices=["batched", "plain"],
                    help="plain: time only the plain FP64 GPU arm as the main value (profiling)")
    ap.add_argument("--plain-steps", type=int, default=1,
                    help="timed steps of the plain FP64 arm measured after the batched arm (0: skip)")
    ap.add_argument("--plain-row-kernels", type=int, default=1, choices=[0, 1])
    ap.add_argument("--ssor-form", type=int, default=1, choices=[0, 1],
                    help="inner FP32 solve of batches without the gradient-space term: "
                         "0 right-preconditioned SSOR-BiCGStab, 1 Eisenstat split form")
    ap.add_argument("--divcorr-precond", type=int, default=1, choices=[0, 1],
                    help="divergence-correction PCG: 0 Jacobi (the reference's), 1 aggregation multigrid")
    ap.add_argument("--row-kernels", type=int, default=1, choices=[0, 1],
                    help="0: CSR rows read by the lanes; 1: slice-staged rows (bulk copies to shared memory)")
    ap.add_argument("--gradcorr", type=int, default=1, choices=[0, 1],
                    help="1: gradient-space term (multigrid V-cycle on the divergence-correction Laplacian) in "
                         "the FP32 inner solve's preconditioner for frequencies <= --gradcorr-fmax")
    ap.add_argument("--gradcorr-fmax", type=float, default=1e30)
    ap.add_argument("--gradcorr-presmooth", type=int, default=0, choices=[0, 1])
    ap.add_argument("--divcorr-mixed", type=int, default=1, choices=[0, 1])
    ap.add_argument("--inner-tol-floor", type=float, default=3e-5)
    ap.add_argument("--residual-replacement", type=int, default=0, choices=[0, 1])
    ap.add_argument("--gradcorr-overlap", type=int, default=1, choices=[0, 1])
    ap.add_argument("--sweep-rows", type=int, default=0,
                    help="SSOR ordering by (super-block, colour), super-blocks of about this many edges (0: off)")
    ap.add_argument("--ssor-relax", type=float, default=1.0,
                    help="SSOR relaxation factor of the FP32 inner solve (1: the reference's symmetric GS)")
    ap.add_argument("--cuda-graphs", type=int, default=0, choices=[0, 1],
                    help="replay the inner solve's 10-iteration chunks from CUDA graphs")
    ap.add_argument("--coop-sweep", type=int, default=0, choices=[0, 1],
                    help="1: each staged SSOR sweep as one cooperative launch over its groups")
    ap.add_argument("--learned-steps", type=int, default=1,
                    help="timed steps of the learned arm (FGMRES with the trained network; 0: skip)")
    ap.add_argument("--learned-pairs", type=int, default=1024, help="training pairs the learned arm collects")
    ap.add_argument("--fgmres-m", type=int, default=40, help="FGMRES restart length of the learned arm")
    ap.add_argument("--kernel-timing", type=int, default=1, choices=[0, 1],
                    help="CUDA events around every launch in the timed steps (kernel classes, roofline)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--cpu-procs", type=int, default=0, help="CPU worker processes (0: all host cores)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# the workload (identical inputs for both arms)
# ---------------------------------------------------------------------------

CONFIG = "c2"
LEVELS = (0, 0)   # profiling overrides of (min, max) octree level


def spec():
    import dataclasses
    from maple3dmt_gb300 import workloads
    sp = {"c2": workloads.C2, "c5": workloads.C5}[CONFIG]
    if LEVELS[0]:
        sp = dataclasses.replace(sp, min_level=LEVELS[0])
    if LEVELS[1]:
        sp = dataclasses.replace(sp, max_level=LEVELS[1])
    return sp


def survey_inputs(stations=None):
    """Stations, frequencies, observed data and errors of the workload."""
    import numpy as np
    from maple3dmt_gb300 import workloads
    sp = spec()
    st = workloads.station_grid(sp.n_side, sp.spacing) if stations is None else stations
    fr = np.asarray(sp.freqs, np.float64)
    obs, err = workloads.halfspace_data(st, fr, seed=42)
    return st, fr, obs, err


def bench_config(ne, nc):
    sp = spec()
    nf = len(sp.freqs)
    model = ("C2: layered+block earth" if CONFIG == "c2" else
             "C5: 100 ohm-m starting halfspace, data from a seeded random layered+blocks model with 5 % noise")
    return {"workload": f"{model}, octree levels {sp.min_level}/{sp.max_level} ({ne} edges, "
                        f"{nc} cells), {sp.n_side * sp.n_side} stations, {nf} freqs "
                        f"{min(sp.freqs):g}-{max(sp.freqs):g} Hz, forward+adjoint+sensitivity gradient step "
                        f"({4 * nf} solves)",
            "tol": TOL, "l2": "inputs larger than L2 (matrix alone 260 MB, K=16 FP32 vector 216 MB at C2)"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = str(gpu_index)
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if parts and parts[0] == self.idx:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel_class):
    """Per-launch DRAM bytes of the class from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith(kernel_class + ":"):
                    return float(line.split(":")[1].split()[0])
    except OSError:
        pass
    return None


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


# ---------------------------------------------------------------------------
# the reference's CPU algorithm (oracle/ C restatement, verbatim arithmetic
# of the reference pinned bit for bit by tests/test_oracle.py)
# ---------------------------------------------------------------------------

CPU_FREQS = 2     # the sample: adjoint solves of the highest CPU_FREQS frequencies


def _cpu_worker(conn, wid, freq_index):
    """One host process = one frequency group of the reference's MPI mode.
    Setup: the leaf list, the reference's forward solve of its frequency (both
    polarisations, timed and reported), the adjoint sources of the weighted
    residual.  Then each 'solve' command runs one complete adjoint solve
    (solve_with_divcorr_, stopped by the reference's own tests at 1e-7)."""
    import numpy as np
    import oracle
    from oracle import leaflist
    from maple3dmt_gb300 import workloads
    lv = leaflist.load("c2")
    sigma = workloads.cell_sigma(lv["cell_type"], lv["cx"], lv["cy"], lv["cz"], workloads.layered_block_sigma)
    st, fr, obs, err = survey_inputs()
    f = float(fr[freq_index])
    case = oracle.Case(domain=lv["domain"], min_level=lv["min_level"], max_level=lv["max_level"],
                       level=lv["level"], cx=lv["cx"], cy=lv["cy"], cz=lv["cz"], cell_type=lv["cell_type"],
                       sigma=sigma, sigma_bg=workloads.SIGMA_BG, stations=st, freqs=[f], tol=TOL, maxiter=5000)
    o = oracle.Oracle(case)
    t0 = time.perf_counter()
    Z = o.solve_frequency(f)
    t_fwd = time.perf_counter() - t0
    it_fwd = o.last_iters()
    e = err[:, freq_index, :]
    w2 = np.where(e > 0, 1.0 / np.where(e > 0, e, 1.0) ** 2, 0.0)
    wr = w2 * np.conj(obs[:, freq_index, :] - Z)
    rhs = o.adjoint_rhs(wr)
    conn.send(("ready", o.ne, o.nc, t_fwd, it_fwd, f))
    k = 0
    while True:
        cmd = conn.recv()
        if cmd != "solve":
            break
        t0 = time.perf_counter()
        o.adjoint_solve(rhs[k % 2])
        dt = time.perf_counter() - t0
        conn.send(("done", dt, o.last_iters()))
        k += 1
    conn.close()


class CpuReference:
    """P spawned worker processes (spawn: safe after CUDA use in the parent)."""

    def __init__(self, procs):
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        self.procs = procs
        self.pipes, self.workers = [], []
        for w in range(procs):
            a, b = ctx.Pipe()
            fi = len(spec().freqs) - 1 - (w % CPU_FREQS)
            p = ctx.Process(target=_cpu_worker, args=(b, w, fi), daemon=True)
            p.start()
            self.pipes.append(a)
            self.workers.append(p)
        t0 = time.perf_counter()
        self.ready = [c.recv() for c in self.pipes]
        self.setup_s = time.perf_counter() - t0
        self.ne, self.nc = self.ready[0][1], self.ready[0][2]

    def step(self, n_workers=None):
        """All (or the first n) workers solve one adjoint RHS at once; returns
        (wall seconds, per-solve seconds, iterations)."""
        use = self.pipes[: n_workers or self.procs]
        t0 = time.perf_counter()
        for c in use:
            c.send("solve")
        res = [c.recv() for c in use]
        wall = time.perf_counter() - t0
        return wall, [r[1] for r in res], [r[2] for r in res]

    def close(self):
        for c in self.pipes:
            try:
                c.send("stop")
            except (OSError, BrokenPipeError):
                pass
        for p in self.workers:
            p.join(timeout=10)

    def describe(self, steps, one_core=None):
        fwd = sorted({(round(r[5], 3), r[3], tuple(r[4])) for r in self.ready})
        d = (f"{self.procs} processes (one per host core, frequency groups as the reference's MPI mode), each "
             f"running complete adjoint solves (solve_with_divcorr_: lexicographic SSOR-BiCGStab with "
             f"divergence correction, the reference's own 1e-7 stopping tests) of the "
             f"{CPU_FREQS} highest C2 frequencies on the full C2 system, {steps} step(s) of {self.procs} "
             f"concurrent solves; setup per process (untimed): the forward solve of its frequency, "
             + ", ".join(f"{f} Hz: {t:.1f} s, iterations {list(it)}" for f, t, it in fwd))
        if one_core is not None:
            d += f"; 1 core alone: {one_core:.3f} solves/s"
        return d


def cpu_measure(steps, warmup, procs, one_core=True):
    procs = procs or (os.cpu_count() or 1)
    ref = CpuReference(procs)
    try:
        for _ in range(warmup):
            ref.step()
        v1 = None
        if one_core:
            wall1, _, _ = ref.step(1)
            v1 = 1.0 / wall1
        walls, iters = [], []
        for _ in range(steps):
            wall, _, it = ref.step()
            walls.append(wall)
            iters += it
        total = sum(walls)
        value = procs * steps / total
        cb = {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
              "sample": ref.describe(steps, v1), "value_1core": v1, "cpu_model": cpu_model(),
              "nproc": os.cpu_count(), "iterations_per_solve": iters[: 2 * CPU_FREQS],
              "setup_s": ref.setup_s}
        return cb, total / steps, ref.ne, ref.nc
    finally:
        ref.close()


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    if CONFIG != "c2" or LEVELS != (0, 0):
        print(json.dumps({"impl": "reference", "unavailable": "the CPU reference sample is defined on the C2 mesh "
                          "(its leaf list is committed; C5 data come from a GPU forward solve)"}), flush=True)
        return
    W, K = args.warmup, args.steps
    # the CPU has no caches or JIT state that warm-up would settle beyond the
    # per-process setup; one warm-up step stands for all W
    cb, sec_per_step, ne, nc = cpu_measure(K, min(W, 1), args.cpu_procs, one_core=True)
    v = cb["value"]
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": K, "warmup": W, "ms_per_step": sec_per_step * 1000.0, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": bench_config(ne, nc), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def solver_params(args, plain):
    p = dict(bicgstab_tol=TOL, bicgstab_maxiter=args.maxiter)
    if plain:   # the reference's algorithm on the GPU: FP64, SSOR alone, Jacobi DivCorr; forward solves run
        # solve_with_divcorr_ like the adjoint ones (the reference's forward strategy, BiCGStab to 1e-7 then one
        # correction, does not reach 1e-7 at 0.01 Hz on this mesh within 5000 iterations)
        p.update(precision=0, forward_interleaved=1, row_kernels=args.plain_row_kernels, divcorr_precond=0,
                 ssor_form=0, gradcorr=0, divcorr_mixed=0)
    else:
        p.update(precision=1 if args.precision == "mixed" else 0,
                 forward_interleaved=1 if args.forward == "interleaved" else 0,
                 row_kernels=args.row_kernels, divcorr_precond=args.divcorr_precond, ssor_form=args.ssor_form,
                 gradcorr=args.gradcorr, gradcorr_fmax=args.gradcorr_fmax,
                 gradcorr_presmooth=args.gradcorr_presmooth, divcorr_mixed=args.divcorr_mixed,
                 inner_tol_floor=args.inner_tol_floor, residual_replacement=args.residual_replacement,
                 gradcorr_overlap=args.gradcorr_overlap, sweep_rows=args.sweep_rows,
                 coop_sweep=args.coop_sweep, ssor_relax=args.ssor_relax, cuda_graphs=args.cuda_graphs)
    return p


def solver_label(args, p, freqs):
    if not p["precision"]:
        return {"arm": "plain FP64: one frequency per call, complex128 SSOR-BiCGStab, "
                       + ["csr", "staged"][p["row_kernels"]]
                       + " row kernels, Jacobi-PCG divergence correction, solve_with_divcorr_ for every solve"}
    gc_all = p["gradcorr"] and p["gradcorr_fmax"] >= max(freqs)
    gc_none = not p["gradcorr"] or p["gradcorr_fmax"] < min(freqs)
    eis = "Eisenstat split form" if p["ssor_form"] else "right-preconditioned"
    form = ("right-preconditioned (every batch carries the gradient-space term)" if gc_all
            else eis if gc_none else f"right-preconditioned with the term, {eis} above {p['gradcorr_fmax']:g} Hz")
    return {"arm": "batched", "precision": args.precision, "inner_tol_floor": p["inner_tol_floor"],
            "forward": args.forward, "row_kernels": ["csr", "staged"][p["row_kernels"]],
            "divcorr_precond": ["jacobi", "multigrid"][p["divcorr_precond"]],
            "divcorr_solve": ["fp64 pcg", "fp32 pcg in fp64 refinement"][p["divcorr_mixed"]],
            "ssor_form_run": form,
            "gradcorr": (f"multigrid gradient-space term, V({p['gradcorr_presmooth']},1)"
                         + (", V-cycle on a second stream" if p["gradcorr_overlap"] else "")) if p["gradcorr"]
            else "off",
            "residual_replacement": bool(p["residual_replacement"]),
            "sweep_rows": p["sweep_rows"], "coop_sweep": bool(p["coop_sweep"]), "ssor_relax": p["ssor_relax"],
            "cuda_graphs": bool(p["cuda_graphs"])}


def run_steps(s, sv, obs, err, steps, warmup, rank, world, dist, clocks=None, per_freq=False, timing=True):
    """Warm-up, then `steps` timed gradient steps; returns timing and stats.
    per_freq: one gradient_batch call per frequency (the plain arm)."""
    import numpy as np
    from maple3dmt_gb300 import freq_parallel

    def allreduce(v):
        import torch
        t = torch.from_numpy(v)
        dist.all_reduce(t)
        return t.numpy()

    calls = []   # per-call stats of the last per-frequency step

    class PerFrequency:   # gradient_batch face, one call per frequency
        nc = s.nc

        @staticmethod
        def gradient_batch(freqs, o, e):
            Zs, g = [], 0.0
            calls.clear()
            for f in range(len(freqs)):
                Zf, gf = s.gradient_batch(freqs[f:f + 1], np.ascontiguousarray(o[:, f:f + 1]),
                                          np.ascontiguousarray(e[:, f:f + 1]))
                calls.append(s.stats())
                Zs.append(Zf)
                g = g + gf
            return np.concatenate(Zs), g

    solver = PerFrequency if per_freq else s

    def step():
        return freq_parallel.gradient_step(solver, sv.freqs, obs, err, rank, world, allreduce if dist else None)

    def barrier():
        if dist:
            dist.barrier()

    for _ in range(warmup):
        step()
    barrier()
    if clocks:
        clocks.start()
    s.set_kernel_timing(timing)
    launches0 = s.stats()["kernel_launches"]
    dev_ms, e2e_s, solves = 0.0, 0.0, 0
    iters, st = [], None
    for _ in range(steps):
        barrier()
        t0 = time.perf_counter()
        s.set_sigma(sv.sigma)                  # host -> device conductivity
        s.timer_start()
        _, _, _, n = step()
        dev_ms += s.timer_stop()
        e2e_s += time.perf_counter() - t0
        solves += n
        st = s.stats()
        iters.append(st["total_iterations"])
    launches = s.stats()["kernel_launches"] - launches0
    kt = s.kernel_times()
    s.set_kernel_timing(False)
    clk = clocks.stop() if clocks else None
    if per_freq and calls:   # the step's calls together
        st = dict(calls[-1])
        st["true_residual"] = [t for c in calls for t in c["true_residual"][:c["n_rhs"]]]
        st["iterations"] = [t for c in calls for t in c["iterations"][:c["n_rhs"]]]
        st["n_rhs"] = len(st["true_residual"])
        for key in ("forward_iterations", "adjoint_iterations", "divcorr_cg_iterations", "divcorr_cg_sweeps"):
            st[key] = sum(c[key] for c in calls)
        iters[-1] = sum(st["iterations"])
    tr = st["true_residual"][:st["n_rhs"]]
    stats = {k: st[k] for k in ("forward_iterations", "adjoint_iterations", "refinements", "divcorr_calls",
                                "divcorr_outer", "divcorr_cg_iterations", "divcorr_cg_sweeps", "replacements")}
    stats.update(iterations_per_rhs=st["iterations"], rhs_at_tol=sum(1 for t in tr if t <= TOL),
                 rhs_reported=len(tr), true_residual_max=max(tr) if tr else None)
    return dict(t_dev=dev_ms / 1000.0, e2e_s=e2e_s, solves=solves, launches=launches, kt=kt, clocks=clk,
                iters=iters, stats=stats)


def run_learned(args, sv, obs, err, local_rank):
    """The learned arm on the same step: a 6-layer 32-channel network on a
    32^3 grid, trained on the GPU from (residual -> error) pairs that the
    plain FP64 SSOR-BiCGStab records while solving the step's frequencies
    from 0.1 Hz up (untimed, reported), then the step with flexible GMRES
    whose every second direction is the two-level step with the network as
    coarse solve, and the same FGMRES without the network (the gain)."""
    from maple3dmt_gb300.solver import solver_for_survey
    p = solver_params(args, False)
    p.update(krylov=1, fgmres_m=args.fgmres_m, learned_period=2)
    s = solver_for_survey(sv, device=local_rank, **p)
    try:
        t0 = time.perf_counter()
        s.learn_setup(grid_level=5, layers=6, hidden=32, seed=1, max_samples=args.learned_pairs)
        n = s.learn_collect(sv.freqs[sv.freqs >= 0.1])
        t1 = time.perf_counter()
        hist, val = s.learn_train(epochs=8, lr=1e-3, batch=16, seed=3, val_frac=0.1)
        t2 = time.perf_counter()
        out = {"unit": UNIT, "steps": args.learned_steps, "warmup": 1, "network": "6 x conv3x3x3, 32 channels, "
               "BF16 tcgen05 kernels, 32^3 grid", "krylov": f"FGMRES({args.fgmres_m}), network every 2nd direction",
               "pairs": n, "collect_s": t1 - t0, "train_s": t2 - t1, "train_loss": [hist[0], hist[-1]],
               "held_out_loss": val}
        for period, key in ((2, "with_network"), (0, "without_network")):
            s.set_params(learned_period=period)
            r = run_steps(s, sv, obs, err, args.learned_steps if period else 1, 1 if period else 0, 0, 1, None)
            out[key] = {"value": r["solves"] / r["t_dev"], "ms_per_step": r["t_dev"] * 1000.0 / max(1, len(r["iters"])),
                        "krylov_iterations_per_step": statistics.mean(r["iters"]),
                        "rhs_at_tol": r["stats"]["rhs_at_tol"], "rhs_reported": r["stats"]["rhs_reported"]}
        out["value"] = out["with_network"]["value"]
        return out
    finally:
        s.close()


def run_ours(args, rank, world, local_rank):
    import numpy as np
    from maple3dmt_gb300 import mesh
    from maple3dmt_gb300.solver import solver_for_survey
    from maple3dmt_gb300 import workloads
    sp = spec()
    plain_main = args.arm == "plain"
    p = solver_params(args, plain_main)
    if CONFIG == "c2":
        sv = mesh.layered_block_survey(min_level=sp.min_level, max_level=sp.max_level, n_side=sp.n_side,
                                       spacing=sp.spacing, freqs=np.asarray(sp.freqs))
        _, _, obs, err = survey_inputs(sv.stations)
        s = solver_for_survey(sv, device=local_rank, **p)
    else:
        # synthetic data: the forward response of the random model, 5 % noise
        sv = mesh.c5_survey()
        s = solver_for_survey(sv, device=local_rank, **p)
        s.set_sigma(sv.meta["sigma_true"])
        Z_true = s.forward_batch(sv.freqs)                          # [nf, ns, 4]
        obs, err = workloads.noisy_data(Z_true.transpose(1, 0, 2), seed=42)
        s.set_sigma(sv.sigma)
    dist = None
    if world > 1:
        import torch.distributed as dist
    r = run_steps(s, sv, obs, err, args.steps, args.warmup, rank, world, dist, ClockSampler(local_rank),
                  per_freq=plain_main, timing=bool(args.kernel_timing))
    t_dev, e2e_s = r["t_dev"], r["e2e_s"]
    solves = r["solves"]
    if dist:
        import torch
        tt = torch.tensor([t_dev, e2e_s, float(solves)], dtype=torch.float64)
        mx = tt[:2].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        tot = tt[2:].clone()
        dist.all_reduce(tot)
        t_dev, e2e_s, solves = float(mx[0]), float(mx[1]), int(tot[0])
    # the plain FP64 arm on the same system, measured in the same run
    plain = None
    if not plain_main and args.plain_steps > 0 and world == 1 and CONFIG == "c2":
        pp = solver_params(args, True)
        sp_ = solver_for_survey(sv, device=local_rank, **pp)
        rp = run_steps(sp_, sv, obs, err, args.plain_steps, 1, rank, world, None, per_freq=True)
        plain = {"value": rp["solves"] / rp["t_dev"], "unit": UNIT, "steps": args.plain_steps, "warmup": 1,
                 "ms_per_step": rp["t_dev"] * 1000.0 / args.plain_steps,
                 "rhs_at_tol": rp["stats"]["rhs_at_tol"], "rhs_reported": rp["stats"]["rhs_reported"],
                 "true_residual_max": rp["stats"]["true_residual_max"],
                 "krylov_iterations_per_step": statistics.mean(rp["iters"]), **solver_label(args, pp, sv.freqs)}
        sp_.close()
    learned = None
    if not plain_main and args.learned_steps > 0 and world == 1 and CONFIG == "c2":
        try:
            learned = run_learned(args, sv, obs, err, local_rank)
        except Exception as exc:  # the learned arm must not hide the headline number
            learned = {"error": f"{type(exc).__name__}: {exc}"}
    if rank != 0:
        return
    value = solves / t_dev
    e2e = solves / e2e_s
    kt = r["kt"]
    # roofline of the dominant kernel class, on its full-width (K = 16)
    # launches: the ones whose DRAM traffic the committed ncu capture measured
    dom = max(("spmv", "ssor", "vector"), key=lambda k: kt[k]["ms"])
    d = kt[dom]
    b16 = d["by_k"].get("K16") or {"launches": 0}
    src = b16 if b16["launches"] else d
    achieved = (src["bytes"] / src["launches"]) / (src["ms"] / src["launches"] * 1e-3) / 1e9 if src["launches"] else 0.0
    achieved_all = d["bytes"] / (d["ms"] * 1e-3) / 1e9 if d["ms"] else 0.0
    peak, peak_kind = measured_peak_hbm()
    traffic = ncu_traffic(dom)
    nf = len(sv.freqs)
    h2d = s.nc * 8 + obs.size * 16 + err.size * 8
    d2h = s.nc * 8 + nf * len(sv.stations) * 4 * 16
    try:
        cb = None
        if not args.no_cpu and world == 1 and CONFIG == "c2" and LEVELS == (0, 0):
            cb = cpu_measure(1, 0, args.cpu_procs, one_core=False)[0]
    except Exception as exc:  # the baseline must not hide the GPU number
        cb = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_dev * 1000.0 / args.steps, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "c128" if not p["precision"] else "c64+c128",
        "data": "synthetic",
        "config": bench_config(s.ne, s.nc),
        "solver": {**solver_label(args, p, sv.freqs), "colours": s.n_colours,
                   "parallelism": f"frequency groups x{world} (round-robin, one gradient SUM)"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "plain": plain,
        "batched_over_plain": value / plain["value"] if plain else None,
        "learned": learned,
        "roofline": {"bound": "hbm", "kernel": dom, "launches": "K=16" if src is b16 else "all",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "achieved_all_widths": achieved_all},
        "kernel_classes": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                               "GB/s": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1) if v["ms"] else None,
                               "frac_of_peak": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9 / peak, 3)
                               if v["ms"] else None,
                               "by_batch_width": {kk: {"ms": round(b["ms"], 1),
                                                       "GB/s": round(b["bytes"] / (b["ms"] * 1e-3) / 1e9, 1)
                                                       if b["ms"] and b["bytes"] else None}
                                                  for kk, b in v["by_k"].items()}}
                           for k, v in kt.items()},
        "krylov_iterations_per_step": statistics.mean(r["iters"]),
        "solver_stats_last_step": r["stats"],
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "cpu_baseline": cb,
    }
    print(json.dumps(line), flush=True)


def run_c3(args, rank, world, local_rank):
    """C3: one mesh per frequency (skin-depth refinement per frequency, so the
    meshes differ in size), the C2 earth with seeded log-normal noise, 121
    stations.  A step is, for every mesh, the forward solve of both
    polarisations and the per-station adjoint gradients of --c3-sources
    station sources (two adjoint solves each), all meshes through one
    m3d_group_station_gradients call that runs them concurrently on the
    device.  The work spans one CUDA stream per mesh, so the step is timed by
    the host clock between device synchronisations (the call returns after
    every mesh's results are on the host); host copies are inside."""
    import numpy as np
    from maple3dmt_gb300 import mesh, workloads
    from maple3dmt_gb300.solver import group_station_gradients, solvers_for_surveys
    if world > 1:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "unavailable": "c3 runs on one GPU"}), flush=True)
        return
    allf = np.asarray(workloads.C3.freqs)
    idx = np.unique(np.round(np.linspace(0, len(allf) - 1, max(1, min(args.c3_freqs, len(allf))))).astype(int))
    freqs = allf[idx]
    t0 = time.perf_counter()
    svs = mesh.c3_surveys(freqs)
    p = solver_params(args, False)
    reps = max(1, args.c3_replicas)
    solvers = solvers_for_surveys([sv for sv in svs for _ in range(reps)], device=local_rank, **p)
    setup_s = time.perf_counter() - t0
    rng = np.random.default_rng(42)
    wr, hfreqs = [], []
    for i, sv in enumerate(svs):
        w = workloads.station_sources(len(sv.stations), rng)[:args.c3_sources]
        wr += [np.ascontiguousarray(part) for part in np.array_split(w, reps)]
        hfreqs += [float(freqs[i])] * reps
    # the workload's solves: 2 forward per mesh, 2 adjoint per station source
    n_solves = sum(2 + 2 * min(args.c3_sources, len(sv.stations)) for sv in svs)
    clocks = ClockSampler(local_rank)

    def step():
        return group_station_gradients(solvers, hfreqs, wr, max_concurrent=args.c3_concurrent)

    for _ in range(args.warmup):
        step()
    clocks.start()
    launches0 = sum(s.stats()["kernel_launches"] for s in solvers)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        step()
        times.append(time.perf_counter() - t)
    clk = clocks.stop()
    sts = [s.stats() for s in solvers]
    launches = sum(st["kernel_launches"] for st in sts) - launches0
    tr = [t for st in sts for t in st["true_residual"][:st["n_rhs"]]]
    total = sum(times)
    # the sequential schedule of the same handles (one at a time) for comparison
    t = time.perf_counter()
    group_station_gradients(solvers, hfreqs, wr, max_concurrent=1)
    one_at_a_time = n_solves / (time.perf_counter() - t)
    ne = [s.ne for s in solvers]
    h2d = sum(w.size * 16 for w in wr)
    d2h = sum(s.ns * 4 * 16 + w.shape[0] * s.nc * 8 for w, s in zip(wr, solvers))
    line = {
        "metric": METRIC, "value": n_solves * args.steps / total, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total * 1000.0 / args.steps, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "c64+c128", "data": "synthetic",
        "config": {"workload": f"C3: one mesh per frequency ({len(freqs)} of 16 frequencies "
                               f"{freqs.min():g}-{freqs.max():g} Hz, {min(ne)}-{max(ne)} edges), C2 earth with "
                               f"log10 sigma + N(0, 0.3^2), 121 stations; per mesh 2 forward + "
                               f"{2 * args.c3_sources} station adjoint solves ({args.c3_sources} station sources) "
                               f"and their per-station gradients ({n_solves} solves per step)",
                   "tol": TOL, "edges_per_mesh": ne[::reps], "handles_per_mesh": reps,
                   "handles_at_once": args.c3_concurrent,
                   "timing": "host clock between device synchronisations (one stream per handle)",
                   "l2": "inputs larger than L2"},
        "solver": {**solver_label(args, p, freqs), "parallelism": "handles run concurrently, one host thread and "
                                                                   "CUDA stream per handle"},
        "e2e": {"value": n_solves * args.steps / total, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "one_handle_at_a_time": {"value": one_at_a_time, "unit": UNIT},
        "rhs_at_tol": sum(1 for t in tr if t <= TOL), "rhs_reported": len(tr),
        "setup_s": setup_s, "gpu_launches": launches, "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    for s in solvers:
        s.close()


def main():
    global CONFIG, LEVELS
    args = parse()
    CONFIG = args.config
    LEVELS = (args.min_level, args.max_level)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
    elif CONFIG == "c3":
        run_c3(args, rank, world, local_rank)
    else:
        run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
