#!/usr/bin/env python
"""Forward + adjoint solves per second on one GB300 (the headline metric).

Workload (the reference's "plain FP64 forward solve on GPU" configuration,
driven to the gradient as an inversion iteration does): a 0.5 ohm-m block in a
10/100/1000 ohm-m three-layer earth, octree min/max level 6/7 (1.69M edges),
121 stations on an 11x11 grid at 1 km, 8 frequencies log-spaced 0.01-100 Hz,
both polarisations.  One step = forward solves for all 16 (frequency,
polarisation) right-hand sides, weighted residual, 16 adjoint solves and the
J^T r sensitivity: 32 solves, each driven to ||b - A x|| / ||b|| <= 1e-7
checked in FP64 (InversionFV::compute_gradient_ of the reference for every
frequency).  Synthetic data: seeded 5 % noise on the 1-D 100 ohm-m halfspace
impedance; random-free model.

  value : solves/s, device-event time of the step with sigma resident
  e2e   : solves/s through the public C ABI with host buffers (set_sigma +
          gradient call, host<->device copies inside the timed region)

`--impl reference` times the reference's CPU algorithm (the C restatement in
oracle/, the only CPU path available on the GPU machine) on the same system.
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--forward", default="reference", choices=["interleaved", "reference"])
    ap.add_argument("--min-level", type=int, default=6)
    ap.add_argument("--max-level", type=int, default=7)
    ap.add_argument("--nfreq", type=int, default=8)
    # profiling runs only (a capped solve is not a bench number): Krylov
    # iteration cap per solve, and skipping the CPU baseline
    ap.add_argument("--maxiter", type=int, default=5000)
    ap.add_argument("--plain", action="store_true",
                    help="the plain GPU arm the batched solve is compared with: one frequency per call, complex128 "
                         "Krylov, CSR row kernels, Jacobi divergence correction, the reference's forward strategy")
    ap.add_argument("--ssor-form", type=int, default=1, choices=[0, 1],
                    help="inner FP32 solve: 0 right-preconditioned SSOR-BiCGStab, 1 Eisenstat split form")
    ap.add_argument("--divcorr-precond", type=int, default=1, choices=[0, 1],
                    help="divergence-correction PCG: 0 Jacobi (the reference's), 1 aggregation multigrid")
    ap.add_argument("--row-kernels", type=int, default=1, choices=[0, 1],
                    help="0: CSR rows read by the lanes; 1: slice-staged rows (bulk copies to shared memory)")
    ap.add_argument("--gradcorr", type=int, default=1, choices=[0, 1],
                    help="1: gradient-space term (multigrid V-cycle on the divergence-correction Laplacian) in "
                         "the FP32 inner solve's preconditioner for frequencies <= --gradcorr-fmax")
    ap.add_argument("--gradcorr-fmax", type=float, default=1e30)
    ap.add_argument("--gradcorr-presmooth", type=int, default=0, choices=[0, 1],
                    help="V-cycle of the gradient-space term: 1 V(1,1), 0 V(0,1)")
    ap.add_argument("--divcorr-mixed", type=int, default=1, choices=[0, 1],
                    help="1: divergence-correction Poisson solve as FP32 PCG inside FP64 refinement")
    ap.add_argument("--inner-tol-floor", type=float, default=3e-5,
                    help="smallest relative residual asked of one complex-FP32 inner solve")
    ap.add_argument("--residual-replacement", type=int, default=0, choices=[0, 1],
                    help="1: inner FP32 solve to the final tolerance with FP64 residual replacement")
    ap.add_argument("--gradcorr-overlap", type=int, default=1, choices=[0, 1],
                    help="1: V-cycles of the gradient-space term on a second stream, overlapping the SSOR sweep")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def workload(args):
    import numpy as np
    from maple3dmt_gb300 import mesh
    freqs = np.logspace(-2, 2, 8) if args.nfreq == 8 else np.logspace(-2, 2, args.nfreq)
    sv = mesh.layered_block_survey(min_level=args.min_level, max_level=args.max_level, freqs=freqs)
    ns, nf = len(sv.stations), len(sv.freqs)
    rng = np.random.default_rng(42)
    om = 2 * math.pi * sv.freqs
    z1 = np.sqrt(1j * om * mesh.MU0 / 0.01)                        # 100 ohm-m halfspace
    obs = np.zeros((ns, nf, 4), np.complex128)
    obs[:, :, 1] = z1[None, :]
    obs[:, :, 2] = -z1[None, :]
    err = np.zeros((ns, nf, 4))
    err[:, :, 1:3] = 0.05 * np.abs(z1)[None, :, None]
    noise = rng.normal(size=(ns, nf, 4)) + 1j * rng.normal(size=(ns, nf, 4))
    obs = obs + 0.05 * np.abs(obs) * noise / math.sqrt(2)
    return sv, obs, err


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


# ---------------------------------------------------------------------------
# CPU baseline: the reference algorithm (oracle restatement) per iteration
# ---------------------------------------------------------------------------

def _cpu_worker(args_tuple):
    min_level, max_level, nfreq, freq, n_iter, q = args_tuple
    import numpy as np  # noqa: F401
    import oracle
    from maple3dmt_gb300 import mesh
    fr = np.logspace(-2, 2, nfreq)
    sv = mesh.layered_block_survey(min_level=min_level, max_level=max_level, freqs=fr)
    o = oracle.Oracle(oracle.Case.from_survey(sv))
    q.put(("ready", os.getpid()))
    t_it, t_setup = o.time_iterations(freq, n_iter)
    q.put(("done", t_it / n_iter, t_setup))


# Iterations per solve of the reference SSOR-BiCGStab on this workload, used
# to turn the CPU per-iteration time into solves/s: forward (reference
# strategy, maxiter 5000, the two 0.01 Hz solves did not converge) and
# adjoint (interleaved divergence correction), per (frequency, polarisation),
# from the FP64 GPU solve of the same systems.
REF_ITERS_FWD = [5000, 5000, 3114, 4073, 1244, 1213, 458, 519, 193, 179, 72, 73, 9, 10, 3, 3]
REF_ITERS_ADJ = [530, 524, 537, 559, 501, 534, 319, 299, 146, 142, 51, 57, 22, 21, 10, 12]


def cpu_reference(args, n_iter=3, procs=None):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    procs = procs or max(1, min(16, os.cpu_count() or 1))
    q = ctx.Queue()
    import numpy as np
    fr = np.logspace(-2, 2, args.nfreq)
    workers = [ctx.Process(target=_cpu_worker, args=((args.min_level, args.max_level, args.nfreq,
                                                      float(fr[i % len(fr)]), n_iter, q),)) for i in range(procs)]
    t0 = time.time()
    for w in workers:
        w.start()
    res = []
    while len(res) < procs:
        m = q.get()
        if m[0] == "done":
            res.append(m)
    for w in workers:
        w.join()
    wall = time.time() - t0
    t_iter = statistics.mean(r[1] for r in res)
    iters = REF_ITERS_FWD + REF_ITERS_ADJ
    solve_s = t_iter * statistics.mean(iters)
    value = procs / solve_s
    return {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
            "sample": (f"{procs} concurrent processes (frequency-parallel like the reference's MPI groups), "
                       f"each {n_iter} reference SSOR-BiCGStab iterations on the assembled C2 system; "
                       f"{t_iter:.3f} s/iteration x mean {statistics.mean(iters):.0f} iterations/solve "
                       f"(reference-strategy iteration counts of the same 32 solves)"),
            "seconds_per_iteration": t_iter, "wall_s": wall}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    W, K = args.warmup, args.steps
    cb = None
    vals = []
    for i in range(max(1, min(K, 1))):
        cb = cpu_reference(args)
        vals.append(cb["value"])
    v = statistics.mean(vals)
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": K, "warmup": W, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic",
            "config": {"workload": f"layered+block earth, octree levels {args.min_level}/{args.max_level}, "
                                   f"121 stations, {args.nfreq} freqs 0.01-100 Hz, fwd+adjoint gradient step",
                       "l2": "inputs larger than L2"},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def run_ours(args, rank, world, local_rank):
    import numpy as np
    from maple3dmt_gb300.solver import solver_for_survey
    sv, obs, err = workload(args)
    if args.plain:
        args.precision, args.forward, args.row_kernels, args.divcorr_precond = "fp64", "reference", 0, 0
        args.ssor_form, args.gradcorr, args.divcorr_mixed = 0, 0, 0
    s = solver_for_survey(sv, device=local_rank, bicgstab_tol=1e-7, bicgstab_maxiter=args.maxiter,
                          precision=1 if args.precision == "mixed" else 0,
                          forward_interleaved=1 if args.forward == "interleaved" else 0,
                          row_kernels=args.row_kernels, divcorr_precond=args.divcorr_precond,
                          ssor_form=args.ssor_form, gradcorr=args.gradcorr, gradcorr_fmax=args.gradcorr_fmax,
                          gradcorr_presmooth=args.gradcorr_presmooth, divcorr_mixed=args.divcorr_mixed,
                          inner_tol_floor=args.inner_tol_floor, residual_replacement=args.residual_replacement,
                          gradcorr_overlap=args.gradcorr_overlap)
    nf = len(sv.freqs)
    solves_per_step = 4 * nf
    dist = None
    if world > 1:
        import torch.distributed as dist

    def barrier():
        if dist:
            dist.barrier()

    def step():
        if not args.plain:
            return s.gradient_batch(sv.freqs, obs, err)
        # one frequency per call (K = 2 forward, 2 adjoint), gradients summed
        Zs, g = [], None
        for fi in range(nf):
            Zf, gf = s.gradient_batch(sv.freqs[fi:fi + 1], obs[:, fi:fi + 1], err[:, fi:fi + 1])
            Zs.append(Zf)
            g = gf if g is None else g + gf
        return np.concatenate(Zs), g

    for _ in range(args.warmup):
        step()
    barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    s.set_kernel_timing(True)
    launches0 = s.stats()["kernel_launches"]
    dev_ms, e2e_s = 0.0, 0.0
    iters, tres, status = [], [], []
    grad = None
    for _ in range(args.steps):
        barrier()
        t0 = time.perf_counter()
        s.set_sigma(sv.sigma)                  # host -> device conductivity
        s.timer_start()
        Z, grad = step()
        dev_ms += s.timer_stop()
        e2e_s += time.perf_counter() - t0
        st = s.stats()
        iters.append(st["total_iterations"])
        solver_stats = {k: st[k] for k in ("forward_iterations", "adjoint_iterations", "refinements",
                                           "divcorr_calls", "divcorr_outer", "divcorr_cg_iterations",
                                           "divcorr_cg_sweeps", "divcorr_setup_ms", "replacements")}
        solver_stats["iterations_per_rhs"] = st["iterations"]
        tr = st["true_residual"][:st["n_rhs"]]
        solver_stats["rhs_at_tol"] = sum(1 for t in tr if t <= 1e-7)
        solver_stats["rhs_reported"] = len(tr)
        solver_stats["true_residual_max"] = max(tr) if tr else None
    launches = s.stats()["kernel_launches"] - launches0
    kt = s.kernel_times()
    s.set_kernel_timing(False)
    clk = clocks.stop()
    t_dev = dev_ms / 1000.0
    if dist:
        import torch
        tt = torch.tensor([t_dev, e2e_s], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_dev, e2e_s = float(tt[0]), float(tt[1])
        g = torch.from_numpy(grad)
        dist.all_reduce(g)                     # frequency-group gradient sum (freq_parallel.cpp:129)
    if rank != 0:
        return
    total_solves = solves_per_step * args.steps * world
    value = total_solves / t_dev
    e2e = total_solves / e2e_s
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
    h2d = s.nc * 8 + obs.size * 16 + err.size * 8
    d2h = s.nc * 8 + nf * len(sv.stations) * 4 * 16
    try:
        cb = None if args.no_cpu else cpu_reference(args)
    except Exception as exc:  # the baseline must not hide the GPU number
        cb = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_dev * 1000.0 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128" if args.precision == "fp64" else "c64+c128",
        "data": "synthetic",
        "config": {"workload": f"layered+block earth, octree levels {args.min_level}/{args.max_level} "
                               f"({s.ne} edges, {s.nc} cells), 121 stations, {nf} freqs 0.01-100 Hz, "
                               f"forward+adjoint+sensitivity gradient step ({solves_per_step} solves)",
                   "tol": 1e-7, "precision": args.precision, "inner_tol_floor": args.inner_tol_floor,
                   "residual_replacement": bool(args.residual_replacement),
                   "forward": args.forward,
                   "colours": s.n_colours, "row_kernels": ["csr", "staged"][args.row_kernels],
                   "divcorr_precond": ["jacobi", "multigrid"][args.divcorr_precond],
                   "divcorr_solve": ["fp64 pcg", "fp32 pcg in fp64 refinement"][args.divcorr_mixed],
                   "ssor_form": ["right-preconditioned", "eisenstat"][args.ssor_form],
                   "gradcorr": (f"multigrid gradient-space term, V({args.gradcorr_presmooth},1), "
                                f"f <= {args.gradcorr_fmax:g} Hz"
                                + (", V-cycle on a second stream" if args.gradcorr_overlap else "")
                                if args.gradcorr else "off"),
                   "arm": "plain (per frequency, complex128)" if args.plain else "batched",
                   "l2": "inputs larger than L2 (matrix alone 260 MB)",
                   "parallelism": f"replica x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": dom, "launches": "K=16" if src is b16 else "all",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "achieved_all_widths": achieved_all},
        "kernel_classes": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                               "GB/s": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1) if v["ms"] else None,
                               "by_batch_width": {kk: {"ms": round(b["ms"], 1),
                                                       "GB/s": round(b["bytes"] / (b["ms"] * 1e-3) / 1e9, 1)
                                                       if b["ms"] and b["bytes"] else None}
                                                  for kk, b in v["by_k"].items()}}
                           for k, v in kt.items()},
        "krylov_iterations_per_step": statistics.mean(iters),
        "solver_stats_last_step": solver_stats,
        "gpu_launches": launches,
        "clocks": clk,
        "cpu_baseline": cb,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
