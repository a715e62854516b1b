"""Benchmark: converged eigenpairs per second on one GB300.

Workload (one "step"): the full BiGlobal pass of the C2 configuration --
Ny = 200 (FD-q q=10) x Nz = 128 (periodic q=6) wavy-wall boundary layer,
bump 0.08, Re 1000, Mach 0.5, alpha 1.8, nev 16, search centre
omega = 0.3 + 0.01i (lambda target 0.01 - 0.3i), tol 1e-10: metrics,
base-flow derivatives, assembly of M_Gamma and L, wall/far-field rows,
factorisation of A - sigma B and shift-and-invert Krylov-Schur, with every
reported eigenpair checked at relative residual <= 1e-10.  Only eigenpairs
passing that check count.

value: device-resident (grid and base flow already in HBM), CUDA events on
the context's stream around the step.  e2e: the same step through the
public API from pinned host buffers (host->device copy of the inputs and
device->host read of eigenvalues and residuals inside the timed region).
Inputs and factors are far larger than L2 (the operator alone is 788 MB),
so no flush is needed.

--impl reference times the reference algorithm's CPU path (the CPU oracle:
C restatement of the assembly, LAPACK zggev boundary rows, SuperLU +
ARPACK shift-invert) on the host cores, on a bounded sample of the same
workload family (a 60 x 32 grid, same physics, nev and target).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "eigenpairs/s at resid<=1e-10"
UNIT = "eigenpairs/s"
C2 = dict(ny=200, nz=128, amplitude=0.08, alpha=1.8, omega=complex(0.3, 0.01), nev=16)
# Krylov-Schur basis size for both forms (the reference leaves it to SLEPc's
# runtime -eps_ncv; 4 nev needs 3 restarts here instead of 13 at 2 nev)
NCV = 64


def c2_case(ny=None, nz=None):
    from tailor_gb300.case import Physics, make_case
    ph = Physics(alpha=C2["alpha"], omega=C2["omega"], nev=C2["nev"], tol=1e-10)
    return make_case(ny or C2["ny"], nz or C2["nz"], amplitude=C2["amplitude"], physics=ph)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            q = ("--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "-i", "0", q, "--format=csv,noheader,nounits"],
                                         capture_output=True, text=True, timeout=5).stdout.strip()
                    if out:
                        self.samples.append([v.strip() for v in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if len(s) > 3 + k and s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


# ------------------------------------------------------------- CUDA events
class Events:
    def __init__(self):
        self.rt = ctypes.CDLL("libcudart.so")
        self.a, self.b = ctypes.c_void_p(), ctypes.c_void_p()
        self.rt.cudaEventCreate(ctypes.byref(self.a))
        self.rt.cudaEventCreate(ctypes.byref(self.b))

    def record(self, ev, stream):
        self.rt.cudaEventRecord(ev, ctypes.c_void_p(stream))

    def elapsed_ms(self):
        self.rt.cudaEventSynchronize(self.b)
        ms = ctypes.c_float()
        self.rt.cudaEventElapsedTime(ctypes.byref(ms), self.a, self.b)
        return ms.value

    def pinned(self, nbytes):
        p = ctypes.c_void_p()
        if self.rt.cudaHostAlloc(ctypes.byref(p), ctypes.c_size_t(nbytes), 0) != 0:
            raise RuntimeError("cudaHostAlloc failed")
        return p


def one_pass(prob, api, precision):
    api.Metrics(prob).compute()
    api.BaseFlowDerivatives(prob).compute()
    op = api.GlobalOperator(prob).assemble()
    api.BoundaryConditions(prob).apply()
    sol = api.EigenSolver(prob).solve(precision=precision, ncv=NCV)
    good = int(np.sum(sol.residual <= 1e-10))
    return good, sol, op


# batched alpha-sweep: 64 instances, grids (60,32), (100,50), (150,64) drawn
# 2:1:1, alpha uniform on [0.5, 4], Re 1000, Mach 0.5, nev 8, tol 1e-10
C3_GRIDS = [(60, 32), (100, 50), (150, 64)]


def c3_sweep_inputs(npoints=64, seed=2026):
    from tailor_gb300.case import Physics, make_case
    ph = Physics(alpha=1.0, omega=0j, nev=8, tol=1e-10)
    cases = [make_case(ny, nz, amplitude=0.05, physics=ph) for ny, nz in C3_GRIDS]
    rng = np.random.default_rng(seed)
    cls = rng.choice([0, 0, 1, 2], size=npoints)
    alphas = rng.uniform(0.5, 4.0, size=npoints)
    return cases, [(int(c), float(a)) for c, a in zip(cls, alphas)]


def run_c3(api, npoints=64):
    """The sweep in the plain FP64 form (one instance at a time, CUDA-core
    FP64 fronts) and in the mixed + batched form (complex64 fronts with
    tensor-core Schur updates and FP64 refinement, eight concurrent instances,
    autotuned kernels): eigenpairs at resid <= 1e-10 per wall second.  With
    several ranks the points are dealt round-robin to the GPUs (replicas) and
    the wall time is the slowest rank's."""
    from tailor_gb300 import replicas
    cases, points = c3_sweep_inputs(npoints)
    out = {}
    for name, kw in (("plain_fp64", dict(precision=0, workers=1, autotune=False)),
                     ("mixed_batched", dict(precision=1, workers=8, autotune=True))):
        replicas.barrier()
        t = time.perf_counter()
        r = replicas.sweep(cases, points, nev=8, ncv=32, raise_on_error=False, **kw)
        wall, _ = replicas.reduce_timing(time.perf_counter() - t, 0)
        good = int(np.sum((r["residual"] >= 0) & (r["residual"] <= 1e-10)))
        d0 = next(d for d in r["rank_diag"] if d)
        out[name] = {"value": good / wall, "unit": UNIT, "wall_s": wall, "eigenpairs": good,
                     "failed_points": int(np.sum(r["status"] != 0)),
                     "workers": d0["workers"], "ranks": r["world"],
                     "solve_block": d0["solve_block"],
                     "tensor_core_schur": [1 - c for c in d0["cuda_core_schur"]]}
    out["points"] = npoints
    out["grids"] = C3_GRIDS
    return out


def cpu_reference_sample(steps=1, threads=None):
    """The CPU path on a bounded sample (60 x 32 grid, C2 physics)."""
    from oracle.oracle import Oracle, boundary_rows, eigen_oracle, to_complex_blocks
    case = c2_case(60, 32)
    o = Oracle()
    sigma = complex(C2["omega"].imag, -C2["omega"].real)
    times, good = [], 0
    for _ in range(steps):
        t = time.perf_counter()
        r = o.full(case)
        A, B, _ = boundary_rows(case, r["metrics"], r["row_ptr"], r["col"],
                                to_complex_blocks(r["mass"]), to_complex_blocks(r["spatial"]))
        lam, _, res = eigen_oracle(r["row_ptr"], r["col"], A, B, case.nodes, sigma,
                                   C2["nev"], tol=1e-12)
        times.append(time.perf_counter() - t)
        good = int(np.sum(res <= 1e-10))
    return good, times, case


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    good, times, case = cpu_reference_sample(steps=max(args.warmup, 0) and 1)
    good, times, case = cpu_reference_sample(steps=args.steps)
    sec = float(np.mean(times))
    value = good / sec
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": "C2 family, bounded CPU sample 60x32 (nev 16, target 0.01-0.3i)",
                   "ny": case.ny, "nz": case.nz},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "one 60x32 eigen solve per step: C oracle assembly, "
                                   "zggev boundary rows, SuperLU+ARPACK"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", type=int, default=1, help="1 mixed (default), 0 FP64")
    ap.add_argument("--plain", action="store_true", help="also time the plain FP64 form")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sweep", action="store_true", help="skip the 64-instance sweep")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # replicas only: barrier + max over ranks
        dist.init_process_group("gloo")

    from tailor_gb300 import api
    from tailor_gb300 import build as tb
    tb.build()
    case = c2_case()
    ev = Events()
    prob = api.Problem(case, device=local)
    stream = prob.lib.tlr_stream(prob.ctx)
    for _ in range(args.warmup):
        one_pass(prob, api, args.precision)

    def barrier():
        if dist:
            dist.barrier()

    # device-resident timing
    clocks = ClockSampler()
    clocks.start()
    barrier()
    launches0 = prob.lib.tlr_kernel_launches()
    ev.record(ev.a, stream)
    good_total, sols = 0, []
    for _ in range(args.steps):
        good, sol, op = one_pass(prob, api, args.precision)
        good_total += good
        sols.append(sol)
    ev.record(ev.b, stream)
    ms = ev.elapsed_ms()
    launches = prob.lib.tlr_kernel_launches() - launches0
    barrier()
    clk = clocks.stop()
    from tailor_gb300 import replicas
    ms, good_total = replicas.reduce_timing(ms, good_total)  # slowest rank, all pairs
    value = good_total / (ms / 1e3)

    # end to end through the public API with pinned host buffers
    gbytes, bbytes = case.grid.nbytes, case.baseflow.nbytes
    pg, pb = ev.pinned(gbytes), ev.pinned(bbytes)
    ctypes.memmove(pg, case.grid.ctypes.data, gbytes)
    ctypes.memmove(pb, case.baseflow.ctypes.data, bbytes)
    barrier()
    ev.record(ev.a, stream)
    good_e2e = 0
    for _ in range(args.steps):
        prob.check(prob.lib.tlr_load_fields(prob.ctx, pg, pb))
        good, sol, _ = one_pass(prob, api, args.precision)
        good_e2e += good
    ev.record(ev.b, stream)
    ms_e2e = ev.elapsed_ms()
    barrier()
    ms_e2e, good_e2e = replicas.reduce_timing(ms_e2e, good_e2e)
    e2e = good_e2e / (ms_e2e / 1e3)
    d2h = C2["nev"] * (16 + 8)

    last = sols[-1].diag
    plain = None
    if args.plain and rank == 0:
        t = time.perf_counter()
        good, sol, _ = one_pass(prob, api, 0)
        plain = {"value": good / (time.perf_counter() - t), "factor_ms": sol.diag["factor_ms"],
                 "krylov_ms": sol.diag["krylov_ms"], "eigenpairs": good}

    sweep = None
    if not args.no_sweep:  # every rank takes its share of the points
        sweep = run_c3(api)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        g, times, c = cpu_reference_sample(steps=1)
        cpu = {"value": g / times[0], "unit": UNIT, "cores": os.cpu_count() or 1,
               "kind": "port",
               "sample": "one 60x32 eigen solve (C2 physics, nev 16): C oracle assembly, "
                         "zggev boundary rows, SuperLU+ARPACK, %.1f s" % times[0]}
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    # dominant kernel: the triangular solves (one CUDA graph per K^-1
    # application), timed live with CUDA events around every graph replay.
    csize = 8 if args.precision == 1 else 16
    tri_bytes = last["factor_bytes"] + 2 * 5 * case.nodes * csize
    tri_avg_ms = last["trisolve_ms"] / max(last["trisolves"], 1)
    achieved = tri_bytes / (tri_avg_ms * 1e-3) / 1e9 if tri_avg_ms > 0 else 0.0
    traffic = None
    tf = ROOT / "profiles" / "trisolve_traffic.json"
    if tf.exists():
        t = json.loads(tf.read_text()).get("c64" if args.precision == 1 else "c128", {})
        traffic = t.get("bytes_per_solve_c2")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 factor + c128 refinement" if args.precision == 1 else "c128",
        "data": "synthetic",
        "config": {"workload": "C2: 200x128 wavy-wall BL, nev 16, target 0.01-0.3i, alpha 1.8",
                   "ny": case.ny, "nz": case.nz, "nev": C2["nev"],
                   "form": "mixed" if args.precision == 1 else "plain-fp64", "ncv": NCV,
                   "l2": "inputs and factors larger than L2 (no flush)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": gbytes + bbytes,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "kernel": "triangular solves (solve graph: k_blk_update, k_border_gemv, "
                               "k_bwd_start, gathers)",
                     "algorithmic_bytes": tri_bytes, "avg_ms": tri_avg_ms,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
        "factor": {"flops": last["factor_flops"], "ms": last["factor_ms"],
                   "tflops": last["factor_flops"] / (last["factor_ms"] * 1e-3) / 1e12
                   if last["factor_ms"] > 0 else 0.0},
        "solve": {k: last[k] for k in ("iterations", "solves", "refinement_steps", "factor_ms",
                                       "krylov_ms", "total_ms", "max_relative_error",
                                       "trisolve_ms", "trisolves", "ortho_ms", "dense_ms",
                                       "residual_ms")},
        "cpu_baseline": cpu,
        "plain_fp64": plain,
        "sweep_c3": sweep,
    }
    if rank == 0:
        print(json.dumps(line))
    prob.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
