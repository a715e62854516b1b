"""Benchmark: converged eigenpairs per second on one GB300.

Headline workload: the neutral-curve sweep at the largest grid -- Ny = 300
(FD-q q=10) x Nz = 192 (periodic q=6), 288 000 complex unknowns per point,
wavy-wall boundary layer (bump 0.05), Mach 0.7, nev 8 nearest lambda = 0,
tol 1e-10, points on the 8 x 4 grid of alpha in [0.5, 3.5] and Re in
[800, 2400], visited in snake order (alpha up on one Re row, down on the
next) so that consecutive points are neighbours.  One "step" is one point:
metrics, base-flow derivatives, assembly of M_Gamma and L at the point's
(alpha, Re), wall and far-field rows, factorisation of A - sigma B and the
shift-and-invert Krylov-Schur solve.  The default 32 steps are the whole
sweep.

The combined form (the line's value) is
  * mixed: complex64 multifrontal factor with tensor-core Schur updates,
    every K^-1 application refined in FP64 against the FP64 operator;
  * batched: the sweep runs as --chains (default 4) concurrent chains on
    the one GPU, each a persistent context (one symbolic analysis, one set
    of factor buffers, captured solve and refinement graphs) with its own
    stream and host thread, walking its own stretch of the snake;
  * learned: in every timed pass the first point of every chain starts
    from the learned proposal (an MLP trained, before the timed region, on
    eigenpairs the solver computed at 60 x 32 over the sweep's parameter
    range, its start vector carried to 300 x 192 by the spline operators);
    every later point starts from its predecessor's Ritz vectors (their
    sum: the wanted modes of the neighbouring point).
The plain FP64 form (complex128 factor, single-vector Krylov-Schur from a
pseudo-random start, the reference's EigenSolver) solves a stated subset of
the same points in the same run.

An eigenpair counts only if its relative residual ||Ax - lambda Bx|| /
(|lambda| ||x||) <= 1e-10 and |dlambda| / |lambda| <= 1e-8 against the FP64
reference eigenvalues of its point (tests/golden/c5_300x192_plain_eigs.txt,
the plain FP64 form's, which is pinned to the CPU oracle at 100 x 50 and
200 x 128).

value: device-resident (grid and base flow in HBM), CUDA events around the
K timed steps: the start event on chain 0's stream, which the other chains'
streams wait on, the end event after every chain's stream has joined it.  e2e: the next K points through
the public API from pinned host buffers (host->device copy of the grid and
base flow and device->host read of eigenvalues and residuals inside the
timed region).  The operator (1.8 GB) and the factor (10 GB) are far larger
than L2, so no flush is needed.

Sub-records: c2 (200 x 128, nev 16, target 0.01 - 0.3i, alpha 1.8; mixed
vs plain FP64, every eigenvalue against the CPU oracle's) and sweep_c3 (64
instances on three grid classes, mixed + batched vs plain FP64).

--impl reference: the reference algorithm's CPU path (the CPU oracle: C
restatement of the assembly, LAPACK zggev boundary rows, SuperLU + ARPACK)
cannot solve one 300 x 192 point within the step budget; it prints the
reason and a measured CPU figure on a smaller grid, and no value.
"""
from __future__ import annotations

import argparse
import ctypes
import dataclasses
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

METRIC = "eigenpairs/s at resid<=1e-10 and |dlambda|/|lambda|<=1e-8"
UNIT = "eigenpairs/s"
RESID_TOL = 1e-10
DLAM_TOL = 1e-8
# combined form on the neutral-curve sweep (block Krylov-Schur, --block,
# needs more operator applications than it saves on this clustered
# spectrum, so the default is the single-vector method)
C5_NEV = 8
C5_BLOCK = 1
C5_NCV = 64
# concurrent chains of sweep points on the one GPU (one context and one host
# thread each; each chain walks its own stretch of the snake)
C5_CHAINS = 4
PLAIN_NCV = 32
# C2: mixed vs plain FP64 at 200 x 128
C2 = dict(ny=200, nz=128, amplitude=0.08, alpha=1.8, omega=complex(0.3, 0.01), nev=16)
C2_NCV = 64
GOLDEN = ROOT / "tests" / "golden"
TRISOLVE_TRAFFIC_RATIO = 538.1 / 518.3


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


# ------------------------------------------------------- parity bookkeeping
def load_c5_reference():
    """{(alpha, Re): FP64 eigenvalues} of the sweep's points, or None."""
    f = GOLDEN / "c5_300x192_plain_eigs.txt"
    if not f.exists():
        return None
    ref = {}
    for row in np.loadtxt(f, ndmin=2):
        lam = row[2::3] + 1j * row[3::3]
        ref[(round(row[0], 9), round(row[1], 6))] = lam
    return ref


def count_pairs(lam, res, ref_lam):
    """(pairs passing both bars, largest |dlambda|/|lambda| against ref).
    Without reference eigenvalues only the residual bar is applied and the
    deviation is None."""
    if ref_lam is None or len(ref_lam) == 0:
        return int(np.sum(np.asarray(res) <= RESID_TOL)), None
    good, worst = 0, 0.0
    for l, r in zip(lam, res):
        d = float(np.min(np.abs(ref_lam - l)) / abs(l))
        worst = max(worst, d)
        if r <= RESID_TOL and d <= DLAM_TOL:
            good += 1
    return good, worst


# ------------------------------------------------------------ learned start
def train_proposal(api, learned, points, grid=(60, 32)):
    """The learned start proposal for the sweep: solver eigenpairs at a
    coarse grid over the sweep's parameter box (alpha in [0.5, 3.5], Re
    log-uniform in [800, 2400], Mach 0.7), an MLP fitted on the GPU by the
    library's kernels.  Returns (proposal, seconds)."""
    from tailor_gb300.neutral_sweep import c5_case
    t = time.perf_counter()
    rng = np.random.default_rng(7)
    train = [(float(rng.uniform(0.5, 3.5)), float(10 ** rng.uniform(np.log10(800), np.log10(2400))),
              0.7) for _ in range(48)]
    case = c5_case(*grid, nev=C5_NEV)
    with api.Problem(case) as prob:
        samples = learned.generate(prob, train, nev=C5_NEV, precision=1)
    prop = learned.Proposal.fit(samples, 0j, epochs=2000, batch=48, lr=1e-3)
    prop.grid = grid
    return prop, time.perf_counter() - t


# ------------------------------------------------------------- C5 headline
def c5_ncv(block):
    return C5_NCV if block == 1 else max(C5_NCV, 6 * block)


def c5_step(api, prob, point, first, proposal, block=C5_BLOCK):
    """One sweep point in the combined form; returns (lam, residual, diag)."""
    _, alpha, re = point
    prob.set_physics(dataclasses.replace(prob.case.physics, alpha=alpha, reynolds=re))
    api.run_pipeline(prob)
    kw = dict(nev=C5_NEV, ncv=c5_ncv(block), precision=1, block=block)
    if first:
        start = proposal.start_on(prob.case, (alpha, re, prob.case.physics.mach)) \
            if proposal is not None else None
        sol = api.EigenSolver(prob).solve(start=start, **kw)
    else:
        sol = api.EigenSolver(prob).solve(warm_start=True, **kw)
    return sol.lam, sol.residual, sol.diag


def plain_step(api, prob, point):
    _, alpha, re = point
    prob.set_physics(dataclasses.replace(prob.case.physics, alpha=alpha, reynolds=re))
    api.run_pipeline(prob)
    sol = api.EigenSolver(prob).solve(nev=C5_NEV, ncv=PLAIN_NCV, precision=0)
    return sol.lam, sol.residual, sol.diag


class Chains:
    """W concurrent chains of sweep points on one GPU: chain w owns one
    Problem (its own context and CUDA stream) and one host thread (the
    library releases the GIL in every call), and warm-starts each point from
    its own previous point."""

    def __init__(self, api, case_fn, width, device, proposal, block):
        self.api, self.proposal, self.block = api, proposal, block
        self.probs = [api.Problem(case_fn(), device=device) for _ in range(width)]
        self.streams = [p.lib.tlr_stream(p.ctx) for p in self.probs]
        self.first = [True] * width

    def run(self, seqs, before=None):
        """seqs[w]: the points of chain w, in order.  before(w, prob) runs
        ahead of each point (e.g. a host->device field load).  Returns, per
        chain, [(point, lam, res, diag)]."""
        out = [[] for _ in self.probs]
        errors = []

        def work(w):
            try:
                for pt in seqs[w]:
                    if before is not None:
                        before(w, self.probs[w])
                    lam, res, diag = c5_step(self.api, self.probs[w], pt, self.first[w],
                                             self.proposal, self.block)
                    self.first[w] = False
                    out[w].append((pt, lam, res, diag))
            except BaseException as e:  # re-raised on the calling thread
                errors.append(e)

        if len(self.probs) == 1:
            work(0)
        else:
            threads = [threading.Thread(target=work, args=(w,)) for w in range(len(self.probs))]
            for t in threads:
                t.start()
            for t in threads:
                t.join()
        if errors:
            raise errors[0]
        return out

    def restart(self):
        """The next point of every chain starts from the learned proposal
        (a random start without one) instead of its predecessor's vectors."""
        self.first = [True] * len(self.probs)

    def timed(self, ev, fn):
        """fn() between CUDA events: the start event on chain 0's stream,
        which every other chain's stream waits on; every other stream's end
        is joined into chain 0's stream before the end event."""
        rt = ev.rt
        ev.record(ev.a, self.streams[0])
        for st in self.streams[1:]:
            rt.cudaStreamWaitEvent(ctypes.c_void_p(st), ev.a, 0)
        out = fn()
        for st in self.streams[1:]:
            e = ctypes.c_void_p()
            rt.cudaEventCreateWithFlags(ctypes.byref(e), 2)  # cudaEventDisableTiming
            rt.cudaEventRecord(e, ctypes.c_void_p(st))
            rt.cudaStreamWaitEvent(ctypes.c_void_p(self.streams[0]), e, 0)
            rt.cudaEventDestroy(e)
        ev.record(ev.b, self.streams[0])
        return out, ev.elapsed_ms()

    def close(self):
        for p in self.probs:
            p.close()


def split_steps(total, width):
    """total points over width chains, the first chains taking the remainder."""
    return [total // width + (1 if w < total % width else 0) for w in range(width)]


def chain_sequences(npoints, steps, width, warmup, offset=0):
    """Point indices each chain visits, in order: warmup points, its timed
    stretch [T_w, T_w + n_w) (T_w = warmup + n_0 + ... + n_(w-1)), the next
    chain's stretch (the end-to-end pass) and one more point.  Returns
    (sequences, timed counts n_w, end-to-end counts).  With steps equal to
    npoints both passes cover every point once."""
    nstep = split_steps(steps, width)
    nnext = [nstep[(w + 1) % width] for w in range(width)]
    starts = [warmup + sum(nstep[:w]) for w in range(width)]
    seqs = [[(offset + starts[w] - warmup + i) % npoints
             for i in range(warmup + nstep[w] + nnext[w] + 1)] for w in range(width)]
    return seqs, nstep, nnext


def run_c2(api, ref_file=GOLDEN / "c2_200x128_eigs.txt"):
    """C2: mixed (single-vector, the bench's earlier headline form) vs plain
    FP64, one pass each after a warm-up, eigenvalues against the oracle."""
    ref = None
    if ref_file.exists():
        r = np.loadtxt(ref_file, ndmin=2)
        ref = r[:, 0] + 1j * r[:, 1]
    case = c2_case()
    out = {"workload": "C2: 200x128, nev 16, target 0.01-0.3i, alpha 1.8", "oracle": ref is not None}
    with api.Problem(case) as prob:
        for name, kw in (("mixed", dict(precision=1)), ("plain_fp64", dict(precision=0))):
            api.run_pipeline(prob)
            api.EigenSolver(prob).solve(nev=C2["nev"], ncv=C2_NCV, **kw)  # warm-up
            t = time.perf_counter()
            api.run_pipeline(prob)
            sol = api.EigenSolver(prob).solve(nev=C2["nev"], ncv=C2_NCV, **kw)
            wall = time.perf_counter() - t
            good, worst = count_pairs(sol.lam, sol.residual, ref) if ref is not None else \
                (int(np.sum(sol.residual <= RESID_TOL)), None)
            out[name] = {"value": good / wall, "unit": UNIT, "wall_s": wall, "eigenpairs": good,
                         "max_dlambda_rel": worst, "factor_ms": sol.diag["factor_ms"],
                         "krylov_ms": sol.diag["krylov_ms"]}
    out["mixed_vs_plain"] = out["mixed"]["value"] / max(out["plain_fp64"]["value"], 1e-300)
    return out


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
    autotuned kernels, each point warm-started from its neighbour in alpha):
    eigenpairs at resid <= 1e-10 per wall second; the
    mixed eigenvalues are compared with the plain ones point by point.  With
    several ranks the points are dealt round-robin to the GPUs (replicas) and
    the wall time is the slowest rank's."""
    from tailor_gb300 import replicas
    cases, points = c3_sweep_inputs(npoints)
    # ordered by grid class and alpha: with warm starts every worker walks a
    # contiguous run of neighbouring points of one class
    points = sorted(points)
    out, lam = {}, {}
    for name, kw in (("plain_fp64", dict(precision=0, workers=1, autotune=False)),
                     ("mixed_batched", dict(precision=1, workers=8, autotune=True,
                                            warm_start=True))):
        replicas.barrier()
        t = time.perf_counter()
        r = replicas.sweep(cases, points, nev=8, ncv=32, raise_on_error=False, **kw)
        wall, _ = replicas.reduce_timing(time.perf_counter() - t, 0)
        lam[name] = (r["lam"], r["residual"])
        good = int(np.sum((r["residual"] >= 0) & (r["residual"] <= RESID_TOL)))
        d0 = next(d for d in r["rank_diag"] if d)
        out[name] = {"value": good / wall, "unit": UNIT, "wall_s": wall, "eigenpairs": good,
                     "failed_points": int(np.sum(r["status"] != 0)),
                     "workers": d0["workers"], "ranks": r["world"],
                     "solve_block": d0["solve_block"],
                     "panel_width": d0.get("panel_width"),
                     "tensor_core_schur": [1 - c for c in d0["cuda_core_schur"]]}
    # mixed pairs count only where they match the plain FP64 eigenvalues
    (lp, rp), (lm, rm) = lam["plain_fp64"], lam["mixed_batched"]
    good, worst = 0, 0.0
    for i in range(len(points)):
        g, w = count_pairs(lm[i], rm[i], lp[i][rp[i] >= 0])
        good, worst = good + g, max(worst, w if w is not None else 0.0)
    out["mixed_batched"]["eigenpairs_matching_plain"] = good
    out["mixed_batched"]["max_dlambda_rel_vs_plain"] = worst
    out["points"] = npoints
    out["grids"] = C3_GRIDS
    return out


def cpu_oracle_sample():
    """The CPU path on a bounded sample: one 60 x 32 point of the sweep's
    physics (Mach 0.7, alpha 2.21, Re 800, nev 8)."""
    from oracle.oracle import Oracle, boundary_rows, eigen_oracle, to_complex_blocks
    from tailor_gb300.neutral_sweep import c5_case
    case = c5_case(60, 32, nev=C5_NEV)
    case.physics = dataclasses.replace(case.physics, alpha=2.21, reynolds=800.0)
    t = time.perf_counter()
    r = Oracle().full(case)
    A, B, _ = boundary_rows(case, r["metrics"], r["row_ptr"], r["col"],
                            to_complex_blocks(r["mass"]), to_complex_blocks(r["spatial"]))
    lam, _, res = eigen_oracle(r["row_ptr"], r["col"], A, B, case.nodes, 0j, C5_NEV, tol=1e-12)
    sec = time.perf_counter() - t
    return int(np.sum(res <= RESID_TOL)), sec


def run_reference(args):
    """The reference's CPU path cannot solve one point of the headline
    workload within the step budget (its LU alone is 21.3 TFLOP at 300 x
    192; the CPU oracle's 200 x 128 solve took 39 min on 8 cores), so this
    arm prints no value, only the reason and a measured sample on a smaller
    grid of the same physics, so that no ratio across different sizes is
    formed."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    good, sec = cpu_oracle_sample()
    cores = os.cpu_count() or 1
    line = {
        "impl": "reference",
        "unavailable": "the CPU oracle (C assembly, zggev rows, SuperLU + ARPACK) cannot solve one "
                       "300x192 point of the headline sweep within the step budget (21.3 TFLOP LU "
                       "per point; its 200x128 solve took 39 min on 8 cores), so no value and no "
                       "ratio; a 60x32 sample of the same physics is measured instead",
        "metric": METRIC, "unit": UNIT, "higher_is_better": True,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "config": {"workload": "C5 neutral-curve sweep, 300x192 (288000 unknowns) per point"},
        "sample": {"value": good / sec, "unit": UNIT, "cores": cores, "kind": "port",
                   "seconds": sec, "eigenpairs": good,
                   "sample": "one 60x32 point of the sweep's physics (Mach 0.7, alpha 2.21, "
                             "Re 800, nev 8): C oracle assembly, zggev boundary rows, SuperLU + "
                             "ARPACK"},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-points", type=int, default=2,
                    help="sweep points solved in the plain FP64 form for the comparison")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sweep", action="store_true", help="skip the 64-instance C3 sweep")
    ap.add_argument("--no-c2", action="store_true", help="skip the 200x128 record")
    ap.add_argument("--no-learned", action="store_true", help="first point from a random start")
    ap.add_argument("--block", type=int, default=C5_BLOCK, choices=[1, 2, 4, 8],
                    help="Krylov block size of the combined form")
    ap.add_argument("--chains", type=int, default=C5_CHAINS,
                    help="concurrent chains of sweep points of the combined form")
    ap.add_argument("--ncv", type=int, default=0,
                    help="Krylov basis size of the combined form (0: 64)")
    args = ap.parse_args()
    if args.ncv > 0:
        global C5_NCV
        C5_NCV = args.ncv
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

    from tailor_gb300 import api, learned, replicas
    from tailor_gb300 import build as tb
    from tailor_gb300.neutral_sweep import c5_case, c5_points
    tb.build()
    ref = load_c5_reference()
    pts = c5_points(snake=True)
    width = max(1, args.chains)
    # replicas: each rank walks the sweep from its own offset.  Chain w times
    # the stretch [T_w, T_w + n_w) of the snake, T_w = warmup + n_0 + ... +
    # n_(w-1), after warming up on the points just before it; its end-to-end
    # pass continues with the next chain's stretch, so with 32 steps both
    # passes cover the 32 points once and every point is warm-started from
    # its neighbour
    off = (rank * len(pts)) // max(world, 1)
    idx, nstep, nnext = chain_sequences(len(pts), args.steps, width, args.warmup, off)
    seqs = [[pts[i] for i in seq] for seq in idx]
    pos = [0] * width

    def take(counts):
        out = []
        for w in range(width):
            out.append(seqs[w][pos[w]:pos[w] + counts[w]])
            pos[w] += counts[w]
        return out

    proposal, train_s = (None, 0.0)
    if not args.no_learned:
        proposal, train_s = train_proposal(api, learned, pts)

    case = c5_case()
    ev = Events()
    chains = Chains(api, c5_case, width, local, proposal, args.block)
    prob, stream = chains.probs[0], chains.streams[0]
    # warm-up on the points before each chain's stretch; the timed passes
    # then start every chain afresh from the learned proposal
    chains.run(take([args.warmup] * width))

    def barrier():
        if dist:
            dist.barrier()

    def tally(results):
        good, worst = 0, None
        for (pt, lam, res, *_) in results:
            rl = ref.get((round(pt[1], 9), round(pt[2], 6))) if ref else None
            gd, w = count_pairs(lam, res, rl)
            good += gd
            worst = w if worst is None else (worst if w is None else max(worst, w))
        return good, worst

    # ---- device-resident timing
    clocks = ClockSampler()
    clocks.start()
    barrier()
    launches0 = prob.lib.tlr_kernel_launches()
    chains.restart()
    per, ms = chains.timed(ev, lambda: chains.run(take(nstep)))
    launches = prob.lib.tlr_kernel_launches() - launches0
    barrier()
    clk = clocks.stop()
    steps = [x for chain in per for x in chain]
    good_total, worst = tally(steps)
    ms, good_total = replicas.reduce_timing(ms, good_total)  # slowest rank, all pairs
    value = good_total / (ms / 1e3)

    # ---- end to end through the public API with pinned host buffers
    gbytes, bbytes = case.grid.nbytes, case.baseflow.nbytes
    pg, pb = ev.pinned(gbytes), ev.pinned(bbytes)
    ctypes.memmove(pg, case.grid.ctypes.data, gbytes)
    ctypes.memmove(pb, case.baseflow.ctypes.data, bbytes)

    def load(w, p):
        p.check(p.lib.tlr_load_fields(p.ctx, pg, pb))

    barrier()
    chains.restart()
    per_e2e, ms_e2e = chains.timed(ev, lambda: chains.run(take(nnext), before=load))
    barrier()
    good_e2e = tally([x for chain in per_e2e for x in chain])[0]
    ms_e2e, good_e2e = replicas.reduce_timing(ms_e2e, good_e2e)
    e2e = good_e2e / (ms_e2e / 1e3)
    d2h = C5_NEV * (16 + 8)

    # ---- the solve kernels alone: with concurrent chains, chain 0 solves one
    # more point by itself, so the per-solve times the roofline uses carry no
    # other chain's kernels
    if width > 1:
        solo = chains.run(take([1] + [0] * (width - 1)))[0]
        rsteps = solo
    else:
        rsteps = steps
    last = rsteps[-1][3]

    # ---- plain FP64 on a stated subset of the same points (rank 0)
    plain = None
    if rank == 0 and args.plain_points > 0:
        sub = [s[0] for s in steps[:args.plain_points]]
        ev.record(ev.a, stream)
        pres = [plain_step(api, prob, pt) for pt in sub]
        ev.record(ev.b, stream)
        pms = ev.elapsed_ms()
        pgood, pworst = tally([(pt, lam, res) for pt, (lam, res, _) in zip(sub, pres)])
        pv = pgood / (pms / 1e3)
        plain = {"value": pv, "unit": UNIT, "points": [[p[1], p[2]] for p in sub],
                 "ms_per_point": pms / len(sub), "eigenpairs": pgood,
                 "max_dlambda_rel": pworst,
                 "factor_ms": [r[2]["factor_ms"] for r in pres],
                 "krylov_ms": [r[2]["krylov_ms"] for r in pres],
                 "combined_vs_plain": value / pv if pv > 0 else None}
    chains.close()

    c2 = None if (args.no_c2 or rank != 0) else run_c2(api)
    sweep = None
    if not args.no_sweep:  # every rank takes its share of the points
        sweep = run_c3(api)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        gd, sec = cpu_oracle_sample()
        cpu = {"value": gd / sec, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": "one 60x32 point of the sweep's physics (Mach 0.7, alpha 2.21, Re 800, "
                         "nev 8): C oracle assembly, zggev boundary rows, SuperLU + ARPACK, "
                         "%.1f s; a smaller grid than the headline" % sec}
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    # dominant kernel: the triangular solves (one CUDA graph per solve of the
    # block's vectors), CUDA events around every replay
    nvec = last.get("block", 1)
    tri_bytes = last["factor_bytes"] + 2 * nvec * 5 * case.nodes * 8
    tri_ms = sum(s[3]["trisolve_ms"] for s in rsteps)
    tri_n = sum(s[3]["trisolves"] for s in rsteps)
    tri_avg_ms = tri_ms / max(tri_n, 1)
    achieved = tri_bytes / (tri_avg_ms * 1e-3) / 1e9 if tri_avg_ms > 0 else 0.0
    # ncu DRAM bytes / algorithmic bytes of the same solve graph, measured on
    # a 100 x 50 capture (538.1 / 518.3 MB per solve: the factor read once,
    # plus the D_b blocks), applied to this solve's algorithmic bytes
    traffic = TRISOLVE_TRAFFIC_RATIO * tri_bytes
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 factor + c128 refinement", "data": "synthetic",
        "config": {"workload": "C5 neutral-curve sweep: 300x192 (288000 unknowns), Mach 0.7, "
                               "alpha x Re on 8x4 in [0.5,3.5]x[800,2400], snake order, one "
                               "point per step, nev 8, target 0",
                   "form": "learned + mixed + batched", "block": args.block,
                   "ncv": c5_ncv(args.block), "chains": width,
                   "points": [[s[0][1], s[0][2]] for s in steps],
                   "l2": "operator 1.8 GB and factor 10 GB per point, larger than L2 (no flush)",
                   "parallelism": "replicas" if world > 1 else
                   ("single" if width == 1 else "%d concurrent chains on one GPU" % width)},
        "parity": {"reference": "tests/golden/c5_300x192_plain_eigs.txt" if ref else None,
                   "max_dlambda_rel": worst, "resid_tol": RESID_TOL, "dlambda_tol": DLAM_TOL},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": gbytes + bbytes,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "kernel": "triangular solves (solve graph: k_blk_update, k_border_gemv_pf, "
                               "k_bwd_start, k_sgather; their _m variants for blocks)",
                     "algorithmic_bytes": tri_bytes, "avg_ms": tri_avg_ms,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
        "factor": {"flops": last["factor_flops"], "ms": last["factor_ms"],
                   "tflops": last["factor_flops"] / (last["factor_ms"] * 1e-3) / 1e12
                   if last["factor_ms"] > 0 else 0.0},
        "solve": {k: last[k] for k in ("iterations", "solves", "refinement_steps", "factor_ms",
                                       "krylov_ms", "total_ms", "max_relative_error",
                                       "solve_ms", "trisolve_ms", "trisolves", "ortho_ms",
                                       "dense_ms", "residual_ms", "conv_checks")},
        "learned": {"train_points": 48, "grid": [60, 32], "train_s": train_s}
        if proposal is not None else None,
        "plain_fp64": plain,
        "cpu_baseline": cpu,
        "c2": c2,
        "sweep_c3": sweep,
    }
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
